#!/usr/bin/env python
"""Benchmark of the tracer's hot path on one GB300 (or N replicas).

Default workload: the mixed-precision forward at 1024^3 fields / nside 1024
(12,582,912 rays) / 512 RK4 steps, synthetic Gaussian fields (P(k) ~ k^-3,
phi rms 1e-5, transverse B rms 1e-7, seeded) generated on the GPU. A step is
one full-sky forward trace (srt_forward) with the fields already resident in
HBM; the headline metric is ray-steps/s = rays x n_steps / time.

Also reported on the same line:
  e2e          the same metric through the C ABI with HOST buffers: upload and
               lay out phi and B from pinned host memory, trace, read the six
               maps back, every step, with the next step's upload overlapping
               this step's trace (a run over a sequence of snapshots);
               e2e_serial is the same one step at a time;
  roofline     the trace kernel's FP32 issue rate (algorithmic FLOP per
               ray-step x ray-steps / CUDA-event time of the kernel) against the
               FP32 FMA rate measured on this GPU by srt_probe_peak;
  compare      the plain FP64 GPU form and the reference-arithmetic (REF16) GPU
               form on one batch of the same workload, the mixed/FP64 speed
               ratio, and per-map errors of the mixed form against FP64;
  cpu_baseline the FP64 CPU oracle timed on a bounded sample of rays of the
               same workload on all host cores;
  adjoint      the mixed vjp against the mixed forward (--adjoint grid,nside,
               n_steps,C[,phi]); --adjoint-only runs this leg alone and prints
               its JSON object (a diagnostic, not the bench line).
--impl reference times the reference's own CPU arithmetic for the path on the
host cores (oracle/_ref where it was built from the reference sources, else
the oracle's REF16 port) on bounded samples of the same workload, and adds
the reference's own GPU build (its raytracing_kernel, compiled unmodified)
timed on one batch of the workload on this GPU as "gpu_build".
"""
import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "snapshot-raytracer_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

# Algorithmic work of one RK4 step of one ray (4 right-hand-side evaluations,
# each with 4 tricubic interpolations of value, gradient and Hessian), counted
# operation by operation from the scheme (snapshot-raytracer.cu:195-550) as
# this build forms it, one FMA = 2 FLOP:
#   tricubic, separable: x pass 16 rows x 3 outputs x 4 taps, y pass 4 x 6 x 4,
#     z pass 10 x 4 multiply-adds = 328 FMA                     ->  656 FLOP
#   Catmull-Rom weights of value, d/dt, d2/dt2 (Horner form, 38 FLOP a set):
#     6 sets per right-hand side (3 centred axes shared by phi and by the two
#     unstaggered axes of each B component, 3 staggered)        ->  228 FLOP
#   right-hand side outside the interpolations: unit n, e1, e2 (27), the B
#     sums n.grad B, e.n.grad B, tidal matrix, n.lap B (3 x 72), the geodesic,
#     transport and Sachs terms with the dA > 1/2 branch (203)  ->  446 FLOP
#   RK4 stage states (3 x 38), accumulation (76), update (57)   ->  247 FLOP
# The packed z pass's idle half-lanes, the perturbation form's compensated
# sums and the exact position split are implementation overhead, not counted.
FLOP_PER_RAY_STEP = 4 * (4 * 656 + 228 + 446) + 247    # = 13,439
# Bytes gathered per ray-step: 4 stages x 4 fields x 64 taps x 4 B (FP32 fields).
GATHER_BYTES_PER_RAY_STEP = 4 * 4 * 64 * 4               # = 4,096
MAP_NAMES = ("dA", "ellipticity1", "ellipticity2", "rotation", "deflection1", "deflection2")


def parse():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--no-ref-gpu", dest="ref_gpu", action="store_false",
                    help="reference arm: skip the reference's own GPU build")
    ap.add_argument("--n", type=int, default=1024, help="grid side")
    ap.add_argument("--nside", type=int, default=1024)
    ap.add_argument("--n-steps", type=int, default=512)
    ap.add_argument("--precision", default="mixed", choices=("mixed", "fp64", "ref16"))
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--no-pairs", dest="pairs", action="store_false",
                    help="lay the fields out without their row-pair copies (SRT_FIELDS_NO_PAIRS): the packed MIXED "
                         "passes then form their tap pairs from the single layout")
    ap.add_argument("--e2e-steps", type=int, default=7,
                    help="timed snapshots of the pipelined end-to-end leg, less one (the serial leg times "
                         "min(this, 3)); 0 skips both")
    ap.add_argument("--compare-batch", type=int, default=5, help="batch used for the FP64 / REF16 legs (-1: skip)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU time of the CPU-baseline sample")
    ap.add_argument("--oracle-sample", type=int, default=3072,
                    help="pixels checked against the FP64 oracle (one run of consecutive pixels in each of the 12 "
                         "batches)")
    ap.add_argument("--cli-timing", metavar="DIR", default="",
                    help="write the workload's fields as the reference's two HDF5 files in DIR, run the CLI on them "
                         "with --timing (read, overlapped upload and layout, trace, FITS write) and print its JSON "
                         "timing line with the file sizes (not the bench line)")
    ap.add_argument("--parity", action="store_true",
                    help="parity record of the workload instead of the bench line: full-sky MIXED, FP64 and REF16 "
                         "forms, the reference's own GPU build batch by batch (all 12 batches), and the FP64 oracle "
                         "on --oracle-sample pixels over all batches; prints one JSON object")
    ap.add_argument("--adjoint", default="256,128,128,12",
                    help="adjoint leg: grid,nside,n_steps,ckpt_every[,phi] ('' to skip; phi: w.r.t. phi only)")
    ap.add_argument("--adjoint-only", action="store_true",
                    help="run only the adjoint leg and print its JSON object (a diagnostic, not the bench line)")
    return ap.parse_args()


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi clock / throttle samples every 200 ms while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx.append(float(f[2]))
                except ValueError:
                    continue
                for name, v in zip(names, f[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(name)
        finally:
            try:
                os.unlink(self.path)
            except OSError:
                pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ helpers

def dist_setup(n_gpus):
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def map_errors(a, b):
    from oracle.oracle import map_errors as _me

    return {name: {"rms_rel": e[0], "max_rel": e[1]} for name, e in zip(MAP_NAMES, _me(a, b))}


def sample_pixels(nside, count, begin=0, total=None, seed=0):
    total = 12 * nside * nside - begin if total is None else total
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(total, size=min(count, total), replace=False)) + begin


def batch_runs(nside, total, seed=0):
    """One run of total // 12 consecutive RING pixels at a seeded offset in
    each of the 12 batches [b nside^2, (b + 1) nside^2): [(begin, count)]."""
    per = max(1, min(total // 12, nside * nside))
    rng = np.random.default_rng(seed)
    return [(b * nside * nside + int(rng.integers(0, nside * nside - per + 1)), per) for b in range(12)]


def time_cpu(fn, target_s, make_sample, start=16):
    """Grow the sample until one call takes >= target_s / 4, then scale to
    ~target_s; returns (rays, seconds)."""
    n = start
    while True:
        pix = make_sample(n)
        t0 = time.perf_counter()
        fn(pix)
        dt = time.perf_counter() - t0
        if dt >= target_s / 4 or n >= 1 << 20:
            break
        n = int(n * max(2.0, min(16.0, (target_s / 4) / max(dt, 1e-3))))
    if dt < target_s * 0.75:
        n = int(n * target_s / max(dt, 1e-3))
        pix = make_sample(n)
        t0 = time.perf_counter()
        fn(pix)
        dt = time.perf_counter() - t0
    return len(pix), dt


# ------------------------------------------------------------ adjoint leg

def run_adjoint_leg(spec, seed, dev):
    """Mixed forward vs mixed vjp (loss = sum of seeded N(0,1) pixel weights x
    maps) at grid,nside,n_steps with checkpoints every ckpt_every steps
    (spec "grid,nside,n_steps,ckpt_every[,phi]"; phi: gradient w.r.t. phi
    only). Up to 256^3 the gradient is checked against the deterministic FP64
    vjp (whole grid) and, on a 64-pixel range, against the oracle's FP64
    forward-mode tangent."""
    import torch

    import srt
    import srt_fields
    from oracle import oracle

    parts = spec.split(",")
    n, nside, S, C = [int(x) for x in parts[:4]]
    wrt = ("phi",) if len(parts) > 4 and parts[4] == "phi" else ("phi", "b")
    npix = 12 * nside * nside
    phi, b = srt_fields.gaussian_fields_torch(n, seed=seed + 101, device=dev)
    w = torch.from_numpy(np.random.default_rng(seed).standard_normal((6, npix)).astype(np.float32)).to(dev)
    out = torch.empty((6, npix), dtype=torch.float32, device=dev)
    gphi = torch.zeros_like(phi)
    gb = torch.zeros_like(b) if "b" in wrt else None
    stream = torch.cuda.current_stream(dev)
    res = {"workload": "%d^3, nside %d (%d rays), %d steps, checkpoints every %d steps, gradient w.r.t. %s" %
                       (n, nside, npix, S, C, " and ".join(wrt))}
    reps = 4 if n <= 512 else 2
    with srt.Fields(phi, b, stream=stream) as f:
        fwd, adj = [], []
        fwd_nr = []
        for i in range(reps):
            _, st = f.forward(nside, S, precision="mixed", out=out, stream=stream)
            _, st2 = f.forward(nside, S, precision="mixed", out=out, stream=stream, refine=False)
            _, _, sa = f.vjp(nside, S, w, precision="mixed", dphi=gphi, db_xyz=gb, ckpt_every=C, stream=stream,
                             wrt=wrt)
            if i > 0:
                fwd.append(st.trace_ms)
                fwd_nr.append(st2.trace_ms)
                adj.append(sa.trace_ms)
        res["forward_ms"] = float(np.median(fwd))
        res["forward_fp32_only_ms"] = float(np.median(fwd_nr))
        res["vjp_ms"] = float(np.median(adj))
        res["vjp_over_forward"] = res["vjp_ms"] / res["forward_ms"]
        res["vjp_over_fp32_forward"] = res["vjp_ms"] / res["forward_fp32_only_ms"]
        res["vjp_ray_steps_per_s"] = npix * S / (res["vjp_ms"] * 1e-3)
        # the forward/vjp pair: a forward that keeps its checkpoints, then the
        # backward sweep alone
        ftape, btape = [], []
        for i in range(reps):
            _, tape, stf = f.forward_tape(nside, S, ckpt_every=C, out=out, stream=stream)
            _, _, stb = tape.vjp(w, dphi=gphi, db_xyz=gb, stream=stream, wrt=wrt)
            tape.close()
            if i > 0:
                ftape.append(stf.trace_ms)
                btape.append(stb.trace_ms)
        res["forward_tape_ms"] = float(np.median(ftape))
        res["vjp_tape_ms"] = float(np.median(btape))
        res["vjp_tape_over_forward"] = res["vjp_tape_ms"] / res["forward_ms"]
        res["vjp_tape_over_fp32_forward"] = res["vjp_tape_ms"] / res["forward_fp32_only_ms"]
        if n > 256 or "b" not in wrt:
            torch.cuda.synchronize()
            del phi, b, gphi, gb, out, w
            torch.cuda.empty_cache()
            return res
        # accuracy: mixed vjp vs deterministic FP64 vjp over the whole grid
        g64 = torch.zeros_like(phi)
        b64 = torch.zeros_like(b)
        _, _, s64 = f.vjp(nside, S, w, precision="fp64", dphi=g64, db_xyz=b64, ckpt_every=C, deterministic=True,
                          stream=stream)
        torch.cuda.synchronize()
        res["fp64_deterministic_vjp_ms"] = s64.trace_ms

        def rel(a, r):
            a, r = a.double(), r.double()
            return float(torch.linalg.vector_norm(a - r) / torch.linalg.vector_norm(r))

        res["mixed_vs_fp64_grad_rel_l2"] = {"phi": rel(gphi, g64), "B": rel(gb, b64)}
        # dot-product test on a 64-pixel range against the oracle tangent
        lo, cnt = 5 * nside * nside + nside, 64
        wpart = w[:, lo:lo + cnt].contiguous()
        gp = torch.zeros_like(phi)
        bp = torch.zeros_like(b)
        f.vjp(nside, S, wpart, pix_begin=lo, pix_count=cnt, precision="fp64", dphi=gp, db_xyz=bp, ckpt_every=C,
              stream=stream)
        gpm = torch.zeros_like(phi)
        bpm = torch.zeros_like(b)
        f.vjp(nside, S, wpart, pix_begin=lo, pix_count=cnt, precision="mixed", dphi=gpm, db_xyz=bpm, ckpt_every=C,
              stream=stream)
        torch.cuda.synchronize()
    phi_np, b_np = phi.cpu().numpy(), b.cpu().numpy()
    rng = np.random.default_rng(seed + 7)
    dp = [rng.standard_normal(phi_np.shape).astype(np.float32) for _ in range(2)] + [None, None]
    db = [None, None] + [rng.standard_normal(b_np.shape).astype(np.float32) for _ in range(2)]
    _, dL = oracle.tangent(phi_np, b_np, nside, S, np.arange(lo, lo + cnt), wpart.cpu().numpy(), dp, db)
    checks = []
    for k in range(4):
        for name, g_, b_ in (("fp64", gp, bp), ("mixed", gpm, bpm)):
            got = (float(np.dot(g_.cpu().numpy().ravel().astype(np.float64), dp[k].ravel())) if dp[k] is not None
                   else float(np.dot(b_.cpu().numpy().ravel().astype(np.float64), db[k].ravel())))
            checks.append({"direction": k, "vjp": name, "rel_err": abs(got - dL[k]) / max(abs(dL[k]), 1e-300)})
    res["tangent_check_64px"] = {"max_rel_err_fp64": max(c["rel_err"] for c in checks if c["vjp"] == "fp64"),
                                 "max_rel_err_mixed": max(c["rel_err"] for c in checks if c["vjp"] == "mixed")}
    del phi, b, gphi, gb, g64, b64, gp, bp, gpm, bpm, out, w
    torch.cuda.empty_cache()
    return res


# ------------------------------------------------------------ parity record

def run_parity(args):
    """Per-map errors of every form at one workload (all 12 batches): MIXED,
    FP64 and REF16 full skies; the reference's own GPU build run batch by batch
    as its CLI runs them (snapshot-raytracer.cu:708-717, :897-901) and the 12
    batch maps summed into a sky; the FP64 oracle on a run of pixels in every
    batch. Errors are relative to each map's rms signal (map_errors)."""
    import torch

    import srt
    import srt_fields
    from oracle import oracle

    n, nside, S = args.n, args.nside, args.n_steps
    npix = 12 * nside * nside
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    phi_d, b_d = srt_fields.gaussian_fields_torch(n, seed=args.seed, device=dev)
    res = {"workload": "%d^3 fields, nside %d (%d rays, 12 batches), %d steps" % (n, nside, npix, S),
           "fields": "gaussian P(k)~k^-3, phi rms 1e-5, transverse B rms 1e-7, torch generator seed %d" % args.seed}
    maps, secs = {}, {}
    with srt.Fields(phi_d, b_d) as f:
        for mode in ("mixed", "fp64", "ref16"):
            o = torch.empty((6, npix), dtype=torch.float32, device=dev)
            f.forward(nside, S, precision=mode, out=o)  # REF16 builds its planes on first use
            _, st = f.forward(nside, S, precision=mode, out=o)
            torch.cuda.synchronize()
            maps[mode] = o.cpu().numpy()
            secs[mode] = {"kernel_ms": st.trace_ms, "ray_steps_per_s": npix * S / (st.trace_ms * 1e-3),
                          "refined_rays": st.refined_rays}
            del o
    res["forms"] = secs
    ref = None
    if oracle.ref_gpu_available():
        ref = np.zeros((6, npix), np.float32)
        kms = 0.0
        for bt in range(12):
            r, ms = oracle.ref_gpu_trace(phi_d, b_d, nside, S, bt * nside * nside, nside * nside)
            ref[:, bt * nside * nside:(bt + 1) * nside * nside] = r.cpu().numpy()
            kms += ms[0]
        res["reference_gpu_build"] = {"kernel_ms_12_batches": kms, "ray_steps_per_s": npix * S / (kms * 1e-3)}
    phi_np, b_np = phi_d.cpu().numpy(), b_d.cpu().numpy()
    del phi_d, b_d
    torch.cuda.empty_cache()
    ranges = batch_runs(nside, args.oracle_sample, seed=1)
    pix = np.concatenate([np.arange(lo, lo + c) for lo, c in ranges])
    t0 = time.perf_counter()
    want = oracle.trace_pixels(phi_np, b_np, nside, S, pix, mode="fp64", threads=oracle.max_threads())
    res["oracle_sample"] = {"pixels": len(pix), "runs": "%d runs of %d consecutive RING pixels, one per batch"
                            % (len(ranges), ranges[0][1]), "cpu_s": time.perf_counter() - t0,
                            "cores": oracle.max_threads()}
    err = {}
    for name in ("fp64", "mixed", "ref16"):
        err["%s_vs_oracle" % name] = map_errors(maps[name][:, pix], want)
    err["mixed_vs_fp64_full_sky"] = map_errors(maps["mixed"], maps["fp64"])
    err["ref16_vs_fp64_full_sky"] = map_errors(maps["ref16"], maps["fp64"])
    if ref is not None:
        err["reference_build_vs_oracle"] = map_errors(ref[:, pix], want)
        err["reference_build_vs_fp64_full_sky"] = map_errors(ref, maps["fp64"])
        err["reference_build_vs_ref16_full_sky"] = map_errors(ref, maps["ref16"])
    res["errors"] = err
    print(json.dumps({"parity": res}), flush=True)


# ------------------------------------------------------ CLI end to end

def run_cli_timing(args):
    """The drop-in CLI on the workload: fields written as /data of two HDF5
    files (phi float32, B array[3] of float32, the reference's layout), then
    `snapshot-raytracer phi.h5 B.h5 nside n_steps --timing --overwrite`; its
    timing line separates the reads, the layout overlapped with them, the part
    of the upload left after the reads, the trace and the FITS writes."""
    import torch

    import srt
    import srt_fields

    n, nside, S = args.n, args.nside, args.n_steps
    os.makedirs(args.cli_timing, exist_ok=True)
    phi_d, b_d = srt_fields.gaussian_fields_torch(n, seed=args.seed, device=torch.device("cuda", 0))
    pp, pb = os.path.join(args.cli_timing, "phi.h5"), os.path.join(args.cli_timing, "B.h5")
    t0 = time.perf_counter()
    srt.h5_write(pp, phi_d.cpu().numpy())
    srt.h5_write(pb, b_d.cpu().numpy(), vector3=True)
    write_s = time.perf_counter() - t0
    del phi_d, b_d
    torch.cuda.empty_cache()
    cli = os.path.join(PKG, "snapshot-raytracer")
    r = subprocess.run([cli, pp, pb, str(nside), str(S), "--timing", "--overwrite", "--outdir", args.cli_timing],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("CLI failed (%d): %s" % (r.returncode, r.stderr[-500:]))
    timing = json.loads(r.stdout.strip().splitlines()[-1])
    print(json.dumps({"cli_timing": {"workload": "%d^3 fields, nside %d, %d steps, two HDF5 files (%.1f GB)" % (
        n, nside, S, (os.path.getsize(pp) + os.path.getsize(pb)) / 1e9), "hdf5_write_s": write_s,
        "stdout": r.stdout.strip().splitlines()[:-1], **timing}}), flush=True)


# --------------------------------------------------------------- our arm

def run_ours(args):
    import torch

    import srt
    import srt_fields

    if args.adjoint_only:
        print(json.dumps({"adjoint": run_adjoint_leg(args.adjoint, args.seed, torch.device("cuda", 0))}), flush=True)
        return
    if args.parity:
        run_parity(args)
        return
    if args.cli_timing:
        run_cli_timing(args)
        return

    rank, world, local = dist_setup(args.gpus)
    dev = torch.device("cuda", local)
    n, nside, S = args.n, args.nside, args.n_steps
    npix = 12 * nside * nside
    cfg = {"workload": "forward trace, %d^3 fields, nside %d (%d rays), %d steps, %s" % (n, nside, npix, S,
                                                                                       args.precision),
           "grid": n, "nside": nside, "rays": npix, "n_steps": S, "precision": args.precision,
           "fields": "gaussian P(k)~k^-3, phi rms 1e-5, B rms 1e-7, seed %d" % (args.seed + rank),
           "l2": "inputs larger than L2 (%.1f GB of fields vs 0.13 GB L2)" % (16 * n ** 3 / 1e9),
           "parallelism": "replicas x%d (pixel-parallel, no collective)" % world}

    phi_d, b_d = srt_fields.gaussian_fields_torch(n, seed=args.seed + rank, device=dev)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream(dev)
    fields = srt.Fields(phi_d, b_d, stream=stream, pairs=args.pairs)
    # the row-pair copies are built only when they fit (not at 2048^3)
    with_pairs = fields.nbytes > 16 * (n + 3) ** 3
    cfg["field_layout"] = "halo-padded planes" + (" + row-pair copies" if with_pairs else
                                                  " (packed passes form their pairs from the single layout)")
    if args.e2e_steps <= 0:  # the laid-out copy is all the trace needs (2048^3: 137 GB freed)
        torch.cuda.synchronize()
        del phi_d, b_d
        torch.cuda.empty_cache()
    out = torch.empty((6, npix), dtype=torch.float32, device=dev)

    # FP32 peak: the larger of the scalar FFMA and packed FFMA2 rates measured here
    peak_fp32 = max(srt.probe_peak("fp32"), srt.probe_peak("fp32x2"))
    peak_fp64 = srt.probe_peak("fp64")

    for _ in range(args.warmup):
        fields.forward(nside, S, precision=args.precision, out=out, stream=stream)
    torch.cuda.synchronize()

    trace_ms, retrace_ms, kernels, refined = [], [], 0, []
    with ClockSampler(local) as clocks:
        barrier(world)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            _, st = fields.forward(nside, S, precision=args.precision, out=out, stream=stream)
            trace_ms.append(st.trace_ms)
            retrace_ms.append(st.retrace_ms)
            kernels += st.kernels
            refined.append(st.refined_rays)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
    clk = clocks.summary()
    elapsed_ms = max_over_ranks(e0.elapsed_time(e1), world)
    ms_per_step = elapsed_ms / args.steps
    ray_steps = npix * S
    value = world * ray_steps / (ms_per_step * 1e-3)
    # the dominant kernel (the trace) alone: srt_forward's events split off the
    # re-trace launches that follow it on the stream (reported beside it)
    retrace_mean = float(np.mean(retrace_ms))
    kernel_ms = float(np.mean(trace_ms)) - retrace_mean
    achieved = FLOP_PER_RAY_STEP * ray_steps / (kernel_ms * 1e-3)

    result = {"metric": "ray-steps/s", "value": value, "unit": "ray-steps/s", "n_gpus": world,
              "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
              "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.precision == "mixed" else
              ("f64" if args.precision == "fp64" else "f32/f16"), "data": "synthetic", "config": cfg,
              "gpu_launches": kernels,
              "refined_rays_per_step": int(np.max(refined)) if refined else 0}
    # DRAM bytes of one trace launch: an ncu capture of a smaller case of the
    # same kernel scaled to this workload (profiles/trace_traffic.json); null
    # for workloads it does not cover
    traffic = None
    prof = os.path.join(ROOT, "profiles", "trace_traffic.json")
    if os.path.isfile(prof):
        try:
            rec = json.load(open(prof)).get("dram_bytes_per_launch", {}).get(args.precision)
            if rec and (rec["grid"], rec["nside"], rec["n_steps"]) == (n, nside, S):
                traffic = rec["read"] + rec["write"]
        except (OSError, ValueError, KeyError):
            traffic = None
    result["roofline"] = {"bound": "fp32", "achieved": achieved / 1e12, "peak": peak_fp32 / 1e12,
                          "unit": "TFLOP/s", "frac": achieved / peak_fp32, "traffic": traffic,
                          "kernel": "trace_kernel (%s)" % args.precision, "kernel_ms": kernel_ms,
                          "retrace_ms": retrace_mean,
                          "frac_with_retrace": FLOP_PER_RAY_STEP * ray_steps / ((kernel_ms + retrace_mean) * 1e-3)
                                               / peak_fp32,
                          "flop_per_ray_step": FLOP_PER_RAY_STEP,
                          "peak_source": "measured on this GPU by srt_probe_peak (FP32 FFMA / FFMA2 loops, burst; the larger)",
                          "fp64_peak_tflops": peak_fp64 / 1e12,
                          "gather_GBps": GATHER_BYTES_PER_RAY_STEP * ray_steps / (kernel_ms * 1e-3) / 1e9}
    result["clocks"] = clk

    # ---- end to end through the C ABI with host buffers
    if args.e2e_steps > 0:
        phi_h = torch.empty(phi_d.shape, dtype=torch.float32, pin_memory=True)
        b_h = torch.empty(b_d.shape, dtype=torch.float32, pin_memory=True)
        phi_h.copy_(phi_d)
        b_h.copy_(b_d)
        fields.close()
        del phi_d, b_d
        torch.cuda.empty_cache()
        phi_np, b_np = phi_h.numpy(), b_h.numpy()
        # the maps land in pinned host memory, as the inputs come from it
        maps_h = torch.zeros((6, npix), dtype=torch.float32, pin_memory=True).numpy()
        h2d, d2h = int(phi_np.nbytes + b_np.nbytes), int(maps_h.nbytes)
        # (1) serial: every step creates the fields from the host arrays
        # (the layout kernel reads the pinned memory directly), traces, reads
        # the maps back and releases the fields
        times, split = [], []
        for i in range(min(args.e2e_steps, 3) + 1):
            barrier(world)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            f = srt.Fields(phi_np, b_np, pairs=args.pairs)
            ta = time.perf_counter()
            f.forward(nside, S, precision=args.precision, out=maps_h)
            tb = time.perf_counter()
            f.close()
            t1 = time.perf_counter()
            if i > 0:
                times.append(t1 - t0)
                split.append(((ta - t0) * 1e3, (tb - ta) * 1e3, (t1 - tb) * 1e3))
        serial_s = max_over_ranks(float(np.mean(times)), world)
        sp = np.mean(np.array(split), axis=0)
        # (2) pipelined, as a run over a sequence of snapshots goes: step i+1's
        # fields are uploaded by the copy engines (SRT_ASYNC, staged) on a
        # high-priority stream while step i traces; every step still copies
        # its 17 GB in and its maps out inside the timed region, and the first
        # upload is not hidden
        # two non-default streams: work on the legacy default stream would wait
        # for the upload stream's work (and the upload for it)
        s_up = torch.cuda.Stream(device=dev, priority=-1)
        s_tr = torch.cuda.Stream(device=dev)
        K = args.e2e_steps + 1

        call_ms = []  # host time of each asynchronous create call (it should return at once)
        marks = []    # CUDA events: (upload start, upload end) on s_up, (trace start, trace end) on s_tr

        def mark(stream):
            e = torch.cuda.Event(enable_timing=True)
            e.record(stream)
            return e

        def create_async(first=False):
            # the first upload has no trace to hide behind: the layout kernel
            # reads the pinned arrays itself, the fastest way in; the others go
            # through the copy engines, which leave the SMs to the trace
            tc = time.perf_counter()
            e0 = mark(s_up)
            f = srt.Fields(phi_np, b_np, stream=s_up, async_=True, staged=not first, pairs=args.pairs)
            marks.append(("up", e0, mark(s_up)))
            call_ms.append(round((time.perf_counter() - tc) * 1e3, 1))
            return f

        def pipeline(steps):
            # the previous step's fields are released before the next upload is
            # queued, so at most two sets (and the staging buffer) are held and
            # the memory pool reuses them instead of mapping new memory
            nxt = create_async(first=True)
            ev = torch.cuda.Event()
            ev.record(s_up)
            prev = None
            for i in range(steps):
                s_tr.wait_event(ev)
                cur = nxt
                if prev is not None:
                    prev.close()
                    prev = None
                if i + 1 < steps:
                    nxt = create_async()
                    ev = torch.cuda.Event()
                    ev.record(s_up)
                e0 = mark(s_tr)
                cur.forward(nside, S, precision=args.precision, out=maps_h, stream=s_tr)
                marks.append(("trace", e0, mark(s_tr)))
                prev = cur
            prev.close()
            torch.cuda.synchronize()

        pipeline(2)  # untimed: the pool grows to the pipeline's working set
        barrier(world)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        del call_ms[:]
        del marks[:]
        pipeline(K)
        pipe_s = max_over_ranks((time.perf_counter() - t0) / K, world)
        # the timeline of the timed pipeline, ms from its first upload's start
        base = marks[0][1]
        timeline = [[kind, round(base.elapsed_time(a), 1), round(base.elapsed_time(b), 1)] for kind, a, b in marks]
        result["e2e"] = {"value": world * ray_steps / pipe_s, "unit": "ray-steps/s",
                         "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": pipe_s * 1e3,
                         "mode": "pipelined over %d steps: step i+1's upload (copy engines, high-priority stream) "
                                 "overlaps step i's trace; the first upload (the layout kernel reading the pinned "
                                 "arrays) is inside the timed region" % K,
                         "create_call_ms": call_ms, "timeline_ms": timeline}
        result["e2e_serial"] = {"value": world * ray_steps / serial_s, "unit": "ray-steps/s",
                                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": serial_s * 1e3,
                                "split_ms": {"fields_create_upload": float(sp[0]),
                                             "forward_and_maps_back": float(sp[1]), "fields_release": float(sp[2])},
                                "create_ms_each": [round(x[0], 1) for x in split],
                                "mode": "one step at a time: create (layout kernel reads the pinned host arrays), "
                                        "trace, maps back, release"}
        fields = srt.Fields(phi_np, b_np, pairs=args.pairs)
    else:
        phi_np = b_np = None

    # ---- comparison legs on one batch (rank 0 only)
    if rank == 0 and args.compare_batch >= 0:
        b0, cnt = args.compare_batch * nside * nside, nside * nside
        legs = {}
        bout = torch.empty((6, cnt), dtype=torch.float32, device=dev)
        maps = {}
        for mode in ("mixed", "fp64", "ref16"):
            fields.forward(nside, S, b0, cnt, precision=mode, out=bout, stream=stream)  # warm (REF16 builds its planes)
            _, st = fields.forward(nside, S, b0, cnt, precision=mode, out=bout, stream=stream)
            torch.cuda.synchronize()
            legs[mode] = {"ray_steps_per_s": cnt * S / (st.trace_ms * 1e-3), "kernel_ms": st.trace_ms,
                          "refined_rays": st.refined_rays}
            maps[mode] = bout.cpu().numpy()
        cmp = {"batch": args.compare_batch, "rays": cnt, "legs": legs,
               "mixed_over_fp64": legs["mixed"]["ray_steps_per_s"] / legs["fp64"]["ray_steps_per_s"],
               "mixed_over_ref16": legs["mixed"]["ray_steps_per_s"] / legs["ref16"]["ray_steps_per_s"],
               "mixed_vs_fp64_error": map_errors(maps["mixed"], maps["fp64"]),
               "ref16_vs_fp64_error": map_errors(maps["ref16"], maps["fp64"])}
        if phi_np is not None and args.oracle_sample > 0:
            from oracle import oracle

            # a run of consecutive RING pixels in each of the 12 batches: the
            # FP64 oracle on all of them, against the MIXED full sky of the
            # timed region and the FP64 GPU form traced on the same runs
            ranges = batch_runs(nside, args.oracle_sample, seed=1)
            pix = np.concatenate([np.arange(lo, lo + c) for lo, c in ranges])
            want = oracle.trace_pixels(phi_np, b_np, nside, S, pix, mode="fp64", threads=oracle.max_threads())
            f64 = np.concatenate([fields.forward(nside, S, lo, c, precision="fp64")[0] for lo, c in ranges], axis=1)
            mixed = out[:, torch.from_numpy(pix).to(dev)].cpu().numpy()
            cmp["oracle_sample"] = {"pixels": len(pix),
                                    "runs": "%d runs of %d consecutive RING pixels, one in each batch" %
                                            (len(ranges), ranges[0][1]),
                                    "fp64_gpu_vs_oracle": map_errors(f64, want),
                                    "mixed_gpu_vs_oracle": map_errors(mixed, want)}
        result["compare"] = cmp

    # ---- adjoint leg (rank 0)
    if rank == 0 and args.adjoint:
        fields.close()
        fields = None
        result["adjoint"] = run_adjoint_leg(args.adjoint, args.seed, dev)

    # ---- CPU baseline: FP64 oracle on a bounded sample (rank 0, N = 1 only)
    if rank == 0 and world == 1 and phi_np is not None and args.cpu_seconds > 0:
        from oracle import oracle

        cores = oracle.max_threads()
        # the fields are laid out once, outside the timed calls, as the GPU
        # arm's fields are resident before its timed region
        with oracle.Fields(phi_np, b_np, mode="fp64") as of:
            rays, dt = time_cpu(lambda pix: of.trace_pixels(nside, S, pix, threads=cores),
                                args.cpu_seconds, lambda k: sample_pixels(nside, k, seed=2))
        result["cpu_baseline"] = {"value": rays * S / dt, "unit": "ray-steps/s", "cores": cores, "kind": "port",
                                  "sample": "%d random pixels of the same workload x %d steps, FP64 oracle, "
                                            "%.1f s" % (rays, S, dt)}
    if fields is not None:
        fields.close()
    if rank == 0:
        print(json.dumps(result))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


# --------------------------------------------------------- reference arm

def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import torch

    import srt_fields
    from oracle import oracle

    n, nside, S = args.n, args.nside, args.n_steps
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    phi_t, b_t = srt_fields.gaussian_fields_torch(n, seed=args.seed, device=dev)
    phi_np, b_np = phi_t.cpu().numpy(), b_t.cpu().numpy()
    gpu_build = None
    if dev == "cuda" and args.ref_gpu:
        gpu_build = run_reference_gpu_build(oracle, phi_t, b_t, nside, S)
    del phi_t, b_t
    use_ref = oracle.ref_available()
    cores = oracle.max_threads()
    # the fields are staged once (FP16 B planes), outside the timed region, as
    # the GPU arm's fields are resident before its timed region
    ofields = oracle.Fields(phi_np, b_np, mode="ref16", reference=use_ref)

    def run(pix):
        ofields.trace_pixels(nside, S, pix, threads=cores)
    make = lambda k: sample_pixels(nside, k, seed=3)  # noqa: E731
    kind = "reference" if use_ref else "port"
    per_step_s = max(2.0, min(20.0, 60.0 / max(args.steps + args.warmup, 1)))
    rays, dt = time_cpu(run, per_step_s, make)
    pix = make(rays)
    for _ in range(args.warmup):
        run(pix)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        run(pix)
    dt = (time.perf_counter() - t0) / args.steps
    ofields.close()
    value = rays * S / dt
    sample = ("%d pixels x %d steps of the %d^3 / nside %d workload per step, %s" %
              (rays, S, n, nside, "reference host code (oracle/_ref)" if use_ref else
               "oracle REF16 port of the reference's arithmetic"))
    res = {"impl": "reference", "metric": "ray-steps/s", "value": value, "unit": "ray-steps/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32/f16", "data": "synthetic",
           "config": {"workload": "forward trace, %d^3 fields, nside %d, %d steps (CPU, reference arithmetic)"
                                  % (n, nside, S), "grid": n, "nside": nside, "n_steps": S},
           "cpu_baseline": {"value": value, "unit": "ray-steps/s", "cores": cores, "kind": kind, "sample": sample},
           "e2e": {"value": value, "unit": "ray-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "gpu_launches": 0}
    if gpu_build is not None:
        res["gpu_build"] = gpu_build
    print(json.dumps(res))


def run_reference_gpu_build(oracle, phi_t, b_t, nside, S):
    """The reference's own GPU build (raytracing_kernel compiled unmodified from
    its source, launched as its main() launches it) on one batch of the same
    workload on this GPU: kernel time by CUDA events, as a second reference
    figure beside the CPU line."""
    if not oracle.ref_gpu_available():
        return {"unavailable": "reference cubin not built (needs the reference sources at build time)"}
    begin, count = 5 * nside * nside, nside * nside
    try:
        _, ms = oracle.ref_gpu_trace(phi_t, b_t, nside, S, begin, count, reps=2)
    except RuntimeError as e:
        return {"unavailable": str(e)}
    t = min(ms)
    return {"value": count * S / (t * 1e-3), "unit": "ray-steps/s", "kernel_ms": t, "rays": count,
            "sample": "batch 5 (RING pixels [5 nside^2, 6 nside^2)) x %d steps; min of 2 launches" % S,
            "build": "nvcc -O3 --use_fast_math, sm_103a, reference source unmodified"}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
