"""GPU parity of the trace kernels (through the C ABI) against the oracle and
against the golden vectors of the reference's own code.

Tolerances (relative to the rms of each map's signal; for dA the rms of its
fluctuation about the mean, see conftest.map_errors):
  FP64  vs oracle FP64      rms <= 1e-9, max <= 1e-7   (only FMA contraction and
                                                        libm ulps differ)
  MIXED vs oracle FP64      rms <= 1e-5, max <= 1e-4   (the FP32 target)
  REF16 vs reference golden rms <= 1e-5, max <= 2e-3   (same FP16/FP32 arithmetic,
                                                        different FP32 rounding order)
Pixel placement and batch masking are compared bit for bit.
"""
import numpy as np
import pytest

import srt_fields
from conftest import golden_fields, map_errors

pytestmark = pytest.mark.gpu

CASES = ["cube16_ns2_s12", "cube32_ns4_s24", "cube24_ns3_s20", "wrap16_ns2_s40", "batch5_cube32_ns4_s16",
         "noncubic_16x20x24_ns2_s14"]
TOL = {"fp64": (1e-9, 1e-7), "mixed": (1e-5, 1e-4), "ref16": (1e-5, 2e-3)}


def _range(meta, case):
    c = meta["cases"][case]
    nside, batch = c["nside"], c["batch"]
    if batch is None:
        return nside, c["n_steps"], 0, 12 * nside * nside
    return nside, c["n_steps"], batch * nside * nside, nside * nside


def _assert_close(got, want, mode, what):
    rms_t, max_t = TOL[mode]
    errs = map_errors(got, want)
    for m, (rms, mx) in enumerate(errs):
        assert rms <= rms_t and mx <= max_t, "%s map %d: rms %.3g max %.3g (tol %.1g/%.1g)" % (
            what, m, rms, mx, rms_t, max_t)
    return errs


@pytest.mark.parametrize("case", CASES)
def test_fp64_matches_oracle(golden, srt, orc, case):
    meta, _ = golden
    phi, b = golden_fields(meta, case)
    nside, steps, begin, count = _range(meta, case)
    with srt.Fields(phi, b) as f:
        got, st = f.forward(nside, steps, begin, count, "fp64")
    assert st.rays == count and st.ray_steps == count * steps and st.kernels >= 1
    want = orc.trace(phi, b, nside, steps, begin, count, mode="fp64")
    _assert_close(got, want, "fp64", case)


@pytest.mark.parametrize("pairs", [True, False], ids=["pair-layout", "single-layout"])
@pytest.mark.parametrize("case", CASES)
def test_mixed_matches_oracle(golden, srt, orc, case, pairs):
    meta, _ = golden
    phi, b = golden_fields(meta, case)
    nside, steps, begin, count = _range(meta, case)
    with srt.Fields(phi, b, pairs=pairs) as f:
        got, _ = f.forward(nside, steps, begin, count, "mixed")
    want = orc.trace(phi, b, nside, steps, begin, count, mode="fp64")
    _assert_close(got, want, "mixed", case)


@pytest.mark.parametrize("case", CASES)
def test_ref16_matches_reference_golden(golden, srt, case):
    meta, maps = golden
    phi, b = golden_fields(meta, case)
    nside, steps, begin, count = _range(meta, case)
    with srt.Fields(phi, b) as f:
        got, _ = f.forward(nside, steps, begin, count, "ref16")
    _assert_close(got, maps[case][:, begin:begin + count], "ref16", case)


@pytest.mark.parametrize("mode", ["fp64", "mixed", "ref16"])
def test_zero_fields_exact(srt, mode):
    n, nside, steps = 16, 4, 9
    phi = np.zeros((n, n, n), np.float32)
    b = np.zeros((n, n, n, 3), np.float32)
    with srt.Fields(phi, b) as f:
        m, _ = f.forward(nside, steps, precision=mode)
    assert np.all(m[0] == steps)
    assert not np.any(m[1:4])
    assert np.abs(m[4:6]).max() < 1e-12


def test_batches_tile_the_sky_bit_exact(srt):
    """Batch b = RING pixels [b nside^2, (b+1) nside^2) (snapshot-raytracer.cu:708-717):
    each batch's values equal the full-sky run's, bit for bit, and the CLI-style
    full maps are zero outside the batch, so the 12 batches sum to the full sky."""
    phi, b = srt_fields.int_noise_fields(32, seed=21)
    nside, steps = 4, 10
    for mode in ("mixed", "fp64"):
        full = srt.trace(phi, b, nside, steps, precision=mode)
        acc = np.zeros_like(full)
        for batch in range(12):
            part = srt.trace(phi, b, nside, steps, batch=batch, precision=mode)
            lo, hi = batch * nside * nside, (batch + 1) * nside * nside
            assert np.array_equal(part[:, lo:hi].view(np.uint32), full[:, lo:hi].view(np.uint32))
            mask = np.ones(12 * nside * nside, bool)
            mask[lo:hi] = False
            assert not np.any(part[:, mask])
            acc += part
        assert np.array_equal(acc.view(np.uint32), full.view(np.uint32))
    with pytest.raises(ValueError):
        srt.trace(phi, b, nside, steps, batch=12)


def test_arbitrary_ranges_and_empty(srt):
    phi, b = srt_fields.int_noise_fields(16, seed=22)
    with srt.Fields(phi, b) as f:
        full, _ = f.forward(3, 7, precision="mixed")
        part, _ = f.forward(3, 7, pix_begin=7, pix_count=13, precision="mixed")
        assert np.array_equal(part.view(np.uint32), full[:, 7:20].view(np.uint32))
        empty, st = f.forward(3, 7, pix_begin=5, pix_count=0)
        assert empty.shape == (6, 0) and st.rays == 0
        last, _ = f.forward(3, 7, pix_begin=107, pix_count=1, precision="mixed")
        assert np.array_equal(last.view(np.uint32), full[:, 107:108].view(np.uint32))


def test_invalid_arguments_raise(srt):
    phi, b = srt_fields.int_noise_fields(16, seed=23)
    with srt.Fields(phi, b) as f:
        for kw in ({"nside": 0, "n_steps": 4}, {"nside": 2, "n_steps": 0}, {"nside": 2, "n_steps": 4, "pix_begin": 49},
                   {"nside": 2, "n_steps": 4, "pix_begin": -1, "pix_count": 3}):
            with pytest.raises((srt.SrtError, ValueError)):
                f.forward(**kw)
        with pytest.raises(KeyError):
            f.forward(2, 4, precision="fp16")


def test_deterministic(srt):
    phi, b = srt_fields.gaussian_fields_np(32, seed=4)
    with srt.Fields(phi, b) as f:
        a, _ = f.forward(8, 20, precision="mixed")
        c, _ = f.forward(8, 20, precision="mixed")
    assert np.array_equal(a.view(np.uint32), c.view(np.uint32))


@pytest.mark.parametrize("mode,pairs", [("fp64", True), ("mixed", True), ("mixed", False)])
def test_gaussian_fields_vs_oracle(srt, orc, mode, pairs):
    phi, b = srt_fields.gaussian_fields_np(64, seed=7)
    nside, steps = 8, 48
    with srt.Fields(phi, b, pairs=pairs) as f:
        got, _ = f.forward(nside, steps, precision=mode)
    want = orc.trace(phi, b, nside, steps, mode="fp64")
    _assert_close(got, want, mode, "gaussian64")


def test_device_buffers_match_host(srt):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch without CUDA")
    phi, b = srt_fields.gaussian_fields_np(32, seed=9)
    with srt.Fields(phi, b) as f:
        host, _ = f.forward(4, 16, precision="mixed")
    tphi, tb = torch.from_numpy(phi).cuda(), torch.from_numpy(b).cuda()
    out = torch.zeros((6, 192), dtype=torch.float32, device="cuda")
    with srt.Fields(tphi, tb) as f:
        f.forward(4, 16, precision="mixed", out=out)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy().view(np.uint32), host.view(np.uint32))


def test_larger_grid_mixed_vs_fp64_and_oracle_sample(srt, orc):
    """256^3 / nside 64 / 128 steps (49k rays): MIXED against the all-FP64 GPU
    form on every pixel, and the FP64 form against the oracle on a sample."""
    phi, b = srt_fields.gaussian_fields_np(256, seed=12)
    nside, steps = 64, 128
    with srt.Fields(phi, b) as f:
        m64, _ = f.forward(nside, steps, precision="fp64")
        mmx, _ = f.forward(nside, steps, precision="mixed")
    with srt.Fields(phi, b, pairs=False) as f:
        mmx1, _ = f.forward(nside, steps, precision="mixed")
    _assert_close(mmx, m64, "mixed", "mixed vs fp64 @256^3")
    _assert_close(mmx1, m64, "mixed", "mixed (single layout) vs fp64 @256^3")
    pix = np.random.default_rng(0).choice(12 * nside * nside, 96, replace=False)
    want = orc.trace_pixels(phi, b, nside, steps, pix, mode="fp64")
    _assert_close(m64[:, pix], want, "fp64", "fp64 sample @256^3")


def test_mixed_refines_face_crossing_rays(srt, orc):
    """MIXED re-traces in FP64 the rays that came within the cell-face guard:
    those rays equal the FP64 form bit for bit, the others stay within the
    FP32 tolerance, and turning the fallback off changes only listed rays."""
    phi, b = srt_fields.gaussian_fields_np(256, seed=13)
    nside, steps = 64, 256
    with srt.Fields(phi, b) as f:
        m64, _ = f.forward(nside, steps, precision="fp64")
        mr, st = f.forward(nside, steps, precision="mixed")
        mn, st0 = f.forward(nside, steps, precision="mixed", refine=False)
    assert st.refined_rays > 0 and st0.refined_rays == 0  # ~1e-3 of the rays at this size
    # the re-trace's device time is reported as its share of trace_ms
    assert 0.0 < st.retrace_ms < st.trace_ms and st0.retrace_ms == 0.0
    assert st.refined_rays < 0.01 * 12 * nside * nside
    same = np.all(mr.view(np.uint32) == m64.view(np.uint32), axis=0)
    changed = np.any(mr.view(np.uint32) != mn.view(np.uint32), axis=0)
    assert changed.sum() <= st.refined_rays   # nothing but listed rays moved
    assert np.all(same[changed])              # and those equal the FP64 form bit for bit
    # this sky holds a ray whose FP32 and FP64 trajectories pass a cell face on
    # different sides (unrefined dA error 5e-3 of the map's rms): refined, the
    # MIXED maps meet the FP32 tolerance
    _assert_close(mr, m64, "mixed", "refined mixed vs fp64")


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_nested_range_matches_ring(srt, precision):
    """SRT_NESTED_RANGE: a NESTED pixel range (here base pixel 5 and a part of
    base pixel 0) gives, pixel for pixel, the maps of the RING full sky."""
    phi, b = srt_fields.gaussian_fields_np(32, seed=12)
    nside, steps = 8, 20
    with srt.Fields(phi, b) as f:
        full, _ = f.forward(nside, steps, precision=precision)
        for begin, count in ((5 * nside * nside, nside * nside), (3, 29)):
            got, st = f.forward(nside, steps, begin, count, precision=precision, nested=True)
            assert st.rays == count
            ring = [srt.nest2ring(nside, begin + i) for i in range(count)]
            assert np.array_equal(got.view(np.uint32), full[:, ring].view(np.uint32))
        with pytest.raises(srt.SrtError):
            f.forward(6, steps, 0, 36, precision=precision, nested=True)


@pytest.mark.parametrize("lanes", [4, 1])
def test_mixed_refine_double_float_path(srt, monkeypatch, lanes):
    """Long re-trace lists run in double-float arithmetic, four lanes per ray
    (forced here with SRT_REFINE_DD_MIN=0 on a small sky) or, for the longest
    lists, one lane per ray (SRT_REFINE_WIDE_MIN=0): the re-traced rays agree
    with the FP64 form to a float ulp or two, everything else is untouched."""
    phi, b = srt_fields.gaussian_fields_np(128, seed=13)
    nside, steps = 32, 128
    with srt.Fields(phi, b) as f:
        m64, _ = f.forward(nside, steps, precision="fp64")
        mn, _ = f.forward(nside, steps, precision="mixed", refine=False)
        monkeypatch.setenv("SRT_REFINE_DD_MIN", "0")
        if lanes == 1:
            monkeypatch.setenv("SRT_REFINE_WIDE_MIN", "0")
        mr, st = f.forward(nside, steps, precision="mixed")
        monkeypatch.delenv("SRT_REFINE_DD_MIN")
        monkeypatch.delenv("SRT_REFINE_WIDE_MIN", raising=False)
    assert st.refined_rays > 0
    changed = np.any(mr.view(np.uint32) != mn.view(np.uint32), axis=0)
    assert changed.sum() <= st.refined_rays
    # float ulps between the re-traced maps and the FP64 ones
    ulps = np.abs(mr[:, changed].view(np.int32).astype(np.int64) - m64[:, changed].view(np.int32).astype(np.int64))
    assert ulps.max() <= 4, ulps.max()


def test_fields_memory_pool_reuse_and_release(srt):
    """Destroyed fields leave their memory in the library's pool, a second
    handle of the same size reuses it, and srt_release_cached_memory returns it."""
    torch = pytest.importorskip("torch")
    phi, b = srt_fields.gaussian_fields_np(64, seed=2)
    srt.release_cached_memory()  # earlier handles' memory may sit in the pool
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    with srt.Fields(phi, b) as f:
        nbytes = f.nbytes
        m1, _ = f.forward(8, 16, precision="mixed")
    held = free0 - torch.cuda.mem_get_info()[0]
    assert held >= 0.9 * nbytes  # kept by the pool
    with srt.Fields(phi, b) as f:
        m2, _ = f.forward(8, 16, precision="mixed")
        assert free0 - torch.cuda.mem_get_info()[0] <= held + (64 << 20)  # reused, not allocated again
    assert np.array_equal(m1.view(np.uint32), m2.view(np.uint32))
    srt.release_cached_memory()
    assert free0 - torch.cuda.mem_get_info()[0] <= 0.1 * nbytes + (64 << 20)


@pytest.mark.parametrize("precision", ["fp64", "mixed", "ref16"])
def test_constant_gradient_potential_analytic(srt, orc, precision):
    """Every precision against the first-order analytic maps of a
    constant-gradient potential."""
    from conftest import check_linear_phi_maps, linear_phi_case

    phi, b, predict = linear_phi_case()
    nside, S = 4, 24
    with srt.Fields(phi, b) as f:
        maps, _ = f.forward(nside, S, precision=precision)
    check_linear_phi_maps(maps, nside, S, predict, orc.pix2ang_ring)


def test_single_layout_packed_path_equals_pair_layout(srt):
    """The MIXED forward and vjp read their packed tap pairs either from the
    row-pair copy of the fields or, with SRT_FIELDS_NO_PAIRS, from the single
    halo layout (two loads per pair): the float2 values and the packed
    operations are the same, so the maps and the refined-ray counts agree bit
    for bit. The sweep's B passes form their tap cotangents and their share of
    the state cotangent from scalar FP32 expressions the compiler may round in
    a different order in the two kernel variants (one float ulp on ~0.5 % of
    the B gradient entries); that state cotangent feeds the phi scatter of the
    earlier stages, so both gradients are compared to 1e-6 of their largest
    entry."""
    import srt_fields

    phi, b = srt_fields.gaussian_fields_np(48, seed=17)
    nside, steps = 16, 48
    w = np.random.default_rng(5).standard_normal((6, 12 * nside * nside)).astype(np.float32)
    out = {}
    for pairs in (True, False):
        with srt.Fields(phi, b, pairs=pairs) as f:
            m, st = f.forward(nside, steps, precision="mixed")
            g, gb, _ = f.vjp(nside, steps, w, precision="mixed", deterministic=True, ckpt_every=7)
            out[pairs] = (m, st.refined_rays, g, gb)
    assert np.array_equal(out[True][0].view(np.uint32), out[False][0].view(np.uint32))
    assert out[True][1] == out[False][1]
    for k in (2, 3):
        a, c = out[True][k], out[False][k]
        err = np.abs(a - c).max() / np.abs(a).max()
        assert err <= 1e-6, ("phi" if k == 2 else "B", err)


@pytest.mark.parametrize("extents", [(24, 24, 24), (5, 3, 4)])
def test_pinned_host_inputs_read_in_place_equal_staged(srt, orc, extents):
    """Host fields in pinned (mapped) memory are laid out by the kernel reading
    them over the host link; pageable ones, or pinned ones with
    SRT_FIELDS_STAGED, go through a device slab. All three give the same
    padded fields: the FP64 maps agree bit for bit with each other and with the
    oracle, on a cube and on a small non-cubic grid whose rays wrap around the
    box many times (every halo copy is read)."""
    torch = pytest.importorskip("torch")
    import srt_fields

    phi, b = srt_fields.int_noise_fields(extents, seed=8)
    pphi = torch.empty(phi.shape, dtype=torch.float32, pin_memory=True)
    pb = torch.empty(b.shape, dtype=torch.float32, pin_memory=True)
    pphi.numpy()[...] = phi
    pb.numpy()[...] = b
    nside, steps = 2, 20
    want = orc.trace(phi, b, nside, steps, mode="fp64")
    got = []
    for src, staged in ((pphi.numpy(), False), (pphi.numpy(), True), (phi, False)):
        bsrc = pb.numpy() if src is not phi else b
        with srt.Fields(src, bsrc, staged=staged) as f:
            got.append(f.forward(nside, steps, precision="fp64")[0])
    for g in got:
        assert np.array_equal(g.view(np.uint32), got[0].view(np.uint32))
    for m, (rms, mx) in enumerate(map_errors(got[0], want)):
        assert rms <= 1e-9 and mx <= 1e-8, (m, rms, mx)


def test_async_staged_upload_overlapping_a_trace(srt):
    """The pipelined use: fields created with SRT_ASYNC on one stream (host
    input through one staging buffer, no host synchronisation) while another
    handle traces on a second stream; after an event the new handle traces.
    The maps equal those of a synchronous create, bit for bit."""
    torch = pytest.importorskip("torch")
    import srt_fields

    phi, b = srt_fields.gaussian_fields_np(40, seed=23)
    pphi = torch.empty(phi.shape, dtype=torch.float32, pin_memory=True)
    pb = torch.empty(b.shape, dtype=torch.float32, pin_memory=True)
    pphi.numpy()[...] = phi
    pb.numpy()[...] = b
    nside, steps = 8, 30
    with srt.Fields(phi, b) as f:
        want, _ = f.forward(nside, steps, precision="mixed")
    s_up = torch.cuda.Stream(priority=-1)
    s_tr = torch.cuda.Stream()
    with srt.Fields(pphi.numpy(), pb.numpy()) as busy:
        out_busy = torch.empty((6, 12 * nside * nside), dtype=torch.float32, device="cuda")
        busy.forward(nside, steps, precision="mixed", out=out_busy, stream=s_tr, async_=True)
        nxt = srt.Fields(pphi.numpy(), pb.numpy(), stream=s_up, async_=True, staged=True)
        ev = torch.cuda.Event()
        ev.record(s_up)
        s_tr.wait_event(ev)
        got = np.zeros_like(want)
        nxt.forward(nside, steps, precision="mixed", out=got, stream=s_tr)
        nxt.close()
        torch.cuda.synchronize()
        assert np.array_equal(out_busy.cpu().numpy().view(np.uint32), want.view(np.uint32))
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
