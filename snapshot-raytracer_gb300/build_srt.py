"""Build recipe of the tracer: libsrt.so (CUDA kernels for sm_103a + C ABI +
host file formats), the `snapshot-raytracer` CLI, and the CPU oracle used by
the tests (oracle/liboracle.so, plus oracle/_ref/libsrt_ref.so when the
reference sources are present on this machine).

Everything is built in-tree with explicit nvcc / g++ / gcc commands, compiled
in parallel. Usage: python snapshot-raytracer_gb300/build_srt.py [-v]
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIBSRT = os.path.join(LIBDIR, "libsrt.so")
CLI = os.path.join(PKG, "snapshot-raytracer")
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIBORACLE = os.path.join(ORACLE_DIR, "liboracle.so")
LIBREF = os.path.join(ORACLE_DIR, "_ref", "libsrt_ref.so")
LIBREFGPU = os.path.join(ORACLE_DIR, "librefgpu.so")
REFCUBIN = os.path.join(ORACLE_DIR, "_ref", "ref_kernel.cubin")

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
CUDA_SOURCES = ["srt_kernels.cu", "srt_adjoint.cu", "srt_api.cu", "srt_noalloc.cu"]
HOST_SOURCES = ["srt_io.cpp"]


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed (%d): %s\n%s" % (r.returncode, " ".join(cmd), r.stdout))
    if verbose and r.stdout.strip():
        print(r.stdout, flush=True)
    return r.stdout


def _nvcc_obj(src, verbose):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    # --use_fast_math (as the reference is built, Makefile:9) touches FP32 only:
    # approximate division and square root, denormals flushed. The MIXED form's
    # error-free transformations (two-sum, FMA two-product) are exact either way,
    # and the FP64 form is unaffected.
    cmd = [NVCC, *GENCODE, "-lineinfo", "-O3", "--use_fast_math", "-std=c++17", "-Xcompiler", "-fPIC",
           "-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "-c", src, "-o", obj]
    # extra nvcc flags, e.g. -DSRT_MIXED_MIN_BLOCKS=3 to compile the MIXED trace
    # for three resident blocks per SM
    cmd[1:1] = os.environ.get("SRT_NVCC_FLAGS", "").split()
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    _run(cmd, verbose)
    return obj


def _gxx_obj(src, verbose):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    cuda_home = os.path.dirname(os.path.dirname(shutil.which(NVCC) or "/usr/local/cuda/bin/nvcc"))
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-pthread", "-Wall", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC,
           "-I" + os.path.join(cuda_home, "include"), "-c", src, "-o", obj]
    _run(cmd, verbose)
    return obj


def build_oracle(verbose=False):
    """The CPU oracle (test infrastructure): the C restatement and its
    dual-number tangent, no FMA contraction."""
    os.makedirs(BUILD, exist_ok=True)
    o1 = os.path.join(BUILD, "srt_oracle.o")
    o2 = os.path.join(BUILD, "srt_oracle_tangent.o")
    _run(["gcc", "-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fPIC", "-c",
          os.path.join(ORACLE_DIR, "srt_oracle.c"), "-o", o1], verbose)
    _run(["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-c",
          os.path.join(ORACLE_DIR, "srt_oracle_tangent.cpp"), "-o", o2], verbose)
    _run(["g++", "-shared", "-fopenmp", "-o", LIBORACLE, o1, o2, "-lm"], verbose)
    # loader of the reference's own GPU build (the cubin comes from build_ref.sh)
    _run([NVCC, *GENCODE, "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC",
          os.path.join(ORACLE_DIR, "ref_gpu.cu"), "-o", LIBREFGPU], verbose)
    return LIBORACLE


def build_reference(verbose=False):
    """The reference's own host code and device code for the path, compiled by
    oracle/build_ref.sh from the reference sources (SRT_REFERENCE_DIR, or the
    directory that recipe names); skipped, with the recipe's message, where the
    sources are absent (e.g. on the GPU machine, which runs the files built here)."""
    cmd = ["sh", os.path.join(ORACLE_DIR, "build_ref.sh")]
    if os.environ.get("SRT_REFERENCE_DIR"):
        cmd.append(os.environ["SRT_REFERENCE_DIR"])
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode == 3:  # the recipe found no reference sources
        if verbose:
            print(r.stdout.strip(), flush=True)
        return None
    if r.returncode != 0:
        raise RuntimeError("build step failed (%d): %s\n%s" % (r.returncode, " ".join(cmd), r.stdout))
    return LIBREF


def build(verbose=False, oracle=True, reference=True):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    jobs = []
    with concurrent.futures.ThreadPoolExecutor(max_workers=8) as ex:
        for s in CUDA_SOURCES:
            jobs.append(ex.submit(_nvcc_obj, os.path.join(CSRC, s), verbose))
        for s in HOST_SOURCES:
            jobs.append(ex.submit(_gxx_obj, os.path.join(CSRC, s), verbose))
        side = []
        if oracle:
            side.append(ex.submit(build_oracle, verbose))
        if reference:
            side.append(ex.submit(build_reference, verbose))
        objs = [j.result() for j in jobs]
        _run([NVCC, *GENCODE, "-shared", "-o", LIBSRT, *objs, "-lpthread"], verbose)
        cli_src = os.path.join(CSRC, "srt_cli.cpp")
        if os.path.isfile(cli_src):
            _run(["g++", "-O2", "-std=c++17", "-Wall", "-pthread", "-I" + os.path.join(ROOT, "include"), cli_src,
                  "-o", CLI, "-L" + LIBDIR, "-lsrt", "-Wl,-rpath,$ORIGIN/lib"], verbose)
        for j in side:
            j.result()
    return LIBSRT


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print("built", LIBSRT)
