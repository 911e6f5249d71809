#!/bin/sh
# Compile the reference's own host code for the tracer's path into
# oracle/_ref/libsrt_ref.so (test infrastructure: golden vectors and the pin of
# the oracle). Reads the reference sources where they lie; writes only into
# oracle/_ref/. Usage: oracle/build_ref.sh [REFERENCE_DIR]
# The reference directory is the argument, else $SRT_REFERENCE_DIR, else the
# read-only mount this recipe was written for (/root/reference). Exit status 3
# (and a message) when none of them holds snapshot-raytracer.cu.
set -e
REF=${1:-${SRT_REFERENCE_DIR:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
[ -f "$REF/snapshot-raytracer.cu" ] || {
  echo "oracle/build_ref.sh: no reference sources in '$REF' (pass the directory holding snapshot-raytracer.cu or set SRT_REFERENCE_DIR); oracle/_ref not built" >&2
  exit 3
}
mkdir -p "$HERE/_ref"
# Reference flags (Makefile:9-10,33): -O3 --use_fast_math -std=c++17 -fopenmp;
# one Blackwell gencode for its device code, which the library never launches.
nvcc -O3 --use_fast_math -std=c++17 -shared -Xcompiler -fopenmp,-fPIC,-ffp-contract=off \
  -gencode arch=compute_103a,code=sm_103a -w \
  -I"$HERE/stubs" -I"$REF" "$HERE/ref_harness.cu" -o "$HERE/_ref/libsrt_ref.so"
# The reference's own device code as a cubin (vector3_to_half, raytracing_kernel),
# launched by oracle/ref_gpu.cu to time the reference's GPU build on the same GPU.
nvcc -cubin -O3 --use_fast_math -std=c++17 -gencode arch=compute_103a,code=sm_103a -w \
  -I"$HERE/stubs" -I"$REF" "$HERE/ref_gpu_unit.cu" -o "$HERE/_ref/ref_kernel.cubin"
