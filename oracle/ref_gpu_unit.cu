// ref_gpu_unit.cu — the reference's OWN device code, compiled unmodified from
// where it lies in the reference tree (snapshot-raytracer.cu) into a cubin,
// oracle/_ref/ref_kernel.cubin, by oracle/build_ref.sh. BASELINE AND TEST
// INFRASTRUCTURE: oracle/ref_gpu.cu loads the cubin and launches the
// reference's vector3_to_half (:585-597) and raytracing_kernel (:552-583) as
// its main() does (:774-898), to time the reference's own GPU build on the
// same GPU and to compare its maps with ours. Nothing of the product links it.
// Reference flags (Makefile:9-10): -O3 --use_fast_math -std=c++17, with one
// GB300 gencode in place of the Makefile's ARCH list.
#define main srt_reference_cli_main
#include "snapshot-raytracer.cu"
#undef main
