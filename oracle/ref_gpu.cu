// ref_gpu.cu — loader for the reference's own GPU build
// (oracle/_ref/ref_kernel.cubin, made from the reference source by
// oracle/build_ref.sh). BASELINE AND TEST INFRASTRUCTURE, used only by
// tests/ and bench.py's reference measurements, never by the product.
//
// srtrefgpu_trace stages the inputs and launches the reference's kernels the
// way its main() does (snapshot-raytracer.cu:774-898): B quantised to three
// FP16 planes by the reference's vector3_to_half, one chunk of N^3 floats per
// launch with grid (ceil(d1*d2/128), d0) x 128 threads; then
// raytracing_kernel with 128 threads per block over the ray list, given
// theta/phi of the RING pixels (the reference computes them on the host with
// chealpix, :857-866). The only difference: the B chunks are read in place
// from the caller's device array instead of being copied through a staging
// buffer first. Outputs are the reference's batch-relative maps [6][nrays].
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdarg.h>
#include <mutex>
#include <vector>
#include <algorithm>

namespace {

// Itanium-mangled names of the reference kernels (snapshot-raytracer.cu:552, :585),
// as nvcc -Xptxas -v reports them for the compiled entry functions.
const char* kTraceName = "_Z17raytracing_kernelPKfPK6__halfS3_S3_PKilliPdS6_PfS7_S7_S7_S7_S7_";
const char* kHalfName = "_Z15vector3_to_halfPKfP6__halfS2_S2_lll";

std::mutex g_mu;
cudaLibrary_t g_lib = nullptr;
cudaKernel_t g_trace = nullptr, g_half = nullptr;

int fail(char* err, size_t n, const char* fmt, ...) {
  if (err && n) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(err, n, fmt, ap);
    va_end(ap);
  }
  return -1;
}

struct Dev {
  void* p = nullptr;
  ~Dev() {
    if (p) cudaFree(p);
  }
};

}  // namespace

extern "C" int srtrefgpu_load(const char* cubin, char* err, size_t errlen) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_lib) return 0;
  cudaError_t e = cudaLibraryLoadFromFile(&g_lib, cubin, nullptr, nullptr, 0, nullptr, nullptr, 0);
  if (e != cudaSuccess) {
    g_lib = nullptr;
    return fail(err, errlen, "cudaLibraryLoadFromFile(%s): %s", cubin, cudaGetErrorString(e));
  }
  e = cudaLibraryGetKernel(&g_trace, g_lib, kTraceName);
  if (e == cudaSuccess) e = cudaLibraryGetKernel(&g_half, g_lib, kHalfName);
  if (e != cudaSuccess) {
    cudaLibraryUnload(g_lib);
    g_lib = nullptr;
    return fail(err, errlen, "reference kernels not found in %s: %s", cubin, cudaGetErrorString(e));
  }
  return 0;
}

// phi: device float[n0*n1*n2] (x fastest); b_xyz: device float[3*n0*n1*n2]
// interleaved; theta/phiang: host doubles [nrays]; maps: device float[6*nrays].
// Runs `reps` launches of raytracing_kernel; ms[r] is each launch's time.
extern "C" int srtrefgpu_trace(const float* phi, const float* b_xyz, int n0, int n1, int n2, const double* theta,
                               const double* phiang, int64_t nrays, int64_t nside, int n_steps, float* maps, int reps,
                               float* ms, char* err, size_t errlen) {
  if (!g_lib) return fail(err, errlen, "reference cubin not loaded");
  if (n0 < 4 || n1 < 4 || n2 < 4 || nrays < 1 || n_steps < 1 || reps < 1 || !phi || !b_xyz || !maps)
    return fail(err, errlen, "invalid arguments");
  // The reference wraps indices with (i + 20 n) % n (:241-256): positions must
  // stay above -19 n. A ray moves about one grid unit per step from n/2.
  const int nmin = std::min(n0, std::min(n1, n2));
  if ((int64_t)n_steps + 2 > 19LL * nmin) return fail(err, errlen, "n_steps %d too large for grid side %d", n_steps, nmin);
  const int64_t nv = (int64_t)n0 * n1 * n2;
  Dev h1, h2, h3, dims, th, ph;
  cudaError_t e = cudaSuccess;
  for (Dev* d : {&h1, &h2, &h3})
    if (e == cudaSuccess) e = cudaMalloc(&d->p, nv * 2);
  if (e == cudaSuccess) e = cudaMalloc(&dims.p, 3 * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&th.p, nrays * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&ph.p, nrays * sizeof(double));
  if (e != cudaSuccess) return fail(err, errlen, "cudaMalloc: %s", cudaGetErrorString(e));
  const int dims_h[3] = {n0, n1, n2};
  e = cudaMemcpy(dims.p, dims_h, sizeof(dims_h), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(th.p, theta, nrays * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(ph.p, phiang, nrays * sizeof(double), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return fail(err, errlen, "cudaMemcpy: %s", cudaGetErrorString(e));
  // B -> three FP16 planes, one chunk of nv floats per launch (:781-836)
  const int64_t xy = (int64_t)n1 * n2;
  const int tpb = 128;
  const dim3 hgrid((unsigned)((xy + tpb - 1) / tpb), (unsigned)n0);
  for (int c = 0; c < 3; ++c) {
    const float* chunk = b_xyz + c * nv;
    int64_t n = nv, off = c * nv;
    void* args[] = {(void*)&chunk, &h1.p, &h2.p, &h3.p, &n, (void*)&xy, &off};
    e = cudaLaunchKernel((const void*)g_half, hgrid, dim3(tpb), args, 0, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return fail(err, errlen, "vector3_to_half: %s", cudaGetErrorString(e));
  }
  float* out[6];
  for (int m = 0; m < 6; ++m) out[m] = maps + m * nrays;
  const int64_t iend = nrays;
  int steps = n_steps;
  void* targs[] = {(void*)&phi, &h1.p, &h2.p, &h3.p, &dims.p, &nside, (void*)&iend, &steps, &th.p, &ph.p,
                   &out[0], &out[1], &out[2], &out[3], &out[4], &out[5]};
  const dim3 grid((unsigned)((nrays + tpb - 1) / tpb));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  for (int r = 0; r < reps && e == cudaSuccess; ++r) {
    cudaEventRecord(e0, 0);
    e = cudaLaunchKernel((const void*)g_trace, grid, dim3(tpb), targs, 0, 0);
    cudaEventRecord(e1, 0);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess && ms) cudaEventElapsedTime(&ms[r], e0, e1);
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return fail(err, errlen, "raytracing_kernel: %s", cudaGetErrorString(e));
  return 0;
}
