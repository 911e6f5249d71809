// srt_adjoint.cu — vjp of the six maps with respect to the phi and B grids
// (srt_vjp in include/srt.h). The reference has no derivatives; what is
// differentiated is its forward scheme, snapshot-raytracer.cu:315-583, as
// restated in srt_scheme.cuh.
//
// Kernels (one thread per ray, rays in the forward's launch order):
//   ray_count_kernel / ray_write_kernel  Morton-ordered list of the RING pixels
//                                        of the requested range
//   ckpt_kernel<MODE>      forward trace storing the state every C steps
//                          (and the final state) in device memory
//   reverse_kernel<MODE>   per segment, backwards: recompute the segment from
//                          its checkpoint storing y_i, k1, k2, k3 per step;
//                          then per step, backwards, the RK4 adjoint
//                            a4 = J(u4)^T l/6, a3 = J(u3)^T (l/3 + a4),
//                            a2 = J(u2)^T (l/3 + a3/2), a1 = J(u1)^T (l/6 + a2/2),
//                            l <- l + a1 + a2 + a3 + a4,
//                          scattering the tap cotangents into halo-padded
//                          gradient grids (FP32 atomics, FP64 atomics, or
//                          64-bit fixed point for SRT_DETERMINISTIC)
//   fold_kernel            sums the halo copies of each voxel back onto the
//                          periodic grid and writes the caller's layout
#include <algorithm>
#include <chrono>
#include <cstring>
#include <vector>
#include "srt_adjoint.cuh"
#include "srt_internal.h"

namespace srt {

// ------------------------------------------------------------- ray list

struct RangeArgs {
  int64_t nside, pix_begin, pix_count, launch_rays;
  int log2p;
};

__device__ __forceinline__ int64_t ring_of_slot(const RangeArgs& a, int64_t t) {
  if (t >= a.launch_rays) return -1;
  const int64_t face = t >> (2 * a.log2p);
  int64_t ix, iy;
  hp_deinterleave(t & ((int64_t(1) << (2 * a.log2p)) - 1), &ix, &iy);
  if (ix >= a.nside || iy >= a.nside) return -1;
  const int64_t ring = hp_xyf2ring(a.nside, ix, iy, (int)face);
  return (ring >= a.pix_begin && ring < a.pix_begin + a.pix_count) ? ring : -1;
}

constexpr int kListBlock = 256;

__global__ void ray_count_kernel(const RangeArgs a, int* counts) {
  const int64_t t = (int64_t)blockIdx.x * kListBlock + threadIdx.x;
  const int in = ring_of_slot(a, t) >= 0;
  const int c = __syncthreads_count(in);
  if (threadIdx.x == 0) counts[blockIdx.x] = c;
}

__global__ void ray_write_kernel(const RangeArgs a, const int64_t* offsets, int64_t* rays) {
  __shared__ int warp_tot[kListBlock / 32];
  const int64_t t = (int64_t)blockIdx.x * kListBlock + threadIdx.x;
  const int64_t ring = ring_of_slot(a, t);
  const unsigned mask = __ballot_sync(0xffffffffu, ring >= 0);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) warp_tot[warp] = __popc(mask);
  __syncthreads();
  int before = 0;
  for (int w = 0; w < warp; ++w) before += warp_tot[w];
  if (ring >= 0) rays[offsets[blockIdx.x] + before + __popc(mask & ((1u << lane) - 1u))] = ring;
}

// ------------------------------------------------------------ arguments

struct AdjArgs {
  FieldPtrs F;
  Geom G;
  int64_t nside, pix_begin, count;
  const int64_t* rays;
  int n_steps, C, nseg;
  const float* w[6];  // map weights, indexed by ring - pix_begin
  void* ckpt;         // [nseg + 1][state][count]
  void* seg;          // [C][state + 57][count]
  void* acc[4];       // padded gradient accumulators B_x, B_y, B_z, phi (NULL: not wanted)
  // forward with a tape (srt_forward_tape): the maps, indexed by ring - pix_begin,
  // and the output slots of rays that came within the cell-face guard
  float* maps[6];
  int64_t* refine_list;
  unsigned long long* refine_count;
};

template <typename T>
__device__ __forceinline__ void store_vec(T* base, int64_t count, int64_t slot, const T* v, int n) {
  for (int j = 0; j < n; ++j) base[(int64_t)j * count + slot] = v[j];
}
template <typename T>
__device__ __forceinline__ void load_vec(const T* base, int64_t count, int64_t slot, T* v, int n) {
  for (int j = 0; j < n; ++j) v[j] = base[(int64_t)j * count + slot];
}

// ------------------------------------------------------------ MIXED mode


// Floats of one step of the MIXED tape: the four stage inputs.
constexpr int kTapeStep = 4 * 19;

// PAIR: the forward steps read the row-pair field arrays (srt_fields.pr).
// Forward trace storing the state every C steps (and the final state). MAPS
// (srt_forward_tape): also the maps, with the cell-face guard of the trace
// kernel and its list of rays to re-trace; the arithmetic is the trace
// kernel's, so the maps are srt_forward's.
template <bool PAIR, bool MAPS>
__global__ void __launch_bounds__(128, MAPS ? 2 : 1) ckpt_kernel_mixed(const AdjArgs A) {
  const int64_t slot = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= A.count) return;
  const int64_t ring = A.rays[slot];
  const RayDir d = ray_dir_pix(A.nside, ring);
  MixedRay R;
  float y[kMixedState], x0[3];
  mixed_observer(A.G, x0);
  init_mixed(d, R, y);
  float* ck = (float*)A.ckpt;
  store_vec(ck, A.count, slot, y, kMixedState);
  // MAPS: the guard of the trace kernel; else disabled (cell-face proximity
  // matters for the maps, not for the gradient)
  __shared__ float guard_m[MAPS ? 128 : 1][2];
  Guard gd;
  if (MAPS) {
    gd.m = guard_m[threadIdx.x];
    gd.m[0] = 0.f;
  }
#pragma unroll 1
  for (int st = 0; st < A.n_steps; ++st) {
    if (MAPS) gd.begin_step(y);
    step_mixed<PAIR>(R, A.F, A.G, x0, st, y, nullptr, 0, gd);
    if (MAPS) gd.end_step(st);
    const int done = st + 1;
    if (done % A.C == 0 || done == A.n_steps) {
      const int k = (done + A.C - 1) / A.C;
      store_vec(ck + (int64_t)k * kMixedState * A.count, A.count, slot, y, kMixedState);
    }
  }
  if (MAPS) {
    const int64_t o = ring - A.pix_begin;
    float out[6];
    extract_mixed(R, A.n_steps, y, out);
#pragma unroll
    for (int m = 0; m < 6; ++m) A.maps[m][o] = out[m];
    if (gd.near && A.refine_list) {
      const unsigned long long k = atomicAdd(A.refine_count, 1ull);
      if (k < (unsigned long long)A.count) A.refine_list[k] = o;
    }
  }
}

// Cotangent of the final state from the map weights (the transpose of
// extract_mixed) -> lam [19][count].
__global__ void __launch_bounds__(128) final_cotangent_kernel_mixed(const AdjArgs A, float* lam) {
  const int64_t slot = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= A.count) return;
  const int64_t ring = A.rays[slot];
  const int64_t o = ring - A.pix_begin;
  const RayDir d = ray_dir_pix(A.nside, ring);
  MixedRay R;
  float y[kMixedState];
  init_mixed(d, R, y);
  load_vec((const float*)A.ckpt + (int64_t)A.nseg * kMixedState * A.count, A.count, slot, y, kMixedState);
  float l[19];
  for (int j = 0; j < 19; ++j) l[j] = 0.f;
  float w[6];
  for (int m = 0; m < 6; ++m) w[m] = A.w[m][o];
  l[12] = w[0];
  l[16] = w[1];
  l[17] = w[2];
  l[18] = w[3];
  const float S = (float)A.n_steps;
  float u[3];
  for (int i = 0; i < 3; ++i) u[i] = (y[i] + y[19 + i]) / S;
  const float q = R.eta[0] - 2.f * (R.n0[0] * u[0] + R.n0[1] * u[1] + R.n0[2] * u[2]) +
                  (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
  const float c = rsqrt1p_m1(q);
  const float r3 = (1.f + c) * (1.f + c) * (1.f + c);  // (1 + q)^(-3/2)
  float Db[3], um[3];
  for (int i = 0; i < 3; ++i) {
    Db[i] = w[4] * R.a0[i] + w[5] * R.b0[i];
    um[i] = u[i] - R.n0[i];
  }
  const float dotv = um[0] * Db[0] + um[1] * Db[1] + um[2] * Db[2];
  for (int i = 0; i < 3; ++i) l[i] = ((1.f + c) * Db[i] - dotv * r3 * um[i]) / S;
  store_vec(lam, A.count, slot, l, 19);
}

// Recompute segment sgi from its checkpoint, storing the four stage inputs
// of every step: tape [C][4 x 19][count].
template <bool PAIR>
__global__ void __launch_bounds__(128, 2) segment_kernel_mixed(const AdjArgs A, int sgi) {
  const int64_t slot = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= A.count) return;
  const RayDir d = ray_dir_pix(A.nside, A.rays[slot]);
  MixedRay R;
  float y[kMixedState], x0[3];
  mixed_observer(A.G, x0);
  init_mixed(d, R, y);
  const int s0 = sgi * A.C, s1 = min(s0 + A.C, A.n_steps);
  load_vec((const float*)A.ckpt + (int64_t)sgi * kMixedState * A.count, A.count, slot, y, kMixedState);
  float* tape = (float*)A.seg;
#pragma unroll 1
  for (int st = s0; st < s1; ++st) {
    Guard gd;  // disabled
    step_mixed<PAIR>(R, A.F, A.G, x0, st, y, tape + (int64_t)(st - s0) * kTapeStep * A.count + slot, A.count, gd);
  }
}

// Backward sweep over segment sgi: per step, backwards, the RK4 adjoint
//   a4 = J(u4)^T l/6, a3 = J(u3)^T (l/3 + a4), a2 = J(u2)^T (l/3 + a3/2),
//   a1 = J(u1)^T (l/6 + a2/2), l <- l + a1 + a2 + a3 + a4,
// with the stage inputs u from the tape (the next stage's inputs are loaded
// while the current stage runs); l carried in lam between segments. l and the
// running sum of the a's live in shared memory (one column per thread) to keep
// registers for the field passes.
template <typename AccB, typename AccP, bool PAIR>
__device__ __forceinline__ void sweep_segment(const AdjArgs& A, int sgi, int64_t slot, const MixedRay& R,
                                              const float* x0, float* lam, const AccB* accb, const AccP& accp,
                                              float (*s_lam)[128], float (*s_tot)[128]) {
  const int t = threadIdx.x;
  for (int j = 0; j < 19; ++j) s_lam[j][t] = lam[(int64_t)j * A.count + slot];
  const float* tape = (const float*)A.seg + slot;
  const int s0 = sgi * A.C, s1 = min(s0 + A.C, A.n_steps);
  // flattened (step, stage) index, descending; u holds the stage inputs of q
  int q = (s1 - s0) * 4 - 1;
  float u[19];
  for (int j = 0; j < 19; ++j) u[j] = ld_stream(tape + ((int64_t)(q >> 2) * kTapeStep + 19 * (q & 3) + j) * A.count);
  float an[19];  // a of the stage after this one (finite; its weight is 0 at stage 3)
  for (int j = 0; j < 19; ++j) an[j] = 0.f;
#pragma unroll 1
  for (; q >= 0; --q) {
    const int st = s0 + (q >> 2), stage = q & 3;
    const float c = (stage == 0) ? 0.f : ((stage == 3) ? 1.f : 0.5f);
    const float wl = (stage == 0 || stage == 3) ? (1.f / 6.f) : (1.f / 3.f);
    const float wa = (stage == 3) ? 0.f : ((stage == 2) ? 1.f : 0.5f);
    float fb[19];
    for (int j = 0; j < 19; ++j) fb[j] = wl * s_lam[j][t] + wa * an[j];
    StageView<float> V;
    stage_view_mixed(u, (float)st + c, R, A.G, x0, V);
    {  // prefetch the next (earlier) stage's inputs (the last stage reloads its own)
      const int qn = q > 0 ? q - 1 : 0;
      for (int j = 0; j < 19; ++j) u[j] = ld_stream(tape + ((int64_t)(qn >> 2) * kTapeStep + 19 * (qn & 3) + j) * A.count);
    }
    for (int j = 0; j < 19; ++j) an[j] = 0.f;
    rhs_vjp<float, AccB, AccP, PAIR>(V, A.F, A.G, fb, an, accb, accp);
    // the step's running sum of the a's restarts at its last stage
    for (int j = 0; j < 19; ++j) s_tot[j][t] = (stage == 3 ? 0.f : s_tot[j][t]) + an[j];
    if (stage == 0)
      for (int j = 0; j < 19; ++j) s_lam[j][t] += s_tot[j][t];
  }
  for (int j = 0; j < 19; ++j) lam[(int64_t)j * A.count + slot] = s_lam[j][t];
}

// Resident blocks of 128 threads per SM the sweep is compiled for (register
// budget 65536 / (128 * blocks)).
#ifndef SRT_SWEEP_MIN_BLOCKS
#define SRT_SWEEP_MIN_BLOCKS 2
#endif

// BGRAD: the B gradient is wanted (else the B passes are compiled without a
// scatter).
template <typename Acc, bool PAIR, bool BGRAD>
__global__ void __launch_bounds__(128, SRT_SWEEP_MIN_BLOCKS) sweep_kernel_mixed(const AdjArgs A, int sgi, float* lam, const Acc a0,
                                                           const Acc a1, const Acc a2, const Acc a3) {
  __shared__ float s_lam[19][128];
  __shared__ float s_tot[19][128];
  const int64_t slot = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= A.count) return;
  typedef typename std::conditional<BGRAD, Acc, AccNone>::type AccB;
  AccB accb[3];
  if constexpr (BGRAD) {
    accb[0] = a0;
    accb[1] = a1;
    accb[2] = a2;
  }
  const RayDir d = ray_dir_pix(A.nside, A.rays[slot]);
  MixedRay R;
  float x0[3];
  {
    float y[kMixedState];
    init_mixed(d, R, y);
  }
  mixed_observer(A.G, x0);
  sweep_segment<AccB, Acc, PAIR>(A, sgi, slot, R, x0, lam, accb, a3, s_lam, s_tot);
}

template <typename Acc>
void launch_sweep(const AdjArgs& A, int sgi, float* lam, const Acc* a, bool pair, bool bgrad, unsigned blocks,
                  cudaStream_t s) {
  if (pair && bgrad)
    sweep_kernel_mixed<Acc, true, true><<<blocks, 128, 0, s>>>(A, sgi, lam, a[0], a[1], a[2], a[3]);
  else if (pair)
    sweep_kernel_mixed<Acc, true, false><<<blocks, 128, 0, s>>>(A, sgi, lam, a[0], a[1], a[2], a[3]);
  else if (bgrad)
    sweep_kernel_mixed<Acc, false, true><<<blocks, 128, 0, s>>>(A, sgi, lam, a[0], a[1], a[2], a[3]);
  else
    sweep_kernel_mixed<Acc, false, false><<<blocks, 128, 0, s>>>(A, sgi, lam, a[0], a[1], a[2], a[3]);
}

// ------------------------------------------------------------- FP64 mode

__global__ void __launch_bounds__(128) ckpt_kernel_fp64(const AdjArgs A) {
  const int64_t slot = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= A.count) return;
  const RayDir d = ray_dir_pix(A.nside, A.rays[slot]);
  double y[19];
  init_std(d, A.G, y);
  double* ck = (double*)A.ckpt;
  store_vec(ck, A.count, slot, y, 19);
#pragma unroll 1
  for (int st = 0; st < A.n_steps; ++st) {
    step_std<kFP64>(A.F, A.G, y, nullptr);
    const int done = st + 1;
    if (done % A.C == 0 || done == A.n_steps) {
      const int k = (done + A.C - 1) / A.C;
      store_vec(ck + (int64_t)k * 19 * A.count, A.count, slot, y, 19);
    }
  }
}

template <typename Acc>
__global__ void __launch_bounds__(128) reverse_kernel_fp64(const AdjArgs A, const Acc a0, const Acc a1,
                                                          const Acc a2, const Acc a3) {
  const int64_t slot = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= A.count) return;
  const Acc acc[4] = {a0, a1, a2, a3};
  const int64_t ring = A.rays[slot];
  const int64_t o = ring - A.pix_begin;
  const RayDir d = ray_dir_pix(A.nside, ring);
  const double* ck = (const double*)A.ckpt;
  double* sg = (double*)A.seg;
  constexpr int kSeg = 19 + 57;
  double y[19], lam[19];
  {
    load_vec(ck + (int64_t)A.nseg * 19 * A.count, A.count, slot, y, 19);
    for (int j = 0; j < 19; ++j) lam[j] = 0.0;
    double w[6];
    for (int m = 0; m < 6; ++m) w[m] = A.w[m][o];
    lam[12] = w[0];
    lam[16] = w[1];
    lam[17] = w[2];
    lam[18] = w[3];
    // deflection = (X/|X| - r_hat) . (e_theta, e2): Xb = (I - X^ X^T) Db / |X|
    double X[3];
    for (int i = 0; i < 3; ++i) X[i] = y[i] - (double)A.G.n[i] * 0.5;
    const double nrm = sqrt(X[0] * X[0] + X[1] * X[1] + X[2] * X[2]);
    const double Db[3] = {w[4] * d.ct * d.cp + w[5] * d.sp, w[4] * d.ct * d.sp - w[5] * d.cp, -w[4] * d.st};
    const double xd = (X[0] * Db[0] + X[1] * Db[1] + X[2] * Db[2]) / nrm;
    for (int i = 0; i < 3; ++i) lam[i] = (Db[i] - X[i] / nrm * xd) / nrm;
  }
#pragma unroll 1
  for (int sgi = A.nseg - 1; sgi >= 0; --sgi) {
    const int s0 = sgi * A.C, s1 = min(s0 + A.C, A.n_steps);
    load_vec(ck + (int64_t)sgi * 19 * A.count, A.count, slot, y, 19);
#pragma unroll 1
    for (int st = s0; st < s1; ++st) {
      double* rec = sg + (int64_t)(st - s0) * kSeg * A.count;
      store_vec(rec, A.count, slot, y, 19);
      double ks[57];
      step_std<kFP64>(A.F, A.G, y, ks);
      store_vec(rec + (int64_t)19 * A.count, A.count, slot, ks, 57);
    }
#pragma unroll 1
    for (int st = s1 - 1; st >= s0; --st) {
      const double* rec = sg + (int64_t)(st - s0) * kSeg * A.count;
      double yi[19], anext[19], atot[19];
      load_vec(rec, A.count, slot, yi, 19);
      for (int j = 0; j < 19; ++j) atot[j] = 0.0;
#pragma unroll 1
      for (int stage = 3; stage >= 0; --stage) {
        double u[19], fb[19];
        const double c = (stage == 0) ? 0.0 : ((stage == 3) ? 1.0 : 0.5);
        if (stage == 0) {
          for (int j = 0; j < 19; ++j) u[j] = yi[j];
        } else {
          double kprev[19];
          load_vec(rec + (int64_t)(19 + 19 * (stage - 1)) * A.count, A.count, slot, kprev, 19);
          for (int j = 0; j < 19; ++j) u[j] = yi[j] + c * kprev[j];
        }
        const double wl = (stage == 0 || stage == 3) ? (1.0 / 6.0) : (1.0 / 3.0);
        const double wa = (stage == 3) ? 0.0 : ((stage == 2) ? 1.0 : 0.5);
        for (int j = 0; j < 19; ++j) fb[j] = wl * lam[j] + (stage == 3 ? 0.0 : wa * anext[j]);
        StageView<double> V;
        stage_view_fp64(u, A.G, V);
        double ub[19];
        for (int j = 0; j < 19; ++j) ub[j] = 0.0;
        rhs_vjp<double, Acc, Acc>(V, A.F, A.G, fb, ub, acc, acc[3]);
        for (int j = 0; j < 19; ++j) {
          anext[j] = ub[j];
          atot[j] += ub[j];
        }
      }
      for (int j = 0; j < 19; ++j) lam[j] += atot[j];
    }
  }
}

// ------------------------------------------------------------------ fold

// Value of padded index q of an accumulator grid.
template <typename G>
struct PadRead;
template <>
struct PadRead<double> {  // FP64 atomics: one entry per padded voxel
  typedef double T;
  const double* g;
  __device__ T operator()(int64_t q) const { return g[q]; }
  __device__ static double value(T s) { return s; }
};
template <>
struct PadRead<unsigned long long> {  // fixed point: exact integer sums
  typedef unsigned long long T;
  const unsigned long long* g;
  __device__ T operator()(int64_t q) const { return g[q]; }
  __device__ static double value(T s) { return (double)(long long)s / kFixedScale; }
};
template <>
struct PadRead<float4> {  // row-expanded FP32: taps of the rows starting at q, q-1, q-2, q-3
  typedef float T;
  const float4* g;
  __device__ T operator()(int64_t q) const {
    float s = g[q].x;
    if (q >= 1) s += g[q - 1].y;
    if (q >= 2) s += g[q - 2].z;
    if (q >= 3) s += g[q - 3].w;
    return s;
  }
  __device__ static double value(T s) { return (double)s; }
};

// For voxel (i, j, k): sum of the padded copies (the interior one and the
// halo copies) -> out[v * stride + comp] (+= when accumulate).
template <typename G>
__global__ void fold_kernel(const G* __restrict__ padded, int64_t n0, int64_t n1, int64_t n2, float* out, int stride,
                            int comp, int accumulate, unsigned* ovf) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n0 * n1 * n2) return;
  const PadRead<G> rd{padded};
  const int64_t i = v % n0, j = (v / n0) % n1, k = v / (n0 * n1);
  const int64_t p0 = n0 + 3, p1 = n1 + 3;
  int64_t pi[4], pj[4], pk[4];
  int ni = 0, nj = 0, nk = 0;
  // padded coordinate q maps to voxel (q - 1) mod n for q in [0, n + 3)
  pi[ni++] = i + 1;
  if (i == n0 - 1) pi[ni++] = 0;
  if (i == 0) pi[ni++] = n0 + 1;
  if (i == 1 % n0) pi[ni++] = n0 + 2;
  pj[nj++] = j + 1;
  if (j == n1 - 1) pj[nj++] = 0;
  if (j == 0) pj[nj++] = n1 + 1;
  if (j == 1 % n1) pj[nj++] = n1 + 2;
  pk[nk++] = k + 1;
  if (k == n2 - 1) pk[nk++] = 0;
  if (k == 0) pk[nk++] = n2 + 1;
  if (k == 1 % n2) pk[nk++] = n2 + 2;
  typename PadRead<G>::T sum = 0;
  for (int a = 0; a < nk; ++a)
    for (int b = 0; b < nj; ++b)
      for (int c = 0; c < ni; ++c) sum += rd(pi[c] + p0 * (pj[b] + p1 * pk[a]));
  const double dval = PadRead<G>::value(sum);
  if (ovf && !(fabs(dval) < kFixedLimit)) atomicOr(ovf, 1u);  // fixed point near or past its range
  const float val = (float)dval;
  float* dst = out + v * stride + comp;
  *dst = accumulate ? *dst + val : val;
}

}  // namespace srt

using namespace srt;

namespace {

struct DevBuf {
  void* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t bytes) { return dev_alloc(&p, bytes); }
};

template <typename Acc, typename E>
void make_acc(Acc* acc, void* const* bufs) {
  for (int f = 0; f < 4; ++f) acc[f].g = (E*)bufs[f];
}

}  // namespace

#define VJP_TRY(expr, what)          \
  do {                               \
    cudaError_t _e = (expr);         \
    if (_e != cudaSuccess) {         \
      rc = cuda_error(_e, what);     \
      goto done;                     \
    }                                \
  } while (0)

namespace {

// Morton-ordered list of the RING pixels in [pix_begin, pix_begin + pix_count)
// (the forward's launch order) -> rays.
int build_ray_list(int64_t nside, int64_t pix_begin, int64_t pix_count, cudaStream_t s, DevBuf& counts,
                   DevBuf& offsets, DevBuf& rays, int64_t* kernels, const char* who) {
  int rc = SRT_OK;
  RangeArgs ra;
  ra.nside = nside;
  int l = 0;
  while ((int64_t(1) << l) < nside) ++l;
  ra.log2p = l;
  ra.launch_rays = 12 * (int64_t(1) << (2 * l));
  ra.pix_begin = pix_begin;
  ra.pix_count = pix_count;
  const int64_t nblk = (ra.launch_rays + kListBlock - 1) / kListBlock;
  std::vector<int> hc(nblk);
  std::vector<int64_t> ho(nblk);
  int64_t run = 0;
  VJP_TRY(counts.alloc(nblk * sizeof(int)), "cudaMalloc(ray counts)");
  VJP_TRY(offsets.alloc(nblk * sizeof(int64_t)), "cudaMalloc(ray offsets)");
  VJP_TRY(rays.alloc(pix_count * sizeof(int64_t)), "cudaMalloc(ray list)");
  ray_count_kernel<<<(unsigned)nblk, kListBlock, 0, s>>>(ra, (int*)counts.p);
  ++*kernels;
  VJP_TRY(cudaGetLastError(), "ray_count_kernel");
  VJP_TRY(cudaMemcpyAsync(hc.data(), counts.p, nblk * sizeof(int), cudaMemcpyDeviceToHost, s), "copy counts");
  VJP_TRY(cudaStreamSynchronize(s), "ray count");
  for (int64_t b = 0; b < nblk; ++b) {
    ho[b] = run;
    run += hc[b];
  }
  if (run != pix_count)
    return set_error(SRT_ERR_CUDA, "%s: ray list has %lld rays, expected %lld", who, (long long)run,
                     (long long)pix_count);
  VJP_TRY(cudaMemcpyAsync(offsets.p, ho.data(), nblk * sizeof(int64_t), cudaMemcpyHostToDevice, s), "copy offsets");
  ray_write_kernel<<<(unsigned)nblk, kListBlock, 0, s>>>(ra, (const int64_t*)offsets.p, (int64_t*)rays.p);
  ++*kernels;
  VJP_TRY(cudaGetLastError(), "ray_write_kernel");
  // the host vectors must outlive the asynchronous copy of the offsets
  VJP_TRY(cudaStreamSynchronize(s), "ray list");
done:
  return rc;
}

}  // namespace

// A forward trace's checkpoints (srt_forward_tape) for srt_vjp_tape.
struct srt_tape {
  const srt_fields* fields = nullptr;
  int device = 0;
  int64_t nside = 0, pix_begin = 0, pix_count = 0;
  int n_steps = 0, C = 0, nseg = 0;
  int64_t* rays = nullptr;  // Morton-ordered RING pixels (device)
  float* ckpt = nullptr;    // [nseg + 1][kMixedState][pix_count] (device)
  int64_t bytes = 0;
};

static int vjp_impl(const srt_fields* fields, int64_t nside, int64_t pix_begin, int64_t pix_count, int n_steps,
                    int precision, const float* const weights[SRT_NUM_MAPS], float* dphi, float* db_xyz,
                    int ckpt_every, unsigned flags, void* stream, srt_stats* stats, const srt_tape* tape);

extern "C" int srt_vjp(const srt_fields* fields, int64_t nside, int64_t pix_begin, int64_t pix_count, int n_steps,
                       int precision, const float* const weights[SRT_NUM_MAPS], float* dphi, float* db_xyz,
                       int ckpt_every, unsigned flags, void* stream, srt_stats* stats) {
  NvtxRange nvtx_("srt_vjp");
  return vjp_impl(fields, nside, pix_begin, pix_count, n_steps, precision, weights, dphi, db_xyz, ckpt_every, flags,
                  stream, stats, nullptr);
}

// srt_vjp; with a tape, the rays and checkpoints of srt_forward_tape replace
// the ray list and the checkpointing forward pass (MIXED only).
static int vjp_impl(const srt_fields* fields, int64_t nside, int64_t pix_begin, int64_t pix_count, int n_steps,
                    int precision, const float* const weights[SRT_NUM_MAPS], float* dphi, float* db_xyz,
                    int ckpt_every, unsigned flags, void* stream, srt_stats* stats, const srt_tape* tape) {
  const auto t_wall = std::chrono::steady_clock::now();
  if (!fields) return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_vjp: fields is NULL");
  if (nside < 1 || nside > (int64_t(1) << 16))
    return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_vjp: invalid nside %lld", (long long)nside);
  const int64_t npix = 12 * nside * nside;
  if (pix_begin < 0 || pix_count < 0 || pix_begin > npix || pix_count > npix - pix_begin)
    return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_vjp: pixel range outside [0, %lld)", (long long)npix);
  if (n_steps < 1 || n_steps > (1 << 22)) return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_vjp: invalid n_steps %d", n_steps);
  if (precision != SRT_PRECISION_FP64 && precision != SRT_PRECISION_MIXED)
    return set_error(precision == SRT_PRECISION_REF16 ? SRT_ERR_UNSUPPORTED : SRT_ERR_INVALID_ARGUMENT,
                     "srt_vjp: precision %d has no adjoint (use SRT_PRECISION_FP64 or SRT_PRECISION_MIXED)", precision);
  if (!weights) return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_vjp: weights is NULL");
  for (int m = 0; m < 6; ++m)
    if (!weights[m] && pix_count > 0) return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_vjp: weights[%d] is NULL", m);
  if (stats) memset(stats, 0, sizeof(*stats));
  const srt_fields* f = fields;
  const int64_t vox = f->n[0] * f->n[1] * f->n[2];
  const int64_t pvox = f->pn[0] * f->pn[1] * f->pn[2];
  const bool dev_io = (flags & SRT_OUTPUT_DEVICE) != 0;
  const bool accumulate = (flags & SRT_ACCUMULATE) != 0;
  const bool determ = (flags & SRT_DETERMINISTIC) != 0;
  const bool fp64 = precision == SRT_PRECISION_FP64;
  cudaStream_t s = (cudaStream_t)stream;
  int C = ckpt_every > 0 ? ckpt_every : (int)std::max(1.0, std::floor(std::sqrt((double)n_steps) + 0.5));
  if (C > n_steps) C = n_steps;
  if (tape) C = tape->C;
  const int nseg = (n_steps + C - 1) / C;
  int rc = SRT_OK;
  int prev = 0;
  cudaGetDevice(&prev);
  if (prev != f->device) cudaSetDevice(f->device);
  DevBuf counts, offsets, rays, wdev, ckpt, seg, lam, gacc[4], gout_phi, gout_b, ovf;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int64_t kernels = 0, h2d = 0, d2h = 0;
  {
    // padded accumulator entry: 8 B (FP64 / fixed point), 16 B (FP32 rows)
    const size_t accsz = (determ || fp64) ? 8 : 16;
    if (!dev_io) {
      // host gradients: start from zero (or from the caller's values when accumulating)
      if (dphi) {
        VJP_TRY(gout_phi.alloc(vox * sizeof(float)), "cudaMalloc(dphi)");
        if (accumulate) {
          VJP_TRY(cudaMemcpyAsync(gout_phi.p, dphi, vox * sizeof(float), cudaMemcpyHostToDevice, s), "copy dphi");
          h2d += vox * sizeof(float);
        }
      }
      if (db_xyz) {
        VJP_TRY(gout_b.alloc(3 * vox * sizeof(float)), "cudaMalloc(db)");
        if (accumulate) {
          VJP_TRY(cudaMemcpyAsync(gout_b.p, db_xyz, 3 * vox * sizeof(float), cudaMemcpyHostToDevice, s), "copy db");
          h2d += 3 * vox * sizeof(float);
        }
      }
    }
    float* out_phi = dev_io ? dphi : (float*)gout_phi.p;
    float* out_b = dev_io ? db_xyz : (float*)gout_b.p;
    if (pix_count > 0 && (dphi || db_xyz)) {
      // ---- ray list (a tape brings its own)
      const int64_t* ray_list = tape ? tape->rays : nullptr;
      if (!tape) {
        rc = build_ray_list(nside, pix_begin, pix_count, s, counts, offsets, rays, &kernels, "srt_vjp");
        if (rc != SRT_OK) goto done;
        ray_list = (const int64_t*)rays.p;
      }

      // ---- weights on the device
      const float* wd[6];
      if (dev_io) {
        for (int m = 0; m < 6; ++m) wd[m] = weights[m];
      } else {
        VJP_TRY(wdev.alloc(6 * pix_count * sizeof(float)), "cudaMalloc(weights)");
        for (int m = 0; m < 6; ++m) {
          VJP_TRY(cudaMemcpyAsync((float*)wdev.p + m * pix_count, weights[m], pix_count * sizeof(float),
                                  cudaMemcpyHostToDevice, s),
                  "copy weights");
          wd[m] = (const float*)wdev.p + m * pix_count;
        }
        h2d += 6 * pix_count * (int64_t)sizeof(float);
      }

      // ---- scratch: checkpoints, segment records, padded accumulators
      const int state = fp64 ? 19 : kMixedState;
      const size_t esz = fp64 ? sizeof(double) : sizeof(float);
      if (!tape) VJP_TRY(ckpt.alloc((size_t)(nseg + 1) * state * pix_count * esz), "cudaMalloc(checkpoints)");
      // per-step records of one segment: FP64 y, k1, k2, k3; MIXED the four stage inputs
      VJP_TRY(seg.alloc((size_t)C * (fp64 ? state + 57 : kTapeStep) * pix_count * esz), "cudaMalloc(segment records)");
      if (!fp64) VJP_TRY(lam.alloc((size_t)19 * pix_count * sizeof(float)), "cudaMalloc(state cotangents)");
      for (int fld = 0; fld < 4; ++fld) {
        const bool want = (fld == 3) ? (dphi != nullptr) : (db_xyz != nullptr);
        if (!want) continue;
        VJP_TRY(gacc[fld].alloc(pvox * accsz), "cudaMalloc(gradient accumulators)");
        VJP_TRY(cudaMemsetAsync(gacc[fld].p, 0, pvox * accsz, s), "clear accumulators");
      }
      if (determ) {  // fixed-point range flag
        VJP_TRY(ovf.alloc(sizeof(unsigned)), "cudaMalloc(overflow flag)");
        VJP_TRY(cudaMemsetAsync(ovf.p, 0, sizeof(unsigned), s), "clear overflow flag");
      }

      AdjArgs A;
      A.F = make_ptrs(f);
      A.G = make_geom(f);
      A.nside = nside;
      A.pix_begin = pix_begin;
      A.count = pix_count;
      A.rays = ray_list;
      A.n_steps = n_steps;
      A.C = C;
      A.nseg = nseg;
      for (int m = 0; m < 6; ++m) A.w[m] = wd[m];
      A.ckpt = tape ? (void*)tape->ckpt : ckpt.p;
      A.seg = seg.p;
      for (int fld = 0; fld < 4; ++fld) A.acc[fld] = gacc[fld].p;
      for (int m = 0; m < 6; ++m) A.maps[m] = nullptr;
      A.refine_list = nullptr;
      A.refine_count = nullptr;

      VJP_TRY(cudaEventCreate(&e0), "cudaEventCreate");
      VJP_TRY(cudaEventCreate(&e1), "cudaEventCreate");
      VJP_TRY(cudaEventRecord(e0, s), "cudaEventRecord");
      const unsigned blocks = (unsigned)((pix_count + 127) / 128);
      if (fp64) {
        ckpt_kernel_fp64<<<blocks, 128, 0, s>>>(A);
        if (determ) {
          AccFixed ac[4];
          make_acc<AccFixed, unsigned long long>(ac, A.acc);
          for (int fld = 0; fld < 4; ++fld) ac[fld].ovf = (unsigned*)ovf.p;
          reverse_kernel_fp64<AccFixed><<<blocks, 128, 0, s>>>(A, ac[0], ac[1], ac[2], ac[3]);
        } else {
          AccF64 ac[4];
          make_acc<AccF64, double>(ac, A.acc);
          reverse_kernel_fp64<AccF64><<<blocks, 128, 0, s>>>(A, ac[0], ac[1], ac[2], ac[3]);
        }
      } else {
        // forward with checkpoints; then per segment, backwards: recompute
        // the segment's tape, sweep it
        const bool pair = f->pr[0] != nullptr;
        if (tape) {
          // the checkpoints come from srt_forward_tape
        } else if (pair) {
          ckpt_kernel_mixed<true, false><<<blocks, 128, 0, s>>>(A);
        } else {
          ckpt_kernel_mixed<false, false><<<blocks, 128, 0, s>>>(A);
        }
        final_cotangent_kernel_mixed<<<blocks, 128, 0, s>>>(A, (float*)lam.p);
        kernels += tape ? 1 : 2;
        AccF32 af[4];
        AccFixed ax[4];
        make_acc<AccF32, float4>(af, A.acc);
        make_acc<AccFixed, unsigned long long>(ax, A.acc);
        for (int fld = 0; fld < 4; ++fld) ax[fld].ovf = (unsigned*)ovf.p;
        const bool bgrad = db_xyz != nullptr;
        for (int sgi = nseg - 1; sgi >= 0; --sgi) {
          if (pair)
            segment_kernel_mixed<true><<<blocks, 128, 0, s>>>(A, sgi);
          else
            segment_kernel_mixed<false><<<blocks, 128, 0, s>>>(A, sgi);
          if (determ)
            launch_sweep<AccFixed>(A, sgi, (float*)lam.p, ax, pair, bgrad, blocks, s);
          else
            launch_sweep<AccF32>(A, sgi, (float*)lam.p, af, pair, bgrad, blocks, s);
          kernels += 2;
        }
      }
      if (fp64) kernels += 2;
      VJP_TRY(cudaGetLastError(), "adjoint kernels");
      // ---- fold onto the periodic grid
      const unsigned fblocks = (unsigned)((vox + 255) / 256);
      for (int fld = 0; fld < 4; ++fld) {
        if (!gacc[fld].p) continue;
        float* dst = (fld == 3) ? out_phi : out_b;
        const int stride = (fld == 3) ? 1 : 3, comp = (fld == 3) ? 0 : fld;
        const int accum = accumulate ? 1 : 0;
        if (determ)
          fold_kernel<unsigned long long><<<fblocks, 256, 0, s>>>((const unsigned long long*)gacc[fld].p, f->n[0],
                                                                 f->n[1], f->n[2], dst, stride, comp, accum,
                                                                 (unsigned*)ovf.p);
        else if (fp64)
          fold_kernel<double><<<fblocks, 256, 0, s>>>((const double*)gacc[fld].p, f->n[0], f->n[1], f->n[2], dst,
                                                     stride, comp, accum, nullptr);
        else
          fold_kernel<float4><<<fblocks, 256, 0, s>>>((const float4*)gacc[fld].p, f->n[0], f->n[1], f->n[2], dst,
                                                     stride, comp, accum, nullptr);
        ++kernels;
      }
      VJP_TRY(cudaGetLastError(), "fold kernel");
      VJP_TRY(cudaEventRecord(e1, s), "cudaEventRecord");
    } else if (!accumulate) {
      if (out_phi) VJP_TRY(cudaMemsetAsync(out_phi, 0, vox * sizeof(float), s), "clear dphi");
      if (out_b) VJP_TRY(cudaMemsetAsync(out_b, 0, 3 * vox * sizeof(float), s), "clear db");
    }
    if (!dev_io) {
      if (dphi) {
        VJP_TRY(cudaMemcpyAsync(dphi, out_phi, vox * sizeof(float), cudaMemcpyDeviceToHost, s), "copy dphi back");
        d2h += vox * sizeof(float);
      }
      if (db_xyz) {
        VJP_TRY(cudaMemcpyAsync(db_xyz, out_b, 3 * vox * sizeof(float), cudaMemcpyDeviceToHost, s), "copy db back");
        d2h += 3 * vox * sizeof(float);
      }
    }
    VJP_TRY(cudaStreamSynchronize(s), "srt_vjp");
    if (ovf.p) {
      unsigned flag = 0;
      VJP_TRY(cudaMemcpy(&flag, ovf.p, sizeof(flag), cudaMemcpyDeviceToHost), "read overflow flag");
      if (flag) {
        rc = set_error(SRT_ERR_OVERFLOW,
                       "srt_vjp: SRT_DETERMINISTIC gradient beyond the fixed-point range (|gradient| >= 2^30 per "
                       "voxel, or not finite); the gradients are not valid (use the FP32/FP64 accumulation)");
        goto done;
      }
    }
    if (stats) {
      float ms = -1.f;
      if (e0 && e1) cudaEventElapsedTime(&ms, e0, e1);
      stats->trace_ms = ms;
      stats->rays = pix_count;
      stats->ray_steps = pix_count * (int64_t)n_steps;
      stats->kernels = kernels;
      stats->h2d_bytes = h2d;
      stats->d2h_bytes = d2h;
    }
  }
done:
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (prev != f->device) cudaSetDevice(prev);
  if (stats)
    stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_wall).count();
  return rc;
}

// ------------------------------------------------------------------ tape

extern "C" int srt_forward_tape(const srt_fields* fields, int64_t nside, int64_t pix_begin, int64_t pix_count,
                                int n_steps, int ckpt_every, float* const maps[SRT_NUM_MAPS], unsigned flags,
                                void* stream, srt_stats* stats, srt_tape** out) {
  NvtxRange nvtx_("srt_forward_tape");
  const auto t_wall = std::chrono::steady_clock::now();
  if (!out) return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_forward_tape: out is NULL");
  *out = nullptr;
  if (!fields) return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_forward_tape: fields is NULL");
  if (nside < 1 || nside > (int64_t(1) << 16))
    return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_forward_tape: invalid nside %lld", (long long)nside);
  const int64_t npix = 12 * nside * nside;
  if (pix_begin < 0 || pix_count < 1 || pix_begin > npix || pix_count > npix - pix_begin)
    return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_forward_tape: pixel range outside [0, %lld) or empty",
                     (long long)npix);
  if (n_steps < 1 || n_steps > (1 << 22))
    return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_forward_tape: invalid n_steps %d", n_steps);
  if (!maps) return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_forward_tape: maps is NULL");
  for (int m = 0; m < 6; ++m)
    if (!maps[m]) return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_forward_tape: maps[%d] is NULL", m);
  if (stats) memset(stats, 0, sizeof(*stats));
  const srt_fields* f = fields;
  cudaStream_t s = (cudaStream_t)stream;
  const bool dev_out = (flags & SRT_OUTPUT_DEVICE) != 0;
  int C = ckpt_every > 0 ? ckpt_every : (int)std::max(1.0, std::floor(std::sqrt((double)n_steps) + 0.5));
  if (C > n_steps) C = n_steps;
  const int nseg = (n_steps + C - 1) / C;
  int rc = SRT_OK;
  int prev = 0;
  cudaGetDevice(&prev);
  if (prev != f->device) cudaSetDevice(f->device);
  srt_tape* t = new (std::nothrow) srt_tape();
  DevBuf counts, offsets, rays, ckpt, dmaps, rlist, rcount;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int64_t kernels = 0;
  if (!t) {
    rc = set_error(SRT_ERR_OUT_OF_MEMORY, "srt_forward_tape: host allocation failed");
    goto done;
  }
  {
    rc = build_ray_list(nside, pix_begin, pix_count, s, counts, offsets, rays, &kernels, "srt_forward_tape");
    if (rc != SRT_OK) goto done;
    VJP_TRY(ckpt.alloc((size_t)(nseg + 1) * kMixedState * pix_count * sizeof(float)), "cudaMalloc(checkpoints)");
    VJP_TRY(rlist.alloc(pix_count * sizeof(int64_t)), "cudaMalloc(refine list)");
    VJP_TRY(rcount.alloc(sizeof(unsigned long long)), "cudaMalloc(refine count)");
    VJP_TRY(cudaMemsetAsync(rcount.p, 0, sizeof(unsigned long long), s), "clear refine count");
    float* dm[6];
    if (dev_out) {
      for (int m = 0; m < 6; ++m) dm[m] = maps[m];
    } else {
      VJP_TRY(dmaps.alloc(6 * pix_count * sizeof(float)), "cudaMalloc(maps)");
      for (int m = 0; m < 6; ++m) dm[m] = (float*)dmaps.p + m * pix_count;
    }
    AdjArgs A;
    memset(&A, 0, sizeof(A));
    A.F = make_ptrs(f);
    A.G = make_geom(f);
    A.nside = nside;
    A.pix_begin = pix_begin;
    A.count = pix_count;
    A.rays = (const int64_t*)rays.p;
    A.n_steps = n_steps;
    A.C = C;
    A.nseg = nseg;
    A.ckpt = ckpt.p;
    for (int m = 0; m < 6; ++m) A.maps[m] = dm[m];
    A.refine_list = (int64_t*)rlist.p;
    A.refine_count = (unsigned long long*)rcount.p;
    VJP_TRY(cudaEventCreate(&e0), "cudaEventCreate");
    VJP_TRY(cudaEventCreate(&e1), "cudaEventCreate");
    VJP_TRY(cudaEventRecord(e0, s), "cudaEventRecord");
    const unsigned blocks = (unsigned)((pix_count + 127) / 128);
    if (f->pr[0])
      ckpt_kernel_mixed<true, true><<<blocks, 128, 0, s>>>(A);
    else
      ckpt_kernel_mixed<false, true><<<blocks, 128, 0, s>>>(A);
    ++kernels;
    VJP_TRY(cudaGetLastError(), "checkpointing forward");
    TraceArgs ta;
    ta.F = A.F;
    ta.G = A.G;
    ta.nside = nside;
    ta.pix_begin = pix_begin;
    ta.pix_count = pix_count;
    ta.n_steps = n_steps;
    for (int m = 0; m < 6; ++m) ta.maps[m] = dm[m];
    ta.refine_list = A.refine_list;
    ta.refine_count = A.refine_count;
    VJP_TRY(launch_refine(ta, s, &kernels), "refine kernel launch");
    VJP_TRY(cudaEventRecord(e1, s), "cudaEventRecord");
    if (!dev_out)
      for (int m = 0; m < 6; ++m)
        VJP_TRY(cudaMemcpyAsync(maps[m], dm[m], pix_count * sizeof(float), cudaMemcpyDeviceToHost, s),
                "copy maps to host");
    VJP_TRY(cudaStreamSynchronize(s), "srt_forward_tape");
    if (stats) {
      float ms = -1.f;
      cudaEventElapsedTime(&ms, e0, e1);
      stats->trace_ms = ms;
      stats->rays = pix_count;
      stats->ray_steps = pix_count * (int64_t)n_steps;
      stats->kernels = kernels;
      stats->d2h_bytes = dev_out ? 0 : 6 * pix_count * (int64_t)sizeof(float);
      unsigned long long cnt = 0;
      if (cudaMemcpy(&cnt, rcount.p, sizeof(cnt), cudaMemcpyDeviceToHost) == cudaSuccess)
        stats->refined_rays = (int64_t)cnt;
    }
    t->fields = f;
    t->device = f->device;
    t->nside = nside;
    t->pix_begin = pix_begin;
    t->pix_count = pix_count;
    t->n_steps = n_steps;
    t->C = C;
    t->nseg = nseg;
    t->rays = (int64_t*)rays.p;
    t->ckpt = (float*)ckpt.p;
    t->bytes = pix_count * (int64_t)sizeof(int64_t) + (int64_t)(nseg + 1) * kMixedState * pix_count * 4;
    rays.p = nullptr;  // owned by the tape from here on
    ckpt.p = nullptr;
    *out = t;
    t = nullptr;
  }
done:
  delete t;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (prev != f->device) cudaSetDevice(prev);
  if (stats)
    stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_wall).count();
  return rc;
}

extern "C" int srt_vjp_tape(const srt_tape* tape, const float* const weights[SRT_NUM_MAPS], float* dphi,
                            float* db_xyz, unsigned flags, void* stream, srt_stats* stats) {
  NvtxRange nvtx_("srt_vjp_tape");
  if (!tape) return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_vjp_tape: tape is NULL");
  return vjp_impl(tape->fields, tape->nside, tape->pix_begin, tape->pix_count, tape->n_steps, SRT_PRECISION_MIXED,
                  weights, dphi, db_xyz, tape->C, flags, stream, stats, tape);
}

extern "C" int64_t srt_tape_bytes(const srt_tape* tape) { return tape ? tape->bytes : 0; }

extern "C" int srt_tape_destroy(srt_tape* tape) {
  if (!tape) return SRT_OK;
  int prev = 0;
  cudaGetDevice(&prev);
  if (prev != tape->device) cudaSetDevice(tape->device);
  if (tape->rays) cudaFree(tape->rays);
  if (tape->ckpt) cudaFree(tape->ckpt);
  if (prev != tape->device) cudaSetDevice(prev);
  delete tape;
  return SRT_OK;
}
