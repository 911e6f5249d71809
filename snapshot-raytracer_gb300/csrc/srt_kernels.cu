// srt_kernels.cu — the tracer's device kernels (sm_103a):
//   * pad_fields_kernel    periodic halo-padded re-layout of the scalar phi or
//                          of the interleaved B field (every source voxel read once)
//                          (replaces vector3_to_half, snapshot-raytracer.cu:585-597,
//                          and the staged uploads of :774-844)
//   * quantize_half_kernel half(B * 2^27) planes for the REF16 mode
//   * trace_kernel<MODE>   one thread per ray: HEALPix pixel centre -> initial
//                          state -> n_steps RK4 steps -> six maps
//                          (replaces raytracing_kernel, :552-583, and the host
//                          pix2ang loop of :857-866)
//   * fma_probe_kernel     FP32 / FP64 FMA issue-rate probe used for the roofline
#include <cstdio>
#include <algorithm>
#include <cstdlib>
#include "srt_internal.h"

namespace srt {

// ------------------------------------------------------------- field layout

// Padded coordinates of source coordinate c on an axis of extent n: padded
// coordinate q holds voxel (q - 1) mod n for q in [0, n + 3), so c appears at
// c + 1 and, near the ends, in the halo (n - 1 -> 0, 0 -> n + 1, 1 -> n + 2).
// Returns how many of out[0..3] it filled.
__device__ __forceinline__ int padded_coords(int64_t c, int64_t n, int64_t out[4]) {
  int m = 0;
  out[m++] = c + 1;
  if (c == n - 1) out[m++] = 0;
  if (c == 0) out[m++] = n + 1;
  if (c == 1 % n) out[m++] = n + 2;
  return m;
}

// One thread per source voxel of planes k0 .. k1-1 (x fastest, `comps` floats
// per voxel: 1 for phi, 3 for the interleaved B), each source byte read once
// and in 16-byte pieces where it is aligned, so this kernel can read the
// source straight from mapped pinned host memory over the host link: a block's
// 256 B voxels (3 KB) are loaded as 192 float4 into shared memory and then
// picked per thread. Component c goes to padded plane array dst[c] at every
// padded position of the voxel (its interior one and its periodic halo
// copies). Replaces vector3_to_half (snapshot-raytracer.cu:585-597) and the
// staged uploads of :774-844. grid: x over a plane, y over planes.
constexpr int kPadThreads = 256;

__global__ void __launch_bounds__(kPadThreads) pad_fields_kernel(const float* __restrict__ src, int comps,
                                                                  float* __restrict__ d0, float* __restrict__ d1,
                                                                  float* __restrict__ d2, int64_t n0, int64_t n1,
                                                                  int64_t n2, int64_t p0, int64_t p1, int64_t k0) {
  __shared__ float4 stage[kPadThreads * 3 / 4];
  const int64_t plane = n0 * n1;
  const int64_t q0 = (int64_t)blockIdx.x * kPadThreads;  // first voxel of the block in its plane
  const int64_t q = q0 + threadIdx.x;
  const int64_t kl = blockIdx.y;  // plane within the launch
  const int64_t v = kl * plane + q;
  float val[3];
  if (comps == 3) {
    const float* blk = src + (kl * plane + q0) * 3;
    const int64_t nv = plane - q0 < kPadThreads ? plane - q0 : kPadThreads;  // voxels of this block
    if (nv == kPadThreads && ((uintptr_t)blk & 15) == 0) {
      // whole block, aligned: 192 float4 loads cover its 768 floats
      if (threadIdx.x < kPadThreads * 3 / 4) stage[threadIdx.x] = reinterpret_cast<const float4*>(blk)[threadIdx.x];
      __syncthreads();
      const float* st = reinterpret_cast<const float*>(stage);
      for (int c = 0; c < 3; ++c) val[c] = st[3 * threadIdx.x + c];
    } else if (q < plane) {
      for (int c = 0; c < 3; ++c) val[c] = src[v * 3 + c];
    }
  } else if (q < plane) {
    val[0] = src[v];
  }
  if (q >= plane) return;
  const int64_t i = q % n0, j = q / n0, k = k0 + kl;
  int64_t pi[4], pj[4], pk[4];
  const int ni = padded_coords(i, n0, pi), nj = padded_coords(j, n1, pj), nk = padded_coords(k, n2, pk);
  float* const dst[3] = {d0, d1, d2};
  for (int a = 0; a < nk; ++a)
    for (int b = 0; b < nj; ++b)
      for (int c = 0; c < ni; ++c) {
        const int64_t o = pi[c] + p0 * (pj[b] + p1 * pk[a]);
        for (int comp = 0; comp < comps; ++comp) dst[comp][o] = val[comp];
      }
}

cudaError_t launch_pad_fields(const float* src, int comps, float* const dst[3], const int64_t n[3],
                              const int64_t pn[3], int64_t k0, int64_t k1, cudaStream_t s) {
  const int64_t plane = n[0] * n[1];
  for (int64_t kb = k0; kb < k1; kb += 65535) {
    const int64_t ke = kb + 65535 < k1 ? kb + 65535 : k1;
    dim3 grid((unsigned)((plane + kPadThreads - 1) / kPadThreads), (unsigned)(ke - kb), 1);
    pad_fields_kernel<<<grid, kPadThreads, 0, s>>>(src + (kb - k0) * plane * comps, comps, dst[0], dst[1], dst[2], n[0],
                                           n[1], n[2], pn[0], pn[1], kb);
  }
  return cudaGetLastError();
}

__global__ void quantize_half_kernel(const float* __restrict__ src, __half* __restrict__ dst, int64_t count) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) dst[i] = __float2half_rn(src[i] * 134217728.0f);
}

cudaError_t launch_quantize_half(const float* src, __half* dst, int64_t count, cudaStream_t s) {
  const int64_t blocks = (count + 255) / 256;
  quantize_half_kernel<<<(unsigned)blocks, 256, 0, s>>>(src, dst, count);
  return cudaGetLastError();
}

// Row-pair array of a padded field: element (i, j, k), j < py - 1, holds
// (f(i, j, k), f(i, j + 1, k)).
__global__ void pair_build_kernel(const float* __restrict__ src, float2* __restrict__ dst, int64_t px, int64_t py,
                                  int64_t pz) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t rows = py - 1;
  if (q >= px * rows * pz) return;
  const int64_t i = q % px, j = (q / px) % rows, k = q / (px * rows);
  const int64_t s0 = i + px * (j + py * k);
  dst[q] = make_float2(src[s0], src[s0 + px]);
}

cudaError_t launch_pair_build(const float* src, float2* dst, const int64_t pn[3], cudaStream_t s) {
  const int64_t count = pn[0] * (pn[1] - 1) * pn[2];
  pair_build_kernel<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(src, dst, pn[0], pn[1], pn[2]);
  return cudaGetLastError();
}

// -------------------------------------------------------------------- trace

// Resident blocks of 128 threads per SM the mixed kernel is compiled for
// (register budget 65536 / (128 * blocks)).
#ifndef SRT_MIXED_MIN_BLOCKS
#define SRT_MIXED_MIN_BLOCKS 2
#endif

template <int MODE>
__global__ void __launch_bounds__(128, (MODE == kMIXED || MODE == kMIXED_PAIR) ? SRT_MIXED_MIN_BLOCKS : 1)
    trace_kernel(const TraceArgs A) {
  const int64_t tl = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (tl >= A.launch_rays) return;
  // launch order: face-major, Morton (NESTED for power-of-two nside) in-face;
  // a NESTED range launches its own slots
  const int64_t t = A.nested ? A.pix_begin + tl : tl;
  const int64_t face = t >> (2 * A.log2p);
  int64_t ix, iy;
  hp_deinterleave(t & ((int64_t(1) << (2 * A.log2p)) - 1), &ix, &iy);
  if (ix >= A.nside || iy >= A.nside) return;
  const int64_t ring = hp_xyf2ring(A.nside, ix, iy, (int)face);
  const int64_t o = A.nested ? tl : ring - A.pix_begin;
  if (o < 0 || o >= A.pix_count) return;
  const RayDir d = ray_dir_pix(A.nside, ring);
  float out[6];
  if (MODE == kMIXED_PAIR || MODE == kMIXED) {
    __shared__ float guard_m[128][2];  // the ray's guard state, out of the register budget
    const bool near = trace_ray_mixed<MODE == kMIXED_PAIR>(A.F, A.G, d, A.n_steps, out, guard_m[threadIdx.x]);
    if (near && A.refine_list) {
      const unsigned long long k = atomicAdd(A.refine_count, 1ull);
      if (k < (unsigned long long)A.pix_count) A.refine_list[k] = o;
    }
  } else {
    trace_ray_std<MODE == kREF16 ? kREF16 : kFP64>(A.F, A.G, d, A.n_steps, out);
  }
#pragma unroll
  for (int m = 0; m < 6; ++m) A.maps[m][o] = out[m];
}

// Re-trace of listed rays (MIXED rays near a cell face) in FP64 arithmetic;
// the list's length is read on the device, so no host round trip is needed.
//
// The rays are few (~0.15% of a sky at 512 steps) and FP64 runs at 1/64 of
// the FP32 rate: a warp of 32 single-thread FP64 rays needs ~0.17-0.25 s for
// 512 steps however few of its lanes are busy, so the launch takes about one
// warp's time. Each ray is therefore traced by a group of four lanes, one per
// field (B_x, B_y, B_z, phi): every lane interpolates its field, the group
// exchanges the four results by shuffles, and every lane forms the rest of the
// right-hand side. Short lists run this in FP64 with the operations of
// rhs_std<kFP64> in the same order (bit-identical maps); long lists run it in
// double-float arithmetic on the FP32 pipes (srt_dd.cuh; trajectory ~1e-14
// from the FP64 one, maps within one float ulp), which is shorter once the
// warps outnumber the SM sub-partitions.
// Re-trace grid: at most 32 one-warp blocks per SM (the SM count is read from
// the device); lists up to two warps per SM sub-partition (8 rays per warp)
// take the FP64 path.
constexpr int64_t kRefineBlocksPerSM = 32;
constexpr int64_t kRefineWarpsPerSubpartition = 2;
constexpr int64_t kRefineWideWarpsPerSubpartition = 4;

__device__ __forceinline__ void shfl_tri(Tri<double>& d, const Tri<double>& s, int src, unsigned mask) {
  d.v = __shfl_sync(mask, s.v, src);
#pragma unroll
  for (int i = 0; i < 3; ++i) d.g[i] = __shfl_sync(mask, s.g[i], src);
#pragma unroll
  for (int i = 0; i < 6; ++i) d.h[i] = __shfl_sync(mask, s.h[i], src);
}

// A lane-group value of the state type (FP64 or double-float) from lane src.
__device__ __forceinline__ double shfl_r(double v, int src, unsigned mask) { return __shfl_sync(mask, v, src); }
__device__ __forceinline__ dd shfl_r(const dd& v, int src, unsigned mask) {
  return dd(__shfl_sync(mask, v.hi, src), __shfl_sync(mask, v.lo, src));
}

// rhs_frame with its three normalisations (a square root and three divisions
// each) shared out over a ray's lane group: lane f normalises vector f (n, e1,
// e2; the phi lane repeats n) with the same operations, and the group
// exchanges the results. gmask: the group's four lanes, which always run
// together (they hold the same state).
template <typename R>
__device__ __forceinline__ void rhs_frame_group(const R* y, R* n, R* a, R* b, int field, int group,
                                                unsigned gmask) {
  const int v = field < 3 ? field : 0;
  const R c0 = v == 0 ? y[3] : (v == 1 ? y[6] : y[9]);
  const R c1 = v == 0 ? y[4] : (v == 1 ? y[7] : y[10]);
  const R c2 = v == 0 ? y[5] : (v == 1 ? y[8] : y[11]);
  const R r = sqrt_r(c0 * c0 + c1 * c1 + c2 * c2);
  const R u[3] = {c0 / r, c1 / r, c2 / r};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    n[i] = shfl_r(u[i], group, gmask);
    a[i] = shfl_r(u[i], group + 1, gmask);
    b[i] = shfl_r(u[i], group + 2, gmask);
  }
}

// The dA > 1/2 branch's four divisions shared out the same way: lane j forms
// quotient j (every lane of a group takes the branch or none does).
template <typename R>
struct GroupDiv {
  int field, group;
  unsigned gmask;
  __device__ void operator()(const R* num, const R* den, R* quo) const {
    const R nj = field == 0 ? num[0] : (field == 1 ? num[1] : (field == 2 ? num[2] : num[3]));
    const R dj = field == 0 ? den[0] : (field == 1 ? den[1] : (field == 2 ? den[2] : den[3]));
    const R mine = nj / dj;
#pragma unroll
    for (int j = 0; j < 4; ++j) quo[j] = shfl_r(mine, group + j, gmask);
  }
};

// rhs_std<kFP64> with the four interpolations, the normalisations and the
// branch's divisions spread over a lane group (field = lane & 3, group = the
// group's first lane, mask = live lanes); every value is formed by the
// operations rhs_std<kFP64> uses, so the results are the same bits.
__device__ __forceinline__ void rhs_fp64_group(const double* y, double* dy, const FieldPtrs& F, const Geom& G,
                                               int field, int group, unsigned mask) {
  const unsigned gmask = 0xfu << group;
  double n[3], a[3], b[3];
  rhs_frame_group<double>(y, n, a, b, field, group, gmask);
  Tri<double> own;
  {
    const float* src = (field == 3) ? F.phi : ((field == 0) ? F.b[0] : ((field == 1) ? F.b[1] : F.b[2]));
    const double ox = (field == 0) ? 0.5 : 0.0, oy = (field == 1) ? 0.5 : 0.0, oz = (field == 2) ? 0.5 : 0.0;
    interp_std<double, float>(src, G, y[0] - ox, y[1] - oy, y[2] - oz, own);
  }
  BSums<double, double> B;
  B.clear();
  Tri<double> r;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    shfl_tri(r, own, group + c, mask);
    B.add(c, r, n, a, b);
  }
  shfl_tri(r, own, group + 3, mask);
  rhs_finish<double, double>(y, n, a, b, B, r, dy, GroupDiv<double>{field, group, gmask});
}

// step_std<kFP64> on rhs_fp64_group.
__device__ __forceinline__ void step_fp64_group(const FieldPtrs& F, const Geom& G, double* y, int field, int group,
                                                unsigned mask) {
  double acc[19], k[19], ys[19];
  for (int j = 0; j < 19; ++j) k[j] = 0.0;
#pragma unroll 1
  for (int st = 0; st < 4; ++st) {
    const double c = (st == 3) ? 1.0 : 0.5;
    for (int j = 0; j < 19; ++j) ys[j] = (st == 0) ? y[j] : y[j] + c * k[j];
    rhs_fp64_group(ys, k, F, G, field, group, mask);
    for (int j = 0; j < 19; ++j) acc[j] = (st == 0) ? k[j] : ((st < 3) ? acc[j] + 2.0 * k[j] : acc[j]);
  }
  for (int j = 0; j < 19; ++j) y[j] += (acc[j] + k[j]) / 6.0;
}

// rhs_dd with the four interpolations spread over a lane group, as
// rhs_fp64_group does for FP64.
__device__ __forceinline__ void shfl_tri_dd(Tri<dd>& d, const Tri<dd>& s, int src, unsigned mask) {
  d.v = dd(__shfl_sync(mask, s.v.hi, src), __shfl_sync(mask, s.v.lo, src));
#pragma unroll
  for (int i = 0; i < 3; ++i) d.g[i] = dd(__shfl_sync(mask, s.g[i].hi, src), __shfl_sync(mask, s.g[i].lo, src));
#pragma unroll
  for (int i = 0; i < 6; ++i) d.h[i] = dd(__shfl_sync(mask, s.h[i].hi, src), __shfl_sync(mask, s.h[i].lo, src));
}

__device__ __forceinline__ void rhs_dd_group(const dd* y, dd* dy, const FieldPtrs& F, const Geom& G, int field,
                                             int group, unsigned mask) {
  const unsigned gmask = 0xfu << group;
  dd n[3], a[3], b[3];
  rhs_frame_group<dd>(y, n, a, b, field, group, gmask);
  Tri<dd> own;
  {
    const float* src = (field == 3) ? F.phi : ((field == 0) ? F.b[0] : ((field == 1) ? F.b[1] : F.b[2]));
    const dd half(0.5f);
    interp_dd(src, G, field == 0 ? y[0] - half : y[0], field == 1 ? y[1] - half : y[1],
              field == 2 ? y[2] - half : y[2], own);
  }
  BSums<dd, dd> B;
  B.clear();
  Tri<dd> r;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    shfl_tri_dd(r, own, group + c, mask);
    B.add(c, r, n, a, b);
  }
  shfl_tri_dd(r, own, group + 3, mask);
  rhs_finish<dd, dd>(y, n, a, b, B, r, dy, GroupDiv<dd>{field, group, gmask});
}

// step_std<kFP64> in double-float on rhs_dd_group, with the state and the RK4
// accumulator in shared memory, one copy per lane group (the four lanes of a
// group form the same values, so each writes what the others write): the
// registers then hold only the stage input, the stage's k and the right-hand
// side's working set.
__device__ __forceinline__ void step_dd_group(const FieldPtrs& F, const Geom& G, dd* y, dd* acc, int field,
                                              int group, unsigned mask) {
  dd k[19];
#pragma unroll 1
  for (int st = 0; st < 4; ++st) {
    const float c = (st == 3) ? 1.f : 0.5f;
    dd ys[19];
    for (int j = 0; j < 19; ++j) ys[j] = (st == 0) ? y[j] : y[j] + c * k[j];
    rhs_dd_group(ys, k, F, G, field, group, mask);
    for (int j = 0; j < 19; ++j) acc[j] = (st == 0) ? k[j] : ((st < 3) ? acc[j] + 2.f * k[j] : acc[j]);
  }
  const dd sixth = dd(1.0 / 6.0);
  for (int j = 0; j < 19; ++j) y[j] += (acc[j] + k[j]) * sixth;
}

// One lane's double-float state in a shared-memory column of a warp's array
// (component j at c[32 j]).
struct DdCol {
  dd* c;
  __device__ dd& operator[](int j) const { return c[32 * j]; }
};

// step_dd_group with one lane doing the whole ray (rhs_dd: all four
// interpolations and the right-hand side once), its state in a DdCol.

__device__ __forceinline__ void step_dd1(const FieldPtrs& F, const Geom& G, const DdCol& y, const DdCol& acc) {
  dd k[19], ys[19];
#pragma unroll 1
  for (int st = 0; st < 4; ++st) {
    const float c = (st == 3) ? 1.f : 0.5f;
    for (int j = 0; j < 19; ++j) ys[j] = (st == 0) ? y[j] : y[j] + c * k[j];
    rhs_dd(ys, k, F, G);
    for (int j = 0; j < 19; ++j) acc[j] = (st == 0) ? k[j] : ((st < 3) ? acc[j] + 2.f * k[j] : acc[j]);
  }
  const dd sixth = dd(1.0 / 6.0);
  for (int j = 0; j < 19; ++j) y[j] += (acc[j] + k[j]) * sixth;
}

// Which re-trace a list of n rays gets:
//   MODE 4 (n <= dd_min): the bit-exact FP64 four-lane groups (up to two
//     warps per sub-partition: latency-bound, and FP64 is then the shorter:
//     163 rays of a 512^3 / 256-step sky take ~36 ms against ~39 ms in
//     double-float, while the 12.4k of a 1024^3 sky take 190 against 113 ms);
//   MODE 1 (dd_min < n <= wide_min): double-float four-lane groups (~1.4x
//     shorter than FP64 one-lane warps at ~19k rays; maps within one float ulp
//     of the FP64 ones);
//   MODE 2 (n > wide_min): double-float, one lane per ray: once the list fills
//     every sub-partition with several warps the launch is bound by the total
//     work, which the four-lane groups raise by repeating the right-hand side
//     on each lane (~48k against ~28k FP32 instructions per ray and stage).
// The environment variables SRT_REFINE_DD_MIN and SRT_REFINE_WIDE_MIN override
// dd_min and wide_min (tests use them to reach every path on small skies).
// The double-float re-traces keep their state in shared memory and fit 12
// one-warp blocks per SM (168 registers, no spill): the ~1,550 four-lane warps
// of a 1024^3 sky's list then run in one wave instead of two (113 against
// 157 ms); the one-lane warps of a 2048^3 sky's ~245k rays gain 0.8 % of the sky.
template <int MODE>
__global__ void __launch_bounds__(32, (MODE == 1 || MODE == 2) ? 12 : 1)
    refine_kernel(const TraceArgs A, int64_t dd_min, int64_t wide_min) {
  constexpr int LANES = MODE == 2 ? 1 : 4;
  constexpr int kRays = 32 / LANES;  // rays per warp
  const int lane = threadIdx.x;
  const unsigned long long count = *A.refine_count;
  const int64_t n = min((int64_t)count, A.pix_count);
  const int mode = n <= dd_min ? 4 : (n <= wide_min ? 1 : 2);
  if (mode != MODE) return;
#pragma unroll 1
  for (int64_t k0 = (int64_t)blockIdx.x * kRays; k0 < n; k0 += (int64_t)gridDim.x * kRays) {
    const int64_t k = k0 + lane / LANES;
    if (k >= n) continue;
    const int64_t o = A.refine_list[k];  // output slot
    const int64_t ring = A.nested ? hp_nest2ring(A.nside, A.pix_begin + o) : A.pix_begin + o;
    const RayDir d = ray_dir_pix(A.nside, ring);
    float out[6];
    if (MODE == 4) {
      double y[19];
      init_std(d, A.G, y);
      // live groups are a prefix of the warp: their lanes form the shuffle mask
      const int64_t live = min((int64_t)kRays, n - k0);
      const unsigned mask = (live >= kRays) ? 0xffffffffu : ((1u << (4 * live)) - 1u);
#pragma unroll 1
      for (int step = 0; step < A.n_steps; ++step) step_fp64_group(A.F, A.G, y, lane & 3, lane & ~3, mask);
      extract_std(d, A.G, y, out);
    } else if (MODE == 2) {
      // raw storage viewed as dd (two floats, as float2): a shared array of a
      // type with a constructor would not be initialised anyway
      __shared__ float2 s_y1[19][32], s_acc1[19][32];
      const DdCol y{reinterpret_cast<dd*>(&s_y1[0][lane])}, acc{reinterpret_cast<dd*>(&s_acc1[0][lane])};
      {
        dd yl[19];
        init_dd(d, A.G, yl);
        for (int j = 0; j < 19; ++j) y[j] = yl[j];
      }
#pragma unroll 1
      for (int step = 0; step < A.n_steps; ++step) step_dd1(A.F, A.G, y, acc);
      {
        dd yl[19];
        for (int j = 0; j < 19; ++j) yl[j] = y[j];
        extract_dd(d, A.G, yl, out);
      }
    } else {
      __shared__ float2 s_y[8][19], s_acc[8][19];  // dd storage, as above
      dd* y = reinterpret_cast<dd*>(s_y[lane >> 2]);
      {
        dd yl[19];
        init_dd(d, A.G, yl);
        for (int j = 0; j < 19; ++j) y[j] = yl[j];
      }
      const int64_t live = min((int64_t)kRays, n - k0);
      const unsigned mask = (live >= kRays) ? 0xffffffffu : ((1u << (4 * live)) - 1u);
#pragma unroll 1
      for (int step = 0; step < A.n_steps; ++step)
        step_dd_group(A.F, A.G, y, reinterpret_cast<dd*>(s_acc[lane >> 2]), lane & 3, lane & ~3, mask);
      {
        dd yl[19];
        for (int j = 0; j < 19; ++j) yl[j] = y[j];
        extract_dd(d, A.G, yl, out);
      }
    }
    if (lane % LANES == 0) {
#pragma unroll
      for (int m = 0; m < 6; ++m) A.maps[m][o] = out[m];
    }
  }
}

cudaError_t launch_refine(const TraceArgs& a, cudaStream_t s, int64_t* kernels) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  int64_t dd_min = kRefineWarpsPerSubpartition * 4 * (int64_t)sms * 8;
  if (const char* v = getenv("SRT_REFINE_DD_MIN")) dd_min = strtoll(v, nullptr, 10);
  // one-lane rays from four warps of 32 per sub-partition on
  int64_t wide_min = kRefineWideWarpsPerSubpartition * 4 * (int64_t)sms * 32;
  if (const char* v = getenv("SRT_REFINE_WIDE_MIN")) wide_min = strtoll(v, nullptr, 10);
  const int64_t blocks = std::min((a.pix_count + 7) / 8, kRefineBlocksPerSM * (int64_t)sms);
  if (blocks < 1) return cudaSuccess;
  const int64_t blocks1 = std::min((a.pix_count + 31) / 32, kRefineBlocksPerSM * (int64_t)sms);
  refine_kernel<4><<<(unsigned)blocks, 32, 0, s>>>(a, dd_min, wide_min);
  refine_kernel<1><<<(unsigned)blocks, 32, 0, s>>>(a, dd_min, wide_min);
  refine_kernel<2><<<(unsigned)blocks1, 32, 0, s>>>(a, dd_min, wide_min);
  if (kernels) *kernels += 3;
  return cudaGetLastError();
}

cudaError_t launch_trace(int mode, const TraceArgs& a, cudaStream_t s, int64_t* kernels) {
  const int threads = 128;
  const int64_t blocks = (a.launch_rays + threads - 1) / threads;
  if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
  switch (mode) {
    case kFP64: trace_kernel<kFP64><<<(unsigned)blocks, threads, 0, s>>>(a); break;
    case kMIXED: trace_kernel<kMIXED><<<(unsigned)blocks, threads, 0, s>>>(a); break;
    case kREF16: trace_kernel<kREF16><<<(unsigned)blocks, threads, 0, s>>>(a); break;
    case kMIXED_PAIR: trace_kernel<kMIXED_PAIR><<<(unsigned)blocks, threads, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  if (kernels) ++*kernels;
  return cudaGetLastError();
}

// ------------------------------------------------------------ peak probes

// Eight independent FMA chains per thread; kind 0 = FP32, 1 = FP64.
template <typename T>
__global__ void fma_probe_kernel(T* out, int iters, T a, T b) {
  T x0 = (T)threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  const T r = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (r == (T)-1.2345) out[0] = r;  // keeps the chains live
}

// The same with packed pairs: eight independent FFMA2 chains per thread
// (two FP32 FMAs per instruction, the form the MIXED tricubic uses).
__global__ void fma2_probe_kernel(float* out, int iters, float a, float b) {
  const float t = (float)threadIdx.x;
  float2 x[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) x[j] = make_float2(t + j, t - j);
  const float2 a2 = make_float2(a, a), b2 = make_float2(b, b);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
#pragma unroll
      for (int j = 0; j < 8; ++j) x[j] = __ffma2_rn(x[j], a2, b2);
    }
  }
  float r = 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) r += x[j].x + x[j].y;
  if (r == -1.2345f) out[0] = r;  // keeps the chains live
}

cudaError_t probe_fma(int kind, double* flops_per_s) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  void* out = nullptr;
  e = cudaMalloc(&out, 64);
  if (e != cudaSuccess) return e;
  const int threads = 256, blocks = sms * 8;
  const int iters = kind == 1 ? 64 : 4096;
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(t0);
    if (kind == 0)
      fma_probe_kernel<float><<<blocks, threads>>>((float*)out, iters, 0.999999f, 1e-7f);
    else if (kind == 2)
      fma2_probe_kernel<<<blocks, threads>>>((float*)out, iters, 0.999999f, 1e-7f);
    else
      fma_probe_kernel<double><<<blocks, threads>>>((double*)out, iters, 0.999999, 1e-7);
    cudaEventRecord(t1);
    e = cudaEventSynchronize(t1);
    if (e != cudaSuccess) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t0, t1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(out);
  if (e != cudaSuccess) return e;
  const double flops = (kind == 2 ? 2.0 : 1.0) * 2.0 * 8.0 * 16.0 * (double)iters * (double)threads * (double)blocks;
  *flops_per_s = flops / (best * 1e-3);
  return cudaGetLastError();
}

}  // namespace srt
