// srt_scheme.cuh — per-ray scheme of the tracer: tricubic Catmull-Rom
// interpolation with gradient and Hessian, the 19-component geodesic +
// Jacobi-map right-hand side, fixed-step RK4 and the map extraction.
//
// Scheme followed (snapshot-raytracer.cu):
//   * 1-D Catmull-Rom value / d/dt / d2/dt2 on four taps       :195-212
//   * separable tricubic pass x -> y -> z, x fastest in memory, :214-312
//     periodic grid, cell ix = floor(x), taps ix-1 .. ix+2
//   * right-hand side (normalised n, e1, e2; staggered B with   :315-510
//     B_x at x-1/2, B_y at y-1/2, B_z at z-1/2; Sachs optical
//     equations; ellipticity and rotation only while dA > 1/2)
//   * classic RK4, h = 1 grid unit                              :513-550
//   * initial state from (theta, phi), extraction of the six    :552-583
//     maps (deflection projected on e_theta and on -e_phi)
// The computation is restated here for the GPU (it is not the reference's
// code): one set of Catmull-Rom weights per axis is formed once per
// interpolation and reused for all 16 x-runs, the passes are streamed over z
// so only ten accumulators stay live, the B contributions are accumulated in a
// loop over components, and fields are read from a halo-padded layout so no
// tap needs a modulo.
//
// Precision modes (SRT_PRECISION_* in srt.h):
//   FP64  — everything in double.
//   REF16 — the reference's arithmetic: B planes hold half(B * 2^27), the
//           interpolation is FP32 with the cell offset taken as
//           float(x) - float(floor(x)), intermediates of the right-hand side
//           that the reference keeps in float are float, state is double.
//   MIXED — FP32 interpolation and right-hand side on a perturbation state
//           delta = y - y0(s), where y0(s) is the exact solution for
//           Phi = B = 0 (a straight ray: x = x0 - s n0, n = n0, e = e0,
//           dA = s, dA' = -1). RK4 is affine, so integrating delta with the
//           perturbation right-hand side f(y0 + delta) - f(y0) gives the same
//           iterates as integrating y. Every FP32 quantity is then small and
//           carries full relative precision; the ray position used to pick
//           the cell is x0 - s n0 + delta_x with s*n0 split exactly (FMA), and
//           the state is accumulated with compensated (two-sum) additions.
//           FP64 is used only for ray setup and map extraction.
#pragma once
#include <stdint.h>
#include <math.h>
#include <cuda_fp16.h>
#include "srt_healpix.cuh"
#include "srt_dd.cuh"

namespace srt {

enum { kFP64 = 0, kMIXED = 1, kREF16 = 2, kMIXED_PAIR = 3 };

#if defined(__CUDA_ARCH__)
template <typename T>
SRT_HD T ldg(const T* p) { return __ldg(p); }
// Streaming (evict-first) store and load for data touched once per pass (the
// adjoint's tape), so it does not displace field taps from L1.
SRT_HD void st_stream(float* p, float v) { __stcs(p, v); }
SRT_HD float ld_stream(const float* p) { return __ldcs(p); }
#else
template <typename T>
SRT_HD T ldg(const T* p) { return *p; }
SRT_HD void st_stream(float* p, float v) { *p = v; }
SRT_HD float ld_stream(const float* p) { return *p; }
#endif

// Halo-padded periodic grid: voxel (i,j,k), -1 <= i <= n0+1 (etc.), lives at
// (i+1) + px*((j+1) + py*(k+1)), px = n0+3, py = n1+3, pxy = px*py.
struct Geom {
  int n[3];
  int64_t px, pxy;
  int64_t pxy2;  // slice stride of the row-pair arrays (float2 units): px * (py - 1)
  float invn[3];
};

struct FieldPtrs {
  const float* phi;     // padded FP32
  const float* b[3];    // padded FP32 B components
  const __half* bh[3];  // padded half(B * 2^27) (REF16 only)
  // Row-pair arrays (MIXED fast path, optional): element (i, j, k), j < py - 1,
  // holds (f(i, j, k), f(i, j + 1, k)) of the padded field; [0..2] B, [3] phi.
  const float2* pr[4];
};

template <typename T>
struct Tri {  // value, gradient, Hessian (xx, xy, xz, yy, yz, zz)
  T v, g[3], h[6];
};

template <typename T>
struct CRW {  // Catmull-Rom weights of the 4 taps for value, d/dt, d2/dt2
  T w[4], g[4], h[4];
};

// Weights of f(t) = sum_i w_i(t) p_i for the Catmull-Rom cubic through p0..p3
// on [p1, p2] (tangents (p2 - p0)/2 and (p3 - p1)/2), and of f', f''.
template <typename T>
SRT_HD void cr_weights(T t, CRW<T>& c) {
  const T t2 = t * t, t3 = t2 * t;
  c.w[0] = T(0.5) * (T(2) * t2 - t - t3);
  c.w[1] = T(0.5) * (T(3) * t3 - T(5) * t2 + T(2));
  c.w[2] = T(0.5) * (T(4) * t2 + t - T(3) * t3);
  c.w[3] = T(0.5) * (t3 - t2);
  c.g[0] = T(0.5) * (T(4) * t - T(3) * t2 - T(1));
  c.g[1] = T(0.5) * (T(9) * t2 - T(10) * t);
  c.g[2] = T(0.5) * (T(8) * t - T(9) * t2 + T(1));
  c.g[3] = T(0.5) * (T(3) * t2 - T(2) * t);
  c.h[0] = T(2) - T(3) * t;
  c.h[1] = T(9) * t - T(5);
  c.h[2] = T(4) - T(9) * t;
  c.h[3] = T(3) * t - T(1);
}

// The same weights in Horner form for the MIXED form's FP32 interpolation
// (22 operations, two of them shared, against ~28 for the expanded
// polynomials; the FP64 and REF16 forms keep cr_weights).
SRT_HD void cr_weights_mixed(float t, CRW<float>& c) {
  const float t2 = t * t;
  const float a2 = fmaf(-1.5f, t, 2.f);  // 2 - 3t/2, in w2 and g0
  c.w[0] = fmaf(fmaf(-0.5f, t, 1.f), t, -0.5f) * t;
  c.w[1] = fmaf(fmaf(1.5f, t, -2.5f), t2, 1.f);
  c.w[2] = fmaf(a2, t, 0.5f) * t;
  c.w[3] = fmaf(0.5f, t, -0.5f) * t2;
  c.g[0] = fmaf(a2, t, -0.5f);
  c.g[1] = fmaf(4.5f, t, -5.f) * t;
  c.g[2] = fmaf(fmaf(-4.5f, t, 4.f), t, 0.5f);
  c.g[3] = fmaf(1.5f, t, -1.f) * t;
  c.h[0] = fmaf(-3.f, t, 2.f);
  c.h[1] = fmaf(9.f, t, -5.f);
  c.h[2] = fmaf(-9.f, t, 4.f);
  c.h[3] = fmaf(3.f, t, -1.f);
}

template <typename T>
SRT_HD T tapv(float x) { return (T)x; }
template <typename T>
SRT_HD T tapv(__half x) { return (T)__half2float(x); }

// Tricubic value/gradient/Hessian from the 4x4x4 taps starting at padded
// index `base` (= the voxel (cx-1, cy-1, cz-1) of cell (cx, cy, cz)).
template <typename T, typename TapT>
SRT_HD void tricubic(const TapT* __restrict__ f, int64_t base, int64_t px, int64_t pxy,
                     const CRW<T>& X, const CRW<T>& Y, const CRW<T>& Z, Tri<T>& r) {
  T v = 0, g0 = 0, g1 = 0, g2 = 0, h00 = 0, h01 = 0, h02 = 0, h11 = 0, h12 = 0, h22 = 0;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    T a = 0, ay = 0, ayy = 0, ax = 0, axy = 0, axx = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const TapT* row = f + base + c * pxy + b * px;
      const T p0 = tapv<T>(ldg(row + 0)), p1 = tapv<T>(ldg(row + 1));
      const T p2 = tapv<T>(ldg(row + 2)), p3 = tapv<T>(ldg(row + 3));
      const T rv = X.w[0] * p0 + X.w[1] * p1 + X.w[2] * p2 + X.w[3] * p3;
      const T rx = X.g[0] * p0 + X.g[1] * p1 + X.g[2] * p2 + X.g[3] * p3;
      const T rxx = X.h[0] * p0 + X.h[1] * p1 + X.h[2] * p2 + X.h[3] * p3;
      a += Y.w[b] * rv;
      ay += Y.g[b] * rv;
      ayy += Y.h[b] * rv;
      ax += Y.w[b] * rx;
      axy += Y.g[b] * rx;
      axx += Y.w[b] * rxx;
    }
    v += Z.w[c] * a;
    g0 += Z.w[c] * ax;
    g1 += Z.w[c] * ay;
    g2 += Z.g[c] * a;
    h00 += Z.w[c] * axx;
    h01 += Z.w[c] * axy;
    h02 += Z.g[c] * ax;
    h11 += Z.w[c] * ayy;
    h12 += Z.g[c] * ay;
    h22 += Z.h[c] * a;
  }
  r.v = v;
  r.g[0] = g0;
  r.g[1] = g1;
  r.g[2] = g2;
  r.h[0] = h00;
  r.h[1] = h01;
  r.h[2] = h02;
  r.h[3] = h11;
  r.h[4] = h12;
  r.h[5] = h22;
}

template <typename T>
SRT_HD void tri_scale(Tri<T>& r, T s) {
  r.v *= s;
  for (int i = 0; i < 3; ++i) r.g[i] *= s;
  for (int i = 0; i < 6; ++i) r.h[i] *= s;
}

// ------------------------------------------------ packed (FFMA2) tricubic

#if defined(__CUDA_ARCH__)
SRT_HD float2 ffma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
SRT_HD float2 fmul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
SRT_HD float2 fadd2(float2 a, float2 b) { return __fadd2_rn(a, b); }
#else
SRT_HD float2 ffma2(float2 a, float2 b, float2 c) { return make_float2(fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y)); }
SRT_HD float2 fmul2(float2 a, float2 b) { return make_float2(a.x * b.x, a.y * b.y); }
SRT_HD float2 fadd2(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
#endif
SRT_HD float2 dup2(float v) { return make_float2(v, v); }
// a - b, one rounding (there is no packed subtract: -1 * b + a)
SRT_HD float2 fsub2(float2 a, float2 b) { return ffma2(dup2(-1.f), b, a); }

// Where the packed passes get their taps: rows y and y+1 of a slice, tap i,
// as one float2. Two sources:
//   PairRows   the row-pair array (srt_fields.pr): one 64-bit load per tap
//              pair; base is the pair index of voxel (cx-1, cy-1, cz-1);
//   SingleRows the halo-padded single layout: two 32-bit loads (rows y and
//              y+1, one row stride apart) placed in the two halves of the
//              pair, so the packed arithmetic needs no second copy of the
//              field; base is the voxel's padded index.
// Both give the same float2 values, so the interpolations agree bit for bit.
struct PairRows {
  const float2* __restrict__ f;
  int64_t base, px, pxy2;
  SRT_HD float2 operator()(int c, int pr, int i) const { return ldg(f + base + c * pxy2 + 2 * pr * px + i); }
};
struct SingleRows {
  const float* __restrict__ f;
  int64_t base, px, pxy;
  SRT_HD float2 operator()(int c, int pr, int i) const {
    const float* r = f + base + c * pxy + 2 * pr * px + i;
    return make_float2(ldg(r), ldg(r + px));
  }
};

// The same interpolation as `tricubic` on packed pairs (two FP32 FMAs per
// instruction): the x pass on rows y and y+1 at once with duplicated x
// weights, the y pass with the weights of rows (0, 1) and (2, 3) (even / odd
// partial sums). Per slice the six y sums are then completed (one add each)
// and the z pass forms the ten outputs as five pairs with no idle lane:
// (v, gx), (gy, hyy) and (hxx, hxy) from the value weight on both lanes,
// (gz, hxz) from the derivative weight on both, and (hyz, hzz) from the
// (derivative, second-derivative) weight pair on (ay, a). Three weight pairs
// and four operand pairs per slice: each output is still its own chain of
// FMAs over the slices, so the results do not depend on the pairing, and this
// one needs the fewest register copies to build the pairs.
template <typename Rows>
SRT_HD void tricubic_pair(const Rows& rows, const CRW<float>& X, const CRW<float>& Y, const CRW<float>& Z,
                          Tri<float>& r) {
  float2 xw[4], xg[4], xh[4];
  for (int i = 0; i < 4; ++i) {
    xw[i] = dup2(X.w[i]);
    xg[i] = dup2(X.g[i]);
    xh[i] = dup2(X.h[i]);
  }
  const float2 yw[2] = {make_float2(Y.w[0], Y.w[1]), make_float2(Y.w[2], Y.w[3])};
  const float2 yg[2] = {make_float2(Y.g[0], Y.g[1]), make_float2(Y.g[2], Y.g[3])};
  const float2 yh[2] = {make_float2(Y.h[0], Y.h[1]), make_float2(Y.h[2], Y.h[3])};
  const float2 z0 = make_float2(0.f, 0.f);
  // z-pass accumulators: (v, gx), (gz, hxz), (gy, hyy), (hyz, hzz), (hxx, hxy)
  float2 VG0 = z0, G2H02 = z0, G1H11 = z0, H12H22 = z0, H00H01 = z0;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    float2 A = z0, AY = z0, AYY = z0, AX = z0, AXY = z0, AXX = z0;
#pragma unroll
    for (int pr = 0; pr < 2; ++pr) {
      const float2 t0 = rows(c, pr, 0), t1 = rows(c, pr, 1), t2 = rows(c, pr, 2), t3 = rows(c, pr, 3);
      float2 RV = fmul2(xw[0], t0), RX = fmul2(xg[0], t0), RXX = fmul2(xh[0], t0);
      RV = ffma2(xw[1], t1, RV);
      RX = ffma2(xg[1], t1, RX);
      RXX = ffma2(xh[1], t1, RXX);
      RV = ffma2(xw[2], t2, RV);
      RX = ffma2(xg[2], t2, RX);
      RXX = ffma2(xh[2], t2, RXX);
      RV = ffma2(xw[3], t3, RV);
      RX = ffma2(xg[3], t3, RX);
      RXX = ffma2(xh[3], t3, RXX);
      A = ffma2(yw[pr], RV, A);
      AY = ffma2(yg[pr], RV, AY);
      AYY = ffma2(yh[pr], RV, AYY);
      AX = ffma2(yw[pr], RX, AX);
      AXY = ffma2(yg[pr], RX, AXY);
      AXX = ffma2(yw[pr], RXX, AXX);
    }
    const float a = A.x + A.y, ax = AX.x + AX.y, ay = AY.x + AY.y;
    const float axx = AXX.x + AXX.y, axy = AXY.x + AXY.y, ayy = AYY.x + AYY.y;
    const float zw = Z.w[c], zg = Z.g[c], zh = Z.h[c];
    VG0 = ffma2(dup2(zw), make_float2(a, ax), VG0);
    G2H02 = ffma2(dup2(zg), make_float2(a, ax), G2H02);
    G1H11 = ffma2(dup2(zw), make_float2(ay, ayy), G1H11);
    H12H22 = ffma2(make_float2(zg, zh), make_float2(ay, a), H12H22);
    H00H01 = ffma2(dup2(zw), make_float2(axx, axy), H00H01);
  }
  r.v = VG0.x;
  r.g[0] = VG0.y;
  r.g[1] = G1H11.x;
  r.g[2] = G2H02.x;
  r.h[0] = H00H01.x;
  r.h[1] = H00H01.y;
  r.h[2] = G2H02.y;
  r.h[3] = G1H11.y;
  r.h[4] = H12H22.x;
  r.h[5] = H12H22.y;
}

// ------------------------------------------------------------ cell lookup

SRT_HD int wrap64(int64_t c, int n) {
  int64_t r = c % n;
  if (r < 0) r += n;
  return (int)r;
}

// c mod n in [0, n) by a float reciprocal, exact for |c| < 2^24 (every
// position FP32 resolves to a cell); any other c (a position made non-finite
// by non-finite field values) is clamped into range, so every tap index stays
// inside the array. Branch-free: selects only.
SRT_HD int wrap32(int c, int n, float invn) {
  const int q = (int)floorf((float)c * invn);
  int r = (int)((unsigned)c - (unsigned)q * (unsigned)n);
  r += r < 0 ? n : 0;
  r -= r >= n ? n : 0;
  r = r < 0 ? 0 : r;
  return r >= n ? n - 1 : r;
}

SRT_HD int64_t cell_base(const Geom& G, int cx, int cy, int cz) {
  return (int64_t)cx + G.px * (int64_t)cy + G.pxy * (int64_t)cz;
}

// The same voxel's index in a row-pair array.
SRT_HD int64_t cell_base_pair(const Geom& G, int cx, int cy, int cz) {
  return (int64_t)cx + G.px * (int64_t)cy + G.pxy2 * (int64_t)cz;
}

// FP64 / REF16 interpolation of one field at a double-precision position.
// IT is the arithmetic type (double for FP64, float for REF16); in REF16 the
// cell offset is float(x) - float(floor(x)) (snapshot-raytracer.cu:223-230).
template <typename IT, typename TapT>
SRT_HD void interp_std(const TapT* f, const Geom& G, double x, double y, double z, Tri<IT>& r) {
  const double fx = floor(x), fy = floor(y), fz = floor(z);
  const int64_t ix = (int64_t)fx, iy = (int64_t)fy, iz = (int64_t)fz;
  IT tx, ty, tz;
  if (sizeof(IT) == sizeof(float)) {
    tx = (IT)((float)x - (float)ix);
    ty = (IT)((float)y - (float)iy);
    tz = (IT)((float)z - (float)iz);
  } else {
    tx = (IT)(x - fx);
    ty = (IT)(y - fy);
    tz = (IT)(z - fz);
  }
  CRW<IT> X, Y, Z;
  cr_weights(tx, X);
  cr_weights(ty, Y);
  cr_weights(tz, Z);
  const int64_t base = cell_base(G, wrap64(ix, G.n[0]), wrap64(iy, G.n[1]), wrap64(iz, G.n[2]));
  tricubic<IT, TapT>(f, base, G.px, G.pxy, X, Y, Z, r);
}

// --------------------------------------------- right-hand side, FP64 / REF16

// Square root of the state type R (double, or the double-float dd).
SRT_HD double sqrt_r(double x) { return sqrt(x); }
SRT_HD dd sqrt_r(const dd& x) { return dd_sqrt(x); }

// Unit vectors n, e1, e2 of the full state y (snapshot-raytracer.cu:338-349).
// R: the state's real type (double; dd in the re-trace of flagged rays).
template <typename R>
SRT_HD void rhs_frame(const R* y, R* n, R* a, R* b) {
  const R rn = sqrt_r(y[3] * y[3] + y[4] * y[4] + y[5] * y[5]);
  const R ra = sqrt_r(y[6] * y[6] + y[7] * y[7] + y[8] * y[8]);
  const R rb = sqrt_r(y[9] * y[9] + y[10] * y[10] + y[11] * y[11]);
  for (int i = 0; i < 3; ++i) {
    n[i] = y[3 + i] / rn;
    a[i] = y[6 + i] / ra;
    b[i] = y[9 + i] / rb;
  }
}

// Sums over the B components of the right-hand side (snapshot-raytracer.cu:377-460):
// n.grad B, the e.n.grad B scalars, the tidal matrix and n . Laplacian B.
// The e_i.grad B vectors the reference also forms there are never used and
// are not computed.
template <typename IT, typename R = double>
struct BSums {
  IT val[3], ngB[3], e1ngB, e2ngB, nlap;
  IT T[6];  // xx, xy, xz, yy, yz, zz
  SRT_HD void clear() {
    for (int i = 0; i < 3; ++i) ngB[i] = 0;
    e1ngB = e2ngB = nlap = 0;
    for (int i = 0; i < 6; ++i) T[i] = 0;
  }
  // Adds component c's value, gradient and Hessian r.
  SRT_HD void add(int c, const Tri<IT>& r, const R* n, const R* a, const R* b) {
    val[c] = r.v;
    for (int i = 0; i < 3; ++i) ngB[i] = (IT)(ngB[i] + r.g[i] * n[c]);
    const R gn = r.g[0] * n[0] + r.g[1] * n[1] + r.g[2] * n[2];
    const R ga = r.g[0] * a[0] + r.g[1] * a[1] + r.g[2] * a[2];
    const R gb = r.g[0] * b[0] + r.g[1] * b[1] + r.g[2] * b[2];
    e1ngB = (IT)(e1ngB + 0.5 * a[c] * gn + 0.5 * n[c] * ga);
    e2ngB = (IT)(e2ngB + 0.5 * b[c] * gn + 0.5 * n[c] * gb);
    // H n for this component's Hessian (rows of the symmetric matrix)
    const R Hn0 = r.h[0] * n[0] + r.h[1] * n[1] + r.h[2] * n[2];
    const R Hn1 = r.h[1] * n[0] + r.h[3] * n[1] + r.h[4] * n[2];
    const R Hn2 = r.h[2] * n[0] + r.h[4] * n[1] + r.h[5] * n[2];
    const R Hn[3] = {Hn0, Hn1, Hn2};
    // T_ij += n_c H_ij - 1/2 (delta_ci (H n)_j + delta_cj (H n)_i)
    const int kIdx[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    for (int i = 0; i < 3; ++i)
      for (int j = i; j < 3; ++j) {
        R d = r.h[kIdx[i][j]] * n[c];
        if (i == c) d -= 0.5 * Hn[j];
        if (j == c) d -= 0.5 * Hn[i];
        T[kIdx[i][j]] = (IT)(T[kIdx[i][j]] + d);
      }
    nlap = (IT)(nlap + (r.h[0] + r.h[3] + r.h[5]) * n[c]);
  }
};

// The four quotients of the dA > 1/2 branch, each divided where it is formed
// (the re-trace's lane groups share them out instead: GroupDiv).
struct LocalDiv {
  template <typename R>
  SRT_HD void operator()(const R* num, const R* den, R* quo) const {
    for (int j = 0; j < 4; ++j) quo[j] = num[j] / den[j];
  }
};

// The right-hand side from the frame, the B sums and phi's interpolation p
// (snapshot-raytracer.cu:462-509).
template <typename IT, typename R = double, typename Div = LocalDiv>
SRT_HD void rhs_finish(const R* y, const R* n, const R* a, const R* b, const BSums<IT, R>& B, const Tri<IT>& p,
                       R* dy, const Div& div = Div()) {
  const R dA = y[12], dAp = y[13], s1 = y[14], s2 = y[15], el1 = y[16], el2 = y[17];
  const R phi1 = 1.0 + 2.0 * p.v;
  for (int i = 0; i < 3; ++i) dy[i] = -n[i] * phi1 - B.val[i];
  // -P_perp v with P_perp = n n^T - I  ->  v - n (n.v)
  const R v0 = 2.0 * p.g[0] + B.ngB[0], v1 = 2.0 * p.g[1] + B.ngB[1], v2 = 2.0 * p.g[2] + B.ngB[2];
  const R nv = n[0] * v0 + n[1] * v1 + n[2] * v2;
  dy[3] = v0 - n[0] * nv;
  dy[4] = v1 - n[1] * nv;
  dy[5] = v2 - n[2] * nv;
  const R ag = a[0] * p.g[0] + a[1] * p.g[1] + a[2] * p.g[2];
  const R bg = b[0] * p.g[0] + b[1] * p.g[1] + b[2] * p.g[2];
  for (int i = 0; i < 3; ++i) {
    dy[6 + i] = -2.0 * n[i] * ag - n[i] * B.e1ngB;
    dy[9 + i] = -2.0 * n[i] * bg - n[i] * B.e2ngB;
  }
  const R L = n[0] * p.g[0] + n[1] * p.g[1] + n[2] * p.g[2] +
                   0.25 * (n[0] * B.ngB[0] + n[1] * B.ngB[1] + n[2] * B.ngB[2]);
  // P_perp : H = n^T H n - tr H
  const R nHn = n[0] * n[0] * p.h[0] + n[1] * n[1] * p.h[3] + n[2] * n[2] * p.h[5] +
                     2.0 * (n[0] * n[1] * p.h[1] + n[0] * n[2] * p.h[2] + n[1] * n[2] * p.h[4]);
  const R PH = nHn - (p.h[0] + p.h[3] + p.h[5]);
  dy[12] = -dAp;
  dy[13] = -4.0 * dAp * L - PH * dA + 0.5 * B.nlap * dA;
  // effective tidal matrix H + T/2 projected on the shear basis
  IT He[6];
  for (int i = 0; i < 6; ++i) He[i] = (IT)(p.h[i] + 0.5 * B.T[i]);
  const R S1 = (a[0] * a[0] - b[0] * b[0]) * He[0] + (a[1] * a[1] - b[1] * b[1]) * He[3] +
                    (a[2] * a[2] - b[2] * b[2]) * He[5] +
                    2.0 * ((a[0] * a[1] - b[0] * b[1]) * He[1] + (a[0] * a[2] - b[0] * b[2]) * He[2] +
                           (a[1] * a[2] - b[1] * b[2]) * He[4]);
  const R S2 = 2.0 * (a[0] * b[0] * He[0] + a[1] * b[1] * He[3] + a[2] * b[2] * He[5]) +
                    2.0 * ((a[0] * b[1] + a[1] * b[0]) * He[1] + (a[0] * b[2] + a[2] * b[0]) * He[2] +
                           (a[1] * b[2] + a[2] * b[1]) * He[4]);
  dy[14] = 4.0 * s1 * L + S1 * dA * dA;
  dy[15] = 4.0 * s2 * L + S2 * dA * dA;
  // the dA > 1/2 branch's terms, formed either way and selected (the same
  // operations when it is taken; where dA = 0 they are not finite and not
  // selected)
  const bool on = dA > 0.5;
  const R dA2 = dA * dA;
  const R q = sqrt_r(4.0 + el1 * el1 + el2 * el2);
  const R num[4] = {s1 * s1 + s2 * s2, -2.0 * s1 * q, -2.0 * s2 * q, -(s1 * el2 - s2 * el1)};
  const R den[4] = {dA2 * dA, dA2, dA2, dA2 * (2.0 + q)};
  R quo[4];
  div(num, den, quo);
  const R zero(0.0);
  const R t13 = dy[13] + quo[0];
  dy[13] = on ? t13 : dy[13];
  dy[16] = on ? quo[1] : zero;
  dy[17] = on ? quo[2] : zero;
  dy[18] = on ? quo[3] : zero;
}

// 19-component right-hand side on the full state y (FP64 or REF16 arithmetic).
// State: 0-2 x, 3-5 n, 6-8 e1, 9-11 e2, 12 dA, 13 dA', 14-15 sigma1/2,
// 16-17 ellipticity1/2, 18 rotation (snapshot-raytracer.cu:317-335).
template <int MODE>
SRT_HD void rhs_std(const double* y, double* dy, const FieldPtrs& F, const Geom& G) {
  typedef typename std::conditional<MODE == kREF16, float, double>::type IT;
  double n[3], a[3], b[3];
  rhs_frame(y, n, a, b);
  BSums<IT> B;
  B.clear();
#pragma unroll 1
  for (int c = 0; c < 3; ++c) {
    const double off[3] = {c == 0 ? 0.5 : 0.0, c == 1 ? 0.5 : 0.0, c == 2 ? 0.5 : 0.0};
    Tri<IT> r;
    if (MODE == kREF16) {
      interp_std<IT, __half>(F.bh[c], G, y[0] - off[0], y[1] - off[1], y[2] - off[2], r);
      tri_scale(r, (IT)(1.0 / 134217728.0));  // taps hold B * 2^27
    } else {
      interp_std<IT, float>(F.b[c], G, y[0] - off[0], y[1] - off[1], y[2] - off[2], r);
    }
    B.add(c, r, n, a, b);
  }
  Tri<IT> p;
  interp_std<IT, float>(F.phi, G, y[0], y[1], y[2], p);
  rhs_finish<IT>(y, n, a, b, B, p, dy);
}

// ------------------------------------------------------------ ray geometry

struct RayDir {  // sin/cos of the pixel centre's colatitude and longitude
  double st, ct, sp, cp;
};

SRT_HD RayDir ray_dir(double theta, double phi) {
  RayDir d;
  d.st = sin(theta);
  d.ct = cos(theta);
  d.sp = sin(phi);
  d.cp = cos(phi);
  return d;
}

// Deflection from the displacement X = x_final - x_observer: the change of
// direction X/|X| - r_hat projected on e_theta and on (sin phi, -cos phi, 0)
// (snapshot-raytracer.cu:566-582).
SRT_HD void extract_deflection(const RayDir& d, double X0, double X1, double X2, float* d1,
                               float* d2) {
  const double nrm = sqrt(X0 * X0 + X1 * X1 + X2 * X2);
  const double D0 = X0 / nrm - d.st * d.cp;
  const double D1 = X1 / nrm - d.st * d.sp;
  const double D2 = X2 / nrm - d.ct;
  *d1 = (float)(D0 * d.ct * d.cp + D1 * d.ct * d.sp - D2 * d.st);
  *d2 = (float)(D0 * d.sp - D1 * d.cp);
}

// ----------------------------------------------------- ray driver, FP64/REF16

// Initial state of the ray (snapshot-raytracer.cu:560).
SRT_HD void init_std(const RayDir& d, const Geom& G, double* y) {
  y[0] = (double)G.n[0] * 0.5;
  y[1] = (double)G.n[1] * 0.5;
  y[2] = (double)G.n[2] * 0.5;
  y[3] = -d.st * d.cp;
  y[4] = -d.st * d.sp;
  y[5] = -d.ct;
  y[6] = d.ct * d.cp;
  y[7] = d.ct * d.sp;
  y[8] = -d.st;
  y[9] = d.sp;
  y[10] = -d.cp;
  y[11] = 0.0;
  y[12] = 0.0;
  y[13] = -1.0;
  for (int j = 14; j < 19; ++j) y[j] = 0.0;
}

// One RK4 step of h = 1 (snapshot-raytracer.cu:524-549); when ks is given,
// the stage derivatives k1, k2, k3 are stored there (3 x 19).
template <int MODE>
SRT_HD void step_std(const FieldPtrs& F, const Geom& G, double* y, double* ks) {
  double acc[19], k[19], ys[19];
  for (int j = 0; j < 19; ++j) k[j] = 0.0;
#pragma unroll 1
  for (int st = 0; st < 4; ++st) {
    const double c = (st == 3) ? 1.0 : 0.5;
    for (int j = 0; j < 19; ++j) ys[j] = (st == 0) ? y[j] : y[j] + c * k[j];
    rhs_std<MODE>(ys, k, F, G);
    if (ks && st < 3)
      for (int j = 0; j < 19; ++j) ks[19 * st + j] = k[j];
    for (int j = 0; j < 19; ++j) acc[j] = (st == 0) ? k[j] : ((st < 3) ? acc[j] + 2.0 * k[j] : acc[j]);
  }
  for (int j = 0; j < 19; ++j) y[j] += (acc[j] + k[j]) / 6.0;
}

// The six maps from the final state (snapshot-raytracer.cu:566-582).
SRT_HD void extract_std(const RayDir& d, const Geom& G, const double* y, float out[6]) {
  out[0] = (float)y[12];
  out[1] = (float)y[16];
  out[2] = (float)y[17];
  out[3] = (float)y[18];
  extract_deflection(d, y[0] - (double)G.n[0] * 0.5, y[1] - (double)G.n[1] * 0.5, y[2] - (double)G.n[2] * 0.5,
                     &out[4], &out[5]);
}

template <int MODE>
SRT_HD void trace_ray_std(const FieldPtrs& F, const Geom& G, const RayDir& d, int n_steps, float out[6]) {
  double y[19];
  init_std(d, G, y);
#pragma unroll 1
  for (int step = 0; step < n_steps; ++step) step_std<MODE>(F, G, y, nullptr);
  extract_std(d, G, y, out);
}

// ------------------------------------------- double-float (dd) ray driver
//
// The FP64 scheme above in double-float arithmetic (srt_dd.cuh), for the
// re-trace of the MIXED form's flagged rays: the same state, stages and
// right-hand side (rhs_frame, BSums, rhs_finish instantiated with dd), the
// interpolation's dot products accumulated in the compensated form of Ogita,
// Rump and Oishi ("Accurate sum and dot product", 2005). The trajectory stays
// ~1e-14 from the FP64 one, far inside the guard's margin.

// Compensated accumulator: s + c, products added with their rounding errors.
struct DdAcc {
  float s = 0.f, c = 0.f;
  SRT_HD void add(const dd& w, float x) {  // += w * x
    const float p = w.hi * x;
    const float e = fmaf(w.hi, x, -p);
    float t, q;
    dd_two_sum(s, p, t, q);
    s = t;
    c += fmaf(w.lo, x, e + q);
  }
  SRT_HD void add(const dd& w, const dd& x) {  // += w * x
    const float p = w.hi * x.hi;
    const float e = fmaf(w.hi, x.hi, -p);
    float t, q;
    dd_two_sum(s, p, t, q);
    s = t;
    c += fmaf(w.hi, x.lo, fmaf(w.lo, x.hi, e + q));
  }
  SRT_HD dd value() const {
    float h, l;
    dd_fast_two_sum(s, c, h, l);
    return dd(h, l);
  }
};

// tricubic<dd, float>: the same passes with compensated accumulation.
SRT_HD void tricubic_dd(const float* __restrict__ f, int64_t base, int64_t px, int64_t pxy, const CRW<dd>& X,
                        const CRW<dd>& Y, const CRW<dd>& Z, Tri<dd>& r) {
  DdAcc v, g0, g1, g2, h00, h01, h02, h11, h12, h22;
#pragma unroll 1
  for (int c = 0; c < 4; ++c) {
    DdAcc a, ay, ayy, ax, axy, axx;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const float* row = f + base + c * pxy + b * px;
      const float p[4] = {ldg(row), ldg(row + 1), ldg(row + 2), ldg(row + 3)};
      DdAcc rv, rx, rxx;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        rv.add(X.w[i], p[i]);
        rx.add(X.g[i], p[i]);
        rxx.add(X.h[i], p[i]);
      }
      const dd RV = rv.value(), RX = rx.value(), RXX = rxx.value();
      a.add(Y.w[b], RV);
      ay.add(Y.g[b], RV);
      ayy.add(Y.h[b], RV);
      ax.add(Y.w[b], RX);
      axy.add(Y.g[b], RX);
      axx.add(Y.w[b], RXX);
    }
    const dd A = a.value(), AY = ay.value(), AYY = ayy.value(), AX = ax.value(), AXY = axy.value(),
             AXX = axx.value();
    v.add(Z.w[c], A);
    g0.add(Z.w[c], AX);
    g1.add(Z.w[c], AY);
    g2.add(Z.g[c], A);
    h00.add(Z.w[c], AXX);
    h01.add(Z.w[c], AXY);
    h02.add(Z.g[c], AX);
    h11.add(Z.w[c], AYY);
    h12.add(Z.g[c], AY);
    h22.add(Z.h[c], A);
  }
  r.v = v.value();
  r.g[0] = g0.value();
  r.g[1] = g1.value();
  r.g[2] = g2.value();
  r.h[0] = h00.value();
  r.h[1] = h01.value();
  r.h[2] = h02.value();
  r.h[3] = h11.value();
  r.h[4] = h12.value();
  r.h[5] = h22.value();
}

// interp_std<double, float> in dd: cell from the dd position, dd offsets.
SRT_HD void interp_dd(const float* f, const Geom& G, const dd& x, const dd& y, const dd& z, Tri<dd>& r) {
  const dd fx = dd_floor(x), fy = dd_floor(y), fz = dd_floor(z);
  const int64_t ix = (int64_t)fx.hi + (int64_t)fx.lo, iy = (int64_t)fy.hi + (int64_t)fy.lo,
                iz = (int64_t)fz.hi + (int64_t)fz.lo;
  CRW<dd> X, Y, Z;
  cr_weights(x - fx, X);
  cr_weights(y - fy, Y);
  cr_weights(z - fz, Z);
  const int64_t base = cell_base(G, wrap64(ix, G.n[0]), wrap64(iy, G.n[1]), wrap64(iz, G.n[2]));
  tricubic_dd(f, base, G.px, G.pxy, X, Y, Z, r);
}

// rhs_std<kFP64> in dd.
SRT_HD void rhs_dd(const dd* y, dd* dy, const FieldPtrs& F, const Geom& G) {
  dd n[3], a[3], b[3];
  rhs_frame<dd>(y, n, a, b);
  BSums<dd, dd> B;
  B.clear();
  const dd half(0.5f);
#pragma unroll 1
  for (int c = 0; c < 3; ++c) {
    Tri<dd> r;
    interp_dd(F.b[c], G, c == 0 ? y[0] - half : y[0], c == 1 ? y[1] - half : y[1], c == 2 ? y[2] - half : y[2], r);
    B.add(c, r, n, a, b);
  }
  Tri<dd> p;
  interp_dd(F.phi, G, y[0], y[1], y[2], p);
  rhs_finish<dd, dd>(y, n, a, b, B, p, dy);
}

// init_std / extract_std in dd (the step is step_dd_group in srt_kernels.cu).
SRT_HD void init_dd(const RayDir& d, const Geom& G, dd* y) {
  double y64[19];
  init_std(d, G, y64);
  for (int j = 0; j < 19; ++j) y[j] = dd(y64[j]);
}


SRT_HD void extract_dd(const RayDir& d, const Geom& G, const dd* y, float out[6]) {
  double y64[19];
  for (int j = 0; j < 19; ++j) y64[j] = (double)y[j];
  extract_std(d, G, y64, out);
}

// -------------------------------------------------------------- MIXED mode

// Exact two-term sum a + b = s + e.
SRT_HD void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// Cells and offsets along one axis for the position x = th + lo (th, lo
// floats; x is their exact sum), on the centred grid (faces at integers) and
// on the grid staggered by -1/2 (faces at half-integers), and x's distance
// from the nearest face of either grid. Every decision and the distance are
// taken from a split of x that is exact up to the rounding of a remainder far
// below the cell-face guard: with fl = floor(th), s + e = (th - fl) + lo
// (two-sum) and u = s - floor(s), the fraction of x is u + e, where e also
// holds the rounding errors of th - fl and of u (nonzero only when th or s
// lies in (-1/2, 0)), so frac(x) - 1/2 = (u - 1/2) + e carries its exact sign. tc / ts: offsets from
// the cells' lower faces (rounded; tc may round to 1 within ~3e-8 of the upper
// face). dface: min(frac, 1 - frac, |frac - 1/2|), each with one rounding.
SRT_HD void locate_mixed(float th, float lo, int n, float invn, int& cc, float& tc, int& cs, float& ts,
                         float& dface) {
  const float fl = floorf(th);
  // th - fl is exact unless -1/2 < th < 0 (then fl = -1 and th + 1 rounds);
  // b is its rounding error (exact: a + fl is exact whenever a was rounded)
  const float a = th - fl;
  const float b = th - (a + fl);
  float s, e;
  two_sum(a, lo, s, e);
  e += b;  // rounded, but with the sign of the exact remainder
  float k = floorf(s);
  if (s == k && e < 0.f) k -= 1.f;  // frac(x) = 1 + e: the cell below
  // u = s - k in [0, 1], exact unless -1/2 < s < 0 (lo took x below the
  // face under th); its rounding error goes to e the same way
  const float u = s - k;
  e += s - (u + k);
  tc = u + e;
  const float v = (u - 0.5f) + e;   // frac(x) - 1/2 (u - 1/2 exact for u >= 1/4)
  // (summed as unsigned: a non-finite position converts to any int, and the
  // cell is then only required to land in range)
  const int c = (int)((unsigned)(int)fl + (unsigned)(int)k);
  const int cw = wrap32(c, n, invn);  // formed either way: a select, not a branch
  cc = (unsigned)c < (unsigned)n ? c : cw;
  const bool up = v >= 0.f;  // x - 1/2 lies in the same cell
  ts = up ? v : v + 1.f;
  cs = up ? cc : (cc == 0 ? n - 1 : cc - 1);
  dface = fminf(fminf(tc, (1.f - u) - e), fabsf(v));
}

struct MixedRay {
  float n0[3], a0[3], b0[3];  // FP32 bases of n, e1, e2 (straight-ray solution)
  float eta[3];               // |base|^2 - 1 of the three bases
  float dn0[3];               // FP64 direction minus its FP32 base (for the extraction)
};

// (1 + q)^(-1/2) - 1 without cancellation, q > -1: -q / (s (1 + s)) with
// s = (1 + q)^(1/2) (the numerator is q itself, the denominator ~2), no branch.
SRT_HD float rsqrt1p_m1(float q) {
  const float s = sqrtf(1.f + q);
  return -q / (s * (1.f + s));
}

// Unit vector of base + delta as (base + D): D = base (r - 1) + delta r with
// r = (1 + q)^(-1/2), q = |base + delta|^2 - 1 = eta + 2 base.delta + delta^2.
SRT_HD void unit_pert(const float* v0, const float* dv, float eta, float* D) {
  const float q = eta + 2.f * (v0[0] * dv[0] + v0[1] * dv[1] + v0[2] * dv[2]) +
                  (dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
  const float rm1 = rsqrt1p_m1(q);
  for (int i = 0; i < 3; ++i) D[i] = v0[i] * rm1 + dv[i] * (1.f + rm1);
}

// Quantities the B components contribute to the right-hand side
// (snapshot-raytracer.cu:377-460), accumulated component by component. With
// G the matrix of B's gradients (row C = grad B_C), ngB = G^T n and
// Gn = G n; the e.n.grad B scalars are e.G n / 2 + n.G e / 2
// = e.(Gn + ngB) / 2, formed once from these two vectors.
struct BAcc {
  float val[3], ngB[3], Gn[3], nlap, T[6];
};

// B component C interpolated at the position staggered by -1/2 along axis C,
// folded into the accumulators. C is a compile-time constant so n[C], a[C]
// and b[C] stay in registers.
template <int C, bool PAIR>
SRT_HD void add_b_component(const FieldPtrs& F, const Geom& G, const int* cc, const int* cs,
                            const float* ts, const CRW<float>& Cx, const CRW<float>& Cy, const CRW<float>& Cz,
                            const float* n, const float* a, const float* b, BAcc& A) {
  CRW<float> S;
  cr_weights_mixed(ts[C], S);
  const int cx = C == 0 ? cs[0] : cc[0], cy = C == 1 ? cs[1] : cc[1], cz = C == 2 ? cs[2] : cc[2];
  Tri<float> r;
  if (PAIR)
    tricubic_pair(PairRows{F.pr[C], cell_base_pair(G, cx, cy, cz), G.px, G.pxy2}, C == 0 ? S : Cx, C == 1 ? S : Cy,
                  C == 2 ? S : Cz, r);
  else
    tricubic_pair(SingleRows{F.b[C], cell_base(G, cx, cy, cz), G.px, G.pxy}, C == 0 ? S : Cx, C == 1 ? S : Cy,
                  C == 2 ? S : Cz, r);
  A.val[C] = r.v;
  for (int i = 0; i < 3; ++i) A.ngB[i] += r.g[i] * n[C];
  A.Gn[C] = r.g[0] * n[0] + r.g[1] * n[1] + r.g[2] * n[2];
  const float Hn[3] = {r.h[0] * n[0] + r.h[1] * n[1] + r.h[2] * n[2], r.h[1] * n[0] + r.h[3] * n[1] + r.h[4] * n[2],
                       r.h[2] * n[0] + r.h[4] * n[1] + r.h[5] * n[2]};
  // T_ij += n_C H_ij - 1/2 (delta_Ci (H n)_j + delta_Cj (H n)_i), ij in xx xy xz yy yz zz
  A.T[0] += r.h[0] * n[C] - (C == 0 ? Hn[0] : 0.f);
  A.T[1] += r.h[1] * n[C] - 0.5f * (C == 0 ? Hn[1] : (C == 1 ? Hn[0] : 0.f));
  A.T[2] += r.h[2] * n[C] - 0.5f * (C == 0 ? Hn[2] : (C == 2 ? Hn[0] : 0.f));
  A.T[3] += r.h[3] * n[C] - (C == 1 ? Hn[1] : 0.f);
  A.T[4] += r.h[4] * n[C] - 0.5f * (C == 1 ? Hn[2] : (C == 2 ? Hn[1] : 0.f));
  A.T[5] += r.h[5] * n[C] - (C == 2 ? Hn[2] : 0.f);
  A.nlap += (r.h[0] + r.h[3] + r.h[5]) * n[C];
}

// Perturbation right-hand side g = f(y0(s) + d) - f(y0(s)) (FP32). `s` is the
// affine parameter of the stage (step + 0, 1/2 or 1), d the stage state
// (delta components in the layout of rhs_std), x0 the observer.
// Cell-face guard. Catmull-Rom's Hessian jumps across cell faces, so where
// the FP32 and FP64 trajectories pass a face on different sides the maps of
// that ray differ by up to ~1% of their rms. The FP32 trajectory's distance
// from the FP64 one was measured on the GPU, stage by stage (a lockstep
// FP64 / MIXED kernel: 256^3 / 256 steps / 49k rays, 512^3 / 512 steps / 49k
// rays, 1024^3 / 1024 steps / 12k rays) against candidate bounds; the one that
// holds with the smallest margin is s Mn, the affine distance times the
// running maximum Mn = max |dn| of the direction perturbation:
// |x32 - x64| <= k (s Mn + 1e-3) with k below 1.6e-7 for 99% of the rays and
// below 3.3e-7 for all, at every length (a bound that also carries
// Mx = max |dx| needed k up to 5.5e-7 at 1024 steps and flags 2-3x more rays).
// A stage whose position lies within g = kFaceGuardRel (s Mn + kFaceGuardFloor)
// of a cell face (either face, centred or staggered grid) marks the ray for
// an FP64 re-trace.
constexpr float kFaceGuardRel = 4e-7f;
constexpr float kFaceGuardFloor = 1e-3f;
// No guard is needed for the dA > 1/2 switch (snapshot-raytracer.cu:497): dA
// passes 1/2 inside the first step, where dA - 1/2 at the midpoint stages is
// either exactly 0 in both precisions (the switch is off in both) or ~k2/2 ~
// n.grad phi ~ 1e-5 with a relative FP32 error ~1e-7, so the two agree on its
// sign; and were they to differ, the switched terms are proportional to the
// shear, which is 0 at the start of the ray.

// Per-ray guard state: the flag, and (through m, two floats the caller
// provides; the trace kernel keeps them in shared memory, out of the register
// budget) the running maximum Mn = max |dn| taken at the start of each step
// and the smallest distance dmin of the step's stage positions from a cell
// face. A step is flagged when dmin < kFaceGuardRel (s_end Mn +
// kFaceGuardFloor), s_end the step's end. Guard{} (m null) is disabled.
struct Guard {
  bool near = false;
  float* m = nullptr;
  SRT_HD void begin_step(const float* y) {
    m[0] = fmaxf(m[0], fmaxf(fabsf(y[3]), fmaxf(fabsf(y[4]), fabsf(y[5]))));
    m[1] = 1.f;
  }
  // a stage's smallest distance from a face
  SRT_HD void face(float d) {
    if (m) m[1] = fminf(m[1], d);
  }
  SRT_HD void end_step(int step) { near |= m[1] < kFaceGuardRel * ((float)(step + 1) * m[0] + kFaceGuardFloor); }
};

template <bool PAIR>
SRT_HD void rhs_mixed(const float* d, float s, const MixedRay& R, const FieldPtrs& F, const Geom& G,
                      const float* x0, float* g, Guard& gd) {
  float Dn[3], Da[3], Db[3];
  unit_pert(R.n0, d + 3, R.eta[0], Dn);
  unit_pert(R.a0, d + 6, R.eta[1], Da);
  unit_pert(R.b0, d + 9, R.eta[2], Db);
  float n[3], a[3], b[3];
  for (int i = 0; i < 3; ++i) {
    n[i] = R.n0[i] + Dn[i];
    a[i] = R.a0[i] + Da[i];
    b[i] = R.b0[i] + Db[i];
  }
  // ray position x0 - s n0 + d_x per axis as th + lo with th + lo exact
  int cc[3], cs[3];
  float tc[3], ts[3], df[3];
  for (int i = 0; i < 3; ++i) {
    const float p = s * R.n0[i];
    const float pe = fmaf(s, R.n0[i], -p);
    float th, tl;
    two_sum(x0[i], -p, th, tl);
    const float lo = (tl - pe) + d[i];
    locate_mixed(th, lo, G.n[i], G.invn[i], cc[i], tc[i], cs[i], ts[i], df[i]);
  }
  // at s = 0 the ray sits exactly on the observer (a grid node, offsets
  // exactly 0) in both precisions, so no cell choice can differ there
  gd.face(s > 0.f ? fminf(fminf(df[0], df[1]), df[2]) : 1.f);
  CRW<float> Cx, Cy, Cz;  // centred weights, shared by phi and two axes of each B component
  cr_weights_mixed(tc[0], Cx);
  cr_weights_mixed(tc[1], Cy);
  cr_weights_mixed(tc[2], Cz);
  BAcc A;
  A.ngB[0] = A.ngB[1] = A.ngB[2] = 0.f;
  A.nlap = 0.f;
  for (int i = 0; i < 6; ++i) A.T[i] = 0.f;
  add_b_component<0, PAIR>(F, G, cc, cs, ts, Cx, Cy, Cz, n, a, b, A);
  add_b_component<1, PAIR>(F, G, cc, cs, ts, Cx, Cy, Cz, n, a, b, A);
  // phi between the second and third B components: the same values in any
  // order (the B sums keep theirs), and this one schedules best (1.0 % over
  // phi last, 3 % over phi first, on the 1024^3 trace)
  Tri<float> p;
  if (PAIR)
    tricubic_pair(PairRows{F.pr[3], cell_base_pair(G, cc[0], cc[1], cc[2]), G.px, G.pxy2}, Cx, Cy, Cz, p);
  else
    tricubic_pair(SingleRows{F.phi, cell_base(G, cc[0], cc[1], cc[2]), G.px, G.pxy}, Cx, Cy, Cz, p);
  add_b_component<2, PAIR>(F, G, cc, cs, ts, Cx, Cy, Cz, n, a, b, A);

  const float dA = s + d[12];
  const float dAp = d[13] - 1.f;
  const float s1 = d[14], s2 = d[15], el1 = d[16], el2 = d[17];
  // x: f = -n (1 + 2 phi) - B, f0 = -n0
  for (int i = 0; i < 3; ++i) g[i] = -Dn[i] - 2.f * p.v * n[i] - A.val[i];
  const float v0 = 2.f * p.g[0] + A.ngB[0], v1 = 2.f * p.g[1] + A.ngB[1], v2 = 2.f * p.g[2] + A.ngB[2];
  const float nv = n[0] * v0 + n[1] * v1 + n[2] * v2;
  g[3] = v0 - n[0] * nv;
  g[4] = v1 - n[1] * nv;
  g[5] = v2 - n[2] * nv;
  // 2 e.grad phi + e.n.grad B = e.(2 grad phi + (Gn + ngB) / 2)
  float w[3];
  for (int i = 0; i < 3; ++i) w[i] = 2.f * p.g[i] + 0.5f * (A.Gn[i] + A.ngB[i]);
  const float aw = a[0] * w[0] + a[1] * w[1] + a[2] * w[2];
  const float bw = b[0] * w[0] + b[1] * w[1] + b[2] * w[2];
  for (int i = 0; i < 3; ++i) {
    g[6 + i] = -n[i] * aw;
    g[9 + i] = -n[i] * bw;
  }
  const float L = n[0] * p.g[0] + n[1] * p.g[1] + n[2] * p.g[2] +
                  0.25f * (n[0] * A.ngB[0] + n[1] * A.ngB[1] + n[2] * A.ngB[2]);
  const float nHn = n[0] * n[0] * p.h[0] + n[1] * n[1] * p.h[3] + n[2] * n[2] * p.h[5] +
                    2.f * (n[0] * n[1] * p.h[1] + n[0] * n[2] * p.h[2] + n[1] * n[2] * p.h[4]);
  const float PH = nHn - (p.h[0] + p.h[3] + p.h[5]);
  g[12] = -d[13];  // f = -dA' = 1 - d13, f0 = 1
  g[13] = -4.f * dAp * L - PH * dA + 0.5f * A.nlap * dA;
  float He[6];
  for (int i = 0; i < 6; ++i) He[i] = p.h[i] + 0.5f * A.T[i];
  // S1 = a.He a - b.He b, S2 = 2 a.He b (He symmetric)
  const float Ha[3] = {He[0] * a[0] + He[1] * a[1] + He[2] * a[2], He[1] * a[0] + He[3] * a[1] + He[4] * a[2],
                       He[2] * a[0] + He[4] * a[1] + He[5] * a[2]};
  const float Hb[3] = {He[0] * b[0] + He[1] * b[1] + He[2] * b[2], He[1] * b[0] + He[3] * b[1] + He[4] * b[2],
                       He[2] * b[0] + He[4] * b[1] + He[5] * b[2]};
  const float S1 = (a[0] * Ha[0] + a[1] * Ha[1] + a[2] * Ha[2]) - (b[0] * Hb[0] + b[1] * Hb[1] + b[2] * Hb[2]);
  const float S2 = 2.f * (a[0] * Hb[0] + a[1] * Hb[1] + a[2] * Hb[2]);
  const float dA2 = dA * dA;
  g[14] = 4.f * s1 * L + S1 * dA2;
  g[15] = 4.f * s2 * L + S2 * dA2;
  // dA > 1/2  <=>  d12 > 1/2 - s (exact for the stage values of s); the
  // branch's terms are formed either way and selected (no branch in the
  // right-hand side; where dA = 0 they are not finite and not selected)
  const bool on = d[12] > 0.5f - s;
  const float q = sqrtf(4.f + el1 * el1 + el2 * el2);
  const float idA2 = 1.f / dA2;
  const float t13 = g[13] + (s1 * s1 + s2 * s2) * idA2 / dA;
  g[13] = on ? t13 : g[13];
  g[16] = on ? -2.f * s1 * q * idA2 : 0.f;
  g[17] = on ? -2.f * s2 * q * idA2 : 0.f;
  g[18] = on ? -(s1 * el2 - s2 * el1) * idA2 / (2.f + q) : 0.f;
}

// Number of leading state components accumulated with a compensation term
// (all of them). The ray position and direction matter most: the position's
// increments are ~1e-4 of its size after a few hundred steps, and any error in
// either moves the trajectory, which changes where the ray crosses cell faces
// (Catmull-Rom's Hessian jumps there); rounding the direction alone doubles the
// deflection error and raises the rate of such crossings.
constexpr int kCompensated = 19;
// Floats of one stored MIXED state: the 19 components and the compensations.
constexpr int kMixedState = 19 + kCompensated;

SRT_HD void mixed_observer(const Geom& G, float* x0) {
  for (int i = 0; i < 3; ++i) x0[i] = (float)((double)G.n[i] * 0.5);
}

// Straight-ray bases of the ray and the initial perturbation state: y holds
// the 19 components followed by the kCompensated compensation terms.
SRT_HD void init_mixed(const RayDir& d, MixedRay& R, float* y) {
  const double n64[3] = {-d.st * d.cp, -d.st * d.sp, -d.ct};
  const double a64[3] = {d.ct * d.cp, d.ct * d.sp, -d.st};
  const double b64[3] = {d.sp, -d.cp, 0.0};
  double qn = -1.0, qa = -1.0, qb = -1.0;
  for (int i = 0; i < 3; ++i) {
    R.n0[i] = (float)n64[i];
    R.a0[i] = (float)a64[i];
    R.b0[i] = (float)b64[i];
    R.dn0[i] = (float)(n64[i] - (double)R.n0[i]);
    y[3 + i] = R.dn0[i];
    y[6 + i] = (float)(a64[i] - (double)R.a0[i]);
    y[9 + i] = (float)(b64[i] - (double)R.b0[i]);
    qn += (double)R.n0[i] * (double)R.n0[i];
    qa += (double)R.a0[i] * (double)R.a0[i];
    qb += (double)R.b0[i] * (double)R.b0[i];
    y[i] = 0.f;
  }
  R.eta[0] = (float)qn;
  R.eta[1] = (float)qa;
  R.eta[2] = (float)qb;
  for (int j = 12; j < kMixedState; ++j) y[j] = 0.f;
}

// Stage input y + c k of the perturbation state (compensations folded in),
// two components per packed instruction.
SRT_HD void mixed_stage(const float* y, const float* k, float c, float* ys) {
  static_assert(kCompensated == 19, "packed stage assumes every component is compensated");
  const float2 c2 = dup2(c);
#pragma unroll
  for (int j = 0; j < 18; j += 2) {
    const float2 r = fadd2(make_float2(y[j], y[j + 1]),
                           ffma2(c2, make_float2(k[j], k[j + 1]), make_float2(y[19 + j], y[20 + j])));
    ys[j] = r.x;
    ys[j + 1] = r.y;
  }
  ys[18] = y[18] + (y[37] + c * k[18]);
}

// One RK4 step from affine parameter `step`; when us is given, the four stage
// inputs (the perturbation states the right-hand side is evaluated at, with
// the compensations folded in) are stored there: component j of stage st at
// us[(19 st + j) * stride]. gd.near is set when a stage of the step came
// within the guards above.
template <bool PAIR = false>
SRT_HD void step_mixed(const MixedRay& R, const FieldPtrs& F, const Geom& G, const float* x0, int step, float* y,
                       float* us, int64_t stride, Guard& gd) {
  float k[19], acc[19], ys[19];
  for (int j = 0; j < 19; ++j) k[j] = acc[j] = 0.f;
  const float s0 = (float)step;
#pragma unroll 1
  for (int st = 0; st < 4; ++st) {
    const float c = (st == 0) ? 0.f : ((st == 3) ? 1.f : 0.5f);
    mixed_stage(y, k, c, ys);
    if (us)
      for (int j = 0; j < 19; ++j) st_stream(us + (19 * st + j) * stride, ys[j]);
    rhs_mixed<PAIR>(ys, s0 + c, R, F, G, x0, k, gd);
    {  // acc = k1 + 2 k2 + 2 k3 with weights 1, 2, 2, 0 on a zeroed accumulator
       // (stage 4's k is added at the update): the same FMAs where a stage
       // adds, exact no-ops where it does not, and no branch
      const float w = st == 0 ? 1.f : (st < 3 ? 2.f : 0.f);
#pragma unroll
      for (int j = 0; j < 18; j += 2) {
        const float2 r = ffma2(dup2(w), make_float2(k[j], k[j + 1]), make_float2(acc[j], acc[j + 1]));
        acc[j] = r.x;
        acc[j + 1] = r.y;
      }
      acc[18] = w * k[18] + acc[18];
    }
  }
  // y += (k1 + 2 k2 + 2 k3 + k4) / 6 with the rounding error of each sum kept
  // in the compensation (two-sum), two components per packed instruction
#pragma unroll
  for (int j = 0; j < 18; j += 2) {
    const float2 a = make_float2(y[j], y[j + 1]);
    const float2 b = fmul2(fadd2(make_float2(acc[j], acc[j + 1]), make_float2(k[j], k[j + 1])), dup2(1.f / 6.f));
    const float2 sm = fadd2(a, b);  // two-sum: sm + e = a + b exactly
    const float2 bb = fsub2(sm, a);
    const float2 e = fadd2(fsub2(a, fsub2(sm, bb)), fsub2(b, bb));
    const float2 yc = fadd2(make_float2(y[19 + j], y[20 + j]), e);
    y[j] = sm.x;
    y[j + 1] = sm.y;
    y[19 + j] = yc.x;
    y[20 + j] = yc.y;
  }
  {
    float sum, err;
    two_sum(y[18], (acc[18] + k[18]) * (1.f / 6.f), sum, err);
    y[18] = sum;
    y[37] += err;
  }
}

// Extraction in FP32 on the perturbation: the displacement is
// X = -S n0 + dx = S (-n0 + u), u = dx / S; X/|X| - r_hat = dn0 + u (1 + c) - n0 c
// with c = |(-n0 + u)|^-1 - 1 and r_hat = -(n0 + dn0) (snapshot-raytracer.cu:566-582).
SRT_HD void extract_mixed(const MixedRay& R, int n_steps, const float* y, float out[6]) {
  const float S = (float)n_steps;
  float u[3];
  for (int i = 0; i < 3; ++i) u[i] = (y[i] + y[19 + i]) / S;
  const float q = R.eta[0] - 2.f * (R.n0[0] * u[0] + R.n0[1] * u[1] + R.n0[2] * u[2]) +
                  (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
  const float cc = rsqrt1p_m1(q);
  float D[3];
  for (int i = 0; i < 3; ++i) D[i] = R.dn0[i] + u[i] * (1.f + cc) - R.n0[i] * cc;
  out[4] = D[0] * R.a0[0] + D[1] * R.a0[1] + D[2] * R.a0[2];
  out[5] = D[0] * R.b0[0] + D[1] * R.b0[1] + D[2] * R.b0[2];
  float dsum, derr;
  two_sum(S, y[12], dsum, derr);
  out[0] = dsum + derr;
  out[1] = y[16];
  out[2] = y[17];
  out[3] = y[18];
}

// Returns true when the ray came within the guards (its FP64 trace may
// differ by a cell choice; the caller re-traces it in FP64).
template <bool PAIR = false>
SRT_HD bool trace_ray_mixed(const FieldPtrs& F, const Geom& G, const RayDir& d, int n_steps, float out[6],
                            float* guard_m) {
  MixedRay R;
  float y[kMixedState], x0[3];
  mixed_observer(G, x0);
  init_mixed(d, R, y);
  Guard gd;
  gd.m = guard_m;
  gd.m[0] = 0.f;
#pragma unroll 1
  for (int step = 0; step < n_steps; ++step) {
    gd.begin_step(y);
    step_mixed<PAIR>(R, F, G, x0, step, y, nullptr, 0, gd);
    gd.end_step(step);
  }
  extract_mixed(R, n_steps, y, out);
  return gd.near;
}

// Ray direction of a RING pixel centre (FP64: cos/sin of the colatitude from
// the ring geometry, sin/cos of pi * u for the longitude).
SRT_HD RayDir ray_dir_pix(int64_t nside, int64_t ring) {
  double z, st, u;
  hp_ring_zu(nside, ring, &z, &st, &u);
  RayDir d;
  d.st = st;
  d.ct = z;
#if defined(__CUDA_ARCH__)
  sincospi(u, &d.sp, &d.cp);
#else
  d.sp = sin(3.141592653589793238462643383279502884 * u);
  d.cp = cos(3.141592653589793238462643383279502884 * u);
#endif
  return d;
}

}  // namespace srt
