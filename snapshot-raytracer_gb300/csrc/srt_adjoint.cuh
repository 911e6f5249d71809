// srt_adjoint.cuh — reverse mode (vector-Jacobian product) of one evaluation of
// the tracer's right-hand side (snapshot-raytracer.cu:315-510), for the vjp of
// the maps with respect to the phi and B grids.
//
// The reverse sweep of an RK4 step (snapshot-raytracer.cu:524-549) needs, for
// each stage input u and output cotangent fb, ub = J(u)^T fb together with the
// cotangents of the grid values the stage read. Derived by hand from the
// forward computation in srt_scheme.cuh:
//   * every intermediate cotangent of the right-hand side (of L = n.g + n.ngB/4,
//     of P_perp:H, of the shear projections S1/S2, of the tidal matrix T, of
//     n.lap B, n.grad B and the e.n.grad B scalars, of phi, grad phi, Hess phi
//     and of the B values) depends on fb and on the state only, so each field's
//     cotangent (value, gradient, Hessian) is known before the field is read;
//   * one fused pass per field then interpolates value, gradient, Hessian and
//     the ten third derivatives (the position cotangent needs d/dx of the
//     Hessian), scatters the 64 tap cotangents into the gradient grid, and
//     adds the field's share of the state cotangents;
//   * the terms that need sums over fields (v = 2g + n.grad B, L, P_perp:H,
//     the effective tidal matrix) are added after the four passes.
// Catmull-Rom's third derivative is piecewise constant: weights (-3, 9, -9, 3).
#pragma once
#include <type_traits>
#include "srt_scheme.cuh"

namespace srt {

template <typename T>
struct CRW4 {  // Catmull-Rom weights for value and d/dt .. d3/dt3
  T w[4], g[4], h[4], k[4];
};

// FP32 (the MIXED form) takes the forward's Horner-form weights.
template <typename T>
SRT_HD void cr_weights4(T t, CRW4<T>& c) {
  CRW<T> b;
  if constexpr (sizeof(T) == sizeof(float))
    cr_weights_mixed(t, b);
  else
    cr_weights(t, b);
  for (int i = 0; i < 4; ++i) {
    c.w[i] = b.w[i];
    c.g[i] = b.g[i];
    c.h[i] = b.h[i];
  }
  c.k[0] = T(-3);
  c.k[1] = T(9);
  c.k[2] = T(-9);
  c.k[3] = T(3);
}

// ---------------------------------------------------------- accumulators

// Where the tap cotangents go: one call per 4-tap x-row of a tricubic
// footprint (padded index `row` of its first tap). Three flavours:
//   AccF32    FP32 atomics into a row-expanded grid: entry r (a float4) holds
//             the four tap contributions of rows starting at padded index r,
//             so one 16-byte vector atomic carries a whole row; the fold
//             kernel adds entry q.x + (q-1).y + (q-2).z + (q-3).w per voxel;
//   AccF64    FP64 atomics into a halo-padded grid (one per tap);
//   AccFixed  64-bit fixed point into a halo-padded grid (order-independent,
//             so repeated runs give identical bits).
// A null grid (gradient not requested) ignores the contributions, and the
// passes skip forming them (active() is false).
struct AccF32 {
  float4* g;
  SRT_HD bool active() const { return g != nullptr; }
  SRT_HD void add_row(int64_t row, float c0, float c1, float c2, float c3) const {
    if (!g) return;
#if defined(__CUDA_ARCH__)
    atomicAdd(g + row, make_float4(c0, c1, c2, c3));
#else
    g[row].x += c0;
    g[row].y += c1;
    g[row].z += c2;
    g[row].w += c3;
#endif
  }
};

struct AccF64 {
  double* g;
  SRT_HD bool active() const { return g != nullptr; }
  SRT_HD void add(int64_t i, double v) const {
#if defined(__CUDA_ARCH__)
    atomicAdd(g + i, v);
#else
    g[i] += v;
#endif
  }
  SRT_HD void add_row(int64_t row, double c0, double c1, double c2, double c3) const {
    if (!g) return;
    add(row, c0);
    add(row + 1, c1);
    add(row + 2, c2);
    add(row + 3, c3);
  }
};

// Fixed point with kFixedScale = 2^32 units per unit of gradient; |gradient|
// per voxel must stay below 2^31. Contributions are rounded to the nearest
// unit before the integer addition, so the result does not depend on the
// order of the additions. A contribution of magnitude 2^30 or more (or one
// that is not finite) sets *ovf, where the integer sum may already have
// wrapped; the fold kernel sets it too for a folded |gradient| >= 2^30, and
// srt_vjp then fails with SRT_ERR_OVERFLOW instead of returning wrapped values.
constexpr double kFixedScale = 4294967296.0;
constexpr double kFixedLimit = 1073741824.0;  // 2^30 units of gradient

struct AccFixed {
  unsigned long long* g;
  unsigned* ovf = nullptr;
  SRT_HD bool active() const { return g != nullptr; }
  SRT_HD void add(int64_t i, double v) const {
    if (!(fabs(v) < kFixedLimit)) {
#if defined(__CUDA_ARCH__)
      if (ovf) atomicOr(ovf, 1u);
#else
      if (ovf) *ovf |= 1u;
#endif
      v = 0.0;  // llrint of it would be undefined
    }
    const long long q = llrint(v * kFixedScale);
#if defined(__CUDA_ARCH__)
    atomicAdd(g + i, (unsigned long long)q);
#else
    g[i] += (unsigned long long)q;
#endif
  }
  SRT_HD void add_row(int64_t row, double c0, double c1, double c2, double c3) const {
    if (!g) return;
    add(row, c0);
    add(row + 1, c1);
    add(row + 2, c2);
    add(row + 3, c3);
  }
};

// No accumulation: the B components' passes when only the phi gradient is
// wanted. active() is false at compile time, so those passes are compiled
// without their scatter (less code, fewer registers).
struct AccNone {
  SRT_HD constexpr bool active() const { return false; }
  template <typename V>
  SRT_HD void add_row(int64_t, V, V, V, V) const {}
};

// ------------------------------------------------- fused field pass (vjp)

// Interpolates one field (value, gradient, Hessian into Q; third derivatives
// used internally), adds qb . dQ/dposition to xb and scatters the cotangent of
// every tap, sum_q qb_q W_q(tap), through `acc`.
// qb: cotangents of (v, gx, gy, gz, hxx, hxy, hxz, hyy, hyz, hzz); the
// Hessian entries are the unique components (off-diagonal cotangents already
// hold both symmetric halves).
template <typename T, typename Acc>
SRT_HD void tricubic_vjp(const float* __restrict__ f, int64_t base, int64_t px, int64_t pxy, T tx, T ty, T tz,
                         const T* qb, Tri<T>& Q, T* xb, const Acc& acc) {
  CRW4<T> X, Y, Z;
  cr_weights4(tx, X);
  cr_weights4(ty, Y);
  cr_weights4(tz, Z);
  const bool scatter = acc.active();  // this field's gradient was requested
  // per-row scatter factors: the tap cotangent of row (b, c) is
  // wx_i Cw + gx_i Cg + hx_i Ch with Cw = wz_c Aw_b + gz_c Bw_b + hz_c Dw_b,
  // Cg = wz_c Ag_b + gz_c Bg_b, Ch = wz_c Ah_b.
  T Aw[4], Bw[4], Dw[4], Ag[4], Bg[4], Ah[4];
  for (int b = 0; b < 4; ++b) {
    Aw[b] = qb[0] * Y.w[b] + qb[2] * Y.g[b] + qb[7] * Y.h[b];
    Bw[b] = qb[3] * Y.w[b] + qb[8] * Y.g[b];
    Dw[b] = qb[9] * Y.w[b];
    Ag[b] = qb[1] * Y.w[b] + qb[5] * Y.g[b];
    Bg[b] = qb[6] * Y.w[b];
    Ah[b] = qb[4] * Y.w[b];
  }
  // 20 accumulators: derivative orders (x, y, z) with x + y + z <= 3
  T o000 = 0, o001 = 0, o002 = 0, o003 = 0, o010 = 0, o011 = 0, o012 = 0, o020 = 0, o021 = 0, o030 = 0;
  T o100 = 0, o101 = 0, o102 = 0, o110 = 0, o111 = 0, o120 = 0, o200 = 0, o201 = 0, o210 = 0, o300 = 0;
#pragma unroll 1
  for (int c = 0; c < 4; ++c) {
    T s00 = 0, s01 = 0, s02 = 0, s03 = 0, s10 = 0, s11 = 0, s12 = 0, s20 = 0, s21 = 0, s30 = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int64_t row = base + c * pxy + b * px;
      const float* rp = f + row;
      const T p0 = (T)ldg(rp), p1 = (T)ldg(rp + 1), p2 = (T)ldg(rp + 2), p3 = (T)ldg(rp + 3);
      const T r0 = X.w[0] * p0 + X.w[1] * p1 + X.w[2] * p2 + X.w[3] * p3;
      const T r1 = X.g[0] * p0 + X.g[1] * p1 + X.g[2] * p2 + X.g[3] * p3;
      const T r2 = X.h[0] * p0 + X.h[1] * p1 + X.h[2] * p2 + X.h[3] * p3;
      const T r3 = X.k[0] * p0 + X.k[1] * p1 + X.k[2] * p2 + X.k[3] * p3;
      s00 += Y.w[b] * r0;
      s01 += Y.g[b] * r0;
      s02 += Y.h[b] * r0;
      s03 += Y.k[b] * r0;
      s10 += Y.w[b] * r1;
      s11 += Y.g[b] * r1;
      s12 += Y.h[b] * r1;
      s20 += Y.w[b] * r2;
      s21 += Y.g[b] * r2;
      s30 += Y.w[b] * r3;
      if (scatter) {
        const T Cw = Z.w[c] * Aw[b] + Z.g[c] * Bw[b] + Z.h[c] * Dw[b];
        const T Cg = Z.w[c] * Ag[b] + Z.g[c] * Bg[b];
        const T Ch = Z.w[c] * Ah[b];
        acc.add_row(row, X.w[0] * Cw + X.g[0] * Cg + X.h[0] * Ch, X.w[1] * Cw + X.g[1] * Cg + X.h[1] * Ch,
                    X.w[2] * Cw + X.g[2] * Cg + X.h[2] * Ch, X.w[3] * Cw + X.g[3] * Cg + X.h[3] * Ch);
      }
    }
    const T zw = Z.w[c], zg = Z.g[c], zh = Z.h[c], zk = Z.k[c];
    o000 += zw * s00; o001 += zg * s00; o002 += zh * s00; o003 += zk * s00;
    o010 += zw * s01; o011 += zg * s01; o012 += zh * s01;
    o020 += zw * s02; o021 += zg * s02;
    o030 += zw * s03;
    o100 += zw * s10; o101 += zg * s10; o102 += zh * s10;
    o110 += zw * s11; o111 += zg * s11;
    o120 += zw * s12;
    o200 += zw * s20; o201 += zg * s20;
    o210 += zw * s21;
    o300 += zw * s30;
  }
  Q.v = o000;
  Q.g[0] = o100;
  Q.g[1] = o010;
  Q.g[2] = o001;
  Q.h[0] = o200;
  Q.h[1] = o110;
  Q.h[2] = o101;
  Q.h[3] = o020;
  Q.h[4] = o011;
  Q.h[5] = o002;
  // xb_j += qb . dQ/dx_j
  xb[0] += qb[0] * o100 + qb[1] * o200 + qb[2] * o110 + qb[3] * o101 + qb[4] * o300 + qb[5] * o210 +
           qb[6] * o201 + qb[7] * o120 + qb[8] * o111 + qb[9] * o102;
  xb[1] += qb[0] * o010 + qb[1] * o110 + qb[2] * o020 + qb[3] * o011 + qb[4] * o210 + qb[5] * o120 +
           qb[6] * o111 + qb[7] * o030 + qb[8] * o021 + qb[9] * o012;
  xb[2] += qb[0] * o001 + qb[1] * o101 + qb[2] * o011 + qb[3] * o002 + qb[4] * o201 + qb[5] * o111 +
           qb[6] * o102 + qb[7] * o021 + qb[8] * o012 + qb[9] * o003;
}

// The same pass in FP32 with every product on packed pairs (two FP32 FMAs
// per instruction), as in tricubic_pair: rows y and y+1 of a slice come as one
// float2 per x tap from `rows` (PairRows: the row-pair array; SingleRows: the
// single layout, two loads per tap pair). base: the single-layout index of
// voxel (cx-1, cy-1, cz-1), where the tap cotangents go.
template <typename Acc, typename Rows>
SRT_HD void tricubic_vjp_pair(const Rows& rows, int64_t base, int64_t px, int64_t pxy, float tx, float ty, float tz,
                              const float* qb, Tri<float>& Q, float* xb, const Acc& acc) {
  CRW4<float> X, Y, Z;
  cr_weights4(tx, X);
  cr_weights4(ty, Y);
  cr_weights4(tz, Z);
  float2 xw[4], xg[4], xh[4];
  for (int i = 0; i < 4; ++i) {
    xw[i] = dup2(X.w[i]);
    xg[i] = dup2(X.g[i]);
    xh[i] = dup2(X.h[i]);
  }
  const bool scatter = acc.active();  // this field's gradient was requested
  // y weights and per-row scatter factors of rows (0, 1) and (2, 3)
  float2 yw[2], yg[2], yh[2], yk[2], Aw[2], Bw[2], Dw[2], Ag[2], Bg[2], Ah[2];
  for (int pr = 0; pr < 2; ++pr) {
    const int b0 = 2 * pr, b1 = 2 * pr + 1;
    yw[pr] = make_float2(Y.w[b0], Y.w[b1]);
    yg[pr] = make_float2(Y.g[b0], Y.g[b1]);
    yh[pr] = make_float2(Y.h[b0], Y.h[b1]);
    yk[pr] = make_float2(Y.k[b0], Y.k[b1]);
    Aw[pr] = ffma2(dup2(qb[0]), yw[pr], ffma2(dup2(qb[2]), yg[pr], fmul2(dup2(qb[7]), yh[pr])));
    Bw[pr] = ffma2(dup2(qb[3]), yw[pr], fmul2(dup2(qb[8]), yg[pr]));
    Dw[pr] = fmul2(dup2(qb[9]), yw[pr]);
    Ag[pr] = ffma2(dup2(qb[1]), yw[pr], fmul2(dup2(qb[5]), yg[pr]));
    Bg[pr] = fmul2(dup2(qb[6]), yw[pr]);
    Ah[pr] = fmul2(dup2(qb[4]), yw[pr]);
  }
  // z pass (and an unconditional prefetch): packed for the passes without a
  // scatter (they have the registers to spare), on the operand pairs the y
  // sums form: value weight (o000, o100)
  // (o010, o110) (o020, o120) (o200, o210) (o030, o300), derivative weight
  // (o001, o101) (o011, o111) (o021, -) (o201, -), second derivative
  // (o002, o102) (o012, -), third (o003, -); scalar where the scatter's
  // working set is live. Every output is the same FMA chain over the slices.
  constexpr bool kPackedZ = std::is_same<Acc, AccNone>::value;
  float o000 = 0, o001 = 0, o002 = 0, o003 = 0, o010 = 0, o011 = 0, o012 = 0, o020 = 0, o021 = 0, o030 = 0;
  float o100 = 0, o101 = 0, o102 = 0, o110 = 0, o111 = 0, o120 = 0, o200 = 0, o201 = 0, o210 = 0, o300 = 0;
  const float2 z0 = make_float2(0.f, 0.f);
  float2 W0 = z0, W1 = z0, W2 = z0, W3 = z0, W4 = z0, G0 = z0, G1 = z0, G2 = z0, G3 = z0, H0 = z0, H1 = z0, K0 = z0;
  // taps of the next slice, loaded while the current one is processed
  float2 nt[8];
  for (int pr = 0; pr < 2; ++pr)
    for (int i = 0; i < 4; ++i) nt[4 * pr + i] = rows(0, pr, i);
#pragma unroll 1
  for (int c = 0; c < 4; ++c) {
    float2 s00 = z0, s01 = z0, s02 = z0, s03 = z0, s10 = z0, s11 = z0, s12 = z0, s20 = z0, s21 = z0, s30 = z0;
    // this slice's z weights by selection (an indexed read of Z would put
    // it in local memory)
    const float zwc = c == 0 ? Z.w[0] : (c == 1 ? Z.w[1] : (c == 2 ? Z.w[2] : Z.w[3]));
    const float zgc = c == 0 ? Z.g[0] : (c == 1 ? Z.g[1] : (c == 2 ? Z.g[2] : Z.g[3]));
    const float zhc = c == 0 ? Z.h[0] : (c == 1 ? Z.h[1] : (c == 2 ? Z.h[2] : Z.h[3]));
    const float zkc = c == 0 ? Z.k[0] : (c == 1 ? Z.k[1] : (c == 2 ? Z.k[2] : Z.k[3]));
    const float2 zw = dup2(zwc), zg = dup2(zgc), zh = dup2(zhc);
    float2 ct[8];
    for (int i = 0; i < 8; ++i) ct[i] = nt[i];
    if constexpr (kPackedZ) {  // the last slice reloads itself: no branch in the loop
      const int cn = c < 3 ? c + 1 : 3;
      for (int pr = 0; pr < 2; ++pr)
        for (int i = 0; i < 4; ++i) nt[4 * pr + i] = rows(cn, pr, i);
    } else if (c < 3) {  // (fewer registers where the scatter's working set is live)
      for (int pr = 0; pr < 2; ++pr)
        for (int i = 0; i < 4; ++i) nt[4 * pr + i] = rows(c + 1, pr, i);
    }
#pragma unroll
    for (int pr = 0; pr < 2; ++pr) {
      const float2 t0 = ct[4 * pr], t1 = ct[4 * pr + 1], t2 = ct[4 * pr + 2], t3 = ct[4 * pr + 3];
      float2 r0 = fmul2(xw[0], t0), r1 = fmul2(xg[0], t0), r2 = fmul2(xh[0], t0), r3 = fmul2(dup2(X.k[0]), t0);
      r0 = ffma2(xw[1], t1, r0);
      r1 = ffma2(xg[1], t1, r1);
      r2 = ffma2(xh[1], t1, r2);
      r3 = ffma2(dup2(X.k[1]), t1, r3);
      r0 = ffma2(xw[2], t2, r0);
      r1 = ffma2(xg[2], t2, r1);
      r2 = ffma2(xh[2], t2, r2);
      r3 = ffma2(dup2(X.k[2]), t2, r3);
      r0 = ffma2(xw[3], t3, r0);
      r1 = ffma2(xg[3], t3, r1);
      r2 = ffma2(xh[3], t3, r2);
      r3 = ffma2(dup2(X.k[3]), t3, r3);
      s00 = ffma2(yw[pr], r0, s00);
      s01 = ffma2(yg[pr], r0, s01);
      s02 = ffma2(yh[pr], r0, s02);
      s03 = ffma2(yk[pr], r0, s03);
      s10 = ffma2(yw[pr], r1, s10);
      s11 = ffma2(yg[pr], r1, s11);
      s12 = ffma2(yh[pr], r1, s12);
      s20 = ffma2(yw[pr], r2, s20);
      s21 = ffma2(yg[pr], r2, s21);
      s30 = ffma2(yw[pr], r3, s30);
      if (scatter) {  // tap cotangents of the two rows
        const float2 Cw = ffma2(zw, Aw[pr], ffma2(zg, Bw[pr], fmul2(zh, Dw[pr])));
        const float2 Cg = ffma2(zw, Ag[pr], fmul2(zg, Bg[pr]));
        const float2 Ch = fmul2(zw, Ah[pr]);
        float2 v[4];
        for (int i = 0; i < 4; ++i) v[i] = ffma2(xw[i], Cw, ffma2(xg[i], Cg, fmul2(xh[i], Ch)));
        const int64_t row = base + c * pxy + 2 * pr * px;
        acc.add_row(row, v[0].x, v[1].x, v[2].x, v[3].x);
        acc.add_row(row + px, v[0].y, v[1].y, v[2].y, v[3].y);
      }
    }
    if constexpr (kPackedZ) {
      const float2 P0 = make_float2(s00.x + s00.y, s10.x + s10.y), P1 = make_float2(s01.x + s01.y, s11.x + s11.y);
      const float2 P2 = make_float2(s02.x + s02.y, s12.x + s12.y), P3 = make_float2(s20.x + s20.y, s21.x + s21.y);
      const float2 P4 = make_float2(s03.x + s03.y, s30.x + s30.y);
      W0 = ffma2(zw, P0, W0);
      W1 = ffma2(zw, P1, W1);
      W2 = ffma2(zw, P2, W2);
      W3 = ffma2(zw, P3, W3);
      W4 = ffma2(zw, P4, W4);
      G0 = ffma2(zg, P0, G0);
      G1 = ffma2(zg, P1, G1);
      G2 = ffma2(zg, P2, G2);
      G3 = ffma2(zg, P3, G3);
      H0 = ffma2(zh, P0, H0);
      H1 = ffma2(zh, P1, H1);
      K0 = ffma2(dup2(zkc), P0, K0);
    } else {
      const float S00 = s00.x + s00.y, S01 = s01.x + s01.y, S02 = s02.x + s02.y, S03 = s03.x + s03.y;
      const float S10 = s10.x + s10.y, S11 = s11.x + s11.y, S12 = s12.x + s12.y;
      const float S20 = s20.x + s20.y, S21 = s21.x + s21.y, S30 = s30.x + s30.y;
      o000 += zwc * S00; o001 += zgc * S00; o002 += zhc * S00; o003 += zkc * S00;
      o010 += zwc * S01; o011 += zgc * S01; o012 += zhc * S01;
      o020 += zwc * S02; o021 += zgc * S02;
      o030 += zwc * S03;
      o100 += zwc * S10; o101 += zgc * S10; o102 += zhc * S10;
      o110 += zwc * S11; o111 += zgc * S11;
      o120 += zwc * S12;
      o200 += zwc * S20; o201 += zgc * S20;
      o210 += zwc * S21;
      o300 += zwc * S30;
    }
  }
  if constexpr (kPackedZ) {
    o000 = W0.x, o100 = W0.y, o010 = W1.x, o110 = W1.y, o020 = W2.x, o120 = W2.y;
    o200 = W3.x, o210 = W3.y, o030 = W4.x, o300 = W4.y;
    o001 = G0.x, o101 = G0.y, o011 = G1.x, o111 = G1.y, o021 = G2.x, o201 = G3.x;
    o002 = H0.x, o102 = H0.y, o012 = H1.x, o003 = K0.x;
  }
  Q.v = o000;
  Q.g[0] = o100;
  Q.g[1] = o010;
  Q.g[2] = o001;
  Q.h[0] = o200;
  Q.h[1] = o110;
  Q.h[2] = o101;
  Q.h[3] = o020;
  Q.h[4] = o011;
  Q.h[5] = o002;
  xb[0] += qb[0] * o100 + qb[1] * o200 + qb[2] * o110 + qb[3] * o101 + qb[4] * o300 + qb[5] * o210 +
           qb[6] * o201 + qb[7] * o120 + qb[8] * o111 + qb[9] * o102;
  xb[1] += qb[0] * o010 + qb[1] * o110 + qb[2] * o020 + qb[3] * o011 + qb[4] * o210 + qb[5] * o120 +
           qb[6] * o111 + qb[7] * o030 + qb[8] * o021 + qb[9] * o012;
  xb[2] += qb[0] * o001 + qb[1] * o101 + qb[2] * o011 + qb[3] * o002 + qb[4] * o201 + qb[5] * o111 +
           qb[6] * o102 + qb[7] * o021 + qb[8] * o012 + qb[9] * o003;
}

// One field's pass: FP32 (MIXED) in the packed form, reading the row-pair
// array (PAIR) or the single layout; FP64 in the plain form.
template <bool PAIR, typename T, typename Acc>
SRT_HD void field_pass(const float* f, const float2* fp, int64_t base, int64_t basep, const Geom& G, const T* t,
                       const T* qb, Tri<T>& Q, T* xb, const Acc& acc) {
  if constexpr (sizeof(T) == sizeof(float)) {
    if constexpr (PAIR)
      tricubic_vjp_pair<Acc>(PairRows{fp, basep, G.px, G.pxy2}, base, G.px, G.pxy, t[0], t[1], t[2], qb, Q, xb, acc);
    else
      tricubic_vjp_pair<Acc>(SingleRows{f, base, G.px, G.pxy}, base, G.px, G.pxy, t[0], t[1], t[2], qb, Q, xb, acc);
  } else {
    tricubic_vjp<T, Acc>(f, base, G.px, G.pxy, t[0], t[1], t[2], qb, Q, xb, acc);
  }
}

// -------------------------------------------------------- stage and core

// What the right-hand-side vjp needs about one stage input, independent of
// the state representation (FP64 full state or MIXED perturbation state).
template <typename T>
struct StageView {
  T n[3], a[3], b[3];  // unit vectors n, e1, e2
  T rn, ra, rb;        // 1 / |raw vector| (normalisation Jacobians)
  T A, Ap, s1, s2, e1, e2;
  bool branch;         // dA > 1/2
  int64_t base[4];     // padded base index per field: B_x, B_y, B_z, phi
  int64_t basep[4];    // the same cells in the row-pair layout
  T t[4][3];           // cell offsets per field and axis
};

// symmetric 3x3 as unique components xx xy xz yy yz zz
SRT_HD int sym_idx(int i, int j) {
  return (i == j) ? (i == 0 ? 0 : (i == 1 ? 3 : 5)) : ((i + j == 1) ? 1 : ((i + j == 2) ? 2 : 4));
}

template <typename T>
SRT_HD T symv(const T* h, int i, int j) { return h[sym_idx(i, j)]; }

// One B component's share of rhs_vjp: its cotangents (value, gradient,
// Hessian) from the state-only intermediate cotangents, the fused pass, the
// forward aggregates and its terms of the state cotangents.
template <int C, bool PAIR, typename T, typename Acc>
SRT_HD void vjp_b_component(const StageView<T>& V, const FieldPtrs& F, const Geom& G, const T* fb, const T* ngBb, T e1b,
                            T e2b, T nlapb, const T* Tb, const Acc& acc, T* xb, T* nb, T* ab, T* bb, T* ngB, T& e1ngB,
                            T& e2ngB, T& nlap, T* Tm) {
  const T* n = V.n;
  const T* a = V.a;
  const T* b = V.b;
  const T nc = n[C], ac = a[C], bc = b[C];
  T qb[10];
  qb[0] = -fb[C];
  for (int i = 0; i < 3; ++i)
    qb[1 + i] = nc * ngBb[i] + T(0.5) * e1b * (ac * n[i] + nc * a[i]) + T(0.5) * e2b * (bc * n[i] + nc * b[i]);
  // Hessian cotangent: n_c Tb + n_c nlapb I - sym(e_c Tb_c. (x) n)
  for (int i = 0; i < 3; ++i)
    for (int j = i; j < 3; ++j) {
      T m = nc * symv(Tb, i, j) + ((i == j) ? nc * nlapb : T(0));
      m -= T(0.5) * (symv(Tb, C, i) * n[j] + symv(Tb, C, j) * n[i]);
      // unique components: off-diagonals hold both halves
      qb[4 + sym_idx(i, j)] = (i == j) ? m : T(2) * m;
    }
  Tri<T> Q;
  field_pass<PAIR, T, Acc>(F.b[C], F.pr[C], V.base[C], V.basep[C], G, V.t[C], qb, Q, xb, acc);
  // forward aggregates
  for (int i = 0; i < 3; ++i) ngB[i] += Q.g[i] * nc;
  const T gn = Q.g[0] * n[0] + Q.g[1] * n[1] + Q.g[2] * n[2];
  const T ga = Q.g[0] * a[0] + Q.g[1] * a[1] + Q.g[2] * a[2];
  const T gbb = Q.g[0] * b[0] + Q.g[1] * b[1] + Q.g[2] * b[2];
  e1ngB += T(0.5) * (ac * gn + nc * ga);
  e2ngB += T(0.5) * (bc * gn + nc * gbb);
  T Hn[3];
  for (int i = 0; i < 3; ++i) Hn[i] = symv(Q.h, i, 0) * n[0] + symv(Q.h, i, 1) * n[1] + symv(Q.h, i, 2) * n[2];
  for (int i = 0; i < 3; ++i)
    for (int j = i; j < 3; ++j) {
      T d = Q.h[sym_idx(i, j)] * nc;
      if (i == C) d -= T(0.5) * Hn[j];
      if (j == C) d -= T(0.5) * Hn[i];
      Tm[sym_idx(i, j)] += d;
    }
  const T trH = Q.h[0] + Q.h[3] + Q.h[5];
  nlap += trH * nc;
  // this component's share of the state cotangents
  T HT = 0;  // H_c : Tb (full contraction)
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) HT += symv(Q.h, i, j) * symv(Tb, i, j);
  nb[C] += Q.g[0] * ngBb[0] + Q.g[1] * ngBb[1] + Q.g[2] * ngBb[2] + trH * nlapb + HT + T(0.5) * e1b * ga +
           T(0.5) * e2b * gbb;
  for (int k = 0; k < 3; ++k) {
    T tk = 0;
    for (int j = 0; j < 3; ++j) tk += symv(Tb, C, j) * symv(Q.h, j, k);
    nb[k] += T(0.5) * e1b * ac * Q.g[k] + T(0.5) * e2b * bc * Q.g[k] - tk;
    ab[k] += T(0.5) * e1b * nc * Q.g[k];
    bb[k] += T(0.5) * e2b * nc * Q.g[k];
  }
  ab[C] += T(0.5) * e1b * gn;
  bb[C] += T(0.5) * e2b * gn;
}

// yb += J(u)^T fb for the stage described by V; tap cotangents go to accb[0..2]
// (B_x, B_y, B_z) and accp (phi).
template <typename T, typename AccB, typename AccP, bool PAIR = false>
SRT_HD void rhs_vjp(const StageView<T>& V, const FieldPtrs& F, const Geom& G, const T* fb, T* yb, const AccB* accb,
                    const AccP& accp) {
  const T* n = V.n;
  const T* a = V.a;
  const T* b = V.b;
  // ---- intermediate cotangents (state only)
  const T nfx = n[0] * fb[0] + n[1] * fb[1] + n[2] * fb[2];
  const T nfn = n[0] * fb[3] + n[1] * fb[4] + n[2] * fb[5];
  const T sab = -(n[0] * fb[6] + n[1] * fb[7] + n[2] * fb[8]);
  const T sbb = -(n[0] * fb[9] + n[1] * fb[10] + n[2] * fb[11]);
  const T phib = T(-2) * nfx;
  T vb[3];
  for (int i = 0; i < 3; ++i) vb[i] = fb[3 + i] - n[i] * nfn;
  const T agb = T(2) * sab, bgb = T(2) * sbb, e1b = sab, e2b = sbb;
  T Apb = -fb[12];
  const T Lb = T(-4) * V.Ap * fb[13] + T(4) * V.s1 * fb[14] + T(4) * V.s2 * fb[15];
  const T PHb = -V.A * fb[13];
  const T nlapb = T(0.5) * V.A * fb[13];
  const T S1b = V.A * V.A * fb[14], S2b = V.A * V.A * fb[15];
  // the dA > 1/2 branch's terms, formed either way and selected (no branch;
  // where dA = 0 they are not finite and not selected)
  T Ab = 0, s1b = 0, s2b = 0, el1b = 0, el2b = 0;
  {
    const T A2 = V.A * V.A, A3 = A2 * V.A;
    const T q = sqrt(T(4) + V.e1 * V.e1 + V.e2 * V.e2);
    T bs1 = T(2) * V.s1 / A3 * fb[13];
    T bs2 = T(2) * V.s2 / A3 * fb[13];
    T bA = T(-3) * (V.s1 * V.s1 + V.s2 * V.s2) / (A3 * V.A) * fb[13];
    bs1 += T(-2) * q / A2 * fb[16];
    T qb = T(-2) * V.s1 / A2 * fb[16];
    bA += T(4) * V.s1 * q / A3 * fb[16];
    bs2 += T(-2) * q / A2 * fb[17];
    qb += T(-2) * V.s2 / A2 * fb[17];
    bA += T(4) * V.s2 * q / A3 * fb[17];
    const T D = A2 * (T(2) + q), N = V.s1 * V.e2 - V.s2 * V.e1;
    const T Nb = -fb[18] / D, Db = N * fb[18] / (D * D);
    bs1 += V.e2 * Nb;
    T be2 = V.s1 * Nb;
    bs2 += -V.e1 * Nb;
    T be1 = -V.s2 * Nb;
    bA += T(2) * V.A * (T(2) + q) * Db;
    qb += A2 * Db;
    be1 += V.e1 / q * qb;
    be2 += V.e2 / q * qb;
    s1b = V.branch ? bs1 : T(0);
    s2b = V.branch ? bs2 : T(0);
    Ab = V.branch ? bA : T(0);
    el1b = V.branch ? be1 : T(0);
    el2b = V.branch ? be2 : T(0);
  }
  // cotangent of the effective tidal matrix He = H + T/2 (full symmetric)
  T Heb[6];
  for (int i = 0; i < 3; ++i)
    for (int j = i; j < 3; ++j)
      Heb[sym_idx(i, j)] = (a[i] * a[j] - b[i] * b[j]) * S1b + (a[i] * b[j] + b[i] * a[j]) * S2b;
  T Tb[6];
  for (int u = 0; u < 6; ++u) Tb[u] = T(0.5) * Heb[u];
  T gb[3], ngBb[3];
  for (int i = 0; i < 3; ++i) {
    gb[i] = T(2) * vb[i] + agb * a[i] + bgb * b[i] + n[i] * Lb;
    ngBb[i] = vb[i] + T(0.25) * n[i] * Lb;
  }
  T nb[3] = {0, 0, 0}, ab[3] = {0, 0, 0}, bb[3] = {0, 0, 0}, xb[3] = {0, 0, 0};
  // aggregates of the forward
  T ngB[3] = {0, 0, 0}, e1ngB = 0, e2ngB = 0, nlap = 0, Tm[6] = {0, 0, 0, 0, 0, 0};

  // ---- B components (compile-time component index: no local-memory arrays)
  vjp_b_component<0, PAIR, T, AccB>(V, F, G, fb, ngBb, e1b, e2b, nlapb, Tb, accb[0], xb, nb, ab, bb, ngB, e1ngB, e2ngB,
                                    nlap, Tm);
  vjp_b_component<1, PAIR, T, AccB>(V, F, G, fb, ngBb, e1b, e2b, nlapb, Tb, accb[1], xb, nb, ab, bb, ngB, e1ngB, e2ngB,
                                    nlap, Tm);
  vjp_b_component<2, PAIR, T, AccB>(V, F, G, fb, ngBb, e1b, e2b, nlapb, Tb, accb[2], xb, nb, ab, bb, ngB, e1ngB, e2ngB,
                                    nlap, Tm);

  // ---- phi
  Tri<T> P;
  {
    T qb[10];
    qb[0] = phib;
    for (int i = 0; i < 3; ++i) qb[1 + i] = gb[i];
    for (int i = 0; i < 3; ++i)
      for (int j = i; j < 3; ++j) {
        const T m = Heb[sym_idx(i, j)] + (n[i] * n[j] - ((i == j) ? T(1) : T(0))) * PHb;
        qb[4 + sym_idx(i, j)] = (i == j) ? m : T(2) * m;
      }
    field_pass<PAIR, T, AccP>(F.phi, F.pr[3], V.base[3], V.basep[3], G, V.t[3], qb, P, xb, accp);
  }
  const T* g = P.g;
  for (int i = 0; i < 3; ++i) {
    nb[i] += -(T(1) + T(2) * P.v) * fb[i];
    ab[i] += agb * g[i];
    bb[i] += bgb * g[i];
    nb[i] += T(2) * PHb * (symv(P.h, i, 0) * n[0] + symv(P.h, i, 1) * n[1] + symv(P.h, i, 2) * n[2]);
  }

  // ---- terms of the field aggregates
  T v[3];
  for (int i = 0; i < 3; ++i) v[i] = T(2) * g[i] + ngB[i];
  const T nv = n[0] * v[0] + n[1] * v[1] + n[2] * v[2];
  const T sa = T(2) * (a[0] * g[0] + a[1] * g[1] + a[2] * g[2]) + e1ngB;
  const T sb = T(2) * (b[0] * g[0] + b[1] * g[1] + b[2] * g[2]) + e2ngB;
  const T L = n[0] * g[0] + n[1] * g[1] + n[2] * g[2] + T(0.25) * (n[0] * ngB[0] + n[1] * ngB[1] + n[2] * ngB[2]);
  for (int i = 0; i < 3; ++i) {
    nb[i] += -nv * fb[3 + i] - v[i] * nfn;
    nb[i] += -sa * fb[6 + i] - sb * fb[9 + i];
    nb[i] += (g[i] + T(0.25) * ngB[i]) * Lb;
  }
  Apb += T(-4) * L * fb[13];
  s1b += T(4) * L * fb[14];
  s2b += T(4) * L * fb[15];
  const T nHn = n[0] * n[0] * P.h[0] + n[1] * n[1] * P.h[3] + n[2] * n[2] * P.h[5] +
                T(2) * (n[0] * n[1] * P.h[1] + n[0] * n[2] * P.h[2] + n[1] * n[2] * P.h[4]);
  const T PH = nHn - (P.h[0] + P.h[3] + P.h[5]);
  Ab += (-PH + T(0.5) * nlap) * fb[13];
  T He[6];
  for (int u = 0; u < 6; ++u) He[u] = P.h[u] + T(0.5) * Tm[u];
  T Hea[3], Heb3[3];
  for (int i = 0; i < 3; ++i) {
    Hea[i] = symv(He, i, 0) * a[0] + symv(He, i, 1) * a[1] + symv(He, i, 2) * a[2];
    Heb3[i] = symv(He, i, 0) * b[0] + symv(He, i, 1) * b[1] + symv(He, i, 2) * b[2];
  }
  const T S1 = (a[0] * Hea[0] + a[1] * Hea[1] + a[2] * Hea[2]) - (b[0] * Heb3[0] + b[1] * Heb3[1] + b[2] * Heb3[2]);
  const T S2 = T(2) * (a[0] * Heb3[0] + a[1] * Heb3[1] + a[2] * Heb3[2]);
  Ab += T(2) * V.A * (S1 * fb[14] + S2 * fb[15]);
  for (int i = 0; i < 3; ++i) {
    ab[i] += T(2) * Hea[i] * S1b + T(2) * Heb3[i] * S2b;
    bb[i] += T(-2) * Heb3[i] * S1b + T(2) * Hea[i] * S2b;
  }

  // ---- through the normalisations, into the state cotangent
  const T nnb = n[0] * nb[0] + n[1] * nb[1] + n[2] * nb[2];
  const T aab = a[0] * ab[0] + a[1] * ab[1] + a[2] * ab[2];
  const T bbb = b[0] * bb[0] + b[1] * bb[1] + b[2] * bb[2];
  for (int i = 0; i < 3; ++i) {
    yb[i] += xb[i];
    yb[3 + i] += V.rn * (nb[i] - n[i] * nnb);
    yb[6 + i] += V.ra * (ab[i] - a[i] * aab);
    yb[9 + i] += V.rb * (bb[i] - b[i] * bbb);
  }
  yb[12] += Ab;
  yb[13] += Apb;
  yb[14] += s1b;
  yb[15] += s2b;
  yb[16] += el1b;
  yb[17] += el2b;
}

// ------------------------------------------------------- stage views

// FP64 full state y (layout of rhs_std).
SRT_HD void stage_view_fp64(const double* y, const Geom& G, StageView<double>& V) {
  const double nr = sqrt(y[3] * y[3] + y[4] * y[4] + y[5] * y[5]);
  const double ar = sqrt(y[6] * y[6] + y[7] * y[7] + y[8] * y[8]);
  const double br = sqrt(y[9] * y[9] + y[10] * y[10] + y[11] * y[11]);
  V.rn = 1.0 / nr;
  V.ra = 1.0 / ar;
  V.rb = 1.0 / br;
  for (int i = 0; i < 3; ++i) {
    V.n[i] = y[3 + i] / nr;
    V.a[i] = y[6 + i] / ar;
    V.b[i] = y[9 + i] / br;
  }
  V.A = y[12];
  V.Ap = y[13];
  V.s1 = y[14];
  V.s2 = y[15];
  V.e1 = y[16];
  V.e2 = y[17];
  V.branch = y[12] > 0.5;
  for (int f = 0; f < 4; ++f) {
    int cell[3];
    for (int i = 0; i < 3; ++i) {
      const double x = y[i] - ((f == i) ? 0.5 : 0.0);
      const double fl = floor(x);
      V.t[f][i] = x - fl;
      cell[i] = wrap64((int64_t)fl, G.n[i]);
    }
    V.base[f] = cell_base(G, cell[0], cell[1], cell[2]);
    V.basep[f] = cell_base_pair(G, cell[0], cell[1], cell[2]);
  }
}

// MIXED perturbation state d at affine parameter s (layout of rhs_mixed).
SRT_HD void stage_view_mixed(const float* d, float s, const MixedRay& R, const Geom& G, const float* x0,
                             StageView<float>& V) {
  const float* v0s[3] = {R.n0, R.a0, R.b0};
  float* outs[3] = {V.n, V.a, V.b};
  float* rs[3] = {&V.rn, &V.ra, &V.rb};
  for (int k = 0; k < 3; ++k) {
    const float* v0 = v0s[k];
    const float* dv = d + 3 + 3 * k;
    const float q = R.eta[k] + 2.f * (v0[0] * dv[0] + v0[1] * dv[1] + v0[2] * dv[2]) +
                    (dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
    const float rm1 = rsqrt1p_m1(q);
    *rs[k] = 1.f + rm1;
    for (int i = 0; i < 3; ++i) outs[k][i] = v0[i] + (v0[i] * rm1 + dv[i] * (1.f + rm1));
  }
  V.A = s + d[12];
  V.Ap = d[13] - 1.f;
  V.s1 = d[14];
  V.s2 = d[15];
  V.e1 = d[16];
  V.e2 = d[17];
  V.branch = d[12] > 0.5f - s;
  int cc[3], cs[3];
  float tc[3], ts[3];
  for (int i = 0; i < 3; ++i) {
    const float p = s * R.n0[i];
    const float pe = fmaf(s, R.n0[i], -p);
    float th, tl;
    two_sum(x0[i], -p, th, tl);
    const float lo = (tl - pe) + d[i];
    float df;
    locate_mixed(th, lo, G.n[i], G.invn[i], cc[i], tc[i], cs[i], ts[i], df);
  }
  for (int f = 0; f < 4; ++f) {
    int cell[3];
    for (int i = 0; i < 3; ++i) {
      const bool stag = (f == i);
      cell[i] = stag ? cs[i] : cc[i];
      V.t[f][i] = stag ? ts[i] : tc[i];
    }
    V.base[f] = cell_base(G, cell[0], cell[1], cell[2]);
    V.basep[f] = cell_base_pair(G, cell[0], cell[1], cell[2]);
  }
}

}  // namespace srt
