// srt_dd.cuh — double-float ("dd") arithmetic: a value is the unevaluated sum
// hi + lo of two floats, |lo| <= ulp(hi) / 2, about 48 significant bits.
//
// The FP64 re-trace of the MIXED form's flagged rays runs in this arithmetic
// on the FP32 pipes: GB300 issues FP32 at 64x its FP64 rate, and a dd
// operation costs 3-20 FP32 instructions, so a dd trajectory comes out several
// times cheaper than an FP64 one while staying ~1e-14 from it (far inside the
// cell-face margin the guard uses, ~1e-8 grid units).
//
// The operations are the classic error-free transformations: Knuth's two-sum,
// the FMA-based two-product, and Dekker/Bailey's double-word addition,
// multiplication, division and square root built on them (Hida, Li and Bailey,
// "Library for double-double and quad-double arithmetic", 2000; Joldes,
// Muller and Popescu, "Tight and rigorous error bounds for basic building
// blocks of double-word arithmetic", 2017).
#pragma once
#include <math.h>
#include <stdint.h>

#ifndef SRT_HD
#if defined(__CUDACC__)
#define SRT_HD __host__ __device__ __forceinline__
#else
#define SRT_HD inline
#endif
#endif

namespace srt {

struct dd {
  float hi, lo;
  SRT_HD dd() : hi(0.f), lo(0.f) {}
  SRT_HD dd(float h, float l) : hi(h), lo(l) {}
  SRT_HD dd(float f) : hi(f), lo(0.f) {}
  SRT_HD dd(int i) : hi((float)i), lo((float)(i - (int)(float)i)) {}
  SRT_HD dd(double d) {
    hi = (float)d;
    lo = (float)(d - (double)hi);
  }
  SRT_HD explicit operator double() const { return (double)hi + (double)lo; }
  SRT_HD explicit operator float() const { return hi + lo; }
};

// s + e = a + b exactly (Knuth)
SRT_HD void dd_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
// s + e = a + b exactly when |a| >= |b| (Dekker)
SRT_HD void dd_fast_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  e = b - (s - a);
}

SRT_HD dd operator+(const dd& a, const dd& b) {
  float s1, s2, t1, t2;
  dd_two_sum(a.hi, b.hi, s1, s2);
  dd_two_sum(a.lo, b.lo, t1, t2);
  s2 += t1;
  dd_fast_two_sum(s1, s2, s1, s2);
  s2 += t2;
  dd_fast_two_sum(s1, s2, s1, s2);
  return dd(s1, s2);
}
SRT_HD dd operator-(const dd& a) { return dd(-a.hi, -a.lo); }
SRT_HD dd operator-(const dd& a, const dd& b) { return a + (-b); }

SRT_HD dd operator*(const dd& a, const dd& b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  float s, t;
  dd_fast_two_sum(p, e, s, t);
  return dd(s, t);
}
SRT_HD dd operator*(const dd& a, float b) {
  const float p = a.hi * b;
  const float e = fmaf(a.lo, b, fmaf(a.hi, b, -p));
  float s, t;
  dd_fast_two_sum(p, e, s, t);
  return dd(s, t);
}
SRT_HD dd operator*(float b, const dd& a) { return a * b; }

SRT_HD dd operator/(const dd& a, const dd& b) {
  // long division: q1 = a/b in float, remainder in dd, one correction
  const float q1 = a.hi / b.hi;
  const dd r = a - b * q1;
  const float q2 = r.hi / b.hi;
  const dd r2 = r - b * q2;
  const float q3 = r2.hi / b.hi;
  float s, e;
  dd_fast_two_sum(q1, q2, s, e);
  return dd(s, e) + dd(q3);
}

SRT_HD dd dd_sqrt(const dd& a) {
  if (a.hi <= 0.f) return dd(0.f);
  const float x = sqrtf(a.hi);
  // one Newton step from x: x + (a - x^2) / (2x)
  const float p = x * x;
  const float e = fmaf(x, x, -p);
  const dd r = a - dd(p, e);
  const float c = r.hi / (2.f * x);
  float s, t;
  dd_fast_two_sum(x, c, s, t);
  return dd(s, t);
}

SRT_HD dd& operator+=(dd& a, const dd& b) { return a = a + b; }
SRT_HD dd& operator-=(dd& a, const dd& b) { return a = a - b; }
SRT_HD dd& operator*=(dd& a, const dd& b) { return a = a * b; }

SRT_HD bool operator>(const dd& a, const dd& b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }
SRT_HD bool operator<(const dd& a, const dd& b) { return b > a; }

// Largest integer <= a, as a double-word integer.
SRT_HD dd dd_floor(const dd& a) {
  float h = floorf(a.hi), l = 0.f;
  if (h == a.hi) {  // hi is an integer: the fraction is in lo
    l = floorf(a.lo);
    dd_fast_two_sum(h, l, h, l);
  }
  return dd(h, l);
}

}  // namespace srt
