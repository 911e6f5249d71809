// Host build of the double-float operations (snapshot-raytracer_gb300/csrc/srt_dd.cuh)
// for tests/test_dd_arith.py: each entry takes and returns (hi, lo) pairs.
#include "srt_dd.cuh"
using srt::dd;
extern "C" {
void dd_add(const float* a, const float* b, float* r) { dd x = dd(a[0], a[1]) + dd(b[0], b[1]); r[0] = x.hi; r[1] = x.lo; }
void dd_mul(const float* a, const float* b, float* r) { dd x = dd(a[0], a[1]) * dd(b[0], b[1]); r[0] = x.hi; r[1] = x.lo; }
void dd_div(const float* a, const float* b, float* r) { dd x = dd(a[0], a[1]) / dd(b[0], b[1]); r[0] = x.hi; r[1] = x.lo; }
void dd_sqrt_(const float* a, float* r) { dd x = srt::dd_sqrt(dd(a[0], a[1])); r[0] = x.hi; r[1] = x.lo; }
void dd_floor_(const float* a, float* r) { dd x = srt::dd_floor(dd(a[0], a[1])); r[0] = x.hi; r[1] = x.lo; }
void dd_from_double(double d, float* r) { dd x(d); r[0] = x.hi; r[1] = x.lo; }
}
