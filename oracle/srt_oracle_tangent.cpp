// srt_oracle_tangent.cpp — TEST INFRASTRUCTURE: forward-mode (tangent)
// derivatives of the FP64 oracle, the independent check of the GPU vjp.
//
// The oracle's FP64 scheme (srt_oracle_scheme.inc, which restates
// snapshot-raytracer.cu:195-550) is compiled here a second time with a dual
// number in place of double: every value carries K directional derivatives
// with respect to the field grids. For a loss L = sum_m sum_p w_m[p] map_m[p]
// and grid directions v_1..v_K this gives L and dL/de_k = <grad L, v_k>
// exactly (to rounding), which must equal <vjp, v_k> — the dot-product test
// of an adjoint, with no finite-difference truncation error. The value parts
// follow the FP64 oracle's operation order, so they equal its maps bit for bit.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int K = 8;  // directions carried per pass

struct Dual {
  double v;
  double d[K];
  Dual() : v(0.0) { std::memset(d, 0, sizeof(d)); }
  Dual(double x) : v(x) { std::memset(d, 0, sizeof(d)); }  // NOLINT (implicit: constants)
};

inline Dual operator+(const Dual& a, const Dual& b) {
  Dual r(a.v + b.v);
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] + b.d[k];
  return r;
}
inline Dual operator-(const Dual& a, const Dual& b) {
  Dual r(a.v - b.v);
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] - b.d[k];
  return r;
}
inline Dual operator*(const Dual& a, const Dual& b) {
  Dual r(a.v * b.v);
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
inline Dual operator/(const Dual& a, const Dual& b) {
  Dual r(a.v / b.v);
  for (int k = 0; k < K; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) / b.v;
  return r;
}
inline Dual operator-(const Dual& a) {
  Dual r(-a.v);
  for (int k = 0; k < K; ++k) r.d[k] = -a.d[k];
  return r;
}
inline Dual operator+(double a, const Dual& b) {
  Dual r(a + b.v);
  for (int k = 0; k < K; ++k) r.d[k] = b.d[k];
  return r;
}
inline Dual operator+(const Dual& a, double b) {
  Dual r(a.v + b);
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k];
  return r;
}
inline Dual operator-(double a, const Dual& b) {
  Dual r(a - b.v);
  for (int k = 0; k < K; ++k) r.d[k] = -b.d[k];
  return r;
}
inline Dual operator-(const Dual& a, double b) {
  Dual r(a.v - b);
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k];
  return r;
}
inline Dual operator*(double a, const Dual& b) {
  Dual r(a * b.v);
  for (int k = 0; k < K; ++k) r.d[k] = a * b.d[k];
  return r;
}
inline Dual operator*(const Dual& a, double b) {
  Dual r(a.v * b);
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b;
  return r;
}
inline Dual operator/(const Dual& a, double b) {
  Dual r(a.v / b);
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] / b;
  return r;
}
inline Dual& operator+=(Dual& a, const Dual& b) { return a = a + b; }
inline Dual& operator/=(Dual& a, const Dual& b) { return a = a / b; }
inline bool operator>(const Dual& a, double b) { return a.v > b; }
inline Dual sqrt(const Dual& a) {
  Dual r(std::sqrt(a.v));
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] / (2.0 * r.v);
  return r;
}
inline double floor(const Dual& a) { return std::floor(a.v); }

struct tan_fields {
  int64_t n[3];
  const float* phi;
  const float* b[3];       // FP32 component planes
  const float* dphi[K];    // directions (may be NULL)
  const float* db[K][3];   // direction component planes (may be NULL)
};

int64_t or_mod(int64_t i, int64_t n) {
  int64_t r = i % n;
  return r < 0 ? r + n : r;
}

#define OR_CUSTOM_TAP
Dual tap_tan(const tan_fields* F, int f, int64_t i) {
  Dual r(f == 3 ? (double)F->phi[i] : (double)F->b[f][i]);
  for (int k = 0; k < K; ++k) {
    const float* d = (f == 3) ? F->dphi[k] : F->db[k][f];
    r.d[k] = d ? (double)d[i] : 0.0;
  }
  return r;
}

#define FN(name) name##_tan
#define IT Dual
#define ST Dual
#define OR_REF16 0
#define OR_FIELDS tan_fields
#include "srt_oracle_scheme.inc"
#undef FN
#undef IT
#undef ST
#undef OR_REF16
#undef OR_FIELDS

}  // namespace

extern "C" void srto_pix2ang_ring(int64_t nside, int64_t pix, double* theta, double* phi);

// L = sum_m sum_i weights[m * count + i] * map_m(pixel pix[i]) and its
// derivatives along up to K grid directions: dir_phi[k] (n0*n1*n2 floats) and
// dir_b[k] (3*n0*n1*n2 floats interleaved like b_xyz), NULL entries meaning
// zero. out: L; dL: ndir derivatives. Maps are the FP64 oracle's, before the
// cast to float.
extern "C" int srto_tangent(const float* phi, const float* b_xyz, int64_t n0, int64_t n1, int64_t n2, int64_t nside,
                            const int64_t* pix, int64_t count, int n_steps, const float* weights,
                            const float* const* dir_phi, const float* const* dir_b, int ndir, double* out, double* dL,
                            int nthreads) {
  if (ndir < 0 || ndir > K || n0 < 1 || n1 < 1 || n2 < 1 || n_steps < 1 || count < 0) return -1;
  const int64_t nv = n0 * n1 * n2;
  std::vector<float> planes((size_t)(3 * nv));
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : omp_get_max_threads())
#endif
  for (int64_t v = 0; v < nv; ++v)
    for (int c = 0; c < 3; ++c) planes[c * nv + v] = b_xyz[3 * v + c];
  bool any_db = false;
  for (int k = 0; k < ndir; ++k) any_db = any_db || (dir_b && dir_b[k]);
  std::vector<float> dplanes(any_db ? (size_t)(3 * nv * ndir) : 0);
  tan_fields F;
  std::memset(&F, 0, sizeof(F));
  F.n[0] = n0;
  F.n[1] = n1;
  F.n[2] = n2;
  F.phi = phi;
  for (int c = 0; c < 3; ++c) F.b[c] = planes.data() + c * nv;
  for (int k = 0; k < ndir; ++k) {
    F.dphi[k] = dir_phi ? dir_phi[k] : nullptr;
    if (dir_b && dir_b[k]) {
      for (int64_t v = 0; v < nv; ++v)
        for (int c = 0; c < 3; ++c) dplanes[(size_t)(k * 3 + c) * nv + v] = dir_b[k][3 * v + c];
      for (int c = 0; c < 3; ++c) F.db[k][c] = dplanes.data() + (size_t)(k * 3 + c) * nv;
    }
  }
  double total = 0.0, dtot[K] = {0};
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
  {
    double lsum = 0.0, dsum[K] = {0};
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
    for (int64_t i = 0; i < count; ++i) {
      double th, ph;
      srto_pix2ang_ring(nside, pix[i], &th, &ph);
      // initial state and extraction as in srt_oracle.c (snapshot-raytracer.cu:560, :566-582)
      Dual y[19] = {(double)n0 * 0.5, (double)n1 * 0.5, (double)n2 * 0.5, -std::sin(th) * std::cos(ph),
                    -std::sin(th) * std::sin(ph), -std::cos(th), std::cos(th) * std::cos(ph),
                    std::cos(th) * std::sin(ph), -std::sin(th), std::sin(ph), -std::cos(ph), 0.0, 0.0, -1.0, 0.0,
                    0.0, 0.0, 0.0, 0.0};
      integrate_tan(y, n_steps, &F);
      y[0] = y[0] - (double)n0 * 0.5;
      y[1] = y[1] - (double)n1 * 0.5;
      y[2] = y[2] - (double)n2 * 0.5;
      const Dual norm = sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
      y[0] = y[0] / norm - std::sin(th) * std::cos(ph);
      y[1] = y[1] / norm - std::sin(th) * std::sin(ph);
      y[2] = y[2] / norm - std::cos(th);
      const Dual maps[6] = {y[12], y[16], y[17], y[18],
                            y[0] * std::cos(th) * std::cos(ph) + y[1] * std::cos(th) * std::sin(ph) - y[2] * std::sin(th),
                            y[0] * std::sin(ph) - y[1] * std::cos(ph)};
      for (int m = 0; m < 6; ++m) {
        const double w = weights[m * count + i];
        lsum += w * maps[m].v;
        for (int k = 0; k < K; ++k) dsum[k] += w * maps[m].d[k];
      }
    }
#ifdef _OPENMP
#pragma omp critical
#endif
    {
      total += lsum;
      for (int k = 0; k < K; ++k) dtot[k] += dsum[k];
    }
  }
  *out = total;
  for (int k = 0; k < ndir; ++k) dL[k] = dtot[k];
  return 0;
}
