/* srt_oracle.c — CPU oracle of the tracer's hot path. TEST INFRASTRUCTURE:
 * only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg (and
 * its reference arm) may load it, and only as the checker or the timed CPU
 * baseline. It is never part of the product path.
 *
 * It restates, in plain C, the per-ray path of the reference program
 * snapshot-raytracer.cu (JulianAdamek/snapshot-raytracer):
 *   - B de-interleave and FP16 x 2^27 quantisation  .cu:585-597, :774-836
 *   - HEALPix RING pixel centres (chealpix pix2ang_ring64, a third-party
 *     library not vendored with the reference, version unpinned; restated
 *     from Gorski et al. 2005)                      .cu:857-866
 *   - Catmull-Rom / tricubic / right-hand side / RK4 .cu:195-550
 *     (srt_oracle_scheme.inc)
 *   - ray initial state and map extraction          .cu:552-583
 *   - pixel range of a batch                        .cu:708-717
 * in two modes: OR_MODE_REF16, the reference's own arithmetic, and
 * OR_MODE_FP64, the same scheme entirely in double. The REF16 mode is pinned
 * bit for bit against the reference's own host-compiled code (oracle/_ref,
 * built from the reference sources by oracle/build_ref.sh) through the golden
 * fixtures in tests/golden/.
 *
 * Build: gcc -O2 -std=c11 -fopenmp -ffp-contract=off -fPIC -shared
 * (no FMA contraction, so results are the same on x86-64 and aarch64 apart
 * from libm's sin/cos/atan2).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_MODE_FP64 0
#define OR_MODE_REF16 2

typedef struct {
  int64_t n[3];
  const float* phi;   /* n0*n1*n2, x fastest */
  const float* b[3];  /* FP32 B component planes (FP64 mode) */
  uint16_t* bh[3];    /* binary16 planes of B * 2^27 (REF16 mode) */
} or_fields;

static int64_t or_mod(int64_t i, int64_t n) {
  int64_t r = i % n;
  return r < 0 ? r + n : r;
}

/* ---------------------------------------------------------- binary16 */

/* float -> binary16, IEEE 754 round to nearest even (the conversion of
 * __float2half used by vector3_to_half, snapshot-raytracer.cu:589-595). */
static uint16_t or_float_to_half(float f) {
  uint32_t x;
  memcpy(&x, &f, 4);
  const uint32_t sign = (x >> 16) & 0x8000u;
  const uint32_t ax = x & 0x7fffffffu;
  if (ax >= 0x7f800000u) return (uint16_t)(sign | 0x7c00u | (ax > 0x7f800000u ? 0x200u : 0u));
  if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u); /* rounds to infinity */
  if (ax < 0x38800000u) {                                   /* half subnormal or zero */
    const uint32_t e = ax >> 23;
    const uint32_t shift = 126u - e;
    if (shift > 24u) return (uint16_t)sign;
    const uint32_t m = (ax & 0x7fffffu) | 0x800000u;
    uint32_t q = m >> shift;
    const uint32_t rem = m & ((1u << shift) - 1u), half = 1u << (shift - 1u);
    if (rem > half || (rem == half && (q & 1u))) ++q;
    return (uint16_t)(sign | q);
  }
  uint32_t q = ((((ax >> 23) - 112u)) << 10) | ((ax & 0x7fffffu) >> 13);
  const uint32_t rem = ax & 0x1fffu;
  if (rem > 0x1000u || (rem == 0x1000u && (q & 1u))) ++q;
  return (uint16_t)(sign | q);
}

static float or_half_to_float(uint16_t h) {
  const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
  const uint32_t e = (h >> 10) & 0x1fu, m = h & 0x3ffu;
  uint32_t x;
  if (e == 0) {
    if (m == 0) {
      x = sign;
    } else { /* subnormal: m * 2^-24 */
      float f = (float)m * 5.9604644775390625e-8f;
      memcpy(&x, &f, 4);
      x |= sign;
    }
  } else if (e == 31) {
    x = sign | 0x7f800000u | (m << 13);
  } else {
    x = sign | ((e + 112u) << 23) | (m << 13);
  }
  float f;
  memcpy(&f, &x, 4);
  return f;
}

uint16_t srto_float_to_half(float f) { return or_float_to_half(f); }
float srto_half_to_float(uint16_t h) { return or_half_to_float(h); }

/* ------------------------------------------------------------ scheme */

#define FN(name) name##_ref16
#define IT float
#define OR_REF16 1
#include "srt_oracle_scheme.inc"
#undef FN
#undef IT
#undef OR_REF16

#define FN(name) name##_fp64
#define IT double
#define OR_REF16 0
#include "srt_oracle_scheme.inc"
#undef FN
#undef IT
#undef OR_REF16

/* ----------------------------------------------------------- HEALPix */

/* Centre (theta, phi) of RING pixel `pix` (Gorski et al. 2005, eqs. 4-9):
 * rings i = 1 .. 4 nside - 1 from the north pole; ring i holds
 * min(4 i, 4 nside, 4 (4 nside - i)) pixels; cos(theta) = 1 - i^2/(3 nside^2)
 * on the north cap, 4/3 - 2 i/(3 nside) on the belt, mirrored on the south
 * cap. Written independently of the product's device implementation so the
 * two check each other. */
void srto_pix2ang_ring(int64_t nside, int64_t pix, double* theta, double* phi) {
  const double pi = 3.14159265358979323846;
  const int64_t ncap = 2 * nside * (nside - 1), npix = 12 * nside * nside;
  int64_t ring, j, nring;
  double z, s;
  if (pix < ncap) {
    ring = (int64_t)floor(0.5 * (1.0 + sqrt(1.0 + 2.0 * (double)pix)));
    if (ring < 1) ring = 1;
    while (2 * ring * (ring - 1) > pix) --ring;   /* rings 1..ring-1 hold 2 ring (ring-1) */
    while (2 * (ring + 1) * ring <= pix) ++ring;
    j = pix - 2 * ring * (ring - 1);             /* 0-based within the ring */
    nring = 4 * ring;
    const double t = (double)(ring * ring) / (3.0 * (double)nside * (double)nside);
    z = 1.0 - t;
    s = sqrt(t * (2.0 - t));
    *phi = (pi / (2.0 * (double)ring)) * ((double)j + 0.5);
  } else if (pix >= npix - ncap) {
    const int64_t q = npix - 1 - pix; /* 0-based from the south pole, reversed */
    ring = (int64_t)floor(0.5 * (1.0 + sqrt(1.0 + 2.0 * (double)q)));
    if (ring < 1) ring = 1;
    while (2 * ring * (ring - 1) > q) --ring;
    while (2 * (ring + 1) * ring <= q) ++ring;
    const int64_t jr = q - 2 * ring * (ring - 1); /* counted from the ring's end */
    nring = 4 * ring;
    j = nring - 1 - jr;
    const double t = (double)(ring * ring) / (3.0 * (double)nside * (double)nside);
    z = t - 1.0;
    s = sqrt(t * (2.0 - t));
    *phi = (pi / (2.0 * (double)ring)) * ((double)j + 0.5);
  } else {
    const int64_t q = pix - ncap;
    ring = nside + q / (4 * nside);
    j = q % (4 * nside);
    nring = 4 * nside;
    z = (4.0 / 3.0) - 2.0 * (double)ring / (3.0 * (double)nside);
    s = sqrt((1.0 - z) * (1.0 + z));
    /* rings with ring - nside even start half a pixel east of phi = 0 */
    const double shift = ((ring - nside) % 2 == 0) ? 0.5 : 0.0;
    *phi = (pi / (2.0 * (double)nside)) * ((double)j + shift);
  }
  (void)nring;
  *theta = atan2(s, z);
}

/* theta, phi of RING pixels [begin, begin + count). */
void srto_pix2ang_ring_range(int64_t nside, int64_t begin, int64_t count, double* theta, double* phi) {
  for (int64_t i = 0; i < count; ++i) srto_pix2ang_ring(nside, begin + i, &theta[i], &phi[i]);
}

/* ------------------------------------------------------------ tracing */

/* Initial state (snapshot-raytracer.cu:560) and extraction (:566-582) around
 * the RK4 integration, for one ray of colatitude th and longitude ph. */
static void or_trace_ray(const or_fields* F, int mode, double th, double ph, int n_steps, float out[6]) {
  double y[19] = {(double)F->n[0] * 0.5,
                  (double)F->n[1] * 0.5,
                  (double)F->n[2] * 0.5,
                  -sin(th) * cos(ph),
                  -sin(th) * sin(ph),
                  -cos(th),
                  cos(th) * cos(ph),
                  cos(th) * sin(ph),
                  -sin(th),
                  sin(ph),
                  -cos(ph),
                  0.0,
                  0.0,
                  -1.0,
                  0.0,
                  0.0,
                  0.0,
                  0.0,
                  0.0};
  if (mode == OR_MODE_REF16)
    integrate_ref16(y, n_steps, F);
  else
    integrate_fp64(y, n_steps, F);
  y[0] -= (double)F->n[0] * 0.5;
  y[1] -= (double)F->n[1] * 0.5;
  y[2] -= (double)F->n[2] * 0.5;
  const double norm = sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
  y[0] = y[0] / norm - sin(th) * cos(ph);
  y[1] = y[1] / norm - sin(th) * sin(ph);
  y[2] = y[2] / norm - cos(th);
  out[0] = (float)y[12];
  out[1] = (float)y[16];
  out[2] = (float)y[17];
  out[3] = (float)y[18];
  out[4] = (float)(y[0] * cos(th) * cos(ph) + y[1] * cos(th) * sin(ph) - y[2] * sin(th));
  out[5] = (float)(y[0] * sin(ph) - y[1] * cos(ph));
}

/* Build the per-mode field view from phi and the interleaved B
 * (b_xyz[3 v + c], snapshot-raytracer.cu:91). REF16 quantises each
 * component as half(B * 2^27) (:589-595). */
static int or_fields_init(or_fields* F, const float* phi, const float* b_xyz, float* planes,
                          int64_t n0, int64_t n1, int64_t n2, int mode) {
  const int64_t nv = n0 * n1 * n2;
  F->n[0] = n0;
  F->n[1] = n1;
  F->n[2] = n2;
  F->phi = phi;
  for (int c = 0; c < 3; ++c) {
    F->b[c] = planes + c * nv;
    F->bh[c] = NULL;
  }
  for (int64_t v = 0; v < nv; ++v)
    for (int c = 0; c < 3; ++c) planes[c * nv + v] = b_xyz[3 * v + c];
  if (mode == OR_MODE_REF16) {
    for (int c = 0; c < 3; ++c) {
      F->bh[c] = (uint16_t*)malloc((size_t)nv * sizeof(uint16_t));
      if (!F->bh[c]) return -3;
      for (int64_t v = 0; v < nv; ++v) F->bh[c][v] = or_float_to_half(planes[c * nv + v] * 134217728.0f);
    }
  }
  return 0;
}

static void or_fields_free(or_fields* F) {
  for (int c = 0; c < 3; ++c) free(F->bh[c]);
}

/* Laid-out fields kept between calls (the planes and, for REF16, the FP16 B
 * planes are built once; phi is read from the caller's array, which must
 * outlive the handle). */
typedef struct {
  or_fields F;
  float* planes;
  int mode;
} srto_handle;

void* srto_fields_new(const float* phi, const float* b_xyz, int64_t n0, int64_t n1, int64_t n2, int mode) {
  if (n0 < 1 || n1 < 1 || n2 < 1) return NULL;
  if (mode != OR_MODE_FP64 && mode != OR_MODE_REF16) return NULL;
  srto_handle* h = (srto_handle*)calloc(1, sizeof(srto_handle));
  if (!h) return NULL;
  h->mode = mode;
  h->planes = (float*)malloc((size_t)(3 * n0 * n1 * n2) * sizeof(float));
  if (!h->planes || or_fields_init(&h->F, phi, b_xyz, h->planes, n0, n1, n2, mode) != 0) {
    or_fields_free(&h->F);
    free(h->planes);
    free(h);
    return NULL;
  }
  return h;
}

void srto_fields_delete(void* hv) {
  srto_handle* h = (srto_handle*)hv;
  if (!h) return;
  or_fields_free(&h->F);
  free(h->planes);
  free(h);
}

/* Trace the RING pixels listed in `pix` (count entries) through the fields of
 * handle h and write maps[m * count + i] for map m of pixel pix[i]. */
int srto_trace_pixels_h(void* hv, int64_t nside, const int64_t* pix, int64_t count, int n_steps, float* maps,
                        int nthreads) {
  srto_handle* h = (srto_handle*)hv;
  if (!h || nside < 1 || n_steps < 1 || count < 0) return -1;
  const int64_t npix = 12 * nside * nside;
  for (int64_t i = 0; i < count; ++i)
    if (pix[i] < 0 || pix[i] >= npix) return -1;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int64_t i = 0; i < count; ++i) {
    double th, ph;
    float out[6];
    srto_pix2ang_ring(nside, pix[i], &th, &ph);
    or_trace_ray(&h->F, h->mode, th, ph, n_steps, out);
    for (int m = 0; m < 6; ++m) maps[m * count + i] = out[m];
  }
  return 0;
}

/* Trace the RING pixels listed in `pix` (count entries) and write
 * maps[m * count + i] for map m of pixel pix[i]. Returns 0, or a negative
 * code on bad arguments / allocation failure. */
int srto_trace_pixels(const float* phi, const float* b_xyz, int64_t n0, int64_t n1, int64_t n2,
                      int64_t nside, const int64_t* pix, int64_t count, int n_steps, int mode,
                      float* maps, int nthreads) {
  if (n0 < 1 || n1 < 1 || n2 < 1 || nside < 1 || n_steps < 1 || count < 0) return -1;
  if (mode != OR_MODE_FP64 && mode != OR_MODE_REF16) return -1;
  const int64_t npix = 12 * nside * nside;
  for (int64_t i = 0; i < count; ++i)
    if (pix[i] < 0 || pix[i] >= npix) return -1;
  void* h = srto_fields_new(phi, b_xyz, n0, n1, n2, mode);
  if (!h) return -3;
  const int rc = srto_trace_pixels_h(h, nside, pix, count, n_steps, maps, nthreads);
  srto_fields_delete(h);
  return rc;
}

/* Trace RING pixels [pix_begin, pix_begin + pix_count). */
int srto_trace(const float* phi, const float* b_xyz, int64_t n0, int64_t n1, int64_t n2, int64_t nside,
               int64_t pix_begin, int64_t pix_count, int n_steps, int mode, float* maps, int nthreads) {
  if (nside < 1 || pix_begin < 0 || pix_count < 0 || pix_begin + pix_count > 12 * nside * nside) return -1;
  int64_t* pix = (int64_t*)malloc((size_t)(pix_count > 0 ? pix_count : 1) * sizeof(int64_t));
  if (!pix) return -3;
  for (int64_t i = 0; i < pix_count; ++i) pix[i] = pix_begin + i;
  const int rc = srto_trace_pixels(phi, b_xyz, n0, n1, n2, nside, pix, pix_count, n_steps, mode, maps, nthreads);
  free(pix);
  return rc;
}

/* Interpolation of one field at one point (test access to the scheme):
 * field 0..2 = B components, 3 = phi; out = value, grad[3], hess (xx, xy, xz,
 * yy, yz, zz). */
int srto_interp(const float* phi, const float* b_xyz, int64_t n0, int64_t n1, int64_t n2, int mode,
                int field, double x, double y, double z, double out[10]) {
  const int64_t nv = n0 * n1 * n2;
  float* planes = (float*)malloc((size_t)(3 * nv) * sizeof(float));
  if (!planes) return -3;
  or_fields F;
  memset(&F, 0, sizeof(F));
  or_fields_init(&F, phi, b_xyz, planes, n0, n1, n2, mode);
  if (mode == OR_MODE_REF16) {
    float g[3], h[3][3];
    const float v = tricubic_ref16(&F, field, x, y, z, g, h);
    out[0] = v;
    for (int i = 0; i < 3; ++i) out[1 + i] = g[i];
    out[4] = h[0][0]; out[5] = h[0][1]; out[6] = h[0][2]; out[7] = h[1][1]; out[8] = h[1][2]; out[9] = h[2][2];
  } else {
    double g[3], h[3][3];
    const double v = tricubic_fp64(&F, field, x, y, z, g, h);
    out[0] = v;
    for (int i = 0; i < 3; ++i) out[1 + i] = g[i];
    out[4] = h[0][0]; out[5] = h[0][1]; out[6] = h[0][2]; out[7] = h[1][1]; out[8] = h[1][2]; out[9] = h[2][2];
  }
  or_fields_free(&F);
  free(planes);
  return 0;
}

int srto_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
