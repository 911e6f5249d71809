// srt_healpix.cuh — HEALPix RING/NESTED geometry for host and device code.
//
// The reference gets ray directions from chealpix pix2ang_ring64 on the host
// (snapshot-raytracer.cu:862-866). chealpix is a third-party dependency that is
// not vendored with the reference and whose version is not pinned (its
// Makefile links -lchealpix). What follows is written from the published
// HEALPix scheme (Gorski et al. 2005, ApJ 622, 759, section 4 and the
// RING/NESTED index relations of its appendix):
//   * 12 base faces, nside^2 pixels each, npix = 12 nside^2;
//   * RING index runs ring by ring from the north pole; the polar caps hold
//     2 nside (nside-1) pixels each, ring i of a cap has 4 i pixels;
//   * z = cos(theta) = 1 - i^2 / (3 nside^2) on north-cap ring i,
//     z = (4/3) - 2 i / (3 nside) on equatorial ring i (nside <= i <= 3 nside);
//   * pixel centres in cap ring i sit at phi = (pi / (2 i)) (j - 1/2),
//     j = 1 .. 4 i; in equatorial ring i at phi = (pi / (2 nside)) (j - f) with
//     f = 1 when i + nside is odd and f = 1/2 otherwise;
//   * NESTED index = face * nside^2 + bit-interleave(ix, iy) of the face
//     coordinates.
// sin(theta) is returned alongside z so callers never form sqrt(1 - z^2) from
// a rounded z near the poles.
#pragma once
#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define SRT_HD __host__ __device__ __forceinline__
#else
#define SRT_HD inline
#endif

namespace srt {

SRT_HD int64_t hp_isqrt(int64_t v) {
  int64_t r = (int64_t)sqrt((double)v);
  while (r * r > v) --r;
  while ((r + 1) * (r + 1) <= v) ++r;
  return r;
}

// Centre of RING pixel `pix`: z = cos(theta), st = sin(theta), and the
// longitude as a fraction of pi, u = phi / pi.
SRT_HD void hp_ring_zu(int64_t nside, int64_t pix, double* z, double* st, double* u) {
  const int64_t npix = 12 * nside * nside;
  const int64_t ncap = 2 * nside * (nside - 1);
  const double inv3n2 = 1.0 / (3.0 * (double)nside * (double)nside);
  if (pix < ncap) {  // north polar cap
    const int64_t i = (1 + hp_isqrt(1 + 2 * pix)) >> 1;
    const int64_t j = pix + 1 - 2 * i * (i - 1);
    const double t = (double)(i * i) * inv3n2;  // 1 - z
    *z = 1.0 - t;
    *st = sqrt(t * (2.0 - t));
    *u = ((double)j - 0.5) / (2.0 * (double)i);
  } else if (pix < npix - ncap) {  // equatorial belt
    const int64_t q = pix - ncap;
    const int64_t i = q / (4 * nside) + nside;
    const int64_t j = q % (4 * nside) + 1;
    const double f = ((i + nside) & 1) ? 1.0 : 0.5;
    const double zz = (double)(2 * nside - i) * (2.0 / (3.0 * (double)nside));
    *z = zz;
    *st = sqrt((1.0 - zz) * (1.0 + zz));
    *u = ((double)j - f) / (2.0 * (double)nside);
  } else {  // south polar cap
    const int64_t q = npix - pix;
    const int64_t i = (1 + hp_isqrt(2 * q - 1)) >> 1;
    const int64_t j = 4 * i + 1 - (q - 2 * i * (i - 1));
    const double t = (double)(i * i) * inv3n2;  // 1 + z
    *z = t - 1.0;
    *st = sqrt(t * (2.0 - t));
    *u = ((double)j - 0.5) / (2.0 * (double)i);
  }
}

// Same centre with the longitude in radians.
SRT_HD void hp_ring_zphi(int64_t nside, int64_t pix, double* z, double* st, double* phi) {
  double u;
  hp_ring_zu(nside, pix, z, st, &u);
  *phi = 3.141592653589793238462643383279502884 * u;
}

// theta, phi of a RING pixel centre (theta from atan2 of the exact sin/cos pair).
SRT_HD void hp_pix2ang_ring(int64_t nside, int64_t pix, double* theta, double* phi) {
  double z, st;
  hp_ring_zphi(nside, pix, &z, &st, phi);
  *theta = atan2(st, z);
}

// Face coordinates <-> in-face NESTED index (Morton interleave: x in even bits).
SRT_HD void hp_deinterleave(int64_t v, int64_t* ix, int64_t* iy) {
  uint64_t x = (uint64_t)v & 0x5555555555555555ull, y = ((uint64_t)v >> 1) & 0x5555555555555555ull;
  x = (x | (x >> 1)) & 0x3333333333333333ull;
  x = (x | (x >> 2)) & 0x0f0f0f0f0f0f0f0full;
  x = (x | (x >> 4)) & 0x00ff00ff00ff00ffull;
  x = (x | (x >> 8)) & 0x0000ffff0000ffffull;
  x = (x | (x >> 16)) & 0x00000000ffffffffull;
  y = (y | (y >> 1)) & 0x3333333333333333ull;
  y = (y | (y >> 2)) & 0x0f0f0f0f0f0f0f0full;
  y = (y | (y >> 4)) & 0x00ff00ff00ff00ffull;
  y = (y | (y >> 8)) & 0x0000ffff0000ffffull;
  y = (y | (y >> 16)) & 0x00000000ffffffffull;
  *ix = (int64_t)x;
  *iy = (int64_t)y;
}

SRT_HD int64_t hp_interleave(int64_t ix, int64_t iy) {
  uint64_t x = (uint64_t)ix, y = (uint64_t)iy;
  x = (x | (x << 16)) & 0x0000ffff0000ffffull;
  x = (x | (x << 8)) & 0x00ff00ff00ff00ffull;
  x = (x | (x << 4)) & 0x0f0f0f0f0f0f0f0full;
  x = (x | (x << 2)) & 0x3333333333333333ull;
  x = (x | (x << 1)) & 0x5555555555555555ull;
  y = (y | (y << 16)) & 0x0000ffff0000ffffull;
  y = (y | (y << 8)) & 0x00ff00ff00ff00ffull;
  y = (y | (y << 4)) & 0x0f0f0f0f0f0f0f0full;
  y = (y | (y << 2)) & 0x3333333333333333ull;
  y = (y | (y << 1)) & 0x5555555555555555ull;
  return (int64_t)(x | (y << 1));
}

// Base-face placement: face f has its southern vertex on ring
// hp_face_ring(f) * nside and is centred at longitude hp_face_phi(f) * pi / 4.
SRT_HD int hp_face_ring(int f) { return f < 4 ? 2 : (f < 8 ? 3 : 4); }
SRT_HD int hp_face_phi(int f) { return f < 4 ? 2 * f + 1 : (f < 8 ? 2 * (f - 4) : 2 * (f - 8) + 1); }

// RING index of the pixel with face coordinates (ix, iy) on base face `face`
// (0 <= ix, iy < nside; any nside >= 1).
SRT_HD int64_t hp_xyf2ring(int64_t nside, int64_t ix, int64_t iy, int face) {
  const int64_t npix = 12 * nside * nside, ncap = 2 * nside * (nside - 1);
  const int64_t jr = (int64_t)hp_face_ring(face) * nside - ix - iy - 1;  // ring, from north
  int64_t nr, nbefore, kshift;
  if (jr < nside) {
    nr = jr;
    nbefore = 2 * nr * (nr - 1);
    kshift = 0;
  } else if (jr > 3 * nside) {
    nr = 4 * nside - jr;
    nbefore = npix - 2 * (nr + 1) * nr;
    kshift = 0;
  } else {
    nr = nside;
    nbefore = ncap + (jr - nside) * 4 * nside;
    kshift = (jr - nside) & 1;
  }
  int64_t jp = ((int64_t)hp_face_phi(face) * nr + ix - iy + 1 + kshift) / 2;
  if (jp > 4 * nr) jp -= 4 * nr;
  if (jp < 1) jp += 4 * nr;
  return nbefore + jp - 1;
}

SRT_HD bool hp_is_pow2(int64_t nside) { return nside > 0 && (nside & (nside - 1)) == 0; }

// NESTED -> RING; the NESTED scheme exists only for power-of-two nside.
SRT_HD int64_t hp_nest2ring(int64_t nside, int64_t ipnest) {
  const int64_t npface = nside * nside;
  int64_t ix, iy;
  hp_deinterleave(ipnest % npface, &ix, &iy);
  return hp_xyf2ring(nside, ix, iy, (int)(ipnest / npface));
}

SRT_HD int64_t hp_ring2nest(int64_t nside, int64_t ipring) {
  const int64_t npix = 12 * nside * nside, ncap = 2 * nside * (nside - 1);
  int64_t iring, iphi, kshift, nr;
  int face;
  if (ipring < ncap) {
    iring = (1 + hp_isqrt(1 + 2 * ipring)) >> 1;
    iphi = ipring + 1 - 2 * iring * (iring - 1);
    kshift = 0;
    nr = iring;
    face = (int)((iphi - 1) / nr);
  } else if (ipring < npix - ncap) {
    const int64_t q = ipring - ncap;
    const int64_t t = q / (4 * nside);
    iring = t + nside;
    iphi = q - t * 4 * nside + 1;
    kshift = (iring + nside) & 1;
    nr = nside;
    const int64_t ire = iring - nside + 1, irm = 2 * nside + 2 - ire;
    const int64_t ifm = (iphi - ire / 2 + nside - 1) / nside;
    const int64_t ifp = (iphi - irm / 2 + nside - 1) / nside;
    if (ifp == ifm)
      face = (int)((ifp == 4) ? 4 : ifp + 4);
    else if (ifp < ifm)
      face = (int)ifp;
    else
      face = (int)(ifm + 8);
  } else {
    const int64_t q = npix - ipring;
    iring = (1 + hp_isqrt(2 * q - 1)) >> 1;
    iphi = 4 * iring + 1 - (q - 2 * iring * (iring - 1));
    kshift = 0;
    nr = iring;
    iring = 4 * nside - iring;
    face = (int)(8 + (iphi - 1) / nr);
  }
  const int64_t irt = iring - (int64_t)hp_face_ring(face) * nside + 1;
  int64_t ipt = 2 * iphi - (int64_t)hp_face_phi(face) * nr - kshift - 1;
  if (ipt >= 2 * nside) ipt -= 8 * nside;
  const int64_t ix = (ipt - irt) >> 1, iy = (-ipt - irt) >> 1;
  return (int64_t)face * nside * nside + hp_interleave(ix, iy);
}

}  // namespace srt
