// Host build of the MIXED form's cell lookup and normalisation term
// (snapshot-raytracer_gb300/csrc/srt_scheme.cuh: locate_mixed, rsqrt1p_m1) for
// tests/test_locate_mixed.py.
#include "srt_scheme.cuh"
extern "C" {
void locate(float th, float lo, int n, int* cc, float* tc, int* cs, float* ts, float* df) {
  srt::locate_mixed(th, lo, n, 1.0f / (float)n, *cc, *tc, *cs, *ts, *df);
}
// (1 + q)^(-1/2) - 1 as the MIXED form's normalisation takes it
float rsqrt1p_m1(float q) { return srt::rsqrt1p_m1(q); }
}

// The MIXED trace of RING pixels [ring_begin, ring_begin + count) on the host,
// from halo-padded fields (extents n + 3 per axis, voxel (i, j, k) at
// (i+1) + px ((j+1) + py (k+1))) and the single layout: maps[m * count + r]
// and whether ray r came within the cell-face guard (the GPU re-traces those
// in FP64; this host build does not).
extern "C" int trace_mixed_host(const float* phi, const float* bx, const float* by, const float* bz, int n0, int n1,
                                int n2, long long nside, long long ring_begin, long long count, int n_steps,
                                float* maps, int* flagged) {
  srt::Geom G;
  const int n[3] = {n0, n1, n2};
  for (int i = 0; i < 3; ++i) {
    G.n[i] = n[i];
    G.invn[i] = 1.0f / (float)n[i];
  }
  G.px = n0 + 3;
  G.pxy = (int64_t)(n0 + 3) * (n1 + 3);
  G.pxy2 = (int64_t)(n0 + 3) * (n1 + 2);
  srt::FieldPtrs F = {};
  F.phi = phi;
  F.b[0] = bx;
  F.b[1] = by;
  F.b[2] = bz;
  for (long long r = 0; r < count; ++r) {
    const srt::RayDir d = srt::ray_dir_pix(nside, ring_begin + r);
    float out[6], m[2];
    flagged[r] = srt::trace_ray_mixed<false>(F, G, d, n_steps, out, m) ? 1 : 0;
    for (int k = 0; k < 6; ++k) maps[k * count + r] = out[k];
  }
  return 0;
}
