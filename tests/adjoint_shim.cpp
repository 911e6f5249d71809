// Host build of the FP64 right-hand side and its hand-written vjp
// (snapshot-raytracer_gb300/csrc/srt_scheme.cuh rhs_std, srt_adjoint.cuh
// rhs_vjp) for tests/test_rhs_vjp_host.py. Fields are halo-padded float arrays
// (extents n + 3, voxel (i, j, k) at (i+1) + px ((j+1) + py (k+1))); the tap
// cotangents are accumulated into padded double arrays.
#include "srt_adjoint.cuh"

namespace {
srt::Geom geom(int n0, int n1, int n2) {
  srt::Geom G;
  const int n[3] = {n0, n1, n2};
  for (int i = 0; i < 3; ++i) {
    G.n[i] = n[i];
    G.invn[i] = 1.0f / (float)n[i];
  }
  G.px = n0 + 3;
  G.pxy = (int64_t)(n0 + 3) * (n1 + 3);
  G.pxy2 = (int64_t)(n0 + 3) * (n1 + 2);
  return G;
}
srt::FieldPtrs ptrs(const float* phi, const float* bx, const float* by, const float* bz) {
  srt::FieldPtrs F = {};
  F.phi = phi;
  F.b[0] = bx;
  F.b[1] = by;
  F.b[2] = bz;
  return F;
}
}  // namespace

extern "C" {
// dy = f(y) of the FP64 form (19 components).
void rhs_fp64(const double* y, double* dy, const float* phi, const float* bx, const float* by, const float* bz,
              int n0, int n1, int n2) {
  srt::rhs_std<srt::kFP64>(y, dy, ptrs(phi, bx, by, bz), geom(n0, n1, n2));
}

// yb += J(y)^T fb, and the cotangents of the four fields' padded values
// (g: B_x, B_y, B_z, phi) += d(fb . f)/d(field value).
void rhs_vjp_fp64(const double* y, const double* fb, double* yb, double* gbx, double* gby, double* gbz, double* gphi,
                  const float* phi, const float* bx, const float* by, const float* bz, int n0, int n1, int n2) {
  const srt::Geom G = geom(n0, n1, n2);
  srt::StageView<double> V;
  srt::stage_view_fp64(y, G, V);
  srt::AccF64 acc[4];
  acc[0].g = gbx;
  acc[1].g = gby;
  acc[2].g = gbz;
  acc[3].g = gphi;
  srt::rhs_vjp<double, srt::AccF64, false>(V, ptrs(phi, bx, by, bz), G, fb, yb, acc);
}
}
