// Host build of the FP64 right-hand side and its hand-written vjp
// (snapshot-raytracer_gb300/csrc/srt_scheme.cuh rhs_std, srt_adjoint.cuh
// rhs_vjp) for tests/test_rhs_vjp_host.py. Fields are halo-padded float arrays
// (extents n + 3, voxel (i, j, k) at (i+1) + px ((j+1) + py (k+1))); the tap
// cotangents are accumulated into padded double arrays.
#include <vector>
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
  srt::rhs_vjp<double, srt::AccF64, srt::AccF64, false>(V, ptrs(phi, bx, by, bz), G, fb, yb, acc, acc[3]);
}

// Index audit of the MIXED sweep (rhs_vjp<float> on stage_view_mixed, as
// sweep_kernel_mixed runs it) on an n0 x n1 x n2 grid: for each ray
// (theta[r], phi[r]) at affine parameter s[r] with the perturbation state
// d[19 r .. 19 r + 18], records the smallest and largest single-layout index
// any tap read or tap-cotangent row touches (rows of 4 taps from `row`) and
// the largest row-pair index the PAIR variant would read. out: [min index,
// max index, max pair index, padded voxel count, row-pair element count].
// The fields are zero (only the indices matter).
namespace {
struct AccAudit {
  int64_t* lo;
  int64_t* hi;
  SRT_HD bool active() const { return true; }
  SRT_HD void add_row(int64_t row, float, float, float, float) const {
    if (row < *lo) *lo = row;
    if (row + 3 > *hi) *hi = row + 3;
  }
};
}  // namespace

void audit_vjp_indices_mixed(int n0, int n1, int n2, int count, const double* theta, const double* phi,
                             const float* s, const float* d, int64_t* out) {
  const srt::Geom G = geom(n0, n1, n2);
  const int64_t pvox = (int64_t)(n0 + 3) * (n1 + 3) * (n2 + 3);
  const int64_t npair = (int64_t)(n0 + 3) * (n1 + 2) * (n2 + 3);
  std::vector<float> zero((size_t)pvox, 0.f);
  const srt::FieldPtrs F = ptrs(zero.data(), zero.data(), zero.data(), zero.data());
  int64_t lo = INT64_MAX, hi = -1, hip = -1;
  AccAudit acc[4];
  for (int f = 0; f < 4; ++f) acc[f] = AccAudit{&lo, &hi};
  float x0[3];
  srt::mixed_observer(G, x0);
  for (int r = 0; r < count; ++r) {
    srt::MixedRay R;
    float y[srt::kMixedState];
    srt::init_mixed(srt::ray_dir(theta[r], phi[r]), R, y);
    srt::StageView<float> V;
    srt::stage_view_mixed(d + 19 * r, s[r], R, G, x0, V);
    float fb[19], yb[19];
    for (int j = 0; j < 19; ++j) {
      fb[j] = 1.f;
      yb[j] = 0.f;
    }
    srt::rhs_vjp<float, AccAudit, AccAudit, false>(V, F, G, fb, yb, acc, acc[3]);
    for (int f = 0; f < 4; ++f) {
      // the PAIR pass reads pair basep + c pxy2 + 2 pr px + i (c <= 3, pr <= 1, i <= 3)
      const int64_t last = V.basep[f] + 3 * G.pxy2 + 2 * G.px + 3;
      if (last > hip) hip = last;
      if (V.basep[f] < lo) lo = V.basep[f];
    }
  }
  out[0] = lo;
  out[1] = hi;
  out[2] = hip;
  out[3] = pvox;
  out[4] = npair;
}
}

