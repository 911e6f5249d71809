// ref_harness.cu — builds the reference's OWN host code for the tracer's path
// (snapshot-raytracer.cu, compiled from where it lies in the reference tree)
// into a shared library, oracle/_ref/libsrt_ref.so. TEST INFRASTRUCTURE: it
// produces the golden vectors of tests/golden/ and pins the oracle port.
//
// The reference's raytracing() (snapshot-raytracer.cu:513-550) and everything
// it calls are __host__ __device__, so including the source and calling
// raytracing() from host code runs the reference's own arithmetic on the CPU.
// The initial state (:560) and the extraction (:566-582) live inside the
// __global__ raytracing_kernel, which cannot run on the host; they are
// restated below around the call. B is quantised exactly as vector3_to_half
// does (:585-597): half(B * 2^27) with __float2half.
// Build recipe: oracle/build_ref.sh (stub hdf5/chealpix headers from
// oracle/stubs; main() renamed so it is not the library's entry point).
#define main srt_reference_cli_main
#include "snapshot-raytracer.cu"
#undef main

#include <cstring>

namespace {
// The reference's device-side inputs, staged once: phi (the caller's array,
// which must outlive the handle), B quantised as vector3_to_half does.
struct RefFields {
  const float* phi;
  std::vector<__half> h1, h2, h3;
  int dims[3];
};
}  // namespace

extern "C" void* srtref_fields_new(const float* phi, const float* b_xyz, int n0, int n1, int n2) {
  RefFields* f = new RefFields;
  const int64_t nv = (int64_t)n0 * n1 * n2;
  f->phi = phi;
  f->h1.resize(nv);
  f->h2.resize(nv);
  f->h3.resize(nv);
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < nv; ++v) {
    f->h1[v] = __float2half(b_xyz[3 * v + 0] * 134217728.0f);
    f->h2[v] = __float2half(b_xyz[3 * v + 1] * 134217728.0f);
    f->h3[v] = __float2half(b_xyz[3 * v + 2] * 134217728.0f);
  }
  f->dims[0] = n0;
  f->dims[1] = n1;
  f->dims[2] = n2;
  return f;
}

extern "C" void srtref_fields_delete(void* h) { delete (RefFields*)h; }

extern "C" int srtref_trace_angles_h(void* h, const double* theta, const double* phiang, int64_t nrays, int n_steps,
                                     float* maps, int nthreads) {
  const RefFields* f = (const RefFields*)h;
  const int* dims = f->dims;
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t i = 0; i < nrays; ++i) {
    const double th = theta[i], ph = phiang[i];
    double y[19] = {static_cast<double>(dims[0]) * 0.5, static_cast<double>(dims[1]) * 0.5,
                    static_cast<double>(dims[2]) * 0.5, -std::sin(th) * std::cos(ph),
                    -std::sin(th) * std::sin(ph), -std::cos(th), std::cos(th) * std::cos(ph),
                    std::cos(th) * std::sin(ph), -std::sin(th), std::sin(ph), -std::cos(ph),
                    0.0, 0.0, -1.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    raytracing(f->phi, f->h1.data(), f->h2.data(), f->h3.data(), dims, y, n_steps);
    y[0] -= static_cast<double>(dims[0]) * 0.5;
    y[1] -= static_cast<double>(dims[1]) * 0.5;
    y[2] -= static_cast<double>(dims[2]) * 0.5;
    const double norm = std::sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
    y[0] = y[0] / norm - std::sin(th) * std::cos(ph);
    y[1] = y[1] / norm - std::sin(th) * std::sin(ph);
    y[2] = y[2] / norm - std::cos(th);
    maps[0 * nrays + i] = static_cast<float>(y[12]);
    maps[1 * nrays + i] = static_cast<float>(y[16]);
    maps[2 * nrays + i] = static_cast<float>(y[17]);
    maps[3 * nrays + i] = static_cast<float>(y[18]);
    maps[4 * nrays + i] = static_cast<float>(y[0] * std::cos(th) * std::cos(ph) +
                                             y[1] * std::cos(th) * std::sin(ph) - y[2] * std::sin(th));
    maps[5 * nrays + i] = static_cast<float>(y[0] * std::sin(ph) - y[1] * std::cos(ph));
  }
  return 0;
}

extern "C" int srtref_trace_angles(const float* phi, const float* b_xyz, int n0, int n1, int n2,
                                   const double* theta, const double* phiang, int64_t nrays,
                                   int n_steps, float* maps, int nthreads) {
  void* h = srtref_fields_new(phi, b_xyz, n0, n1, n2);
  const int rc = srtref_trace_angles_h(h, theta, phiang, nrays, n_steps, maps, nthreads);
  srtref_fields_delete(h);
  return rc;
}

// The reference's own tricubic_interpolation (snapshot-raytracer.cu:215-312)
// at one point, for unit tests of the oracle's interpolation. field 0..2 =
// B components (half planes), 3 = phi. out = value, grad[3], hess xx xy xz yy yz zz.
extern "C" int srtref_interp(const float* phi, const float* b_xyz, int n0, int n1, int n2, int field,
                             double x, double y, double z, double* out) {
  const int64_t nv = (int64_t)n0 * n1 * n2;
  const int dims[3] = {n0, n1, n2};
  float g[3], h[3][3], v;
  if (field == 3) {
    v = tricubic_interpolation(phi, dims, x, y, z, g, h);
  } else {
    std::vector<__half> hb(nv);
    for (int64_t i = 0; i < nv; ++i) hb[i] = __float2half(b_xyz[3 * i + field] * 134217728.0f);
    v = tricubic_interpolation(hb.data(), dims, x, y, z, g, h);
  }
  out[0] = v;
  for (int i = 0; i < 3; ++i) out[1 + i] = g[i];
  out[4] = h[0][0]; out[5] = h[0][1]; out[6] = h[0][2]; out[7] = h[1][1]; out[8] = h[1][2]; out[9] = h[2][2];
  return 0;
}
