// srt_cli.cpp — the snapshot-raytracer command line, a drop-in for the
// reference's main() (snapshot-raytracer.cu:600-1007) on top of libsrt:
//
//   snapshot-raytracer <hdf5_file_potential> <hdf5_file_B> <Nside> <n_steps> [<batch>]
//
// Same positional arguments, same /data datasets, same stdout progress lines,
// same stderr diagnostics and exit status (255 for every error the reference
// reports with `return -1`), and the same six RING-ordered FITS maps in the
// working directory: dAmap_batchN.fits, ellipticity1map_batchN.fits,
// ellipticity2map_batchN.fits, rotationmap_batchN.fits,
// deflection1map_batchN.fits, deflection2map_batchN.fits, zero outside the
// batch's RING pixel range [batch*Nside^2, (batch+1)*Nside^2) (without a
// batch: all pixels, written as batch0). Like cfitsio, an existing output file
// is not replaced (a message goes to stderr and the run continues).
//
// Options after the positional arguments (none changes their meaning):
//   --precision mixed|fp64|ref16  arithmetic of the trace (default mixed; also
//                                 taken from SRT_PRECISION); ref16 reproduces
//                                 the reference's FP16/FP32 arithmetic
//   --overwrite                   replace existing output files
//   --outdir DIR                  write the maps to DIR instead of the cwd
//   --timing                      print one JSON line with phase timings
//   --base-pixel                  batch b is HEALPix base pixel b (the NESTED
//                                 range [b*Nside^2, (b+1)*Nside^2), which the
//                                 reference's README describes; Nside a power
//                                 of two) instead of the RING range
//   --xyz-order hdf5              x is the fastest HDF5 axis with its own
//                                 extent (n0 = dims[2], n2 = dims[0]), which
//                                 keeps non-cubic grids consistent; by default
//                                 n0 = dims[0], as the reference does
//   --rescale-phi F, --rescale-b F
//                                 multiply the potential / the B field by F
//                                 after loading, with the reference's message
//                                 (its compile-time RESCALE_DATA / RESCALE_BDATA,
//                                 snapshot-raytracer.cu:663-670, :681-688):
//                                 each value is multiplied in double and
//                                 rounded back to float
//
// The six maps are written by six threads at once.
//
// Deviations, all on inputs the reference mishandles: a non-numeric Nside /
// n_steps / batch is reported as an error instead of an uncaught exception, and
// B dimensions that differ from phi's are rejected (the reference would read
// out of bounds, snapshot-raytracer.cu:676).
#include <cerrno>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <thread>
#include <vector>
#include "srt.h"

namespace {

std::string last_error() {
  char buf[1024];
  srt_last_error(buf, sizeof(buf));
  return buf;
}

bool parse_i64(const char* s, int64_t* v) {
  char* end = nullptr;
  errno = 0;
  const long long x = strtoll(s, &end, 10);
  if (end == s || errno != 0) return false;
  *v = x;
  return true;
}

bool parse_f64(const char* s, double* v) {
  char* end = nullptr;
  errno = 0;
  const double x = strtod(s, &end);
  if (end == s || *end != '\0' || errno != 0 || !(x - x == 0.0)) return false;
  *v = x;
  return true;
}

// data[i] = float(data[i] * factor) over count values, on all host threads.
void rescale(float* data, int64_t count, double factor) {
  unsigned nt = std::thread::hardware_concurrency();
  if (nt < 1) nt = 1;
  if (count < (int64_t(1) << 20)) nt = 1;
  std::vector<std::thread> pool;
  const int64_t chunk = (count + nt - 1) / nt;
  for (unsigned t = 0; t < nt; ++t) {
    const int64_t lo = t * chunk, hi = lo + chunk < count ? lo + chunk : count;
    if (lo >= hi) break;
    pool.emplace_back([=] {
      for (int64_t i = lo; i < hi; ++i) data[i] = (float)((double)data[i] * factor);
    });
  }
  for (auto& th : pool) th.join();
}

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

void usage(const char* prog) {
  std::cerr << "Usage: " << prog << " <hdf5_file_potential> <hdf5_file_B> <Nside> <n_steps> [<batch>]" << std::endl;
  std::cerr << "  <hdf5_file_potential>: HDF5 file containing a snapshot of the Weyl potential" << std::endl;
  std::cerr << "  <hdf5_file_B>: HDF5 file containing a snapshot of the frame-dragging potential (shift)" << std::endl;
  std::cerr << "  <Nside>: HEALPix Nside parameter for output maps" << std::endl;
  std::cerr << "  <n_steps>: Number of integration steps for raytracing (1 step = 1 grid unit)" << std::endl;
  std::cerr << "  [<batch>]: Optional batch index for processing a subset of pixels" << std::endl;
  std::cerr << "  options: [--precision mixed|fp64|ref16] [--overwrite] [--outdir DIR] [--timing] [--base-pixel]"
               " [--xyz-order reference|hdf5] [--rescale-phi F] [--rescale-b F]" << std::endl;
}

}  // namespace

int main(int argc, char* argv[]) {
  std::vector<const char*> pos;
  int precision = SRT_PRECISION_MIXED;
  bool overwrite = false, timing = false, base_pixel = false, hdf5_order = false;
  bool rescale_phi = false, rescale_b = false;
  double phi_factor = 1.0, b_factor = 1.0;
  std::string outdir;
  if (const char* e = getenv("SRT_PRECISION")) {
    if (!strcmp(e, "fp64")) precision = SRT_PRECISION_FP64;
    else if (!strcmp(e, "ref16")) precision = SRT_PRECISION_REF16;
  }
  for (int i = 1; i < argc; ++i) {
    if (!strcmp(argv[i], "--precision") && i + 1 < argc) {
      const char* p = argv[++i];
      if (!strcmp(p, "mixed")) precision = SRT_PRECISION_MIXED;
      else if (!strcmp(p, "fp64")) precision = SRT_PRECISION_FP64;
      else if (!strcmp(p, "ref16")) precision = SRT_PRECISION_REF16;
      else {
        std::cerr << "Invalid precision: " << p << std::endl;
        return -1;
      }
    } else if (!strcmp(argv[i], "--overwrite")) {
      overwrite = true;
    } else if (!strcmp(argv[i], "--timing")) {
      timing = true;
    } else if (!strcmp(argv[i], "--outdir") && i + 1 < argc) {
      outdir = argv[++i];
    } else if (!strcmp(argv[i], "--base-pixel")) {
      base_pixel = true;
    } else if ((!strcmp(argv[i], "--rescale-phi") || !strcmp(argv[i], "--rescale-b")) && i + 1 < argc) {
      const bool is_phi = !strcmp(argv[i], "--rescale-phi");
      const char* v = argv[++i];
      double x = 0.0;
      if (!parse_f64(v, &x)) {
        std::cerr << "Invalid rescaling factor: " << v << std::endl;
        return -1;
      }
      (is_phi ? phi_factor : b_factor) = x;
      (is_phi ? rescale_phi : rescale_b) = true;
    } else if (!strcmp(argv[i], "--xyz-order") && i + 1 < argc) {
      const char* o = argv[++i];
      if (!strcmp(o, "hdf5")) hdf5_order = true;
      else if (strcmp(o, "reference")) {
        std::cerr << "Invalid xyz order: " << o << std::endl;
        return -1;
      }
    } else {
      pos.push_back(argv[i]);
    }
  }
  if (pos.size() < 4) {
    usage(argv[0]);
    return -1;
  }
  int64_t nside = 0, steps64 = 0, batch64 = -1;
  if (!parse_i64(pos[2], &nside)) {
    std::cerr << "Invalid Nside value: " << pos[2] << std::endl;
    return -1;
  }
  if (nside <= 0) {
    std::cerr << "Invalid Nside value: " << nside << std::endl;
    return -1;
  }
  if (!parse_i64(pos[3], &steps64) || steps64 > 0x7fffffff || steps64 < -0x7fffffffll) {
    std::cerr << "Invalid n_steps value: " << pos[3] << std::endl;
    return -1;
  }
  const int n_steps = (int)steps64;
  if (n_steps <= 0) {
    std::cerr << "Invalid n_steps value: " << n_steps << std::endl;
    return -1;
  }
  int batch = -1;
  if (pos.size() > 4) {
    if (!parse_i64(pos[4], &batch64) || batch64 > 0x7fffffff || batch64 < -0x7fffffffll) {
      std::cerr << "Invalid batch value: " << pos[4] << std::endl;
      return -1;
    }
    batch = (int)batch64;
    if (batch < 0) {
      std::cerr << "Invalid batch value: " << batch << std::endl;
      return -1;
    }
  }
  const double t_start = now_ms();
  std::cout << "Nside: " << nside << std::endl;
  std::cout << "n_steps: " << n_steps << std::endl;
  std::cout << "Loading potential data from HDF5 file " << pos[0] << " ..." << std::endl;

  float* phi = nullptr;
  int64_t dims[8] = {0};
  int rank = 0;
  if (srt_h5_read_scalar(pos[0], "/data", &phi, dims, &rank) != SRT_OK) {
    std::cerr << last_error() << std::endl;
    return -1;
  }
  if (rank < 3) {
    std::cerr << "Expected a 3D potential dataset, got rank=" << rank << std::endl;
    srt_free(phi);
    return -1;
  }
  std::cout << "Data dimensions: " << dims[0] << " x " << dims[1] << " x " << dims[2] << std::endl;
  if (rescale_phi) {
    std::cout << "Rescaling potential data by factor " << phi_factor << std::endl;
    int64_t count = 1;
    for (int d = 0; d < rank; ++d) count *= dims[d];
    rescale(phi, count, phi_factor);
  }
  const double t_phi = now_ms();

  std::cout << "Loading B field data from HDF5 file " << pos[1] << " ..." << std::endl;
  float* bxyz = nullptr;
  int64_t bdims[3] = {0, 0, 0};
  if (srt_h5_read_vector3(pos[1], "/data", &bxyz, bdims) != SRT_OK) {
    std::cerr << last_error() << std::endl;
    srt_free(phi);
    return -1;
  }
  if (bdims[0] != dims[0] || bdims[1] != dims[1] || bdims[2] != dims[2]) {
    std::cerr << "B field dimensions " << bdims[0] << " x " << bdims[1] << " x " << bdims[2]
              << " differ from the potential's" << std::endl;
    srt_free(phi);
    srt_free(bxyz);
    return -1;
  }
  {
    // the reference's size warning for a large B (snapshot-raytracer.cu:159-161)
    const double b_bytes = 3.0 * (double)bdims[0] * (double)bdims[1] * (double)bdims[2] * sizeof(float);
    if (b_bytes > 8.0 * 1024 * 1024 * 1024)
      std::cerr << "Warning: allocating ~" << b_bytes / (1024.0 * 1024 * 1024) << " GiB for vector field." << std::endl;
  }
  if (rescale_b) {
    std::cout << "Rescaling B field data by factor " << b_factor << std::endl;
    rescale(bxyz, 3 * bdims[0] * bdims[1] * bdims[2], b_factor);
  }
  const double t_b = now_ms();

  const int64_t npix = 12 * nside * nside;
  int64_t istart = 0, count = npix;
  if (batch >= 0) {
    istart = (int64_t)batch * nside * nside;
    count = nside * nside;
    if (istart >= npix) {
      std::cerr << "Batch exceeds total number of pixels" << std::endl;
      srt_free(phi);
      srt_free(bxyz);
      return -1;
    }
  }
  const bool nested = base_pixel && batch >= 0;
  if (nested && (nside & (nside - 1)) != 0) {
    std::cerr << "--base-pixel needs a power-of-two Nside, got " << nside << std::endl;
    srt_free(phi);
    srt_free(bxyz);
    return -1;
  }
  // grid extents, fastest first
  const int64_t g0 = hdf5_order ? dims[2] : dims[0], g2 = hdf5_order ? dims[0] : dims[2];

  std::cout << "Allocating device memory and copying data to device..." << std::endl;
  srt_fields* fields = nullptr;
  if (srt_fields_create(phi, bxyz, g0, dims[1], g2, 0, nullptr, &fields) != SRT_OK) {
    std::cerr << "Failed to copy data to device: " << last_error() << std::endl;
    srt_free(phi);
    srt_free(bxyz);
    return -1;
  }
  srt_free(bxyz);
  srt_free(phi);
  const double t_up = now_ms();

  std::cout << "Computing theta and phi angles..." << std::endl;
  std::vector<float> part((size_t)(6 * count));
  float* rows[6];
  for (int m = 0; m < 6; ++m) rows[m] = part.data() + (size_t)m * count;
  std::cout << "Launching raytracing kernel..." << std::endl;
  srt_stats st;
  if (srt_forward(fields, nside, istart, count, n_steps, precision, rows, nested ? SRT_NESTED_RANGE : 0u, nullptr,
                  &st) != SRT_OK) {
    std::cerr << "Kernel execution error: " << last_error() << std::endl;
    srt_fields_destroy(fields);
    return -1;
  }
  std::cout << "Raytracing completed." << std::endl;
  srt_fields_destroy(fields);
  const double t_trace = now_ms();

  std::cout << "Saving results to FITS files..." << std::endl;
  if (batch < 0) batch = 0;
  static const char* names[6] = {"dAmap", "ellipticity1map", "ellipticity2map", "rotationmap", "deflection1map",
                                 "deflection2map"};
  // one full-sky RING map per thread: the batch's values at their RING
  // index (a NESTED range is scattered through nest2ring), zero elsewhere
  std::vector<std::string> errors(6);
  std::vector<std::thread> writers;
  for (int m = 0; m < 6; ++m) {
    writers.emplace_back([&, m]() {
      std::vector<float> full((size_t)npix, 0.0f);
      if (nested) {
        for (int64_t i = 0; i < count; ++i) full[(size_t)srt_nest2ring(nside, istart + i)] = rows[m][i];
      } else {
        memcpy(full.data() + istart, rows[m], (size_t)count * sizeof(float));
      }
      char fname[512];
      snprintf(fname, sizeof(fname), "%s%s%s_batch%d.fits", outdir.c_str(), outdir.empty() ? "" : "/", names[m],
               batch);
      if (srt_fits_write_map(fname, full.data(), nside, 0, "C", overwrite ? 1 : 0) != SRT_OK)
        errors[m] = last_error();
    });
  }
  for (auto& w : writers) w.join();
  for (int m = 0; m < 6; ++m)
    if (!errors[m].empty()) std::cerr << errors[m] << std::endl;
  const double t_end = now_ms();
  std::cout << "All done!" << std::endl;
  if (timing) {
    printf("{\"load_phi_ms\": %.3f, \"load_b_ms\": %.3f, \"upload_ms\": %.3f, \"trace_ms\": %.3f, "
           "\"trace_kernel_ms\": %.3f, \"write_ms\": %.3f, \"total_ms\": %.3f, \"rays\": %lld, \"ray_steps\": %lld}\n",
           t_phi - t_start, t_b - t_phi, t_up - t_b, t_trace - t_up, st.trace_ms, t_end - t_trace, t_end - t_start,
           (long long)st.rays, (long long)st.ray_steps);
  }
  return 0;
}
