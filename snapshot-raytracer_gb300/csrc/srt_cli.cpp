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

  // Both files are read by the library's reader thread while every finished
  // run of planes is laid out on the device (the reference reads both files,
  // then copies: snapshot-raytracer.cu:640, :676, :752-855); the progress
  // callback prints the reference's lines in the reference's order.
  // batch checks once both files are read, where the reference makes them
  // (snapshot-raytracer.cu:708-717)
  const int64_t npix = 12 * nside * nside;
  int64_t istart = 0, count = npix;
  if (batch >= 0) {
    istart = (int64_t)batch * nside * nside;
    count = nside * nside;
  }
  const bool nested = base_pixel && batch >= 0;
  struct Ctx {
    const char* b_path;
    bool rescale_phi, rescale_b;
    double phi_factor, b_factor;
    bool batch_past_end, bad_nested;
    int64_t nside;
  } ctx{pos[1], rescale_phi, rescale_b, phi_factor, b_factor, istart >= npix,
        nested && (nside & (nside - 1)) != 0, nside};
  auto on_progress = [](int event, const int64_t* d, void* vp) -> int {
    Ctx* c = (Ctx*)vp;
    if (event == SRT_LOAD_PHI_DIMS) {
      std::cout << "Data dimensions: " << d[0] << " x " << d[1] << " x " << d[2] << std::endl;
      if (c->rescale_phi) std::cout << "Rescaling potential data by factor " << c->phi_factor << std::endl;
    } else if (event == SRT_LOAD_B_START) {
      std::cout << "Loading B field data from HDF5 file " << c->b_path << " ..." << std::endl;
    } else if (event == SRT_LOAD_B_DIMS) {
      // the reference's size warning for a large B (snapshot-raytracer.cu:159-161)
      const double b_bytes = 3.0 * (double)d[0] * (double)d[1] * (double)d[2] * sizeof(float);
      if (b_bytes > 8.0 * 1024 * 1024 * 1024)
        std::cerr << "Warning: allocating ~" << b_bytes / (1024.0 * 1024 * 1024) << " GiB for vector field."
                  << std::endl;
      if (c->rescale_b) std::cout << "Rescaling B field data by factor " << c->b_factor << std::endl;
    } else if (event == SRT_LOAD_UPLOAD) {
      if (c->batch_past_end) {
        std::cerr << "Batch exceeds total number of pixels" << std::endl;
        return 1;
      }
      if (c->bad_nested) {
        std::cerr << "--base-pixel needs a power-of-two Nside, got " << c->nside << std::endl;
        return 1;
      }
      std::cout << "Allocating device memory and copying data to device..." << std::endl;
    }
    return 0;
  };
  srt_fields* fields = nullptr;
  srt_load_stats ls;
  const unsigned lflags = hdf5_order ? SRT_LOAD_XYZ_HDF5 : 0u;
  const int lrc = srt_fields_load_h5(pos[0], pos[1], "/data", lflags, rescale_phi ? phi_factor : 1.0,
                                     rescale_b ? b_factor : 1.0, on_progress, &ctx, &fields, &ls);
  if (lrc != SRT_OK) {
    if (lrc != SRT_ERR_CANCELLED) std::cerr << last_error() << std::endl;  // else the callback said why
    return -1;
  }
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
    // read_*: the reader thread; layout_ms: copies and layout, overlapped with
    // the reads; after_read_ms: from the end of the reads to the fields being
    // ready (what the upload adds to the reads); trace_kernel_ms: the trace
    // and re-trace launches (device time), retrace_ms the re-trace's share
    printf("{\"read_phi_ms\": %.3f, \"read_b_ms\": %.3f, \"layout_ms\": %.3f, \"after_read_ms\": %.3f, "
           "\"load_ms\": %.3f, \"trace_ms\": %.3f, \"trace_kernel_ms\": %.3f, \"retrace_ms\": %.3f, "
           "\"write_ms\": %.3f, \"total_ms\": %.3f, \"rays\": %lld, \"ray_steps\": %lld}\n",
           ls.read_phi_ms, ls.read_b_ms, ls.layout_ms, ls.after_read_ms, t_up - t_start, t_trace - t_up, st.trace_ms,
           st.retrace_ms, t_end - t_trace, t_end - t_start, (long long)st.rays, (long long)st.ray_steps);
  }
  return 0;
}
