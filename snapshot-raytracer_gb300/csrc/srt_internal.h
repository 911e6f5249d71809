// srt_internal.h — shared declarations between the libsrt translation units.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include <functional>
#include <string>
#include <nvtx3/nvToolsExt.h>
#include "srt.h"
#include "srt_scheme.cuh"

// Device memory of one set of laid-out fields (see srt_fields_create).
struct srt_fields {
  int device = 0;
  int64_t n[3] = {0, 0, 0};
  int64_t pn[3] = {0, 0, 0};  // padded extents n + 3
  float* phi = nullptr;       // padded FP32 planes
  float* b[3] = {nullptr, nullptr, nullptr};
  __half* bh[3] = {nullptr, nullptr, nullptr};  // padded half(B * 2^27), made on first REF16 use
  float2* pr[4] = {nullptr, nullptr, nullptr, nullptr};  // row-pair arrays B_x, B_y, B_z, phi (MIXED fast path)
  int64_t bytes = 0;
};

namespace srt {

// Device memory of fields: a per-device stream-ordered pool that keeps freed
// memory for reuse (srt_release_cached_memory trims it).
cudaError_t pool_alloc(void** p, size_t bytes, cudaStream_t s);
void pool_free(void* p, cudaStream_t s);
int64_t pool_reusable_bytes(int dev);
// cudaMalloc / cudaMallocAsync behind the failure-injection hook
// (srt_debug_fail_alloc); pool_alloc checks the hook too.
cudaError_t dev_alloc(void** p, size_t bytes);
cudaError_t dev_alloc_async(void** p, size_t bytes, cudaStream_t s);

// NVTX range over a scope (the public entry points and their phases), for
// profilers' timelines and range filters; header-only, inert unless a tool
// is attached.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// Error reporting (thread-local last error message).
int set_error(int code, const char* fmt, ...);
int cuda_error(cudaError_t e, const char* what);

struct TraceArgs {
  FieldPtrs F;
  Geom G;
  int64_t nside = 0;
  int log2p = 0;            // launch order: Morton over a 2^log2p square per face
  int64_t launch_rays = 0;  // launch slots: 12 * 4^log2p (RING ranges) or pix_count (NESTED)
  int64_t pix_begin = 0, pix_count = 0;
  bool nested = false;      // [pix_begin, pix_begin + pix_count) is a NESTED range
  int n_steps = 0;
  float* maps[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  // MIXED: the output slots of rays that came within the cell-face guard are
  // appended here (NULL: no fallback) and re-traced in FP64 by launch_refine.
  int64_t* refine_list = nullptr;
  unsigned long long* refine_count = nullptr;
};

Geom make_geom(const srt_fields* f);
FieldPtrs make_ptrs(const srt_fields* f);

// Field layout kernels.
// src: planes k0 .. k1-1 of phi (comps 1, dst[0]) or of the interleaved B
// (comps 3, dst[0..2]); device memory or mapped pinned host memory.
cudaError_t launch_pad_fields(const float* src, int comps, float* const dst[3], const int64_t n[3],
                              const int64_t pn[3], int64_t k0, int64_t k1, cudaStream_t s);
cudaError_t launch_quantize_half(const float* src, __half* dst, int64_t count, cudaStream_t s);
cudaError_t launch_pair_build(const float* src, float2* dst, const int64_t pn[3], cudaStream_t s);

// Trace kernel launch (mode = kFP64 / kMIXED / kREF16).
cudaError_t launch_trace(int mode, const TraceArgs& a, cudaStream_t s, int64_t* kernels);
// FP64 re-trace of the rays listed by a MIXED trace (count read on the device).
cudaError_t launch_refine(const TraceArgs& a, cudaStream_t s, int64_t* kernels);

// Progressive reads of an HDF5 field (srt_io.cpp), for srt_fields_load_h5.
// h5_field_open reads the header and checks the dataset as
// srt_h5_read_scalar (vector3 false) or srt_h5_read_vector3 (true) do;
// h5_field_read fills `out` (all elements as floats, times `scale`) in order
// along the slowest axis and calls ready(n) once the first n floats are final;
// ready returning false stops the read (the call then returns
// SRT_ERR_CANCELLED).
struct H5Field;
int h5_field_open(const char* path, const char* dset, bool vector3, int64_t dims[8], int* rank, H5Field** out);
int h5_field_read(H5Field* h, float* out, double scale, const std::function<bool(int64_t)>& ready);
void h5_field_close(H5Field* h);

// Forgets srt_forward_noalloc's cached scratch addresses (srt_noalloc.cu).
void noalloc_forget_scratch();

// Peak issue-rate probes (FMA loop kernels); returns achieved FLOP/s.
cudaError_t probe_fma(int kind, double* flops_per_s);

}  // namespace srt
