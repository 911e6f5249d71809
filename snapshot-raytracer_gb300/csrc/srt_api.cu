// srt_api.cu — the C ABI of libsrt (declared in include/srt.h): field upload
// and layout, the forward trace, HEALPix helpers and error reporting.
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <thread>
#include "srt_internal.h"

namespace {
thread_local std::string g_last_error;

// Device memory of the fields (and of their upload slabs): a stream-ordered
// pool per device that keeps what is handed back (release threshold:
// unlimited), so that creating fields of the same size again reuses the
// mapped memory instead of paying the driver's mapping cost (~0.3 s for the
// 52 GB of a 1024^3 handle). A failed allocation trims the pool and retries
// once; srt_release_cached_memory() trims it on request.
constexpr int kMaxPoolDevices = 64;
std::mutex g_pool_mutex;
cudaMemPool_t g_pool[kMaxPoolDevices] = {};

cudaError_t device_pool(int dev, cudaMemPool_t* out) {
  if (dev < 0 || dev >= kMaxPoolDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_pool_mutex);
  if (!g_pool[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    cudaError_t e = cudaMemPoolCreate(&pool, &props);
    if (e != cudaSuccess) return e;
    uint64_t keep = ~0ull;
    e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    if (e != cudaSuccess) {
      cudaMemPoolDestroy(pool);
      return e;
    }
    g_pool[dev] = pool;
  }
  *out = g_pool[dev];
  return cudaSuccess;
}
}  // namespace

namespace srt {

// Failure injection (srt_debug_fail_alloc): device allocations still to
// succeed before one fails; negative when disarmed.
std::atomic<int64_t> g_alloc_fault_after{-1};

// True for the allocation the hook makes fail (which disarms it).
bool alloc_fault() {
  int64_t v = g_alloc_fault_after.load();
  while (v >= 0)
    if (g_alloc_fault_after.compare_exchange_weak(v, v - 1)) return v == 0;
  return false;
}

cudaError_t dev_alloc(void** p, size_t bytes) {
  if (alloc_fault()) return cudaErrorMemoryAllocation;
  return cudaMalloc(p, bytes ? bytes : 1);
}

cudaError_t dev_alloc_async(void** p, size_t bytes, cudaStream_t s) {
  if (alloc_fault()) return cudaErrorMemoryAllocation;
  return cudaMallocAsync(p, bytes ? bytes : 1, s);
}

cudaError_t pool_alloc(void** p, size_t bytes, cudaStream_t s) {
  if (alloc_fault()) return cudaErrorMemoryAllocation;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  cudaMemPool_t pool = nullptr;
  if (e == cudaSuccess) e = device_pool(dev, &pool);
  if (e != cudaSuccess) return e;
  e = cudaMallocFromPoolAsync(p, bytes ? bytes : 1, pool, s);
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    cudaStreamSynchronize(s);
    cudaMemPoolTrimTo(pool, 0);
    e = cudaMallocFromPoolAsync(p, bytes ? bytes : 1, pool, s);
  }
  return e;
}

void pool_free(void* p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

// Bytes the device's pool holds but does not use (reusable by pool_alloc).
int64_t pool_reusable_bytes(int dev) {
  cudaMemPool_t pool = nullptr;
  if (device_pool(dev, &pool) != cudaSuccess) return 0;
  uint64_t reserved = 0, used = 0;
  if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved) != cudaSuccess ||
      cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) != cudaSuccess)
    return 0;
  return reserved > used ? (int64_t)(reserved - used) : 0;
}

}  // namespace srt

namespace {

struct HostTimer {
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  double ms() const {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
};

// Largest slab of a host field staged on the device at a time.
constexpr int64_t kSlabBytes = 512ll << 20;


// Device address of host memory the GPU can read directly (pinned and mapped:
// cudaHostAlloc, or cudaHostRegister with mapping), or NULL.
const float* mapped_device_pointer(const float* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
  return (const float*)a.devicePointer;
}

bool dims_ok(int64_t n0, int64_t n1, int64_t n2) {
  const int64_t lim = int64_t(1) << 20;
  if (n0 < 1 || n1 < 1 || n2 < 1 || n0 > lim || n1 > lim || n2 > lim) return false;
  // positions and cell indices are kept in 32-bit integers / FP32 on the mixed path
  return true;
}
}  // namespace

namespace srt {

int set_error(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int cuda_error(cudaError_t e, const char* what) {
  if (e == cudaErrorMemoryAllocation)
    return set_error(SRT_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
    return set_error(SRT_ERR_NO_DEVICE, "%s: %s", what, cudaGetErrorString(e));
  return set_error(SRT_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

Geom make_geom(const srt_fields* f) {
  Geom g;
  for (int i = 0; i < 3; ++i) {
    g.n[i] = (int)f->n[i];
    g.invn[i] = 1.0f / (float)f->n[i];
  }
  g.px = f->pn[0];
  g.pxy = f->pn[0] * f->pn[1];
  g.pxy2 = f->pn[0] * (f->pn[1] - 1);
  return g;
}

FieldPtrs make_ptrs(const srt_fields* f) {
  FieldPtrs p;
  p.phi = f->phi;
  for (int c = 0; c < 3; ++c) {
    p.b[c] = f->b[c];
    p.bh[c] = f->bh[c];
  }
  for (int c = 0; c < 4; ++c) p.pr[c] = f->pr[c];
  return p;
}

}  // namespace srt

using namespace srt;

#define SRT_CUDA_TRY(expr, what)                 \
  do {                                           \
    cudaError_t _e = (expr);                     \
    if (_e != cudaSuccess) {                     \
      rc = cuda_error(_e, what);                 \
      goto fail;                                 \
    }                                            \
  } while (0)

extern "C" {

int srt_abi_version(void) { return SRT_ABI_VERSION; }

int srt_last_error(char* buf, size_t len) {
  if (buf && len > 0) {
    strncpy(buf, g_last_error.c_str(), len - 1);
    buf[len - 1] = '\0';
  }
  return (int)g_last_error.size();
}

int srt_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

}  // extern "C"

namespace {

// Row-pair arrays for the packed MIXED path, when they fit with room to spare
// (unless SRT_FIELDS_NO_PAIRS).
int build_row_pairs(srt_fields* f, unsigned flags, cudaStream_t s) {
  if (flags & SRT_FIELDS_NO_PAIRS) return SRT_OK;
  const int64_t pair_bytes = 4 * f->pn[0] * (f->pn[1] - 1) * f->pn[2] * (int64_t)sizeof(float2);
  size_t free_b = 0, total_b = 0;
  const bool have = cudaMemGetInfo(&free_b, &total_b) == cudaSuccess;
  const int64_t avail = (int64_t)free_b + pool_reusable_bytes(f->device);
  if (!have || pair_bytes + (int64_t(4) << 30) >= avail) return SRT_OK;
  const float* srcs[4] = {f->b[0], f->b[1], f->b[2], f->phi};
  cudaError_t e = cudaSuccess;
  for (int c = 0; c < 4 && e == cudaSuccess; ++c) {
    e = pool_alloc((void**)&f->pr[c], pair_bytes / 4, s);
    if (e != cudaSuccess) return cuda_error(e, "allocate row pairs");
    e = launch_pair_build(srcs[c], f->pr[c], f->pn, s);
  }
  if (e != cudaSuccess) return cuda_error(e, "row pairs");
  f->bytes += pair_bytes;
  if (!(flags & SRT_ASYNC)) {
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_error(e, "row pairs");
  }
  return SRT_OK;
}

// Device arrays of the laid-out fields of an n0 x n1 x n2 grid (no contents).
int alloc_fields(srt_fields* f, int64_t n0, int64_t n1, int64_t n2, cudaStream_t s) {
  cudaGetDevice(&f->device);
  for (int i = 0; i < 3; ++i) {
    f->n[i] = (i == 0 ? n0 : (i == 1 ? n1 : n2));
    f->pn[i] = f->n[i] + 3;
  }
  const int64_t pvox = f->pn[0] * f->pn[1] * f->pn[2];
  cudaError_t e = pool_alloc((void**)&f->phi, pvox * sizeof(float), s);
  if (e != cudaSuccess) return cuda_error(e, "allocate phi");
  for (int c = 0; c < 3; ++c) {
    e = pool_alloc((void**)&f->b[c], pvox * sizeof(float), s);
    if (e != cudaSuccess) return cuda_error(e, "allocate B");
  }
  f->bytes = 4 * pvox * (int64_t)sizeof(float);
  return SRT_OK;
}

}  // namespace

extern "C" {

int srt_fields_create(const float* phi, const float* b_xyz, int64_t n0, int64_t n1, int64_t n2,
                      unsigned flags, void* stream, srt_fields** out) {
  NvtxRange nvtx_("srt_fields_create");
  if (!out) return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_fields_create: out is NULL");
  *out = nullptr;
  if (!phi || !b_xyz) return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_fields_create: phi and b_xyz are required");
  if (!dims_ok(n0, n1, n2))
    return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_fields_create: bad grid extents %lld x %lld x %lld",
                     (long long)n0, (long long)n1, (long long)n2);
  if (srt_device_count() < 1) return set_error(SRT_ERR_NO_DEVICE, "srt_fields_create: no CUDA device");
  cudaStream_t s = (cudaStream_t)stream;
  const bool dev_in = (flags & SRT_INPUT_DEVICE) != 0;
  int rc = SRT_OK;
  float* slab = nullptr;
  srt_fields* f = new (std::nothrow) srt_fields();
  if (!f) return set_error(SRT_ERR_OUT_OF_MEMORY, "srt_fields_create: host allocation failed");
  {
    cudaGetDevice(&f->device);
    for (int i = 0; i < 3; ++i) {
      f->n[i] = (i == 0 ? n0 : (i == 1 ? n1 : n2));
      f->pn[i] = f->n[i] + 3;
    }
    const int64_t pvox = f->pn[0] * f->pn[1] * f->pn[2];
    const int64_t plane = n0 * n1;
    const int64_t vox = plane * n2;
    SRT_CUDA_TRY(pool_alloc((void**)&f->phi, pvox * sizeof(float), s), "allocate phi");
    for (int c = 0; c < 3; ++c) SRT_CUDA_TRY(pool_alloc((void**)&f->b[c], pvox * sizeof(float), s), "allocate B");
    f->bytes = 4 * pvox * (int64_t)sizeof(float);
    float* const phi_dst[3] = {f->phi, nullptr, nullptr};
    // host inputs in mapped pinned memory (cudaHostAlloc / cudaHostRegister)
    // are read by the layout kernel itself over the host link, with no
    // staging copy; other host memory streams through a device slab
    const float* phi_src = phi;
    const float* b_src = b_xyz;
    bool direct = dev_in;
    if (!dev_in && !(flags & SRT_FIELDS_STAGED)) {
      const float* dp = mapped_device_pointer(phi);
      const float* db = mapped_device_pointer(b_xyz);
      if (dp && db) {
        phi_src = dp;
        b_src = db;
        direct = true;
      }
    }
    if (direct) {
      NvtxRange upload(dev_in ? "layout" : "layout from mapped host memory");
      SRT_CUDA_TRY(launch_pad_fields(phi_src, 1, phi_dst, f->n, f->pn, 0, n2, s), "pad phi");
      SRT_CUDA_TRY(launch_pad_fields(b_src, 3, f->b, f->n, f->pn, 0, n2, s), "pad B");
    } else if ((flags & SRT_ASYNC) && pool_alloc((void**)&slab, 4 * vox * sizeof(float), s) == cudaSuccess) {
      // asynchronous: the whole input through one staging buffer, so the
      // copy engines move it without waiting for a layout kernel between
      // slabs (those would wait for SM slots while other work runs), then
      // one layout kernel per field
      NvtxRange upload("upload (one staging buffer) and layout");
      SRT_CUDA_TRY(cudaMemcpyAsync(slab, phi, vox * sizeof(float), cudaMemcpyHostToDevice, s), "copy phi");
      SRT_CUDA_TRY(cudaMemcpyAsync(slab + vox, b_xyz, 3 * vox * sizeof(float), cudaMemcpyHostToDevice, s), "copy B");
      SRT_CUDA_TRY(launch_pad_fields(slab, 1, phi_dst, f->n, f->pn, 0, n2, s), "pad phi");
      SRT_CUDA_TRY(launch_pad_fields(slab + vox, 3, f->b, f->n, f->pn, 0, n2, s), "pad B");
    } else {
      cudaGetLastError();  // a failed whole-input staging allocation falls back to slabs
      // Stream host planes through one device slab on s: H2D copy, then the
      // pad kernel. (A second slab with the copies on their own stream was
      // measured slower in steady use: 250-310 ms against 190-210 ms for the
      // 17 GB of a 1024^3 handle from pinned memory.)
      int64_t kslab = kSlabBytes / (plane * 3 * (int64_t)sizeof(float));
      if (kslab < 1) kslab = 1;
      if (kslab > n2) kslab = n2;
      SRT_CUDA_TRY(pool_alloc((void**)&slab, kslab * plane * 3 * sizeof(float), s), "allocate slab");
      // pass 0: phi (one component per voxel); pass 1: B (three, interleaved)
      NvtxRange upload("upload and layout");
      for (int pass = 0; pass < 2; ++pass) {
        const int comps = pass == 0 ? 1 : 3;
        const float* src = pass == 0 ? phi : b_xyz;
        for (int64_t k0 = 0; k0 < n2; k0 += kslab) {
          const int64_t k1 = k0 + kslab < n2 ? k0 + kslab : n2;
          SRT_CUDA_TRY(cudaMemcpyAsync(slab, src + comps * k0 * plane, comps * (k1 - k0) * plane * sizeof(float),
                                       cudaMemcpyHostToDevice, s),
                       "copy field slab");
          SRT_CUDA_TRY(launch_pad_fields(slab, comps, pass == 0 ? phi_dst : f->b, f->n, f->pn, k0, k1, s),
                       pass == 0 ? "pad phi" : "pad B");
        }
      }
    }
    if (!(flags & SRT_ASYNC)) SRT_CUDA_TRY(cudaStreamSynchronize(s), "field layout");
    pool_free(slab, s);  // stream-ordered: after the last pad kernel on s
    slab = nullptr;
    rc = build_row_pairs(f, flags, s);
    if (rc != SRT_OK) goto fail;
  }
  *out = f;
  return SRT_OK;
fail:
  cudaStreamSynchronize(s);
  pool_free(slab, s);
  srt_fields_destroy(f);
  return rc;
}

int srt_fields_destroy(srt_fields* f) {
  NvtxRange nvtx_("srt_fields_destroy");
  if (!f) return SRT_OK;
  int prev = 0;
  cudaGetDevice(&prev);
  if (prev != f->device) cudaSetDevice(f->device);
  // no kernel may still read the fields (cudaFree synchronised the device too)
  cudaDeviceSynchronize();
  pool_free(f->phi, 0);
  for (int c = 0; c < 3; ++c) {
    pool_free(f->b[c], 0);
    pool_free(f->bh[c], 0);
  }
  for (int c = 0; c < 4; ++c) pool_free(f->pr[c], 0);
  cudaDeviceSynchronize();
  if (prev != f->device) cudaSetDevice(prev);
  delete f;
  return SRT_OK;
}

int srt_release_cached_memory(void) {
  noalloc_forget_scratch();
  int n = 0;
  cudaGetDeviceCount(&n);
  int prev = 0;
  cudaGetDevice(&prev);
  for (int d = 0; d < n && d < kMaxPoolDevices; ++d) {
    cudaMemPool_t pool = nullptr;
    {
      std::lock_guard<std::mutex> lock(g_pool_mutex);
      pool = g_pool[d];
    }
    if (!pool) continue;
    cudaSetDevice(d);
    cudaDeviceSynchronize();
    cudaMemPoolTrimTo(pool, 0);
  }
  cudaSetDevice(prev);
  return SRT_OK;
}

int64_t srt_fields_bytes(const srt_fields* f) { return f ? f->bytes : 0; }

int srt_forward(const srt_fields* fields, int64_t nside, int64_t pix_begin, int64_t pix_count, int n_steps,
                int precision, float* const maps[SRT_NUM_MAPS], unsigned flags, void* stream,
                srt_stats* stats) {
  NvtxRange nvtx_("srt_forward");
  HostTimer wall;
  if (!fields) return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_forward: fields is NULL");
  if (nside < 1 || nside > (int64_t(1) << 16))
    return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_forward: invalid nside %lld", (long long)nside);
  const int64_t npix = 12 * nside * nside;
  if (pix_begin < 0 || pix_count < 0 || pix_begin > npix || pix_count > npix - pix_begin)
    return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_forward: pixel range [%lld, %lld) outside [0, %lld)",
                     (long long)pix_begin, (long long)(pix_begin + pix_count), (long long)npix);
  const bool nested = (flags & SRT_NESTED_RANGE) != 0;
  if (nested && (nside & (nside - 1)) != 0)
    return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_forward: NESTED pixel ranges need a power-of-two nside, got %lld",
                     (long long)nside);
  if (n_steps < 1 || n_steps > (1 << 22))
    return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_forward: invalid n_steps %d", n_steps);
  if (precision != SRT_PRECISION_FP64 && precision != SRT_PRECISION_MIXED && precision != SRT_PRECISION_REF16)
    return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_forward: unknown precision %d", precision);
  if (!maps) return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_forward: maps is NULL");
  for (int m = 0; m < SRT_NUM_MAPS; ++m)
    if (!maps[m] && pix_count > 0) return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_forward: maps[%d] is NULL", m);
  if (stats) memset(stats, 0, sizeof(*stats));
  if (pix_count == 0) return SRT_OK;

  srt_fields* f = const_cast<srt_fields*>(fields);
  cudaStream_t s = (cudaStream_t)stream;
  const bool dev_out = (flags & SRT_OUTPUT_DEVICE) != 0;
  int rc = SRT_OK;
  float* dmaps = nullptr;
  int64_t* refine_list = nullptr;
  unsigned long long* refine_count = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr, em = nullptr;
  int64_t kernels = 0;
  int prev = 0;
  cudaGetDevice(&prev);
  if (prev != f->device) cudaSetDevice(f->device);
  {
    if (precision == SRT_PRECISION_REF16 && !(f->bh[0] && f->bh[1] && f->bh[2])) {
      // half(B * 2^27) planes for the reference arithmetic, made once per handle
      const int64_t pvox = f->pn[0] * f->pn[1] * f->pn[2];
      __half* h[3] = {nullptr, nullptr, nullptr};
      cudaError_t e = cudaSuccess;
      for (int c = 0; c < 3 && e == cudaSuccess; ++c) e = pool_alloc((void**)&h[c], pvox * sizeof(__half), s);
      for (int c = 0; c < 3 && e == cudaSuccess; ++c) {
        e = launch_quantize_half(f->b[c], h[c], pvox, s);
        ++kernels;
      }
      if (e != cudaSuccess) {
        for (int c = 0; c < 3; ++c) pool_free(h[c], s);
        rc = cuda_error(e, "REF16 B planes");
        goto fail;
      }
      for (int c = 0; c < 3; ++c) f->bh[c] = h[c];
      f->bytes += 3 * pvox * (int64_t)sizeof(__half);
    }
    TraceArgs a;
    a.F = make_ptrs(f);
    a.G = make_geom(f);
    a.nside = nside;
    int l = 0;
    while ((int64_t(1) << l) < nside) ++l;
    a.log2p = l;
    a.launch_rays = nested ? pix_count : 12 * (int64_t(1) << (2 * l));
    a.pix_begin = pix_begin;
    a.pix_count = pix_count;
    a.nested = nested;
    a.n_steps = n_steps;
    a.refine_list = nullptr;
    a.refine_count = nullptr;
    const bool refine = precision == SRT_PRECISION_MIXED && !(flags & SRT_MIXED_NO_REFINE);
    if (refine) {
      SRT_CUDA_TRY(dev_alloc_async((void**)&refine_list, pix_count * sizeof(int64_t), s), "cudaMallocAsync(refine list)");
      SRT_CUDA_TRY(dev_alloc_async((void**)&refine_count, sizeof(unsigned long long), s), "cudaMallocAsync(refine count)");
      SRT_CUDA_TRY(cudaMemsetAsync(refine_count, 0, sizeof(unsigned long long), s), "clear refine count");
      a.refine_list = refine_list;
      a.refine_count = refine_count;
    }
    if (dev_out) {
      for (int m = 0; m < 6; ++m) a.maps[m] = maps[m];
    } else {
      // stream-ordered: a plain device allocation issued here would keep this
      // trace from running beside work already queued on other streams
      SRT_CUDA_TRY(dev_alloc_async((void**)&dmaps, 6 * pix_count * sizeof(float), s), "cudaMallocAsync(maps)");
      for (int m = 0; m < 6; ++m) a.maps[m] = dmaps + m * pix_count;
    }
    const bool timed = !(flags & SRT_ASYNC);
    if (timed) {
      SRT_CUDA_TRY(cudaEventCreate(&e0), "cudaEventCreate");
      SRT_CUDA_TRY(cudaEventCreate(&e1), "cudaEventCreate");
      SRT_CUDA_TRY(cudaEventCreate(&em), "cudaEventCreate");
      SRT_CUDA_TRY(cudaEventRecord(e0, s), "cudaEventRecord");
    }
    const int kmode = (precision == SRT_PRECISION_MIXED && f->pr[0]) ? kMIXED_PAIR : precision;
    SRT_CUDA_TRY(launch_trace(kmode, a, s, &kernels), "trace kernel launch");
    if (timed) SRT_CUDA_TRY(cudaEventRecord(em, s), "cudaEventRecord");  // trace kernel done
    if (refine) SRT_CUDA_TRY(launch_refine(a, s, &kernels), "refine kernel launch");
    if (timed) SRT_CUDA_TRY(cudaEventRecord(e1, s), "cudaEventRecord");
    if (!dev_out) {
      for (int m = 0; m < 6; ++m)
        SRT_CUDA_TRY(cudaMemcpyAsync(maps[m], a.maps[m], pix_count * sizeof(float), cudaMemcpyDeviceToHost, s),
                     "copy maps to host");
    }
    if (timed || !dev_out) SRT_CUDA_TRY(cudaStreamSynchronize(s), "trace");
    if (stats) {
      float ms = -1.f, rms = 0.f;
      if (timed) {
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventElapsedTime(&rms, em, e1);
      }
      stats->trace_ms = ms;
      stats->retrace_ms = refine ? rms : 0.0;
      stats->rays = pix_count;
      stats->ray_steps = pix_count * (int64_t)n_steps;
      stats->kernels = kernels;
      stats->d2h_bytes = dev_out ? 0 : 6 * pix_count * (int64_t)sizeof(float);
      if (refine && timed) {
        unsigned long long cnt = 0;
        if (cudaMemcpy(&cnt, refine_count, sizeof(cnt), cudaMemcpyDeviceToHost) == cudaSuccess)
          stats->refined_rays = (int64_t)cnt;
      }
    }
  }
fail:
  if (dmaps) cudaFreeAsync(dmaps, s);
  // stream-ordered release: the refine kernel may still be queued (SRT_ASYNC)
  if (refine_list) cudaFreeAsync(refine_list, s);
  if (refine_count) cudaFreeAsync(refine_count, s);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (em) cudaEventDestroy(em);
  if (prev != f->device) cudaSetDevice(prev);
  if (stats) stats->total_ms = wall.ms();
  return rc;
}

int srt_fields_load_h5(const char* phi_path, const char* b_path, const char* dset, unsigned flags, double phi_scale,
                       double b_scale, srt_load_progress progress, void* ctx, srt_fields** out,
                       srt_load_stats* stats) {
  NvtxRange nvtx_("srt_fields_load_h5");
  const auto t_start = std::chrono::steady_clock::now();
  auto ms_since = [&](std::chrono::steady_clock::time_point t) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t).count();
  };
  if (!out) return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_fields_load_h5: out is NULL");
  *out = nullptr;
  if (!phi_path || !b_path || !dset) return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_fields_load_h5: NULL path");
  if (stats) memset(stats, 0, sizeof(*stats));
  // ---- phi's header (the extents); file errors come before device errors,
  // as in the reference, which reads its files before touching the device
  H5Field* hphi = nullptr;
  int64_t pd[8] = {0};
  int prank = 0;
  int rc = h5_field_open(phi_path, dset, false, pd, &prank, &hphi);
  if (rc != SRT_OK) return rc;
  if (prank < 3) {
    h5_field_close(hphi);
    return set_error(SRT_ERR_FORMAT, "Expected a 3D potential dataset, got rank=%d", prank);
  }
  // grid extents, fastest first: the reference takes the HDF5 extents in file
  // order (snapshot-raytracer.cu:645), SRT_LOAD_XYZ_HDF5 the fastest axis first
  const bool hdf5_order = (flags & SRT_LOAD_XYZ_HDF5) != 0;
  const int64_t n0 = hdf5_order ? pd[2] : pd[0], n1 = pd[1], n2 = hdf5_order ? pd[0] : pd[2];
  if (!dims_ok(n0, n1, n2)) {
    h5_field_close(hphi);
    return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_fields_load_h5: bad grid extents %lld x %lld x %lld",
                     (long long)n0, (long long)n1, (long long)n2);
  }
  // without a device both files are still read (and checked) before the
  // device error, in the reference's order
  const bool have_device = srt_device_count() > 0;
  bool cancelled = progress && progress(SRT_LOAD_PHI_DIMS, pd, ctx) != 0;
  if (cancelled) {
    h5_field_close(hphi);
    return set_error(SRT_ERR_CANCELLED, "srt_fields_load_h5: stopped by the progress callback");
  }
  const int64_t plane = n0 * n1, vox = plane * n2;
  int64_t phi_count = 1;  // every element of phi is read (the first vox are traced)
  for (int d = 0; d < prank; ++d) phi_count *= pd[d];
  float* hphi_data = (float*)malloc((size_t)phi_count * sizeof(float));
  float* hb_data = (float*)malloc((size_t)(3 * vox) * sizeof(float));
  if (!hphi_data || !hb_data) {
    free(hphi_data);
    free(hb_data);
    h5_field_close(hphi);
    return set_error(SRT_ERR_OUT_OF_MEMORY, "srt_fields_load_h5: cannot allocate host memory for the fields");
  }
  // ---- the reader thread: phi, then B; progress published under a mutex
  struct Shared {
    std::mutex m;
    std::condition_variable cv;
    int64_t ready[2] = {0, 0};  // floats of phi / B in their final host values
    int stage = 0;              // 0 reading phi, 1 phi read, 2 B header read, 3 done
    int rc = SRT_OK;
    std::string err;
    int64_t bd[8] = {0};
    double read_ms[2] = {0, 0};
    bool stop = false;  // set by this thread when it gives up: the reader stops
  } sh;
  auto publish = [&](int field, int64_t n) {
    std::lock_guard<std::mutex> lk(sh.m);
    sh.ready[field] = n;
    sh.cv.notify_all();
    return !sh.stop;
  };
  std::thread reader([&, hphi]() {
    char buf[1024];
    auto t0 = std::chrono::steady_clock::now();
    int r = h5_field_read(hphi, hphi_data, phi_scale, [&](int64_t n) { return publish(0, n); });
    h5_field_close(hphi);
    auto fail_with = [&](int code) {
      srt_last_error(buf, sizeof(buf));
      std::lock_guard<std::mutex> lk(sh.m);
      sh.rc = code;
      sh.err = buf;
      sh.stage = 3;
      sh.cv.notify_all();
    };
    if (r != SRT_OK) return fail_with(r);
    {
      std::lock_guard<std::mutex> lk(sh.m);
      sh.read_ms[0] = ms_since(t0);
      sh.stage = 1;
      sh.cv.notify_all();
    }
    H5Field* hb = nullptr;
    int64_t bd[8] = {0};
    int brank = 0;
    {
      std::lock_guard<std::mutex> lk(sh.m);
      if (sh.stop) return;
    }
    r = h5_field_open(b_path, dset, true, bd, &brank, &hb);
    if (r == SRT_OK && (bd[0] != pd[0] || bd[1] != pd[1] || bd[2] != pd[2]))
      r = set_error(SRT_ERR_FORMAT, "B field dimensions %lld x %lld x %lld differ from the potential's",
                    (long long)bd[0], (long long)bd[1], (long long)bd[2]);
    if (r != SRT_OK) {
      if (hb) h5_field_close(hb);
      return fail_with(r);
    }
    {
      std::lock_guard<std::mutex> lk(sh.m);
      for (int i = 0; i < 3; ++i) sh.bd[i] = bd[i];
      sh.stage = 2;
      sh.cv.notify_all();
    }
    t0 = std::chrono::steady_clock::now();
    r = h5_field_read(hb, hb_data, b_scale, [&](int64_t n) { return publish(1, n); });
    h5_field_close(hb);
    std::lock_guard<std::mutex> lk(sh.m);
    sh.read_ms[1] = ms_since(t0);
    if (r != SRT_OK) {
      srt_last_error(buf, sizeof(buf));
      sh.rc = r;
      sh.err = buf;
    }
    sh.stage = 3;
    sh.cv.notify_all();
  });
  // ---- this thread: lay out each run of planes as soon as it has been read
  cudaStream_t s = nullptr;
  srt_fields* f = new (std::nothrow) srt_fields();
  float* slab = nullptr;
  double layout_ms = 0.0, tail_ms = 0.0;
  bool announced_b = false, announced_bdims = false, announced_upload = false;
  rc = f ? SRT_OK : set_error(SRT_ERR_OUT_OF_MEMORY, "srt_fields_load_h5: host allocation failed");
  if (rc == SRT_OK && have_device) rc = alloc_fields(f, n0, n1, n2, s);
  int64_t kslab = kSlabBytes / (plane * 3 * (int64_t)sizeof(float));
  if (kslab < 1) kslab = 1;
  if (kslab > n2) kslab = n2;
  if (rc == SRT_OK && have_device) {
    cudaError_t e = pool_alloc((void**)&slab, kslab * plane * 3 * sizeof(float), s);
    if (e != cudaSuccess) rc = cuda_error(e, "allocate slab");
  }
  auto announce = [&](int event, const int64_t* d) {
    if (progress && !cancelled && progress(event, d, ctx) != 0) cancelled = true;
  };
  std::chrono::steady_clock::time_point t_read_end;
  for (int field = 0; field < 2 && rc == SRT_OK; ++field) {
    const int comps = field == 0 ? 1 : 3;
    const float* host = field == 0 ? hphi_data : hb_data;
    float* const phi_dst[3] = {f->phi, nullptr, nullptr};
    for (int64_t k0 = 0; k0 < n2 && rc == SRT_OK; k0 += kslab) {
      const int64_t k1 = k0 + kslab < n2 ? k0 + kslab : n2;
      const int64_t need = k1 * plane * comps;
      {
        std::unique_lock<std::mutex> lk(sh.m);
        while (true) {
          // the steps the reference prints, in its order, as they happen
          if (!announced_b && sh.stage >= 1 && sh.read_ms[0] > 0.0) {
            announced_b = true;
            lk.unlock();
            announce(SRT_LOAD_B_START, pd);
            lk.lock();
            continue;
          }
          if (!announced_bdims && sh.stage >= 2 && sh.rc == SRT_OK) {
            announced_bdims = true;
            int64_t bd[3] = {sh.bd[0], sh.bd[1], sh.bd[2]};
            lk.unlock();
            announce(SRT_LOAD_B_DIMS, bd);
            lk.lock();
            continue;
          }
          if (sh.rc != SRT_OK || cancelled) break;
          if (sh.ready[field] >= need) break;
          sh.cv.wait(lk);
        }
        if (sh.rc != SRT_OK) {
          rc = set_error(sh.rc, "%s", sh.err.c_str());
          break;
        }
        if (cancelled) {
          rc = set_error(SRT_ERR_CANCELLED, "srt_fields_load_h5: stopped by the progress callback");
          break;
        }
        if (sh.stage == 3 && announced_bdims && !announced_upload) {
          announced_upload = true;
          t_read_end = std::chrono::steady_clock::now();
          lk.unlock();
          announce(SRT_LOAD_UPLOAD, sh.bd);
          lk.lock();
        }
      }
      if (cancelled) {
        rc = set_error(SRT_ERR_CANCELLED, "srt_fields_load_h5: stopped by the progress callback");
        break;
      }
      if (!have_device) continue;  // read and checked only
      const auto tl = std::chrono::steady_clock::now();
      cudaError_t e = cudaMemcpyAsync(slab, host + k0 * plane * comps, (k1 - k0) * plane * comps * sizeof(float),
                                      cudaMemcpyHostToDevice, s);
      if (e == cudaSuccess) e = launch_pad_fields(slab, comps, field == 0 ? phi_dst : f->b, f->n, f->pn, k0, k1, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) rc = cuda_error(e, "srt_fields_load_h5: layout");
      layout_ms += ms_since(tl);
    }
  }
  if (rc != SRT_OK) {  // let the reader stop at its next progress call
    std::lock_guard<std::mutex> lk(sh.m);
    sh.stop = true;
  }
  reader.join();
  if (rc == SRT_OK && sh.rc != SRT_OK) rc = set_error(sh.rc, "%s", sh.err.c_str());
  if (rc == SRT_OK && !announced_upload) {
    t_read_end = std::chrono::steady_clock::now();
    announce(SRT_LOAD_UPLOAD, sh.bd);
    if (cancelled) rc = set_error(SRT_ERR_CANCELLED, "srt_fields_load_h5: stopped by the progress callback");
  }
  if (rc == SRT_OK && !have_device) rc = set_error(SRT_ERR_NO_DEVICE, "srt_fields_load_h5: no CUDA device");
  free(hphi_data);
  free(hb_data);
  if (slab) pool_free(slab, s);
  if (rc == SRT_OK) {
    const auto tt = std::chrono::steady_clock::now();
    rc = build_row_pairs(f, flags & SRT_FIELDS_NO_PAIRS, s);
    if (rc == SRT_OK) {
      cudaError_t e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) rc = cuda_error(e, "srt_fields_load_h5");
    }
    tail_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_read_end).count();
    (void)tt;
  }
  if (rc != SRT_OK) {
    cudaStreamSynchronize(s);
    srt_fields_destroy(f);
    return rc;
  }
  if (stats) {
    stats->read_phi_ms = sh.read_ms[0];
    stats->read_b_ms = sh.read_ms[1];
    stats->layout_ms = layout_ms;
    stats->after_read_ms = tail_ms;
    stats->total_ms = ms_since(t_start);
    stats->h2d_bytes = 4 * vox * (int64_t)sizeof(float);
    for (int i = 0; i < 3; ++i) stats->n[i] = f->n[i];
  }
  *out = f;
  return SRT_OK;
}

int srt_pix2ang_ring(int64_t nside, int64_t pix, double* theta, double* phi) {
  if (nside < 1 || nside > (int64_t(1) << 29) || pix < 0 || pix >= 12 * nside * nside || !theta || !phi)
    return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_pix2ang_ring: bad arguments");
  hp_pix2ang_ring(nside, pix, theta, phi);
  return SRT_OK;
}

int64_t srt_nest2ring(int64_t nside, int64_t ipnest) {
  if (!hp_is_pow2(nside) || nside > (int64_t(1) << 29) || ipnest < 0 || ipnest >= 12 * nside * nside) return -1;
  return hp_nest2ring(nside, ipnest);
}

int64_t srt_ring2nest(int64_t nside, int64_t ipring) {
  if (!hp_is_pow2(nside) || nside > (int64_t(1) << 29) || ipring < 0 || ipring >= 12 * nside * nside) return -1;
  return hp_ring2nest(nside, ipring);
}

int srt_debug_fail_alloc(int64_t after) {
  g_alloc_fault_after.store(after < 0 ? -1 : after);
  return SRT_OK;
}

int srt_probe_peak(int kind, double* flops_per_s) {
  if (!flops_per_s || kind < 0 || kind > 2) return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_probe_peak: bad arguments");
  if (srt_device_count() < 1) return set_error(SRT_ERR_NO_DEVICE, "srt_probe_peak: no CUDA device");
  cudaError_t e = probe_fma(kind, flops_per_s);
  if (e != cudaSuccess) return cuda_error(e, "srt_probe_peak");
  return SRT_OK;
}

void srt_free(void* p) { free(p); }

}  // extern "C"
