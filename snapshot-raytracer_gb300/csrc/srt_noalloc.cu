// srt_noalloc.cu — srt_forward_noalloc: the forward trace for callers that
// cannot allocate device memory when they trace.
//
// srt_forward allocates per call: the list of rays the MIXED trace re-traces
// in FP64 (and, for host outputs, device map buffers). Some callers cannot do
// that: applications whose device memory is reserved up front by their own
// pool (a fresh cudaMalloc fails once the pool holds the card), and loops that
// cannot take the device-wide synchronisation a cudaMalloc / cudaFree pair may
// imply. This entry point gives them the same trace with the scratch in a
// file-scope device array instead:
//   * kNoAllocMaxRays = 2^20 entries of ray indices (8 MiB) plus one counter,
//     held by every GPU that loads the library until the process exits;
//   * one call traces at most kNoAllocMaxRays rays; larger ranges are rejected;
//   * the caller passes the fields handle (made earlier, where allocating is
//     allowed) and device map buffers; nothing here calls cudaMalloc,
//     cudaMallocAsync, cudaFree or an allocating library routine;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress, with that device current) and caches it; make
//     that first call before any stream capture;
//   * every call shares the array: the counter is cleared on the stream at the
//     start of each call, and calls whose work overlaps on the GPU race for it;
//   * the cached address belongs to the device's primary context: after
//     cudaDeviceReset (or anything else that tears that context down) call
//     srt_release_cached_memory, which forgets it, before the next call;
//   * flags: SRT_ASYNC, SRT_NESTED_RANGE and SRT_MIXED_NO_REFINE act as in
//     srt_forward (SRT_OUTPUT_DEVICE is implied and accepted); any other flag
//     is refused with SRT_ERR_UNSUPPORTED rather than ignored.
#include <mutex>
#include "srt_internal.h"

namespace {

constexpr int64_t kNoAllocMaxRays = int64_t(1) << 20;
constexpr int kMaxDevices = 64;

// The scratch of every call on a device (see above).
static __device__ __align__(256) int64_t g_refine_list[kNoAllocMaxRays];
static __device__ __align__(256) unsigned long long g_refine_count;

struct DeviceScratch {
  int64_t* list = nullptr;
  unsigned long long* count = nullptr;
};
DeviceScratch g_scratch[kMaxDevices];
std::mutex g_scratch_mutex;

// Device addresses of the scratch on `dev` (the current device), looked up once.
int scratch_for(int dev, DeviceScratch* out) {
  if (dev < 0 || dev >= kMaxDevices)
    return srt::set_error(SRT_ERR_UNSUPPORTED, "srt_forward_noalloc: device ordinal %d beyond %d", dev, kMaxDevices);
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  DeviceScratch& s = g_scratch[dev];
  if (!s.list) {
    void* list = nullptr;
    void* count = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&list, g_refine_list);
    if (e != cudaSuccess) return srt::cuda_error(e, "srt_forward_noalloc: cudaGetSymbolAddress(ray list)");
    e = cudaGetSymbolAddress(&count, g_refine_count);
    if (e != cudaSuccess) return srt::cuda_error(e, "srt_forward_noalloc: cudaGetSymbolAddress(counter)");
    s.list = (int64_t*)list;
    s.count = (unsigned long long*)count;
  }
  *out = s;
  return SRT_OK;
}

}  // namespace

namespace srt {
// Forgets the cached scratch addresses (srt_release_cached_memory calls this,
// so that a context torn down and made again gets its addresses looked up anew).
void noalloc_forget_scratch() {
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  for (int d = 0; d < kMaxDevices; ++d) g_scratch[d] = DeviceScratch();
}
}  // namespace srt

extern "C" int srt_forward_noalloc(const srt_fields* fields, int64_t nside, int64_t pix_begin, int64_t pix_count,
                                   int n_steps, int precision, float* const maps[SRT_NUM_MAPS], unsigned flags,
                                   void* stream) {
  using namespace srt;
  if (!fields) return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_forward_noalloc: fields is NULL");
  if (nside < 1 || nside > (int64_t(1) << 16))
    return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_forward_noalloc: invalid nside %lld", (long long)nside);
  const int64_t npix = 12 * nside * nside;
  if (pix_begin < 0 || pix_count < 0 || pix_begin > npix || pix_count > npix - pix_begin)
    return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_forward_noalloc: pixel range outside [0, %lld)", (long long)npix);
  if (pix_count > kNoAllocMaxRays)
    return set_error(SRT_ERR_INVALID_ARGUMENT,
                     "srt_forward_noalloc: %lld rays requested, at most %lld per call (trace larger ranges in parts "
                     "or with srt_forward)",
                     (long long)pix_count, (long long)kNoAllocMaxRays);
  const unsigned known = SRT_ASYNC | SRT_NESTED_RANGE | SRT_MIXED_NO_REFINE | SRT_OUTPUT_DEVICE;
  if (flags & ~known)
    return set_error(SRT_ERR_UNSUPPORTED, "srt_forward_noalloc: flags 0x%x not supported (SRT_ASYNC, SRT_NESTED_RANGE, "
                     "SRT_MIXED_NO_REFINE; maps are always device buffers)", flags & ~known);
  const bool nested = (flags & SRT_NESTED_RANGE) != 0;
  if (nested && (nside & (nside - 1)) != 0)
    return set_error(SRT_ERR_INVALID_ARGUMENT,
                     "srt_forward_noalloc: NESTED pixel ranges need a power-of-two nside, got %lld", (long long)nside);
  if (n_steps < 1 || n_steps > (1 << 22))
    return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_forward_noalloc: invalid n_steps %d", n_steps);
  if (precision != SRT_PRECISION_MIXED && precision != SRT_PRECISION_FP64)
    return set_error(SRT_ERR_UNSUPPORTED,
                     "srt_forward_noalloc: precision %d not available (MIXED or FP64; REF16 builds FP16 planes on "
                     "first use)",
                     precision);
  if (!maps) return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_forward_noalloc: maps is NULL");
  for (int m = 0; m < SRT_NUM_MAPS; ++m)
    if (!maps[m] && pix_count > 0)
      return set_error(SRT_ERR_INVALID_ARGUMENT, "srt_forward_noalloc: maps[%d] is NULL", m);
  if (pix_count == 0) return SRT_OK;
  cudaStream_t s = (cudaStream_t)stream;
  int prev = 0;
  cudaGetDevice(&prev);
  if (prev != fields->device) cudaSetDevice(fields->device);
  int rc = SRT_OK;
  do {
    DeviceScratch sc;
    rc = scratch_for(fields->device, &sc);
    if (rc != SRT_OK) break;
    TraceArgs a;
    a.F = make_ptrs(fields);
    a.G = make_geom(fields);
    a.nside = nside;
    int l = 0;
    while ((int64_t(1) << l) < nside) ++l;
    a.log2p = l;
    a.launch_rays = nested ? pix_count : 12 * (int64_t(1) << (2 * l));
    a.pix_begin = pix_begin;
    a.pix_count = pix_count;
    a.nested = nested;
    a.n_steps = n_steps;
    for (int m = 0; m < 6; ++m) a.maps[m] = maps[m];
    const bool refine = precision == SRT_PRECISION_MIXED && !(flags & SRT_MIXED_NO_REFINE);
    a.refine_list = refine ? sc.list : nullptr;
    a.refine_count = refine ? sc.count : nullptr;
    cudaError_t e = cudaSuccess;
    if (refine) e = cudaMemsetAsync(sc.count, 0, sizeof(unsigned long long), s);
    const int kmode = (precision == SRT_PRECISION_MIXED && fields->pr[0]) ? kMIXED_PAIR : precision;
    if (e == cudaSuccess) e = launch_trace(kmode, a, s, nullptr);
    if (e == cudaSuccess && refine) e = launch_refine(a, s, nullptr);
    if (e == cudaSuccess && !(flags & SRT_ASYNC)) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = cuda_error(e, "srt_forward_noalloc");
  } while (false);
  if (prev != fields->device) cudaSetDevice(prev);
  return rc;
}
