/*
 * srt.h — C ABI of the GB300-native snapshot ray tracer (libsrt.so).
 *
 * The reference program (snapshot-raytracer.cu) has no library API: its only
 * boundary is the CLI in main() (snapshot-raytracer.cu:600-1007) and, inside
 * it, one device launch of raytracing_kernel (snapshot-raytracer.cu:552-583,
 * launched at :897-901). Each entry point below names the part of that program
 * it replaces. All functions:
 *   - return SRT_OK (0) on success and a negative SRT_ERR_* code on failure;
 *     the message of the last failure on the calling thread is available from
 *     srt_last_error(); nothing here calls exit();
 *   - take plain pointers and sizes; "host" pointers are ordinary CPU memory
 *     (pinned or pageable), "device" pointers are CUDA global memory of the
 *     current device;
 *   - are synchronous unless SRT_ASYNC is passed, in which case work is
 *     ordered on the given cudaStream_t (passed as void*; NULL = legacy
 *     default stream).
 * A handle may be used from one thread at a time.
 *
 * Grid convention (mirrors snapshot-raytracer.cu:216-256, :560, :645): a
 * scalar field is a flat array of n0*n1*n2 floats in which voxel (i,j,k)
 * lives at index i + n0*(j + n1*k); i is the x axis and varies fastest. The
 * CLI passes the HDF5 extents of /data in file order (dims[0], dims[1],
 * dims[2]) as (n0, n1, n2), exactly as the reference does, which is only
 * self-consistent for cubic grids. The grid is periodic; voxel i sits at
 * coordinate x = i and the observer at (n0/2, n1/2, n2/2).
 *
 * Maps (order used everywhere below, the reference's write order,
 * snapshot-raytracer.cu:941-987):
 *   0 dA, 1 ellipticity1, 2 ellipticity2, 3 rotation, 4 deflection1,
 *   5 deflection2.
 */
#ifndef SRT_H
#define SRT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SRT_ABI_VERSION 4

/* status codes */
#define SRT_OK 0
#define SRT_ERR_INVALID_ARGUMENT (-1)
#define SRT_ERR_CUDA (-2)
#define SRT_ERR_OUT_OF_MEMORY (-3)
#define SRT_ERR_IO (-4)
#define SRT_ERR_FORMAT (-5)
#define SRT_ERR_NO_DEVICE (-6)
#define SRT_ERR_UNSUPPORTED (-7)
#define SRT_ERR_OVERFLOW (-8) /* srt_vjp, SRT_DETERMINISTIC: a gradient beyond the
                                 fixed-point range */
#define SRT_ERR_CANCELLED (-9) /* srt_fields_load_h5: the progress callback asked
                                  to stop */

/* precision modes of srt_forward / srt_vjp */
#define SRT_PRECISION_FP64 0  /* all-FP64 interpolation, right-hand side and state */
#define SRT_PRECISION_MIXED 1 /* FP32 interpolation and right-hand side on a
                                 perturbation state; FP64 only at ray setup
                                 and map extraction */
#define SRT_PRECISION_REF16 2 /* the reference's own arithmetic: B quantised to
                                 FP16 x 2^27, FP32 interpolation with the cell
                                 offset taken in FP32, FP64 state */

/* flags */
#define SRT_INPUT_DEVICE 1u  /* srt_fields_create: phi / b point to device memory */
#define SRT_OUTPUT_DEVICE 2u /* srt_forward / srt_vjp: outputs are device memory */
#define SRT_ASYNC 4u         /* do not synchronise; order work on `stream` (host
                                buffers must stay valid until it completes) */
#define SRT_ACCUMULATE 8u    /* srt_vjp: add into the gradient grids instead of
                                overwriting them */
#define SRT_DETERMINISTIC 16u /* srt_vjp: order-independent (bitwise
                                 reproducible) FP64 gradient accumulation */
#define SRT_FIELDS_NO_PAIRS 32u /* srt_fields_create: do not build the row-pair
                                   copies of the fields (2x the field memory)
                                   that the MIXED forward reads when present */
#define SRT_FIELDS_STAGED 256u /* srt_fields_create: copy host inputs through a
                                  device slab even when they are mapped pinned
                                  memory the layout kernel could read directly */
#define SRT_MIXED_NO_REFINE 64u /* srt_forward, MIXED: keep the FP32 result of
                                   rays that passed within 1e-7 cell of a cell
                                   face instead of re-tracing them in FP64 */
#define SRT_NESTED_RANGE 128u /* srt_forward: [pix_begin, pix_begin + pix_count)
                                 is a range of NESTED pixel indices (nside a power
                                 of two; base pixel b is [b nside^2, (b+1) nside^2))
                                 and maps[m][i] belongs to NESTED pixel
                                 pix_begin + i */

#define SRT_NUM_MAPS 6

typedef struct srt_fields srt_fields;

typedef struct srt_stats {
  double trace_ms;     /* device time of the trace (or adjoint) kernels, CUDA events */
  double total_ms;     /* host wall time of the call */
  int64_t rays;        /* rays traced */
  int64_t ray_steps;   /* rays x n_steps */
  int64_t kernels;     /* kernels this call launched */
  int64_t h2d_bytes;   /* bytes copied host -> device by this call */
  int64_t d2h_bytes;   /* bytes copied device -> host by this call */
  int64_t refined_rays; /* MIXED: rays re-traced in FP64 (synchronous calls) */
  double retrace_ms;    /* srt_forward, MIXED: the re-trace launches' share of trace_ms
                           (synchronous calls; 0 elsewhere). Added in ABI version 4. */
} srt_stats;

/* ---------------------------------------------------------------- library */

/* ABI version (SRT_ABI_VERSION). */
int srt_abi_version(void);

/* Message of the last failure on this thread ("" if none); returns the
 * message length. Replaces the reference's std::cerr diagnostics
 * (snapshot-raytracer.cu:30-186, :602-631, :721-913). */
int srt_last_error(char* buf, size_t len);

/* Number of CUDA devices visible (0 when there is no GPU; never fails). */
int srt_device_count(void);

/* --------------------------------------------------------------- fields */

/* Upload (or adopt from device memory) the Weyl potential phi and the shift
 * vector field B and lay them out for tracing: a periodic halo of one voxel
 * before and two after on every axis, one FP32 plane per B component.
 * phi: n0*n1*n2 floats; b_xyz: 3*n0*n1*n2 floats interleaved per voxel
 * (B_x, B_y, B_z of voxel v at b_xyz[3v+0..2]), the layout of the reference's
 * HDF5 vector read (snapshot-raytracer.cu:89-186). Host inputs in mapped
 * pinned memory (cudaHostAlloc, or cudaHostRegister with mapping) are read by
 * the layout kernel directly over the host link; other host inputs (or all,
 * with SRT_FIELDS_STAGED) are streamed through a device slab, so peak device
 * memory is the laid-out fields plus one slab.
 * Unless SRT_FIELDS_NO_PAIRS, and when device memory allows, each field is
 * also stored as row pairs (f(i,j,k), f(i,j+1,k)) for the packed-FMA MIXED
 * forward; without them MIXED reads the single copy.
 * Replaces snapshot-raytracer.cu:752-855 (cudaMalloc of the fields, the three
 * staged vector3_to_half passes and the phi copy). */
int srt_fields_create(const float* phi, const float* b_xyz, int64_t n0, int64_t n1,
                      int64_t n2, unsigned flags, void* stream, srt_fields** out);

/* Progress of srt_fields_load_h5, reported on the calling thread in this order
 * (dims: the extents of the dataset concerned, in file order). The callback
 * returns 0 to go on; anything else stops the load, which then releases what
 * it holds and returns SRT_ERR_CANCELLED. */
#define SRT_LOAD_PHI_DIMS 1 /* phi's header is read; its data are being read */
#define SRT_LOAD_B_START 2  /* phi is read; the B file's data are being read */
#define SRT_LOAD_B_DIMS 3   /* B's extents (checked against phi's) */
#define SRT_LOAD_UPLOAD 4   /* both files are read; the last planes are being laid out */
typedef int (*srt_load_progress)(int event, const int64_t dims[3], void* ctx);

#define SRT_LOAD_XYZ_HDF5 512u /* srt_fields_load_h5: x is the fastest (last)
                                  HDF5 axis with its own extent; by default the
                                  extents are taken in file order, as the
                                  reference does */

typedef struct srt_load_stats {
  double read_phi_ms;   /* reading (and converting) phi's data, reader thread */
  double read_b_ms;     /* the same for B */
  double layout_ms;     /* host->device copies and layout, overlapped with the reads */
  double after_read_ms; /* from the end of the reads to the fields being ready */
  double total_ms;      /* wall time of the call */
  int64_t h2d_bytes;    /* bytes copied host -> device */
  int64_t n[3];         /* grid extents of the handle, fastest first (n0, n1, n2) */
} srt_load_stats;

/* Read dataset `dset` of the potential file and of the B file (any float or
 * integer element type for phi, array[3] of float for B, with the checks of
 * srt_h5_read_scalar / srt_h5_read_vector3) and lay them out on the device
 * while they are read: a reader thread fills host memory in file order, and
 * every run of planes is copied and laid out as soon as it is complete, so the
 * upload overlaps the read. phi_scale / b_scale multiply the values (1: as
 * read). flags: SRT_LOAD_XYZ_HDF5, SRT_FIELDS_NO_PAIRS. progress (may be NULL)
 * reports the steps the reference prints. Without a CUDA device both files are
 * still read and checked (file errors first, as the reference reports them)
 * before SRT_ERR_NO_DEVICE. Replaces snapshot-raytracer.cu:640
 * and :676 (load_hdf5_array, load_hdf5_vector_field) followed by :752-855
 * (device allocation and the staged copies). */
int srt_fields_load_h5(const char* phi_path, const char* b_path, const char* dset, unsigned flags,
                       double phi_scale, double b_scale, srt_load_progress progress, void* ctx,
                       srt_fields** out, srt_load_stats* stats);

/* Release the device memory of a fields handle (NULL is a no-op). Replaces
 * the reference's cudaFree calls (snapshot-raytracer.cu:917-920, :993-998). */
int srt_fields_destroy(srt_fields* fields);

/* Device bytes held by a fields handle. */
int64_t srt_fields_bytes(const srt_fields* fields);

/* Field memory comes from a per-device pool that keeps what srt_fields_destroy
 * hands back, so that the next srt_fields_create of the same size is not slowed
 * down by the driver mapping tens of GB again. This returns the pool's unused
 * memory to the device (a failed allocation also does, before retrying), and
 * forgets the device addresses srt_forward_noalloc looked up (call it after a
 * cudaDeviceReset, before the next srt_forward_noalloc). No counterpart in the
 * reference. */
int srt_release_cached_memory(void);

/* Failure injection for tests: after `after` more device allocations by this
 * library have succeeded, the next one fails as if the device were out of
 * memory (the call making it returns SRT_ERR_OUT_OF_MEMORY, frees what it had
 * allocated and leaves earlier handles usable); the hook then disarms itself.
 * after < 0 disarms it. Process-wide, for all devices and threads. The
 * reference reports a failed cudaMalloc and returns -1
 * (snapshot-raytracer.cu:752-772); this lets tests drive that path without
 * exhausting a device. */
int srt_debug_fail_alloc(int64_t after);

/* -------------------------------------------------------------- forward */

/* Trace one ray per HEALPix RING pixel p in [pix_begin, pix_begin+pix_count)
 * for n_steps RK4 steps of one grid unit and write the six maps:
 * maps[m][p - pix_begin] (m in the map order above; each maps[m] holds
 * pix_count floats, on the host unless SRT_OUTPUT_DEVICE).
 * Rays are set up from the pixel centres and the observer at the box centre on
 * the device and launched in NESTED order for locality; results are stored at
 * their RING index. MIXED traces in FP32 and re-traces in FP64 the few rays
 * (~0.1% at 512 steps) whose stage positions pass a cell face closer than
 * the FP32 trajectory's error bound, 4e-7 (s max|dn| + 1e-3) grid units at
 * affine distance s, where the FP32 and FP64 trajectories could pick different cells (the
 * Catmull-Rom Hessian jumps across faces); those rays then equal the FP64
 * result bit for bit (SRT_MIXED_NO_REFINE skips this). The CLI's batch b is
 * pix_begin = b*nside^2, pix_count = nside^2 (snapshot-raytracer.cu:708-717);
 * all pixels is pix_begin = 0, pix_count = 12*nside^2. With SRT_NESTED_RANGE
 * the range counts NESTED pixels instead (HEALPix base pixel b, the batch the
 * reference's README describes, is [b*nside^2, (b+1)*nside^2)), and
 * maps[m][i] belongs to NESTED pixel pix_begin + i.
 * Replaces snapshot-raytracer.cu:857-913 (pix2ang loop, theta/phi upload,
 * raytracing_kernel launch) and the map read-back of :941-987.
 * Errors: nside < 1 or nside > 2^16, pix range outside [0, 12*nside^2],
 * n_steps < 1 or > 2^22, unknown precision, SRT_NESTED_RANGE with an nside
 * that is not a power of two -> SRT_ERR_INVALID_ARGUMENT. */
int srt_forward(const srt_fields* fields, int64_t nside, int64_t pix_begin, int64_t pix_count,
                int n_steps, int precision, float* const maps[SRT_NUM_MAPS], unsigned flags,
                void* stream, srt_stats* stats);

/* Forward trace that allocates no device memory, for callers that cannot
 * allocate when they trace: applications whose device memory is reserved up
 * front by their own pool (a fresh cudaMalloc fails there) and loops that
 * cannot take the device-wide synchronisation a cudaMalloc / cudaFree may
 * imply. Same arguments and results as srt_forward with SRT_OUTPUT_DEVICE
 * (maps are device buffers of pix_count floats each), MIXED or FP64. The
 * scratch (the list of rays MIXED re-traces in FP64) lives in a file-scope
 * device array of 2^20 ray indices (8 MiB) that every GPU loading the library
 * holds until exit, so one call traces at most 2^20 rays; larger ranges are
 * rejected with SRT_ERR_INVALID_ARGUMENT. The first call on a device looks up
 * the array's address (make it before any stream capture). Calls share the
 * array: calls whose work overlaps on the GPU race. Synchronous unless
 * SRT_ASYNC; SRT_NESTED_RANGE and SRT_MIXED_NO_REFINE act as in srt_forward;
 * any other flag (bar SRT_OUTPUT_DEVICE, which is implied) is refused with
 * SRT_ERR_UNSUPPORTED. No counterpart in the reference (it has no library
 * API). */
int srt_forward_noalloc(const srt_fields* fields, int64_t nside, int64_t pix_begin, int64_t pix_count,
                        int n_steps, int precision, float* const maps[SRT_NUM_MAPS], unsigned flags,
                        void* stream);

/* ------------------------------------------------------------------ vjp */

/* Gradient of L = sum_m sum_p weights[m][p] * maps[m][p] (maps as produced by
 * srt_forward with the same arguments) with respect to the phi grid and the
 * three B component grids. dphi: n0*n1*n2 floats; db_xyz: 3*n0*n1*n2 floats
 * interleaved like the b_xyz input. Either may be NULL to skip it. The forward
 * state is checkpointed every ckpt_every steps (<= 0 picks ~sqrt(n_steps)) and
 * each segment is recomputed during the reverse sweep. Gradients are
 * overwritten unless SRT_ACCUMULATE. SRT_DETERMINISTIC accumulates in 64-bit
 * fixed point (2^32 units per unit of gradient) so repeated calls give
 * identical bits; a voxel whose gradient, or a single contribution to it,
 * reaches 2^30 in magnitude (or is not finite) makes the call fail with
 * SRT_ERR_OVERFLOW instead of returning wrapped sums.
 * No counterpart in the reference (it has no derivatives); the forward it
 * differentiates is snapshot-raytracer.cu:315-583. */
int srt_vjp(const srt_fields* fields, int64_t nside, int64_t pix_begin, int64_t pix_count,
            int n_steps, int precision, const float* const weights[SRT_NUM_MAPS], float* dphi,
            float* db_xyz, int ckpt_every, unsigned flags, void* stream, srt_stats* stats);

/* A forward trace's checkpoints, for srt_vjp_tape. */
typedef struct srt_tape srt_tape;

/* srt_forward (MIXED) that also keeps, on the device, the state of every ray
 * every ckpt_every steps (<= 0 picks ~sqrt(n_steps)), so that srt_vjp_tape can
 * form the gradient without tracing the rays forward again: the forward half
 * of a forward/vjp pair. The maps are srt_forward's (flagged rays re-traced
 * in FP64). The tape holds (n_steps/ckpt_every + 1) x 38 floats and one
 * index per ray; the fields must outlive it. pix_count >= 1; flags:
 * SRT_OUTPUT_DEVICE. No counterpart in the reference (it has no
 * derivatives). */
int srt_forward_tape(const srt_fields* fields, int64_t nside, int64_t pix_begin, int64_t pix_count,
                     int n_steps, int ckpt_every, float* const maps[SRT_NUM_MAPS], unsigned flags,
                     void* stream, srt_stats* stats, srt_tape** tape);

/* srt_vjp (MIXED) of the tape's forward: the same gradient as srt_vjp with the
 * tape's arguments and checkpoint interval, without its checkpointing forward
 * pass. flags: SRT_OUTPUT_DEVICE, SRT_ACCUMULATE, SRT_DETERMINISTIC. The tape
 * can be swept any number of times (e.g. for several weight sets). */
int srt_vjp_tape(const srt_tape* tape, const float* const weights[SRT_NUM_MAPS], float* dphi,
                 float* db_xyz, unsigned flags, void* stream, srt_stats* stats);

/* Device bytes held by a tape. */
int64_t srt_tape_bytes(const srt_tape* tape);

/* Release a tape (NULL is a no-op). */
int srt_tape_destroy(srt_tape* tape);

/* ---------------------------------------------------------- measurement */

/* Measured FMA issue rate of the current GPU (FLOP/s, one FMA = 2 FLOP):
 * kind 0 = FP32, kind 1 = FP64, kind 2 = packed FP32 pairs (FFMA2). This is the roofline denominator of the trace
 * kernels, which are bound by CUDA-core issue rather than by a tensor core or
 * by HBM. No counterpart in the reference. */
int srt_probe_peak(int kind, double* flops_per_s);

/* ------------------------------------------------------------- HEALPix */

/* RING pixel centre: colatitude theta and longitude phi (radians). Replaces
 * chealpix pix2ang_ring64 (snapshot-raytracer.cu:865). */
int srt_pix2ang_ring(int64_t nside, int64_t pix, double* theta, double* phi);
/* NESTED -> RING and RING -> NESTED pixel index (-1 on bad input). */
int64_t srt_nest2ring(int64_t nside, int64_t ipnest);
int64_t srt_ring2nest(int64_t nside, int64_t ipring);

/* ----------------------------------------------------- files (host only) */

/* Read dataset `dset` (e.g. "/data") of an HDF5 file as native float, any
 * rank. On success *data is malloc'ed (free with srt_free), dims[0..*rank-1]
 * hold the extents in file order. Replaces load_hdf5_array
 * (snapshot-raytracer.cu:22-87). */
int srt_h5_read_scalar(const char* path, const char* dset, float** data, int64_t dims[8],
                       int* rank);
/* Read a rank-3 dataset whose element type is array[3] of float (the B
 * field); *data holds 3*n voxels interleaved. Replaces load_hdf5_vector_field
 * (snapshot-raytracer.cu:89-186), including its rank and element-type checks. */
int srt_h5_read_vector3(const char* path, const char* dset, float** data, int64_t dims[3]);
/* Write a float32 dataset (rank 1..8, dims in file order); vector3 != 0 writes
 * array[3] of float elements over a rank-3 dataspace (3 floats per element). */
int srt_h5_write(const char* path, const char* dset, const float* data, const int64_t* dims,
                 int rank, int vector3);
/* Write a HEALPix map as a FITS binary table (one float32 column, RING or
 * NESTED ordering keyword, COORDSYS). Replaces chealpix write_healpix_map
 * (snapshot-raytracer.cu:947-987). overwrite == 0 refuses to replace an
 * existing file, as cfitsio does for a plain file name. */
int srt_fits_write_map(const char* path, const float* map, int64_t nside, int nest,
                       const char* coordsys, int overwrite);
/* Read back a map written by srt_fits_write_map (or any single-column float32
 * HEALPix BINTABLE); *map is malloc'ed (free with srt_free). */
int srt_fits_read_map(const char* path, float** map, int64_t* npix, int64_t* nside, int* nest);
void srt_free(void* p);

#ifdef __cplusplus
}
#endif
#endif /* SRT_H */
