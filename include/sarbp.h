/*
 * sarbp.h -- C ABI of the GB300 SAR time-domain back-projection focuser.
 *
 * One shared library (libsarbp.so) with plain-C entry points: plain pointers
 * and sizes, no C++ types and no exceptions across the boundary.  Every call
 * returns an int status (SARBP_OK == 0, negative on error) and leaves a
 * human-readable message for sarbp_last_error() on the calling thread.
 *
 * All array pointers are DEVICE pointers (any allocator: PyTorch tensors,
 * cudaMalloc, ...), and `stream` is a cudaStream_t passed as void* (NULL =
 * legacy default stream).  Calls are stream-ordered and asynchronous unless
 * stated otherwise; they are safe to make from several host threads as long
 * as no two concurrent calls share an output or workspace buffer.
 *
 * The call these entry points replace is the reference's focusing function
 *   FocalizzatoreBpPx(xxg1, yyg1, zzg1, mask, index, wgsx, wgsy, wgsz,
 *                     Raw_Data, near_range, dra, lambda_val, Sint)
 * (sar_focuser_puntual_noui.py:149-284, per-pixel body :9-144) and its GPU
 * twins FocalizzatoreBpCuPy / FocalizzatoreBpCuPy_Batched
 * (gpu_small_dataset.py:113-223, :229-362, kernel :9-108) and the chunked
 * driver's kernel (main_gpu.py:60-155).
 */
#ifndef SARBP_H
#define SARBP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SARBP_API __attribute__((visibility("default")))

/* Status codes. */
#define SARBP_OK            0
#define SARBP_EINVAL       -1   /* bad argument (NULL pointer, bad size, ...) */
#define SARBP_EWORKSPACE   -2   /* workspace missing or too small */
#define SARBP_ECUDA        -3   /* CUDA runtime error (message has details) */
#define SARBP_ETIMEOUT     -4   /* a bounded device wait gave up */
#define SARBP_ERANGE       -5   /* size beyond a documented limit */
#define SARBP_EDEVICE      -6   /* device is not a GB300-class sm_103 GPU */
#define SARBP_ECANCELED    -7   /* a serving-queue job was cancelled before admission */

/*
 * One focusing scene: the reference's 13 positional arguments
 * (sar_focuser_puntual_noui.py:149, argument order xxg1, yyg1, zzg1, mask,
 * index, wgsx, wgsy, wgsz, Raw_Data, near_range, dra, lambda_val, Sint).
 *
 * DEM grid arrays hold dim0*dim1 pixels flattened in column-major (Fortran)
 * order, pixel ii = i0 + dim0*i1, exactly as the reference flattens them
 * (sar_focuser_puntual_noui.py:183-188).  The output image uses the same
 * order.
 *
 * Raw data are complex64 stored as interleaved float pairs (re, im), range
 * fastest: sample (range bin r, pulse a) is at raw[2*(a*raw_pitch + r)].  With
 * raw_pitch == nra this is the reference's column-major (Nra, Naz) complex64
 * RawData array as read from RawData_Cmplx_<Nra>x<Naz>.dat.  raw_pitch may be
 * larger (padded rows); the mixed-precision path wants raw + 2*raw_pitch
 * floats to be 16-byte aligned, i.e. raw 16-byte aligned and raw_pitch even.
 */
typedef struct sarbp_scene {
    int64_t dim0, dim1;                       /* DEM grid shape (xxg1.shape) */
    const double  *dem_x, *dem_y, *dem_z;     /* xxg1, yyg1, zzg1 [dim0*dim1] */
    const uint8_t *mask;                      /* Mask_Byte: 1 = focus        */
    const int32_t *index;                     /* Index_Long: aperture centre */
    const int32_t *sint;                      /* Sint_Long: aperture length, -9999 = none */
    const double  *traj_x, *traj_y, *traj_z;  /* wgsx, wgsy, wgsz [>= naz]   */
    const float   *raw;                       /* Raw_Data, see above         */
    int64_t nra, naz, raw_pitch;              /* Raw_Data.shape, row pitch   */
    double near_range, delta_range, lambda;   /* near_range, dra, lambda_val */
} sarbp_scene;

/*
 * Tuning of the mixed-precision kernel.  An all-zero struct (or NULL) selects
 * the library default; sarbp_default_tuning() fills the defaults explicitly.
 * Supported: staged=0 with chunk 32/64 and tiles 32x8, 64x4, 16x16; staged=1,
 * 2 or 3 with chunk 32, 64 or 128 and (tile, window, stage) 16x16/208/32,
 * 16x16/192/32, 16x16/160/32, 16x16/160/16, 16x16/128/32, 16x8/128/32,
 * 16x8/128/16, 32x8/128/32, 64x4/128/32.  The staged kernels copy raw data in 16- or 32-pulse stages
 * through a ring of 64 pulses; the chunk is the pulse group that shares one
 * float-float reference (mid-chunk pulse).  staged=2 and 3 run the staged
 * kernel on a persistent grid that drains a queue of the scene's tiles
 * (built by sarbp_mixed_prepare, a few bytes per tile of workspace): in
 * decreasing estimated cost (2) or increasing last pulse (3, for streamed
 * uploads).  Images are bit-identical across staged=1, 2 and 3.
 */
typedef struct sarbp_tuning {
    int32_t chunk;        /* pulses per chunk: 32, 64 (128: staged only)      */
    int32_t tile0;        /* pixel-tile extent along dim0 (power of two)      */
    int32_t tile1;        /* pixel-tile extent along dim1                     */
    int32_t staged;       /* 0: L1/L2 gathers; 1: TMA-staged raw window, one CTA per
                             tile; 2 / 3: staged, persistent grid over a tile queue
                             ordered by cost / by last pulse */
    int32_t window;       /* staged: range bins staged per pulse stage (0: default) */
    int32_t stage;        /* staged: pulses per TMA stage, 16 or 32 (0: default)   */
    int32_t wait_polls;   /* staged, diagnostic: mbarrier polls before a stage wait
                             gives up (0: default 2^22) */
    int32_t withhold;     /* staged, diagnostic: 1 never issues the first stage's
                             copies of each pass, so that stage's wait runs out
                             (exercises the timeout path, see sarbp_mixed_status);
                             0 in normal use */
} sarbp_tuning;

/* Device counters written by the mixed kernel when `counters` is non-NULL. */
#define SARBP_CTR_AMBIGUOUS   0   /* range bins re-derived in FP64 (near .5 ties) */
#define SARBP_CTR_WINDOW_MISS 1   /* staged-window misses served from L2         */
#define SARBP_CTR_CHUNKS      2   /* pixel x chunk work items processed          */
#define SARBP_CTR_TIMEOUTS    3   /* bounded waits that gave up                  */
#define SARBP_NUM_COUNTERS    8

/* Library version (major*10000 + minor*100 + patch). */
SARBP_API int sarbp_version(void);

/* Last error message on the calling thread ("" if none). */
SARBP_API const char *sarbp_last_error(void);

/* Fill `t` with the library defaults. */
SARBP_API int sarbp_default_tuning(sarbp_tuning *t);

/*
 * Plain FP64 focusing, one thread per pixel, with the reference CPU path's
 * exact semantics: nearest range bin with round-half-to-even, strict pulse
 * bounds 0 < a < Naz-1, bins 0 <= bin < Nra-1, float32-literal pi, beta*R^2
 * phase term, division by the contributor count.
 * Replaces process_point + the pixel loop of FocalizzatoreBpPx
 * (sar_focuser_puntual_noui.py:9-144, :232-241) and the CuPy kernel
 * process_point_kernel (gpu_small_dataset.py:9-108), whose rounding
 * (half away from zero) it does NOT copy.
 *
 * out       complex128 image, dim0*dim1 (re, im) double pairs, column-major.
 * nvalid    optional (NULL): per-pixel contributor count.
 * checksum  optional (NULL): per-pixel sum of mix64(pulse, bin) over the
 *           contributing pulses (bit-exact range-bin selection check).
 */
SARBP_API int sarbp_focus_fp64(const sarbp_scene *scene, double *out,
                               int32_t *nvalid, uint64_t *checksum,
                               void *stream);

/*
 * Bytes of device workspace the mixed-precision path needs for `scene`
 * (>= 0), or a negative status.  The workspace holds the per-pulse chunk
 * table, per-tile plans and a status block; it can be reused across calls
 * on the same stream.
 */
SARBP_API int64_t sarbp_mixed_workspace_size(const sarbp_scene *scene,
                                             const sarbp_tuning *tuning);

/*
 * Mixed-precision focusing: FP64 slant range and phase wrap at each pulse-
 * chunk reference, FP32 differential range / phase / accumulation per pulse,
 * compensated (Kahan) summation across chunks, range bins that match the
 * FP64 path bit-exactly (ambiguous ties are re-derived in FP64).
 * Same outputs as sarbp_focus_fp64.  `counters` (optional, device,
 * SARBP_NUM_COUNTERS uint64) is incremented, not cleared.
 * Replaces the same reference code as sarbp_focus_fp64.
 */
SARBP_API int sarbp_focus_mixed(const sarbp_scene *scene,
                                const sarbp_tuning *tuning,
                                double *out, int32_t *nvalid,
                                uint64_t *checksum, uint64_t *counters,
                                void *workspace, size_t workspace_bytes,
                                void *stream);

/*
 * The two halves of sarbp_focus_mixed, for callers that keep a scene
 * resident and focus it repeatedly (serving, benchmarking): _prepare builds
 * the per-pulse chunk tables in the workspace (they depend on the trajectory
 * only) and, for staged=2, the cost-ordered tile queue (it depends on the
 * mask, sint and index arrays); _prepared runs the focusing kernel on a
 * prepared workspace.
 * sarbp_focus_mixed == sarbp_mixed_prepare + sarbp_focus_mixed_prepared.
 * Same reference counterpart as sarbp_focus_fp64.
 */
SARBP_API int sarbp_mixed_prepare(const sarbp_scene *scene, const sarbp_tuning *tuning,
                                  void *workspace, size_t workspace_bytes, void *stream);
SARBP_API int sarbp_focus_mixed_prepared(const sarbp_scene *scene, const sarbp_tuning *tuning,
                                         double *out, int32_t *nvalid, uint64_t *checksum,
                                         uint64_t *counters, void *workspace,
                                         size_t workspace_bytes, void *stream);

/*
 * Status of the mixed-path kernels that ran on `workspace` since it was last
 * prepared or queried: SARBP_ETIMEOUT when a bounded device wait gave up
 * (the kernel then stopped early, its image is incomplete, and the context
 * stays usable), SARBP_OK otherwise.  Synchronises `stream`, then clears the
 * status.  No counterpart in the reference (its kernels have no device-side
 * waits).
 */
SARBP_API int sarbp_mixed_status(void *workspace, size_t workspace_bytes, void *stream);

/*
 * Streamed focusing (tuning.staged = 3: the prepared workspace holds the
 * scene's tiles ordered by their last aperture pulse).  A caller that uploads
 * the raw data in pulse blocks reads the queue's keys (one past each tile's
 * last pulse, ascending; sarbp_tile_queue_keys synchronises `stream`) and
 * launches sarbp_focus_mixed_range over the queue items whose key is covered
 * as each block lands, so focusing overlaps the upload.  With staged = 2 the
 * keys are the tiles' costs, descending.  No reference counterpart (the
 * reference uploads a whole raw window before each launch,
 * main_gpu.py:430-470).
 */
SARBP_API int sarbp_tile_queue_keys(const sarbp_scene *scene, const sarbp_tuning *tuning,
                                    void *workspace, size_t workspace_bytes, uint32_t *keys,
                                    int64_t n, void *stream);
SARBP_API int sarbp_focus_mixed_range(const sarbp_scene *scene, const sarbp_tuning *tuning,
                                      double *out, int32_t *nvalid, uint64_t *checksum,
                                      uint64_t *counters, void *workspace,
                                      size_t workspace_bytes, int64_t first, int64_t count,
                                      void *stream);

/*
 * Range bins the focusing can read: a superset [range[0], range[1]] of every
 * valid range bin of every (pixel, pulse) pair inside the pixels' apertures,
 * from the pulse-segment bounds the staged kernels use for their windows
 * (endpoint and closest-point distances plus the chord deviation, one bin of
 * margin each side).  `workspace` must hold tables prepared by
 * sarbp_mixed_prepare with a staged tuning; `scene->raw` is not read.
 * Synchronises `stream`; range[0] > range[1] when no pixel has an aperture.
 * With it a caller uploads only the reachable part of each pulse row
 * (sarbp_upload_raw_bins): the kernels never read outside it.  No reference
 * counterpart (the reference reads Raw_Data where it lies).
 */
SARBP_API int sarbp_raw_bin_range(const sarbp_scene *scene, const sarbp_tuning *tuning,
                                  void *workspace, size_t workspace_bytes, int64_t *range,
                                  void *stream);

/*
 * sarbp_raw_bin_range without the synchronisation: the bound is computed and
 * copied into host_range[0..1] (int32, page-locked host memory for the copy
 * to be asynchronous) in stream order, as [1, 0] when no pixel has an
 * aperture; the values are valid once `stream` has passed this call (an
 * event recorded after it has completed).  Lets a serving loop admit a job
 * without waiting for the copies queued ahead of it.  No reference
 * counterpart.
 */
SARBP_API int sarbp_raw_bin_range_async(const sarbp_scene *scene, const sarbp_tuning *tuning,
                                        void *workspace, size_t workspace_bytes,
                                        int32_t *host_range, void *stream);

/*
 * Host -> device copy of range bins [bin_lo, bin_lo + nbins) of `npulses`
 * pulse rows (complex64, row pitches in elements) into the same positions of
 * a device raw buffer: one 2-D copy, asynchronous when `src` is pinned.
 */
SARBP_API int sarbp_upload_raw_bins(void *dst, int64_t dst_pitch, const void *src,
                                    int64_t src_pitch, int64_t bin_lo, int64_t nbins,
                                    int64_t npulses, void *stream);

/*
 * The same copies done by SM loads instead of a copy engine, for callers
 * whose latency depends on their uploads: on the GB300 machines this library is
 * measured on, copy-engine host-to-device transfers stall for 10-100 ms every
 * so often while kernels reading the same memory over the CPU-GPU link did
 * not (at ~90 % of the copy engine's bandwidth).  `src` must be page-locked
 * host memory mapped into the device's address space (cudaHostAlloc, torch
 * pin_memory) or device memory, else SARBP_EINVAL before any launch.
 * sarbp_upload_raw_bins_sm takes sarbp_upload_raw_bins's arguments;
 * sarbp_copy_to_device_sm copies `bytes` bytes.  Stream-ordered, no
 * synchronisation.  No reference counterpart.
 */
SARBP_API int sarbp_upload_raw_bins_sm(void *dst, int64_t dst_pitch, const void *src,
                                       int64_t src_pitch, int64_t bin_lo, int64_t nbins,
                                       int64_t npulses, void *stream);
SARBP_API int sarbp_copy_to_device_sm(void *dst, const void *src, int64_t bytes, void *stream);

/*
 * n host-to-device copies in one call: bytes[i] bytes from src[i] (host) to
 * dst[i] (device), by SM loads where the source is page-locked, else by the
 * copy engine (cudaMemcpyAsync; a pageable source is staged by the driver
 * before the call returns).  All arguments are checked before the first
 * copy.  Used by the drop-in call for the DEM, masks and trajectory (nine
 * arrays, one foreign call).  No reference counterpart.
 */
SARBP_API int sarbp_upload_host_arrays(int32_t n, void *const *dst, const void *const *src,
                                       const int64_t *bytes, void *stream);

/*
 * 1 when the current device loads from and stores to pageable host memory
 * through the host's page tables (cudaDevAttrPageableMemoryAccess and
 * ...UsesHostPageTables: coherent CPU-GPU systems such as GB300 over
 * NVLink-C2C), else 0.  On such a device every SM-load copy above also takes
 * plain (pageable) host memory, read in place at the link's rate rather than
 * staged by the driver.  Such a range is checked on the host first: every
 * page mapped (else SARBP_EINVAL), and each page a copy will write touched
 * on the host, so a bad pointer fails there, not in a kernel.  A file
 * mapping (mmap, np.memmap) is read too, but
 * its pages not yet mapped are faulted in from the device one by one: copy
 * such data into ordinary or page-locked memory first (the Python drop-in
 * does this by leaving file mappings to the driver's staged copies).  No
 * reference counterpart.
 */
SARBP_API int sarbp_device_reads_pageable(void);

/*
 * Device-to-host copy by SM stores: `bytes` bytes from device memory `src`
 * into page-locked host memory (through its mapping) or, on a device that
 * reads pageable memory (above), into any host memory.  Stream-ordered; the
 * data are in host memory once the stream has passed the copy.  The drop-in
 * call writes its fresh result array this way.  No reference counterpart.
 */
SARBP_API int sarbp_copy_to_host_sm(void *dst, const void *src, int64_t bytes, void *stream);

/*
 * The same rows in pulse blocks, copied by one persistent grid of `ctas`
 * CTAs that signals each block: block k is rows [block_ends[k-1],
 * block_ends[k]) (block_ends non-decreasing, at most 32 blocks); when every
 * CTA has copied its share of block k, flags[k] (device uint32) is set to
 * `generation` (non-zero; use a new value per call, e.g. a counter, since
 * flags are never cleared).  counters (device uint32[nblocks]) is scratch,
 * cleared by the call in stream order.  sarbp_stream_wait_flag holds a
 * stream until a flag has reached a value (cuStreamWaitValue32, greater or
 * equal in wrap-around order): work that needs block k is queued behind
 * flags[k] and starts while later blocks are still being copied, and the
 * copy occupies only `ctas` SMs.  Source as for sarbp_upload_raw_bins_sm,
 * 16-byte aligned; both pitches even; the destination 16-byte aligned.
 * No reference counterpart.
 */
SARBP_API int sarbp_upload_raw_blocks_sm(void *dst, int64_t dst_pitch, const void *src,
                                         int64_t src_pitch, int64_t bin_lo, int64_t nbins,
                                         const int64_t *block_ends, int32_t nblocks,
                                         uint32_t *flags, uint32_t *counters,
                                         uint32_t generation, int32_t ctas, void *stream);
/* The same, with the bin interval read by the copy kernel from `bound`
 * (int32[2], inclusive, as sarbp_raw_bin_range_async leaves it: empty when
 * bound[0] > bound[1]; clipped to the rows), device memory or page-locked
 * host memory written in stream order before the copy starts: the copy can
 * be queued behind the bound's computation without the host waiting for it.
 * Every flag is still set when the interval is empty. */
SARBP_API int sarbp_upload_raw_blocks_bound_sm(void *dst, int64_t dst_pitch, const void *src,
                                               int64_t src_pitch, const int32_t *bound,
                                               const int64_t *block_ends, int32_t nblocks,
                                               uint32_t *flags, uint32_t *counters,
                                               uint32_t generation, int32_t ctas, void *stream);
SARBP_API int sarbp_stream_wait_flag(void *stream, const uint32_t *flag, uint32_t value);
/* 1 when the driver provides the stream wait sarbp_stream_wait_flag uses
 * (cuStreamWaitValue32), else 0: callers fall back to event ordering. */
SARBP_API int sarbp_stream_wait_supported(void);

/*
 * Batches: many scenes of uneven size in one persistent launch.
 * Replaces the reference's per-batch host loops (gpu_small_dataset.py:285-339,
 * main_gpu.py:415-586), which launch one kernel per pixel batch and copy
 * results back after each; here all scenes' pixel tiles are items of one
 * device work queue, drained by a persistent grid (one launch, capturable in
 * a CUDA graph).
 *
 * sarbp_tile_count / sarbp_tile_costs: number of pixel tiles of a scene under
 *   `tuning`, and per tile (device int64 array) the sum of its pixels' kept
 *   aperture lengths -- the cost estimate used to order the queue.
 * sarbp_batch_workspace_size: bytes of the batch workspace (scene
 *   descriptors + queue) for `nscenes` scenes and up to `max_items` items.
 * sarbp_batch_set_scene: describe scene `slot` (its mixed workspace must be
 *   prepared with sarbp_mixed_prepare under the same tuning); the descriptor
 *   is written in stream order by a kernel that receives it as a parameter,
 *   so the host never waits.
 * sarbp_batch_set_items: upload the queue, `n_items` (scene slot, tile index)
 *   int32 pairs in processing order (decreasing cost balances the load); from
 *   pageable host memory the copy first waits for `stream`.
 * sarbp_batch_focus: reset the queue cursor and launch the persistent kernel;
 *   stream-ordered, no host synchronisation, capturable in a CUDA graph.
 *   `diagnostics` != 0 also writes the scenes' checksum outputs.
 * The batch path needs the staged kernel (tuning.staged = 1; 32-, 64- or
 * 128-pulse chunks).
 */
SARBP_API int64_t sarbp_tile_count(const sarbp_scene *scene, const sarbp_tuning *tuning);
SARBP_API int sarbp_tile_costs(const sarbp_scene *scene, const sarbp_tuning *tuning,
                               int64_t *costs, void *stream);
SARBP_API int64_t sarbp_batch_workspace_size(int32_t nscenes, int64_t max_items);
SARBP_API int sarbp_batch_set_scene(void *batch_ws, size_t batch_bytes, int32_t nscenes,
                                    int32_t slot, const sarbp_scene *scene,
                                    const sarbp_tuning *tuning, void *scene_ws,
                                    size_t scene_ws_bytes, double *out, int32_t *nvalid,
                                    uint64_t *checksum, void *stream);
SARBP_API int sarbp_batch_set_items(void *batch_ws, size_t batch_bytes, int32_t nscenes,
                                    const int32_t *items, int64_t n_items, void *stream);
SARBP_API int sarbp_batch_focus(void *batch_ws, size_t batch_bytes, int32_t nscenes,
                                const sarbp_tuning *tuning, int64_t n_items, int32_t diagnostics,
                                uint64_t *counters, void *stream);

/*
 * Mixed-precision focusing for callers that cannot allocate device memory.
 * No counterpart in the reference: it exists for callers that only hold the
 * device pointers of their inputs and outputs -- plugins inside applications
 * whose memory pool owns the device, real-time pipelines that may not call
 * cudaMalloc (it can synchronise the device and has unbounded latency), thin
 * bindings without an allocator.  Same arguments and results as
 * sarbp_focus_mixed minus the workspace: the scratch lives in one
 * library-owned device array of about 7 MiB, sized for scenes of at most
 * SARBP_NOALLOC_MAX_PULSES pulses (larger scenes are rejected with
 * SARBP_ERANGE), which every GPU that loads the library keeps until the
 * process exits.  The first call in a device's CUDA context looks up the
 * array's device address in that context, so make it before any stream
 * capture.  Every call shares the one array: calls whose work overlaps on
 * the GPU (different streams, or other host threads) race and must be
 * serialised by the caller.  Unlike sarbp_focus_mixed this call waits for
 * `stream` before it returns: it reads the array's status block back and
 * returns SARBP_ETIMEOUT when a bounded device wait gave up (the image is
 * then incomplete).  Calls no cudaMalloc/cudaFree.
 */
#define SARBP_NOALLOC_MAX_PULSES 131072
SARBP_API int sarbp_focus_mixed_noalloc(const sarbp_scene *scene,
                                        const sarbp_tuning *tuning,
                                        double *out, int32_t *nvalid,
                                        uint64_t *checksum, uint64_t *counters,
                                        void *stream);

/*
 * Serving queue: continuous batching of focusing jobs on one device.
 * sarbp_queue_create starts a worker thread on the calling thread's current
 * device with two streams and two batch workspaces (`max_slots` scenes
 * resident at once, waves of up to `wave_items` tiles; 0 picks 6 per SM;
 * tuning.staged must be 1).  sarbp_queue_submit enqueues a device-resident
 * scene (caller-owned buffers, valid until the job is done) with its device
 * output (npix complex128) and returns a job id (>= 0) or a negative status.
 * The worker admits jobs into free slots in arrival order and runs waves of
 * the persistent batch kernel over the tiles of every admitted job; a job's
 * image equals sarbp_focus_mixed's bit for bit.  sarbp_queue_poll returns 1
 * when the job is done, 0 while it is not, a negative status if it failed
 * (SARBP_ETIMEOUT when a bounded device wait gave up); sarbp_queue_wait
 * blocks until done.  Completion is reported once: the job id is released
 * then.  sarbp_queue_destroy finishes the submitted jobs, stops the worker
 * and frees the queue.  Replaces the reference's per-batch host loops
 * (gpu_small_dataset.py:285-339) for many independent requests; the
 * reference has no serving component.
 */
typedef struct sarbp_queue sarbp_queue;
SARBP_API int sarbp_queue_create(sarbp_queue **queue, const sarbp_tuning *tuning,
                                 int32_t max_slots, int64_t wave_items);
SARBP_API int64_t sarbp_queue_submit(sarbp_queue *queue, const sarbp_scene *scene, double *out);
SARBP_API int sarbp_queue_poll(sarbp_queue *queue, int64_t job);
SARBP_API int sarbp_queue_wait(sarbp_queue *queue, int64_t job);
SARBP_API int sarbp_queue_destroy(sarbp_queue *queue);

/*
 * Host-memory jobs of the serving queue: the whole request path runs on the
 * queue's worker thread, none of it on the caller's.
 * sarbp_queue_reserve sets aside `bytes` of device memory (one allocation,
 * made here, freed by sarbp_queue_destroy) from which each host job's
 * device copies are carved -- DEM, masks, trajectory, raw rows, image and
 * chunk tables, sarbp_queue_job_bytes(queue, scene) bytes; jobs are
 * admitted in arrival order when a scene slot is free and their bytes fit.
 * sarbp_queue_submit_host takes a scene whose array pointers are HOST
 * pointers (same layouts as a device scene: column-major DEM grid arrays,
 * raw data as rows of raw_pitch complex64 bins per pulse) and a host output
 * of npix complex128; the worker uploads the small inputs, prepares the
 * chunk tables, bounds the range bins the apertures can reach and uploads
 * only those bins of each pulse row, runs the job's tiles in waves with
 * the other jobs' and copies the image to `host_out` (bit-identical to
 * sarbp_focus_mixed's).  Page-locked host memory (cudaHostAlloc, torch
 * pin_memory) is read by SM loads and written asynchronously; pageable
 * memory goes through the copy engine and holds the worker while it copies.
 * The caller's buffers must stay valid until the job is reported done.
 * sarbp_queue_completed drains up to `max` finished jobs (host or device)
 * into ids[], with their completion time in seconds of the monotonic clock
 * (CLOCK_MONOTONIC; Python's time.monotonic) in done_s[] and their status
 * in status[] (both optional); it returns how many it reported.  A job is
 * reported once, by whichever of sarbp_queue_completed / _poll / _wait sees
 * it first.  No reference counterpart (the reference has no serving path).
 */
SARBP_API int sarbp_queue_reserve(sarbp_queue *queue, size_t bytes);
SARBP_API int64_t sarbp_queue_job_bytes(sarbp_queue *queue, const sarbp_scene *scene);
SARBP_API int64_t sarbp_queue_submit_host(sarbp_queue *queue, const sarbp_scene *host_scene,
                                          double *host_out);
SARBP_API int64_t sarbp_queue_completed(sarbp_queue *queue, int64_t *ids, double *done_s,
                                        int32_t *status, int64_t max);
/*
 * Totals since the queue was created, into stats[0..4]: jobs completed,
 * waves launched, kernel launches (waves, and for host jobs their copies,
 * chunk tables, bound and batch-slot kernels), bytes copied host -> device
 * and device -> host for host jobs.  No reference counterpart.
 */
SARBP_API int sarbp_queue_stats(sarbp_queue *queue, int64_t *stats);
/*
 * Cancel a job that is still waiting for admission: it is reported done with
 * status SARBP_ECANCELED (through sarbp_queue_completed, _poll or _wait) and
 * none of its buffers is touched.  SARBP_EINVAL for a job that is already
 * admitted (its work is on the device) or unknown.  No reference
 * counterpart.
 */
SARBP_API int sarbp_queue_cancel(sarbp_queue *queue, int64_t job);

/*
 * 8-bit amplitude preview of a focused image: out[i] = clip(|image[i]| *
 * 255 / (scale_factor * mean|image|), 0, 255) truncated to uint8 -- the
 * reference visualiser's scaling (img_visualizer.py:23-46, scale_factor 15)
 * computed on the device.  image: npix complex128 (re, im) pairs; out: npix
 * bytes (same pixel order); mean: optional (NULL), one double receiving
 * mean|image|; scratch: device memory for the fixed-order partial sums (one
 * double per block; SARBP_PREVIEW_SCRATCH_BYTES is enough on any GPU).  All
 * pointers are device pointers.  Stream-ordered, no synchronisation.
 */
#define SARBP_PREVIEW_SCRATCH_BYTES 16384
SARBP_API int sarbp_amplitude_u8(const double *image, int64_t npix, double scale_factor,
                                 uint8_t *out, double *mean, double *scratch,
                                 size_t scratch_bytes, void *stream);

/*
 * Measurement helper (no counterpart in the reference, which publishes no
 * roofline): measures this device's issue rates with probe kernels on
 * `stream` and returns them in rates[0..3] = FP32 FMA lanes/s, SFU sin
 * evaluations/s, FP64 FMA lanes/s, SM count.  Synchronises the stream.
 */
SARBP_API int sarbp_probe_issue_rates(double *rates, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* SARBP_H */
