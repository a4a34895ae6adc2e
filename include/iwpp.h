/*
 * iwpp.h -- C ABI of the GB300 reconstruction-by-dilation library (libiwpp.so).
 *
 * Plain pointers and sizes only; `stream` is a cudaStream_t passed as void*
 * (NULL = the legacy default stream).  Images are row-major with byte
 * pitches and live in device memory unless stated otherwise.
 *
 * Semantics (all entry points): in place on `marker`, the result is the least
 * image m >= marker with m[c] >= min(m[p], mask[c]) for every pair of
 * neighbouring pixels p, c (4- or 8-connectivity; pixels outside the image do
 * not exist).  With marker <= mask this is the grayscale reconstruction by
 * dilation of marker under mask, the same bytes the reference computes
 * (IWPP MP/src/MorphologicalReconstruction.cu:43-44 is the rule).
 */
#ifndef IWPP_H
#define IWPP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IWPP_API __attribute__((visibility("default")))

typedef enum iwpp_status {
    IWPP_OK = 0,
    IWPP_ERR_INVALID = 1,   /* bad argument */
    IWPP_ERR_OOM = 2,       /* device allocation failed */
    IWPP_ERR_TIMEOUT = 3,   /* a bounded device-side wait ran out */
    IWPP_ERR_CUDA = 4,      /* a CUDA runtime call failed */
    IWPP_ERR_OVERFLOW = 5,  /* queue overflowed more often than max_restarts */
    IWPP_ERR_NO_DEVICE = 6, /* no CUDA device, or not a GB300-class (sm_103) one */
    IWPP_ERR_BUSY = 7,      /* a server's queue is full or it is shutting down; a
                               waited-for request is not finished yet */
    IWPP_ERR_TOO_LARGE = 8, /* the image needs more workspace than the static scratch of
                               iwpp_reconstruct_noalloc holds, or more device memory
                               than a server's budget */
    IWPP_ERR_INTERNAL = 9   /* a device-side consistency check failed (a queue entry that
                               names no tile): a library defect, reported instead of
                               touching memory outside the job */
} iwpp_status;

typedef enum iwpp_dtype { IWPP_U8 = 0, IWPP_U16 = 1, IWPP_I32 = 2 } iwpp_dtype;

/* The reference's three global-queue implementations (one per source
 * directory).  Same result, different work queue. */
typedef enum iwpp_queue_variant {
    IWPP_QUEUE_DEFAULT = -1, /* IWPP_QUEUE_VARIANT env var, else ASYNC */
    IWPP_QUEUE_MUTEX = 0,    /* IWPP MP: LIFO stack under one spin mutex, one persistent launch */
    IWPP_QUEUE_DOUBLE = 1,   /* IWPP MP DQ: read/write queues swapped every round */
    IWPP_QUEUE_UNIQUE = 2,   /* IWPP MP UQ: double queue, each tile at most once per round */
    IWPP_QUEUE_ASYNC = 3     /* no reference counterpart: the unique queue without rounds
                                (lock-free ring, fetch-and-add claims) */
} iwpp_queue_variant;

/* Fields left at their defaults (tile_rows 0, queue_capacity 0,
 * init_passes -1, solver 0, front_passes 0; or cfg NULL) are taken from the
 * tuning table when it holds an entry for the job's workload class
 * (iwpp_autotune). */
typedef struct iwpp_config {
    int tile_rows;             /* 32 or 64 rows per tile; 0 = default: 64, or 32 when the
                                  job has fewer than 2.5 64-row tiles per resident warp
                                  (mutex queue: always 64) */
    long long queue_capacity;  /* entries per queue buffer; 0 = default; < 0: that multiple
                                  of the job's tile count */
    int init_passes;           /* whole-image passes first (+X, +Y, -X, -Y each); -1 = default
                                  (0; 2 inside the front stage) */
    int grid_ctas;             /* persistent grid size; 0 = one full wave */
    int max_restarts;          /* queue-overflow restarts allowed; 0 = default (64) */
    int timeout_ms;            /* bound on every device-side wait; 0 = default (10000) */
    int clip_marker;           /* 1: marker = min(marker, mask) before reconstructing */
    int plain_loads;           /* 1: never use TMA box loads (else TMA whenever base and
                                  pitch are 16-byte aligned) */
    int solver;                /* in-tile solver: 0 = automatic, 1 = row sweeps (fewest
                                  instructions), 2 = vertical / horizontal passes
                                  (shortest latency), 3 = revisits by a per-tile pixel
                                  queue in shared memory (first visits by passes) */
    int front_passes;          /* the front stage: the pixels at the mask's largest value
                                  raised by connected-component labelling, init_passes
                                  whole-image passes (default 2), and the tile engine started
                                  from the tiles still holding a pixel a neighbour can raise:
                                  0 = default (the tuning table's choice, else 3 when the job's
                                  largest image has 2^26 pixels or more and 2 below that),
                                  1 = always, 2 = never, 3 = decided on the device per job: a
                                  seed check over the untouched images measures the initial
                                  front, and fewer than one tile in 64 with a pixel a neighbour
                                  can raise (a few sparse seeds: long propagation paths) takes
                                  the stage, more leaves the job to the engine (seeded from that
                                  check), 4 = the seed check alone: the engine starts from the
                                  tiles holding a pixel a neighbour can raise instead of every
                                  tile (no labelling, no passes) */
    int phantom_work;          /* fault-injection hook for tests, 0 normally.  1: the job counts
                                  one unit of work that never arrives (a queue entry nobody
                                  inserts; for the round-based queues a CTA that never reaches
                                  the round barrier), so every device-side wait runs out and the
                                  call returns IWPP_ERR_TIMEOUT after timeout_ms, the kernel
                                  having returned */
} iwpp_config;

typedef struct iwpp_stats {
    long long tiles;     /* tiles in the job */
    long long visits;    /* tile visits (loads + local convergence) */
    long long sweeps;    /* in-tile raster / anti-raster sweeps */
    long long pushes;    /* queue insertions */
    int rounds;          /* queue rounds (double / unique) */
    int restarts;        /* overflow restarts from a full queue */
    int status;          /* iwpp_status of the device run */
    int variant;         /* queue variant used */
    double device_ms;    /* device time of the reconstruction (events) */
    long long row_steps; /* tile rows processed by the sweeps */
    /* SM cycles summed over warps per phase, as the reference's clock64
     * timers (IWPP MP/src/MorphologicalReconstruction.cu:199-206, indices
     * MorphologicalReconstruction.cuh:9-13): queue read (waiting for and
     * taking an entry), tile fetch, processing (sweeps), dump (write-back and
     * neighbour detection), queue write (state updates and insertions). */
    long long phase_cycles[5];
    long long launches;    /* kernels this library launched for the job */
    long long top_pixels;   /* pixels the top-level stage labelled (0 without it) */
    long long front_stage;  /* 1: the job ran the front stage, 0: the tile engine alone */
} iwpp_stats;

/* One image of a batch. */
typedef struct iwpp_image {
    void *marker;
    const void *mask;
    size_t pitch_marker;
    size_t pitch_mask;
    int width;
    int height;
    int dtype;
    int connectivity;
} iwpp_image;

typedef struct iwpp_handle_s *iwpp_handle;
typedef struct iwpp_plan_s *iwpp_plan;

/* ---- library ------------------------------------------------------------ */
IWPP_API const char *iwpp_status_string(int status);
IWPP_API int iwpp_version(void);
/* Workspace owner (queues, tile states, counters) bound to one device.
 * Calls that share a handle must be ordered on one stream. */
IWPP_API int iwpp_handle_create(iwpp_handle *out, int device);
IWPP_API int iwpp_handle_destroy(iwpp_handle h);
/* Bytes of device workspace a job of `tiles` tiles needs. */
IWPP_API long long iwpp_workspace_bytes(long long tiles, int variant, long long queue_capacity);
/* Tiles of one image for a dtype and tile height (0 = the default height a
 * single-image call on the current device picks). */
IWPP_API long long iwpp_tile_count(int width, int height, int dtype, int tile_rows);

/* ---- plain reconstruction (replaces MorphologicalReconstruction,
 *      IWPP MP/include/MorphologicalReconstruction.cuh:45-46, generalised to
 *      any size, pitch, dtype, connectivity and queue variant) ------------- */
IWPP_API int iwpp_reconstruct(iwpp_handle h, void *marker, const void *mask, size_t pitch_marker, size_t pitch_mask,
                              int width, int height, int dtype, int connectivity, int variant,
                              const iwpp_config *cfg, void *stream, iwpp_stats *stats);
/* Same, asynchronous: enqueues on `stream` and returns; iwpp_handle_sync
 * waits and reports the device status and counters of the last job. */
IWPP_API int iwpp_reconstruct_async(iwpp_handle h, void *marker, const void *mask, size_t pitch_marker,
                                    size_t pitch_mask, int width, int height, int dtype, int connectivity,
                                    int variant, const iwpp_config *cfg, void *stream);
IWPP_API int iwpp_handle_sync(iwpp_handle h, iwpp_stats *stats);

/* ---- batched: all images in one persistent launch ----------------------- */
IWPP_API int iwpp_reconstruct_batch(iwpp_handle h, const iwpp_image *images, int n, int variant,
                                    const iwpp_config *cfg, void *stream, iwpp_stats *stats);
/* Same, asynchronous on `stream`; iwpp_handle_sync reports the result. */
IWPP_API int iwpp_reconstruct_batch_async(iwpp_handle h, const iwpp_image *images, int n, int variant,
                                          const iwpp_config *cfg, void *stream);
/* A batch captured once into a CUDA graph (state reset + launches); every
 * iwpp_plan_launch re-runs the reconstruction on the same buffers. */
IWPP_API int iwpp_plan_create(iwpp_plan *out, iwpp_handle h, const iwpp_image *images, int n, int variant,
                              const iwpp_config *cfg);
IWPP_API int iwpp_plan_launch(iwpp_plan p, void *stream);
IWPP_API int iwpp_plan_sync(iwpp_plan p, iwpp_stats *stats);
IWPP_API int iwpp_plan_destroy(iwpp_plan p);

/* ---- queue self-test ------------------------------------------------------ */
/* The counterpart of the reference's queue test (IWPP MP DQ/src/
 * globalQueue.cu:161-253, testGlobalQueue / verifyQueue / compareKernel):
 * every warp of a full grid inserts every id of a grid_side x grid_side tile
 * grid `copies` times at once through the variant's own insertion path
 * (mutex stack, write-queue reservations, unique dedup through the tile
 * state word, async ring); the queue is then counted per id on the device.
 * Each id must appear `copies` times (once for the unique queue).  Returns
 * the device status of the run; `out` says whether the counts were right. */
typedef struct iwpp_queue_test_result {
    long long entries;     /* entries found in the queue */
    long long expected;    /* entries the inserts should leave */
    long long mismatched;  /* ids seen a wrong number of times */
    long long first_bad;   /* the smallest such id, -1 if none */
    int status;            /* device status of the run */
    int variant;           /* queue variant tested */
} iwpp_queue_test_result;
IWPP_API int iwpp_queue_selftest(int device, int variant, int grid_side, int copies, iwpp_queue_test_result *out);

/* ---- autotuner ------------------------------------------------------------ */
/* No counterpart in the reference (its tile size, queue sizes and number of
 * initial passes are compile-time constants, IWPP MP/include/
 * MorphologicalReconstruction.cuh:6-7, and commented-out sweeps, MR.cu:792-795).
 * Times candidate configurations on the caller's own batch -- the untuned
 * default for large images, tile rows 64 / 32 x in-tile solver, the best of
 * those started from a seed check, the front stage with 1 / 2 / 3 / 4 / 8
 * whole-image passes, then (if it lost) 1, 2, 4, ... 64 initial raster +
 * anti-raster passes while each doubling is faster, then (mutex / double
 * queues) queue capacity 1x / 16x the tiles --
 * each the median of `repeats` runs (0 = 3) from the same markers, records
 * the fastest in the process-wide tuning table under the batch's workload
 * class (queue variant, pixel type, connectivity, floor(log2(pixels)),
 * single image or batch) and returns it.  On success the markers hold the
 * reconstruction; on failure they are as they came. */
typedef struct iwpp_tune_result {
    iwpp_config best;  /* fastest configuration */
    double best_ms;    /* its median device time */
    double default_ms; /* median device time of the untuned default (default tile height, automatic
                          solver; front_passes 3 with 2 passes for images of 2^26 pixels or more) */
    int candidates;    /* configurations timed */
    int reserved;
} iwpp_tune_result;
IWPP_API int iwpp_autotune(iwpp_handle h, const iwpp_image *images, int n, int variant, int repeats, void *stream,
                           iwpp_tune_result *out);
/* The tuning table as text (one line per class); load merges, a malformed
 * file changes nothing. */
IWPP_API int iwpp_tune_save(const char *path);
IWPP_API int iwpp_tune_load(const char *path);
IWPP_API int iwpp_tune_clear(void);
IWPP_API int iwpp_tune_entries(void);
/* The entry for one image class (batch 0) or batch class (batch 1), as a
 * config; IWPP_ERR_INVALID when there is none. */
IWPP_API int iwpp_tune_lookup(int variant, int dtype, int connectivity, long long pixels, int batch,
                              iwpp_config *out);

/* ---- precondition helper (replaces the reference's clipImage kernel,
 *      IWPP MP/src/MorphologicalReconstruction.cu:827-836) ----------------- */
IWPP_API int iwpp_clip(void *marker, const void *mask, size_t pitch_marker, size_t pitch_mask, int width,
                       int height, int dtype, void *stream);

/* ---- result check ------------------------------------------------------------ */
/* Counts the pixels c of `result` that a neighbour p could still raise,
 * min(result[p], mask[c]) > result[c]: zero for every reconstruction.  A
 * size-independent check for images too large to compare on the CPU.
 * Synchronous on `stream`; any pixel-aligned pitch. */
IWPP_API int iwpp_fixed_point_violations(const void *result, const void *mask, size_t pitch_result,
                                         size_t pitch_mask, int width, int height, int dtype, int connectivity,
                                         void *stream, unsigned long long *count);

/* ---- whole-image raster / anti-raster sweeps (the reference's
 *      *PropagationEntireImage kernels, MR.cu:547-753, and iRec1D*,
 *      IWPP MP DQ/src/MorphologicalReconstruction.cu:817-1074) ------------ */
/* direction: 0 = +X (left to right), 1 = +Y (top to bottom), 2 = -X, 3 = -Y.
 * Each applies the propagation rule along the whole row / column (8-conn
 * also takes the two diagonal pixels of the previous row / column). */
IWPP_API int iwpp_sweep(void *marker, const void *mask, size_t pitch_marker, size_t pitch_mask, int width,
                        int height, int dtype, int connectivity, int direction, void *stream);
/* Times the four sweeps (+X, +Y, -X, -Y) once with CUDA events, like the
 * reference's one_current_pass (DQ MR.cu:1136-1178); ms_out receives 4
 * floats. */
IWPP_API int iwpp_sweep_timing(void *marker, const void *mask, size_t pitch_marker, size_t pitch_mask, int width,
                               int height, int dtype, int connectivity, float *ms_out);

/* ---- reconstruction that allocates nothing ----------------------------- */
/* No counterpart in the reference.  For callers that cannot call cudaMalloc
 * where they reconstruct -- e.g. a framework whose caching allocator owns
 * the device memory budget, or a latency-critical loop that cannot afford
 * the device-wide synchronisation of cudaMalloc / cudaFree.  The caller
 * passes device marker / mask buffers (rows 4-byte aligned, any pitch,
 * uint8 / uint16 / int32, 4- or 8-connectivity); the queues, tile states and
 * counters live in a static device array of IWPP_NOALLOC_SCRATCH_BYTES that
 * every GPU loading the library keeps until the process exits.  It holds
 * images up to about 340 000 tiles (e.g. 32768 x 32768 uint8, 16384 x 16384
 * int32); larger images return IWPP_ERR_TOO_LARGE.  Uses the async queue,
 * 64-row tiles, plain loads; synchronous on `stream` (NULL = legacy default
 * stream).  The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) and the engine's launch shape with that device
 * current.  Both are kept until the process exits, so a cudaDeviceReset
 * between calls is not supported (the kept address would be stale).  All calls share the one
 * array: calls whose work overlaps on the GPU (concurrent host threads or
 * streams) race and must be serialised by the caller.  Each call clears the
 * state it needs; the array otherwise keeps the last call's contents. */
#define IWPP_NOALLOC_SCRATCH_BYTES (4u << 20)
IWPP_API int iwpp_reconstruct_noalloc(void *marker, const void *mask, size_t pitch_marker, size_t pitch_mask,
                                      int width, int height, int dtype, int connectivity, void *stream);

/* ---- serving: a request loop with continuous batching ------------------ */
/* No counterpart in the reference (its only caller is one main() per image,
 * IWPP MP/src/main.cu:59).  Requests (host marker / mask / result buffers)
 * are submitted from any thread and admitted in arrival order while their
 * device bytes (staging copies of both planes plus queue state) fit the
 * memory budget and the device's free memory at admission time (minus a
 * headroom), so memory that other users of the device take or return after
 * the server was created is seen by the next admission.  `lanes` worker threads, each with its own stream and
 * workspace, take every admitted request that is waiting when they come
 * free and run them as one batch (one persistent launch), so requests
 * arriving while others run join the next batch and their copies and
 * kernels overlap on the device.  Device memory comes from a pool that keeps
 * what it allocated resident for the life of the server. */
typedef struct iwpp_server_config {
    int lanes;                 /* concurrent batches, 0 = 3 */
    int max_batch;             /* requests per batch, 0 = 256 */
    int max_pending;           /* waiting requests before submit says BUSY, 0 = 65536 */
    int variant;               /* queue variant, IWPP_QUEUE_DEFAULT = async */
    int tile_rows;             /* 0 = default; batches start the tile engine from a seed check
                                  (front_passes 4) */
    int lane_ctas;             /* CTAs per batch launch, 0 = the whole GPU */
    int timeout_ms;            /* device wait bound per batch, 0 = 60000 */
    long long memory_budget;   /* device bytes for admitted requests, 0 = half the free memory at creation */
    long long memory_headroom; /* device bytes every admission leaves free for other users of
                                  the device: a batch is admitted only while the device's free
                                  memory at that moment (plus what the server's pool holds
                                  unused) covers it and this headroom; 0 = 256 MiB, < 0 = no
                                  live check (the budget alone) */
} iwpp_server_config;

typedef struct iwpp_request_result {
    int status;                /* IWPP_OK or the error of the request's batch */
    int lane;                  /* lane that ran it */
    int batch_size;            /* requests in its batch */
    int reserved;
    double latency_us;         /* submit -> result in the host buffer */
    double queue_us;           /* submit -> admitted into a batch */
    double service_us;         /* admitted -> result in the host buffer */
} iwpp_request_result;

typedef struct iwpp_server_stats {
    long long submitted, completed, failed, rejected;
    long long batches, largest_batch;
    long long pixels;          /* pixels of completed requests */
    long long bytes_in_use;    /* device bytes held by admitted requests now */
    long long bytes_peak;      /* most ever held at once */
    long long memory_budget;
    long long held_back;       /* admissions deferred because the device's free memory at the
                                  time (minus the headroom) could not hold the next request */
} iwpp_server_stats;

typedef struct iwpp_server_s *iwpp_server;

IWPP_API int iwpp_server_create(iwpp_server *out, int device, const iwpp_server_config *cfg);
/* Enqueues one request; returns at once.  marker and mask are read, out
 * (out_pitch bytes per row) receives the reconstruction; all three stay
 * owned by the caller and must stay valid until iwpp_server_wait returns
 * for the ticket.  Pinned host memory makes the copies asynchronous.
 * IWPP_ERR_BUSY: max_pending requests are waiting; IWPP_ERR_TOO_LARGE: the
 * request alone exceeds the memory budget. */
IWPP_API int iwpp_server_submit(iwpp_server s, const void *marker, const void *mask, void *out, size_t pitch_marker,
                                size_t pitch_mask, size_t pitch_out, int width, int height, int dtype,
                                int connectivity, unsigned long long *ticket);
/* Waits up to timeout_ms (< 0: forever) for a ticket; IWPP_ERR_BUSY if it
 * is not finished by then.  On completion returns the request's status,
 * fills `result` (nullable) and forgets the ticket: one waiter gets the
 * result, any other wait on the same ticket returns IWPP_ERR_INVALID. */
IWPP_API int iwpp_server_wait(iwpp_server s, unsigned long long ticket, int timeout_ms, iwpp_request_result *result);
IWPP_API int iwpp_server_stats_get(iwpp_server s, iwpp_server_stats *stats);
/* Finishes every submitted request, then stops the lanes and frees the pool. */
IWPP_API int iwpp_server_destroy(iwpp_server s);

/* ---- reference-compatible entry points --------------------------------- */
/* Exactly the reference signature (IWPP MP/include/MorphologicalReconstruction.cuh:45-46;
 * DQ :53-54, UQ :59-60): uint8, square size x size, 4-connectivity, default
 * stream, synchronous, in place on marker.  The queue variant is
 * IWPP_QUEUE_VARIANT (mutex | double | unique | async), default async.  Errors are
 * kept for iwpp_last_status(). */
IWPP_API void MorphologicalReconstruction(unsigned char *marker, unsigned char *mask, size_t pitchMarker,
                                          size_t pitchMask, int size);
/* The reference raises the device heap limit for its in-kernel queue
 * allocation (IWPP MP/src/globalQueue.cu:3-6).  This library allocates its
 * queues from the host, so this is a no-op kept for source compatibility. */
IWPP_API void configureHeapSize(void);
IWPP_API int iwpp_last_status(void);

#ifdef __cplusplus
}
#endif
#endif
