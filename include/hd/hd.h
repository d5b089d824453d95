/*
 * hd.h -- C ABI of the GB300 dilation-based Hausdorff distance library
 * (libhd_gb300.so).
 *
 * This is the drop-in boundary for the reference's single entry point
 *     int HausdorffDistance::computeDistance(Volume* img1, Volume* img2);
 * (forBench/HausdorffDistance.cuh:17, implemented at
 * forBench/HausdorffDistance.cu:101-187).  Plain pointers and sizes only.
 *
 * Masks: uint8, nonzero = foreground, x fastest, index x + W*y + W*H*z, the
 * layout of Volume (forBench/Volume.h:51-54; `bool` is one byte).  Both masks
 * of a pair share one W x H x D (the reference reads img1's sizes only,
 * forBench/HausdorffDistance.cu:103).
 *
 * Distances are integer dilation counts under a structuring element:
 *   HD_SE6            6 face neighbours (Manhattan metric)
 *                     = IS_3D 1, CHEBYSHEV 0 at forBench/HausdorffDistance.cuh:7-8
 *   HD_SE18_FORBENCH  the reference's shipped default, CHEBYSHEV 1: faces,
 *                     4 in-plane xy diagonals, 8 corners
 *                     (forBench/HausdorffDistance.cu:35-58)
 * hd = min{k : D^k(A) contains B and D^k(B) contains A}, the value the
 * reference returns.  avg_hd = (sum_ab + sum_ba) / (n_a + n_b) with exact
 * integer sums of the per-voxel distances (the per-voxel value is the one
 * hello.cu:1588-1625 records for each newly covered voxel).
 *
 * Conventions that differ from the reference on purpose:
 *   - every call returns an hd_status; nothing exits the process and nothing
 *     resets the device (the reference exits at :189-195 and calls
 *     cudaDeviceReset at :181);
 *   - exactly one empty mask returns HD_EMPTY_MASK at once (the reference
 *     loops forever); two empty masks give hd = 0;
 *   - device state belongs to an hd_context; calls on one context are
 *     serialised by the context's lock; separate contexts run independently.
 */
#ifndef HD_HD_H
#define HD_HD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum hd_status {
    HD_OK = 0,
    HD_EMPTY_MASK = 1,       /* exactly one mask is empty: HD undefined */
    HD_ERR_BAD_ARG = 2,      /* null pointer, non-positive size, unknown metric ... */
    HD_ERR_OOM = 3,          /* device or pinned-host allocation failed */
    HD_ERR_CUDA = 4,         /* a CUDA runtime call failed */
    HD_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up */
    HD_ERR_CANCELLED = 6,    /* server request cancelled */
    HD_ERR_ITER_LIMIT = 7,   /* more dilation steps than the volume's diameter */
    HD_ERR_NOT_READY = 8,    /* server request still in flight */
    HD_ERR_UNSUPPORTED = 9,  /* feature not compiled in (e.g. HDF5) */
    HD_ERR_BUSY = 10         /* server admission queue full */
} hd_status;

typedef enum hd_metric {
    HD_SE6 = 0,
    HD_SE18_FORBENCH = 1
} hd_metric;

/* Per-pair result.  _ab is "A measured against B": sum_ab = sum over a in A
 * of d(a, B), hd_ab = max over a in A of d(a, B). */
typedef struct hd_result {
    int32_t hd;          /* max(hd_ab, hd_ba); -1 when status != HD_OK */
    int32_t iterations;  /* grid-barrier iterations of the device loop for this call (each runs one
                            or more dilation steps, see hd_options.kernel) */
    uint64_t sum_ab;
    uint64_t sum_ba;
    uint64_t n_a;
    uint64_t n_b;
    uint64_t n_a_not_b;
    uint64_t n_b_not_a;
    double avg_hd;       /* (sum_ab + sum_ba) / (n_a + n_b); NaN on HD_EMPTY_MASK */
    int32_t status;      /* hd_status of this pair */
    int32_t hd_ab;
    int32_t hd_ba;
    int32_t hd_robust;   /* percentile HD (hd_options.percentile), stopping rule of hello.cu:1751-1758 */
} hd_result;

/* Options of a context.  Fill with hd_options_init, then override. */
typedef struct hd_options {
    int32_t brick_x_words;       /* kernel 1 brick width in 32-voxel words: 2, 4, 8; 0 = tuned */
    int32_t brick_z;             /* brick depth in planes: 4, 8, 16 (kernel 1), 8, 16 (kernel 2); 0 = tuned */
    int32_t ctas_per_sm;         /* persistent CTAs per SM; 0 = occupancy maximum */
    int32_t max_iterations;      /* cap on dilation steps; 0 = W + H + D */
    int64_t barrier_timeout_ns;  /* give-up time of one grid-barrier wait; 0 = 10 s */
    float percentile;            /* hd_robust percentile in (0, 1]; default 0.95 */
    int32_t zero_copy;           /* hd_compute_u8: kernels read host masks in place when the
                                    device can address them (default 1) */
    const char* tuning_table;    /* autotuner JSON table to load/store; NULL = none */
    int32_t record_timings;      /* record CUDA events around each kernel (hd_context_last_timings) */
    int32_t kernel;              /* dilation kernel: 0 = tuned/default, 1 = one step per grid barrier
                                    (brick_x_words x 32/brick_x_words rows x brick_z planes),
                                    2 = temporally blocked (steps_per_barrier steps per barrier,
                                    4 words x (32 - 2 steps) rows x brick_z planes) */
    int32_t steps_per_barrier;   /* kernel 2: 1, 2 (brick_z 8 or 16), 3, 4 or 5 (brick_z 8); 0 = tuned/default */
    int32_t label;               /* foreground voxels: 0 = every nonzero byte (default); 1..255 = the bytes
                                    equal to `label` (the prototype's numberToLookFor, hello.cu:133,615),
                                    so one uint8 label volume serves every structure it holds */
} hd_options;

/* Device durations of the last call's kernels (record_timings = 1), measured
 * with CUDA events on the stream the kernels were launched on. */
typedef struct hd_timings {
    float pack_ms;       /* bit packing + bounding box + counts */
    float setup_ms;      /* crop into job domains + first-step queue */
    float solve_ms;      /* persistent dilation loop */
    float total_ms;      /* first launch to last kernel end */
    int32_t iterations;  /* grid-barrier iterations run by the persistent loop */
    int32_t grid_ctas;   /* CTAs of the persistent launch */
    int32_t brick_x_words, brick_z;
    int32_t kernel;      /* 1 = one step per barrier, 2 = temporally blocked */
    int32_t steps_per_barrier;
    int32_t brick_rows;
    int32_t dilation_partitions; /* pipelined entry on split SMs: dilations in
                                    flight side by side on disjoint SM groups
                                    (1 to 3); 0 on the other entries */
} hd_timings;

typedef struct hd_context hd_context;

void hd_options_init(hd_options* opt);
const char* hd_status_string(hd_status s);
/* Library version string, e.g. "hd_gb300 1.0 sm_103a". */
const char* hd_version(void);

/* Creates a context on `device` (the reference hard-codes device 0,
 * forBench/HausdorffDistance.cuh:5).  opt may be NULL. */
hd_status hd_context_create(int device, const hd_options* opt, hd_context** out);
hd_status hd_context_destroy(hd_context* ctx);
/* Text of the last error seen by this context ("" if none). */
const char* hd_context_last_error(hd_context* ctx);
/* Kernel timings of the context's last pair computation (zeros unless the
 * context was created with record_timings = 1).  After a pipelined call on
 * split SMs: its packing and set-up on their SMs and its dilation on the
 * others (iterations -1), HD_ERR_NOT_READY until that dilation is done. */
hd_status hd_context_last_timings(hd_context* ctx, hd_timings* out);

/* Drop-in for HausdorffDistance::computeDistance (forBench/HausdorffDistance.cu:101):
 * host masks in, result out.  Host-to-device copies (or zero-copy reads) are
 * part of the call; the call returns when the result is on the host. */
hd_status hd_compute_u8(hd_context* ctx, const uint8_t* a, const uint8_t* b, int32_t W, int32_t H,
                        int32_t D, hd_metric metric, hd_result* out);

/* Same, with the masks already in device memory.  `stream` is a
 * cudaStream_t (NULL = the context's own stream).  Returns when the result is
 * on the host. */
hd_status hd_compute_u8_device(hd_context* ctx, const uint8_t* d_a, const uint8_t* d_b, int32_t W,
                               int32_t H, int32_t D, hd_metric metric, void* stream,
                               hd_result* out);

/* One pair of a batch. */
typedef struct hd_pair_desc {
    const uint8_t* a;
    const uint8_t* b;
    int32_t W, H, D;
    int32_t metric;      /* hd_metric */
    int32_t on_device;   /* 1: a and b are device pointers; 0: host pointers */
    int32_t reserved;
} hd_pair_desc;

/* Asynchronous form of hd_compute_u8_device; no counterpart in the reference
 * (whose calls block).  Enqueues the whole computation on `stream` (NULL =
 * the context's stream) and returns: the result is decoded on the device into
 * *d_out (DEVICE memory, sizeof(hd_result)), valid once the stream reaches
 * it; errors found on the device are in d_out->status, launch errors are
 * returned.  Back-to-back calls overlap the host's work with the device's.
 * The context's workspace is reused by every call, so all calls on one
 * context (synchronous ones included) must be ordered on one stream.
 * hd_context_last_timings is not updated. */
hd_status hd_compute_u8_device_async(hd_context* ctx, const uint8_t* d_a, const uint8_t* d_b, int32_t W,
                                     int32_t H, int32_t D, hd_metric metric, void* stream, hd_result* d_out);

/* Pipelined form of hd_compute_u8_device_async; no counterpart in the
 * reference.  The masks must be ready in `stream` order when the call is
 * made, as there.  The result of a call is complete once `stream` reaches a
 * later hd_pipeline_flush(ctx, stream) (any other call on the context also
 * waits for it first), so a pair's packing and set-up may run while the
 * previous pair still dilates: single pairs of up to 2^26 voxels on a GPU
 * whose SMs can be split (green contexts) run their packing and set-up on a
 * few SMs (56 on GB300) and their dilation on one of three groups of the
 * rest (32 SMs each), consecutive pairs side by side, with two workspaces per
 * group in turn.  A lone pair's dilation takes longer on its group than on
 * the whole GPU: for the latency of single pairs use the other entries.
 * `stream` is made to wait for the packing's reads of the masks (not for the
 * dilation), so work queued on it after the call may overwrite or free them.
 * Otherwise the call behaves like hd_compute_u8_device_async. */
hd_status hd_compute_u8_device_pipelined(hd_context* ctx, const uint8_t* d_a, const uint8_t* d_b, int32_t W,
                                         int32_t H, int32_t D, hd_metric metric, void* stream, hd_result* d_out);

/* Makes `stream` (NULL = the context's stream) wait for every pipelined call
 * made so far on the context; their results are complete once it gets
 * there. */
hd_status hd_pipeline_flush(hd_context* ctx, void* stream);

/* Asynchronous form of hd_compute_u8 (HOST masks); no counterpart in the
 * reference.  The masks are copied by DMA on the context's copy stream into
 * one of two device staging buffers, so the copy of one pair overlaps the
 * kernels of the previous one; the rest is as hd_compute_u8_device_async
 * (result decoded into *d_out, device memory, when `stream` reaches it).
 * The host masks must stay unchanged until then; pinned memory makes the
 * copy asynchronous (pageable memory is copied before the call returns). */
hd_status hd_compute_u8_async(hd_context* ctx, const uint8_t* a, const uint8_t* b, int32_t W, int32_t H,
                              int32_t D, hd_metric metric, void* stream, hd_result* d_out);

/* Solves n pairs of independent shapes with one packing launch, one set-up
 * launch and ONE persistent dilation launch over a shared (pair, brick) work
 * queue.  Per-pair results are bit-identical to hd_compute_u8.  out[i].status
 * is the status of pair i; the return value is the first hard error.
 * This call, hd_profile_u8_device, hd_distance_map_device and hd_autotune run
 * on the context's own (non-blocking) stream: device masks must be complete
 * before the call (synchronise the stream that wrote them). */
hd_status hd_batch_compute(hd_context* ctx, const hd_pair_desc* pairs, int32_t n, hd_result* out);

/* Instrumented run (not for timing): also returns, per direction, the number
 * of origin-aligned 32x32x32 tiles that received newly dilated voxels at each
 * step k (tiles_ab[k]: dilation of B that covers A; tiles_ba[k]: dilation of
 * A that covers B), k = 0..len-1, and the number of bricks processed. */
hd_status hd_profile_u8_device(hd_context* ctx, const uint8_t* d_a, const uint8_t* d_b, int32_t W,
                               int32_t H, int32_t D, hd_metric metric, hd_result* out,
                               uint64_t* tiles_ab, uint64_t* tiles_ba, int32_t len,
                               uint64_t* bricks_processed);

/* Per-voxel distances (dense int32, -1 outside the other-mask-complement):
 * map_a[v] = d(v, B) for v in A \ B, map_b[v] = d(v, A) for v in B \ A, 0 on
 * A and B overlap, -1 elsewhere.  Device pointers, N = W*H*D int32 each.
 * Counterpart of the result lists of hello.cu:1588-1625 and the dense map of
 * hello.cu:2122-2170. */
hd_status hd_distance_map_device(hd_context* ctx, const uint8_t* d_a, const uint8_t* d_b, int32_t W,
                                 int32_t H, int32_t D, hd_metric metric, int32_t* d_map_a,
                                 int32_t* d_map_b, hd_result* out);

/* Autotuner (replaces the occupancy-API launch choice of hello.cu:1910-1954):
 * times every compiled brick shape and persistent-grid size on the given
 * pairs (one metric), then the queue schedule (pair order of a batch: as
 * given or largest first; queue items to warps: CTA-major or spread over the
 * SMs) on the three fastest; checks that every candidate gives identical
 * results (every field but `iterations`), keeps the fastest for this
 * workload class in the context and, when the context was created with
 * hd_options.tuning_table, writes the table there as JSON (a later context
 * created with that table uses it).  `repeats` timed runs per candidate
 * (median).  A human-readable report of the timings goes to `report` (may be
 * NULL). */
hd_status hd_autotune(hd_context* ctx, const hd_pair_desc* pairs, int32_t n, int32_t repeats,
                      char* report, size_t report_len);

/* ---- serving: continuous batching under a device-memory budget ---------- */
typedef struct hd_server hd_server;

typedef struct hd_server_options {
    uint64_t hbm_budget_bytes;   /* device bytes the server may hold; 0 = 120 GiB */
    int32_t max_inflight;        /* admitted pairs at once; 0 = unlimited (budget-bound) */
    int32_t max_queue;           /* waiting requests before submit returns HD_ERR_BUSY; 0 = 4096 */
    int32_t tick_iterations;     /* grid-barrier iterations per device tick at most; 0 = 64.  A tick
                                    also ends when every resident pair has finished, or at its next
                                    barrier once a request is submitted while it runs */
    int32_t metric;              /* hd_metric of every request of this server */
} hd_server_options;

void hd_server_options_init(hd_server_options* opt);
/* Starts a server with its own scheduler thread on ctx's device. */
hd_status hd_server_create(hd_context* ctx, const hd_server_options* opt, hd_server** out);
/* Queues a pair (host masks are copied in before submit returns unless
 * on_device; device masks must stay valid until the request completes). */
hd_status hd_server_submit(hd_server* srv, const hd_pair_desc* pair, uint64_t* ticket);
/* HD_ERR_NOT_READY while in flight; otherwise fills *out and forgets the ticket. */
hd_status hd_server_poll(hd_server* srv, uint64_t ticket, hd_result* out);
/* Blocks until the request finishes (timeout_ms < 0: no limit; else
 * HD_ERR_NOT_READY once timeout_ms have passed).  The waits poll (one atomic
 * count, not the server lock) for up to 1 ms (within the timeout) before they
 * sleep, and the scheduler thread polls for up to 2 ms for new requests
 * when it runs out of work: each costs a CPU core while it polls, and saves
 * a condition-variable wake-up (tens of microseconds) on a request's latency. */
hd_status hd_server_wait(hd_server* srv, uint64_t ticket, int64_t timeout_ms, hd_result* out);
/* Blocks until any request finishes (timeout_ms < 0: no limit) and returns
 * the earliest finished one not yet taken: its ticket and result (the
 * ticket is then forgotten).  HD_ERR_NOT_READY on timeout. */
hd_status hd_server_wait_any(hd_server* srv, int64_t timeout_ms, uint64_t* ticket, hd_result* out);
hd_status hd_server_cancel(hd_server* srv, uint64_t ticket);
/* Counters: submitted, completed, resident pairs, ticks, device bytes in use. */
typedef struct hd_server_stats {
    uint64_t submitted, completed, cancelled, ticks;
    uint64_t resident_pairs, waiting_pairs;
    uint64_t bytes_in_use, bytes_peak;
} hd_server_stats;
hd_status hd_server_get_stats(hd_server* srv, hd_server_stats* out);
hd_status hd_server_destroy(hd_server* srv);

/* ---- allocation-free variant ---------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory when they need a distance (all HBM handed to another allocator, a
 * loop that must not call cudaMalloc/cudaFree, which can block and
 * synchronise the device): hd_compute_u8_device with every intermediate buffer
 * inside one fixed 80 MiB device array of the library (each GPU that loads the
 * library holds it until exit).  No context, no allocation.  Masks and the
 * result are the caller's DEVICE memory; the call only enqueues work on
 * `stream` (cudaStream_t, NULL = legacy default stream) and *d_out is valid
 * once the stream reaches it.  d_out->hd_robust uses the 0.95 percentile.
 * Pairs whose buffers do not fit the array (about one byte per voxel;
 * 512 x 512 x 256 fits) return HD_ERR_BAD_ARG before any work is enqueued.
 * The first call on a device looks up the array's address with that device
 * current: make it before any stream capture.  All calls share the array and
 * it keeps the last call's contents (each call clears what must start at
 * zero); calls that overlap on the GPU race on it. */
hd_status hd_compute_u8_device_noalloc(const uint8_t* d_a, const uint8_t* d_b, int32_t W, int32_t H,
                                       int32_t D, hd_metric metric, void* stream, hd_result* d_out);

/* ---- HDF5 input (forBench/hdf5Manag.cu:44-86, loadHDFIntoBoolArr) -------- */
/* Reads a boolean dataset (read as HDF5's native boolean, narrowed to one
 * byte per element, nonzero = 1) into a malloc'd byte array; *n = elements.
 * Returns HD_ERR_UNSUPPORTED when the library was built without HDF5. */
hd_status hd_load_hdf5_bool(const char* path, const char* dataset, uint8_t** out, size_t* n);
/* The reference's host path for one pair (loadHDF -> loadHDFIntoBoolArr x 2
 * -> Volumes -> computeDistance, forBench/hdf5Manag.cu:196-214, 93-111):
 * loads two flat boolean datasets of W*H*D elements (x fastest) and computes
 * the pair with hd_compute_u8.  HD_ERR_BAD_ARG when a dataset is missing or
 * its size differs from W*H*D; HD_ERR_UNSUPPORTED without HDF5. */
hd_status hd_compute_hdf5(hd_context* ctx, const char* path_a, const char* dataset_a, const char* path_b,
                          const char* dataset_b, int32_t W, int32_t H, int32_t D, hd_metric metric, hd_result* out);
void hd_free(void* p);

#ifdef __cplusplus
}
#endif

#endif /* HD_HD_H */
