/*
 * velo_search.h -- C ABI of the GB300 (sm_103a) search-by-triplet VELO track
 * reconstruction.
 *
 * It replaces the OpenCL device layer of dcampora/cl_forward:
 * invokeParallelSearch (KernelInvoker.h:27-31, KernelInvoker.cpp:14-275) and
 * the kernel it launches, clSearchByTriplets (Kernel.cl:597-816).  The
 * reference's C++ entry points keep their signatures in
 * GpuPixelSearchByTriplet.h and are implemented on top of this ABI.
 *
 * Input: per event, one blob in the layout of setHPointersFromInput
 * (Tools.cpp:68-80):
 *     int32 S, H; int32 sensor_Zs[S], sensor_hitStarts[S], sensor_hitNums[S];
 *     uint32 hit_IDs[H]; float32 hit_Xs[H], hit_Ys[H], hit_Zs[H]
 * with each module's hits x-sorted (velo_sort_by_x applies the reference's
 * preorder_by_x, Tools.cpp:46-66).
 * Output: per event, velo_track records (bit-identical to the reference's
 * Track, KernelDefinitions.h:59-62) whose hits are event-local indices into
 * the x-sorted hit arrays.
 *
 * All entry points are plain C: pointers, sizes and status codes.  A context
 * owns one CUDA stream and its device buffers; use one context per host
 * thread.  Nothing here is re-entrant on the same context.
 */
#ifndef VELO_SEARCH_H
#define VELO_SEARCH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VELO_MAX_TRACK_SIZE 24      /* KernelDefinitions.h:16 */
#define VELO_MAX_TRACKS 3000        /* KernelDefinitions.h:15 */
#define VELO_TTF_MODULO 2000        /* KernelDefinitions.h:23 */
#define VELO_MAX_MODULES 255        /* this implementation's limit on S */
#define VELO_MAX_MODULE_HITS 16383  /* this implementation's limit on hits per module */

/* Track {uint hitsNum; uint hits[24];}: 100 bytes, KernelDefinitions.h:59-62 */
typedef struct velo_track {
  uint32_t hitsNum;
  uint32_t hits[VELO_MAX_TRACK_SIZE];
} velo_track;

/* Straight-line fit of one track: x = x0 + tx z, y = y0 + ty z (mm, z in mm),
 * least squares with equal hit weights; chi2_ndf uses the pixel weight
 * PARAM_W = 3966.94 / mm^2 (KernelDefinitions.h:25).  No counterpart in the
 * search kernel; it is the stage that follows it. */
typedef struct velo_track_fit {
  float x0, tx, y0, ty, chi2_ndf;
} velo_track_fit;

typedef enum velo_status {
  VELO_OK = 0,
  VELO_ERR_INVALID_ARGUMENT = -1,
  VELO_ERR_INVALID_EVENT = -2,     /* an event blob failed validation (see event status) */
  VELO_ERR_CAPACITY = -3,          /* caller's track buffer too small; counts are valid */
  VELO_ERR_CUDA = -4,              /* CUDA runtime error; see velo_last_error */
  VELO_ERR_TIMEOUT = -5,           /* reserved: no kernel here waits on a flag or a peer, so no
                                      entry point returns it today; kept so that the codes of
                                      the others stay fixed */
  VELO_ERR_NO_DEVICE = -6,
  VELO_ERR_OUT_OF_MEMORY = -7,
  VELO_ERR_NOT_STAGED = -8         /* velo_run/velo_fetch without staged input */
} velo_status;

/* Per-event status bits (event_status_out).  Bits 0x1, 0x2, 0x4 and 0x10 mark
 * events on which the reference itself has undefined or schedule-dependent
 * behaviour; results there are this implementation's (it never overruns). */
#define VELO_EVENT_RING_OVERFLOW 0x1u   /* > TTF_MODULO ring entries in flight (Kernel.cl:344,354,565) */
#define VELO_EVENT_TRACK_OVERFLOW 0x2u  /* a track needed a 25th hit (Kernel.cl:321) */
#define VELO_EVENT_MAX_TRACKS 0x4u      /* more than MAX_TRACKS tracks (Kernel.cl:336,810) */
#define VELO_EVENT_INVALID 0x8u         /* blob failed validation; no tracks */
#define VELO_EVENT_DEGENERATE 0x10u     /* an inf/NaN fit (two modules' hits at equal z) */
#define VELO_EVENT_LEARNED_FALLBACK 0x20u  /* learned seeding not trusted (too few doublets kept, or
                                              more hits than max_event_hits): plain method */

typedef enum velo_launch_mode {
  VELO_LAUNCH_PER_EVENT = 0,   /* one CTA per event (the reference's one work-group per event) */
  VELO_LAUNCH_PERSISTENT = 1   /* persistent CTAs pulling events, largest first, from a work queue */
} velo_launch_mode;

typedef struct velo_options {
  int32_t y_lanes;            /* reference local size dim 1 (1..16); its output uses 4 */
  int32_t threads_per_event;  /* 32, 64, 128, 256 or 512 */
  int32_t launch_mode;        /* velo_launch_mode */
  int32_t smem_hits;          /* largest event (hits) staged in shared memory; 0 = auto */
  int32_t narrow_windows;     /* 1: binary-search narrowing of x windows (decisions unchanged) */
  int32_t ctas_per_sm;        /* persistent mode: resident CTAs per SM; 0 = auto */
  int32_t use_graph;          /* 1: capture the launch sequence in a CUDA graph and replay it */
  int32_t register_ctas;      /* 4 or 5: kernel build whose registers fit that many 256-thread
                                 CTAs per SM (64 or 48 registers); 18: the 64-thread build with
                                 56 registers (18 CTAs per SM; threads_per_event <= 64 only);
                                 0 = 18 for <= 64 threads, else 5 */
  int32_t learned;            /* 1: seeding prunes doublets with the MLP set by velo_set_mlp
                                 (approximate; no counterpart in the reference) */
  int32_t pipeline_events;    /* velo_search / velo_search_packed: > 0 cuts a batch of more than
                                 twice this many events into parts of this size whose copies
                                 and searches overlap on two streams (same results); the
                                 context then holds no staged batch afterwards.  0 = off */
  int32_t host_direct;        /* velo_search_packed: 1 = when the event buffer and the track
                                 buffer are pinned host memory (cudaHostAlloc/cudaHostRegister,
                                 mapped), the kernel reads the events and writes the tracks in
                                 place over the host link instead of staging copies; other
                                 buffers are copied as usual.  velo_search and
                                 velo_sort_search: the same, and on a device with coherent
                                 access to pageable host memory (NVLink-C2C) the events are
                                 read from the caller's own buffers, unpacked (and with
                                 velo_sort_search sorted in device memory and written back).
                                 Results are identical; the context holds no staged batch
                                 afterwards.  0 = off */
  int32_t device_budget_mb;   /* velo_search / velo_search_packed: device memory one call may
                                 use; a batch that needs more (about 275 B per hit) is cut into
                                 pipelined parts that fit.  0 = half the free device memory */
  int32_t seed_lanes;         /* seeding: lanes given to one h0's h1 candidates, 8, 16 or 32 (a
                                 warp then seeds 32 / seed_lanes h0s at once); below 32 it must
                                 be a multiple of y_lanes.  The width of the seeding window a
                                 warp slides over an h0's h1 candidates (the reference's Y-lanes
                                 per h0, Kernel.cl:435-436, set how many work-items share one
                                 h0).  Results do not depend on it.  0 = automatic */
  int32_t learned_min_window; /* learned seeding: only doublets whose exact h2 window holds at
                                 least this many hits are scored; narrower ones are searched
                                 exactly (their search costs less than scoring).  0 = score all */
  int32_t reserved[2];
} velo_options;

typedef struct velo_stats {
  float kernel_ms;            /* device time of the last velo_run (CUDA events) */
  uint32_t launches;          /* kernels launched by the last velo_run */
  uint32_t n_events;
  uint64_t total_hits;
  uint64_t total_tracks;
  uint64_t input_bytes;       /* event blob bytes staged */
  uint64_t output_bytes;      /* 4 B count + 100 B per track */
  int32_t smem_bytes_per_cta;
  int32_t grid;
  int32_t block;
  int32_t events_in_global;   /* events too large for the shared-memory arena */
  float host_stage_ms;        /* host time of the last stage: checks, metadata, enqueueing copies */
  float host_launch_ms;       /* host time of the last velo_run: launch preparation and enqueueing */
  float host_fetch_ms;        /* host time of the last fetch after the search finished: result copies */
} velo_stats;

typedef struct velo_ctx velo_ctx;

/* Defaults: Y = 4, persistent CTAs of 64 threads, 50-hit shared-memory
 * tile, narrowing on, automatic register build, no graph, no pipelining, no
 * in-place host I/O, plain (not learned) seeding. */
void velo_default_options(velo_options* opts);
const char* velo_status_string(velo_status s);

/* Create a context on CUDA device `device`. */
velo_status velo_create(velo_ctx** ctx, int32_t device);
void velo_destroy(velo_ctx* ctx);
const char* velo_last_error(const velo_ctx* ctx);

/* Host-only helpers (no GPU needed). */
velo_status velo_validate_event(const uint8_t* blob, uint64_t size);
/* preorder_by_x (Tools.cpp:46-66) of one event, in place; same permutation
 * as the reference's quicksort, equal x values included. */
velo_status velo_sort_by_x(uint8_t* blob, uint64_t size);
/* Upper bound on the tracks n events can produce (sum of max(H, 1)). */
uint64_t velo_track_capacity(const uint8_t* const* events, const uint64_t* sizes, int32_t n_events);

/*
 * One call, host buffers in and out (replaces invokeParallelSearch).
 * Event e's tracks are tracks_out[first_out[e] .. first_out[e] + counts_out[e]).
 * track_capacity is the room in tracks_out; velo_track_capacity() is always
 * enough.  event_status_out gets the VELO_EVENT_* bits.
 */
velo_status velo_search(velo_ctx* ctx, const uint8_t* const* events, const uint64_t* sizes,
                        int32_t n_events, const velo_options* opts, velo_track* tracks_out,
                        uint64_t track_capacity, uint32_t* counts_out, uint64_t* first_out,
                        uint32_t* event_status_out);

/*
 * The standalone path of the reference in one call: sorts each module's hits
 * by x in the caller's event buffers, in place and with the reference's
 * permutation (preorder_by_x, Tools.cpp:46-66, which mutates its input the
 * same way; GpuPixelSearchByTriplet.cpp:19), then searches the sorted
 * events.  Outputs as for velo_search.  Each event buffer must be 4-byte
 * aligned.  With opts->host_direct on a device that reads and writes
 * pageable host memory coherently (cudaDevAttrPageableMemoryAccess and
 * ...UsesHostPageTables, as a Grace-coupled GPU over NVLink-C2C does), the
 * device copies each event from the caller's buffer into its own memory,
 * sorts and searches it there, writes the sorted hit arrays back into the
 * caller's buffer and the tracks into tracks_out in place; otherwise the
 * events are packed into pinned memory, sorted and searched there, and the
 * sorted bytes are copied back.
 * A batch larger than the device budget is refused (VELO_ERR_OUT_OF_MEMORY):
 * call with fewer events.  Events that fail validation are left unsorted.
 */
velo_status velo_sort_search(velo_ctx* ctx, uint8_t* const* events, const uint64_t* sizes, int32_t n_events,
                             const velo_options* opts, velo_track* tracks_out, uint64_t track_capacity,
                             uint32_t* counts_out, uint64_t* first_out, uint32_t* event_status_out);

/*
 * Streaming form, for a host that consumes events while the device is still
 * searching (it hides the host's per-event work behind the search).  It
 * needs a device that reads and writes pageable host memory coherently
 * (NVLink-C2C); elsewhere velo_search_begin returns VELO_ERR_INVALID_ARGUMENT
 * and nothing starts.  No counterpart in the reference, whose host waits for
 * the whole launch (KernelInvoker.cpp:197-206).
 *
 * velo_search_begin enqueues the search (with sort != 0 after the in-place
 * sort of velo_sort_search, events 4-byte aligned) and returns.  As each
 * event finishes, the device writes its tracks to tracks_out and then its
 * record results[e]; `ready` is written last, after a system-scope fence,
 * so a host thread that reads ready == 1 (with acquire ordering) may read
 * the record and the event's tracks.  tracks_out and results stay the
 * caller's and must not be touched by it before velo_search_end except to
 * read finished events; track_capacity must be at least
 * velo_track_capacity() of the batch.  velo_search_end waits for the
 * search (and the sort's write-back) and returns the per-event outputs and
 * the status of velo_search.  Until then every other call on the context
 * that stages, launches or fetches returns VELO_ERR_INVALID_ARGUMENT.
 */
typedef struct velo_event_result {
  uint64_t first;        /* first track of the event in tracks_out */
  uint32_t count;        /* its tracks */
  uint32_t status;       /* VELO_EVENT_* bits */
  uint32_t ready;        /* set to 1 by the device, last */
  uint32_t reserved[3];
} velo_event_result;
velo_status velo_search_begin(velo_ctx* ctx, uint8_t* const* events, const uint64_t* sizes, int32_t n_events,
                              const velo_options* opts, int32_t sort, velo_track* tracks_out,
                              uint64_t track_capacity, velo_event_result* results);
velo_status velo_search_end(velo_ctx* ctx, uint32_t* counts_out, uint64_t* first_out,
                            uint32_t* event_status_out);

/* Same as velo_search, for events already packed in one host buffer (event e
 * at buf + offsets[e], 4-byte aligned).  A pinned buffer is copied directly. */
velo_status velo_search_packed(velo_ctx* ctx, const uint8_t* buf, const uint64_t* offsets,
                               const uint64_t* sizes, int32_t n_events, const velo_options* opts,
                               velo_track* tracks_out, uint64_t track_capacity,
                               uint32_t* counts_out, uint64_t* first_out,
                               uint32_t* event_status_out);

/* Split form, for device-resident pipelines and timing:
 *   velo_stage  validates and copies the events into device memory;
 *   velo_run    launches the search on the staged events (asynchronous);
 *   velo_fetch  waits and copies the results of the last run to the host. */
velo_status velo_stage(velo_ctx* ctx, const uint8_t* buf, const uint64_t* offsets,
                       const uint64_t* sizes, int32_t n_events);
velo_status velo_run(velo_ctx* ctx, const velo_options* opts);
velo_status velo_fetch(velo_ctx* ctx, velo_track* tracks_out, uint64_t track_capacity,
                       uint32_t* counts_out, uint64_t* first_out, uint32_t* event_status_out);
velo_status velo_synchronize(velo_ctx* ctx);

/* preorder_by_x (Tools.cpp:46-66) on the device: sorts each module's hits of
 * the staged events by x, in place, with the same permutation as the
 * reference (equal x included).  Sort once per staged batch, before
 * velo_run; output hit indices then refer to the sorted order, which
 * velo_fetch_staged returns (the staged bytes, in the layout given to
 * velo_stage: event e at buf + offsets[e] - min(offsets)). */
velo_status velo_sort_staged(velo_ctx* ctx);

/* Fits every track of the last run (velo_run / velo_search) on the device and
 * copies the fits to fits_out, in the order of the tracks velo_fetch returns
 * (fits_out[first[e] + i] belongs to tracks_out[first[e] + i]). */
velo_status velo_fit_tracks(velo_ctx* ctx, velo_track_fit* fits_out, uint64_t capacity);
velo_status velo_fetch_staged(velo_ctx* ctx, uint8_t* buf, uint64_t size);
velo_status velo_get_stats(const velo_ctx* ctx, velo_stats* stats);

/* `iters` back-to-back velo_run calls on the staged events, timed with CUDA
 * events on the context's stream after `warmup` untimed runs.  Between timed
 * runs a buffer larger than L2 is rewritten when flush_l2 != 0.
 * ms_out receives the mean device milliseconds per run. */
velo_status velo_time_runs(velo_ctx* ctx, const velo_options* opts, int32_t warmup, int32_t iters,
                           int32_t flush_l2, float* ms_out);

/* Autotuner, in two stages on the staged events, every run with L2 flushed.
 * Stage 1 times a grid of launch configurations, `iters` runs each: threads
 * per event {64, 128, 256, 512} x shared-memory tile {auto, 50, 100, 200,
 * 300, 600, 900, 1200, 1600, 2400 hits} x register build {4, 5, 18} x launch
 * style {per event, persistent}, where the 18-CTA build is the 64-thread one
 * and only build 5 runs 512 threads (104 configurations).  Stage 2 takes the
 * three fastest and times each with seed_lanes 8, 16 and 32 (below 32 only
 * multiples of y_lanes) over max(4 iters, 12) runs.  best_out gets the
 * fastest median of stage 2, best_ms_out its milliseconds.  Every
 * configuration gives the same tracks; y_lanes and use_graph are taken from
 * `base`. */
velo_status velo_autotune(velo_ctx* ctx, const velo_options* base, int32_t iters,
                          velo_options* best_out, float* best_ms_out);

/*
 * Learned doublet pruning (no counterpart in the reference).  A 10 -> 32 -> 32
 * -> 2 ReLU MLP scores each (h0, h1) seed doublet before its h2 search: a
 * keep logit, and the half-width (mm) of the x window around the predicted h2
 * position.  Doublets whose logit is below keep_threshold are skipped; the
 * others search h2 only within half-width + window_margin (never wider than
 * the exact cut).  An event whose kept fraction of doublets falls below
 * min_keep_rate is re-searched by the plain method, and an event with more
 * than max_event_hits hits (outside the range the network was trained on;
 * 0 = no limit) is searched by the plain method from the start; both are
 * flagged VELO_EVENT_LEARNED_FALLBACK.  Parameters: W1[32][10] b1[32]
 * W2[32][32] b2[32] W3[2][32] b3[2], FP32 (inference rounds them to FP16).
 */
#define VELO_MLP_INPUTS 10
#define VELO_MLP_HIDDEN 32
#define VELO_MLP_OUTPUTS 2
#define VELO_MLP_PARAMS 1474
velo_status velo_set_mlp(velo_ctx* ctx, const float* weights, float keep_threshold, float window_margin,
                         float min_keep_rate, uint32_t max_event_hits);

/* Training data: runs the plain search on the staged events and records,
 * for one in `keep_one_in` of the doublets that reach the h2 search (hashed
 * on event, h0, h1), the VELO_MLP_INPUTS features the learned seeding sees
 * and {event, h0, h1}.  Up to `capacity` records; count_out gets how many
 * were produced (possibly more than capacity).  velo_fetch then returns the
 * tracks, from which labels follow. */
velo_status velo_dump_doublets(velo_ctx* ctx, const velo_options* opts, uint32_t keep_one_in,
                               float* features_out, uint32_t* ids_out, uint64_t capacity,
                               uint64_t* count_out);

/* MLP training and evaluation on the current CUDA device (hand-written
 * kernels; inputs are host arrays, n samples of VELO_MLP_INPUTS features,
 * labels in {0, 1}, width targets in mm).  velo_mlp_train runs `steps` Adam
 * steps on batches of `batch` samples drawn without replacement per epoch and
 * updates weights_inout; loss_per_step (optional) receives each step's mean
 * loss.  velo_mlp_grad gives the mean-loss gradient at `weights`;
 * velo_mlp_forward the n x 2 outputs. */
velo_status velo_mlp_train(const float* x, const float* label, const float* target, int64_t n, int32_t steps,
                           int32_t batch, float lr, uint64_t seed, float* weights_inout, float* loss_per_step);
velo_status velo_mlp_grad(const float* weights, const float* x, const float* label, const float* target,
                          int64_t n, float* grad_out, float* loss_out);
velo_status velo_mlp_forward(const float* weights, const float* x, int64_t n, float* out);

/* Pinned host memory (cudaHostAlloc), for callers without a CUDA runtime. */
velo_status velo_host_alloc(velo_ctx* ctx, uint64_t bytes, void** ptr);
velo_status velo_host_free(velo_ctx* ctx, void* ptr);

/* Number of streaming multiprocessors of the context's device. */
int32_t velo_device_sm_count(const velo_ctx* ctx);

/*
 * Search without any device allocation.  No counterpart in the reference: it
 * is for callers that cannot call cudaMalloc themselves -- code under a
 * framework that owns every device allocation, or a path that must keep a
 * fixed device footprint and may not allocate or free at run time.
 *
 * The caller passes device pointers: the packed events (event e at
 * d_input + d_offsets[e], d_sizes[e] bytes, 4-byte aligned, x-sorted), and the
 * result buffers (d_tracks_out with room for track_capacity tracks, and
 * n_events entries of d_counts / d_first / d_status, filled as velo_search
 * fills its host outputs).  The work is enqueued on `stream` (a cudaStream_t;
 * NULL = the legacy default stream) and the results are valid once it is
 * synchronised.  Y-lanes as in velo_options; narrowing is on.
 *
 * All other memory is one file-scope device array of about 20 MB per GPU,
 * held from library load to process exit.  Limits per call, rejected with
 * VELO_ERR_CAPACITY: n_events <= VELO_STATIC_MAX_EVENTS;
 * total_hits + n_events <= VELO_STATIC_MAX_HIT_ROWS (total_hits = the sum of
 * the events' hit counts); track_capacity >= total_hits + n_events;
 * max_event_hits (an upper bound on any event's hit count) small enough to
 * stage the event in shared memory: 10,676 hits.  Events that break
 * their declared bounds get VELO_EVENT_INVALID and no tracks.
 *
 * The first call on a device takes the array's device address (with that
 * device current), so make that first call before any stream capture.  The
 * address is kept for the life of the process and belongs to the device's
 * primary context, the one the CUDA runtime uses: call this entry point with
 * that context current, and not again after cudaDeviceReset on the device.
 * Every call reuses the same array: calls whose GPU work overlaps (other
 * streams, other host threads) race and must be serialised by the caller.
 */
#define VELO_STATIC_MAX_EVENTS 4096
#define VELO_STATIC_MAX_HIT_ROWS 131072
velo_status velo_search_device_static(const uint8_t* d_input, const uint64_t* d_offsets,
                                      const uint64_t* d_sizes, int32_t n_events, uint64_t total_hits,
                                      uint32_t max_event_hits, int32_t y_lanes,
                                      velo_track* d_tracks_out, uint64_t track_capacity,
                                      uint32_t* d_counts, uint64_t* d_first, uint32_t* d_status,
                                      void* stream);

#ifdef __cplusplus
}
#endif
#endif
