/*
 * tsgpu.h — C ABI of the GB300-native texture-synthesis hot loop.
 *
 * The entry points mirror the reference's Rust API for the synthesis path
 * (EmbarkStudios/texture-synthesis):
 *
 *   Session::builder() -> SessionBuilder setters -> build() -> Session::run()
 *   -> GeneratedImage
 *
 * so that a Rust (or any FFI) front end can keep that API and forward every
 * call here.  Images cross the boundary as already-decoded RGBA8 buffers
 * (row-major, 4 bytes per pixel, no padding); decoding files stays with the
 * caller.  The library copies every input buffer when it is passed, so the
 * caller may free it immediately.  All computation runs on one CUDA device:
 * there is no CPU fallback, and a missing or unusable device is reported as
 * TS_ERR_CUDA.
 *
 * Errors: every fallible call returns a ts_status.  Builder and session
 * objects keep a message for the last error (ts_builder_last_error,
 * ts_session_last_error).  No exception crosses the ABI.
 *
 * Threading: objects are independent and may be used from different host
 * threads, but one object must not be used by two threads at once.
 * ts_session_run blocks the calling thread and invokes the progress
 * callback on it.
 */
#ifndef TSGPU_H
#define TSGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  TS_ERR_INVALID_RANGE, TS_ERR_SIZE_MISMATCH,
 * TS_ERR_EXAMPLE_GUIDE_MISMATCH, TS_ERR_NO_EXAMPLES and
 * TS_ERR_MAPS_COUNT_MISMATCH mirror texture_synthesis::Error
 * (lib/src/errors.rs:37-57); TS_ERR_IMAGE stands for Error::Image (a buffer
 * whose size does not match its dimensions). */
/* A random candidate (ms.rs:549-599) draws (x, y) pairs until one lies in
 * its example's sample mask.  The reference draws without end; here the
 * GPU path and the CPU oracle both give up after this many pairs and report
 * TS_ERR_NO_VALID_SAMPLE.  A mask whose valid fraction is f runs out with
 * probability (1 - f)^TS_MAX_SAMPLE_DRAWS per candidate. */
#define TS_MAX_SAMPLE_DRAWS (1u << 22)

typedef enum ts_status {
  TS_OK = 0,
  TS_ERR_INVALID_RANGE = 1,
  TS_ERR_SIZE_MISMATCH = 2,
  TS_ERR_EXAMPLE_GUIDE_MISMATCH = 3,
  TS_ERR_NO_EXAMPLES = 4,
  TS_ERR_MAPS_COUNT_MISMATCH = 5,
  TS_ERR_IMAGE = 6,
  /* A feature of the reference that this library does not provide. */
  TS_ERR_UNSUPPORTED = 7,
  /* A sample mask with no usable texel, or one so sparse that
   * TS_MAX_SAMPLE_DRAWS draws of a random candidate all miss it: the
   * reference keeps drawing (ms.rs:562-574), forever when nothing is valid;
   * this library refuses it. */
  TS_ERR_NO_VALID_SAMPLE = 8,
  /* A map id beyond the non-ignored example list, where the reference
   * panics on an out-of-bounds index. */
  TS_ERR_INDEX = 9,
  TS_ERR_CUDA = 10,
  /* A call out of order: a consumed builder or session used again. */
  TS_ERR_STATE = 11,
  /* A parameter beyond this library's stated limits (ts_limits). */
  TS_ERR_LIMIT = 12,
  TS_ERR_OUT_OF_MEMORY = 13,
  TS_ERR_NULL = 14
} ts_status;

/* SampleMethod (lib.rs:458-484). */
typedef enum ts_sample_method {
  TS_SAMPLE_ALL = 0,
  TS_SAMPLE_IGNORE = 1,
  TS_SAMPLE_IMAGE = 2
} ts_sample_method;

/* ChannelMask (utils.rs:46-53). */
typedef enum ts_channel { TS_CHANNEL_R = 0, TS_CHANNEL_G = 1, TS_CHANNEL_B = 2, TS_CHANNEL_A = 3 } ts_channel;

typedef struct ts_builder ts_builder;
typedef struct ts_session ts_session;
typedef struct ts_generated ts_generated;

/* One example image with its optional guide and sample mask
 * (Example / ExampleBuilder, lib.rs:486-623).  guide == NULL means no guide;
 * mask is read when sample_method == TS_SAMPLE_IMAGE (its R channel != 0
 * marks texels that may be sampled, ms.rs:1544-1547). */
typedef struct ts_example_desc {
  const uint8_t *rgba;
  uint32_t width, height;
  const uint8_t *guide_rgba;
  uint32_t guide_width, guide_height;
  int32_t sample_method; /* ts_sample_method */
  const uint8_t *mask_rgba;
  uint32_t mask_width, mask_height;
} ts_example_desc;

/* Stated limits of this implementation. */
typedef struct ts_limits {
  uint32_t max_nearest_neighbors;    /* k */
  uint32_t max_random_sample_locations; /* m */
  uint32_t max_examples;
  uint32_t max_image_side;           /* example and output sides */
} ts_limits;

/* Progress, once per synthesis stage, on the thread that called run
 * (GeneratorProgress / ProgressUpdate, session.rs:527-558).  image points at
 * the current output RGBA8 (width*height*4) and stays valid only during the
 * call. */
typedef struct ts_progress {
  const uint8_t *image;
  uint32_t width, height;
  uint64_t total_current, total_total;
  uint64_t stage_current, stage_total;
} ts_progress;
typedef void (*ts_progress_fn)(const ts_progress *update, void *user);

/* Kernel kinds of a run, for per-kernel timings. */
enum {
  TS_KERNEL_RANDOM_CANDIDATES = 0,
  TS_KERNEL_KNN_WALK = 1,
  TS_KERNEL_KNN_EXHAUSTIVE = 2,
  TS_KERNEL_RESOLVE = 3,
  TS_KERNEL_COMMIT = 4,
  TS_KERNEL_LEVEL_SWITCH = 5,
  TS_KERNEL_MEAN = 6,
  /* Not a kernel: the main stream waiting for a chunk of neighbour lists
   * made ahead on the k-NN stream (plain path, power-of-two outputs);
   * its time is the main stream's stall. */
  TS_KERNEL_KNN_WAIT = 7,
  TS_KERNEL_KINDS = 8
};

/* Run statistics of a generated image. */
typedef struct ts_run_stats {
  uint64_t resolves;      /* work items resolved in the stage loop */
  uint64_t cost_evals;    /* candidate-cost evaluations (coherence + random candidates) */
  uint64_t batches;       /* batch steps */
  uint64_t stages;
  uint64_t kernel_launches;
  double gpu_ms;          /* device time of run (CUDA events) */
  double wall_ms;         /* host wall time of run */
  /* Filled when the builder enabled ts_builder_profile_kernels: launches
   * and summed device time (CUDA events around each launch) per kernel
   * kind, indexed by TS_KERNEL_*. */
  uint64_t kernel_count[8];
  double kernel_ms[8];
  /* Host time of run(): schedule planning, device allocation, enqueueing
   * uploads and launches, waiting for the device, converting the results. */
  double host_plan_ms, host_alloc_ms, host_enqueue_ms, host_wait_ms, host_finish_ms;
  /* Device time of the initial uploads and of reading the results back
   * (CUDA events; part of gpu_ms). */
  double upload_ms, readback_ms;
  /* Parts of host_enqueue_ms: waiting for the pick chain
   * (pick_random_unresolved, on its own host thread) to finish a stage, and
   * the rest (uploads, launches and stream-order calls, and the read-back
   * copies, which wait for the device). */
  double host_pick_ms, host_launch_ms;
  /* Chunks of batches whose neighbour lists were made ahead on a side
   * stream (power-of-two outputs with k > 0); 0 when every batch step made
   * its own. */
  uint64_t knn_chunks;
} ts_run_stats;

const char *ts_status_str(int status);
void ts_get_limits(ts_limits *out);

/* ImagePyramid::new(img, Some(levels)) (img_pyramid.rs:7-37) on the device:
 * max(levels, 1) RGBA8 images of width x height, coarsest first, each level
 * a Gaussian downscale by 2^i resized back up; the last is the image itself.
 * rgba and out_rgba are host buffers (out: max(levels,1)*width*height*4
 * bytes).  The session builds the same pyramids for its examples and
 * guides. */
int ts_image_pyramid(const uint8_t *rgba, uint32_t width, uint32_t height, uint32_t levels, uint8_t *out_rgba,
                     int32_t device);

/* transform_to_guide_map + match_histograms (utils.rs:101-183) on the
 * device: the automatic guide that build() makes for an example without a
 * guide when a target guide is loaded (lib.rs:575-582).  imageops::blur with
 * sigma 2, grayscale (0.2126 R + 0.7152 G + 0.0722 B, truncated), then the
 * luma histogram matched to channel 0 of the target guide.  out_rgba:
 * width*height*4 bytes of (v, v, v, 255). */
int ts_guide_map(const uint8_t *rgba, uint32_t width, uint32_t height, const uint8_t *target_rgba,
                 uint32_t target_width, uint32_t target_height, uint8_t *out_rgba, int32_t device);

/* ts_image_pyramid_noalloc: no counterpart in the reference.  The same
 * pyramid as ts_image_pyramid, byte for byte, for callers that cannot let a
 * library allocate device memory: an engine or renderer that hands its whole
 * device budget to its own allocator, a framework whose caching allocator
 * holds the device, or a frame loop where cudaMalloc/cudaFree would stall
 * the device.  This call allocates nothing and frees nothing.
 *
 * d_rgba (width*height*4 bytes) and d_out (max(levels,1)*width*height*4
 * bytes) are device buffers of the current device, owned by the caller;
 * they must not overlap.  The work is enqueued on `stream` (a cudaStream_t;
 * NULL is the legacy default stream) and the call returns without waiting
 * for it, so d_out is ready once the stream reaches that point.  It
 * enqueues only kernels, device-to-device copies and memsets: the filter
 * taps travel inside kernel parameters, so no copy from host memory makes
 * the call wait for earlier work on the stream.  No buffer needs to start
 * at zero.
 *
 * Intermediate images and filter taps live in one fixed device array of
 * the library (9.4 MiB, held on every device the library runs on until
 * the process exits).  Hence the limits: width*height <=
 * TS_NOALLOC_MAX_PIXELS, each side <= TS_NOALLOC_MAX_SIDE, levels <=
 * TS_NOALLOC_MAX_LEVELS; larger requests return TS_ERR_LIMIT before any
 * work is enqueued.  Because that array is shared, two calls on the same
 * device must not overlap on the device: issue them on one stream or order
 * them with events, or they race on the array and give wrong images.
 * The first call on a device looks up the array's device address (a
 * one-time set-up per device); make it before any stream capture.  That
 * address is kept for the life of the process, so resetting the device
 * (cudaDeviceReset) between calls is not supported.  If a CUDA error is
 * already pending in the calling thread when the call begins, the call
 * enqueues nothing, returns TS_ERR_CUDA and leaves that error in place.
 * Returns TS_OK, TS_ERR_NULL, TS_ERR_IMAGE (zero side), TS_ERR_LIMIT or
 * TS_ERR_CUDA. */
#define TS_NOALLOC_MAX_PIXELS (1024u * 1024u)
#define TS_NOALLOC_MAX_SIDE 4096u
#define TS_NOALLOC_MAX_LEVELS 16u
int ts_image_pyramid_noalloc(const uint8_t *d_rgba, uint32_t width, uint32_t height, uint32_t levels, uint8_t *d_out,
                             void *stream);

/* ts_measure_gather_peak: no counterpart in the reference; measurement only.
 * The rate at which the GPU serves the cost loop's loads (better_match,
 * ms.rs:1225-1288 reads k example texels per candidate), measured with
 * kernels that do nothing else, at full occupancy, on a table of
 * width x height 32-bit texels (plus a 12-texel border) that the call
 * allocates, fills and frees:
 *   patch_gbs   a pseudo-random centre per thread and the k offsets nearest
 *               the origin around it (the cost loop's access shape);
 *   random_gbs  independent pseudo-random texels.
 * Both count 4 bytes per load, are timed with four and with eight loads in
 * flight per thread (the faster is reported, its depth in *_ilp), and take
 * the best of `reps` timed launches (CUDA events) after one warm-up.
 * k <= 256, sides <= 16384. */
typedef struct ts_gather_peak {
  double patch_gbs, random_gbs;
  double table_bytes;
  uint32_t threads;
  float patch_ms, random_ms;
  int32_t patch_ilp, random_ilp;
} ts_gather_peak;
int ts_measure_gather_peak(int32_t device, uint32_t width, uint32_t height, uint32_t k, int32_t reps,
                           ts_gather_peak *out);

/* ---- SessionBuilder (session.rs:69-448) ---------------------------------- */

/* Session::builder(): a builder with the reference defaults (lib.rs:342-359):
 * k=50, m=50, cauchy 1.0, backtrack 0.5 x 5, output 500x500, alpha 0.8,
 * seed 0, no tiling, no random init. */
ts_builder *ts_builder_new(void);
void ts_builder_free(ts_builder *b);
const char *ts_builder_last_error(const ts_builder *b);

/* SessionBuilder::add_example (session.rs:98-101) */
int ts_builder_add_example(ts_builder *b, const ts_example_desc *ex);
/* SessionBuilder::inpaint_example (session.rs:147-159): mask R<255 marks the
 * pixels to synthesise; width x height is the output (and input) size. */
int ts_builder_inpaint_example(ts_builder *b, const uint8_t *mask_rgba, uint32_t mask_width, uint32_t mask_height,
                               const ts_example_desc *ex, uint32_t width, uint32_t height);
/* SessionBuilder::inpaint_example_channel (session.rs:177-190) */
int ts_builder_inpaint_example_channel(ts_builder *b, int32_t channel, const ts_example_desc *ex, uint32_t width,
                                       uint32_t height);
/* SessionBuilder::load_target_guide (session.rs:200-203) */
int ts_builder_load_target_guide(ts_builder *b, const uint8_t *rgba, uint32_t width, uint32_t height);
/* SessionBuilder::resize_input (session.rs:206-209) */
int ts_builder_resize_input(ts_builder *b, uint32_t width, uint32_t height);
/* SessionBuilder::seed (session.rs:216-219) */
int ts_builder_seed(ts_builder *b, uint64_t seed);
/* SessionBuilder::tiling_mode (session.rs:224-227) */
int ts_builder_tiling_mode(ts_builder *b, int32_t tiling);
/* SessionBuilder::nearest_neighbors (session.rs:234-237) */
int ts_builder_nearest_neighbors(ts_builder *b, uint32_t count);
/* SessionBuilder::random_sample_locations (session.rs:245-248) */
int ts_builder_random_sample_locations(ts_builder *b, uint64_t count);
/* SessionBuilder::random_init (session.rs:254-257) */
int ts_builder_random_init(ts_builder *b, uint64_t count);
/* SessionBuilder::cauchy_dispersion (session.rs:269-272) */
int ts_builder_cauchy_dispersion(ts_builder *b, float value);
/* SessionBuilder::guide_alpha (session.rs:284-287) */
int ts_builder_guide_alpha(ts_builder *b, float value);
/* SessionBuilder::backtrack_percent (session.rs:293-296) */
int ts_builder_backtrack_percent(ts_builder *b, float value);
/* SessionBuilder::backtrack_stages (session.rs:305-308) */
int ts_builder_backtrack_stages(ts_builder *b, uint32_t stages);
/* SessionBuilder::output_size (session.rs:313-316) */
int ts_builder_output_size(ts_builder *b, uint32_t width, uint32_t height);
/* SessionBuilder::max_thread_count (session.rs:329-332).  Validated as in the
 * reference (0 is an error); the GPU schedule does not depend on it. */
int ts_builder_max_thread_count(ts_builder *b, uint64_t count);

/* GB300-specific knobs (no reference counterpart).  batch_divisor sets the
 * batch-snapshot schedule: each batch step holds max(1, R / divisor) work
 * items, R being the resolved count when the batch starts (default 8);
 * 0 gives batches of one item, the reference's single-thread semantics.
 * max_batch caps a batch (0 = no cap). */
int ts_builder_batch_schedule(ts_builder *b, uint32_t batch_divisor, uint32_t max_batch);
/* Kernel forms of the resolve step, all with identical results: batches of
 * at most `full_max_batch` items score every candidate of an item with one
 * CTA (lowest latency); up to `team_max_batch` items, one CTA per item with
 * early exit; larger batches, one warp per item (highest throughput).
 * Defaults 2048 and 256. */
int ts_builder_resolve_team(ts_builder *b, uint32_t team_max_batch, uint32_t full_max_batch);
/* CUDA device ordinal (default 0). */
int ts_builder_device(ts_builder *b, int32_t device);
/* Time every kernel launch of run() with CUDA events (adds host overhead;
 * for measurement runs only). */
int ts_builder_profile_kernels(ts_builder *b, int32_t on);

/* SessionBuilder::build (session.rs:336-448).  Consumes the builder on
 * success and on failure (as the Rust method takes self); the builder must
 * still be freed with ts_builder_free, which is then the only valid call
 * besides ts_builder_last_error.  Validation mirrors
 * check_parameters_validity / check_images_validity (session.rs:450-524);
 * example pyramids are built on the device here. */
int ts_builder_build(ts_builder *b, ts_session **out);

/* ---- Session (session.rs:22-66) ------------------------------------------ */

/* Session::run: random init (if set), then the coarse-to-fine stage loop.
 * Consumes the session: afterwards only ts_session_free and
 * ts_session_last_error are valid.  progress may be NULL. */
int ts_session_run(ts_session *s, ts_progress_fn progress, void *user, ts_generated **out);
void ts_session_free(ts_session *s);
const char *ts_session_last_error(const ts_session *s);

/* ---- Batched form (no counterpart in the reference) ---------------------
 * Many independent sessions synthesised together.  Each session's result is
 * byte-identical to ts_session_run on it (the same batch schedule, the same
 * kernels' arithmetic); what changes is how the work reaches the GPU: every
 * batch step of every session becomes one segment of a shared launch per
 * phase (k-NN, mean, resolve, commit, ...), so one launch carries the step
 * of up to all sessions at once instead of one tiny launch per session. */
typedef struct ts_batch ts_batch;
typedef struct ts_batch_stats {
  uint64_t sessions;
  uint64_t steps;          /* global batch steps (the longest session's) */
  uint64_t launches;       /* kernel launches of the run */
  uint64_t output_pixels;  /* summed output sizes */
  uint64_t resolves, cost_evals;
  double gpu_ms;           /* device time of the run: uploads, launches, read-back */
  double wall_ms;
  double plan_ms;          /* host time spent planning the sessions' schedules */
  /* With ts_batch_profile on: launches and summed device time per phase
   * (level switch, random candidates, k-NN walk, exhaustive k-NN, mean,
   * resolve warp form, resolve team form, resolve full team form, commit). */
  uint64_t phase_launches[9];
  double phase_ms[9];
  /* Device time from the run's start until every session's initial state
   * is on the device, and from the last launch until the results are
   * read back (both part of gpu_ms). */
  double upload_ms, readback_ms;
} ts_batch_stats;
ts_batch *ts_batch_new(int32_t device);
void ts_batch_free(ts_batch *b);
const char *ts_batch_last_error(const ts_batch *b);
/* Hands a built session to the batch: the session is consumed (only
 * ts_session_free and ts_session_last_error remain valid on it) and is run
 * by the next ts_batch_run.  Its device must be the batch's. */
int ts_batch_add(ts_batch *b, ts_session *s);
uint64_t ts_batch_size(const ts_batch *b);
/* Launch the whole run as one CUDA graph (captured and instantiated by the
 * call) instead of stream launches; the results are the same. */
int ts_batch_use_graph(ts_batch *b, int32_t on);
/* Time every launch with CUDA events (stream launches only; adds a little
 * host time per launch). */
int ts_batch_profile(ts_batch *b, int32_t on);
/* Host threads that plan the sessions' schedules (default: the hardware
 * concurrency, at most 32; 1 plans on the calling thread). */
int ts_batch_plan_threads(ts_batch *b, uint32_t n);
/* Resolve kernel form per batch step from the step's items summed over all
 * sessions: one CTA per item up to team_max_items (every candidate scored
 * in full up to full_max_items), one warp per item above.  Defaults 2048
 * and 256; the results do not depend on them. */
int ts_batch_resolve_team(ts_batch *b, uint32_t team_max_items, uint32_t full_max_items);
/* Runs every added session; out[i] receives the result of the i-th added
 * session (free each with ts_generated_free).  The batch is then empty and
 * may take new sessions.  On failure no result is returned and the message
 * names the session. */
int ts_batch_run(ts_batch *b, ts_generated **out);
void ts_batch_stats_get(const ts_batch *b, ts_batch_stats *out);

/* ---- Served form (no counterpart in the reference) ----------------------
 * Continuous batching of requests.  A request is a built session, handed to
 * ts_server_submit (which plans its schedule on the calling thread).  A
 * driver thread admits queued requests into session slots while their
 * device memory fits the budget (a request that does not fit waits; one
 * that does not fit an empty server runs alone), then runs ticks: each tick
 * issues one batch step of every admitted request as shared launches, so a
 * request admitted while others run overlaps with them on the device from
 * its first step.  Results are byte-identical to ts_session_run on the same
 * session, alone or in any mix.  Device memory of finished requests is
 * returned in stream order, without waiting for the device. */
typedef struct ts_server ts_server;
typedef struct ts_request_times {
  double submit_ms, admit_ms, done_ms;  /* host clock, from the server's creation */
} ts_request_times;
typedef struct ts_server_stats {
  uint64_t submitted, admitted, completed, failed;
  uint64_t ticks, launches;
  uint64_t peak_active;   /* most requests on the device at once */
  uint64_t peak_bytes;    /* most budget charged at once */
  uint64_t budget_bytes;
  uint64_t output_pixels, cost_evals;
  /* host time of the driver thread, microseconds: enqueueing ticks (of
   * which the kernel launch calls take driver_launch_us), waiting for a ring
   * slot (the device running behind), waiting for pickers (the pick chains
   * running behind) */
  uint64_t driver_tick_us, driver_ring_wait_us, driver_pick_wait_us, driver_launch_us;
} ts_server_stats;
/* hbm_budget_bytes 0: half the device's free memory; max_active 0: 64
 * session slots.  NULL if the device cannot be used. */
ts_server *ts_server_new(int32_t device, uint64_t hbm_budget_bytes, uint32_t max_active);
/* Waits for every submitted request, then stops; results not collected
 * with ts_server_wait are freed. */
void ts_server_free(ts_server *s);
const char *ts_server_last_error(const ts_server *s);
/* As ts_batch_resolve_team, over the items of a tick. */
int ts_server_resolve_team(ts_server *s, uint32_t team_max_items, uint32_t full_max_items);
/* Consumes the session (only ts_session_free and ts_session_last_error
 * remain valid on it) and queues it; *ticket names the request. */
int ts_server_submit(ts_server *s, ts_session *session, uint64_t *ticket);
/* Blocks until the request is done; *out receives its result (free with
 * ts_generated_free), times its host timestamps (may be NULL).  A ticket
 * can be waited for once. */
int ts_server_wait(ts_server *s, uint64_t ticket, ts_generated **out, ts_request_times *times);
/* 1 when done, 0 while queued or running, -1 for an unknown ticket. */
int ts_server_done(ts_server *s, uint64_t ticket);
void ts_server_stats_get(ts_server *s, ts_server_stats *out);

/* ---- Autotuner (no counterpart in the reference) ------------------------
 * Each batch step's launch shape follows its item count: one warp per item
 * for large steps (throughput), one CTA of 128 threads per item with early
 * exit, or of 256 threads scoring every candidate, for small ones
 * (latency); on the plain path, the k-NN walk of a small step may also
 * build a bitmap window in shared memory.  The thresholds between these
 * never change a result, only the speed, which depends on the GPU, the
 * sizes, k and m.  The tuner runs the caller's own workload under candidate
 * thresholds, one threshold at a time starting from the defaults, and keeps
 * a candidate only when its median device time over `repeats` runs beats
 * the best so far by more than 1%. */
typedef struct ts_tuning {
  uint32_t team_max_items;         /* a CTA per item in steps of at most this many items */
  uint32_t team_full_max_items;    /* ... scoring every candidate up to this many */
  uint32_t walk_window_max_items;  /* plain path: walk steps up to this many items may build a window */
  uint32_t trials;                 /* runs the tuner made (0 for ts_tuning_default) */
  double gpu_ms;                   /* median device time of the workload with this setting */
  double default_gpu_ms;           /* the same with the defaults */
} ts_tuning;
/* The defaults: 2048, 256 and 4096 items. */
void ts_tuning_default(ts_tuning *out);
/* A fresh, configured builder for one run of the workload on each call; the
 * tuner builds it, runs it and frees it.  NULL ends the tuning with
 * TS_ERR_STATE. */
typedef ts_builder *(*ts_builder_factory)(void *user);
/* Tunes the plain path on the workload `make` describes. */
int ts_autotune_session(ts_builder_factory make, void *user, uint32_t repeats, ts_tuning *out);
/* Adds the sessions of one run of the workload to the (empty) batch; a
 * nonzero return ends the tuning with that status. */
typedef int (*ts_batch_filler)(ts_batch *b, void *user);
/* Tunes the batched form (the two team thresholds) on batches of `device`
 * filled by `fill`. */
int ts_autotune_batch(int32_t device, ts_batch_filler fill, void *user, uint32_t repeats, ts_tuning *out);
/* Apply a setting: to a builder's session (all three thresholds), to a
 * batch or a server (the team thresholds over a step's summed items). */
int ts_builder_tuning(ts_builder *b, const ts_tuning *t);
int ts_batch_tuning(ts_batch *b, const ts_tuning *t);
int ts_server_tuning(ts_server *s, const ts_tuning *t);

/* ---- GeneratedImage (lib.rs:378-455) ------------------------------------- */

void ts_generated_dims(const ts_generated *g, uint32_t *width, uint32_t *height);
/* The output image, width*height*4 bytes (GeneratedImage::into_image). */
int ts_generated_image(const ts_generated *g, uint8_t *out_rgba);
/* Source coordinate of every output pixel: width*height*3 u32 (x, y, map),
 * the buffer behind get_coordinate_transform (ms.rs:655-684). */
int ts_generated_coord_map(const ts_generated *g, uint32_t *out_xym);
/* Patch id and map id of every output pixel: width*height*2 u32
 * (ms.rs:605-636). */
int ts_generated_id_map(const ts_generated *g, uint32_t *out_pm);
/* Length of the resolved list, and the list itself (flat pixel index) with
 * the score recorded when each entry was first resolved (ms.rs:639-653). */
uint64_t ts_generated_resolved_count(const ts_generated *g);
int ts_generated_resolved(const ts_generated *g, uint32_t *out_flat, float *out_score);
void ts_generated_stats(const ts_generated *g, ts_run_stats *out);
/* One timed kernel launch of a profiled run (ts_builder_profile_kernels). */
typedef struct ts_launch_record {
  int32_t kind;         /* TS_KERNEL_* */
  int32_t stage;        /* p_stage (backtrack stage), -1 outside the stage loop */
  uint32_t batch_items; /* work items of the batch (stage items for per-stage kernels) */
  float ms;             /* device time between CUDA events around the launch */
} ts_launch_record;
/* Number of launch records, and the records themselves (`out` holds at
 * least that many). */
uint64_t ts_generated_launch_count(const ts_generated *g);
int ts_generated_launches(const ts_generated *g, ts_launch_record *out);
void ts_generated_free(ts_generated *g);

/* Debug maps (GeneratedImage::save_debug, lib.rs:404-419; ms.rs:604-653),
 * computed on the device: width*height*4 bytes each.  Patch-id and map-id
 * colours of every pixel (channels drawn from Pcg32 streams seeded by the
 * id), and the uncertainty map: (s, 255 - s, 0, 255) with
 * s = (min(score, 1) * 255) as u8 at every resolved pixel, 0 elsewhere. */
int ts_generated_debug_maps(const ts_generated *g, uint8_t *patch_id_rgba, uint8_t *map_id_rgba,
                            uint8_t *uncertainty_rgba, int32_t device);

/* ---- CoordinateTransform (lib.rs:162-325) -------------------------------- */
typedef struct ts_transform ts_transform;
/* A decoded RGBA8 image (row-major, 4 bytes per pixel). */
typedef struct ts_image_desc {
  const uint8_t *rgba;
  uint32_t width, height;
} ts_image_desc;
/* GeneratedImage::get_coordinate_transform: the source (x, y, map) of every
 * output pixel and the loaded size of every example. */
ts_transform *ts_generated_coord_transform(const ts_generated *g);
void ts_transform_free(ts_transform *t);
void ts_transform_dims(const ts_transform *t, uint32_t *width, uint32_t *height, uint32_t *n_maps);
int ts_transform_map_dims(const ts_transform *t, uint32_t index, uint32_t *width, uint32_t *height);
/* CoordinateTransform::write: u32 little-endian words {0x12340001, width,
 * height, n_maps}, n_maps (w, h) pairs, then width*height (x, y, map)
 * triples.  out == NULL: *written receives the size only; TS_ERR_LIMIT if
 * capacity is short. */
int ts_transform_write(const ts_transform *t, uint8_t *out, size_t capacity, size_t *written);
/* CoordinateTransform::read of that format (version 1); malformed or short
 * data gives TS_ERR_INVALID_RANGE. */
int ts_transform_read(const uint8_t *data, size_t len, ts_transform **out);
/* CoordinateTransform::apply on the device: source i is resized (Catmull-Rom,
 * as load_image) to original map i's size, then every output pixel takes
 * texel (x, y) of source `map`.  Sources beyond n_maps are ignored, fewer
 * give TS_ERR_MAPS_COUNT_MISMATCH; an entry outside its map (the reference
 * panics) gives TS_ERR_INDEX.  out_rgba: width*height*4 bytes. */
int ts_transform_apply(const ts_transform *t, const ts_image_desc *sources, uint32_t n_sources, uint8_t *out_rgba,
                       int32_t device);

#ifdef __cplusplus
}
#endif

#endif /* TSGPU_H */
