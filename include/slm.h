/*
 * slm.h — C ABI of libslm, the GB300 (sm_103a) descriptor matcher.
 *
 * libslm replaces the descriptor-matching hot path of skylens-stream-rs:
 *   ratio_match      crates/core/src/matching.rs:167  (all-pairs squared L2,
 *                    best/second-best per row, Lowe ratio, mutual check)
 *   candidate_pairs  crates/core/src/matching.rs:18   (image-pair generator)
 *   scheduled_pairs  crates/core/src/matching.rs:103  (run's pair generator)
 *   match_pairs      crates/core/src/pipeline.rs:485  (per-pair loop that
 *                    calls ratio_match(fa, fb, 0.8, true) over the pairs)
 *
 * Conventions
 *   - Descriptors are row-major float32 arrays of n x 128 (Feature::desc,
 *     features.rs:499-502, marshalled contiguously by the caller).
 *   - A match is slm_pair {i, j}: row i of `a` matched to row j of `b`. Lists
 *     are in ascending i with each i at most once, exactly as ratio_match
 *     returns them; the results are bit-identical to the reference.
 *   - Every entry point returns an slm_status; no exception or abort crosses
 *     the ABI. On SLM_CAPACITY the required count is still written to the
 *     count output so the caller can grow its buffer and call again.
 *   - There is no CPU fallback: without a usable CUDA device calls return
 *     SLM_NO_DEVICE.
 *   - A context may be used from several host threads at once (the reference
 *     calls ratio_match from rayon workers, pipeline.rs:487-492, and from a
 *     second OS thread, pipeline.rs:2894-2918). Stores and plans are owned by
 *     one thread at a time.
 */
#ifndef SLM_H
#define SLM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SLM_DESC_LEN 128 /* features.rs:496 DESC_LEN */

typedef enum {
    SLM_OK = 0,
    SLM_INVALID_ARG = 1, /* NULL pointer, ratio not finite, bad view id, ... */
    SLM_CAPACITY = 2,    /* output buffer too small; required count reported */
    SLM_OOM = 3,         /* device allocation failed or HBM budget exceeded */
    SLM_CUDA_ERROR = 4,  /* a CUDA runtime call failed (see slm_last_error) */
    SLM_TIMEOUT = 5,     /* a bounded device-side wait gave up */
    SLM_NO_DEVICE = 6,   /* no CUDA device / device is not sm_103 */
    SLM_INTERNAL = 7,    /* invariant violated inside the library */
    SLM_CANCELLED = 8    /* a serving request withdrawn by slm_server_cancel */
} slm_status;

typedef enum {
    SLM_PREC_FP32 = 0, /* plain exact FP32 kernel */
    SLM_PREC_BF16 = 1, /* tcgen05 BF16 shortlist + exact FP32 rescore */
    SLM_PREC_FP8 = 2,  /* tcgen05 FP8 E4M3 shortlist + exact FP32 rescore */
    SLM_PREC_AUTO = 3  /* BF16 from SLM_AUTO_BF16_DISTANCES distances up (one call or one
                          batch), FP32 below, where the shortlist's fixed cost dominates */
} slm_precision;

/* SLM_PREC_AUTO's switch point, measured on GB300 through slm_ratio_match from
 * host arrays: 2500 x 2500 descriptors FP32 0.18 ms / BF16 0.19 ms,
 * 3072 x 3072 0.21 / 0.20 ms, 4096 x 4096 0.31 / 0.22 ms. */
#define SLM_AUTO_BF16_DISTANCES 8000000ull

typedef struct {
    uint32_t i, j;
} slm_pair;

/* Counters of one call. All fields are filled by every matching entry point. */
typedef struct {
    uint64_t pairs;             /* image pairs matched */
    uint64_t distances;         /* sum over pairs of na*nb */
    uint64_t matches;           /* pairs written */
    uint64_t rows_recomputed;   /* shortlist rows settled by an exact scan (rows of routed pairs included) */
    uint64_t cols_recomputed;   /* columns settled by an exact scan (columns of routed pairs included) */
    uint64_t rows_rescored;     /* rows whose shortlist was rescored exactly */
    float kernel_ms;            /* device time of the main matching kernel, last launch */
    float max_abs_err;          /* max |approx - exact| seen on rescored pairs */
    uint64_t kernel_launches;   /* kernels one launch of the batch runs */
    float pass_ms[2];           /* BF16/FP8: tensor-core passes 1 and 2; FP32: [0] = exact kernel */
    uint64_t pairs_routed;      /* BF16/FP8: pairs whose error bound was too loose to certify
                                   their rows, matched whole by the exact FP32 kernel */
    uint64_t pairs_rescued;     /* FP8: pairs whose FP8 bound was too loose for their distances,
                                   settled by the BF16 shortlist passes instead */
    uint64_t rows_rescued;      /* FP8: rows of those pairs */
} slm_stats;

typedef struct slm_ctx slm_ctx;
typedef struct slm_store slm_store;
typedef struct slm_plan slm_plan;

typedef struct {
    int device;          /* CUDA device ordinal */
    void *stream;        /* cudaStream_t for all work; NULL: the context creates one */
    uint64_t hbm_budget; /* bytes the context may allocate; 0 = free HBM at creation */
} slm_opts;

/* ------------------------------------------------------------ context */

const char *slm_status_str(slm_status s);
/* Detail of the last failing call on this host thread ("" if none). */
const char *slm_last_error(void);
slm_status slm_ctx_create(const slm_opts *opts, slm_ctx **out);
slm_status slm_ctx_destroy(slm_ctx *ctx);
/* The cudaStream_t the context launches on. */
void *slm_ctx_stream(slm_ctx *ctx);
/* Bytes currently allocated by the context and its stores/plans. */
uint64_t slm_ctx_bytes_in_use(slm_ctx *ctx);
/* Coalescing of concurrent single-pair calls (no reference counterpart: the
 * reference's rayon workers call ratio_match once per pair, matching.rs:167
 * from pipeline.rs:487-493). With max_pairs > 0, slm_ratio_match calls made
 * with SLM_PREC_AUTO from any thread are queued; a worker thread matches up to
 * max_pairs of them (same ratio and cross-check) in one batch once the batch
 * is full or its oldest call has waited window_us, while a second batch
 * gathers, and returns each caller its own list (bit-identical to the call
 * made alone). max_pairs = 0 turns it off. Not to be called while other
 * threads call slm_ratio_match on the context; max_pairs <= 4096,
 * window_us <= 1000000. */
slm_status slm_ctx_set_coalescing(slm_ctx *ctx, uint32_t window_us, uint32_t max_pairs);
/* Counters of the coalescer since it was set: batches run, calls matched in
 * them, the largest batch (calls). All 0 while coalescing is off. */
slm_status slm_ctx_coalescing_stats(slm_ctx *ctx, uint64_t *batches, uint64_t *calls, uint64_t *max_batch);
/* Self-test of the bounded device waits (no reference counterpart): one GPU
 * thread waits on a barrier that nothing completes and gives up after `polls`
 * polls (1..65536). Returns SLM_TIMEOUT, the status every timed-out kernel
 * wait reports, with the context still usable; anything else is a failure. */
slm_status slm_selftest_wait_timeout(slm_ctx *ctx, uint32_t polls);

/* ------------------------------------------------------ single pair */

/* Drop-in for ratio_match(a, b, ratio, mutual) (matching.rs:167-215).
 * a: na x 128 float32, b: nb x 128 float32 in host memory. Writes the match
 * list to out (capacity cap pairs; na pairs always suffice) and its length to
 * *n_out. Empty a or b, or nb < 2, gives an empty list (matching.rs:160-166).
 * Blocks until the result is in host memory. st may be NULL. */
slm_status slm_ratio_match(slm_ctx *ctx, const float *a, uint32_t na, const float *b, uint32_t nb, float ratio,
                           int mutual, slm_precision prec, slm_pair *out, uint32_t cap, uint32_t *n_out,
                           slm_stats *st);

/* The same on device memory: d_a, d_b, d_out (cap pairs) and d_count (one
 * uint32) are device pointers; work is enqueued on the context stream and the
 * call returns without synchronising. */
slm_status slm_ratio_match_device(slm_ctx *ctx, const float *d_a, uint32_t na, const float *d_b, uint32_t nb,
                                  float ratio, int mutual, slm_precision prec, slm_pair *d_out, uint32_t cap,
                                  uint32_t *d_count);

/* The same exact FP32 match without any device allocation. No counterpart in
 * the reference. For callers that cannot call cudaMalloc: an application whose
 * framework owns all device memory through its own pool, or a latency-critical
 * loop where an allocation (which may synchronise the device) would stall other
 * streams. No context is needed: work goes to `stream` (a cudaStream_t; NULL is
 * the legacy default stream) on the current device. Scratch comes from one
 * fixed device array inside the library (about 5 MiB, held by every device
 * that loads the library until exit), which limits na and nb to
 * SLM_NOALLOC_MAX_DESCS each; larger sizes return SLM_INVALID_ARG. d_a and d_b
 * must be 16-byte aligned. The first call on a device sets that device up
 * (make it before any stream capture). Calls share the array: calls that
 * overlap on the GPU race. *d_count receives the match count (0xffffffff if a
 * bounded device wait gave up; d_out's first cap pairs are then unspecified);
 * at most cap pairs are written to d_out, which needs only slm_pair's own
 * 4-byte alignment. */
#define SLM_NOALLOC_MAX_DESCS 4096
slm_status slm_ratio_match_device_noalloc(const float *d_a, uint32_t na, const float *d_b, uint32_t nb, float ratio,
                                          int mutual, slm_pair *d_out, uint32_t cap, uint32_t *d_count,
                                          void *stream);

/* ---------------------------------------------------- pair generators */

/* candidate_pairs (matching.rs:18-40). views: 2*nv uint64 (camera, position).
 * Writes up to cap pairs (view indices i < j, sorted) and the total to *n_out;
 * SLM_CAPACITY when the total exceeds cap. Host-only, no device needed. */
slm_status slm_candidate_pairs(const uint64_t *views, uint32_t nv, uint64_t temporal, uint64_t cross,
                               uint64_t pow2_max, slm_pair *out, uint64_t cap, uint64_t *n_out);

/* CrossSchedule (matching.rs:48-71) and PairSchedule (:74-101). */
typedef struct {
    uint64_t temporal; /* PAIR_TEMPORAL = 5 */
    uint64_t pow2_max; /* PAIR_POW2_MAX = 16 */
    int spec;          /* 1: CrossSchedule::Spec{range}; 0: Formation */
    uint64_t range;    /* Spec: cross-camera position gap 0..=range */
    uint64_t right_min, left_min, max, step; /* Formation (FORMATION = 20, 20, 40, 4) */
} slm_pair_schedule;

/* PairSchedule::default() (matching.rs:82-90) / PairSchedule::spec() (:94-100). */
slm_pair_schedule slm_pair_schedule_default(void);
slm_pair_schedule slm_pair_schedule_spec(void);

/* scheduled_pairs (matching.rs:103-142). Same output contract as
 * slm_candidate_pairs. */
slm_status slm_scheduled_pairs(const uint64_t *views, uint32_t nv, const slm_pair_schedule *sch, slm_pair *out,
                               uint64_t cap, uint64_t *n_out);

/* ------------------------------------------- device descriptor store */

/* A device-resident set of views (images). Capacity is fixed at creation. */
slm_status slm_store_create(slm_ctx *ctx, uint64_t max_descs, uint32_t max_views, slm_store **out);
slm_status slm_store_destroy(slm_store *st);
/* Append one view: copies n x 128 host floats to the device and lays them out
 * for the kernels (asynchronous on the context stream; desc must stay valid
 * until the next synchronising call). Returns its id in *view_id. */
slm_status slm_store_add_view(slm_store *st, const float *desc, uint32_t n, uint32_t *view_id);
/* Append many views from one buffer: view v has counts[v] rows starting at
 * row offsets[v] of desc. ids[v] receives its id. desc may be pageable host
 * memory (one copy and a scatter kernel), pinned host memory or device memory
 * (one copy per view, copy engines only; up to 4096 views per call).
 * Asynchronous on the context stream like slm_store_add_view. */
slm_status slm_store_add_views(slm_store *st, const float *desc, const uint64_t *offsets, const uint32_t *counts,
                               uint32_t nviews, uint32_t *ids);
/* Forget every view (capacity is kept). */
slm_status slm_store_clear(slm_store *st);
uint32_t slm_store_num_views(slm_store *st);

/* ------------------------------------------------- batched matching */

/* Tuning knobs; zero fields take the autotuned or default values. */
typedef struct {
    uint32_t items_per_sm;  /* FP32: target work items per SM when splitting columns */
    uint32_t shortlist_k;   /* BF16/FP8: shortlist capacity, records of 4-column hit groups per
                               row, column range and column half, 1..32 (0: 16) */
    uint32_t use_graph;     /* 1: replay a captured CUDA graph (default), 2: plain launches */
    uint32_t variant;       /* FP32: 0 packed f32x2 arithmetic (default), 1 all
                               scalar; both IEEE, bit-exact.
                               BF16/FP8: 2 keeps the approximate distances of pair 0
                               for slm_plan_debug_dump (diagnostics) */
    uint32_t row_tiles;     /* BF16/FP8: 128-row a tiles per work item, 1 or 2 (0: 2) */
    uint32_t autotune;      /* 1: use the context's tuned setting for this batch shape
                               (slm_autotune), tuning it first if none is cached */
} slm_tune;

/* Time a grid of settings on this batch with CUDA events (FP32: items per SM
 * {2, 4, 8} x arithmetic variant; BF16/FP8: items per SM {2, 4, 8} x row tiles
 * per work item {1, 2} x shortlist_k {8, 12, 16}) and return the fastest in
 * *best (and its time in *best_ms). The result is cached in the context under
 * the batch's shape (precision, mean rows per pair, pair count), which plans
 * with slm_tune.autotune = 1 use. Launches the batch several times. */
slm_status slm_autotune(slm_ctx *ctx, slm_store *st, const slm_pair *pairs, uint32_t np, float ratio, int mutual,
                        slm_precision prec, slm_tune *best, float *best_ms);

/* Plan the matching of np image pairs (view-id pairs in `pairs`, the
 * match_pairs loop of pipeline.rs:485-493) on a store. The plan owns its
 * device scratch and a CUDA graph of the whole batch. */
slm_status slm_plan_create(slm_ctx *ctx, slm_store *st, const slm_pair *pairs, uint32_t np, float ratio,
                           int mutual, slm_precision prec, const slm_tune *tune, slm_plan **out);
slm_status slm_plan_destroy(slm_plan *p);
/* Enqueue one run of the plan on the context stream (no host sync). */
slm_status slm_plan_launch(slm_plan *p);
/* Wait for the last launch, then copy results to the host. Pair k's matches
 * are out[offsets[k] .. offsets[k+1]) (offsets has np+1 entries). On
 * SLM_CAPACITY offsets[np] holds the required capacity. st may be NULL. */
slm_status slm_plan_results(slm_plan *p, slm_pair *out, uint64_t cap, uint64_t *offsets, slm_stats *st);
/* Device-side results of the last launch: per-pair match counts (np uint32)
 * and the padded match slots (pair k at row offset slot_offsets[k]). */
slm_status slm_plan_device_results(slm_plan *p, const uint32_t **d_counts, const slm_pair **d_slots,
                                   const uint64_t **h_slot_offsets);
/* Diagnostics: the tensor-core distance estimates d~ of the plan's first
 * pair (na x nb floats, row-major) from its last launch. Only for plans made
 * with slm_tune.variant = 2 and precision BF16 or FP8. */
slm_status slm_plan_debug_dump(slm_plan *p, float *out, uint64_t cap);
/* Bytes of device scratch the plan holds. */
uint64_t slm_plan_bytes(slm_plan *p);

/* match_pairs' filter (pipeline.rs:494-496): pairs with fewer than
 * min_matches matches report none from the next launch on (their lists are
 * not gathered or copied). 0 or 1: no filter. */
slm_status slm_plan_set_min_matches(slm_plan *p, uint32_t min_matches);

/* The matching half of match_pairs (pipeline.rs:485-496) in one call:
 * scheduled_pairs(views, sch) (NULL: PairSchedule::default()), ratio_match of
 * every pair as one batch (store view i = views[i]), and the pairs with at
 * least min_matches matches, in schedule order: pair k of the result is
 * pairs_out[k] and its matches are out[offsets[k] .. offsets[k+1]) (offsets
 * has pairs_cap + 1 entries). SLM_CAPACITY when more than pairs_cap pairs are
 * kept (*n_pairs = the count needed) or out has fewer than offsets[*n_pairs]
 * entries. */
slm_status slm_match_pairs(slm_ctx *ctx, slm_store *st, const uint64_t *views, uint32_t nv,
                           const slm_pair_schedule *sch, float ratio, int mutual, slm_precision prec,
                           uint32_t min_matches, slm_pair *pairs_out, uint64_t pairs_cap, uint64_t *n_pairs,
                           slm_pair *out, uint64_t cap, uint64_t *offsets, slm_stats *stats);

/* ------------------------------------------ RANSAC hypothesis scoring */

/* Sampson scoring of essential-matrix hypotheses, batched over image pairs:
 * the per-hypothesis work of the RANSAC stage that runs on every pair
 * match_pairs keeps (pipeline.rs:505 -> two_view.rs:774
 * ransac_essential_candidates_stats). Replaces, for each hypothesis,
 * count_at_least(e, need) and inliers_of(e) of ransac_essential_inner
 * (two_view.rs:804-823), built on sampson_residual (two_view.rs:456-465);
 * the caller keeps the sampling, the 5-point solver and the pool logic, and
 * count_at_least(e, need) is counts[h] >= need ? counts[h] : none.
 *   pts       the matches of all pairs, 4 doubles each: a.x, a.y, b.x, b.y
 *             (the normalized coordinates n1[i], n2[i]); pair p's matches are
 *             pts[pair_off[p] .. pair_off[p+1]), pair_off[0] = 0.
 *   thresh    per pair, the normalized threshold (threshold_px / focal_px).
 *   E         nh hypotheses, 9 doubles each, row-major (Matrix3::new order);
 *             hyp_pair[h] is hypothesis h's pair.
 *   counts    counts[h] = #{i : |residual| < thresh} (strict), in f64 with the
 *             reference's operation order: the counts and masks are its own.
 *   mask_off  optional (NULL: no masks): where mask_off[h] != UINT64_MAX, bit
 *             i % 32 of masks[mask_off[h] + i / 32] is match i's inlier flag
 *             (inliers_of); every other word of masks (mask_words words) is 0.
 * Blocks until the results are in host memory. */
slm_status slm_sampson_score(slm_ctx *ctx, const double *pts, const uint64_t *pair_off, uint32_t np,
                             const double *thresh, const double *E, const uint32_t *hyp_pair, uint32_t nh,
                             uint32_t *counts, const uint64_t *mask_off, uint32_t *masks, uint64_t mask_words);

/* One-shot: plan, launch, read back, destroy. */
slm_status slm_match_batch(slm_ctx *ctx, slm_store *st, const slm_pair *pairs, uint32_t np, float ratio,
                           int mutual, slm_precision prec, slm_pair *out, uint64_t cap, uint64_t *offsets,
                           slm_stats *stats);

/* ------------------------------------------------------------- serving */

/* A serving engine for views that stream in (a new zone filling up): each
 * submission adds one view to a device-resident store and asks for its
 * ratio_match against partners already submitted, as the pipeline's
 * match_pairs (pipeline.rs:485-493) does for a whole region. A worker thread
 * batches pending submissions every tick and admits a batch when one of
 * `slots` streams is free and the batch fits that slot's share of the HBM
 * budget; admitted batches run concurrently on their streams, so requests
 * that arrive while others are on the GPU start as soon as a slot frees.
 * A request's results do not depend on what it was batched with. */
typedef struct slm_server slm_server;

typedef struct {
    int device;
    uint64_t hbm_budget;      /* bytes for store + batches; 0: 80 % of free HBM */
    uint64_t max_descs;       /* store capacity (descriptors) */
    uint32_t max_views;       /* store capacity (views) */
    uint32_t slots;           /* concurrent batches (streams); 0: 3 */
    uint32_t max_batch_pairs; /* image pairs per batch; 0: 256 (batches of about 0.5 ms of BF16 work on
                                 views of ~1700 descriptors: under a backlog, batches pipeline over the
                                 slots instead of one large batch finishing last) */
    uint32_t tick_us;         /* batching tick; 0: 200 us */
    float ratio;              /* Lowe ratio (0.8 in the pipeline) */
    int mutual;
    slm_precision prec;
} slm_server_opts;

/* Placeholder for the submitted view itself in a submission's pair list. */
#define SLM_SELF 0xffffffffu

typedef struct {
    uint64_t submitted, completed, batches, pairs, matches;
    uint64_t max_batch_requests; /* most requests seen in one batch */
    uint64_t max_inflight;       /* most batches on the GPU at once */
    uint64_t bytes_in_use;
} slm_server_stats;

slm_status slm_server_create(const slm_server_opts *opts, slm_server **out);
/* Waits for work in flight, then frees everything. */
slm_status slm_server_destroy(slm_server *srv);
/* Queue one view (n x 128 floats, copied before returning) and the image
 * pairs to match once it is on the device: pairs[k] = (a, b) of view ids
 * where one side is SLM_SELF (this view) and the other an id returned by an
 * earlier submission. Returns the view's id and a ticket. */
slm_status slm_server_submit(slm_server *srv, const float *desc, uint32_t n, const slm_pair *pairs, uint32_t np,
                             uint32_t *view_id, uint64_t *ticket);
/* slm_server_submit without the copy (no reference counterpart: a client that
 * already holds the view's descriptors, e.g. the feature cache of
 * pipeline.rs:2614-2651, saves a host copy per request). desc is read where it
 * lies when the request is admitted (by the device directly where it can read
 * host memory and desc is 16-byte aligned, else by a copy); the caller keeps it
 * valid and unchanged until slm_server_wait returns for the ticket (also after
 * slm_server_cancel). */
slm_status slm_server_submit_ptr(slm_server *srv, const float *desc, uint32_t n, const slm_pair *pairs, uint32_t np,
                                 uint32_t *view_id, uint64_t *ticket);
/* Wait up to timeout_ms (0: poll) for a ticket. SLM_TIMEOUT if not done yet.
 * On completion copies pair k's matches to out[offsets[k] .. offsets[k+1])
 * (offsets has np+1 entries) and the request's latency (submit -> results on
 * the host) to *latency_ms; the ticket is then released. At most one thread
 * waits on a given ticket at a time. */
slm_status slm_server_wait(slm_server *srv, uint64_t ticket, uint32_t timeout_ms, slm_pair *out, uint64_t cap,
                           uint64_t *offsets, double *latency_ms);
slm_status slm_server_stats_get(slm_server *srv, slm_server_stats *st);
/* Withdraw a submitted request's matching. Not yet admitted: its pairs are
 * dropped (its view is still added to the store, so later submissions may
 * name it). Admitted (its batch on the GPU): the batch runs to completion and
 * the request's results are discarded. Already finished: its results are
 * discarded. slm_server_wait then returns SLM_CANCELLED for the ticket and
 * releases it; other requests are unaffected. */
slm_status slm_server_cancel(slm_server *srv, uint64_t ticket);

/* ------------------------------------------------ descriptor producer */

/* Keypoint (features.rs:296-304): input-image pixels, scale sigma, DoG
 * response, dominant orientation in radians [0, 2 pi). */
typedef struct {
    float x, y, sigma, response, angle;
} slm_keypoint;

/* DetectorConfig (features.rs:253-293). */
typedef struct {
    uint32_t octaves;       /* at most 16 */
    uint32_t scales;        /* intervals per octave s (DoG layers s + 2), 1..32 */
    float sigma0;
    float contrast;         /* minimum |DoG| (brightness in [0, 1]) */
    float edge_ratio;       /* principal curvature ratio bound r */
    uint32_t max_features;
    uint32_t upscale_below; /* 0: never detect on the 2x upsampled image */
    int32_t upscale_fill;
} slm_detector_config;

/* DetectorConfig::default() (features.rs:278-293). */
void slm_detector_config_default(slm_detector_config *cfg);

/* detect_and_describe (features.rs:594) for n gray images of w x h pixels
 * (row-major f32, GrayImage::data; host or device memory), run together on
 * the GPU: Gaussian pyramid, DoG extrema refined to sub-pixel and sub-scale,
 * contrast and edge tests, dominant orientations, 128-d descriptors, the
 * |response| order and max_features cut, and for images below upscale_below
 * that found too few features, the de-duplicated features of the 2x
 * upsampled image. Image k's features are kps[off[k] .. off[k+1]) and rows
 * off[k] .. off[k+1]) of desc (n_features x 128 floats; host or device
 * memory); off has n + 1 entries and is always written. SLM_CAPACITY when
 * off[n] > cap (nothing else is written). kps or desc may be NULL.
 * Arithmetic follows the reference's f32 operation order; its per-pixel and
 * per-keypoint exp, atan2, powf, cos and sin are evaluated correctly rounded,
 * where the reference calls the platform's float functions (equal wherever
 * those are correctly rounded). Images up to 32767 pixels a side. */
slm_status slm_detect_and_describe(slm_ctx *ctx, const float *imgs, uint32_t n, uint32_t w, uint32_t h,
                                   const slm_detector_config *cfg, slm_keypoint *kps, float *desc, uint64_t cap,
                                   uint64_t *off);
/* The same from interleaved 8-bit RGB images (n x h x w x 3 bytes), converted
 * on the device as GrayImage::from_rgb (features.rs:165-189) does. */
slm_status slm_detect_and_describe_rgb8(slm_ctx *ctx, const uint8_t *rgb, uint32_t n, uint32_t w, uint32_t h,
                                        const slm_detector_config *cfg, slm_keypoint *kps, float *desc,
                                        uint64_t cap, uint64_t *off);
/* describe(img, x, y, sigma, angle) (features.rs:509) for n keypoints of one
 * gray image (response ignored; 0 < sigma <= 64, |x|, |y| <= 1e6): desc is
 * n x 128 floats (host or device memory). */
slm_status slm_describe(slm_ctx *ctx, const float *img, uint32_t w, uint32_t h, const slm_keypoint *kps, uint32_t n,
                        float *desc);

/* ---------------------------------------------------------- tracks */

/* One image pair's verified matches (PairMatches, tracks.rs:44-50):
 * matches[first .. first + count) of a flat slm_pair array, i = feature of
 * image_a, j = feature of image_b. */
typedef struct {
    uint32_t image_a, image_b;
    uint64_t first, count;
} slm_pair_matches;

/* TrackStats (tracks.rs:130-152) of ConflictPolicy::Drop. */
typedef struct {
    uint64_t edges;           /* distinct (image, feature) edges */
    uint64_t invalid_matches; /* same-image pairs and out-of-range indices */
    uint64_t conflicts;       /* components dropped for holding two features of one image */
    uint64_t too_short;       /* components below min_length */
    uint64_t truncated;       /* tracks beyond max_tracks */
    uint64_t tracks;
} slm_track_stats;

/* build_tracks(pairs, keypoints, &TrackConfig { policy: ConflictPolicy::Drop,
 * min_length, max_tracks }) (tracks.rs:190): the connected components of the
 * verified matches over nodes (image, feature), n_features[i] features in
 * image i; a component holding two features of one image is dropped, one
 * shorter than max(min_length, 2) too; select_tracks (tracks.rs:786) keeps at
 * most max_tracks (longest, then widest image span, then first observation),
 * in first-observation order. Track t is obs[track_off[t] .. track_off[t+1])
 * (i = image, j = feature, ascending); track_off has cap_tracks + 1 entries.
 * SLM_CAPACITY when the tracks or observations do not fit (*n_tracks and
 * *n_obs give the sizes needed). The graph work (edge set, components) runs
 * on the GPU; the result is the reference's exactly (integer work). The
 * default policy, ConflictPolicy::Split, is not provided. */
slm_status slm_build_tracks_drop(slm_ctx *ctx, const uint32_t *n_features, uint32_t n_images,
                                 const slm_pair_matches *pairs, uint32_t n_pairs, const slm_pair *matches,
                                 uint32_t min_length, uint64_t max_tracks, uint64_t *track_off, uint64_t cap_tracks,
                                 slm_pair *obs, uint64_t cap_obs, uint64_t *n_tracks, uint64_t *n_obs,
                                 slm_track_stats *stats);

#ifdef __cplusplus
}
#endif
#endif /* SLM_H */
