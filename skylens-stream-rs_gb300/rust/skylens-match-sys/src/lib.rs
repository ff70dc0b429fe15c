//! Raw bindings of `include/slm.h`. Every function returns an `SlmStatus`;
//! see the header for the contract of each entry point.
#![allow(non_camel_case_types)]
use std::os::raw::{c_char, c_int, c_void};

pub type SlmStatus = c_int;
pub const SLM_OK: SlmStatus = 0;
pub const SLM_INVALID_ARG: SlmStatus = 1;
pub const SLM_CAPACITY: SlmStatus = 2;
pub const SLM_OOM: SlmStatus = 3;
pub const SLM_CUDA_ERROR: SlmStatus = 4;
pub const SLM_TIMEOUT: SlmStatus = 5;
pub const SLM_NO_DEVICE: SlmStatus = 6;
pub const SLM_INTERNAL: SlmStatus = 7;
pub const SLM_CANCELLED: SlmStatus = 8;

pub type SlmPrecision = c_int;
pub const SLM_PREC_FP32: SlmPrecision = 0;
pub const SLM_PREC_BF16: SlmPrecision = 1;
pub const SLM_PREC_FP8: SlmPrecision = 2;
/// BF16 from SLM_AUTO_BF16_DISTANCES distances (one call or batch), FP32 below.
pub const SLM_PREC_AUTO: SlmPrecision = 3;
pub const SLM_AUTO_BF16_DISTANCES: u64 = 8_000_000;

#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq, Eq)]
pub struct slm_pair {
    pub i: u32,
    pub j: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct slm_stats {
    pub pairs: u64,
    pub distances: u64,
    pub matches: u64,
    pub rows_recomputed: u64,
    pub cols_recomputed: u64,
    pub rows_rescored: u64,
    pub kernel_ms: f32,
    pub max_abs_err: f32,
    pub kernel_launches: u64,
    pub pass_ms: [f32; 2],
    pub pairs_routed: u64,
    pub pairs_rescued: u64,
    pub rows_rescued: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct slm_opts {
    pub device: c_int,
    pub stream: *mut c_void,
    pub hbm_budget: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct slm_pair_schedule {
    pub temporal: u64,
    pub pow2_max: u64,
    pub spec: c_int,
    pub range: u64,
    pub right_min: u64,
    pub left_min: u64,
    pub max: u64,
    pub step: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct slm_tune {
    pub items_per_sm: u32,
    pub shortlist_k: u32,
    pub use_graph: u32,
    pub variant: u32,
    pub row_tiles: u32,
    pub autotune: u32,
}

#[repr(C)]
pub struct slm_ctx {
    _private: [u8; 0],
}
#[repr(C)]
pub struct slm_store {
    _private: [u8; 0],
}
/// Keypoint (features.rs:296-304).
#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq)]
pub struct slm_keypoint {
    pub x: f32,
    pub y: f32,
    pub sigma: f32,
    pub response: f32,
    pub angle: f32,
}
/// PairMatches (tracks.rs:44-50): matches[first .. first + count) of a flat slm_pair array.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct slm_pair_matches {
    pub image_a: u32,
    pub image_b: u32,
    pub first: u64,
    pub count: u64,
}
/// TrackStats (tracks.rs:130-152) of ConflictPolicy::Drop.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq, Eq)]
pub struct slm_track_stats {
    pub edges: u64,
    pub invalid_matches: u64,
    pub conflicts: u64,
    pub too_short: u64,
    pub truncated: u64,
    pub tracks: u64,
}
/// DetectorConfig (features.rs:253-293).
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct slm_detector_config {
    pub octaves: u32,
    pub scales: u32,
    pub sigma0: f32,
    pub contrast: f32,
    pub edge_ratio: f32,
    pub max_features: u32,
    pub upscale_below: u32,
    pub upscale_fill: i32,
}
#[repr(C)]
pub struct slm_plan {
    _private: [u8; 0],
}

extern "C" {
    pub fn slm_status_str(s: SlmStatus) -> *const c_char;
    pub fn slm_last_error() -> *const c_char;
    pub fn slm_selftest_wait_timeout(ctx: *mut slm_ctx, polls: u32) -> SlmStatus;
    pub fn slm_ctx_set_coalescing(ctx: *mut slm_ctx, window_us: u32, max_pairs: u32) -> SlmStatus;
    pub fn slm_ctx_coalescing_stats(ctx: *mut slm_ctx, batches: *mut u64, calls: *mut u64,
                                    max_batch: *mut u64) -> SlmStatus;
    pub fn slm_ctx_create(opts: *const slm_opts, out: *mut *mut slm_ctx) -> SlmStatus;
    pub fn slm_ctx_destroy(ctx: *mut slm_ctx) -> SlmStatus;
    pub fn slm_ctx_stream(ctx: *mut slm_ctx) -> *mut c_void;
    pub fn slm_ctx_bytes_in_use(ctx: *mut slm_ctx) -> u64;
    pub fn slm_ratio_match(ctx: *mut slm_ctx, a: *const f32, na: u32, b: *const f32, nb: u32, ratio: f32,
                           mutual: c_int, prec: SlmPrecision, out: *mut slm_pair, cap: u32, n_out: *mut u32,
                           st: *mut slm_stats) -> SlmStatus;
    pub fn slm_ratio_match_device(ctx: *mut slm_ctx, d_a: *const f32, na: u32, d_b: *const f32, nb: u32,
                                  ratio: f32, mutual: c_int, prec: SlmPrecision, d_out: *mut slm_pair, cap: u32,
                                  d_count: *mut u32) -> SlmStatus;
    /// No counterpart in the reference: for callers that cannot allocate device
    /// memory; na, nb <= 4096, overlapping calls race (include/slm.h).
    pub fn slm_ratio_match_device_noalloc(d_a: *const f32, na: u32, d_b: *const f32, nb: u32, ratio: f32,
                                          mutual: c_int, d_out: *mut slm_pair, cap: u32, d_count: *mut u32,
                                          stream: *mut c_void) -> SlmStatus;
    pub fn slm_candidate_pairs(views: *const u64, nv: u32, temporal: u64, cross: u64, pow2_max: u64,
                               out: *mut slm_pair, cap: u64, n_out: *mut u64) -> SlmStatus;
    pub fn slm_pair_schedule_default() -> slm_pair_schedule;
    pub fn slm_pair_schedule_spec() -> slm_pair_schedule;
    pub fn slm_scheduled_pairs(views: *const u64, nv: u32, sch: *const slm_pair_schedule, out: *mut slm_pair,
                               cap: u64, n_out: *mut u64) -> SlmStatus;
    pub fn slm_store_create(ctx: *mut slm_ctx, max_descs: u64, max_views: u32, out: *mut *mut slm_store) -> SlmStatus;
    pub fn slm_store_destroy(st: *mut slm_store) -> SlmStatus;
    pub fn slm_store_add_view(st: *mut slm_store, desc: *const f32, n: u32, view_id: *mut u32) -> SlmStatus;
    pub fn slm_store_add_views(st: *mut slm_store, desc: *const f32, offsets: *const u64, counts: *const u32,
                               nviews: u32, ids: *mut u32) -> SlmStatus;
    pub fn slm_store_clear(st: *mut slm_store) -> SlmStatus;
    pub fn slm_store_num_views(st: *mut slm_store) -> u32;
    pub fn slm_plan_create(ctx: *mut slm_ctx, st: *mut slm_store, pairs: *const slm_pair, np: u32, ratio: f32,
                           mutual: c_int, prec: SlmPrecision, tune: *const slm_tune, out: *mut *mut slm_plan)
                           -> SlmStatus;
    pub fn slm_plan_destroy(p: *mut slm_plan) -> SlmStatus;
    pub fn slm_plan_launch(p: *mut slm_plan) -> SlmStatus;
    pub fn slm_plan_results(p: *mut slm_plan, out: *mut slm_pair, cap: u64, offsets: *mut u64, st: *mut slm_stats)
                            -> SlmStatus;
    pub fn slm_plan_bytes(p: *mut slm_plan) -> u64;
    pub fn slm_autotune(ctx: *mut slm_ctx, st: *mut slm_store, pairs: *const slm_pair, np: u32, ratio: f32,
                        mutual: c_int, prec: SlmPrecision, best: *mut slm_tune, best_ms: *mut f32) -> SlmStatus;
    pub fn slm_match_batch(ctx: *mut slm_ctx, st: *mut slm_store, pairs: *const slm_pair, np: u32, ratio: f32,
                           mutual: c_int, prec: SlmPrecision, out: *mut slm_pair, cap: u64, offsets: *mut u64,
                           stats: *mut slm_stats) -> SlmStatus;
    pub fn slm_plan_set_min_matches(p: *mut slm_plan, min_matches: u32) -> SlmStatus;
    pub fn slm_match_pairs(ctx: *mut slm_ctx, st: *mut slm_store, views: *const u64, nv: u32,
                           sch: *const slm_pair_schedule, ratio: f32, mutual: c_int, prec: SlmPrecision,
                           min_matches: u32, pairs_out: *mut slm_pair, pairs_cap: u64, n_pairs: *mut u64,
                           out: *mut slm_pair, cap: u64, offsets: *mut u64, stats: *mut slm_stats) -> SlmStatus;
    pub fn slm_sampson_score(ctx: *mut slm_ctx, pts: *const f64, pair_off: *const u64, np: u32, thresh: *const f64,
                             e: *const f64, hyp_pair: *const u32, nh: u32, counts: *mut u32, mask_off: *const u64,
                             masks: *mut u32, mask_words: u64) -> SlmStatus;
    pub fn slm_detector_config_default(cfg: *mut slm_detector_config);
    pub fn slm_detect_and_describe(ctx: *mut slm_ctx, imgs: *const f32, n: u32, w: u32, h: u32,
                                   cfg: *const slm_detector_config, kps: *mut slm_keypoint, desc: *mut f32,
                                   cap: u64, off: *mut u64) -> SlmStatus;
    pub fn slm_detect_and_describe_rgb8(ctx: *mut slm_ctx, rgb: *const u8, n: u32, w: u32, h: u32,
                                        cfg: *const slm_detector_config, kps: *mut slm_keypoint, desc: *mut f32,
                                        cap: u64, off: *mut u64) -> SlmStatus;
    pub fn slm_describe(ctx: *mut slm_ctx, img: *const f32, w: u32, h: u32, kps: *const slm_keypoint, n: u32,
                        desc: *mut f32) -> SlmStatus;
    pub fn slm_build_tracks_drop(ctx: *mut slm_ctx, n_features: *const u32, n_images: u32,
                                 pairs: *const slm_pair_matches, n_pairs: u32, matches: *const slm_pair,
                                 min_length: u32, max_tracks: u64, track_off: *mut u64, cap_tracks: u64,
                                 obs: *mut slm_pair, cap_obs: u64, n_tracks: *mut u64, n_obs: *mut u64,
                                 stats: *mut slm_track_stats) -> SlmStatus;
}
