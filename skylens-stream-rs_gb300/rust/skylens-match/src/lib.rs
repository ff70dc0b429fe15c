//! Safe wrapper over libslm with the reference's signatures:
//!
//! * `ratio_match(a, b, ratio, mutual) -> Vec<(usize, usize)>`
//!   (skylens_core::matching::ratio_match, crates/core/src/matching.rs:167)
//! * `candidate_pairs(views, temporal, cross, pow2_max)` (matching.rs:18)
//! * `match_pairs(descs, pairs, ratio, mutual)`: the matching half of
//!   pipeline.rs:485-493 as one GPU batch.
//! * `detect_and_describe_rgb8(images, w, h, cfg)`: features of images of one
//!   size (features.rs:594 detect_and_describe after GrayImage::from_rgb).
//! * `build_tracks_drop(n_features, pairs, min_length, max_tracks)`: tracks of
//!   verified matches with ConflictPolicy::Drop (tracks.rs:190).
//! * `sampson_counts(pts, th, hyps)`: inlier counts of essential-matrix
//!   hypotheses over one pair's matches (two_view.rs:804-823, count_at_least),
//!   for a block of RANSAC iterations at once.
//!
//! The one deviation from the reference: it cannot fail on the CPU, this can
//! fail on the GPU; a non-OK status panics with libslm's message (there is no
//! CPU fallback). The process-wide context is thread-safe, so the function may
//! be called from rayon workers as the reference is.
use skylens_match_sys as sys;
use std::ffi::CStr;
use std::sync::OnceLock;

/// Anything that carries a 128-float descriptor (skylens_core's `Feature`
/// implements it with `fn desc(&self) -> &[f32; 128] { &self.desc }`).
pub trait Descriptor {
    fn desc(&self) -> &[f32; 128];
}

/// Which kernel family computes the distances (all give identical results).
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
pub enum Precision {
    Fp32,
    Bf16,
    Fp8,
    /// BF16 for large calls and batches, FP32 for small ones (libslm decides).
    Auto,
}

impl Precision {
    fn raw(self) -> sys::SlmPrecision {
        match self {
            Precision::Fp32 => sys::SLM_PREC_FP32,
            Precision::Bf16 => sys::SLM_PREC_BF16,
            Precision::Fp8 => sys::SLM_PREC_FP8,
            Precision::Auto => sys::SLM_PREC_AUTO,
        }
    }
}

struct Ctx(*mut sys::slm_ctx);
// libslm contexts are safe to share across threads (include/slm.h).
unsafe impl Send for Ctx {}
unsafe impl Sync for Ctx {}

fn check(st: sys::SlmStatus, what: &str) {
    if st != sys::SLM_OK {
        let msg = unsafe { CStr::from_ptr(sys::slm_last_error()) }.to_string_lossy().into_owned();
        let name = unsafe { CStr::from_ptr(sys::slm_status_str(st)) }.to_string_lossy().into_owned();
        panic!("{what}: {name}: {msg}");
    }
}

fn ctx() -> *mut sys::slm_ctx {
    static CTX: OnceLock<Ctx> = OnceLock::new();
    CTX.get_or_init(|| {
        let opts = sys::slm_opts { device: 0, stream: std::ptr::null_mut(), hbm_budget: 0 };
        let mut h = std::ptr::null_mut();
        check(unsafe { sys::slm_ctx_create(&opts, &mut h) }, "slm_ctx_create");
        Ctx(h)
    })
    .0
}

fn pack<D: Descriptor>(v: &[D]) -> Vec<f32> {
    let mut out = Vec::with_capacity(v.len() * 128);
    for d in v {
        out.extend_from_slice(d.desc());
    }
    out
}

/// Batch concurrent `ratio_match` calls of the process-wide context (rayon
/// workers calling it once per pair): up to `max_pairs` calls per batch, each
/// waiting at most `window_us` for company; `max_pairs = 0` turns it off.
/// Call it before the workers start. Results are unchanged (bit-exact).
pub fn set_coalescing(window_us: u32, max_pairs: u32) {
    check(unsafe { sys::slm_ctx_set_coalescing(ctx(), window_us, max_pairs) }, "slm_ctx_set_coalescing");
}

/// Drop-in for `skylens_core::matching::ratio_match` (exact; the BF16
/// shortlist for large pairs, the plain FP32 kernel for small ones).
pub fn ratio_match<D: Descriptor>(a: &[D], b: &[D], ratio: f32, mutual: bool) -> Vec<(usize, usize)> {
    ratio_match_with(a, b, ratio, mutual, Precision::Auto)
}

pub fn ratio_match_with<D: Descriptor>(a: &[D], b: &[D], ratio: f32, mutual: bool, p: Precision)
                                       -> Vec<(usize, usize)> {
    let (fa, fb) = (pack(a), pack(b));
    let mut out = vec![sys::slm_pair::default(); a.len().max(1)];
    let mut n = 0u32;
    check(
        unsafe {
            sys::slm_ratio_match(ctx(), fa.as_ptr(), a.len() as u32, fb.as_ptr(), b.len() as u32, ratio,
                                 mutual as i32, p.raw(), out.as_mut_ptr(), out.len() as u32, &mut n,
                                 std::ptr::null_mut())
        },
        "slm_ratio_match",
    );
    out.truncate(n as usize);
    out.into_iter().map(|p| (p.i as usize, p.j as usize)).collect()
}

/// `candidate_pairs` (matching.rs:18-40), computed by libslm's host code.
pub fn candidate_pairs(views: &[(usize, usize)], temporal: usize, cross: usize, pow2_max: usize)
                       -> Vec<(usize, usize)> {
    let flat: Vec<u64> = views.iter().flat_map(|&(c, p)| [c as u64, p as u64]).collect();
    let mut n = 0u64;
    let st = unsafe {
        sys::slm_candidate_pairs(flat.as_ptr(), views.len() as u32, temporal as u64, cross as u64,
                                 pow2_max as u64, std::ptr::null_mut(), 0, &mut n)
    };
    if st != sys::SLM_CAPACITY && st != sys::SLM_OK {
        check(st, "slm_candidate_pairs");
    }
    let mut out = vec![sys::slm_pair::default(); n as usize];
    check(
        unsafe {
            sys::slm_candidate_pairs(flat.as_ptr(), views.len() as u32, temporal as u64, cross as u64,
                                     pow2_max as u64, out.as_mut_ptr(), n, &mut n)
        },
        "slm_candidate_pairs",
    );
    out.into_iter().map(|p| (p.i as usize, p.j as usize)).collect()
}

/// The matching half of `pipeline::match_pairs` (pipeline.rs:485-493): every
/// pair's `ratio_match(fa, fb, ratio, mutual)` in one GPU batch. `views[v]` are
/// the features of view v; returns one match list per pair, in pair order.
pub fn match_pairs<D: Descriptor>(views: &[&[D]], pairs: &[(usize, usize)], ratio: f32, mutual: bool)
                                  -> Vec<Vec<(usize, usize)>> {
    let c = ctx();
    let total: usize = views.iter().map(|v| v.len()).sum();
    let mut store = std::ptr::null_mut();
    check(unsafe { sys::slm_store_create(c, total as u64, views.len() as u32, &mut store) }, "slm_store_create");
    let mut desc = Vec::with_capacity(total * 128);
    let (mut offsets, mut counts) = (Vec::new(), Vec::new());
    for v in views {
        offsets.push((desc.len() / 128) as u64);
        counts.push(v.len() as u32);
        desc.extend(pack(v));
    }
    let mut ids = vec![0u32; views.len()];
    check(
        unsafe {
            sys::slm_store_add_views(store, desc.as_ptr(), offsets.as_ptr(), counts.as_ptr(), views.len() as u32,
                                     ids.as_mut_ptr())
        },
        "slm_store_add_views",
    );
    let raw: Vec<sys::slm_pair> =
        pairs.iter().map(|&(i, j)| sys::slm_pair { i: ids[i], j: ids[j] }).collect();
    let cap: usize = pairs.iter().map(|&(i, _)| views[i].len()).sum::<usize>().max(1);
    let mut out = vec![sys::slm_pair::default(); cap];
    let mut off = vec![0u64; pairs.len() + 1];
    let st = unsafe {
        sys::slm_match_batch(c, store, raw.as_ptr(), raw.len() as u32, ratio, mutual as i32, sys::SLM_PREC_AUTO,
                             out.as_mut_ptr(), cap as u64, off.as_mut_ptr(), std::ptr::null_mut())
    };
    unsafe { sys::slm_store_destroy(store) };
    check(st, "slm_match_batch");
    (0..pairs.len())
        .map(|k| out[off[k] as usize..off[k + 1] as usize].iter().map(|p| (p.i as usize, p.j as usize)).collect())
        .collect()
}

/// The matching half of `pipeline::match_pairs` with its own pair set and
/// filter (pipeline.rs:485-496): `scheduled_pairs(views,
/// &PairSchedule::default())`, `ratio_match(fa, fb, 0.8, true)` per pair on the
/// GPU, and the pairs with at least `min_matches` matches (20 in the pipeline),
/// in schedule order. `imgs[v]` are the features of view v, `views[v]` its
/// (camera, position).
pub fn match_scheduled_pairs<D: Descriptor>(imgs: &[&[D]], views: &[(usize, usize)], min_matches: u32)
                                            -> Vec<(usize, usize, Vec<(usize, usize)>)> {
    assert_eq!(imgs.len(), views.len(), "one feature list per view");
    let c = ctx();
    let total: usize = imgs.iter().map(|v| v.len()).sum();
    let mut store = std::ptr::null_mut();
    check(unsafe { sys::slm_store_create(c, total as u64, imgs.len() as u32, &mut store) }, "slm_store_create");
    let mut desc = Vec::with_capacity(total * 128);
    let (mut offsets, mut counts) = (Vec::new(), Vec::new());
    for v in imgs {
        offsets.push((desc.len() / 128) as u64);
        counts.push(v.len() as u32);
        desc.extend(pack(v));
    }
    check(
        unsafe {
            sys::slm_store_add_views(store, desc.as_ptr(), offsets.as_ptr(), counts.as_ptr(), imgs.len() as u32,
                                     std::ptr::null_mut())
        },
        "slm_store_add_views",
    );
    let flat: Vec<u64> = views.iter().flat_map(|&(c, p)| [c as u64, p as u64]).collect();
    let sch = unsafe { sys::slm_pair_schedule_default() };
    let mut np = 0u64;
    let st = unsafe {
        sys::slm_scheduled_pairs(flat.as_ptr(), views.len() as u32, &sch, std::ptr::null_mut(), 0, &mut np)
    };
    if st != sys::SLM_CAPACITY && st != sys::SLM_OK {
        unsafe { sys::slm_store_destroy(store) };
        check(st, "slm_scheduled_pairs");
    }
    let mut sched = vec![sys::slm_pair::default(); (np as usize).max(1)];
    check(
        unsafe {
            sys::slm_scheduled_pairs(flat.as_ptr(), views.len() as u32, &sch, sched.as_mut_ptr(), np, &mut np)
        },
        "slm_scheduled_pairs",
    );
    // a row matches at most once: the rows of every pair's first view bound the matches
    let cap = sched[..np as usize].iter().map(|p| imgs[p.i as usize].len()).sum::<usize>().max(1);
    let mut pairs_out = vec![sys::slm_pair::default(); (np as usize).max(1)];
    let mut off = vec![0u64; pairs_out.len() + 1];
    let mut out = vec![sys::slm_pair::default(); cap];
    let mut kept = 0u64;
    let st = unsafe {
        sys::slm_match_pairs(c, store, flat.as_ptr(), views.len() as u32, &sch, 0.8, 1,
                             sys::SLM_PREC_AUTO, min_matches, pairs_out.as_mut_ptr(), pairs_out.len() as u64,
                             &mut kept, out.as_mut_ptr(), cap as u64, off.as_mut_ptr(), std::ptr::null_mut())
    };
    unsafe { sys::slm_store_destroy(store) };
    check(st, "slm_match_pairs");
    (0..kept as usize)
        .map(|k| {
            let m = out[off[k] as usize..off[k + 1] as usize].iter().map(|p| (p.i as usize, p.j as usize)).collect();
            (pairs_out[k].i as usize, pairs_out[k].j as usize, m)
        })
        .collect()
}

/// Inlier counts of `hyps` (row-major 3x3 matrices, `Matrix3::new` order) over
/// one pair's matches `pts` (`[n1.x, n1.y, n2.x, n2.y]` in normalized
/// coordinates): `#{i : |sampson_residual(e, n1[i], n2[i])| < th}` for each, in
/// the reference's f64 order (two_view.rs:456-465, 804-823).
pub fn sampson_counts(pts: &[[f64; 4]], th: f64, hyps: &[[f64; 9]]) -> Vec<u32> {
    if hyps.is_empty() {
        return Vec::new();
    }
    let off = [0u64, pts.len() as u64];
    let hp = vec![0u32; hyps.len()];
    let mut counts = vec![0u32; hyps.len()];
    check(
        unsafe {
            sys::slm_sampson_score(ctx(), pts.as_ptr() as *const f64, off.as_ptr(), 1, &th,
                                   hyps.as_ptr() as *const f64, hp.as_ptr(), hyps.len() as u32,
                                   counts.as_mut_ptr(), std::ptr::null(), std::ptr::null_mut(), 0)
        },
        "slm_sampson_score",
    );
    counts
}

/// `DetectorConfig::default()` (features.rs:278-293) as libslm takes it.
pub fn detector_config_default() -> sys::slm_detector_config {
    let mut c = sys::slm_detector_config::default();
    unsafe { sys::slm_detector_config_default(&mut c) };
    c
}

/// `detect_and_describe(&GrayImage::from_rgb(w, h, rgb), cfg)` for several
/// images of one size in one GPU call (pipeline.rs:452-463 `load` does one
/// per image): per image, its keypoints and 128-float descriptors in the
/// reference's order.
pub fn detect_and_describe_rgb8(images: &[&[u8]], w: u32, h: u32, cfg: &sys::slm_detector_config)
                                -> Vec<(Vec<sys::slm_keypoint>, Vec<[f32; 128]>)> {
    let n = images.len();
    let px = w as usize * h as usize * 3;
    let mut rgb = Vec::with_capacity(n * px);
    for im in images {
        assert_eq!(im.len(), px, "image buffer is not w x h x 3 bytes");
        rgb.extend_from_slice(im);
    }
    let cap = n * cfg.max_features as usize;
    let mut kps = vec![sys::slm_keypoint::default(); cap.max(1)];
    let mut desc = vec![[0f32; 128]; cap.max(1)];
    let mut off = vec![0u64; n + 1];
    check(
        unsafe {
            sys::slm_detect_and_describe_rgb8(ctx(), rgb.as_ptr(), n as u32, w, h, cfg, kps.as_mut_ptr(),
                                              desc.as_mut_ptr() as *mut f32, cap as u64, off.as_mut_ptr())
        },
        "slm_detect_and_describe_rgb8",
    );
    (0..n)
        .map(|k| {
            let (a, b) = (off[k] as usize, off[k + 1] as usize);
            (kps[a..b].to_vec(), desc[a..b].to_vec())
        })
        .collect()
}

/// `build_tracks(pairs, keypoints, &TrackConfig { policy: ConflictPolicy::Drop,
/// min_length, max_tracks })` (tracks.rs:190) on the GPU: per track its
/// (image, feature) observations in ascending order (the caller attaches
/// `keypoints[image][feature]`), tracks in first-observation order, and the
/// counts. `pairs` holds (image_a, image_b, matches of (feature a, feature b)).
pub fn build_tracks_drop(n_features: &[usize], pairs: &[(usize, usize, Vec<(usize, usize)>)], min_length: usize,
                         max_tracks: usize) -> (Vec<Vec<(usize, usize)>>, sys::slm_track_stats) {
    let nf: Vec<u32> = n_features.iter().map(|&n| n as u32).collect();
    let mut pm = Vec::with_capacity(pairs.len());
    let mut flat: Vec<sys::slm_pair> = Vec::new();
    for (a, b, m) in pairs {
        pm.push(sys::slm_pair_matches { image_a: *a as u32, image_b: *b as u32, first: flat.len() as u64,
                                        count: m.len() as u64 });
        flat.extend(m.iter().map(|&(i, j)| sys::slm_pair { i: i as u32, j: j as u32 }));
    }
    let cap_t = flat.len().max(1);
    let cap_o = (2 * flat.len()).max(1);
    let mut toff = vec![0u64; cap_t + 1];
    let mut obs = vec![sys::slm_pair { i: 0, j: 0 }; cap_o];
    let (mut nt, mut no) = (0u64, 0u64);
    let mut st = sys::slm_track_stats::default();
    check(
        unsafe {
            sys::slm_build_tracks_drop(ctx(), nf.as_ptr(), nf.len() as u32, pm.as_ptr(), pm.len() as u32,
                                       flat.as_ptr(), min_length as u32, max_tracks as u64, toff.as_mut_ptr(),
                                       cap_t as u64, obs.as_mut_ptr(), cap_o as u64, &mut nt, &mut no, &mut st)
        },
        "slm_build_tracks_drop",
    );
    let tracks = (0..nt as usize)
        .map(|t| obs[toff[t] as usize..toff[t + 1] as usize].iter().map(|o| (o.i as usize, o.j as usize)).collect())
        .collect();
    (tracks, st)
}
