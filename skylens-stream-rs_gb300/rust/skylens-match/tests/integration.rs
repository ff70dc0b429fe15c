//! Integration tests of the safe wrapper against a plain Rust statement of
//! the reference's rules (crates/core/src/matching.rs:144-215): the distance
//! in the reference's summation order (component 8i+k into lane k, lanes
//! summed 0..7), the row's best with the lowest j on ties and the second
//! smallest of the multiset, `d1 < (r*r)*d2`, and the cross-check against the
//! column's best (smallest distance, lowest i). Needs a GB300 and libslm
//! (SLM_LIB_DIR at build time, LD_LIBRARY_PATH at run time).
use skylens_match::{build_tracks_drop, candidate_pairs, detect_and_describe_rgb8, detector_config_default, match_pairs,
                    ratio_match, ratio_match_with, Descriptor, Precision};

struct Feat([f32; 128]);

impl Descriptor for Feat {
    fn desc(&self) -> &[f32; 128] {
        &self.0
    }
}

/// xorshift64*: a small seeded generator for test inputs.
struct Rng(u64);

impl Rng {
    fn next_f32(&mut self) -> f32 {
        self.0 ^= self.0 >> 12;
        self.0 ^= self.0 << 25;
        self.0 ^= self.0 >> 27;
        let x = self.0.wrapping_mul(0x2545_F491_4F6C_DD1D);
        ((x >> 40) as f32) / ((1u64 << 24) as f32)
    }
}

fn normalise(v: &mut [f32; 128]) {
    let n = v.iter().map(|x| x * x).sum::<f32>().sqrt();
    if n > 0.0 {
        v.iter_mut().for_each(|x| *x /= n);
    }
}

/// Unit descriptor, clipped at 0.2 and renormalised (features.rs:575-582).
fn sift_like(rng: &mut Rng) -> Feat {
    let mut v = [0f32; 128];
    v.iter_mut().for_each(|x| *x = rng.next_f32());
    normalise(&mut v);
    v.iter_mut().for_each(|x| *x = x.min(0.2));
    normalise(&mut v);
    Feat(v)
}

/// A copy of `f` with uniform noise of amplitude `amp`, renormalised the same way.
fn noisy(rng: &mut Rng, f: &Feat, amp: f32) -> Feat {
    let mut v = f.0;
    v.iter_mut().for_each(|x| *x = (*x + amp * (rng.next_f32() - 0.5)).max(0.0));
    normalise(&mut v);
    v.iter_mut().for_each(|x| *x = x.min(0.2));
    normalise(&mut v);
    Feat(v)
}

fn pair(na: usize, nb: usize, seed: u64) -> (Vec<Feat>, Vec<Feat>) {
    let mut rng = Rng(seed.wrapping_mul(0x9E37_79B9_7F4A_7C15) | 1);
    let b: Vec<Feat> = (0..nb).map(|_| sift_like(&mut rng)).collect();
    let a: Vec<Feat> = (0..na)
        .map(|i| if i % 2 == 0 && nb > 0 { noisy(&mut rng, &b[(i * 7) % nb], 0.05) } else { sift_like(&mut rng) })
        .collect();
    (a, b)
}

fn sq_dist(p: &[f32; 128], r: &[f32; 128]) -> f32 {
    let mut acc = [0f32; 8];
    for i in 0..16 {
        for k in 0..8 {
            let t = p[8 * i + k] - r[8 * i + k];
            acc[k] += t * t;
        }
    }
    let mut s = 0f32;
    for k in 0..8 {
        s += acc[k];
    }
    s
}

fn naive(a: &[Feat], b: &[Feat], ratio: f32, mutual: bool) -> Vec<(usize, usize)> {
    if a.is_empty() || b.len() < 2 {
        return vec![];
    }
    let d: Vec<Vec<f32>> = a.iter().map(|p| b.iter().map(|r| sq_dist(&p.0, &r.0)).collect()).collect();
    let mut out = vec![];
    for i in 0..a.len() {
        let (mut d1, mut d2, mut j1) = (f32::INFINITY, f32::INFINITY, usize::MAX);
        for j in 0..b.len() {
            let v = d[i][j];
            if v < d1 {
                d2 = d1;
                d1 = v;
                j1 = j;
            } else if v < d2 {
                d2 = v;
            }
        }
        if j1 == usize::MAX || !d2.is_finite() || d1 >= (ratio * ratio) * d2 {
            continue;
        }
        if mutual {
            let (mut cd, mut ci) = (f32::INFINITY, usize::MAX);
            for r in 0..a.len() {
                if d[r][j1] < cd {
                    cd = d[r][j1];
                    ci = r;
                }
            }
            if ci != i {
                continue;
            }
        }
        out.push((i, j1));
    }
    out
}

#[test]
fn ratio_match_equals_the_rules_for_every_precision() {
    let shapes = [(0, 5), (5, 0), (5, 1), (1, 2), (63, 64), (129, 257), (300, 700), (1000, 3)];
    for (s, &(na, nb)) in shapes.iter().enumerate() {
        let (a, b) = pair(na, nb, 100 + s as u64);
        for &mutual in &[true, false] {
            let want = naive(&a, &b, 0.8, mutual);
            assert_eq!(ratio_match(&a, &b, 0.8, mutual), want, "auto {na}x{nb} mutual={mutual}");
            for &p in &[Precision::Fp32, Precision::Bf16, Precision::Fp8] {
                assert_eq!(ratio_match_with(&a, &b, 0.8, mutual, p), want, "{p:?} {na}x{nb} mutual={mutual}");
            }
        }
    }
}

#[test]
fn ratio_match_from_many_threads() {
    let (a, b) = pair(400, 500, 7);
    let want = naive(&a, &b, 0.8, true);
    std::thread::scope(|sc| {
        for _ in 0..8 {
            sc.spawn(|| {
                for _ in 0..4 {
                    assert_eq!(ratio_match(&a, &b, 0.8, true), want);
                }
            });
        }
    });
}

#[test]
fn candidate_pairs_counts() {
    // 3 cameras x P positions: 48 P - 177 pairs (tests/perf_structure.rs:29-47)
    for p in [48usize, 80] {
        let views: Vec<(usize, usize)> = (0..p).flat_map(|pos| (0..3).map(move |c| (c, pos))).collect();
        assert_eq!(candidate_pairs(&views, 5, 4, 16).len(), 48 * p - 177);
    }
}

#[test]
fn match_pairs_equals_one_call_per_pair() {
    let feats: Vec<Vec<Feat>> = (0..6).map(|v| pair(200 + 37 * v, 0, v as u64).0).collect();
    // views that share descriptors: view v+1 holds noisy copies of half of view v
    let mut views: Vec<Vec<Feat>> = vec![];
    let mut rng = Rng(99);
    for (v, f) in feats.into_iter().enumerate() {
        if v == 0 {
            views.push(f);
            continue;
        }
        let prev = &views[v - 1];
        let mut cur: Vec<Feat> = prev.iter().step_by(2).map(|x| noisy(&mut rng, x, 0.05)).collect();
        cur.extend(f);
        views.push(cur);
    }
    let refs: Vec<&[Feat]> = views.iter().map(|v| v.as_slice()).collect();
    let pairs = vec![(0, 1), (1, 2), (0, 2), (3, 4), (4, 5), (2, 5), (5, 0)];
    let got = match_pairs(&refs, &pairs, 0.8, true);
    assert_eq!(got.len(), pairs.len());
    for (k, &(u, v)) in pairs.iter().enumerate() {
        assert_eq!(got[k], naive(&views[u], &views[v], 0.8, true), "pair ({u}, {v})");
    }
}

/// build_tracks with ConflictPolicy::Drop: the reference's known answers
/// (tracks.rs:1346-1447, the Drop half): the conflicting component dropped
/// whole, invalid and short matches counted.
#[test]
fn tracks_drop_known_answers() {
    let pairs = vec![
        (0, 1, vec![(0, 0), (2, 2)]),
        (1, 2, vec![(0, 0), (2, 2)]),
        (2, 0, vec![(0, 1)]),
        (2, 3, vec![(2, 2)]),
    ];
    let (t, st) = build_tracks_drop(&[3, 3, 3, 3], &pairs, 3, 100_000);
    assert_eq!(st.conflicts, 1);
    assert_eq!(t, vec![vec![(0, 2), (1, 2), (2, 2), (3, 2)]]);
    let pairs = vec![(0, 0, vec![(0, 1)]), (0, 1, vec![(5, 0), (0, 0)])];
    let (t, st) = build_tracks_drop(&[2, 2, 2], &pairs, 3, 100_000);
    assert_eq!((st.invalid_matches, st.too_short), (2, 1));
    assert!(t.is_empty());
}

/// detect_and_describe on a gaussian blob (features.rs:846-885): the
/// strongest keypoint at the blob's centre within 0.1 px, unit descriptors.
#[test]
fn detect_and_describe_finds_the_blob() {
    let (w, h) = (140u32, 120u32);
    let (cx, cy, s) = (61.3f32, 47.6f32, 4.0f32);
    let mut rgb = vec![0u8; (w * h * 3) as usize];
    for y in 0..h {
        for x in 0..w {
            let r2 = (x as f32 - cx).powi(2) + (y as f32 - cy).powi(2);
            let v = ((0.2 + 0.6 * (-r2 / (2.0 * s * s)).exp()) * 255.0).round() as u8;
            let o = ((y * w + x) * 3) as usize;
            rgb[o..o + 3].copy_from_slice(&[v, v, v]);
        }
    }
    let out = detect_and_describe_rgb8(&[&rgb], w, h, &detector_config_default());
    let (kps, descs) = &out[0];
    assert!(!kps.is_empty());
    assert!(((kps[0].x - cx).powi(2) + (kps[0].y - cy).powi(2)).sqrt() < 0.1);
    for d in descs {
        let n = d.iter().map(|v| v * v).sum::<f32>().sqrt();
        assert!((n - 1.0).abs() < 1e-4);
    }
}
