"""CPU: the oracle's restatement of build_tracks with ConflictPolicy::Drop
(oracle/tracks.c, crates/core/src/tracks.rs:190-259, 472-500, 786-799),
pinned by the reference's known-answer tests for that policy
(tracks.rs:1346-1552): a conflicting component dropped whole, invalid and
short matches excluded with their counts, the cap preferring long then wide
tracks, and the result independent of pair order, direction, match order and
duplicates."""
import numpy as np

import oracle as O


def test_conflicting_component_is_dropped():
    # tracks.rs:1346-1413 (the Drop half)
    kp = [3, 3, 3, 3]
    pairs = [(0, 1, [(0, 0), (2, 2)]), (1, 2, [(0, 0), (2, 2)]), (2, 0, [(0, 1)]), (2, 3, [(2, 2)])]
    t, st = O.build_tracks_drop(kp, pairs)
    assert st["conflicts"] == 1
    assert t == [[(0, 2), (1, 2), (2, 2), (3, 2)]]
    for tr in t:
        assert all(a[0] < b[0] for a, b in zip(tr, tr[1:]))


def test_short_and_invalid_matches_are_excluded():
    # tracks.rs:1414-1447
    kp = [2, 2, 2]
    pairs = [(0, 0, [(0, 1)]), (0, 1, [(5, 0), (0, 0)])]
    t, st = O.build_tracks_drop(kp, pairs, min_length=3)
    assert st["invalid_matches"] == 2 and st["too_short"] == 1 and t == []
    t, _ = O.build_tracks_drop(kp, pairs, min_length=2)
    assert len(t) == 1 and len(t[0]) == 2


def test_cap_prefers_long_then_wide_tracks():
    # tracks.rs:1489-1531, select_tracks through build_tracks: track k joins
    # feature k of its images
    spec = [([0, 1], 0), ([0, 1, 2], 1), ([0, 5], 2), ([3, 4, 5], 3), ([0, 1, 9], 4)]
    pairs = []
    for imgs, f in spec:
        for a, b in zip(imgs, imgs[1:]):
            pairs.append((a, b, [(f, f)]))
    kp = [5] * 10
    t, st = O.build_tracks_drop(kp, pairs, min_length=2, max_tracks=3)
    assert [tr[0][1] for tr in t] == [1, 4, 3] and st["truncated"] == 2
    t, _ = O.build_tracks_drop(kp, pairs, min_length=2, max_tracks=4)
    assert [tr[0][1] for tr in t] == [1, 2, 4, 3]


def random_graph(seed, n_images=12, n_feat=60, n_points=150, outliers=40):
    """Scene points seen by runs of images, matched pairwise with some pairs
    missing, plus random wrong matches (the reference's synthetic scenes are
    its test code)."""
    rng = np.random.default_rng(seed)
    nf = rng.integers(n_feat // 2, n_feat, n_images)
    obs = {}
    for p in range(n_points):
        first = int(rng.integers(0, n_images - 1))
        for i in range(first, min(n_images, first + int(rng.integers(2, 6)))):
            obs.setdefault(p, []).append((i, int(rng.integers(0, nf[i]))))
    by_pair = {}
    for p, lst in obs.items():
        for (ia, fa), (ib, fb) in zip(lst, lst[1:]):
            if rng.random() < 0.8:
                by_pair.setdefault((ia, ib), []).append((fa, fb))
    for _ in range(outliers):
        a, b = sorted(rng.choice(n_images, 2, replace=False))
        by_pair.setdefault((int(a), int(b)), []).append((int(rng.integers(0, nf[a])), int(rng.integers(0, nf[b]))))
    return [int(x) for x in nf], [(a, b, m) for (a, b), m in sorted(by_pair.items())]


def test_order_independent():
    # tracks.rs:1448-1488: reversed pair order, swapped directions, shuffled
    # matches and a duplicated pair give the same tracks and counts
    nf, pairs = random_graph(0)
    t0, st0 = O.build_tracks_drop(nf, pairs, min_length=2)
    rng = np.random.default_rng(9)
    alt = []
    for k, (a, b, m) in enumerate(reversed(pairs)):
        m = [m[i] for i in rng.permutation(len(m))]
        alt.append((b, a, [(y, x) for x, y in m]) if k % 2 == 0 else (a, b, m))
    alt.append(pairs[0])
    t1, st1 = O.build_tracks_drop(nf, alt, min_length=2)
    assert t0 == t1 and st0["conflicts"] == st1["conflicts"] and st0["tracks"] == st1["tracks"]
    assert len(t0) > 20 and st0["conflicts"] > 0
