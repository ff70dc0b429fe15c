"""GPU: slm_build_tracks_drop (build_tracks with ConflictPolicy::Drop,
crates/core/src/tracks.rs:190) against the oracle's restatement: the
reference's known-answer cases, seeded random graphs (wrong matches,
duplicates, swapped directions, invalid indices, caps), the 240-view zone's
match lists (1.7 M matches) and the argument checks. Integer work: tracks and
counts must be identical."""
import ctypes

import numpy as np
import pytest

import oracle as O
from skylens_match import synth
from skylens_match import tracks as T

pytestmark = pytest.mark.gpu


def both(matcher, nf, pairs, **kw):
    g = T.build_tracks_drop(matcher, nf, pairs, **kw)
    o = O.build_tracks_drop(nf, pairs, **kw)
    assert g[0] == o[0]
    assert g[1] == o[1]
    return g


def test_known_answers(matcher):
    t, st = both(matcher, [3, 3, 3, 3],
                 [(0, 1, [(0, 0), (2, 2)]), (1, 2, [(0, 0), (2, 2)]), (2, 0, [(0, 1)]), (2, 3, [(2, 2)])])
    assert st["conflicts"] == 1 and t == [[(0, 2), (1, 2), (2, 2), (3, 2)]]
    t, st = both(matcher, [2, 2, 2], [(0, 0, [(0, 1)]), (0, 1, [(5, 0), (0, 0)])], min_length=3)
    assert st["invalid_matches"] == 2 and st["too_short"] == 1 and t == []
    spec = [([0, 1], 0), ([0, 1, 2], 1), ([0, 5], 2), ([3, 4, 5], 3), ([0, 1, 9], 4)]
    pairs = [(a, b, [(f, f)]) for imgs, f in spec for a, b in zip(imgs, imgs[1:])]
    t, _ = both(matcher, [5] * 10, pairs, min_length=2, max_tracks=3)
    assert [tr[0][1] for tr in t] == [1, 4, 3]


def random_graph(seed, n_images=40, n_feat=300, n_points=2000, outliers=400, invalid=20):
    rng = np.random.default_rng(seed)
    nf = rng.integers(n_feat // 2, n_feat, n_images)
    by_pair = {}
    for p in range(n_points):
        first = int(rng.integers(0, n_images - 1))
        lst = [(i, int(rng.integers(0, nf[i]))) for i in range(first, min(n_images, first + int(rng.integers(2, 8))))]
        for (ia, fa), (ib, fb) in zip(lst, lst[1:]):
            if rng.random() < 0.8:
                by_pair.setdefault((ia, ib), []).append((fa, fb))
            if rng.random() < 0.3 and ib + 1 < n_images:
                by_pair.setdefault((ia, min(ib + 1, n_images - 1)), []).append((fa, int(rng.integers(0, nf[min(ib + 1, n_images - 1)]))))
    for _ in range(outliers):
        a, b = (int(x) for x in rng.choice(n_images, 2, replace=False))
        by_pair.setdefault((a, b), []).append((int(rng.integers(0, nf[a])), int(rng.integers(0, nf[b]))))
    pairs = [(a, b, m) for (a, b), m in by_pair.items()]
    for _ in range(invalid):  # out-of-range features, same-image and out-of-range images
        a = int(rng.integers(0, n_images))
        pairs.append((a, int(rng.integers(0, n_images + 2)), [(int(nf[a]) + 3, 0)]))
    order = rng.permutation(len(pairs))
    return [int(x) for x in nf], [pairs[k] for k in order]


@pytest.mark.parametrize("seed", [1, 2, 3])
@pytest.mark.parametrize("kw", [dict(), dict(min_length=2), dict(min_length=4, max_tracks=50)])
def test_random_graphs(matcher, seed, kw):
    nf, pairs = random_graph(seed)
    t, st = both(matcher, nf, pairs, **kw)
    assert st["edges"] > 1000 and st["invalid_matches"] > 0


def test_empty_and_edgeless(matcher):
    assert both(matcher, [], [])[0] == []
    assert both(matcher, [4, 4], [])[0] == []
    assert both(matcher, [4, 4], [(0, 1, [])])[0] == []


def test_zone_match_lists(matcher):
    # the 240-view zone's BF16 match lists as the verified matches of every pair
    import skylens_match as sm
    z = synth.zone(positions=80, seed=3)
    st = sm.DescriptorStore(matcher, int(z.counts.sum()) + 1024, len(z.counts))
    st.add_views_packed(z.desc, z.offsets, z.counts)
    plan = st.plan(z.pairs, 0.8, True, "bf16")
    plan.launch()
    res, off = plan.results()
    pairs = [(int(u), int(v), res[int(off[k]):int(off[k + 1])]) for k, (u, v) in enumerate(z.pairs.tolist())]
    t, stats = both(matcher, [int(c) for c in z.counts], pairs)
    # the zone's views observe shared landmarks: thousands of long tracks
    assert stats["edges"] > 1_000_000 and stats["tracks"] > 1000
    assert sum(len(tr) for tr in t) / len(t) > 10
    plan.close()
    st.close()


def test_argument_checks(matcher):
    L = matcher._L
    nt, no = ctypes.c_uint64(), ctypes.c_uint64()
    assert L.slm_build_tracks_drop(None, None, 0, None, 0, None, 3, 10, None, 0, None, 0, ctypes.byref(nt),
                                   ctypes.byref(no), None) != 0
    # capacity: the sizes needed are reported
    arr, flat = T.pack([(0, 1, [(0, 0)]), (1, 2, [(0, 0)])])
    nf = np.array([1, 1, 1], np.uint32)
    P = ctypes.POINTER
    st = L.slm_build_tracks_drop(matcher.handle, nf.ctypes.data_as(P(ctypes.c_uint32)), 3, arr, 2,
                                 flat.ctypes.data_as(P(T.SlmPair)), 3, 10, None, 0, None, 0, ctypes.byref(nt),
                                 ctypes.byref(no), None)
    assert st == 2 and nt.value == 1 and no.value == 3
    # a pair naming an image beyond the list is an invalid match, not an error
    t, stats = T.build_tracks_drop(matcher, [1, 1], [(0, 5, [(0, 0)])], min_length=2)
    assert t == [] and stats["invalid_matches"] == 1


def test_matches_read_in_place_or_copied(matcher):
    # 8-byte aligned host matches are read where they lie (where the device can
    # read host memory); a buffer 4 bytes off is copied first; device matches
    # are read in place: the same tracks every way
    import torch
    nf, pairs = random_graph(7)
    want = T.build_tracks_drop(matcher, nf, pairs)
    arr, flat = T.pack(pairs)
    P = ctypes.POINTER
    nfa = np.ascontiguousarray(nf, dtype=np.uint32)
    odd = np.zeros(flat.size + 1, np.uint32)
    odd[1:] = flat.reshape(-1)
    dev = torch.from_numpy(flat.reshape(-1).astype(np.int32)).cuda()
    for ptr in (odd.ctypes.data + 4, dev.data_ptr()):
        cap_t, cap_o = len(flat) + 1, 2 * len(flat) + 1
        toff = np.zeros(cap_t + 1, np.uint64)
        obs = np.zeros((cap_o, 2), np.uint32)
        nt, no = ctypes.c_uint64(), ctypes.c_uint64()
        st = T.SlmTrackStats()
        assert matcher._L.slm_build_tracks_drop(matcher.handle, nfa.ctypes.data_as(P(ctypes.c_uint32)), len(nfa), arr,
                                                len(pairs), ctypes.cast(ptr, P(T.SlmPair)), 3, 100000,
                                                toff.ctypes.data_as(P(ctypes.c_uint64)), cap_t,
                                                obs.ctypes.data_as(P(T.SlmPair)), cap_o, ctypes.byref(nt),
                                                ctypes.byref(no), ctypes.byref(st)) == 0
        got = [[(int(i), int(f)) for i, f in obs[int(toff[t]):int(toff[t + 1])]] for t in range(nt.value)]
        assert got == want[0] and st.as_dict() == want[1]
