"""GPU: pairs the shortlist's first tier cannot settle.

A pair whose FP8 bound is too loose to certify its rows (E4M3 on unit-length
descriptors: eps about 0.1 against distance gaps of the same size) is
rescued, after FP8 pass 1, by the BF16 passes of the same launch when its
near-chunk counts predict shortlist overflow. It is matched whole by the
tiled exact FP32 kernel after pass 2 when its rows' shortlists did grow
wide, and before pass 1 when its inputs are not finite. Whichever way a pair
goes, its match list is the reference's.
"""
import numpy as np
import pytest

import oracle as O
from skylens_match import synth

pytestmark = pytest.mark.gpu


def ref(a, b, mutual=True):
    return O.ratio_match_np(a, b, 0.8, mutual, threads=16)


@pytest.mark.parametrize("mutual", [True, False])
def test_fp8_large_pair_is_rescued_by_bf16(matcher, mutual):
    a, b = synth.pair_large(4096, 0.4, (0.02, 0.08), seed=5)
    got = matcher.ratio_match_np(a, b, 0.8, mutual, "fp8")
    s = matcher.last_stats
    print("fp8 4096x4096:", s)
    assert np.array_equal(got, ref(a, b, mutual))
    assert s["pairs_rescued"] == 1 and s["rows_rescued"] == 4096
    assert s["pairs_routed"] == 0
    # the BF16 bound settles almost every row; a few go to the exact rescore
    assert s["rows_recomputed"] <= 0.01 * 4096
    assert s["rows_rescored"] <= 0.2 * 4096


def test_fp8_small_pair_is_routed_after_pass2(matcher):
    """400 columns are 25 chunks of 16, so the near-chunk estimate (> 32) cannot
    route the pair after pass 1; its overflowing rows route it after pass 2."""
    a, b = synth.pair_large(400, 0.4, 0.05, seed=6)
    got = matcher.ratio_match_np(a, b, 0.8, True, "fp8")
    s = matcher.last_stats
    print("fp8 400x400:", s)
    assert np.array_equal(got, ref(a, b))
    assert s["pairs_routed"] == 1
    assert s["rows_recomputed"] == 400


@pytest.mark.parametrize("prec", ["bf16", "fp8"])
def test_non_finite_pair_is_routed(matcher, prec):
    rng = np.random.Generator(np.random.PCG64(9))
    a = synth.sift_like(rng, 300)
    b = np.concatenate([synth.noisy_copy(rng, a[:150], 0.05), synth.sift_like(rng, 200)])
    b[17, 5] = np.nan
    got = matcher.ratio_match_np(a, b, 0.8, True, prec)
    s = matcher.last_stats
    assert np.array_equal(got, ref(a, b))
    assert s["pairs_routed"] == 1


def test_bf16_does_not_route(matcher):
    """The bf16 bound is tight enough: no pair of a zone or a large pair is routed."""
    z = synth.zone(positions=8, seed=21)
    st = matcher.store(int(z.counts.sum()), len(z.counts))
    st.add_views_packed(z.desc, z.offsets, z.counts)
    plan = st.plan(z.pairs, 0.8, True, "bf16")
    plan.launch()
    got = plan.per_pair()
    assert plan.stats["pairs_routed"] == 0
    for k in range(0, len(z.pairs), 7):
        u, v = map(int, z.pairs[k])
        assert np.array_equal(got[k], ref(z.view(u), z.view(v))), k
    plan.close()
    st.close()
    # single large pairs: pass 1 splits their rows into many column ranges
    for a, b in (synth.pair_large(8192, 0.5, 0.05, seed=2), synth.pair_fp8(32768, seed=4)):
        matcher.ratio_match_np(a, b, 0.8, True, "bf16")
        print(f"bf16 {len(a)}x{len(b)}:", matcher.last_stats)
        assert matcher.last_stats["pairs_routed"] == 0


def test_mixed_fp8_batch(matcher):
    """One batch: routed pairs (after pass 1, after pass 2, non-finite) beside
    pairs the shortlist settles (too few columns to overflow) and empty views;
    replayed twice, since the routing is decided afresh in every launch."""
    rng = np.random.Generator(np.random.PCG64(10))
    big_a, big_b = synth.pair_large(2500, 0.4, (0.02, 0.08), seed=11)
    mid_a, mid_b = synth.pair_large(300, 0.4, 0.05, seed=12)
    tiny_a = synth.sift_like(rng, 40)
    tiny_b = np.concatenate([synth.noisy_copy(rng, tiny_a[:10], 0.05), synth.sift_like(rng, 6)])
    bad = synth.sift_like(rng, 200)
    bad[3, 0] = np.inf
    empty = np.zeros((0, 128), np.float32)
    views = [big_a, big_b, mid_a, mid_b, tiny_a, tiny_b, bad, empty]
    # (4, 5) and (2, 5) have 16 columns: a column half holds all of them, no overflow
    pairs = [(0, 1), (2, 3), (4, 5), (6, 0), (7, 1), (1, 7), (2, 5), (3, 2), (1, 0)]
    st = matcher.store(sum(len(v) for v in views), len(views))
    for v in views:
        st.add_view(v)
    plan = st.plan(pairs, 0.8, True, "fp8")
    for rep in range(2):
        plan.launch()
        got = plan.per_pair()
        s = plan.stats
        print("mixed fp8 batch:", s)
        for k, (u, v) in enumerate(pairs):
            assert np.array_equal(got[k], ref(views[u], views[v])), (rep, k)
        # rescued by BF16 after pass 1: (0,1), (1,0); routed to the exact kernel
        # after pass 2: (2,3), (3,2); unsafe: (6,0)
        assert s["pairs_rescued"] == 2
        assert s["pairs_routed"] == 3
    plan.close()
    st.close()


def test_fp8_item_with_a_rescued_and_a_routed_pair(matcher):
    """The last, odd row tiles of two pairs with the same b view share one
    item: here one pair (unit descriptors against unit descriptors) is rescued
    by the BF16 passes while the other (a non-finite view) goes to the exact
    kernel; FP8 pass 2 skips the item, the BF16 passes work on the rescued
    pair's tile only, and both lists equal the oracle's."""
    rng = np.random.Generator(np.random.PCG64(14))
    big_a, big_b = synth.pair_large(2500, 0.4, (0.02, 0.08), seed=13)
    big_a = big_a[:2400]               # 19 row tiles: the last one is odd
    bad = big_b[::25][:100].copy()     # 1 row tile: copies of b's rows, one of them not finite
    bad[7, 3] = np.nan
    views = [big_a, big_b, bad, synth.sift_like(rng, 300)]
    pairs = [(0, 1), (2, 1), (3, 1)]
    st = matcher.store(sum(len(v) for v in views), len(views))
    for v in views:
        st.add_view(v)
    plan = st.plan(pairs, 0.8, True, "fp8")
    for rep in range(2):
        plan.launch()
        got = plan.per_pair()
        s = plan.stats
        print("fp8 shared item:", s)
        for k, (u, v) in enumerate(pairs):
            assert np.array_equal(got[k], ref(views[u], views[v])), (rep, k)
        assert len(got[1]) >= 90  # the finite copies find their originals
        # (0,1) and (3,1) rescued; (2,1) unsafe
        assert s["pairs_rescued"] == 2 and s["rows_rescued"] == 2700
        assert s["pairs_routed"] == 1
    plan.close()
    st.close()
