"""GPU: the matching half of match_pairs (pipeline.rs:485-496).

scheduled_pairs(views, PairSchedule::default()) forms the pairs, ratio_match
(0.8, cross-check) matches each, and pairs with fewer than 20 matches are
dropped before RANSAC. The batch does all of it on the device (the filter
zeroes the counts of dropped pairs before compaction); the kept pairs, their
order and their match lists must equal the oracle's.
"""
import numpy as np
import pytest

import oracle as O
import skylens_match as sm
from skylens_match import synth

pytestmark = pytest.mark.gpu


def oracle_match_pairs(z, min_matches=20):
    out = []
    for i, j in O.scheduled_pairs(z.views):
        m = O.ratio_match_np(z.view(i), z.view(j), 0.8, True, threads=8)
        if len(m) >= min_matches:
            out.append((i, j, m))
    return out


@pytest.mark.parametrize("prec", ["fp32", "bf16", "fp8"])
def test_match_scheduled_pairs_equals_oracle(matcher, prec):
    # landmarks live 5 positions: distant scheduled pairs share few (110 of 147 kept)
    z = synth.zone(positions=12, n_range=(150, 900), seed=31, lifetime=5)
    st = matcher.store(int(z.counts.sum()), len(z.counts))
    st.add_views_packed(z.desc, z.offsets, z.counts)
    got = sm.match_scheduled_pairs(st, z.views, precision=prec, min_matches=20)
    want = oracle_match_pairs(z)
    n_sched = len(O.scheduled_pairs(z.views))
    print(f"{prec}: {n_sched} scheduled pairs, {len(want)} kept")
    assert 0 < len(want) < n_sched  # the filter drops some pairs and keeps others
    assert [(i, j) for i, j, _ in got] == [(i, j) for i, j, _ in want]
    for (i, j, a), (_, _, b) in zip(got, want):
        assert np.array_equal(a, b), (i, j)
    st.close()


def test_plan_min_matches_replayed(matcher):
    """The filter on a captured plan: set, replayed, changed, removed."""
    z = synth.zone(positions=6, n_range=(150, 900), seed=32)
    st = matcher.store(int(z.counts.sum()), len(z.counts))
    st.add_views_packed(z.desc, z.offsets, z.counts)
    plan = st.plan(z.pairs, 0.8, True, "bf16")
    plan.launch()
    full = plan.per_pair()
    sizes = sorted(len(a) for a in full)
    cut = sizes[len(sizes) // 2]  # about half of the pairs fall below
    for min_matches in (cut, cut, 0, cut + 1):
        plan.set_min_matches(min_matches)
        plan.launch()
        got = plan.per_pair()
        for a, b in zip(full, got):
            assert np.array_equal(b, a if len(a) >= min_matches else a[:0])
    plan.close()
    st.close()
