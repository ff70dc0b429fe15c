"""GPU: skewed and extreme pair shapes, every precision, single calls and one batch.

A single row against tens of thousands of columns (one row tile, its columns
split over many work items: the shortlist's shared-row path with atomic
candidate slots), tens of thousands of rows against two or three columns
(nothing but ragged column tiles), sizes one past a tile boundary, and the
smallest pairs that can match at all (nb = 2). Every list must equal the
oracle's.
"""
import numpy as np
import pytest

import oracle as O
from skylens_match import synth

pytestmark = pytest.mark.gpu

SHAPES = [(1, 2), (2, 2), (1, 40000), (3, 65536), (40000, 2), (65536, 3), (130, 30000), (30000, 130),
          (4097, 4095), (129, 129)]


def make_pair(na, nb, seed):
    """b: fresh SIFT-like rows; a: noisy copies of some rows of b (matches exist)
    and fresh rows."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = synth.sift_like(rng, nb)
    k = min(na, nb) // 2 + (1 if na else 0)
    k = min(k, na, nb)
    a = np.concatenate([synth.noisy_copy(rng, b[rng.permutation(nb)[:k]], 0.05), synth.sift_like(rng, na - k)])
    return np.ascontiguousarray(a[rng.permutation(na)]), b


@pytest.fixture(scope="module")
def cases():
    out = []
    for s, (na, nb) in enumerate(SHAPES):
        a, b = make_pair(na, nb, 500 + s)
        want = {m: O.ratio_match_np(a, b, 0.8, m, threads=16) for m in (True, False)}
        out.append((a, b, want))
    return out


@pytest.mark.parametrize("prec", ["fp32", "bf16", "fp8"])
def test_single_calls(matcher, cases, prec):
    for a, b, want in cases:
        for mutual in (True, False):
            got = matcher.ratio_match_np(a, b, 0.8, mutual, prec)
            assert np.array_equal(got, want[mutual]), (len(a), len(b), prec, mutual)


@pytest.mark.parametrize("prec", ["fp32", "bf16", "fp8"])
def test_one_batch(matcher, cases, prec):
    st = matcher.store(sum(len(a) + len(b) for a, b, _ in cases), 2 * len(cases))
    pairs = []
    for a, b, _ in cases:
        pairs.append((st.add_view(a), st.add_view(b)))
    plan = st.plan(pairs, 0.8, True, prec)
    plan.launch()
    got = plan.per_pair()
    for k, (a, b, want) in enumerate(cases):
        assert np.array_equal(got[k], want[True]), (len(a), len(b), prec)
    plan.close()
    st.close()


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_repeated_launches_give_identical_bytes(matcher, cases, prec):
    """Candidate slots and column counters are filled by atomics in whatever
    order the CTAs run; the compacted lists must not depend on it: five
    launches of one plan (rows split over many work items among its pairs)
    return the same bytes."""
    st = matcher.store(sum(len(a) + len(b) for a, b, _ in cases), 2 * len(cases))
    pairs = [(st.add_view(a), st.add_view(b)) for a, b, _ in cases]
    plan = st.plan(pairs, 0.8, True, prec)
    plan.launch()
    first = plan.results()
    for _ in range(4):
        plan.launch()
        again = plan.results()
        assert np.array_equal(again[0], first[0]) and np.array_equal(again[1], first[1])
    plan.close()
    st.close()
