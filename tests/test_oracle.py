"""CPU: the oracle against the reference's own known answers (golden vectors).

The oracle (oracle/oracle.c) is the checker for every GPU parity test, so it is
pinned first: the reference's tests, restated in refcases.py, must pass on it.
"""
import json
import os

import numpy as np
import pytest

import oracle as O
import refcases

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


def oracle_rm(a, b, ratio, mutual):
    return O.ratio_match(a, b, ratio, mutual, threads=2)


@pytest.mark.parametrize("case", refcases.ALL, ids=lambda f: f.__name__)
def test_reference_case_on_oracle(case):
    case(oracle_rm)


def test_golden_fixture_pins():
    """The fixture the regression hash is computed on is regenerated bit for bit."""
    import hashlib
    fx = GOLDEN["regression_hash"]["fixture"]
    a, b = O.match_fixture(fx["seed"], fx["na"], fx["extra"])
    assert len(b) == fx["nb"]
    assert hashlib.sha256(a.tobytes()).hexdigest() == fx["sha256_a"]
    assert hashlib.sha256(b.tobytes()).hexdigest() == fx["sha256_b"]


def test_oracle_threads_do_not_change_result():
    a, b = O.match_fixture(21, 2000, 700)
    ref = O.ratio_match(a, b, 0.8, True, threads=1)
    assert O.ratio_match(a, b, 0.8, True, threads=7) == ref


def test_sq_dist_spec_differs_from_sequential_sometimes():
    """The spec order (8 lanes) is not the sequential sum: the boundary test relies on it."""
    g = O.Lcg(93)
    diff = 0
    for _ in range(100):
        a, b = g.feature(), g.feature()
        diff += O.sq_dist(a, b) != O.sq_dist_seq(a, b)
    assert diff > 10


def test_candidate_pairs_counts():
    """matching.rs:1402-1413, 1415-1452; perf_structure.rs:29-47."""
    cp = GOLDEN["candidate_pairs"]
    rig = lambda p: [(c, q) for q in range(p) for c in range(3)]
    pairs = O.candidate_pairs(rig(10), 2, 1, 0)
    assert len(pairs) == cp["rig10_t2_c1_p0"]
    assert all(i < j for i, j in pairs)
    v80 = rig(80)
    assert len(O.candidate_pairs(v80, 5, 4, 16)) == cp["rig80_spec"]
    assert len(O.candidate_pairs(v80, 5, 4, 2**64 - 1)) == cp["rig80_pow2_unbounded"]
    assert len(O.candidate_pairs(v80, 5, 4, 0)) == cp["rig80_pow2_zero"]
    for p, n in cp["pairs_48P_minus_177"].items():
        assert len(O.candidate_pairs(rig(int(p)), 5, 4, 16)) == n
    pairs = O.candidate_pairs(v80, 5, 4, 16)
    deg = np.zeros(240, int)
    for i, j in pairs:
        deg[i] += 1
        deg[j] += 1
    assert deg.max() <= 32 and deg[3 * 40] == 32


def test_scheduled_pairs_spec_equals_candidate_pairs():
    """matching.rs:2668-2703."""
    views = [(c, p) for p in range(30) for c in range(3)]
    spec = O.scheduled_pairs(views, spec_range=4)
    assert spec == O.candidate_pairs(views, 5, 4, 16)
    f = O.scheduled_pairs(views)
    kinds = set()
    for i, j in f:
        (ca, pa), (cb, pb) = views[i], views[j]
        assert i < j
        if ca != cb:
            (cf, pf), (co, po) = ((ca, pa), (cb, pb)) if ca == 0 else ((cb, pb), (ca, pa))
            assert pf + 20 <= po <= pf + 40 and (po - pf) % 4 == 0
            kinds.add(co)
    assert sorted(kinds) == [1, 2]
    same = lambda v: sum(1 for i, j in v if views[i][0] == views[j][0])
    assert same(f) == same(spec)


def test_oracle_nan_semantics():
    """A NaN distance never updates a best (matching.rs:182-190 use `<`)."""
    g = O.Lcg(3)
    a = np.stack([g.feature() for _ in range(3)])
    b = np.stack([g.feature() for _ in range(4)])
    b[1, 5] = np.nan
    rj, d1, d2, ci, cd = O.ratio_states(a, b)
    assert not np.any(rj == 1)
    assert np.all(np.isfinite(d1))
