"""The reference's ratio_match tests, restated against any `rm(a, b, ratio, mutual)`.

Each function follows one #[test] of crates/core/src/matching.rs and asserts
what it asserts. Fixtures come from the oracle's restatement of the test Lcg
(matching.rs:1140-1153), `feature` (:1580-1596) and `match_fixture` (:1638-1656).
"""
from __future__ import annotations

import math

import numpy as np

import oracle as O

MATCH_BLOCK = 64  # matching.rs:158


def _arr(rows):
    return np.ascontiguousarray(np.stack(rows).astype(np.float32)) if len(rows) else np.zeros((0, 128), np.float32)


def equals_reference(rm):
    """matching.rs:1658-1685 ratio_match_equals_reference."""
    for seed, na, extra in [(1, 1, 0), (2, 63, 5), (3, 64, 64), (4, 65, 10), (5, 700, 300)]:
        a, b = O.match_fixture(seed, na, extra)
        for mutual in (True, False):
            for ratio in (0.6, 0.8, 1.0):
                fast = rm(a, b, ratio, mutual)
                slow = O.ratio_match_naive(a, b, ratio, mutual)
                assert fast == slow, f"seed {seed} mutual {mutual} ratio {ratio}"
                fast = rm(b, a, ratio, mutual)
                slow = O.ratio_match_naive(b, a, ratio, mutual)
                assert fast == slow, f"rev seed {seed} mutual {mutual} ratio {ratio}"
    a, _ = O.match_fixture(9, 10, 0)
    empty = np.zeros((0, 128), np.float32)
    assert rm(a, empty, 0.8, True) == []
    assert rm(empty, a, 0.8, True) == []


def regression_hash(rm):
    """matching.rs:1880-1901 ratio_match_regression_hash."""
    a, b = O.match_fixture(21, 2000, 700)
    m = rm(a, b, 0.8, True)
    n = rm(a, b, 0.95, False)
    assert (len(m), O.pairs_hash(m)) == (1145, 0x22CA99B86722152D)
    assert (len(n), O.pairs_hash(n)) == (1282, 0x7D0CD9993D0C89E5)


def rounding_boundary(rm) -> int:
    """matching.rs:2359-2406 ratio_match_rounding_boundary: rows whose ratio sits
    between the spec-order sum and the sequential sum; only the spec order passes."""
    g = O.Lcg(93)
    found = 0
    f32 = np.float32
    for _ in range(200):
        a = g.feature()
        b1 = g.feature()
        b2 = g.feature()
        d1 = f32(O.sq_dist(a, b1))
        d2 = f32(O.sq_dist(a, b2))
        s1 = f32(O.sq_dist_seq(a, b1))
        if s1 == d1 or d1 >= d2:
            continue
        target = 0.5 * (float(d1) + float(s1)) / float(d2)
        r = f32(math.sqrt(target))

        def between(r):
            lim = f32(f32(r * r) * d2)
            return (d1 < lim) != (s1 < lim)

        for _ in range(64):
            if between(r):
                break
            r = np.frombuffer((np.frombuffer(r.tobytes(), np.uint32) + np.uint32(1)).tobytes(), np.float32)[0]
        if not between(r):
            continue
        found += 1
        m = rm(a[None, :], np.stack([b1, b2]), float(r), False)
        expect = bool(d1 < f32(f32(r * r) * d2))
        assert (len(m) > 0) == expect, "boundary row decided differently from the spec order"
    assert found >= 5, f"too few boundary rows: {found}"
    return found


def ties_take_lower_index(rm):
    """matching.rs:2407-2434 ratio_match_ties_take_lower_index."""
    g = O.Lcg(11)
    b = _arr([g.feature() for _ in range(20)])
    for dup in (1, MATCH_BLOCK + 6):
        a = [g.feature() for _ in range(dup + 4)]
        x = b[3].copy()
        x[0] = np.float32(x[0] + np.float32(1e-3))
        a[0] = x.copy()
        a[dup] = x.copy()
        m = rm(_arr(a), b, 0.8, True)
        assert (0, 3) in m, f"dup {dup}: {m}"
        assert not any(i == dup for i, _ in m), f"dup {dup}: {m}"


def needs_second_neighbour(rm):
    """matching.rs:1775-1790 ratio_match_needs_second_neighbour."""
    g = O.Lcg(5)
    a = _arr([g.feature(), g.feature()])
    b = _arr([g.feature()])
    for mutual in (False, True):
        for ratio in (0.6, 0.8, 1.0):
            assert rm(a, b, ratio, mutual) == []
    b2 = _arr([a[0], g.feature()])
    assert rm(a[:1], b2, 0.8, False) == [(0, 0)]


def recovers_permutation(rm):
    """matching.rs:1710-1746 ratio_match_recovers_permutation."""
    g = O.Lcg(11)
    a = [g.feature() for _ in range(100)]
    b = []
    for i, f in enumerate(a):
        b.append((g.perturb(f, 0.01), i))
        if i < 10:
            b.append((g.perturb(f, 0.01), None))
    for _ in range(100):
        b.append((g.feature(), None))
    for i in range(len(b) - 1, 0, -1):
        j = int(g.next() * (i + 1))
        b[i], b[j] = b[j], b[i]
    bf = _arr([x[0] for x in b])
    m = rm(_arr(a), bf, 0.8, True)
    correct = sum(1 for i, j in m if b[j][1] == i)
    assert correct == len(m), f"wrong pairs {len(m) - correct}"
    assert len(m) == 90, f"matches {len(m)}"
    assert all(i >= 10 for i, _ in m)


ALL = [equals_reference, regression_hash, rounding_boundary, ties_take_lower_index, needs_second_neighbour,
       recovers_permutation]
