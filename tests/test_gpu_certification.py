"""GPU: the shortlist's certification on inputs built to break it.

Every BF16 / FP8 match decision is either proved by the per-pair bound eps
on |d~ - d| or settled with exact spec-order FP32 distances. The bound
assumes the tensor core's FP32 accumulation loses no more than 2^-11 of the
summed product magnitudes; SIFT-like inputs never come near that. Here the
inputs are hostile (tests/hostile.py): mixed signs, norms up to just under
the routing limit of 64, one dominant component beside 127 tiny ones, and
rows and columns placed within a fraction of eps of the ratio test's edge
and of a cross-check tie, single pairs and a batch of 96 pairs. For each:

  - the tensor-core estimates of the first pair (the plan's debug dump) lie
    within eps of the FP64 distances, everywhere; for BF16 the accumulation's
    own error (against the exact sum of the rounded operands) stays within
    the 2^-11 relative allowance the bound makes for it;
  - the match lists equal the oracle's bit for bit (single calls through
    slm_ratio_match and batch plans);
  - the counters show that the rows no bound of that width can settle went
    to the exact rescore or scan (rows rescored + rows recomputed >= rows with
    |d1 - r^2 d2| <= eps / 4), and that columns with two rows within eps / 4
    of each other were checked exactly (columns recomputed >= their number).
    eps is the bound of the tier that settled the pair: an FP8 pair whose
    bound is too loose for its distances is rescued by the BF16 passes, and
    then the BF16 bound decides (the FP8 estimates are still checked against
    the FP8 bound).
"""
import numpy as np
import pytest

import hostile as H
import oracle as O

pytestmark = pytest.mark.gpu

PRECS = ["bf16", "fp8"]

CASES = {
    "mixed_sign": lambda: H.mixed_sign(11, 700, 900),
    "large_norm_63": lambda: H.large_norm(12, 700, 900, 0.05, 63.0),
    "large_norm_4": lambda: H.large_norm(13, 700, 900, 0.25, 4.0),
    "swamped_1e-2": lambda: H.swamped(14, 700, 900, 1e-2),
    "swamped_1e-3": lambda: H.swamped(15, 700, 900, 1e-3),
    "swamped_3e-5": lambda: H.swamped(16, 700, 900, 3e-5),
    "boundary": lambda: H.boundary_pair(17, 500, 150, 300),
}


def _check_counters(stats, d, eps, mutual, ratio=0.8):
    near = H.near_boundary_rows(d, ratio, eps / 4)
    settled = stats["rows_rescored"] + stats["rows_recomputed"]
    assert settled >= near, f"{near} rows within eps/4 of the ratio edge, only {settled} settled exactly"
    tied = H.tied_columns(d, ratio, eps / 4) if mutual else 0
    assert stats["cols_recomputed"] >= tied, f"{tied} tied columns, {stats['cols_recomputed']} checked exactly"
    return near, tied


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("case", sorted(CASES))
def test_hostile_pair_bound_and_parity(matcher, case, prec):
    a, b = CASES[case]()
    na, nb = len(a), len(b)
    eps = H.eps_bound(a, b, prec)
    st = matcher.store(na + nb, 2)
    st.add_view(a)
    st.add_view(b)
    plan = st.plan([(0, 1)], 0.8, True, prec, variant=2)
    plan.launch()
    got, _ = plan.results()
    stats = plan.stats
    dt = plan.debug_dump(na, nb)
    plan.close()
    st.close()
    ref64 = O.dist_matrix_f64(a, b)
    err = np.abs(dt.astype(np.float64) - ref64)
    print(f"{case} {prec}: eps {eps:.4g}, max |d~ - d64| {err.max():.4g} ({err.max() / eps:.3f} eps), "
          f"rescored {stats['rows_rescored']} recomputed {stats['rows_recomputed']} "
          f"cols {stats['cols_recomputed']} routed {stats['pairs_routed']}")
    assert np.isfinite(dt).all()
    assert err.max() <= eps
    if prec == "bf16":
        # the accumulation alone, against the exact sum of the rounded operands
        rel = H.bf16_accumulation_error(a, b, dt)
        print(f"  bf16 accumulation error {rel:.3g} relative ({np.log2(max(rel, 1e-300)):.1f} bits)")
        assert rel <= 2.0 ** -11
    want = O.ratio_match_np(a, b, 0.8, True, threads=8)
    assert np.array_equal(got, want)
    eps_tier = H.eps_bound(a, b, "bf16") if stats["pairs_rescued"] else eps
    _check_counters(stats, O.dist_matrix(a, b), eps_tier, True)
    # the single-pair drop-in, both cross-check settings
    assert np.array_equal(matcher.ratio_match_np(a, b, 0.8, True, prec), want)
    assert np.array_equal(matcher.ratio_match_np(a, b, 0.95, False, prec),
                          O.ratio_match_np(a, b, 0.95, False, threads=8))


def _boundary_batch(npairs=48, seed=100):
    views, pairs = [], []
    for k in range(npairs):
        a, b = H.boundary_pair(seed + k, 400, 120, 400, exact_ties=8)
        views += [a, b]
        pairs.append((2 * k, 2 * k + 1))
    nv = len(views)
    # unrelated pairs between the views of different sets (views shared by pairs)
    pairs += [(2 * k, (2 * k + 3) % nv) for k in range(npairs)]
    return views, pairs


@pytest.fixture(scope="module")
def boundary_batch():
    views, pairs = _boundary_batch()
    want = {}
    for mutual in (True, False):
        want[mutual] = [O.ratio_match_np(views[u], views[v], 0.8, mutual, threads=16) for u, v in pairs]
    dists = [O.dist_matrix(views[u], views[v]) for u, v in pairs[:48]]
    return views, pairs, want, dists


@pytest.mark.parametrize("mutual", [True, False])
@pytest.mark.parametrize("prec", ["bf16", "fp8", "fp32"])
def test_boundary_batch(matcher, boundary_batch, prec, mutual):
    views, pairs, want, dists = boundary_batch
    st = matcher.store(sum(len(v) for v in views), len(views))
    for v in views:
        st.add_view(v)
    plan = st.plan(pairs, 0.8, mutual, prec, variant=2 if prec != "fp32" else 0)
    for rep in range(2):  # the second launch replays the captured graph
        plan.launch()
        got = plan.per_pair()
        for k in range(len(pairs)):
            assert np.array_equal(got[k], want[mutual][k]), f"{prec} pair {k} {pairs[k]} launch {rep}"
    stats = plan.stats
    if prec != "fp32":
        a, b = views[0], views[1]
        dt = plan.debug_dump(len(a), len(b))
        err = np.abs(dt.astype(np.float64) - O.dist_matrix_f64(a, b)).max()
        eps0 = H.eps_bound(a, b, prec)
        assert err <= eps0
        # the bound of a pair follows its own views; the counters sum over pairs
        near = tied = near_own = 0
        for k in range(48):
            u, v = pairs[k]
            eps = H.eps_bound(views[u], views[v], prec)
            near_own += H.near_boundary_rows(dists[k], 0.8, eps / 4)
            if stats["pairs_rescued"]:  # some pairs settled by the BF16 tier: its (smaller) bound
                eps = min(eps, H.eps_bound(views[u], views[v], "bf16"))
            near += H.near_boundary_rows(dists[k], 0.8, eps / 4)
            tied += H.tied_columns(dists[k], 0.8, eps / 4) if mutual else 0
        print(f"batch {prec} mutual={mutual}: near rows {near} ({near_own} by its own bound), tied columns "
              f"{tied}, stats {stats}, pair-0 max err {err:.4g} of eps {eps0:.4g}")
        assert near_own >= 2000  # the batch does put thousands of rows at the edge
        assert stats["rows_rescored"] + stats["rows_recomputed"] >= near
        assert stats["cols_recomputed"] >= tied
    plan.close()
    st.close()
