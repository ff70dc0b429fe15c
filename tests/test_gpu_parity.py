"""GPU: every precision (plain FP32, BF16 and FP8 shortlists) against the
oracle and the reference's tests.

Every comparison is exact equality of match lists (bit-exact integer output):
the shortlist paths settle every decision their error bound cannot certify
with exact FP32 arithmetic, so they too must equal the reference.
"""
import threading

import numpy as np
import pytest

import oracle as O
import refcases
import skylens_match as sm
from skylens_match import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(params=["fp32", "bf16", "fp8"])
def prec(request):
    return request.param


def rm_of(matcher, prec):
    return lambda a, b, ratio, mutual: matcher.ratio_match(a, b, ratio, mutual, prec)


@pytest.mark.parametrize("case", refcases.ALL, ids=lambda f: f.__name__)
def test_reference_case(matcher, case, prec):
    case(rm_of(matcher, prec))


def check(matcher, a, b, ratio=0.8, mutual=True, prec="fp32", threads=8):
    got = matcher.ratio_match_np(a, b, ratio, mutual, prec)
    ref = O.ratio_match_np(a, b, ratio, mutual, threads=threads)
    assert got.shape == ref.shape and np.array_equal(got, ref), (
        f"{len(got)} vs {len(ref)} matches; first diff at "
        f"{next((k for k in range(min(len(got), len(ref))) if tuple(got[k]) != tuple(ref[k])), None)}")
    return got


def test_pair_800(matcher, prec):
    a, b = synth.pair_800(0)
    for mutual in (True, False):
        check(matcher, a, b, 0.8, mutual, prec)


def test_pair_8192_full_size(matcher, prec):
    a, b = synth.pair_large(8192, 0.5, 0.05, seed=2)
    m = check(matcher, a, b, 0.8, True, prec, threads=16)
    assert len(m) > 1000


@pytest.mark.parametrize("na,nb", [(1, 2), (2, 1), (1, 1), (63, 64), (64, 63), (65, 129), (127, 128), (128, 127),
                                   (129, 257), (255, 1), (257, 300), (1000, 3), (3, 1000), (600, 900)])
def test_ragged_sizes(matcher, na, nb, prec):
    rng = np.random.Generator(np.random.PCG64(na * 1000 + nb))
    a = synth.sift_like(rng, na)
    k = min(na, nb) // 2
    b = np.concatenate([synth.noisy_copy(rng, a[:k], 0.03), synth.sift_like(rng, nb - k)])
    for ratio in (0.8, 1.0, 0.0, 1.5):
        for mutual in (True, False):
            check(matcher, a, b, ratio, mutual, prec)


def test_empty_inputs(matcher, prec):
    a, _ = O.match_fixture(9, 10, 0)
    e = np.zeros((0, 128), np.float32)
    assert matcher.ratio_match(a, e, 0.8, True, prec) == []
    assert matcher.ratio_match(e, a, 0.8, True, prec) == []
    assert matcher.ratio_match(e, e, 0.8, False, prec) == []


def test_exact_duplicates_and_ties(matcher, prec):
    """Duplicate rows of b tie at the row minimum (d1 == d2: no match); duplicate
    rows of a tie at a column minimum (the lower i wins), across tile borders."""
    rng = np.random.Generator(np.random.PCG64(7))
    a = synth.sift_like(rng, 300)
    b = synth.noisy_copy(rng, a, 0.02)
    b[50] = b[10]
    b[200] = b[10]
    a[130] = a[5]
    a[260] = a[5]
    a[299] = a[129]
    for mutual in (True, False):
        check(matcher, a, b, 0.8, mutual, prec)
        check(matcher, b, a, 0.8, mutual, prec)


def test_nan_and_unnormalised_inputs(matcher, prec):
    rng = np.random.Generator(np.random.PCG64(8))
    a = synth.sift_like(rng, 200) * 3.0
    b = np.concatenate([synth.noisy_copy(rng, a[:100] / 3.0, 0.03), synth.sift_like(rng, 150)]) * 0.5
    a[7, 3] = np.nan
    b[11, 0] = np.nan
    b[12] = np.inf
    a[20] = 0.0
    for mutual in (True, False):
        check(matcher, a.astype(np.float32), b.astype(np.float32), 0.8, mutual, prec)


def test_concurrent_callers(matcher, prec):
    """ratio_match is called from many rayon workers at once (pipeline.rs:487-492)."""
    z = synth.zone(positions=6, n_range=(200, 700), seed=11)
    pairs = [tuple(map(int, p)) for p in z.pairs[:24]]
    ref = {p: O.ratio_match_np(z.view(p[0]), z.view(p[1]), 0.8, True, threads=2) for p in pairs}
    got, errs = {}, []

    def worker(chunk):
        try:
            for p in chunk:
                got[p] = matcher.ratio_match_np(z.view(p[0]), z.view(p[1]), 0.8, True, prec)
        except Exception as e:  # surfaced below
            errs.append(e)

    ths = [threading.Thread(target=worker, args=(pairs[k::6],)) for k in range(6)]
    [t.start() for t in ths]
    [t.join() for t in ths]
    assert not errs, errs
    for p in pairs:
        assert np.array_equal(got[p], ref[p]), p


def zone_check(matcher, z, prec, pairs=None, threads=16):
    st = matcher.store(int(z.counts.sum()), len(z.counts))
    ids = st.add_views_packed(z.desc, z.offsets, z.counts)
    assert ids == list(range(len(z.counts)))
    pairs = z.pairs if pairs is None else pairs
    plan = st.plan(pairs, 0.8, True, prec)
    for rep in range(2):  # the second launch replays the captured graph
        plan.launch()
        per = plan.per_pair()
        for k, (u, v) in enumerate(pairs):
            ref = O.ratio_match_np(z.view(int(u)), z.view(int(v)), 0.8, True, threads=threads)
            assert np.array_equal(per[k], ref), f"pair {k} ({u},{v}) rep {rep}: {len(per[k])} vs {len(ref)}"
    stats = plan.stats
    plan.close()
    st.close()
    return stats


def test_small_zone_batch(matcher, prec):
    z = synth.zone(positions=10, n_range=(100, 900), seed=5)
    zone_check(matcher, z, prec)


def test_batch_with_repeated_and_reversed_pairs(matcher, prec):
    z = synth.zone(positions=4, n_range=(50, 400), seed=6)
    pairs = np.array([[0, 1], [1, 0], [0, 1], [2, 2], [3, 5], [5, 3]], np.uint32)
    zone_check(matcher, z, prec, pairs)


def test_device_entry_point(matcher, prec):
    """Device arrays: 16-byte aligned ones are gathered where they lie, the
    others (here 4 or 8 bytes past an aligned address) copied first."""
    torch = pytest.importorskip("torch")
    a, b = synth.pair_800(1)
    ref = O.ratio_match_np(a, b, 0.8, True, threads=4)
    for shift in (0, 1, 2):
        da = torch.zeros(a.size + 4, dtype=torch.float32, device="cuda")
        db = torch.zeros(b.size + 4, dtype=torch.float32, device="cuda")
        da[shift:shift + a.size] = torch.from_numpy(a.reshape(-1)).cuda()
        db[shift:shift + b.size] = torch.from_numpy(b.reshape(-1)).cuda()
        out = torch.zeros((800, 2), dtype=torch.int32, device="cuda")
        cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()  # inputs are ready before the library stream reads them
        matcher.ratio_match_device(da.data_ptr() + 4 * shift, 800, db.data_ptr() + 4 * shift, 800, 0.8, True, prec,
                                   out.data_ptr(), 800, cnt.data_ptr())
        torch.cuda.ExternalStream(matcher.stream).synchronize()
        n = int(cnt.item())
        assert n == len(ref), shift
        assert np.array_equal(out[:n].cpu().numpy().astype(np.uint32), ref), shift


def plan_rm(matcher, prec, variant):
    """ratio_match through a one-pair batch plan (lets a test pick the kernel variant)."""
    def rm(a, b, ratio, mutual):
        a = np.ascontiguousarray(a, np.float32).reshape(-1, 128)
        b = np.ascontiguousarray(b, np.float32).reshape(-1, 128)
        st = matcher.store(len(a) + len(b), 2)
        st.add_view(a)
        st.add_view(b)
        p = st.plan([(0, 1)], ratio, mutual, prec, variant=variant)
        p.launch()
        got = p.per_pair()[0]
        p.close()
        st.close()
        return [tuple(x) for x in got.tolist()]
    return rm


@pytest.mark.parametrize("case", refcases.ALL, ids=lambda f: f.__name__)
@pytest.mark.parametrize("variant", [1, 0], ids=["fp32-scalar", "fp32-packed"])
def test_reference_case_fp32_variants(matcher, case, variant):
    case(plan_rm(matcher, "fp32", variant))


@pytest.mark.parametrize("variant", [1, 0], ids=["fp32-scalar", "fp32-packed"])
def test_zone_batch_fp32_variants(matcher, variant):
    z = synth.zone(positions=8, n_range=(100, 1200), seed=9)
    st = matcher.store(int(z.counts.sum()), len(z.counts))
    st.add_views_packed(z.desc, z.offsets, z.counts)
    plan = st.plan(z.pairs, 0.8, True, "fp32", variant=variant)
    plan.launch()
    per = plan.per_pair()
    for k, (u, v) in enumerate(z.pairs):
        assert np.array_equal(per[k], O.ratio_match_np(z.view(int(u)), z.view(int(v)), 0.8, True, threads=16)), k
    plan.close()
    st.close()


@pytest.mark.parametrize("prec", ["bf16", "fp8"])
def test_zone_batch_one_row_tile_per_item(matcher, prec):
    """Items of one 128-row tile (M = 128 per CTA) give the same lists."""
    z = synth.zone(positions=8, n_range=(100, 1300), seed=13)
    st = matcher.store(int(z.counts.sum()), len(z.counts))
    st.add_views_packed(z.desc, z.offsets, z.counts)
    plan = st.plan(z.pairs, 0.8, True, prec, row_tiles=1)
    plan.launch()
    per = plan.per_pair()
    for k, (u, v) in enumerate(z.pairs):
        assert np.array_equal(per[k], O.ratio_match_np(z.view(int(u)), z.view(int(v)), 0.8, True, threads=16)), k
    plan.close()
    st.close()


@pytest.fixture(scope="module")
def tune_zone():
    z = synth.zone(positions=6, n_range=(200, 1500), seed=19)
    want = [O.ratio_match_np(z.view(int(u)), z.view(int(v)), 0.8, True, threads=16) for u, v in z.pairs]
    return z, want


@pytest.mark.parametrize("prec", ["bf16", "fp8"])
@pytest.mark.parametrize("row_tiles", [1, 2])
@pytest.mark.parametrize("shortlist_k", [8, 12, 16, 2])
def test_tuning_grid_points(matcher, tune_zone, prec, row_tiles, shortlist_k):
    """Every setting the autotuner can pick gives the oracle's lists (shortlist
    capacity 2 records per row half, below the grid, forces overflows: those
    rows are scanned exactly)."""
    z, want = tune_zone
    st = matcher.store(int(z.counts.sum()), len(z.counts))
    st.add_views_packed(z.desc, z.offsets, z.counts)
    for ipsm in (2, 8):
        plan = st.plan(z.pairs, 0.8, True, prec, items_per_sm=ipsm, row_tiles=row_tiles, shortlist_k=shortlist_k)
        plan.launch()
        per = plan.per_pair()
        for k in range(len(z.pairs)):
            assert np.array_equal(per[k], want[k]), (ipsm, k)
        if shortlist_k == 2 and prec == "bf16":
            assert plan.stats["rows_recomputed"] > 0  # overflowed rows went to the exact scan
        plan.close()
    st.close()


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_autotuned_plan(matcher, prec):
    z = synth.zone(positions=6, n_range=(200, 1000), seed=17)
    st = matcher.store(int(z.counts.sum()), len(z.counts))
    st.add_views_packed(z.desc, z.offsets, z.counts)
    best, ms = st.autotune(z.pairs, 0.8, True, prec)
    assert ms > 0 and best["items_per_sm"] in (2, 4, 8)
    if prec != "fp32":
        assert best["shortlist_k"] in (8, 12, 16) and best["row_tiles"] in (1, 2)
    plan = st.plan(z.pairs, 0.8, True, prec, autotune=True)
    plan.launch()
    per = plan.per_pair()
    for k, (u, v) in enumerate(z.pairs):
        assert np.array_equal(per[k], O.ratio_match_np(z.view(int(u)), z.view(int(v)), 0.8, True, threads=16)), k
    plan.close()
    st.close()


def test_auto_precision(matcher):
    """SLM_PREC_AUTO: the plain FP32 kernel below SLM_AUTO_BF16_DISTANCES, the
    BF16 shortlist from there up (3 kernels per call, and more than 10);
    exact both ways."""
    for n, path in ((800, "fp32"), (3500, "bf16")):
        a, b = synth.pair_large(n, 0.5, 0.05, seed=n)
        got = matcher.ratio_match_np(a, b, 0.8, True, "auto")
        launches = matcher.last_stats["kernel_launches"]
        assert (launches < 10) == (path == "fp32"), (n, launches)
        assert np.array_equal(got, O.ratio_match_np(a, b, 0.8, True, threads=16)), n
    z = synth.zone(positions=4, n_range=(100, 300), seed=43)  # a small batch: 2.4M distances in total
    st = matcher.store(int(z.counts.sum()), len(z.counts))
    st.add_views_packed(z.desc, z.offsets, z.counts)
    plan = st.plan(z.pairs, 0.8, True, "auto")
    plan.launch()
    got = plan.per_pair()
    assert plan.stats["kernel_launches"] < 10
    for k, (u, v) in enumerate(z.pairs):
        assert np.array_equal(got[k], O.ratio_match_np(z.view(int(u)), z.view(int(v)), 0.8, True, threads=8))
    plan.close()
    st.close()


@pytest.mark.parametrize("seed", [101, 102, 103])
def test_random_batches(matcher, prec, seed):
    """Seeded random batches: views of 0-700 rows built from a shared pool of
    descriptors (exact duplicates, near-duplicates at sigma 0.001-0.05, fresh
    draws), random pairs including self-pairs and repeats, both mutual
    settings; every pair's list equals the oracle's."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pool = synth.sift_like(rng, 3000)
    views = []
    for _ in range(24):
        n = int(rng.choice([0, 1, 2, 3, 17, 127, 128, 129]) if rng.random() < 0.3 else rng.integers(30, 701))
        src = pool[rng.integers(0, len(pool), size=n)]
        kind = rng.random(n)
        sig = rng.choice([0.001, 0.01, 0.05], size=n).astype(np.float32)
        noisy = synth.noisy_copy(rng, src, sig)
        fresh = synth.sift_like(rng, n)
        v = np.where(kind[:, None] < 0.3, src, np.where(kind[:, None] < 0.8, noisy, fresh)).astype(np.float32)
        views.append(np.ascontiguousarray(v))
    counts = np.array([len(v) for v in views], np.int64)
    offsets = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int64)
    desc = np.concatenate([v for v in views if len(v)] or [np.zeros((0, 128), np.float32)]).astype(np.float32)
    pairs = rng.integers(0, len(views), size=(60, 2)).astype(np.uint32)
    st = matcher.store(int(counts.sum()), len(views))
    st.add_views_packed(desc, offsets, counts)
    for mutual in (True, False):
        ratio = 0.8 if mutual else 0.95
        plan = st.plan(pairs, ratio, mutual, prec)
        plan.launch()
        got = plan.per_pair()
        for k, (u, v) in enumerate(pairs):
            want = O.ratio_match_np(views[int(u)], views[int(v)], ratio, mutual, threads=8)
            assert np.array_equal(got[k], want), (prec, seed, mutual, k, int(u), int(v))
        plan.close()
    st.close()


def test_single_call_input_alignment(matcher, prec):
    """Single calls read 16-byte-aligned host inputs where they lie (when the
    device can read pageable memory) and copy the others first; both give the
    reference's lists."""
    a, b = synth.pair_800(3)
    want = O.ratio_match_np(a, b, 0.8, True, threads=8)
    for shift_a, shift_b in ((0, 0), (1, 0), (0, 3), (2, 2)):
        ba = np.empty(a.size + 4, np.float32)
        bb = np.empty(b.size + 4, np.float32)
        ua = ba[shift_a:shift_a + a.size].reshape(a.shape)
        ub = bb[shift_b:shift_b + b.size].reshape(b.shape)
        ua[...] = a
        ub[...] = b
        assert np.array_equal(matcher.ratio_match_np(ua, ub, 0.8, True, prec), want), (shift_a, shift_b)
