"""GPU: slm_sampson_score, the RANSAC stage's hypothesis scoring.

Counts and inlier masks of essential-matrix hypotheses over each pair's
matches must equal the oracle's bit for bit (two_view.rs:456-465, 804-823):
pairs of 0 to 1000 matches (32-match groups, ragged ends), hypotheses from the
true matrix to random and degenerate ones, thresholds set exactly on a match's
residual (the strict `<` decides), masks for some hypotheses only, and
malformed arguments refused before any launch.
"""
import ctypes

import numpy as np
import pytest

import oracle as O
from skylens_match import SlmError, synth

pytestmark = pytest.mark.gpu


def batch(seed, sizes, hyps_per_pair, boundary=False):
    rng = np.random.default_rng(seed)
    pts, off, th, hyps, hp = [], [0], [], [], []
    for p, n in enumerate(sizes):
        n1, n2, e = synth.two_view(rng, max(n, 1), inlier_frac=rng.uniform(0.2, 0.9))
        pp = np.concatenate([n1, n2], 1)[:n]
        pts.append(pp)
        off.append(off[-1] + n)
        t = 1.5 / 800.0
        if boundary and n:
            # the threshold exactly on one match's residual under the true matrix
            t = abs(O.sampson_residual(e, pp[n // 2, :2], pp[n // 2, 2:]))
        th.append(t)
        h = synth.essential_hypotheses(rng, e, hyps_per_pair)
        hyps.append(h)
        hp += [p] * len(h)
    return (np.concatenate(pts) if pts else np.zeros((0, 4))), np.asarray(off, np.uint64), np.asarray(th), \
        np.concatenate(hyps), np.asarray(hp, np.uint32)


@pytest.mark.parametrize("boundary", [False, True])
def test_counts_and_masks_equal_the_oracle(matcher, boundary):
    sizes = [0, 1, 5, 31, 32, 33, 64, 100, 257, 1000]
    pts, off, th, hyps, hp = batch(7 + boundary, sizes, 40, boundary)
    masks_for = list(range(0, len(hyps), 5))
    got, gm = matcher.sampson_score(pts, off, th, hyps, hp, masks_for=masks_for)
    mo = np.full(len(hyps), 2**64 - 1, np.uint64)
    words = 0
    for h in masks_for:
        mo[h] = words
        words += (int(off[hp[h] + 1] - off[hp[h]]) + 31) // 32
    want, wm = O.sampson_score(pts, off, th, hyps, hp, mask_off=mo, threads=8)
    assert np.array_equal(got, want)
    for h in masks_for:
        n = int(off[hp[h] + 1] - off[hp[h]])
        bits = np.unpackbits(wm[int(mo[h]):int(mo[h]) + (n + 31) // 32].view(np.uint8), bitorder="little")[:n]
        assert np.array_equal(gm[h], bits.astype(bool)), h
    if boundary:
        # the match whose residual is the threshold is not an inlier of the
        # true matrix (hypothesis 0 of each pair; strict <)
        for p, n in enumerate(sizes):
            if n:
                assert not gm[40 * p][n // 2], p


def test_large_batch_equals_the_oracle(matcher):
    """A block of RANSAC iterations for 40 pairs: 500 hypotheses each."""
    rng = np.random.default_rng(11)
    sizes = rng.integers(20, 800, 40).tolist()
    pts, off, th, hyps, hp = batch(12, sizes, 500)
    got, _ = matcher.sampson_score(pts, off, th, hyps, hp)
    want, _ = O.sampson_score(pts, off, th, hyps, hp, threads=16)
    assert np.array_equal(got, want)
    assert (got == np.asarray([off[p + 1] - off[p] for p in hp])).sum() >= 40  # the zero matrices count all


def test_bad_arguments_are_refused(matcher):
    pts, off, th, hyps, hp = batch(13, [10, 20], 4)
    bad = hp.copy()
    bad[0] = 2
    with pytest.raises(SlmError):
        matcher.sampson_score(pts, off, th, hyps, bad)
    with pytest.raises(SlmError):
        matcher.sampson_score(pts, np.asarray([0, 20, 10], np.uint64), th, hyps, hp)
    L = matcher._L
    counts = np.zeros(len(hyps), np.uint32)
    mo = np.zeros(len(hyps), np.uint64)  # every mask at word 0 of a 0-word buffer: does not fit
    P = ctypes.POINTER
    st = L.slm_sampson_score(matcher.handle, pts.ctypes.data_as(P(ctypes.c_double)), off.ctypes.data_as(P(ctypes.c_uint64)),
                             2, th.ctypes.data_as(P(ctypes.c_double)), hyps.ctypes.data_as(P(ctypes.c_double)),
                             hp.ctypes.data_as(P(ctypes.c_uint32)), len(hyps), counts.ctypes.data_as(P(ctypes.c_uint32)),
                             mo.ctypes.data_as(P(ctypes.c_uint64)), counts.ctypes.data_as(P(ctypes.c_uint32)), 0)
    assert st == 1  # SLM_INVALID_ARG
