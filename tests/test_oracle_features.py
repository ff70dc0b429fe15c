"""CPU: the oracle's restatement of the descriptor producer
(oracle/features.c, crates/core/src/features.rs).

The reference's feature tests are property tests (features.rs:820-1130; no
golden vectors), so they pin the restatement's behaviour, not its bits: blur
of a constant image, blob position and scale with sub-pixel refinement,
orientation under rotation, repeatability and matching under rotation and
scale with the reference's thresholds, unit-length descriptors. Their scenes
here are this repository's seeded textures, resampled exactly (the
reference's textures are its test code). The oracle runs with the platform's
float functions (`cr=False`, what the reference calls) and correctly rounded
ones (`cr=True`, what the GPU computes); the two agree within a few ulps.
"""
import numpy as np
import pytest

import oracle as O
from skylens_match import synth


def blob(w, h, cx, cy, s):
    y, x = np.mgrid[0:h, 0:w].astype(np.float32)
    r2 = (x - cx) ** 2 + (y - cy) ** 2
    return (0.2 + 0.6 * np.exp(-r2 / (2 * s * s))).astype(np.float32)


_BIG = {}


def warped(w, h, th, sc, seed=7):
    """A w x h view of an 800 x 800 texture rotated by th and scaled by sc
    about the centre, bilinear resampling."""
    if seed not in _BIG:
        _BIG[seed] = synth.scene_canvas(800, 800, seed=seed, density=0.003)
    big = _BIG[seed]
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    fx, fy = x - w / 2.0, y - h / 2.0
    c, s = np.cos(th), np.sin(th)
    ox = (c * fx + s * fy) / sc + 400.0
    oy = (-s * fx + c * fy) / sc + 400.0
    x0, y0 = np.floor(ox).astype(int), np.floor(oy).astype(int)
    ax, ay = ox - x0, oy - y0
    at = lambda xx, yy: big[np.clip(yy, 0, 799), np.clip(xx, 0, 799)]
    v = (1 - ay) * ((1 - ax) * at(x0, y0) + ax * at(x0 + 1, y0)) + ay * ((1 - ax) * at(x0, y0 + 1) + ax * at(x0 + 1, y0 + 1))
    return v.astype(np.float32)


def test_blur_preserves_constant():
    img = np.full((10, 20), 0.7, np.float32)
    assert np.all(np.abs(O.gaussian_blur(img, 2.0) - 0.7) < 1e-5)
    k = O.blur_taps(1.6)
    assert len(k) == 2 * 5 + 1 and abs(float(k.sum()) - 1.0) < 1e-6


@pytest.mark.parametrize("cr", [False, True])
def test_blob_position_scale_and_subpixel(cr):
    for sb, cx, cy in [(4.0, 61.0, 47.0), (8.0, 70.0, 66.0)]:
        kp, _ = O.detect_and_describe(blob(140, 120, cx, cy, sb), cr=cr)
        b = kp[0]
        err = np.hypot(b[0] - cx, b[1] - cy)
        assert err < 0.1
        assert abs(b[2] / sb * 2 ** (1 / 6) - 1.0) < 0.03
    for cx, cy in [(61.3, 47.6), (60.75, 48.2)]:
        kp, _ = O.detect_and_describe(blob(140, 120, cx, cy, 4.0), cr=cr)
        assert np.hypot(kp[0, 0] - cx, kp[0, 1] - cy) < 0.1


def test_orientation_follows_rotation():
    worst = 0.0
    for k in range(12):
        th = np.float32(k * np.deg2rad(30.0) + 0.1)
        img = blob(128, 128, 64.0, 64.0, 6.0)
        y, x = np.mgrid[0:128, 0:128].astype(np.float32)
        img = (img + np.float32(0.02) * ((x - 64.0) * np.cos(th) + (y - 64.0) * np.sin(th))).astype(np.float32)
        oris = O.dominant_orientations(O.gaussian_blur(img, 2.0), 64.0, 64.0, 4.0)
        d = np.abs((oris - th + np.pi) % (2 * np.pi) - np.pi)
        worst = max(worst, float(d.min()))
    assert np.rad2deg(worst) < 3.0


def _map(kp, th, sc, w, h):
    c, s = np.cos(th), np.sin(th)
    fx, fy = kp[:, 0] - w / 2.0, kp[:, 1] - h / 2.0
    return sc * (c * fx - s * fy) + w / 2.0, sc * (s * fx + c * fy) + h / 2.0


@pytest.mark.parametrize("deg,sc,min_rate", [(0.0, 1.0, 0.99), (30.0, 1.0, 0.85), (90.0, 1.0, 0.95),
                                             (45.0, 0.8, 0.70), (0.0, 1.25, 0.70)])
def test_repeatability_under_rotation_and_scale(deg, sc, min_rate):
    th = np.deg2rad(deg)
    a, _ = O.detect_and_describe(warped(240, 240, 0.0, 1.0))
    b, _ = O.detect_and_describe(warped(240, 240, th, sc))
    ex, ey = _map(a, th, sc, 240, 240)
    inside = (ex >= 16) & (ey >= 16) & (ex <= 224) & (ey <= 224)
    assert inside.sum() >= 30
    d = np.hypot(b[None, :, 0] - ex[inside, None], b[None, :, 1] - ey[inside, None])
    assert (d.min(1) < 2.0).mean() >= min_rate


@pytest.mark.parametrize("deg,sc", [(0.0, 1.0), (30.0, 1.0), (90.0, 1.0), (45.0, 0.8), (0.0, 1.25)])
def test_matching_under_rotation_and_scale(deg, sc):
    th = np.deg2rad(deg)
    cfg = O.DetectorConfig(upscale_below=0)
    ka, da = O.detect_and_describe(warped(240, 240, 0.0, 1.0), cfg)
    kb, db = O.detect_and_describe(warped(240, 240, th, sc), cfg)
    m = O.ratio_match_np(da, db, 0.8, False)
    assert len(m) >= 40
    ex, ey = _map(ka[m[:, 0]], th, sc, 240, 240)
    good = np.hypot(kb[m[:, 1], 0] - ex, kb[m[:, 1], 1] - ey) < 2.0
    assert good.mean() >= 0.95


def test_descriptors_unit_length_and_both_modes_agree():
    img = O.gray_from_rgb8(synth.scene_views(1, 320, 240, seed=21)[0])
    k0, d0 = O.detect_and_describe(img, cr=False)
    k1, d1 = O.detect_and_describe(img, cr=True)
    assert len(k0) > 50
    n = np.linalg.norm(d0, axis=1)
    assert np.all(np.abs(n - 1.0) < 1e-4) and d0.min() >= 0.0
    # the platform's float functions against correctly rounded ones: the same
    # keypoints (positions and responses exactly), scales and angles within a
    # few ulps, descriptors within 1e-6
    assert len(k0) == len(k1)
    assert np.array_equal(k0[:, [0, 1, 3]], k1[:, [0, 1, 3]])
    assert np.allclose(k0[:, [2, 4]], k1[:, [2, 4]], rtol=4e-7, atol=0)
    assert np.abs(d0 - d1).max() <= 1e-6
