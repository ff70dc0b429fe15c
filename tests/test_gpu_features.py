"""GPU: the descriptor producer (slm_detect_and_describe, slm_describe)
against the oracle's restatement of crates/core/src/features.rs.

The GPU evaluates the reference's per-pixel and per-keypoint exp, atan2,
powf, cos and sin correctly rounded; the oracle's `cr=True` mode does the
same, so keypoints and descriptors must equal it bit for bit (tolerance 0).
Every other f32 operation is the reference's, in its order. Cases: the
reference's own feature tests (blob position and scale, sub-pixel centres,
orientation under rotation), textured scenes at the pipeline's 960 x 540 and
small sizes that take the 2x upsampled detection, batches of several images,
configurations (no upsampling, a small max_features cut with tied responses,
fewer octaves and scales, another contrast), tiny and empty images, RGB8
input against the gray conversion, and describe() on given keypoints.
"""
import numpy as np
import pytest

import oracle as O
from skylens_match import SlmError, synth
from skylens_match import features as F

pytestmark = pytest.mark.gpu


def ocfg(c):
    return O.DetectorConfig(c.octaves, c.scales, c.sigma0, c.contrast, c.edge_ratio, c.max_features,
                            c.upscale_below, c.upscale_fill)


def blob(w, h, cx, cy, s):
    """features.rs tests' blob image: 0.2 + 0.6 exp(-r^2 / (2 s^2)) (the
    exponential here is numpy's; the image is an input like any other)."""
    y, x = np.mgrid[0:h, 0:w].astype(np.float32)
    r2 = (x - cx) ** 2 + (y - cy) ** 2
    return (0.2 + 0.6 * np.exp(-r2 / (2 * s * s))).astype(np.float32)


def check_equal(got, img, cfg):
    kp, desc = O.detect_and_describe(img, ocfg(cfg), cr=True)
    gk, gd = got
    assert len(gk) == len(kp), (len(gk), len(kp))
    assert np.array_equal(gk.view(np.uint32), kp.view(np.uint32))
    assert np.array_equal(gd.view(np.uint32), desc.view(np.uint32))
    return len(kp)


@pytest.mark.parametrize("sb,cx,cy", [(4.0, 61.0, 47.0), (8.0, 70.0, 66.0), (4.0, 61.3, 47.6), (4.0, 60.75, 48.2)])
def test_blob_detection_matches_oracle(matcher, sb, cx, cy):
    img = blob(140, 120, cx, cy, sb)
    cfg = F.detector_config()
    got = F.detect_and_describe(matcher, img, cfg)[0]
    n = check_equal(got, img, cfg)
    assert n > 0
    best = got[0][0]
    # the reference's properties (features.rs:846-885)
    assert np.hypot(best[0] - cx, best[1] - cy) < 0.1
    assert abs(best[2] / sb * 2 ** (1 / 6) - 1.0) < 0.03


def test_scene_960x540_batch(matcher):
    views = synth.scene_views(3, 960, 540, seed=11)
    cfg = F.detector_config()
    got = F.detect_and_describe(matcher, views, cfg)
    total = 0
    for k in range(3):
        total += check_equal(got[k], O.gray_from_rgb8(views[k]), cfg)
    assert total > 1000
    # descriptors are unit length, clipped at 0.2 before the second normalisation
    d = np.concatenate([g[1] for g in got])
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-5)
    assert d.min() >= 0.0 and d.max() < 0.35


def test_gray_and_rgb_entry_points_agree(matcher):
    views = synth.scene_views(2, 320, 200, seed=3)
    gray = np.stack([O.gray_from_rgb8(v) for v in views])
    a = F.detect_and_describe(matcher, views)
    b = F.detect_and_describe(matcher, gray)
    for (ka, da), (kb, db) in zip(a, b):
        assert np.array_equal(ka, kb) and np.array_equal(da, db)


@pytest.mark.parametrize("w,h,seed", [(240, 180, 5), (160, 120, 6), (10, 10, 7), (17, 33, 8), (15, 15, 9)])
def test_small_images_take_the_upsampled_detection(matcher, w, h, seed):
    img = O.gray_from_rgb8(synth.scene_views(1, w, h, seed=seed)[0])
    cfg = F.detector_config()
    check_equal(F.detect_and_describe(matcher, img, cfg)[0], img, cfg)


@pytest.mark.parametrize("over", [dict(upscale_below=0), dict(max_features=40), dict(max_features=1),
                                  dict(octaves=2, scales=2), dict(scales=4, sigma0=1.2),
                                  dict(contrast=0.02, edge_ratio=5.0), dict(upscale_fill=1, max_features=300),
                                  dict(octaves=0)])
def test_configurations(matcher, over):
    views = synth.scene_views(2, 300, 220, seed=12)
    cfg = F.detector_config(**over)
    got = F.detect_and_describe(matcher, views, cfg)
    for k in range(2):
        check_equal(got[k], O.gray_from_rgb8(views[k]), cfg)


def test_tied_responses_keep_the_reference_order(matcher):
    # a symmetric pattern: mirrored blobs give equal |response| in several places,
    # so the stable sort's tie order (emission order) decides the list
    img = np.full((96, 128), 0.3, np.float32)
    for cx, cy in [(30, 30), (97, 30), (30, 65), (97, 65)]:
        img += blob(128, 96, cx, cy, 3.0) - 0.2
    cfg = F.detector_config(max_features=6, upscale_below=0)
    check_equal(F.detect_and_describe(matcher, img, cfg)[0], img, cfg)


def test_empty_batches_and_images(matcher):
    assert F.detect_and_describe(matcher, np.zeros((0, 50, 50), np.float32)) == []
    k, d = F.detect_and_describe(matcher, np.zeros((1, 0), np.float32))[0]
    assert len(k) == 0 and len(d) == 0
    flat = np.full((64, 64), 0.5, np.float32)  # no extrema anywhere
    k, d = F.detect_and_describe(matcher, flat)[0]
    assert len(k) == 0


def test_describe_given_keypoints(matcher):
    rng = np.random.default_rng(4)
    img = O.gray_from_rgb8(synth.scene_views(1, 200, 150, seed=4)[0])
    kps = np.stack([rng.uniform(-5, 205, 64), rng.uniform(-5, 155, 64), rng.uniform(0.8, 9.0, 64),
                    np.zeros(64), rng.uniform(0, 2 * np.pi, 64)], 1).astype(np.float32)
    got = F.describe(matcher, img, kps)
    for i in range(64):
        ref = O.describe(img, *kps[i, [0, 1, 2, 4]], cr=True)
        assert np.array_equal(got[i].view(np.uint32), ref.view(np.uint32)), i


def test_orientation_follows_rotation(matcher):
    # features.rs:887-917: a ramp rising along theta plus an unrelated blob;
    # the dominant orientation at the centre is within 3 degrees of theta
    worst = 0.0
    for k in range(12):
        th = np.float32(k * np.deg2rad(30.0) + 0.1)
        img = blob(128, 128, 64.0, 64.0, 6.0)
        y, x = np.mgrid[0:128, 0:128].astype(np.float32)
        img = img + np.float32(0.02) * ((x - 64.0) * np.cos(th) + (y - 64.0) * np.sin(th))
        g = O.gaussian_blur(img.astype(np.float32), 2.0)
        oris = O.dominant_orientations(g, 64.0, 64.0, 4.0, cr=True)
        d = np.abs((oris - th + np.pi) % (2 * np.pi) - np.pi)
        worst = max(worst, float(d.min()))
        # the descriptor of each orientation on the GPU equals the oracle's
        kps = np.array([[64.0, 64.0, 4.0, 0.0, a] for a in oris], np.float32)
        got = F.describe(matcher, g, kps)
        for i, a in enumerate(oris):
            assert np.array_equal(got[i], O.describe(g, 64.0, 64.0, 4.0, a, cr=True))
    assert np.rad2deg(worst) < 3.0


def test_argument_checks(matcher):
    img = np.zeros((20, 20), np.float32)
    with pytest.raises(SlmError):
        F.detect_and_describe(matcher, img, F.detector_config(scales=0))
    with pytest.raises(SlmError):
        F.detect_and_describe(matcher, img, F.detector_config(sigma0=-1.0))
    with pytest.raises(SlmError):
        F.describe(matcher, img, np.array([[5, 5, 0.0, 0.0, 0.0]], np.float32))  # sigma 0
    with pytest.raises(SlmError):
        F.describe(matcher, img, np.array([[5, 5, 1.0, 0.0, np.inf]], np.float32))


def test_images_to_store_to_matches_on_the_device(matcher):
    """The pipeline's load -> match_pairs chain without descriptors crossing to
    the host: detect_and_describe writes descriptors to device memory, the
    store takes them from there, and a BF16 batch matches the views; the lists
    equal ratio_match on the same features (oracle)."""
    import ctypes

    import torch

    import skylens_match as sm
    views = synth.scene_views(4, 480, 270, seed=17)
    cfg = F.detector_config()
    n, cap = len(views), len(views) * int(cfg.max_features)
    d_img = torch.from_numpy(views).cuda()
    d_desc = torch.empty((cap, 128), dtype=torch.float32, device="cuda")
    kps = np.empty((cap, 5), np.float32)
    off = np.zeros(n + 1, np.uint64)
    st = matcher._L.slm_detect_and_describe_rgb8(matcher.handle, ctypes.c_void_p(d_img.data_ptr()), n, 480, 270,
                                                 ctypes.byref(cfg), ctypes.c_void_p(kps.ctypes.data),
                                                 ctypes.c_void_p(d_desc.data_ptr()), cap,
                                                 off.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
    assert st == 0
    counts = np.diff(off).astype(np.uint32)
    assert counts.min() > 20
    store = sm.DescriptorStore(matcher, int(off[-1]) + 1024, n)
    ids = store.add_views_ptr(d_desc.data_ptr(), off[:-1], counts)
    pairs = [(0, 1), (1, 2), (0, 2), (2, 3), (0, 3)]
    plan = store.plan(pairs, 0.8, True, "bf16")
    plan.launch()
    res, roff = plan.results()
    got = [res[int(roff[k]):int(roff[k + 1])] for k in range(len(pairs))]
    host = d_desc.cpu().numpy()
    for k, (u, v) in enumerate(pairs):
        a = host[int(off[ids[u]]):int(off[ids[u] + 1])]
        b = host[int(off[ids[v]]):int(off[ids[v] + 1])]
        want = O.ratio_match_np(a, b, 0.8, True, threads=8)
        assert np.array_equal(got[k], want), (u, v)
    # neighbouring views share the scene: many matches
    assert len(got[0]) > 50
    plan.close()
    store.close()


@pytest.mark.parametrize("n,w,h,seed", [(5, 320, 200, 31), (4, 150, 110, 32), (9, 64, 48, 33)])
def test_batches_split_over_two_workspaces(matcher, n, w, h, seed):
    # from 4 images a call runs its two halves on two workspaces; the features
    # come back in image order, each image's equal to the oracle's (the small
    # sizes take the upsampled detection in both halves)
    views = synth.scene_views(n, w, h, seed=seed)
    cfg = F.detector_config()
    got = F.detect_and_describe(matcher, views, cfg)
    assert len(got) == n
    for k in range(n):
        check_equal(got[k], O.gray_from_rgb8(views[k]), cfg)


def test_candidate_overflow_reruns_with_room(matcher):
    # a dense texture of 2400 x 2400 with the contrast test off gives about
    # 23,000 refined extrema (23,182 distinct keypoints in the oracle), more
    # than the first candidate buffer of a one-image call holds (16,384): the
    # library runs the pyramid again with room for all of them, and the list
    # (cut at max_features) equals the oracle's
    img = synth.scene_canvas(2400, 2400, seed=41, density=0.012)
    cfg = F.detector_config(contrast=0.0, edge_ratio=1000.0, upscale_below=0)
    got = F.detect_and_describe(matcher, img, cfg)[0]
    assert len(got[0]) == int(cfg.max_features)
    check_equal(got, img, cfg)
