"""Descriptor producer on the GPU: detect_and_describe and describe of
crates/core/src/features.rs (:594 and :509) through libslm's C ABI.

Images are gray f32 arrays of h x w (GrayImage::data) or h x w x 3 uint8 RGB
(GrayImage::from_rgb); a batch of images of one size runs in one call.
Keypoints come back as (n, 5) float32 arrays (x, y, sigma, response, angle),
descriptors as (n, 128) float32.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import SlmDetectorConfig, SlmKeypoint, check

P = ctypes.POINTER


def detector_config(**overrides) -> SlmDetectorConfig:
    """DetectorConfig::default() (features.rs:278-293) with fields replaced."""
    from ._lib import load
    cfg = SlmDetectorConfig()
    load().slm_detector_config_default(ctypes.byref(cfg))
    for k, v in overrides.items():
        if not hasattr(cfg, k):
            raise TypeError(f"DetectorConfig has no field {k}")
        setattr(cfg, k, int(v) if k != "sigma0" and k not in ("contrast", "edge_ratio") else float(v))
    return cfg


def detect_and_describe(matcher, images, cfg: SlmDetectorConfig | None = None):
    """slm_detect_and_describe(_rgb8) over a batch of images of one size.
    images: (h, w) or (n, h, w) float32, or (h, w, 3) / (n, h, w, 3) uint8.
    Returns a list of (keypoints (k, 5), descriptors (k, 128)), one per image."""
    L = matcher._L
    imgs = np.asarray(images)
    rgb = imgs.dtype == np.uint8
    if rgb:
        if imgs.ndim == 3:
            imgs = imgs[None]
        imgs = np.ascontiguousarray(imgs, dtype=np.uint8)
        n, h, w, ch = imgs.shape
        if ch != 3:
            raise ValueError("RGB images need 3 channels")
    else:
        if imgs.ndim == 2:
            imgs = imgs[None]
        imgs = np.ascontiguousarray(imgs, dtype=np.float32)
        n, h, w = imgs.shape
    cfg = cfg or detector_config()
    cap = max(1, n * int(cfg.max_features))
    kps = np.empty((cap, 5), np.float32)
    desc = np.empty((cap, 128), np.float32)
    off = np.zeros(n + 1, np.uint64)
    fn = L.slm_detect_and_describe_rgb8 if rgb else L.slm_detect_and_describe
    check(fn(matcher.handle, ctypes.c_void_p(imgs.ctypes.data), n, w, h, ctypes.byref(cfg),
             ctypes.c_void_p(kps.ctypes.data), ctypes.c_void_p(desc.ctypes.data), cap,
             off.ctypes.data_as(P(ctypes.c_uint64))), "slm_detect_and_describe")
    return [(kps[int(off[k]):int(off[k + 1])].copy(), desc[int(off[k]):int(off[k + 1])].copy()) for k in range(n)]


def describe(matcher, img, keypoints) -> np.ndarray:
    """slm_describe: descriptors of keypoints (k, 5) or (k, 4) (x, y, sigma,
    angle for 4 columns) of one gray image -> (k, 128)."""
    img = np.ascontiguousarray(img, dtype=np.float32)
    kp = np.asarray(keypoints, dtype=np.float32)
    if kp.ndim == 1:
        kp = kp[None]
    if kp.shape[1] == 4:
        kp = np.stack([kp[:, 0], kp[:, 1], kp[:, 2], np.zeros(len(kp), np.float32), kp[:, 3]], axis=1)
    kp = np.ascontiguousarray(kp, dtype=np.float32)
    out = np.empty((max(len(kp), 1), 128), np.float32)
    check(matcher._L.slm_describe(matcher.handle, ctypes.c_void_p(img.ctypes.data), img.shape[1], img.shape[0],
                                  ctypes.c_void_p(kp.ctypes.data), len(kp), ctypes.c_void_p(out.ctypes.data)),
          "slm_describe")
    return out[:len(kp)]
