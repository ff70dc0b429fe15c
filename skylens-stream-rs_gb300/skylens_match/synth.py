"""Seeded synthetic descriptor workloads (no dataset is involved).

SIFT-like descriptors follow the reference's normalisation (features.rs:575-582):
per component |N(0,1)|, L2-normalise (f32), clip at 0.2, L2-normalise again.
A "noisy copy" adds N(0, sigma) per component and normalises the same way.
Random numbers come from numpy's PCG64 seeded with the workload seed.

Workloads (sizes as named by the benchmark configurations):
  pair_800        800 vs 800: 480 noisy permuted copies (sigma 0.05) + 320 fresh
  pair_large      n vs n, a fraction of true correspondences (8192, 50 %)
  pair_fp8        n vs n, 40 % true, sigma ~ U[0.02, 0.08] per copy (32768)
  zone            3 cameras x P positions, n_v ~ U[300, 2000], candidate_pairs
                  (5, 4, 16); views share landmarks so that overlapping pairs
                  share 30-60 % of their descriptors
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

CLIP = np.float32(0.2)


def _normalise(x: np.ndarray) -> np.ndarray:
    x = x.astype(np.float32, copy=False)
    n = np.sqrt(np.sum(x * x, axis=1, dtype=np.float32), dtype=np.float32)
    n = np.where(n > 0, n, np.float32(1))
    x = x / n[:, None]
    x = np.minimum(x, CLIP)
    n = np.sqrt(np.sum(x * x, axis=1, dtype=np.float32), dtype=np.float32)
    n = np.where(n > 0, n, np.float32(1))
    return np.ascontiguousarray((x / n[:, None]).astype(np.float32))


def sift_like(rng: np.random.Generator, n: int) -> np.ndarray:
    """n SIFT-like unit descriptors (n, 128) float32."""
    return _normalise(np.abs(rng.standard_normal((n, 128), dtype=np.float32)))


def noisy_copy(rng: np.random.Generator, x: np.ndarray, sigma) -> np.ndarray:
    """Each row + N(0, sigma) per component, re-normalised; sigma scalar or per row."""
    sig = np.asarray(sigma, dtype=np.float32)
    if sig.ndim == 1:
        sig = sig[:, None]
    return _normalise(x + rng.standard_normal(x.shape, dtype=np.float32) * sig)


def pair_800(seed: int = 0):
    """800 vs 800: B = 480 noisy copies of a random permutation of A's rows
    (sigma 0.05) plus 320 fresh draws, rows of B shuffled."""
    rng = np.random.Generator(np.random.PCG64(seed))
    a = sift_like(rng, 800)
    perm = rng.permutation(800)[:480]
    b = np.concatenate([noisy_copy(rng, a[perm], 0.05), sift_like(rng, 320)])
    order = rng.permutation(len(b))
    return a, np.ascontiguousarray(b[order])


def pair_large(n: int = 8192, true_frac: float = 0.5, sigma=0.05, seed: int = 2):
    """n vs n with round(true_frac*n) true correspondences (noisy copies)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    a = sift_like(rng, n)
    k = int(round(true_frac * n))
    src = rng.permutation(n)[:k]
    if isinstance(sigma, tuple):
        sig = rng.uniform(sigma[0], sigma[1], size=k).astype(np.float32)
    else:
        sig = sigma
    b = np.concatenate([noisy_copy(rng, a[src], sig), sift_like(rng, n - k)])
    order = rng.permutation(n)
    return a, np.ascontiguousarray(b[order])


def pair_fp8(n: int = 32768, seed: int = 4):
    """n vs n, 40 % true correspondences with sigma ~ U[0.02, 0.08] per copy."""
    return pair_large(n, 0.4, (0.02, 0.08), seed)


def rig_views(positions: int, cameras: int = 3):
    """(camera, position) of every view, id = cameras*pos + cam (synth.rs:284-291)."""
    return [(c, p) for p in range(positions) for c in range(cameras)]


@dataclass
class Zone:
    views: list            # (cam, pos) per view
    desc: np.ndarray       # all descriptors, (N, 128) float32
    offsets: np.ndarray    # first row of each view (uint64)
    counts: np.ndarray     # rows per view (uint32)
    pairs: np.ndarray      # (P, 2) view-id pairs from candidate_pairs
    landmark: np.ndarray   # landmark id of each row (-1: unique to the view)

    def view(self, v: int) -> np.ndarray:
        o, n = int(self.offsets[v]), int(self.counts[v])
        return self.desc[o:o + n]

    @property
    def distances(self) -> int:
        c = self.counts.astype(np.int64)
        return int(np.sum(c[self.pairs[:, 0]] * c[self.pairs[:, 1]]))

    def overlap(self, u: int, v: int) -> float:
        """Shared landmarks / min(n_u, n_v)."""
        lu = self.landmark[int(self.offsets[u]):int(self.offsets[u]) + int(self.counts[u])]
        lv = self.landmark[int(self.offsets[v]):int(self.offsets[v]) + int(self.counts[v])]
        s = len(np.intersect1d(lu[lu >= 0], lv[lv >= 0]))
        return s / max(1, min(len(lu), len(lv)))


def candidate_pairs_np(views, temporal=5, cross=4, pow2_max=16) -> np.ndarray:
    """Vectorised candidate_pairs (same rule as matching.rs:18-40) for workload setup."""
    v = np.asarray(views, dtype=np.int64)
    i, j = np.triu_indices(len(v), k=1)
    ca, pa, cb, pb = v[i, 0], v[i, 1], v[j, 0], v[j, 1]
    d = np.abs(pa - pb)
    pow2 = (d > 0) & ((d & (d - 1)) == 0)
    same = (ca == cb) & (d >= 1) & ((d <= temporal) | (pow2 & (d <= pow2_max)))
    other = (ca != cb) & (d <= cross)
    keep = same | other
    return np.stack([i[keep], j[keep]], axis=1).astype(np.uint32)


def zone(positions: int = 80, cameras: int = 3, n_range=(300, 2000), sigma: float = 0.05, seed: int = 3,
         n_sampler=None, lifetime: int = 40, shared_frac: float = 0.595, alive: int = 1500) -> Zone:
    """A zone of cameras x positions views whose overlapping pairs share landmarks.

    Landmarks live for `lifetime` consecutive positions and carry a strength;
    a view keeps its round(shared_frac * n_v) strongest live landmarks, each
    as a noisy copy with sigma/sqrt(2) per component (so two observations of
    one landmark differ by noise of sigma), and fills the rest with fresh
    descriptors. Two views g positions apart then share about
    shared_frac * (1 - g/lifetime) of the smaller view: 0.36-0.59 for the
    candidate_pairs gaps (1..5, 8, 16 on one camera; 0..4 across cameras).
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    views = rig_views(positions, cameras)
    nv = len(views)
    if n_sampler is None:
        counts = rng.integers(n_range[0], n_range[1] + 1, size=nv).astype(np.int64)
    else:
        counts = np.asarray(n_sampler(rng, nv), dtype=np.int64)
    births_per_pos = alive / lifetime
    first = -lifetime
    n_land = int(np.ceil((positions - first) * births_per_pos))
    birth = np.sort(rng.uniform(first, positions, size=n_land))
    strength = rng.random(n_land)
    base = sift_like(rng, n_land)
    sig_view = np.float32(sigma / np.sqrt(2.0))
    rows, lmk = [], []
    for v, (c, p) in enumerate(views):
        n = int(counts[v])
        live = np.nonzero((birth <= p) & (birth + lifetime > p))[0]
        k = min(len(live), int(round(shared_frac * n)))
        pick = live[np.argsort(-strength[live], kind="stable")[:k]]
        obs = noisy_copy(rng, base[pick], sig_view)
        fresh = sift_like(rng, n - k)
        d = np.concatenate([obs, fresh])
        lm = np.concatenate([pick, -np.ones(n - k, np.int64)])
        order = rng.permutation(n)
        rows.append(d[order])
        lmk.append(lm[order])
    desc = np.ascontiguousarray(np.concatenate(rows))
    offsets = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.uint64)
    pairs = candidate_pairs_np(views)
    return Zone(views, desc, offsets, counts.astype(np.uint32), pairs, np.concatenate(lmk))


def two_view(rng: np.random.Generator, n: int, inlier_frac: float = 0.6, noise_px: float = 0.5,
             focal: float = 800.0):
    """Calibrated two-view correspondences of a random scene, the input of the
    RANSAC stage (normalized coordinates, as pipeline.rs:497-498 forms them): a
    random pose (rotation of 3-20 degrees about a random axis, unit
    translation), points 4-10 units in front of both cameras, Gaussian pixel
    noise (noise_px / focal in normalized units), and (1 - inlier_frac) of the
    matches replaced by random points. Returns (n1 (n, 2), n2 (n, 2), E (3, 3)
    = [t]x R, row-major)."""
    ax = rng.normal(size=3)
    ax /= np.linalg.norm(ax)
    ang = rng.uniform(0.05, 0.35)
    k = np.array([[0.0, -ax[2], ax[1]], [ax[2], 0.0, -ax[0]], [-ax[1], ax[0], 0.0]])
    r = np.eye(3) + np.sin(ang) * k + (1.0 - np.cos(ang)) * (k @ k)
    t = rng.normal(size=3)
    t /= np.linalg.norm(t)
    x = np.stack([rng.uniform(-3, 3, n), rng.uniform(-3, 3, n), rng.uniform(4, 10, n)], 1)
    x2 = x @ r.T + 0.5 * t
    n1 = x[:, :2] / x[:, 2:3]
    n2 = x2[:, :2] / x2[:, 2:3]
    n1 = n1 + rng.normal(0.0, noise_px / focal, n1.shape)
    n2 = n2 + rng.normal(0.0, noise_px / focal, n2.shape)
    bad = rng.permutation(n)[: int(round(n * (1.0 - inlier_frac)))]
    if len(bad):
        lo, hi = n2.min(0), n2.max(0)
        n2[bad] = rng.uniform(lo, hi, (len(bad), 2))
    tx = np.array([[0.0, -t[2], t[1]], [t[2], 0.0, -t[0]], [-t[1], t[0], 0.0]])
    return n1, n2, tx @ r


def essential_hypotheses(rng: np.random.Generator, e_true: np.ndarray, count: int) -> np.ndarray:
    """Hypotheses like a RANSAC pool's: the true matrix, perturbations of it at
    scales 1e-6 .. 1e-1, random essential matrices, scaled copies and the zero
    matrix (whose residuals are all 0). (count, 3, 3) f64."""
    out = [e_true, np.zeros((3, 3)), 1e-3 * e_true, 1e3 * e_true]
    while len(out) < count:
        kind = len(out) % 3
        if kind == 0:
            out.append(e_true + rng.normal(0.0, 10.0 ** rng.uniform(-6, -1), (3, 3)))
        else:
            _, _, e = two_view(rng, 1)
            out.append(e * 10.0 ** rng.uniform(-2, 2))
    return np.asarray(out[:count], dtype=np.float64)


def scene_canvas(width: int, height: int, seed: int = 11, density: float = 0.004) -> np.ndarray:
    """A seeded textured scene for the descriptor producer: gaussian spots of
    radius 1.5-8 px and signed contrast over a slow brightness ramp, float32
    in [0, 1]. `density` spots per pixel."""
    rng = np.random.Generator(np.random.PCG64(seed))
    yy, xx = np.mgrid[0:height, 0:width].astype(np.float32)
    img = 0.45 + 0.1 * np.sin(xx / 97.0) * np.cos(yy / 61.0)
    n = int(density * width * height)
    cx = rng.uniform(0, width, n).astype(np.float32)
    cy = rng.uniform(0, height, n).astype(np.float32)
    rad = rng.uniform(1.5, 8.0, n).astype(np.float32)
    amp = rng.uniform(-0.35, 0.35, n).astype(np.float32)
    for k in range(n):
        r = int(np.ceil(3.5 * rad[k]))
        x0, x1 = max(0, int(cx[k]) - r), min(width, int(cx[k]) + r + 1)
        y0, y1 = max(0, int(cy[k]) - r), min(height, int(cy[k]) + r + 1)
        if x0 >= x1 or y0 >= y1:
            continue
        d2 = (xx[y0:y1, x0:x1] - cx[k]) ** 2 + (yy[y0:y1, x0:x1] - cy[k]) ** 2
        img[y0:y1, x0:x1] += amp[k] * np.exp(-d2 / (2.0 * rad[k] * rad[k]))
    return np.clip(img, 0.0, 1.0).astype(np.float32)


def scene_views(n: int, width: int = 960, height: int = 540, step: int = 24, seed: int = 11) -> np.ndarray:
    """n RGB8 views (n, height, width, 3) of one scene, each shifted `step`
    pixels along x from the last (a camera moving along a facade), so
    neighbouring views share most of their content; 8-bit quantised like
    decoded photos, a faint colour tint per channel."""
    canvas = scene_canvas(width + step * max(n - 1, 0), height, seed)
    out = np.empty((n, height, width, 3), np.uint8)
    tint = np.array([1.0, 0.97, 0.93], np.float32)
    for k in range(n):
        v = canvas[:, k * step:k * step + width, None] * tint
        out[k] = np.clip(np.rint(v * 255.0), 0, 255).astype(np.uint8)
    return out
