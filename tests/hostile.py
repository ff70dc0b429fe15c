"""Seeded descriptor sets built to stress the shortlist's error bound.

The BF16 / FP8 shortlist certifies a match decision only when the per-pair
bound eps on |d~ - d| proves it, and settles everything else with exact
spec-order FP32 distances (matching.rs:146-155). SIFT-like unit descriptors
(non-negative, clipped) leave most decisions far from the bound. These sets
go where the bound is thin:

  mixed_sign       components of both signs (dot products cancel)
  large_norm       row norms spread up to just under the routing limit of 64
  swamped          one dominant component per row plus 127 tiny ones, the
                   case where a tensor-core accumulator loses the small
                   products next to the large one
  boundary_pair    rows whose exact d1 sits within a fraction of eps of
                   r^2 d2 (the ratio test's edge, as in the reference's
                   ratio_match_rounding_boundary, matching.rs:2359-2406, but
                   at the scale of eps instead of one f32 ulp), and columns
                   whose two nearest rows lie within eps of each other,
                   some exactly tied

All draws come from numpy's PCG64 with the given seed; every array is f32.
"""
from __future__ import annotations

import numpy as np


def _unit(x: np.ndarray) -> np.ndarray:
    x = x.astype(np.float64)
    return x / np.linalg.norm(x, axis=1, keepdims=True)


def _ortho_unit(rng, base: np.ndarray) -> np.ndarray:
    """Unit vectors orthogonal to each (unit) row of base."""
    g = rng.standard_normal(base.shape)
    g -= np.sum(g * base, axis=1, keepdims=True) * base
    return _unit(g)


def _copies(rng, src: np.ndarray, sigma: float) -> np.ndarray:
    """Rows of src plus N(0, sigma * |row| / sqrt(128)) per component."""
    s = np.linalg.norm(src.astype(np.float64), axis=1, keepdims=True) / np.sqrt(128.0)
    return src + rng.standard_normal(src.shape) * sigma * s


def _pair_from(rng, a: np.ndarray, fresh_b: np.ndarray, n_true: int, sigma: float):
    """b = noisy copies of n_true random rows of a, then fresh_b, shuffled."""
    src = rng.permutation(len(a))[:n_true]
    b = np.concatenate([_copies(rng, a[src], sigma), fresh_b])
    b = b[rng.permutation(len(b))]
    return np.ascontiguousarray(a, np.float32), np.ascontiguousarray(b, np.float32)


def mixed_sign(seed: int, na: int, nb: int, sigma: float = 0.15):
    """Unit descriptors with N(0, 1) components (both signs), half of b noisy copies."""
    rng = np.random.Generator(np.random.PCG64(seed))
    a = _unit(rng.standard_normal((na, 128)))
    k = min(na, nb) // 2
    return _pair_from(rng, a, _unit(rng.standard_normal((nb - k, 128))), k, sigma)


def large_norm(seed: int, na: int, nb: int, lo: float = 0.05, hi: float = 63.0, sigma: float = 0.15):
    """Mixed-sign rows with norms log-uniform in [lo, hi] (all below the limit of 64)."""
    rng = np.random.Generator(np.random.PCG64(seed))

    def rows(n):
        s = np.exp(rng.uniform(np.log(lo), np.log(hi), size=(n, 1)))
        return _unit(rng.standard_normal((n, 128))) * s

    a = rows(na)
    k = min(na, nb) // 2
    a32, b32 = _pair_from(rng, a, rows(nb - k), k, sigma)
    # the copies' noise can push a norm up a little: keep every row below hi
    for x in (a32, b32):
        n = np.linalg.norm(x.astype(np.float64), axis=1)
        over = n > hi
        x[over] *= np.float32(hi / n[over])[:, None]
    return a32, b32


def swamped(seed: int, na: int, nb: int, tiny: float):
    """Per row one component of magnitude in [0.5, 1] (at a random position)
    and 127 of magnitude about `tiny` (mixed signs); b holds copies of half of
    a's rows with only the tiny components perturbed, so that rows sharing a
    dominant position differ only in the products the accumulator may swamp."""
    rng = np.random.Generator(np.random.PCG64(seed))

    def rows(n):
        x = rng.standard_normal((n, 128)) * tiny
        pos = rng.integers(0, 128, size=n)
        x[np.arange(n), pos] = rng.uniform(0.5, 1.0, size=n) * rng.choice([-1.0, 1.0], size=n)
        return x

    a = rows(na)
    k = min(na, nb) // 2
    src = rng.permutation(na)[:k]
    cp = a[src].copy()
    big = np.abs(cp) >= 0.5
    cp += np.where(big, 0.0, rng.standard_normal(cp.shape) * tiny * 0.3)
    b = np.concatenate([cp, rows(nb - k)])
    b = b[rng.permutation(len(b))]
    return np.ascontiguousarray(a, np.float32), np.ascontiguousarray(b, np.float32)


def boundary_pair(seed: int, n_ratio: int, n_tie: int, n_fresh: int, ratio: float = 0.8, width: float = 0.006,
                  tie_width: float = 0.002, exact_ties: int = 16):
    """One image pair (a, b) of three kinds of rows, shuffled:

    - n_ratio rows a_i (unit, non-negative) with two dedicated columns
      b = a_i + delta u (u a unit vector orthogonal to a_i): the second at
      squared distance D2 ~ U[0.15, 0.3], the first at r^2 D2 + w,
      w ~ U[-width, width], so d1 / (r^2 d2) is within a few eps of 1;
    - n_tie columns b_j (unit) with two rows at squared distances D and
      D + v, D ~ U[0.05, 0.15], v ~ U[-tie_width, tie_width]; for the first
      `exact_ties` of them the second row is the mirror b_j - delta u (the
      same distance in real arithmetic, often the same f32 value), so the
      cross-check's lowest-index rule decides;
    - n_fresh unrelated rows on each side.
    Returns (a, b) f32."""
    rng = np.random.Generator(np.random.PCG64(seed))
    r2 = ratio * ratio
    base = _unit(np.abs(rng.standard_normal((n_ratio, 128))))
    d2 = rng.uniform(0.15, 0.3, size=n_ratio)
    d1 = r2 * d2 + rng.uniform(-width, width, size=n_ratio)
    b1 = base + np.sqrt(d1)[:, None] * _ortho_unit(rng, base)
    b2 = base + np.sqrt(d2)[:, None] * _ortho_unit(rng, base)

    cols = _unit(np.abs(rng.standard_normal((n_tie, 128))))
    dd = rng.uniform(0.05, 0.15, size=n_tie)
    u = _ortho_unit(rng, cols)
    t1 = cols + np.sqrt(dd)[:, None] * u
    dd2 = dd + rng.uniform(-tie_width, tie_width, size=n_tie)
    t2 = cols + np.sqrt(dd2)[:, None] * _ortho_unit(rng, cols)
    m = min(exact_ties, n_tie)
    t2[:m] = cols[:m] - np.sqrt(dd[:m])[:, None] * u[:m]

    fa = _unit(np.abs(rng.standard_normal((n_fresh, 128))))
    fb = _unit(np.abs(rng.standard_normal((n_fresh, 128))))
    a = np.concatenate([base, t1, t2, fa])
    b = np.concatenate([b1, b2, cols, fb])
    a = a[rng.permutation(len(a))]
    b = b[rng.permutation(len(b))]
    return np.ascontiguousarray(a, np.float32), np.ascontiguousarray(b, np.float32)


def eps_bound(a: np.ndarray, b: np.ndarray, prec: str) -> float:
    """The per-pair bound the eps kernel derives from the two views' statistics
    (Cauchy-Schwarz on the operand rounding residuals, plus accumulation and
    rounding terms); q() is the operand rounding: bf16 round-to-nearest, or
    E4M3 with a per-descriptor power-of-two scale (max |a| scaled to <= 448)."""
    import torch

    def q(x):
        if prec == "bf16":
            return torch.from_numpy(x).to(torch.bfloat16).to(torch.float32).numpy()
        amax = np.abs(x).max(axis=1, keepdims=True)
        amax = np.where(amax > 0, amax, 1.0)
        e = np.frexp(448.0 / amax)[1]
        s = np.ldexp(1.0, e - 1).astype(np.float32)
        return torch.from_numpy(x * s).to(torch.float8_e4m3fn).to(torch.float32).numpy() / s

    qa, qb = q(a), q(b)
    nrm = lambda x: np.linalg.norm(x.astype(np.float64), axis=1).max()
    A, B = nrm(a), nrm(b)
    Ra, Rb = nrm(a - qa), nrm(b - qb)
    Qa, Qb = nrm(qa), nrm(qb)
    eps = 2 * (Ra * B + Qa * Rb) * (1 + 1e-3)
    eps += 5e-4 * Qa * Qb + 5e-5 * (A * A + B * B) + 2e-5 * (A + B) ** 2 + 1e-6
    if prec == "bf16":  # the norms are folded into the tensor-core product
        eps += 5e-4 * (A * A + B * B)
    return float(eps)


def near_boundary_rows(d: np.ndarray, ratio: float, width: float) -> int:
    """Rows of an exact f32 distance matrix whose (d1, d2) satisfy
    |d1 - r^2 d2| <= width, d2 finite (the rows no bound of that width can
    settle either way)."""
    part = np.partition(d, 1, axis=1)
    d1, d2 = part[:, 0].astype(np.float64), part[:, 1].astype(np.float64)
    r2 = float(np.float32(ratio) * np.float32(ratio))
    return int(np.sum(np.isfinite(d2) & (np.abs(d1 - r2 * d2) <= width)))


def tied_columns(d: np.ndarray, ratio: float, width: float) -> int:
    """Columns j whose two nearest rows are within `width` of each other and
    both choose j as a clear ratio-test match (d1 < r^2 d2 by more than
    4 width): their cross-check needs the exact column minimum."""
    part = np.partition(d, 1, axis=1)
    j1 = np.argmin(d, axis=1)
    r2 = float(np.float32(ratio) * np.float32(ratio))
    clear = part[:, 0] < r2 * part[:, 1] - 4 * width
    cpart = np.partition(d, 1, axis=0)
    close = (cpart[1] - cpart[0]) <= width
    i1 = np.argmin(d, axis=0)
    # the second nearest row of each column
    masked = d.copy()
    masked[i1, np.arange(d.shape[1])] = np.inf
    i2 = np.argmin(masked, axis=0)
    cols = np.arange(d.shape[1])
    ok = close & clear[i1] & clear[i2] & (j1[i1] == cols) & (j1[i2] == cols)
    return int(np.sum(ok))


def bf16_accumulation_error(a: np.ndarray, b: np.ndarray, dump: np.ndarray) -> float:
    """Largest error of the tensor core's FP32 accumulation in a BF16 pass,
    relative to the magnitude it accumulates.

    The BF16 accumulator holds d~ / 2 = (hi_a + lo_a) + (hi_b + lo_b) - q(a).q(b)
    (q: bf16 rounding; hi + lo: the bf16 split of the f32 half norm |v|^2 / 2,
    summed in component order as the pack kernel does). Given the rounded
    operands that sum is exact in f64, so |dump / 2 - exact| over
    sum_k |q(a)_k q(b)_k| + |hi_a| + |lo_a| + |hi_b| + |lo_b| is the
    accumulation's own relative error, which the bound allows up to 2^-11."""
    import torch

    def bf(x):
        return torch.from_numpy(np.ascontiguousarray(x, np.float32)).to(torch.bfloat16).to(torch.float32).numpy()

    def split(x):
        nrm = np.zeros(len(x), np.float32)
        for k in range(x.shape[1]):
            nrm = (nrm + x[:, k] * x[:, k]).astype(np.float32)
        half = (np.float32(0.5) * nrm).astype(np.float32)
        hi = bf(half)
        lo = bf((half - hi).astype(np.float32))
        return hi.astype(np.float64), lo.astype(np.float64)

    qa, qb = bf(a).astype(np.float64), bf(b).astype(np.float64)
    ha, la = split(a)
    hb, lb = split(b)
    exact = (ha + la)[:, None] + (hb + lb)[None, :] - qa @ qb.T
    mag = np.abs(qa) @ np.abs(qb).T + (np.abs(ha) + np.abs(la))[:, None] + (np.abs(hb) + np.abs(lb))[None, :]
    got = dump.astype(np.float64) / 2.0
    return float(np.max(np.abs(got - exact) / np.maximum(mag, 1e-300)))
