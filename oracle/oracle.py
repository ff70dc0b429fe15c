"""ctypes front end of the C oracle (oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and
by the ``cpu_baseline`` / ``--impl reference`` legs of bench.py, always as the
checker or the timed CPU baseline, never as the product path.

Each wrapper names the reference function it restates (paths inside
skylens-stream-rs).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "oracle.c")
SRCS = [SRC, os.path.join(HERE, "features.c"), os.path.join(HERE, "tracks.c")]

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile oracle.c with gcc (-O3, no FMA contraction) into _build/liboracle.so."""
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(f) for f in SRCS):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O3", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-o", tmp, *SRCS, "-lm", "-lpthread"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB)
            P = ctypes.POINTER
            u64p = P(ctypes.c_uint64)
            f32p = P(ctypes.c_float)
            u32p = P(ctypes.c_uint32)
            i64 = ctypes.c_int64
            L.orc_lcg_next.argtypes = [u64p]
            L.orc_lcg_next.restype = ctypes.c_double
            L.orc_lcg_gauss.argtypes = [u64p]
            L.orc_lcg_gauss.restype = ctypes.c_double
            L.orc_feature.argtypes = [u64p, f32p]
            L.orc_perturb.argtypes = [u64p, f32p, ctypes.c_float]
            L.orc_match_fixture_copies.argtypes = [i64]
            L.orc_match_fixture_copies.restype = i64
            L.orc_match_fixture.argtypes = [ctypes.c_uint64, i64, i64, f32p, f32p]
            L.orc_sq_dist.argtypes = [f32p, f32p]
            L.orc_sq_dist.restype = ctypes.c_float
            L.orc_sq_dist_seq.argtypes = [f32p, f32p]
            L.orc_sq_dist_seq.restype = ctypes.c_float
            L.orc_sq_dist_f64.argtypes = [f32p, f32p]
            L.orc_sq_dist_f64.restype = ctypes.c_double
            L.orc_dist_matrix.argtypes = [f32p, i64, f32p, i64, f32p]
            L.orc_dist_matrix_f64.argtypes = [f32p, i64, f32p, i64, P(ctypes.c_double)]
            L.orc_ratio_match.argtypes = [f32p, i64, f32p, i64, ctypes.c_float, ctypes.c_int, ctypes.c_int, u32p]
            L.orc_ratio_match.restype = i64
            L.orc_ratio_match_naive.argtypes = [f32p, i64, f32p, i64, ctypes.c_float, ctypes.c_int, u32p]
            L.orc_ratio_match_naive.restype = i64
            L.orc_ratio_states.argtypes = [f32p, i64, f32p, i64, u32p, f32p, f32p, u32p, f32p]
            L.orc_pairs_hash.argtypes = [u32p, i64]
            L.orc_pairs_hash.restype = ctypes.c_uint64
            L.orc_candidate_pairs.argtypes = [u64p, i64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, u32p, i64]
            L.orc_candidate_pairs.restype = i64
            L.orc_scheduled_pairs.argtypes = [u64p, i64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
                                              ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                              ctypes.c_uint64, u32p, i64]
            L.orc_scheduled_pairs.restype = i64
            f64p = P(ctypes.c_double)
            L.orc_sampson_residual.argtypes = [f64p] + [ctypes.c_double] * 4
            L.orc_sampson_residual.restype = ctypes.c_double
            L.orc_sampson_score.argtypes = [f64p, u64p, f64p, f64p, u32p, i64, u32p, u64p, u32p, ctypes.c_int]
            L.orc_match_pairs.argtypes = [f32p, P(ctypes.c_int64), P(ctypes.c_int64), u32p, i64, ctypes.c_float,
                                          ctypes.c_int, ctypes.c_int, P(ctypes.c_int64)]
            L.orc_match_pairs.restype = i64
            i32 = ctypes.c_int
            f32 = ctypes.c_float
            L.orc_blur_taps.argtypes = [f32, f32p]
            L.orc_blur_taps.restype = i64
            L.orc_gaussian_blur.argtypes = [f32p, i64, i64, f32, f32p]
            L.orc_upsample2.argtypes = [f32p, i64, i64, f32p]
            L.orc_gray_from_rgb8.argtypes = [P(ctypes.c_uint8), i64, f32p]
            L.orc_orientations.argtypes = [f32p, f32p, i64, i64, f32, f32, f32, i32, f32p]
            L.orc_orientations.restype = i64
            L.orc_describe.argtypes = [f32p, i64, i64, f32, f32, f32, f32, i32, f32p]
            L.orc_dominant_orientations.argtypes = [f32p, i64, i64, f32, f32, f32, i32, f32p]
            L.orc_dominant_orientations.restype = i64
            L.orc_detect_and_describe.argtypes = [f32p, i64, i64, ctypes.c_void_p, i32, f32p, f32p, i64]
            L.orc_detect_and_describe.restype = i64
            L.orc_build_tracks_drop.argtypes = [u32p, i64, ctypes.c_void_p, i64, u32p, i64, i64, u64p, i64, u64p, i64,
                                                ctypes.c_void_p]
            L.orc_build_tracks_drop.restype = i64
            _lib = L
    return _lib


def _f32(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    return x


def _p(x: np.ndarray, t):
    return x.ctypes.data_as(ctypes.POINTER(t))


class Lcg:
    """matching.rs:1140-1153 (test Lcg): 64-bit LCG with Box-Muller gauss."""

    def __init__(self, seed: int):
        self.s = ctypes.c_uint64(seed)

    def next(self) -> float:
        return lib().orc_lcg_next(ctypes.byref(self.s))

    def gauss(self) -> float:
        return lib().orc_lcg_gauss(ctypes.byref(self.s))

    def feature(self) -> np.ndarray:
        """matching.rs:1580-1596 (`feature`): unit-length uniform descriptor."""
        out = np.empty(128, np.float32)
        lib().orc_feature(ctypes.byref(self.s), _p(out, ctypes.c_float))
        return out

    def features(self, n: int) -> np.ndarray:
        return np.stack([self.feature() for _ in range(n)]) if n else np.zeros((0, 128), np.float32)

    def perturb(self, h: np.ndarray, scale: float) -> np.ndarray:
        """h[k] += scale * (f32)gauss() for k in 0..128 (matching.rs:1649-1651)."""
        h = np.array(h, dtype=np.float32, copy=True)
        lib().orc_perturb(ctypes.byref(self.s), _p(h, ctypes.c_float), ctypes.c_float(scale))
        return h


def match_fixture(seed: int, na: int, extra: int):
    """matching.rs:1638-1656 (`match_fixture`)."""
    L = lib()
    nb = L.orc_match_fixture_copies(na) + extra
    a = np.empty((na, 128), np.float32)
    b = np.empty((nb, 128), np.float32)
    L.orc_match_fixture(seed, na, extra, _p(a, ctypes.c_float), _p(b, ctypes.c_float))
    return a, b


def sq_dist(p, r) -> float:
    """matching.rs:144-155 spec order (8 lanes, then lanes 0..7)."""
    p, r = _f32(p), _f32(r)
    return float(np.float32(lib().orc_sq_dist(_p(p, ctypes.c_float), _p(r, ctypes.c_float))))


def sq_dist_seq(p, r) -> float:
    """matching.rs:2373-2377: sequential fold."""
    p, r = _f32(p), _f32(r)
    return float(np.float32(lib().orc_sq_dist_seq(_p(p, ctypes.c_float), _p(r, ctypes.c_float))))


def dist_matrix(a, b) -> np.ndarray:
    a, b = _f32(a).reshape(-1, 128), _f32(b).reshape(-1, 128)
    out = np.empty((len(a), len(b)), np.float32)
    lib().orc_dist_matrix(_p(a, ctypes.c_float), len(a), _p(b, ctypes.c_float), len(b), _p(out, ctypes.c_float))
    return out


def dist_matrix_f64(a, b) -> np.ndarray:
    a, b = _f32(a).reshape(-1, 128), _f32(b).reshape(-1, 128)
    out = np.empty((len(a), len(b)), np.float64)
    lib().orc_dist_matrix_f64(_p(a, ctypes.c_float), len(a), _p(b, ctypes.c_float), len(b),
                              _p(out, ctypes.c_double))
    return out


def ratio_match(a, b, ratio: float, mutual: bool, threads: int = 1) -> list[tuple[int, int]]:
    """matching.rs:167-215 (`ratio_match`): blocked spec-order version."""
    return [tuple(p) for p in ratio_match_np(a, b, ratio, mutual, threads).tolist()]


def ratio_match_np(a, b, ratio: float, mutual: bool, threads: int = 1) -> np.ndarray:
    a, b = _f32(a).reshape(-1, 128), _f32(b).reshape(-1, 128)
    out = np.empty((max(len(a), 1), 2), np.uint32)
    n = lib().orc_ratio_match(_p(a, ctypes.c_float), len(a), _p(b, ctypes.c_float), len(b),
                              ctypes.c_float(ratio), int(bool(mutual)), int(threads), _p(out, ctypes.c_uint32))
    return out[:n].copy()


def ratio_match_naive(a, b, ratio: float, mutual: bool) -> list[tuple[int, int]]:
    """matching.rs:1597-1636 (`ratio_match_reference`): sequential sums."""
    a, b = _f32(a).reshape(-1, 128), _f32(b).reshape(-1, 128)
    out = np.empty((max(len(a), 1), 2), np.uint32)
    n = lib().orc_ratio_match_naive(_p(a, ctypes.c_float), len(a), _p(b, ctypes.c_float), len(b),
                                    ctypes.c_float(ratio), int(bool(mutual)), _p(out, ctypes.c_uint32))
    return [tuple(p) for p in out[:n].tolist()]


def ratio_states(a, b):
    """Exact per-row (j1, d1, d2) and per-column (i1, d1) states."""
    a, b = _f32(a).reshape(-1, 128), _f32(b).reshape(-1, 128)
    na, nb = len(a), len(b)
    rj = np.empty(na, np.uint32)
    rd1 = np.empty(na, np.float32)
    rd2 = np.empty(na, np.float32)
    ci = np.empty(nb, np.uint32)
    cd = np.empty(nb, np.float32)
    lib().orc_ratio_states(_p(a, ctypes.c_float), na, _p(b, ctypes.c_float), nb, _p(rj, ctypes.c_uint32),
                           _p(rd1, ctypes.c_float), _p(rd2, ctypes.c_float), _p(ci, ctypes.c_uint32),
                           _p(cd, ctypes.c_float))
    return rj, rd1, rd2, ci, cd


def pairs_hash(m) -> int:
    """matching.rs:1866-1878 (`pairs_hash`): FNV-1a 64."""
    arr = np.ascontiguousarray(np.asarray(m, dtype=np.uint32).reshape(-1, 2))
    return int(lib().orc_pairs_hash(_p(arr, ctypes.c_uint32), len(arr)))


def _views(views) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(views, dtype=np.uint64).reshape(-1, 2))


def candidate_pairs(views, temporal: int, cross: int, pow2_max: int) -> list[tuple[int, int]]:
    """matching.rs:14-40."""
    v = _views(views)
    n = lib().orc_candidate_pairs(_p(v, ctypes.c_uint64), len(v), temporal, cross, min(pow2_max, 2**64 - 1),
                                  None, 0)
    out = np.empty((max(n, 1), 2), np.uint32)
    lib().orc_candidate_pairs(_p(v, ctypes.c_uint64), len(v), temporal, cross, min(pow2_max, 2**64 - 1),
                              _p(out, ctypes.c_uint32), n)
    return [tuple(p) for p in out[:n].tolist()]


def scheduled_pairs(views, temporal=5, pow2_max=16, spec_range=None, formation=(20, 20, 40, 4)):
    """matching.rs:103-142. spec_range given -> CrossSchedule::Spec, else Formation."""
    v = _views(views)
    spec = spec_range is not None
    rm, lm, mx, st = formation
    args = (_p(v, ctypes.c_uint64), len(v), temporal, pow2_max, int(spec), spec_range or 0, rm, lm, mx, st)
    n = lib().orc_scheduled_pairs(*args, None, 0)
    out = np.empty((max(n, 1), 2), np.uint32)
    lib().orc_scheduled_pairs(*args, _p(out, ctypes.c_uint32), n)
    return [tuple(p) for p in out[:n].tolist()]


def match_pairs(desc, view_off, view_n, pairs, ratio: float, mutual: bool, threads: int):
    """Serial loop over pairs, each ratio_match'ed with `threads` (benches/pipeline.rs:247-253).
    Returns (total matches, per-pair counts)."""
    desc = _f32(desc)
    vo = np.ascontiguousarray(view_off, dtype=np.int64)
    vn = np.ascontiguousarray(view_n, dtype=np.int64)
    pr = np.ascontiguousarray(np.asarray(pairs, dtype=np.uint32).reshape(-1, 2))
    counts = np.empty(len(pr), np.int64)
    tot = lib().orc_match_pairs(_p(desc, ctypes.c_float), _p(vo, ctypes.c_int64), _p(vn, ctypes.c_int64),
                                _p(pr, ctypes.c_uint32), len(pr), ctypes.c_float(ratio), int(bool(mutual)),
                                int(threads), _p(counts, ctypes.c_int64))
    return tot, counts


def sampson_residual(e, a, b) -> float:
    """two_view.rs:456-465: signed Sampson residual of one correspondence
    (a, b: normalized coordinates) under the row-major 3x3 matrix e."""
    e = np.ascontiguousarray(e, dtype=np.float64).reshape(9)
    return lib().orc_sampson_residual(_p(e, ctypes.c_double), float(a[0]), float(a[1]), float(b[0]), float(b[1]))


def sampson_score(pts, pair_off, thresh, E, hyp_pair, mask_off=None, threads: int = 1):
    """two_view.rs:804-823 (inliers_of, count_at_least), batched: counts (and
    inlier bit masks where mask_off[h] != 2**64 - 1) of every hypothesis over
    its pair's matches. pts: (M, 4) f64 (a.x, a.y, b.x, b.y); pair_off: (P+1,)
    uint64; thresh: (P,) f64; E: (H, 3, 3) f64; hyp_pair: (H,) uint32."""
    pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 4)
    po = np.ascontiguousarray(pair_off, dtype=np.uint64)
    th = np.ascontiguousarray(thresh, dtype=np.float64)
    E = np.ascontiguousarray(E, dtype=np.float64).reshape(-1, 9)
    hp = np.ascontiguousarray(hyp_pair, dtype=np.uint32)
    counts = np.empty(len(E), np.uint32)
    masks = None
    mo = None
    if mask_off is not None:
        mo = np.ascontiguousarray(mask_off, dtype=np.uint64)
        nwords = 0
        for h in range(len(E)):
            if mo[h] != np.uint64(2**64 - 1):
                n = int(po[hp[h] + 1] - po[hp[h]])
                nwords = max(nwords, int(mo[h]) + (n + 31) // 32)
        masks = np.zeros(max(nwords, 1), np.uint32)
    lib().orc_sampson_score(_p(pts, ctypes.c_double), _p(po, ctypes.c_uint64), _p(th, ctypes.c_double),
                            _p(E, ctypes.c_double), _p(hp, ctypes.c_uint32), len(E), _p(counts, ctypes.c_uint32),
                            None if mo is None else _p(mo, ctypes.c_uint64),
                            None if masks is None else _p(masks, ctypes.c_uint32), int(threads))
    return counts, masks


# ---- descriptor producer (features.c; crates/core/src/features.rs) -------

class DetectorConfig(ctypes.Structure):
    """DetectorConfig (features.rs:253-293), defaults of `Default` (:278-293)."""
    _fields_ = [("octaves", ctypes.c_int64), ("scales", ctypes.c_int64), ("sigma0", ctypes.c_float),
                ("contrast", ctypes.c_float), ("edge_ratio", ctypes.c_float), ("max_features", ctypes.c_int64),
                ("upscale_below", ctypes.c_int64), ("upscale_fill", ctypes.c_int)]

    def __init__(self, octaves=4, scales=3, sigma0=1.6, contrast=0.01, edge_ratio=10.0, max_features=8192,
                 upscale_below=800, upscale_fill=False):
        super().__init__(octaves, scales, sigma0, contrast, edge_ratio, max_features, upscale_below,
                         int(bool(upscale_fill)))


def _img(img) -> np.ndarray:
    img = np.ascontiguousarray(img, dtype=np.float32)
    assert img.ndim == 2
    return img


def gray_from_rgb8(rgb) -> np.ndarray:
    """GrayImage::from_rgb (features.rs:165-189): (0.299 r + 0.587 g + 0.114 b) / 255 in f32."""
    rgb = np.ascontiguousarray(rgb, dtype=np.uint8)
    h, w, _ = rgb.shape
    out = np.empty((h, w), np.float32)
    lib().orc_gray_from_rgb8(_p(rgb, ctypes.c_uint8), h * w, _p(out, ctypes.c_float))
    return out


def blur_taps(sigma: float) -> np.ndarray:
    """gaussian_blur's normalised taps (features.rs:215-220)."""
    k = np.empty(4096, np.float32)
    r = lib().orc_blur_taps(ctypes.c_float(sigma), _p(k, ctypes.c_float))
    return k[:2 * r + 1].copy()


def gaussian_blur(img, sigma: float) -> np.ndarray:
    """gaussian_blur (features.rs:214-250)."""
    img = _img(img)
    out = np.empty_like(img)
    lib().orc_gaussian_blur(_p(img, ctypes.c_float), img.shape[1], img.shape[0], ctypes.c_float(sigma),
                            _p(out, ctypes.c_float))
    return out


def upsample2(img) -> np.ndarray:
    """GrayImage::upsample2 (features.rs:62-85)."""
    img = _img(img)
    out = np.empty((img.shape[0] * 2, img.shape[1] * 2), np.float32)
    lib().orc_upsample2(_p(img, ctypes.c_float), img.shape[1], img.shape[0], _p(out, ctypes.c_float))
    return out


def dominant_orientations(img, x: float, y: float, sigma: float, cr: bool = False) -> np.ndarray:
    """dominant_orientations (features.rs:314-323); cr: transcendental
    functions correctly rounded through double (as the GPU), else the
    platform's float functions (as the reference)."""
    img = _img(img)
    out = np.empty(36, np.float32)
    n = lib().orc_dominant_orientations(_p(img, ctypes.c_float), img.shape[1], img.shape[0], ctypes.c_float(x),
                                        ctypes.c_float(y), ctypes.c_float(sigma), int(cr), _p(out, ctypes.c_float))
    return out[:n].copy()


def describe(img, x: float, y: float, sigma: float, angle: float, cr: bool = False) -> np.ndarray:
    """describe (features.rs:509-592)."""
    img = _img(img)
    out = np.empty(128, np.float32)
    lib().orc_describe(_p(img, ctypes.c_float), img.shape[1], img.shape[0], ctypes.c_float(x), ctypes.c_float(y),
                       ctypes.c_float(sigma), ctypes.c_float(angle), int(cr), _p(out, ctypes.c_float))
    return out


def detect_and_describe(img, cfg: DetectorConfig | None = None, cr: bool = False):
    """detect_and_describe (features.rs:594-648) -> (keypoints (n, 5): x, y,
    sigma, response, angle; descriptors (n, 128))."""
    img = _img(img)
    cfg = cfg or DetectorConfig()
    L = lib()
    h, w = img.shape
    cap = max(int(cfg.max_features), 1)  # the original features plus the added ones never exceed it
    kps = np.empty((cap, 5), np.float32)
    desc = np.empty((cap, 128), np.float32)
    n = L.orc_detect_and_describe(_p(img, ctypes.c_float), w, h, ctypes.byref(cfg), int(cr),
                                  _p(kps, ctypes.c_float), _p(desc, ctypes.c_float), cap)
    assert n <= cap
    return kps[:n].copy(), desc[:n].copy()


# ---- tracks, ConflictPolicy::Drop (tracks.c; crates/core/src/tracks.rs) ---

class PairMatches(ctypes.Structure):
    """PairMatches (tracks.rs:44-50): matches[first .. first + count) of a flat array."""
    _fields_ = [("image_a", ctypes.c_uint32), ("image_b", ctypes.c_uint32), ("first", ctypes.c_uint64),
                ("count", ctypes.c_uint64)]


class TrackStats(ctypes.Structure):
    _fields_ = [("edges", ctypes.c_uint64), ("invalid_matches", ctypes.c_uint64), ("conflicts", ctypes.c_uint64),
                ("too_short", ctypes.c_uint64), ("truncated", ctypes.c_uint64), ("tracks", ctypes.c_uint64)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


def pack_pairs(pairs):
    """[(image_a, image_b, [(fa, fb), ...]), ...] -> (PairMatches array, flat uint32 (M, 2))."""
    arr = (PairMatches * max(len(pairs), 1))()
    flat, first = [], 0
    for k, (a, b, m) in enumerate(pairs):
        m = np.asarray(m, dtype=np.uint32).reshape(-1, 2)
        arr[k] = PairMatches(a, b, first, len(m))
        flat.append(m)
        first += len(m)
    flat = np.ascontiguousarray(np.concatenate(flat) if flat else np.zeros((0, 2), np.uint32))
    return arr, flat


def build_tracks_drop(n_features, pairs, min_length: int = 3, max_tracks: int = 100_000):
    """build_tracks with ConflictPolicy::Drop (tracks.rs:190-259) -> (tracks as
    lists of (image, feature), stats dict)."""
    nf = np.ascontiguousarray(n_features, dtype=np.uint32)
    arr, flat = pack_pairs(pairs)
    off = np.concatenate([[0], np.cumsum(nf, dtype=np.uint64)])
    cap_n = max(2 * len(flat), 1)
    toff = np.zeros(cap_n + 1, np.uint64)
    nodes = np.zeros(cap_n, np.uint64)
    st = TrackStats()
    nt = lib().orc_build_tracks_drop(_p(nf, ctypes.c_uint32), len(nf), ctypes.cast(arr, ctypes.c_void_p), len(pairs),
                                     _p(flat, ctypes.c_uint32), min_length, max_tracks, _p(toff, ctypes.c_uint64),
                                     cap_n, _p(nodes, ctypes.c_uint64), cap_n, ctypes.byref(st))
    img = np.searchsorted(off, np.arange(int(off[-1])), side="right") - 1 if len(off) > 1 else np.zeros(0, int)
    tracks = []
    for t in range(nt):
        ns = nodes[int(toff[t]):int(toff[t + 1])]
        tracks.append([(int(img[x]), int(x - off[img[x]])) for x in ns])
    return tracks, st.as_dict()
