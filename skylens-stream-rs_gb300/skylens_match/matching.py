"""Python mirror of skylens_core::matching's hot path over libslm.

Names, argument meaning and results follow the reference:
  ratio_match(a, b, ratio, mutual)        crates/core/src/matching.rs:167
  candidate_pairs(views, t, c, p2)        crates/core/src/matching.rs:18
  scheduled_pairs(views, schedule)        crates/core/src/matching.rs:103
  PairSchedule.default() / .spec()        crates/core/src/matching.rs:82-100
  match_pairs(store, pairs, ...)          crates/core/src/pipeline.rs:485-493 (matching half)
Descriptors are float32 arrays of shape (n, 128). Matches come back as lists
of (i, j) in ascending i, exactly as ratio_match returns them. The one
deviation from the reference's infallible signature: a GPU error raises
SlmError (there is no CPU fallback).
"""
from __future__ import annotations

import atexit
import ctypes
import threading
import weakref
from dataclasses import dataclass

import numpy as np

from ._lib import (PRECISIONS, SLM_CAPACITY, SlmError, SlmOpts, SlmPair, SlmPairSchedule, SlmStats, SlmTune, check,
                   load)

PAIR_TEMPORAL = 5    # matching.rs:8
PAIR_CROSS = 4       # matching.rs:10
PAIR_POW2_MAX = 16   # matching.rs:12
CAM_FRONT, CAM_RIGHT, CAM_LEFT = 0, 1, 2  # matching.rs:42-45
USIZE_MAX = 2**64 - 1

_f32p = ctypes.POINTER(ctypes.c_float)


def _desc(x) -> np.ndarray:
    a = np.ascontiguousarray(x, dtype=np.float32)
    if a.ndim == 1 and a.size == 0:
        a = a.reshape(0, 128)
    if a.ndim != 2 or a.shape[1] != 128:
        raise ValueError(f"descriptors must have shape (n, 128), got {a.shape}")
    return a


def _prec(p) -> int:
    if isinstance(p, int):
        return p
    return PRECISIONS[p]


def _pairs_array(pairs) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(pairs, dtype=np.uint32).reshape(-1, 2))


_live_matchers: "weakref.WeakSet[Matcher]" = weakref.WeakSet()


@atexit.register
def _close_live_matchers() -> None:
    """Free contexts (and their stores and plans) while the CUDA runtime is
    still up: objects left to interpreter shutdown would be freed after it."""
    for m in list(_live_matchers):
        try:
            m.close()
        except Exception:
            pass


class Matcher:
    """A libslm context on one CUDA device (thread-safe)."""

    def __init__(self, device: int = 0, stream: int | None = None, hbm_budget: int = 0):
        self._L = load()
        opts = SlmOpts(device, ctypes.c_void_p(stream or 0), hbm_budget)
        h = ctypes.c_void_p()
        check(self._L.slm_ctx_create(ctypes.byref(opts), ctypes.byref(h)), "slm_ctx_create")
        self._h = h
        self.last_stats: dict | None = None
        self._stores = weakref.WeakSet()  # closed before the context
        _live_matchers.add(self)

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        return int(self._L.slm_ctx_stream(self._h) or 0)

    def bytes_in_use(self) -> int:
        return int(self._L.slm_ctx_bytes_in_use(self._h))

    def set_coalescing(self, window_us: int = 50, max_pairs: int = 256) -> None:
        """slm_ctx_set_coalescing: batch concurrent AUTO ratio_match calls
        (max_pairs = 0 turns it off)."""
        check(self._L.slm_ctx_set_coalescing(self._h, window_us, max_pairs), "slm_ctx_set_coalescing")

    def coalescing_stats(self) -> dict:
        b, c, m = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        check(self._L.slm_ctx_coalescing_stats(self._h, ctypes.byref(b), ctypes.byref(c), ctypes.byref(m)),
              "slm_ctx_coalescing_stats")
        return {"batches": b.value, "calls": c.value, "max_batch": m.value}

    def selftest_wait_timeout(self, polls: int = 256) -> int:
        """Runs the bounded-wait self-test (slm_selftest_wait_timeout) and
        returns its status: SLM_TIMEOUT when the device wait gave up as it must."""
        return int(self._L.slm_selftest_wait_timeout(self._h, polls))

    def close(self) -> None:
        if self._h:
            for st in list(self._stores):
                st.close()
            self._L.slm_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------- one pair
    def ratio_match_np(self, a, b, ratio: float = 0.8, mutual: bool = True, precision="fp32") -> np.ndarray:
        """matching.rs:167 ratio_match; returns an (n, 2) uint32 array."""
        a, b = _desc(a), _desc(b)
        na, nb = len(a), len(b)
        out = (SlmPair * max(na, 1))()
        n = ctypes.c_uint32(0)
        st = SlmStats()
        check(self._L.slm_ratio_match(self._h, a.ctypes.data_as(_f32p), na, b.ctypes.data_as(_f32p), nb,
                                      ctypes.c_float(ratio), int(bool(mutual)), _prec(precision), out, max(na, 1),
                                      ctypes.byref(n), ctypes.byref(st)), "slm_ratio_match")
        self.last_stats = st.as_dict()
        arr = np.frombuffer(out, dtype=np.uint32, count=2 * n.value).reshape(-1, 2).copy()
        return arr

    def ratio_match(self, a, b, ratio: float = 0.8, mutual: bool = True, precision="fp32"):
        return [tuple(p) for p in self.ratio_match_np(a, b, ratio, mutual, precision).tolist()]

    def ratio_match_device(self, d_a: int, na: int, d_b: int, nb: int, ratio: float, mutual: bool, precision,
                           d_out: int, cap: int, d_count: int) -> None:
        """Device-pointer variant (asynchronous on the context stream)."""
        check(self._L.slm_ratio_match_device(self._h, ctypes.c_void_p(d_a), na, ctypes.c_void_p(d_b), nb,
                                             ctypes.c_float(ratio), int(bool(mutual)), _prec(precision),
                                             ctypes.c_void_p(d_out), cap, ctypes.c_void_p(d_count)),
              "slm_ratio_match_device")

    # ------------------------------------------------------ RANSAC scoring
    def sampson_score(self, pts, pair_off, thresh, E, hyp_pair, masks_for=None):
        """slm_sampson_score: inlier counts of every essential-matrix hypothesis
        over its pair's matches (two_view.rs:804-823, count_at_least /
        inliers_of). pts (M, 4) f64 (a.x, a.y, b.x, b.y); pair_off (P + 1,)
        uint64 from 0; thresh (P,) f64 (threshold_px / focal_px); E (H, 3, 3)
        f64; hyp_pair (H,) uint32. masks_for: hypotheses whose inlier masks to
        return. Returns (counts (H,) uint32, {h: bool mask of its pair's matches})."""
        pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 4)
        po = np.ascontiguousarray(pair_off, dtype=np.uint64)
        th = np.ascontiguousarray(thresh, dtype=np.float64)
        Ev = np.ascontiguousarray(E, dtype=np.float64).reshape(-1, 9)
        hp = np.ascontiguousarray(hyp_pair, dtype=np.uint32)
        nh = len(Ev)
        counts = np.empty(max(nh, 1), np.uint32)
        mo = masks = None
        words = 0
        if masks_for is not None and len(masks_for):
            mo = np.full(max(nh, 1), np.uint64(2**64 - 1), np.uint64)
            for h in masks_for:
                mo[h] = words
                words += (int(po[hp[h] + 1] - po[hp[h]]) + 31) // 32
            masks = np.zeros(max(words, 1), np.uint32)
        P = ctypes.POINTER
        check(self._L.slm_sampson_score(self._h, pts.ctypes.data_as(P(ctypes.c_double)),
                                        po.ctypes.data_as(P(ctypes.c_uint64)), len(po) - 1,
                                        th.ctypes.data_as(P(ctypes.c_double)), Ev.ctypes.data_as(P(ctypes.c_double)),
                                        hp.ctypes.data_as(P(ctypes.c_uint32)), nh,
                                        counts.ctypes.data_as(P(ctypes.c_uint32)),
                                        None if mo is None else mo.ctypes.data_as(P(ctypes.c_uint64)),
                                        None if masks is None else masks.ctypes.data_as(P(ctypes.c_uint32)),
                                        words), "slm_sampson_score")
        out = {}
        if mo is not None:
            for h in masks_for:
                n = int(po[hp[h] + 1] - po[hp[h]])
                bits = np.unpackbits(masks[int(mo[h]):int(mo[h]) + (n + 31) // 32].view(np.uint8), bitorder="little")
                out[h] = bits[:n].astype(bool)
        return counts[:nh], out

    # ------------------------------------------------------------ batches
    def store(self, max_descs: int, max_views: int) -> "DescriptorStore":
        return DescriptorStore(self, max_descs, max_views)


class DescriptorStore:
    """Device-resident descriptors of many views (images)."""

    def __init__(self, m: Matcher, max_descs: int, max_views: int):
        self.m = m
        self._L = m._L
        h = ctypes.c_void_p()
        check(self._L.slm_store_create(m.handle, max_descs, max_views, ctypes.byref(h)), "slm_store_create")
        self._h = h
        self.counts: list[int] = []
        self._plans = weakref.WeakSet()  # closed before the store
        m._stores.add(self)

    @property
    def handle(self):
        return self._h

    def add_view(self, desc) -> int:
        d = _desc(desc)
        vid = ctypes.c_uint32()
        check(self._L.slm_store_add_view(self._h, d.ctypes.data_as(ctypes.c_void_p), len(d), ctypes.byref(vid)),
              "slm_store_add_view")
        self.counts.append(len(d))
        self._keep = d  # the copy is asynchronous: keep the host buffer alive
        return vid.value

    def add_views_packed(self, desc: np.ndarray, offsets, counts) -> list[int]:
        """All views from one (N, 128) host buffer (pinned memory copies fastest)."""
        d = desc if isinstance(desc, np.ndarray) else np.asarray(desc)
        off = np.ascontiguousarray(offsets, dtype=np.uint64)
        cnt = np.ascontiguousarray(counts, dtype=np.uint32)
        ids = np.empty(len(cnt), np.uint32)
        check(self._L.slm_store_add_views(self._h, ctypes.c_void_p(d.ctypes.data), off.ctypes.data_as(
            ctypes.POINTER(ctypes.c_uint64)), cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), len(cnt),
            ids.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))), "slm_store_add_views")
        self.counts.extend(int(c) for c in cnt)
        self._keep = d
        return ids.tolist()

    def add_views_ptr(self, host_ptr: int, offsets, counts) -> list[int]:
        """Like add_views_packed for a raw pointer to pinned host or device memory
        (e.g. a torch tensor): one asynchronous copy per view, so the buffer must
        stay alive and unchanged until the next synchronising call (a plan's
        results, or the context stream's synchronisation)."""
        off = np.ascontiguousarray(offsets, dtype=np.uint64)
        cnt = np.ascontiguousarray(counts, dtype=np.uint32)
        ids = np.empty(len(cnt), np.uint32)
        check(self._L.slm_store_add_views(self._h, ctypes.c_void_p(host_ptr), off.ctypes.data_as(
            ctypes.POINTER(ctypes.c_uint64)), cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), len(cnt),
            ids.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))), "slm_store_add_views")
        self.counts.extend(int(c) for c in cnt)
        return ids.tolist()

    def clear(self) -> None:
        check(self._L.slm_store_clear(self._h), "slm_store_clear")
        self.counts = []

    def __len__(self) -> int:
        return int(self._L.slm_store_num_views(self._h))

    def close(self) -> None:
        if self._h:
            for p in list(self._plans):
                p.close()
            self._L.slm_store_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def plan(self, pairs, ratio: float = 0.8, mutual: bool = True, precision="fp32", *, items_per_sm: int = 0,
             shortlist_k: int = 0, use_graph: int = 1, variant: int = 0, row_tiles: int = 0,
             autotune: bool = False) -> "BatchPlan":
        return BatchPlan(self, pairs, ratio, mutual, precision, items_per_sm, shortlist_k, use_graph, variant,
                         row_tiles, autotune)

    def autotune(self, pairs, ratio: float = 0.8, mutual: bool = True, precision="bf16"):
        """Time a grid of settings on this batch; returns (best setting dict, best ms)."""
        pr = _pairs_array(pairs)
        t = SlmTune()
        ms = ctypes.c_float()
        check(self._L.slm_autotune(self.m.handle, self._h, pr.ctypes.data_as(ctypes.POINTER(SlmPair)), len(pr),
                                   ctypes.c_float(ratio), int(bool(mutual)), _prec(precision), ctypes.byref(t),
                                   ctypes.byref(ms)), "slm_autotune")
        return t.as_dict(), ms.value


class BatchPlan:
    """A planned batch of image pairs (pipeline.rs:485-493), replayed as one CUDA graph."""

    def __init__(self, store: DescriptorStore, pairs, ratio, mutual, precision, items_per_sm=0, shortlist_k=0,
                 use_graph=1, variant=0, row_tiles=0, autotune=False):
        self.store = store
        self._L = store._L
        pr = _pairs_array(pairs)
        self.np = len(pr)
        self.total_rows = int(sum(store.counts[int(u)] for u, _ in pr)) if len(pr) else 0
        self.distances = int(sum(store.counts[int(u)] * store.counts[int(v)] for u, v in pr)) if len(pr) else 0
        tune = SlmTune(items_per_sm, shortlist_k, use_graph, variant, row_tiles, int(bool(autotune)))
        h = ctypes.c_void_p()
        check(self._L.slm_plan_create(store.m.handle, store.handle, pr.ctypes.data_as(ctypes.POINTER(SlmPair)),
                                      self.np, ctypes.c_float(ratio), int(bool(mutual)), _prec(precision),
                                      ctypes.byref(tune), ctypes.byref(h)), "slm_plan_create")
        self._h = h
        self._out = None
        self.stats: dict | None = None
        store._plans.add(self)

    def launch(self) -> None:
        check(self._L.slm_plan_launch(self._h), "slm_plan_launch")

    def results(self):
        """(pairs (M, 2) uint32, offsets (np+1,) uint64) of the last launch."""
        if self._out is None or len(self._out) < max(self.total_rows, 1):
            self._out = (SlmPair * max(self.total_rows, 1))()
        offsets = np.empty(self.np + 1, np.uint64)
        st = SlmStats()
        check(self._L.slm_plan_results(self._h, self._out, max(self.total_rows, 1),
                                       offsets.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), ctypes.byref(st)),
              "slm_plan_results")
        self.stats = st.as_dict()
        total = int(offsets[-1])
        pairs = np.frombuffer(self._out, dtype=np.uint32, count=2 * total).reshape(-1, 2).copy()
        return pairs, offsets

    def results_into(self, out: np.ndarray, offsets: np.ndarray) -> int:
        """slm_plan_results straight into caller buffers (no copy): out is a
        C-contiguous (cap, 2) uint32 array (pinned memory reads back fastest),
        offsets a (np + 1,) uint64 array. Returns the number of matches."""
        assert out.dtype == np.uint32 and out.ndim == 2 and out.shape[1] == 2 and out.flags.c_contiguous
        assert offsets.dtype == np.uint64 and offsets.shape == (self.np + 1,) and offsets.flags.c_contiguous
        st = SlmStats()
        check(self._L.slm_plan_results(self._h, out.ctypes.data_as(ctypes.POINTER(SlmPair)), len(out),
                                       offsets.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), ctypes.byref(st)),
              "slm_plan_results")
        self.stats = st.as_dict()
        return int(offsets[-1])

    def per_pair(self):
        pairs, off = self.results()
        return [pairs[int(off[k]):int(off[k + 1])] for k in range(self.np)]

    def set_min_matches(self, min_matches: int) -> None:
        """match_pairs' filter (pipeline.rs:494-496): from the next launch on,
        pairs with fewer matches report none (dropped on the device)."""
        check(self._L.slm_plan_set_min_matches(self._h, int(min_matches)), "slm_plan_set_min_matches")

    def nbytes(self) -> int:
        return int(self._L.slm_plan_bytes(self._h))

    def debug_dump(self, na: int, nb: int) -> np.ndarray:
        """Tensor-core distance estimates of the first pair (plans made with variant=2)."""
        out = np.empty((na, nb), np.float32)
        check(self._L.slm_plan_debug_dump(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), out.size),
              "slm_plan_debug_dump")
        return out

    def close(self) -> None:
        if self._h:
            self._L.slm_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- module API
_default: Matcher | None = None
_default_lock = threading.Lock()


def default_matcher() -> Matcher:
    global _default
    with _default_lock:
        if _default is None:
            _default = Matcher()
        return _default


def ratio_match(a, b, ratio: float, mutual: bool, precision="fp32") -> list[tuple[int, int]]:
    """matching.rs:167: `ratio_match(a, b, ratio, mutual) -> Vec<(usize, usize)>` on the GPU."""
    return default_matcher().ratio_match(a, b, ratio, mutual, precision)


def match_pairs(store: DescriptorStore, pairs, ratio: float = 0.8, mutual: bool = True, precision="fp32"):
    """The matching half of pipeline.rs:485-493: one batch over all pairs; a list of (M_k, 2) arrays."""
    plan = store.plan(pairs, ratio, mutual, precision)
    plan.launch()
    out = plan.per_pair()
    plan.close()
    return out


def _views_array(views) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(views, dtype=np.uint64).reshape(-1, 2))


def _collect(fn, where: str) -> list[tuple[int, int]]:
    n = ctypes.c_uint64(0)
    st = fn(None, 0, ctypes.byref(n))
    if st not in (0, SLM_CAPACITY):
        check(st, where)
    out = (SlmPair * max(n.value, 1))()
    check(fn(out, n.value, ctypes.byref(n)), where)
    return [(out[k].i, out[k].j) for k in range(n.value)]


def candidate_pairs(views, temporal: int, cross: int, pow2_max: int) -> list[tuple[int, int]]:
    """matching.rs:18-40 (host code in libslm; needs no GPU)."""
    L = load()
    v = _views_array(views)
    vp = v.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
    return _collect(lambda o, cap, n: L.slm_candidate_pairs(vp, len(v), temporal, cross, min(pow2_max, USIZE_MAX),
                                                             o, cap, n), "slm_candidate_pairs")


@dataclass
class PairSchedule:
    """matching.rs:74-101 PairSchedule with its CrossSchedule (matching.rs:48-71)."""
    temporal: int = PAIR_TEMPORAL
    pow2_max: int = PAIR_POW2_MAX
    spec: bool = False
    range: int = PAIR_CROSS
    right_min: int = 20
    left_min: int = 20
    max: int = 40
    step: int = 4

    @staticmethod
    def default() -> "PairSchedule":
        return PairSchedule()

    @staticmethod
    def spec_schedule() -> "PairSchedule":
        return PairSchedule(spec=True)

    def _c(self) -> SlmPairSchedule:
        return SlmPairSchedule(self.temporal, self.pow2_max, int(self.spec), self.range, self.right_min,
                               self.left_min, self.max, self.step)


def scheduled_pairs(views, schedule: PairSchedule | None = None) -> list[tuple[int, int]]:
    """matching.rs:103-142 (host code in libslm)."""
    L = load()
    sch = (schedule or PairSchedule.default())._c()
    v = _views_array(views)
    vp = v.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
    return _collect(lambda o, cap, n: L.slm_scheduled_pairs(vp, len(v), ctypes.byref(sch), o, cap, n),
                    "slm_scheduled_pairs")


def match_scheduled_pairs(store: DescriptorStore, views, schedule: PairSchedule | None = None, ratio: float = 0.8,
                          mutual: bool = True, precision="bf16", min_matches: int = 20):
    """The matching half of match_pairs (pipeline.rs:485-496): scheduled_pairs(views,
    schedule or PairSchedule::default()), ratio_match of every pair as one GPU batch
    (store view i is views[i]), and the pairs with at least min_matches matches, in
    schedule order. Returns [(i, j, (M, 2) uint32 matches)]."""
    L = store._L
    sch = (schedule or PairSchedule.default())._c()
    v = _views_array(views)
    vp = v.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
    pair_cap = max(1, len(scheduled_pairs(views, schedule)))
    cap = max(1, sum(store.counts[: len(v)]) * 4)
    while True:
        pairs_out = (SlmPair * pair_cap)()
        offsets = np.zeros(pair_cap + 1, np.uint64)
        out = (SlmPair * cap)()
        n = ctypes.c_uint64()
        st = SlmStats()
        status = L.slm_match_pairs(store.m.handle, store.handle, vp, len(v), ctypes.byref(sch), ctypes.c_float(ratio),
                                   int(bool(mutual)), _prec(precision), int(min_matches), pairs_out, pair_cap,
                                   ctypes.byref(n), out, cap, offsets.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                   ctypes.byref(st))
        if status == SLM_CAPACITY and n.value <= pair_cap and int(offsets[n.value]) > cap:
            cap = int(offsets[n.value])  # more matches than room: once more with the count needed
            continue
        check(status, "slm_match_pairs")
        store.m.last_stats = st.as_dict()
        k = n.value
        pr = np.frombuffer(pairs_out, dtype=np.uint32, count=2 * k).reshape(-1, 2)
        mt = np.frombuffer(out, dtype=np.uint32, count=2 * int(offsets[k])).reshape(-1, 2)
        return [(int(pr[q, 0]), int(pr[q, 1]), mt[int(offsets[q]):int(offsets[q + 1])].copy()) for q in range(k)]
