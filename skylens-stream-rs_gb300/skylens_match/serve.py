"""Serving: views of a zone stream in and are matched against the views
already on the device (libslm's slm_server_* engine: per-tick continuous
batching, admission by free HBM, concurrent batches on separate streams).

`Server` wraps the C engine; `stream_zone` drives it with Poisson arrivals and
returns per-request latencies and throughput.
"""
from __future__ import annotations

import ctypes
import threading
import time

import numpy as np

from ._lib import SLM_TIMEOUT, SlmPair, SlmServerOpts, SlmServerStats, check, load
from .matching import _desc, _prec
from . import synth

SELF = 0xFFFFFFFF  # SLM_SELF: the submitted view itself in a pair list


class Server:
    """libslm serving engine on one GPU."""

    def __init__(self, max_descs: int, max_views: int, precision="bf16", ratio: float = 0.8, mutual: bool = True,
                 slots: int = 3, max_batch_pairs: int = 0, tick_us: int = 200, device: int = 0,
                 hbm_budget: int = 0):
        self._L = load()
        o = SlmServerOpts(device, hbm_budget, max_descs, max_views, slots, max_batch_pairs, tick_us,
                          ctypes.c_float(ratio), int(bool(mutual)), _prec(precision))
        h = ctypes.c_void_p()
        check(self._L.slm_server_create(ctypes.byref(o), ctypes.byref(h)), "slm_server_create")
        self._h = h
        self._np = {}
        self._keep = {}  # arrays of copy=False submissions, until their wait returns

    def submit(self, desc, pairs, copy: bool = True) -> tuple[int, int]:
        """Add one view and request the listed pairs (use SELF for this view).
        copy=False (slm_server_submit_ptr): the rows are read where they lie
        when the request is admitted; this object keeps the array alive until
        the ticket's wait returns."""
        d = _desc(desc)
        pr = np.ascontiguousarray(np.asarray(pairs, dtype=np.uint32).reshape(-1, 2))
        vid, t = ctypes.c_uint32(), ctypes.c_uint64()
        fn = self._L.slm_server_submit if copy else self._L.slm_server_submit_ptr
        check(fn(self._h, ctypes.c_void_p(d.ctypes.data), len(d), pr.ctypes.data_as(ctypes.POINTER(SlmPair)),
                 len(pr), ctypes.byref(vid), ctypes.byref(t)), "slm_server_submit")
        self._np[t.value] = len(pr)
        if not copy:
            self._keep[t.value] = d
        return vid.value, t.value

    def wait(self, ticket: int, cap: int, timeout_s: float = 120.0):
        """(per-pair match arrays, latency ms); cap bounds the total matches."""
        np_ = self._np[ticket]
        out = np.empty((max(cap, 1), 2), np.uint32)
        off = np.empty(np_ + 1, np.uint64)
        lat = ctypes.c_double()
        deadline = time.monotonic() + timeout_s
        while True:
            st = self._L.slm_server_wait(self._h, ticket, 1000, out.ctypes.data_as(ctypes.POINTER(SlmPair)),
                                         max(cap, 1), off.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                         ctypes.byref(lat))
            if st != SLM_TIMEOUT or time.monotonic() > deadline:
                break
        if st != SLM_TIMEOUT:  # the ticket is released: its rows are no longer read
            self._np.pop(ticket, None)
            self._keep.pop(ticket, None)
        check(st, "slm_server_wait")
        # per-pair views of one array (no copies)
        return [out[int(off[k]):int(off[k + 1])] for k in range(np_)], lat.value

    def cancel(self, ticket: int) -> None:
        """slm_server_cancel: the request's pairs are dropped (or its results
        discarded); wait() on the ticket then raises SlmError(SLM_CANCELLED)."""
        check(self._L.slm_server_cancel(self._h, ticket), "slm_server_cancel")

    def stats(self) -> dict:
        s = SlmServerStats()
        check(self._L.slm_server_stats_get(self._h, ctypes.byref(s)), "slm_server_stats_get")
        return s.as_dict()

    def close(self) -> None:
        if self._h:
            self._L.slm_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def zone_requests(z: synth.Zone, view_offset: int = 0):
    """Views arrive in zone order (trajectory order); view v asks for every
    candidate pair (u, v) with u < v, oriented as candidate_pairs orients it.
    view_offset: the server's id of the zone's first view (a server that has
    taken other views before)."""
    by_v = {}
    for u, v in z.pairs.tolist():
        by_v.setdefault(v, []).append((u + view_offset, SELF))
    return [(v, by_v.get(v, [])) for v in range(len(z.counts))]


def stream_zone(srv: Server, z: synth.Zone, rate: float | None, seed: int = 0, copy: bool = False,
                view_offset: int = 0):
    """Submit the zone's views with Poisson arrivals at `rate` views/s (None:
    all at once) and collect every result. Returns (results per view, latencies
    ms, wall seconds from first submit to last result). copy=False submits the
    zone's rows where they lie (slm_server_submit_ptr), copy=True copies each
    view at submission (slm_server_submit). view_offset: as zone_requests."""
    reqs = zone_requests(z, view_offset)
    rng = np.random.Generator(np.random.PCG64(seed))
    gaps = rng.exponential(1.0 / rate, size=len(reqs)) if rate else np.zeros(len(reqs))
    tickets = [None] * len(reqs)
    ready = threading.Semaphore(0)
    t0 = time.perf_counter()

    def producer():
        t = t0
        for k, (v, pairs) in enumerate(reqs):
            t += gaps[k]
            dt = t - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            tickets[k] = srv.submit(z.view(v), pairs, copy=copy)[1]
            ready.release()

    if rate:
        th = threading.Thread(target=producer)
        th.start()
    else:  # all at once: every submission before the first wait (no thread to share the interpreter with)
        producer()
        th = None
    results, lats = [], []
    for k, (v, pairs) in enumerate(reqs):
        ready.acquire()
        res, lat = srv.wait(tickets[k], cap=max(1, int(z.counts[v])) * max(1, len(pairs)))
        results.append(res)
        lats.append(lat)
    wall = time.perf_counter() - t0
    if th is not None:
        th.join()
    return results, np.asarray(lats), wall


def serving_zone(positions: int = 48, seed: int = 5) -> synth.Zone:
    """Serving workload: 3 cameras x `positions`, n ~ log-uniform[500, 4000]."""
    return synth.zone(positions=positions, seed=seed,
                      n_sampler=lambda rng, nv: np.exp(rng.uniform(np.log(500), np.log(4000), size=nv)).astype(int))
