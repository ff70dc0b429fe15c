"""GPU: coalescing of concurrent single-pair calls (slm_ctx_set_coalescing).

Host threads call ratio_match once per pair, as the reference's rayon workers
do (pipeline.rs:487-493); with coalescing on, the context gathers the waiting
calls into batch launches. Every caller must get the list of the call made
alone (the oracle's), whatever the batch it landed in, with mixed ratios and
cross-check settings among the concurrent calls.
"""
import threading

import numpy as np
import pytest

import oracle as O
import skylens_match as sm
from skylens_match import synth

pytestmark = pytest.mark.gpu


def run_threads(m, z, jobs, nthreads):
    res, errs = {}, []
    lock = threading.Lock()
    it = iter(range(len(jobs)))

    def work():
        while True:
            with lock:
                k = next(it, None)
            if k is None:
                return
            u, v, ratio, mutual = jobs[k]
            try:
                res[k] = m.ratio_match_np(z.view(u), z.view(v), ratio, mutual, "auto")
            except Exception as e:  # noqa: BLE001 - reported below
                errs.append(e)

    ths = [threading.Thread(target=work) for _ in range(nthreads)]
    [t.start() for t in ths]
    [t.join() for t in ths]
    assert not errs, errs[:3]
    return res


def test_coalesced_calls_equal_oracle():
    z = synth.zone(positions=8, n_range=(100, 1500), seed=61)
    settings = [(0.8, True), (0.95, False), (0.7, True)]
    jobs = [(int(u), int(v)) + settings[k % 3] for k, (u, v) in enumerate(z.pairs)]
    with sm.Matcher() as m:
        m.set_coalescing(window_us=300, max_pairs=48)
        res = run_threads(m, z, jobs, 12)
        stats = m.coalescing_stats()
        print("coalescing:", stats)
        assert stats["calls"] == len(jobs)
        assert stats["max_batch"] > 1 and stats["batches"] < len(jobs)
        for k, (u, v, ratio, mutual) in enumerate(jobs):
            want = O.ratio_match_np(z.view(u), z.view(v), ratio, mutual, threads=8)
            assert np.array_equal(res[k], want), (k, u, v, ratio, mutual)
        # off again: calls go one by one and still match
        m.set_coalescing(0, 0)
        assert m.coalescing_stats()["calls"] == 0
        u, v, ratio, mutual = jobs[0]
        assert np.array_equal(m.ratio_match_np(z.view(u), z.view(v), ratio, mutual, "auto"), res[0])


def test_coalescing_arguments():
    with sm.Matcher() as m:
        for w, p in ((0, 4097), (1000001, 8)):
            with pytest.raises(sm.SlmError):
                m.set_coalescing(w, p)
        m.set_coalescing(0, 1)  # batches of one call: the path itself
        a, b = synth.pair_800(2)
        assert np.array_equal(m.ratio_match_np(a, b, 0.8, True, "auto"), O.ratio_match_np(a, b, 0.8, True, threads=8))
        assert m.coalescing_stats()["batches"] == 1
