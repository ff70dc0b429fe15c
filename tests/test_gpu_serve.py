"""GPU: the serving engine (continuous batching over streaming views).

Each request's match lists must be the same when it runs alone (one slot, one
request at a time) and when it is batched with others and overlaps other
batches on the device (three slots, a burst of requests, small batches), and
must equal the oracle's ratio_match for every pair.
"""
import numpy as np
import pytest

import oracle as O
from skylens_match import serve, synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["bf16", "fp32", "fp8"])
def test_serving_results_same_alone_and_in_the_mix(prec):
    z = synth.zone(positions=7, n_range=(150, 900), seed=21)
    reqs = serve.zone_requests(z)
    total = int(z.counts.sum())

    alone = serve.Server(total, len(z.counts), prec, slots=1, max_batch_pairs=4096)
    res_alone = []
    for v, pairs in reqs:
        _, t = alone.submit(z.view(v), pairs)
        res_alone.append(alone.wait(t, cap=int(z.counts[v]) * max(1, len(pairs)))[0])
    st_alone = alone.stats()
    alone.close()

    mix = serve.Server(total, len(z.counts), prec, slots=3, max_batch_pairs=6)
    res_mix, lats, wall = serve.stream_zone(mix, z, rate=None)
    st_mix = mix.stats()
    mix.close()

    assert st_alone["max_batch_requests"] == 1
    assert st_mix["batches"] > 1 and st_mix["max_inflight"] >= 2, st_mix
    for (v, pairs), ra, rm in zip(reqs, res_alone, res_mix):
        assert len(ra) == len(rm) == len(pairs)
        for (u, _), a_k, m_k in zip(pairs, ra, rm):
            assert np.array_equal(a_k, m_k), (u, v)
            assert np.array_equal(a_k, O.ratio_match_np(z.view(u), z.view(v), 0.8, True, threads=8)), (u, v)


def test_serving_within_a_small_hbm_budget():
    """Admission by free HBM: with a budget that holds the store and only a few
    requests' batches, requests queue and run in more, smaller batches; every
    result is still the oracle's and the device memory in use stays within
    the budget."""
    z = synth.zone(positions=7, n_range=(150, 900), seed=22)
    reqs = serve.zone_requests(z)
    total = int(z.counts.sum())
    # store (~12 MB) plus about one batch per slot: a one-request batch of this
    # zone splits its pairs' columns into up to 4 ranges, each with its own
    # candidate records per row (about 17 MB of scratch)
    budget = 96 << 20
    srv = serve.Server(total, len(z.counts), "bf16", slots=3, hbm_budget=budget)
    res, lats, wall = serve.stream_zone(srv, z, rate=None)
    st = srv.stats()
    srv.close()
    print("small budget:", st)
    assert st["completed"] == len(reqs)
    assert 0 < st["bytes_in_use"] <= budget
    for (v, pairs), rv in zip(reqs, res):
        for (u, _), m_k in zip(pairs, rv):
            assert np.array_equal(m_k, O.ratio_match_np(z.view(u), z.view(v), 0.8, True, threads=8)), (u, v)


def test_cancelled_requests_and_the_rest():
    """slm_server_cancel on every third request of a burst (some still queued,
    some already on the GPU): those tickets report SLM_CANCELLED; every other
    request, including those that match against a cancelled request's view,
    still gets the oracle's lists."""
    from skylens_match import _lib
    z = synth.zone(positions=7, n_range=(150, 900), seed=23)
    reqs = serve.zone_requests(z)
    total = int(z.counts.sum())
    srv = serve.Server(total, len(z.counts), "bf16", slots=2, max_batch_pairs=6)
    tickets = [srv.submit(z.view(v), pairs)[1] for v, pairs in reqs]
    cancelled = set(range(0, len(tickets), 3))
    for k in sorted(cancelled):
        srv.cancel(tickets[k])
    with pytest.raises(_lib.SlmError):
        srv.cancel(10 ** 9)  # unknown ticket
    for k, ((v, pairs), t) in enumerate(zip(reqs, tickets)):
        if k in cancelled:
            with pytest.raises(_lib.SlmError) as e:
                srv.wait(t, cap=int(z.counts[v]) * max(1, len(pairs)))
            assert e.value.status == _lib.SLM_CANCELLED
            continue
        res, _ = srv.wait(t, cap=int(z.counts[v]) * max(1, len(pairs)))
        for (u, _), m_k in zip(pairs, res):
            assert np.array_equal(m_k, O.ratio_match_np(z.view(u), z.view(v), 0.8, True, threads=8)), (u, v)
    st = srv.stats()
    srv.close()
    print("cancel:", st)
    assert st["submitted"] == len(reqs)
