"""GPU: slm_ratio_match_device_noalloc, the entry point that allocates nothing.

It exists for callers that cannot call cudaMalloc (a framework that owns all
device memory through its own pool, or a latency-critical loop where an
allocation would stall other streams). Its scratch is one fixed device array
in the library, so this checks that two calls in a row (the second smaller than
the first, so the array still holds the first call's data) return exactly what
the allocating entry point slm_ratio_match_device returns, with and without the
cross-check, and that sizes past the array's limit are refused. The output
buffer is exercised in every form the header allows: room for every match
(cap = na and cap > na), a smaller buffer (the first cap pairs and the full
count), and a buffer that is only 4-byte aligned (slm_pair's own alignment),
which must take the field-by-field copy rather than 8-byte stores. This file
sorts last so a failure here comes after every other test has run.
"""
import ctypes

import numpy as np
import pytest

import oracle as O
import skylens_match as sm
from skylens_match import _lib, synth

pytestmark = pytest.mark.gpu

MAX_DESCS = 4096


def _pair(seed, na, nb):
    rng = np.random.Generator(np.random.PCG64(seed))
    a = synth.sift_like(rng, na)
    k = min(na, nb) // 2
    b = np.concatenate([synth.noisy_copy(rng, a[rng.permutation(na)[:k]], 0.05), synth.sift_like(rng, nb - k)])
    return a, np.ascontiguousarray(b[rng.permutation(nb)])


def _noalloc(L, m, da, na, db, nb, mutual, out_ptr, cap, cnt):
    st = L.slm_ratio_match_device_noalloc(ctypes.c_void_p(da.data_ptr()), na, ctypes.c_void_p(db.data_ptr()), nb,
                                          ctypes.c_float(0.8), int(mutual), ctypes.c_void_p(out_ptr), cap,
                                          ctypes.c_void_p(cnt.data_ptr()), ctypes.c_void_p(m.stream))
    _lib.check(st, "slm_ratio_match_device_noalloc")


@pytest.mark.parametrize("mutual", [True, False])
def test_noalloc_equals_allocating_entry_point_twice(mutual):
    torch = pytest.importorskip("torch")
    L = sm.load()
    m = sm.Matcher()
    stream = torch.cuda.ExternalStream(m.stream)
    for seed, na, nb in [(1, 4096, 3900), (2, 700, 1300)]:
        a, b = _pair(seed, na, nb)
        da = torch.from_numpy(a).cuda()
        db = torch.from_numpy(b).cuda()
        ref_out = torch.zeros((na, 2), dtype=torch.int32, device="cuda")
        ref_cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
        out = torch.full((na, 2), -1, dtype=torch.int32, device="cuda")
        cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        m.ratio_match_device(da.data_ptr(), na, db.data_ptr(), nb, 0.8, mutual, "fp32", ref_out.data_ptr(), na,
                             ref_cnt.data_ptr())
        _noalloc(L, m, da, na, db, nb, mutual, out.data_ptr(), na, cnt)
        stream.synchronize()
        n_ref, n = int(ref_cnt.item()), int(cnt.item())
        assert n == n_ref
        got = out[:n].cpu().numpy().astype(np.uint32)
        assert np.array_equal(got, ref_out[:n_ref].cpu().numpy().astype(np.uint32))
        want = O.ratio_match_np(a, b, 0.8, mutual, threads=8)
        assert np.array_equal(got, want)
        # an output buffer larger than needed: the list, nothing past it
        big = torch.full((na + 7, 2), -1, dtype=torch.int32, device="cuda")
        cnt.zero_()
        torch.cuda.synchronize()
        _noalloc(L, m, da, na, db, nb, mutual, big.data_ptr(), na + 7, cnt)
        stream.synchronize()
        assert int(cnt.item()) == len(want)
        big_out = big.cpu().numpy()
        assert np.array_equal(big_out[:len(want)].astype(np.uint32), want)
        assert (big_out[len(want):] == -1).all()
        # an output buffer smaller than na: the first `cap` pairs and the full count
        cap = max(1, len(want) // 3)
        small = torch.full((cap + 1, 2), -1, dtype=torch.int32, device="cuda")
        cnt.zero_()
        torch.cuda.synchronize()
        _noalloc(L, m, da, na, db, nb, mutual, small.data_ptr(), cap, cnt)
        stream.synchronize()
        assert int(cnt.item()) == len(want)
        sm_out = small.cpu().numpy()
        assert np.array_equal(sm_out[:cap].astype(np.uint32), want[:cap])
        assert (sm_out[cap] == -1).all()  # nothing written past cap
        # an output buffer at 4 mod 8 bytes (legal for slm_pair), with room
        # for every match: served through the field-by-field copy
        raw = torch.full((2 * na + 4,), -1, dtype=torch.int32, device="cuda")
        odd = raw[1:]
        assert odd.data_ptr() % 8 == 4
        cnt.zero_()
        torch.cuda.synchronize()
        _noalloc(L, m, da, na, db, nb, mutual, odd.data_ptr(), na, cnt)
        stream.synchronize()
        assert int(cnt.item()) == len(want)
        odd_out = odd[:2 * na].view(na, 2).cpu().numpy()
        assert np.array_equal(odd_out[:len(want)].astype(np.uint32), want)
        assert (odd_out[len(want):] == -1).all()
        assert int(raw[0].item()) == -1  # nothing written before the buffer
    m.close()


def test_noalloc_refuses_sizes_beyond_its_array():
    torch = pytest.importorskip("torch")
    L = sm.load()
    a = torch.zeros((MAX_DESCS + 1, 128), dtype=torch.float32, device="cuda")
    out = torch.zeros((MAX_DESCS + 1, 2), dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = L.slm_ratio_match_device_noalloc(ctypes.c_void_p(a.data_ptr()), MAX_DESCS + 1, ctypes.c_void_p(a.data_ptr()),
                                          16, ctypes.c_float(0.8), 1, ctypes.c_void_p(out.data_ptr()),
                                          MAX_DESCS + 1, ctypes.c_void_p(cnt.data_ptr()), None)
    assert st == _lib.SLM_INVALID_ARG
    assert b"at most 4096" in L.slm_last_error()
