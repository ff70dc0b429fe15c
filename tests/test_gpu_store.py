"""GPU: the descriptor store's batched upload (slm_store_add_views).

Many views come from one host buffer: from pageable memory through one
host-to-device copy and a scatter kernel into padded store rows; from pinned
or device memory by one copy per view. Views may be empty, listed out of
buffer order, leave gaps in the buffer or share rows; a batch that does not
fit is refused whole, leaving the store as it was.
"""
import numpy as np
import pytest

import oracle as O
import skylens_match as sm
from skylens_match import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("memory", ["pageable", "pinned", "device"])
def test_add_views_layouts(matcher, memory):
    rng = np.random.Generator(np.random.PCG64(41))
    buf = synth.sift_like(rng, 1000)
    # (offset, count) per view: out of order, a gap (rows 600-699 unused), an
    # empty view, one view that overlaps another, a single row
    spec = [(700, 300), (0, 250), (250, 0), (250, 350), (100, 200), (999, 1)]
    st = matcher.store(sum(c for _, c in spec), len(spec))
    if memory == "pageable":
        ids = st.add_views_packed(buf, [o for o, _ in spec], [c for _, c in spec])
    else:
        torch = pytest.importorskip("torch")
        t = torch.from_numpy(buf)
        t = t.pin_memory() if memory == "pinned" else t.cuda()
        torch.cuda.synchronize()
        ids = st.add_views_ptr(t.data_ptr(), [o for o, _ in spec], [c for _, c in spec])
        st._keep_tensor = t  # the copies are asynchronous
    assert ids == list(range(len(spec)))
    views = [buf[o:o + c] for o, c in spec]
    pairs = [(u, v) for u in range(len(spec)) for v in range(len(spec)) if u != v]
    for prec in ("fp32", "bf16"):
        plan = st.plan(pairs, 0.8, True, prec)
        plan.launch()
        got = plan.per_pair()
        for k, (u, v) in enumerate(pairs):
            assert np.array_equal(got[k], O.ratio_match_np(views[u], views[v], 0.8, True, threads=8)), (prec, u, v)
        plan.close()
    st.close()


def test_add_views_refused_whole(matcher):
    rng = np.random.Generator(np.random.PCG64(42))
    buf = synth.sift_like(rng, 300)
    st = matcher.store(300, 3)
    st.add_views_packed(buf, [0], [100])
    with pytest.raises(sm.SlmError) as e:
        st.add_views_packed(buf, [0, 100, 200], [100, 100, 100])  # four views in a store of three
    assert "capacity" in str(e.value)
    assert len(st) == 1
    # the store still works and takes a batch that fits
    assert st.add_views_packed(buf, [100, 200], [100, 100]) == [1, 2]
    plan = st.plan([(0, 1), (2, 0)], 0.8, True, "bf16")
    plan.launch()
    got = plan.per_pair()
    assert np.array_equal(got[0], O.ratio_match_np(buf[:100], buf[100:200], 0.8, True, threads=4))
    assert np.array_equal(got[1], O.ratio_match_np(buf[200:], buf[:100], 0.8, True, threads=4))
    plan.close()
    st.close()


@pytest.mark.parametrize("memory", ["pageable", "device"])
def test_more_views_than_one_copy_each(matcher, memory):
    """Above 4096 views per call the upload is one staging copy and a scatter
    kernel, also from device memory."""
    rng = np.random.Generator(np.random.PCG64(43))
    counts = rng.integers(1, 4, size=5000).astype(np.uint32)
    offsets = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.uint64)
    buf = synth.sift_like(rng, int(counts.sum()))
    st = matcher.store(int(counts.sum()), len(counts))
    if memory == "pageable":
        ids = st.add_views_packed(buf, offsets, counts)
    else:
        torch = pytest.importorskip("torch")
        t = torch.from_numpy(buf).cuda()
        torch.cuda.synchronize()
        ids = st.add_views_ptr(t.data_ptr(), offsets, counts)
        st._keep_tensor = t
    assert ids == list(range(len(counts)))
    # random pairs of these 1-3 row views (a one-row b view has no second neighbour: an empty list)
    pairs = [(int(u), int(v)) for u, v in rng.integers(0, len(counts), size=(64, 2))]
    plan = st.plan(pairs, 0.8, True, "fp32")
    plan.launch()
    got = plan.per_pair()
    for k, (u, v) in enumerate(pairs):
        a = buf[int(offsets[u]):int(offsets[u]) + int(counts[u])]
        b = buf[int(offsets[v]):int(offsets[v]) + int(counts[v])]
        assert np.array_equal(got[k], O.ratio_match_np(a, b, 0.8, True, threads=2)), (u, v)
    plan.close()
    st.close()
