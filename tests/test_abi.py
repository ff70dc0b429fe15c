"""CPU: libslm loads, exports every symbol include/slm.h declares, and its
host-only entry points (pair generators, argument checks) behave like the
reference. No kernel is launched here."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import oracle as O
import skylens_match as sm
from skylens_match import _lib

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "slm.h")


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(slm_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_bound_functions():
    assert set(header_functions()) == set(_lib.SIGNATURES)


def test_library_exports_every_declared_symbol():
    L = sm.load()
    for name in header_functions():
        assert hasattr(L, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", sm.library_path()], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\b(slm_[a-z0-9_]+)\b", out))
    assert set(header_functions()) <= exported


def test_status_strings():
    L = sm.load()
    assert L.slm_status_str(0) == b"SLM_OK"
    assert L.slm_status_str(2) == b"SLM_CAPACITY"


def rig(p):
    return [(c, q) for q in range(p) for c in range(3)]


@pytest.mark.parametrize("args", [(10, 2, 1, 0), (80, 5, 4, 16), (80, 5, 4, 2**64 - 1), (80, 5, 4, 0), (33, 3, 2, 8)])
def test_candidate_pairs_abi_equals_oracle(args):
    p, t, c, p2 = args
    assert sm.candidate_pairs(rig(p), t, c, p2) == O.candidate_pairs(rig(p), t, c, p2)


def test_candidate_pairs_counts_abi():
    for p in (20, 40, 80, 160):
        assert len(sm.candidate_pairs(rig(p), sm.PAIR_TEMPORAL, sm.PAIR_CROSS, sm.PAIR_POW2_MAX)) == 48 * p - 177


def test_scheduled_pairs_abi_equals_oracle():
    views = rig(60)
    assert sm.scheduled_pairs(views, sm.PairSchedule.default()) == O.scheduled_pairs(views)
    assert sm.scheduled_pairs(views, sm.PairSchedule.spec_schedule()) == O.scheduled_pairs(views, spec_range=4)
    assert sm.scheduled_pairs(views, sm.PairSchedule.spec_schedule()) == sm.candidate_pairs(views, 5, 4, 16)


def test_candidate_pairs_capacity_reports_total():
    L = sm.load()
    v = np.ascontiguousarray(np.asarray(rig(10), np.uint64))
    out = (_lib.SlmPair * 3)()
    n = ctypes.c_uint64()
    st = L.slm_candidate_pairs(v.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), len(v), 2, 1, 0, out, 3,
                               ctypes.byref(n))
    assert st == _lib.SLM_CAPACITY and n.value == 135
    assert [(out[k].i, out[k].j) for k in range(3)] == O.candidate_pairs(rig(10), 2, 1, 0)[:3]


def test_null_arguments_are_rejected():
    L = sm.load()
    n = ctypes.c_uint64()
    assert L.slm_candidate_pairs(None, 5, 1, 1, 1, None, 0, ctypes.byref(n)) == _lib.SLM_INVALID_ARG
    assert L.slm_ratio_match(None, None, 0, None, 0, 0.8, 1, 0, None, 0, None, None) == _lib.SLM_INVALID_ARG
    assert L.slm_ctx_create(None, None) == _lib.SLM_INVALID_ARG


def test_no_device_is_an_error_not_a_fallback():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(sm.SlmError) as e:
        sm.Matcher()
    assert e.value.status == _lib.SLM_NO_DEVICE


def test_detector_config_default_is_the_reference_default():
    # DetectorConfig::default() (features.rs:278-293), without a GPU
    from skylens_match import features as F
    c = F.detector_config()
    o = O.DetectorConfig()
    for f in ("octaves", "scales", "max_features", "upscale_below", "upscale_fill"):
        assert getattr(c, f) == getattr(o, f), f
    for f in ("sigma0", "contrast", "edge_ratio"):
        assert np.float32(getattr(c, f)) == np.float32(getattr(o, f)), f


def test_descriptor_producer_argument_checks_need_no_device():
    from skylens_match import features as F
    L = sm.load()
    cfg = F.detector_config()
    off = np.zeros(2, np.uint64)
    offp = off.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
    img = np.zeros((8, 8), np.float32)
    # NULL context, NULL images with n > 0, oversized images, too many (image, layer) grid slots
    assert L.slm_detect_and_describe(None, ctypes.c_void_p(img.ctypes.data), 1, 8, 8, ctypes.byref(cfg), None, None,
                                     0, offp) == _lib.SLM_INVALID_ARG
    bad = F.detector_config(scales=0)
    assert L.slm_detect_and_describe(None, None, 0, 8, 8, ctypes.byref(bad), None, None, 0, offp) == _lib.SLM_INVALID_ARG
    assert L.slm_describe(None, None, 8, 8, None, 0, None) == _lib.SLM_INVALID_ARG


def test_track_builder_argument_checks_need_no_device():
    L = sm.load()
    nt, no = ctypes.c_uint64(), ctypes.c_uint64()
    assert L.slm_build_tracks_drop(None, None, 0, None, 0, None, 3, 10, None, 0, None, 0, ctypes.byref(nt),
                                   ctypes.byref(no), None) == _lib.SLM_INVALID_ARG
