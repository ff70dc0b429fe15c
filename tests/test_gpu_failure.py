"""GPU: the failure path of the bounded device waits, exercised without a fault.

Every wait in libslm's kernels (mbarrier phases, TMEM and TMA completions)
gives up after a fixed number of polls, records an error word and lets the
kernel return; the host turns the word into SLM_TIMEOUT. The self-test entry
point runs that path on purpose on a barrier nothing completes. The wait must
give up, the status must say so, and the same context must go on matching
bit-exactly afterwards.
"""
import numpy as np
import pytest

import oracle as O
from skylens_match import _lib, synth

pytestmark = pytest.mark.gpu


def test_wait_timeout_reported_and_context_survives(matcher):
    for polls in (1, 256, 4096):
        assert matcher.selftest_wait_timeout(polls) == _lib.SLM_TIMEOUT, polls
    detail = _lib.load().slm_last_error().decode()
    assert "gave up" in detail
    rng = np.random.Generator(np.random.PCG64(71))
    a, b = synth.sift_like(rng, 500), synth.sift_like(rng, 700)
    want = O.ratio_match_np(a, b, 0.8, True, threads=8)
    for prec in ("fp32", "bf16"):
        assert np.array_equal(matcher.ratio_match_np(a, b, 0.8, True, prec), want), prec


def test_wait_selftest_rejects_bad_poll_counts(matcher):
    for polls in (0, 65537):
        assert matcher.selftest_wait_timeout(polls) == _lib.SLM_INVALID_ARG, polls
