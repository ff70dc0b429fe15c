"""GPU: the tensor-core distance estimates of the shortlist path.

The estimate d~ = |a|^2 + |b|^2 - 2 a.b computed from BF16 (or scaled FP8 E4M3)
operands with FP32 accumulation must stay within the per-pair bound eps that
certifies the shortlist; this checks the tcgen05 operand layout and the
bound against an FP64 oracle, and reports the certification counters.
"""
import numpy as np
import pytest

import oracle as O
from skylens_match import synth

pytestmark = pytest.mark.gpu


def eps_bound(a, b, prec):
    """The bound the eps kernel derives (Cauchy-Schwarz on the rounding residuals)."""
    import torch
    def q(x):
        t = torch.from_numpy(x)
        if prec == "bf16":
            return t.to(torch.bfloat16).to(torch.float32).numpy()
        amax = np.abs(x).max(axis=1, keepdims=True)
        e = np.frexp(448.0 / amax)[1]
        s = np.ldexp(1.0, e - 1).astype(np.float32)
        return (torch.from_numpy(x * s).to(torch.float8_e4m3fn).to(torch.float32).numpy() / s)
    qa, qb = q(a), q(b)
    A, B = np.linalg.norm(a, axis=1).max(), np.linalg.norm(b, axis=1).max()
    Ra, Rb = np.linalg.norm(a - qa, axis=1).max(), np.linalg.norm(b - qb, axis=1).max()
    Qa, Qb = np.linalg.norm(qa, axis=1).max(), np.linalg.norm(qb, axis=1).max()
    eps = 2 * (Ra * B + Qa * Rb) * (1 + 1e-3)
    eps += 5e-4 * Qa * Qb + 5e-5 * (A * A + B * B) + 2e-5 * (A + B) ** 2 + 1e-6
    if prec == "bf16":  # the norms are folded into the tensor-core product
        eps += 5e-4 * (A * A + B * B)
    return eps


@pytest.mark.parametrize("prec", ["bf16", "fp8"])
@pytest.mark.parametrize("na,nb", [(200, 300), (129, 77), (300, 513)])
def test_distance_estimates_within_bound(matcher, prec, na, nb):
    rng = np.random.Generator(np.random.PCG64(na + 7 * nb))
    a = synth.sift_like(rng, na)
    b = np.concatenate([synth.noisy_copy(rng, a[: min(na, nb) // 2], 0.05), synth.sift_like(rng, nb - min(na, nb) // 2)])
    st = matcher.store(na + nb, 2)
    st.add_view(a)
    st.add_view(b)
    plan = st.plan([(0, 1)], 0.8, True, prec, variant=2)
    plan.launch()
    got, off = plan.results()
    dt = plan.debug_dump(na, nb)
    ref64 = O.dist_matrix_f64(a, b)
    err = np.abs(dt.astype(np.float64) - ref64)
    eps = eps_bound(a, b, prec)
    print(f"{prec} {na}x{nb}: max |d~ - d64| = {err.max():.3e}, bound eps = {eps:.3e}")
    assert np.isfinite(dt).all()
    assert err.max() <= eps
    # and the match list is the reference's
    assert np.array_equal(got, O.ratio_match_np(a, b, 0.8, True, threads=4))
    plan.close()
    st.close()


def test_bf16_certifies_most_rows(matcher):
    """On the 8192-descriptor pair the approximate bounds settle almost every row."""
    a, b = synth.pair_large(8192, 0.5, 0.05, seed=2)
    got = matcher.ratio_match_np(a, b, 0.8, True, "bf16")
    s = matcher.last_stats
    print("bf16 8192x8192 stats:", s)
    assert np.array_equal(got, O.ratio_match_np(a, b, 0.8, True, threads=16))
    assert s["rows_recomputed"] <= 0.01 * 8192
    assert s["rows_rescored"] <= 0.2 * 8192
