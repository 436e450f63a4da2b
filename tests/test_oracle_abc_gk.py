"""g-and-k ABC in the oracle (oracle.gk_simulate, oracle.abc_gk_run; mocat/src/abc/scenarios/gk.py,
tests/test_abc_gk.py): the simulator against a float64 evaluation of the reference's
formula on the same uniform draws, Phi against the exact normal cdf, and the reference's
own check of MetropolisedABCSMCSampler on the scenario (TestMetSMCGK / TestMetSMCGKOnlyA)."""
import math

import numpy as np
import pytest
from scipy.special import ndtr, ndtri

import oracle as O

TRUE4 = np.array([3.0, 1.0, 2.0, 0.5])
TRUE1 = np.array([3.0])


def _unconstrain(c):
    return ndtri(np.asarray(c) / 10.0)


def _f64_summary(x, key, d, n_raw=1000, n_sum=100, c=0.8, buffer=1e-5):
    q = 10.0 * ndtr(np.asarray(x, np.float64))
    A, B, g, k = (q[0], q[1], q[2], q[3]) if d == 4 else (q[0], 1.0, 2.0, c)
    bits = np.asarray(O.random_bits(key, n_raw), np.uint32)
    f = ((bits >> np.uint32(9)) | np.uint32(0x3f800000)).view(np.float32).astype(np.float64) - 1.0
    u = np.maximum(buffer, f * (1 - 2 * buffer) + buffer)
    z = ndtri(u)
    e = np.exp(-g * z)
    v = A + B * (1 + c * (1 - e) / (1 + e)) * z * (1 + z * z) ** k
    return np.sort(v)[(np.arange(n_sum) * n_raw) // n_sum]


def test_normal_cdf_fit():
    """the Numerical Recipes erfc fit behind Phi: within 2e-7 of the exact cdf"""
    xs = np.linspace(-6, 6, 241).astype(np.float32).reshape(-1, 1)
    keys = np.stack([O.PRNGKey(0)] * xs.shape[0])
    # d = 1 rows with one draw: the constrained A = 10 Phi(x) is the summary's offset
    s, _ = O.gk_simulate(xs, keys, 1, n_raw=1, n_sum=1)
    s0, _ = O.gk_simulate(np.zeros_like(xs), keys, 1, n_raw=1, n_sum=1)
    phi = (s[:, 0] - s0[:, 0] + 5.0) / 10.0
    assert np.abs(phi - ndtr(xs[:, 0].astype(np.float64))).max() < 2e-6


@pytest.mark.parametrize("d", [4, 1])
def test_simulator_matches_float64_formula(d):
    rng = np.random.default_rng(d)
    x = rng.standard_normal((6, d)).astype(np.float32) * 0.7
    keys = np.stack([O.PRNGKey(s) for s in range(6)])
    s, _ = O.gk_simulate(x, keys, d)
    for r in range(6):
        ref = _f64_summary(x[r], keys[r], d)
        np.testing.assert_allclose(s[r], ref, rtol=2e-4, atol=2e-4)
    data = s[0]
    _, dist = O.gk_simulate(x, keys, d, data=data)
    assert dist[0] == 0.0 and (dist[1:] > 0).all()


@pytest.mark.parametrize("onlyA", [False, True])
@pytest.mark.parametrize("mode", ["schedule", "adaptive"])
def test_reference_smc_check(onlyA, mode):
    """TestMetSMCGK(OnlyA): n = 1e3, data = likelihood_sample(true params, PRNGKey(0)),
    threshold schedule linspace(100, 10, 10) or retain 0.8 with termination_alpha 0.1:
    |true unconstrained params - mean of the final particles|_1 < 3"""
    d = 1 if onlyA else 4
    true_u = _unconstrain(TRUE1 if onlyA else TRUE4).astype(np.float32)
    data, _ = O.gk_simulate(true_u[None], O.PRNGKey(0)[None], d)
    kw = dict(schedule=np.linspace(100.0, 10.0, 10)) if mode == "schedule" else dict(retain=0.8, term_alpha=0.1)
    out = O.abc_gk_run(d, data[0], 1000, O.PRNGKey(0), **kw)
    assert np.abs(true_u - out["value"].mean(0)).sum() < 3.0
    assert out["iterations"] >= 1
