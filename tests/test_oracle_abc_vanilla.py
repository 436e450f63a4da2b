"""VanillaABC in the oracle (oracle.abc_vanilla; mocat/src/abc/importance.py:16-118 run as
mocat.run): pinned against a pure-Python float32 restatement of the key chain, prior draws
and simulations on the ABC linear-Gaussian scenario, and checked with the reference's own
TestVanillaLinearGaussianABC (tests/test_abc_linear_gaussian.py)."""
import numpy as np
import pytest

import oracle as O
from test_oracle_abc import F, _fma, _normals, _prior_pot_exact, _sim_dist, params, posterior


def _python_vanilla(p, n, key, thr, rate):
    d = p["m0"].size
    K, s = O.split(key, 2)
    pk, sk = [s], []
    K = O.split(K, 2)[0]
    K, k = O.split(K, 2)
    sk.append(k)
    for _ in range(1, n):
        K, k1, _k2, k3 = O.split(K, 4)
        pk.append(k1)
        sk.append(k3)
    x = np.zeros((n, d), np.float32)
    dist = np.zeros(n, np.float32)
    for i in range(n):
        e = _normals(pk[i], d)
        for r in range(d):
            v = F(p["C0"][r, 0] * e[0])
            for c in range(1, d):
                v = _fma(p["C0"][r, c], e[c], v)
            x[i, r] = F(p["m0"][r] + v)
        dist[i] = _sim_dist(p, x[i], sk[i])
    if rate is not None:
        pos = F(F(rate) * F(n - 1))
        lo, hi = F(np.floor(pos)), F(np.ceil(pos))
        hw = F(pos - lo)
        srt = np.sort(dist)
        thr = F(F(srt[int(lo)] * F(F(1) - hw)) + F(srt[int(hi)] * hw))
    lw = np.where(dist < F(thr), F(0), F(-np.inf)).astype(np.float32)
    return x, dist, lw, F(thr)


@pytest.mark.parametrize("thr,rate", [(1.0, None), (np.inf, 0.3)])
def test_oracle_matches_python_restatement(thr, rate):
    p = params()
    key = O.PRNGKey(5)
    x, dist, lw, t = _python_vanilla(p, 40, key, thr, rate)
    out = O.abc_vanilla(40, key, thr, rate, lg_params=p)
    assert np.array_equal(out["value"], x)
    assert np.array_equal(out["distance"], dist)
    assert np.array_equal(out["log_weight"], lw)
    assert out["threshold"] == t
    assert np.array_equal(out["prior_potential"], np.array([_prior_pot_exact(p, xi) for xi in x], np.float32))


def test_reference_vanilla_checks():
    """TestVanillaLinearGaussianABC: n = 1e5; threshold 5, then acceptance_rate 0.1: the accepted
    particles' mean and covariance within 10 (absolute error sums) of the posterior's, and the
    acceptance fraction 0.1 to 3 decimals"""
    p = params()
    pm, pc = posterior()
    for kw in (dict(threshold=5.0), dict(acceptance_rate=0.1)):
        out = O.abc_vanilla(100000, O.PRNGKey(0), lg_params=p, **kw)
        acc = out["log_weight"] > -np.inf
        x = out["value"][acc].astype(np.float64)
        assert np.abs(pm - x.mean(0)).sum() < 10.0
        assert np.abs(pc - np.cov(x.T)).sum() < 10.0
        if "acceptance_rate" in kw:
            np.testing.assert_almost_equal(acc.mean(), 0.1, decimal=3)
            assert np.isfinite(out["threshold"])
