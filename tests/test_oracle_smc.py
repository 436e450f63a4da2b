"""The float64 SMC restatement used to check the GPU sampler (CPU only): its
potential gradient matches finite differences, and its log_norm_constant
estimates the exact d = 2 log evidence (quadrature) within Monte Carlo error --
the reference's own SMC test compares log_norm_constant with a closed form
(test_transport.py:49-55)."""
import numpy as np

import oracle as O
from oracle import smc


def _data(n=100, d=2, seed=0):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, d)).astype(np.float32)
    bt = rng.standard_normal(d)
    y = (rng.random(n) < 1 / (1 + np.exp(-X @ bt))).astype(np.float32)
    return X, y


def test_potential_gradient_finite_differences():
    X, y = _data(50, 3)
    b = np.random.default_rng(1).standard_normal((2, 3))
    _, g = smc.potential_grad(X, y, b)
    h = 1e-6
    for k in range(3):
        e = np.zeros(3)
        e[k] = h
        fd = (smc.potential_grad(X, y, b + e)[0] - smc.potential_grad(X, y, b - e)[0]) / (2 * h)
        np.testing.assert_allclose(fd, g[:, k], rtol=1e-6, atol=1e-6)


def test_restatement_log_evidence_matches_quadrature():
    X, y = _data()
    exact = smc.log_evidence_2d(X, y, 1.0)
    zs = [smc.run(X, y, 1.0, 256, O.PRNGKey(s), stepsize=0.2, mcmc_steps=5, retain=0.5)["log_norm_constant"][-1]
          for s in range(6)]
    se = np.std(zs) / np.sqrt(len(zs))
    assert abs(np.mean(zs) - exact) < 4 * se + 0.02, (np.mean(zs), exact, se)
