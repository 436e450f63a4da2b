"""The float64 SMC restatement used to check the GPU sampler (CPU only): its
potential gradient matches finite differences, and its log_norm_constant
estimates the exact d = 2 log evidence (quadrature) within Monte Carlo error --
the reference's own SMC test compares log_norm_constant with a closed form
(test_transport.py:49-55)."""
import math

import numpy as np
import pytest

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


def _gauss_exact_logz(S, s, t):
    """log of integral N(x; 0, s^2 I) exp(-t/2 x' S^-1 x) dx"""
    d = S.shape[0]
    C = np.linalg.inv(t * np.linalg.inv(S) + np.eye(d) / s ** 2)
    return 0.5 * (np.linalg.slogdet(C)[1] - d * np.log(s ** 2))


@pytest.mark.parametrize("move,kw", [("random_walk", dict(stepsize=1.0, schedule=np.arange(0.1, 1.01, 0.1))),
                                     ("underdamped", dict(stepsize=0.5, leapfrog_steps=3, friction=1.0)),
                                     ("underdamped", dict(stepsize=0.7, leapfrog_steps=1, friction=math.inf,
                                                          schedule=np.linspace(0.05, 1.0, 6)))])
def test_general_restatement_gaussian_log_norm_constant(move, kw):
    """the generalised restatement (RandomWalk / Underdamped with leapfrog steps and friction /
    temperature schedules) on toy_examples.Gaussian reaches the exact tempered evidence"""
    S = np.array([[1.0, 0.9], [0.9, 2.0]])
    Ps = np.linalg.inv(np.linalg.cholesky(S))
    out = smc.run_general(lambda b: smc.gaussian_potential_grad(np.zeros(2), Ps, b), 2, 7.0, 600, O.PRNGKey(4),
                          mcmc_steps=2, retain=0.5, move=move, **kw)
    if "schedule" in kw:
        np.testing.assert_array_equal(out["temperature"], np.asarray(kw["schedule"], np.float32).astype(np.float64))
    assert out["temperature"][-1] >= 1.0
    exact = np.array([_gauss_exact_logz(S, 7.0, t) for t in out["temperature"]])
    assert np.abs(out["log_norm_constant"] - exact).max() < 0.2, (out["log_norm_constant"], exact)
