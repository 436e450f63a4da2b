"""The d-dimensional stochastic-volatility restatement (oracle/oracle.c o_svd_*) pinned on
the CPU: its potential equals the reference's gaussian_potential for a diagonal
likelihood covariance R exp(x) (stochastic_volatility.py:96-102, utils.py:49-105)
computed in float64; at d = 1 its filter matches the pinned dim-1 restatement; the
C-ABI entry points refuse bad arguments before any device call."""
import ctypes

import numpy as np
import pytest

import oracle as O
from oracle import models


def _params(d, seed=0, dense=True):
    rng = np.random.default_rng(seed)
    A = models.random_stable_matrix(d, seed) * 0.9
    Q = 0.2 * np.eye(d) + (0.05 * np.ones((d, d)) if dense else 0)
    R = rng.uniform(0.5, 2.0, d)
    S0 = 0.5 * np.eye(d)
    return models.svd_params(0.1 * np.ones(d), S0, A, Q, R)


@pytest.mark.parametrize("d", [1, 3, 6])
def test_potential_is_the_reference_gaussian_potential(d):
    p = _params(d, seed=d)
    n = 64
    y0 = np.random.default_rng(1).standard_normal(d).astype(np.float32)
    x, lw = O.svd_init(p, n, O.PRNGKey(4), y0)
    R = p["R"]
    for i in range(n):
        var = R * np.exp(x[i].astype(np.float64))
        ref = 0.5 * np.sum(y0.astype(np.float64) ** 2 / var) + 0.5 * np.sum(np.log(2 * np.pi * var))
        assert abs(-float(lw[i]) - ref) <= 2e-5 * max(1.0, abs(ref))


def test_initial_draws_have_the_initial_moments():
    d = 3
    p = _params(d, seed=2)
    x, _ = O.svd_init(p, 200000, O.PRNGKey(5), None)
    np.testing.assert_allclose(x.mean(0), p["m0"], atol=0.01)
    np.testing.assert_allclose(np.cov(x.T), p["S0"], atol=0.01)


def test_dimension_one_matches_the_scalar_restatement():
    """at d = 1 the transition rounds differently (A x + (Lq e) sqrt(dt) against
    fma(x, phi, e bsig)), so the filters agree to rounding, not bit for bit"""
    phi, sigma, R = 0.9, 0.4, 1.3
    p = models.svd_params(np.zeros(1), np.eye(1) * sigma ** 2 / (1 - phi ** 2), phi * np.eye(1),
                          sigma ** 2 * np.eye(1), np.array([R]))
    ps = models.sv_params(phi, sigma, R, initial_variance=sigma ** 2 / (1 - phi ** 2))
    T = 40
    t = np.cumsum(np.r_[0.0, np.random.default_rng(0).uniform(0.5, 1.5, T - 1)]).astype(np.float32)
    _, y = models.simulate_svd(p, t, O.PRNGKey(0))
    a = O.svd_run_hist(p, 4000, O.PRNGKey(2), y, t, 0.5, "systematic")
    b = O.sv_run_hist(ps, 4000, O.PRNGKey(2), y[:, 0], t, 0.5, "systematic")
    assert abs(a["log_z"] - b["log_z"]) <= 1e-3 * abs(b["log_z"])
    np.testing.assert_allclose(a["value"][:, :, 0], b["value"], atol=1e-3)


def test_svd_entry_points_reject_bad_arguments_on_host():
    from mocat_gb300 import _lib
    L = _lib.lib()
    p = ctypes.c_void_p(256)
    eye = np.eye(33, dtype=np.float32)
    v = np.ones(33, np.float32)
    m = _lib.SVDModel(33, eye.ctypes.data, eye.ctypes.data, eye.ctypes.data, v.ctypes.data, v.ctypes.data, 0.0)
    need = L.mgb_pf_svd_workspace(1000, 10, 33, 0)
    assert L.mgb_pf_svd_run(ctypes.byref(m), 1000, 10, p, p, p, 0.5, 0, p, need, None, None) == 2
    assert L.mgb_pf_svd_init(ctypes.byref(m), 1000, p, p, p, p, None) == 2
    m.d = 3
    assert L.mgb_pf_svd_propagate(ctypes.byref(m), 1000, p, p, -1.0, p, None, None, p, p, None) == 1
    assert L.mgb_pf_svd_run(ctypes.byref(m), 1000, 10, p, p, p, 0.5, 7, p, 1 << 30, None, None) == 1
    assert L.mgb_pf_svd_run(ctypes.byref(m), 1000, 10, p, p, p, 0.5, 0, p, 16, None, None) == 4
    m.A = None
    assert L.mgb_pf_svd_init(ctypes.byref(m), 1000, p, p, p, p, None) == 1
