"""GPU optimal-proposal particle filter (linear transition, linear-Gaussian
observations) vs the oracle and the Kalman filter.

Bit-exact: particles, log-weights, ancestors and resampling decisions; log Z
relative 1e-5 (float partial sums in a different order).  One key drives the
whole (n, d) proposal draw (nonlinear_gaussian.py:275).
"""
import numpy as np
import pytest
import torch

import oracle as O
from oracle import kalman, models

pytestmark = pytest.mark.gpu


def _models(d, dy=None, seed=0):
    dy = dy or d
    rng = np.random.default_rng(seed)
    F = models.random_stable_matrix(d, seed)
    Q = 0.1 * np.eye(d) + (0.02 * np.ones((d, d)) if d > 1 else 0)
    H = np.eye(d) if dy == d else rng.standard_normal((dy, d)) / np.sqrt(d)
    R = 0.5 * np.eye(dy) + (0.1 * np.ones((dy, dy)) if dy > 1 else 0)
    S0 = np.eye(d)
    p = models.opt_params(np.zeros(d), S0, F, Q, H, R)
    import mocat_gb300 as mg
    ssm = mg.ssm.TimeHomogenousLinearGaussian(np.zeros(d), S0, F, Q, H, R)
    pf = mg.ssm.OptimalNonLinearGaussianParticleFilter()
    pf.startup(ssm)
    return p, ssm, pf


@pytest.mark.parametrize("n", [3000, 3001])
@pytest.mark.parametrize("d,dy", [(1, 1), (2, 1), (3, 3), (10, 10), (10, 1),
                                  (6, 6), (7, 3), (2, 4), (32, 5)])  # the last four: run-time dimensions
def test_init_and_step_bit_exact(cuda, d, dy, n):
    import mocat_gb300 as mg
    from mocat_gb300.ssm import _step
    p, ssm, pf = _models(d, dy, seed=d)
    _, y = models.simulate_lg(models.lg_params(np.zeros(d), np.eye(d), p["F"], 0.1 * np.eye(d), p["H"],
                                               0.5 * np.eye(dy)), 3, O.PRNGKey(0))
    key = O.PRNGKey(1)
    x0, lw0 = O.opt_init(p, n, key, y[0])
    ip = mg.ssm.initiate_particles(ssm, pf, n, key, y[0])
    assert np.array_equal(ip.value[0].cpu().numpy(), x0)
    assert np.array_equal(ip.log_weight[0].cpu().numpy(), lw0)
    kt = O.split(O.PRNGKey(2), 1)[0]
    anc = np.sort(np.random.default_rng(0).integers(0, n, n)).astype(np.int32)
    lw_in = np.random.default_rng(1).standard_normal(n).astype(np.float32)
    for a, lwp in ((None, lw_in), (anc, None)):
        xr, lr = O.opt_propagate(p, kt, y[1], x0, a, lwp)
        xs = torch.from_numpy(np.ascontiguousarray(x0.T)).cuda()
        xn, ln = _step(pf._struct, n, torch.from_numpy(kt.view(np.int32)).cuda().view(torch.uint32),
                       torch.from_numpy(y[1]).cuda(), xs, None if a is None else torch.from_numpy(a).cuda(),
                       None if lwp is None else torch.from_numpy(lwp).cuda(), "mgb_pf_opt")
        assert np.array_equal(xn.t().cpu().numpy(), xr)
        assert np.array_equal(ln.cpu().numpy(), lr)


@pytest.mark.parametrize("scheme", ["systematic", "multinomial", "categorical"])
@pytest.mark.parametrize("d,dy", [(1, 1), (3, 3), (10, 10), (6, 6), (7, 3)])  # 6, 7: run-time dimensions
@pytest.mark.parametrize("odd", [False, True])
def test_run_matches_oracle(cuda, scheme, d, dy, odd):
    import mocat_gb300 as mg
    p, ssm, pf = _models(d, dy, seed=10 + d)
    n = 2001 if odd else 2000
    T = 25
    _, y = models.simulate_lg(models.lg_params(np.zeros(d), np.eye(d), p["F"], 0.1 * np.eye(d), p["H"],
                                               0.5 * np.eye(dy)), T, O.PRNGKey(3))
    key = O.PRNGKey(4)
    ref = O.opt_run(p, n, key, y, ess_threshold=0.8, scheme=scheme, history=True)
    out = mg.ssm.run_particle_filter_for_marginals(ssm, pf, y, np.arange(T), key, n=n, ess_threshold=0.8,
                                                   resampling=scheme)
    assert np.array_equal(out.resampled.cpu().numpy(), ref["resampled"])
    assert ref["resampled"].sum() > 0
    assert np.array_equal(out.value.cpu().numpy(), ref["value"])
    assert np.array_equal(out.log_weight.cpu().numpy(), ref["log_weight"])
    np.testing.assert_allclose(out.ess.cpu().numpy(), ref["ess"], rtol=1e-5)
    np.testing.assert_allclose(float(out.log_z), ref["log_z"], rtol=1e-5)


def test_log_z_close_to_kalman(cuda):
    """The optimal proposal for a linear-Gaussian model at n = 65536: log Z close to
    the exact Kalman log-likelihood without its t = 0 term."""
    import mocat_gb300 as mg
    d = 10
    F = models.random_stable_matrix(d, 0)
    Q, H, R, S0 = 0.1 * np.eye(d), np.eye(d), 0.5 * np.eye(d), np.eye(d)
    ssm = mg.ssm.TimeHomogenousLinearGaussian(np.zeros(d), S0, F, Q, H, R)
    pf = mg.ssm.OptimalNonLinearGaussianParticleFilter()
    T = 200
    _, y = models.simulate_lg(models.lg_params(np.zeros(d), S0, F, Q, H, R), T, O.PRNGKey(0))
    out = mg.ssm.run_particle_filter_for_marginals(ssm, pf, y, np.arange(T), O.PRNGKey(1), n=65536, history=False)
    ll = kalman.loglik(F, Q, H, R, np.zeros(d), S0, y.astype(np.float64))
    # the reference's initial weights are zero (initial_sample_and_weight_vectorised,
    # nonlinear_gaussian.py:223-230), so its estimate leaves out log p(y_0)
    Sy = H @ S0 @ H.T + R
    y0 = y[0].astype(np.float64)
    lp0 = -0.5 * (d * np.log(2 * np.pi) + np.linalg.slogdet(Sy)[1] + y0 @ np.linalg.solve(Sy, y0))
    assert abs(float(out.log_z) - (ll - lp0)) < 0.05 * np.sqrt(T), (float(out.log_z), ll - lp0)
