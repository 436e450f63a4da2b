"""NonLinearGaussian (mocat/src/ssm/nonlinear_gaussian.py:19-131) with a user
transition function, through the generic GPU driver, with BootstrapFilter and with
OptimalNonLinearGaussianParticleFilter (:134-281).

* One step of each filter against a float64 numpy restatement of the reference's
  formulas on the same draws (the library's normals equal the oracle's): particles and
  log-weights within float32 rounding.
* With a linear transition function the filters' log Z estimates agree with the exact
  Kalman log-likelihood (oracle.kalman) within Monte Carlo error.
"""
import numpy as np
import pytest
import torch

import oracle as O
from oracle import kalman, models

pytestmark = pytest.mark.gpu


def _scenario(d, dy, seed, nonlinear, dense=True):
    import mocat_gb300 as mg
    rng = np.random.default_rng(seed)
    F = models.random_stable_matrix(d, seed)
    Q = 0.2 * np.eye(d) + (0.05 * np.ones((d, d)) if dense else 0)
    H = rng.standard_normal((dy, d)) / np.sqrt(d)
    R = 0.3 * np.eye(dy) + (0.05 * np.ones((dy, dy)) if dense else 0)
    S0 = np.eye(d)
    Ft = torch.as_tensor(F.astype(np.float32)).cuda()

    class User(mg.ssm.NonLinearGaussian):
        def transition_function(self, x_previous, t_previous, t_new):
            fx = x_previous @ Ft.T
            return fx + 0.5 * torch.sin(x_previous) if nonlinear else fx

    return User(np.zeros(d), S0, Q, H, R), dict(F=F, Q=Q, H=H, R=R, S0=S0, m0=np.zeros(d))


def _f64(x):
    return np.asarray(x.cpu() if isinstance(x, torch.Tensor) else x, np.float64)


def test_dimension_and_routing(cuda):
    import mocat_gb300 as mg
    m, _ = _scenario(3, 2, 0, True)
    assert m.dim == 3 and m.dim_obs == 2
    assert not mg.ssm._fused(m, mg.ssm.BootstrapFilter())
    assert not mg.ssm._fused(m, mg.ssm.OptimalNonLinearGaussianParticleFilter())
    with pytest.raises(NotImplementedError):
        mg.ssm.NonLinearGaussian(np.zeros(2)).transition_function(torch.zeros(1, 2).cuda(), 0.0, 1.0)


@pytest.mark.parametrize("d,dy", [(2, 1), (4, 3)])
def test_one_step_matches_the_reference_formulas(cuda, d, dy):
    import mocat_gb300 as mg
    m, a = _scenario(d, dy, 10 + d, True)
    n = 1000
    keys = mg.random.split(mg.random.PRNGKey(7), n)
    rng = np.random.default_rng(1)
    xp = torch.as_tensor(rng.standard_normal((n, d)).astype(np.float32)).cuda()
    y = rng.standard_normal(dy).astype(np.float32)
    fx = _f64(xp) @ a["F"].T + 0.5 * np.sin(_f64(xp))
    LR = np.linalg.cholesky(a["R"])
    P = np.linalg.inv(LR)
    c = (dy * np.log(2 * np.pi) + np.log(np.linalg.det(a["R"]))) / 2
    # bootstrap: f(x) + e @ chol(Q) with per-particle normals; potential 0.5 |(y - H x) P|^2 + c
    e = np.stack([O.normal(k, d) for k in keys.cpu().numpy()]).astype(np.float64)
    xb = m.transition_sample(xp, 0.0, 1.0, keys)
    np.testing.assert_allclose(_f64(xb), fx + e @ np.linalg.cholesky(a["Q"]), atol=2e-5)
    v = (y - _f64(xb) @ a["H"].T) @ P
    np.testing.assert_allclose(_f64(m.likelihood_potential(xb, y, 1.0)), 0.5 * (v * v).sum(1) + c, rtol=2e-5,
                               atol=2e-5)
    # optimal proposal: one (n, d) normal draw from the first key
    pf = mg.ssm.OptimalNonLinearGaussianParticleFilter()
    pf.startup(m)
    xo, lo = pf.propose_and_intermediate_weight_vectorised(m, xp, 0.0, y, 1.0, keys)
    E = O.normal(keys[0].cpu().numpy(), (n, d)).astype(np.float64)
    r = y - fx @ a["H"].T
    xr = fx + r @ pf.proposal_kalman_gain.T + E @ pf.proposal_covariance_sqrt.T
    np.testing.assert_allclose(_f64(xo), xr, atol=3e-5)
    w = r @ pf.weight_precision_sqrt
    lr = -(0.5 * (w * w).sum(1) + (dy * np.log(2 * np.pi) - np.log(pf.weight_precision_det)) / 2)
    np.testing.assert_allclose(_f64(lo), lr, rtol=2e-5, atol=2e-5)
    xi, li = pf.initial_sample_and_weight_vectorised(m, y, 0.0, keys)
    mean = a["m0"] + pf.initial_kalman_gain @ (y - a["H"] @ a["m0"])
    np.testing.assert_allclose(_f64(xi), mean + E @ pf.initial_conditioned_covariance_sqrt, atol=3e-5)
    assert float(li.abs().max()) == 0.0


def test_linear_transition_log_z_matches_kalman(cuda):
    """f(x) = F x written by the user: both filters estimate the exact log-likelihood.
    Diagonal Q and R: the reference's NonLinearGaussian.transition_sample draws e @ chol(Q)
    (covariance chol(Q)^T chol(Q)) and its optimal filter's initial conditioned precision uses
    H^T inv(chol(R)) inv(chol(R))^T H; both equal the textbook quantities only for diagonal
    matrices, which the one-step test above covers with dense ones."""
    import mocat_gb300 as mg
    d, dy, T = 3, 2, 30
    m, a = _scenario(d, dy, 3, False, dense=False)
    p = models.lg_params(a["m0"], a["S0"], a["F"], a["Q"], a["H"], a["R"])
    _, y = models.simulate_lg(p, T, O.PRNGKey(0))
    L = np.linalg.cholesky(a["Q"])
    # the reference's optimal filter gives the initial particles zero log-weights
    # (nonlinear_gaussian.py:217-229), so its log Z leaves out log p(y_0)
    S = a["H"] @ a["S0"] @ a["H"].T + a["R"]
    r0 = y[0].astype(np.float64) - a["H"] @ a["m0"]
    logp0 = -0.5 * (r0 @ np.linalg.solve(S, r0) + np.log(np.linalg.det(2 * np.pi * S)))
    exact = {"optimal": kalman.loglik(a["F"], a["Q"], a["H"], a["R"], a["m0"], a["S0"], y.astype(np.float64))
             - logp0,
             "bootstrap": kalman.loglik(a["F"], L.T @ L, a["H"], a["R"], a["m0"], a["S0"], y.astype(np.float64))}
    zs = {}
    for name, pf, n in (("bootstrap", mg.ssm.BootstrapFilter(), 20000),
                        ("optimal", mg.ssm.OptimalNonLinearGaussianParticleFilter(), 4000)):
        vals = []
        for k in range(4):
            out = mg.ssm.run_particle_filter_for_marginals(m, pf, y, np.arange(T), mg.random.PRNGKey(10 + k), n=n,
                                                           history=False)
            vals.append(float(out.log_z))
        zs[name] = np.array(vals)
    assert abs(zs["bootstrap"].mean() - exact["bootstrap"]) < 0.25, (zs, exact)
    assert abs(zs["optimal"].mean() - exact["optimal"]) < 0.1, (zs, exact)
    assert zs["optimal"].std() < zs["bootstrap"].std() + 0.05
