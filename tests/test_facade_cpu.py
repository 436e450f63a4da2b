"""Host-side pieces of the Python facade that need no GPU: the optimal-proposal
filter's startup constants (nonlinear_gaussian.py:154-184) equal the oracle's,
and the stochastic-volatility constants follow the oracle's definitions."""
import numpy as np

from oracle import models


def test_optimal_proposal_startup_matches_oracle():
    import mocat_gb300 as mg
    for d, dy, seed in [(1, 1, 1), (3, 3, 3), (10, 10, 10), (5, 1, 5)]:
        rng = np.random.default_rng(seed)
        F = models.random_stable_matrix(d, seed)
        Q = 0.1 * np.eye(d) + (0.02 * np.ones((d, d)) if d > 1 else 0)
        H = np.eye(d) if dy == d else rng.standard_normal((dy, d)) / np.sqrt(d)
        R = 0.5 * np.eye(dy) + (0.1 * np.ones((dy, dy)) if dy > 1 else 0)
        p = models.opt_params(np.zeros(d), np.eye(d), F, Q, H, R)
        ssm = mg.ssm.TimeHomogenousLinearGaussian(np.zeros(d), np.eye(d), F, Q, H, R)
        pf = mg.ssm.OptimalNonLinearGaussianParticleFilter()
        pf.startup(ssm)
        for k in ("F", "H", "K", "S", "W", "K0", "C0c", "m0", "cw"):
            assert np.array_equal(np.asarray(pf._consts[k]), np.asarray(p[k])), (d, dy, k)


def test_stochastic_volatility_constants():
    import mocat_gb300 as mg
    sc = mg.ssm.StochasticVolatility(dim=1, initial_covariance=0.3 ** 2 / (1 - 0.95 ** 2), transition_matrix=0.95,
                                     transition_covariance=0.09, likelihood_covariance_diag=1.0)
    p, s = sc.derived()
    q = models.sv_params(phi=0.95, sigma=0.3, likelihood_variance=1.0)
    for k in ("phi", "bsig", "r2", "cB", "c0", "m0"):
        assert np.float32(p[k]) == np.float32(q[k]), k
    assert s.phi == np.float32(0.95)


def test_sv_smoothing_checks():
    """the online smoother takes the stochastic-volatility model with the bootstrap filter
    and refuses other filters"""
    import pytest
    import mocat_gb300 as mg
    ssm = mg.ssm.StochasticVolatility(dim=1)
    mg.ssm._check_smoother(ssm, mg.ssm.BootstrapFilter())
    with pytest.raises(NotImplementedError):
        mg.ssm._check_smoother(ssm, mg.ssm.OptimalNonLinearGaussianParticleFilter())
    phi, pq = ssm.transition_constants()
    assert phi == 1.0 and pq == 1.0


def test_fused_routing():
    """built-in models with built-in filters stay on the fused kernels; subclasses that keep
    the plugin methods too; overriding a plugin method, or a model of the user's own,
    routes to the generic driver"""
    import mocat_gb300 as mg
    lg = mg.ssm.TimeHomogenousLinearGaussian(np.zeros(2), np.eye(2), 0.5 * np.eye(2), np.eye(2), np.eye(2), np.eye(2))
    assert mg.ssm._fused(lg, mg.ssm.BootstrapFilter())

    class Named(mg.ssm.TimeHomogenousLinearGaussian):
        name = "mine"
    assert mg.ssm._fused(Named(np.zeros(2), np.eye(2), 0.5 * np.eye(2), np.eye(2), np.eye(2), np.eye(2)),
                         mg.ssm.BootstrapFilter())

    class MyBoot(mg.ssm.BootstrapFilter):
        def propose_and_intermediate_weight_vectorised(self, *a):
            return super().propose_and_intermediate_weight_vectorised(*a)
    assert not mg.ssm._fused(lg, MyBoot())

    class Mine(mg.ssm.StateSpaceModel):
        dim = dim_obs = 1
    assert not mg.ssm._fused(Mine(), mg.ssm.BootstrapFilter())
