"""Host-side logic of the façade (no GPU): sampler parameter handling and scenario constants
that the kernels receive."""
import math

import numpy as np
import pytest


def test_smc_schedule_rules():
    """TemperedSMCSampler.__setattr__ / MetropolisedSMCSampler.__init__ (smc.py:113-125, 243-265):
    a leading 0 is removed; max_temperature and max_iter follow the schedule"""
    import mocat_gb300 as mg
    s = mg.smc.MetropolisedSMCSampler(mg.smc.RandomWalk(stepsize=1.0), temperature_schedule=np.arange(0.0, 1.1, 0.1))
    assert s.temperature_schedule.dtype == np.float32 and s.temperature_schedule[0] > 0
    assert s.max_iter == 10 and s.max_temperature == pytest.approx(1.0)
    s.set_schedule(np.array([0.5, 0.75]))
    assert s.max_iter == 2 and s.max_temperature == 0.75
    with pytest.raises(NotImplementedError):
        mg.smc.MetropolisedSMCSampler(mg.smc.RandomWalk())          # a stepsize is needed
    with pytest.raises(ValueError):
        mg.smc.MetropolisedSMCSampler(mg.smc.Underdamped(stepsize=0.1, leapfrog_steps=0))


def test_gaussian_scenario_constants():
    """toy_examples.Gaussian: precision_sqrt = inv(chol(covariance)); the prior scales"""
    import mocat_gb300 as mg
    S = np.array([[1.0, 0.9], [0.9, 2.0]])
    g = mg.smc.Gaussian(covariance=S, prior_scale=49.0, prior_sample_scale=7.0)
    np.testing.assert_allclose(g.precision_sqrt, np.linalg.inv(np.linalg.cholesky(S)))
    assert g.dim == 2 and g.prior_scale == 49.0 and g.prior_sample_scale == 7.0
    g1 = mg.smc.Gaussian(dim=3)
    np.testing.assert_allclose(g1.covariance, np.eye(3))
    assert mg.smc.Gaussian(covariance=S).prior_sample_scale == 1.0


def test_gk_constrain_round_trip():
    import mocat_gb300 as mg
    sc = mg.abc.GKThinOrder()
    c = np.array([3.0, 1.0, 2.0, 0.5])
    np.testing.assert_allclose(sc.constrain(sc.unconstrain(c)), c, rtol=1e-10)
    m = sc.model()
    assert (m.d, m.n_unsummarised, m.n_summary) == (4, 1000, 100)
    assert mg.abc.GKOnlyAThinOrder().dim == 1


def test_vanilla_abc_parameters():
    import mocat_gb300 as mg
    v = mg.abc.VanillaABC(threshold=5.0)
    assert v.parameters.threshold == 5.0 and not hasattr(v.parameters, "acceptance_rate")
    v = mg.abc.VanillaABC(acceptance_rate=0.1)
    assert v.parameters.threshold == math.inf and v.parameters.acceptance_rate == 0.1


def test_sv_transition_constants():
    import mocat_gb300 as mg
    sv = mg.ssm.StochasticVolatility(dim=1, transition_matrix=0.95, transition_covariance=0.09)
    phi, pq = sv.transition_constants()
    assert phi == np.float32(0.95) and pq == np.float32(np.float32(1) / np.float32(0.3))
    p, _ = sv.derived(1.0)
    assert p["bsig"] == np.float32(0.3)
