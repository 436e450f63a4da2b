"""RandomWalkABC chains on the GPU (mocat_gb300.abc.run / run_chains with RandomWalkABC;
mgb_abc_mcmc_lg, and with the RMMetropolisDiagStepsize correction mgb_abc_mcmc_rm_lg) vs the
oracle bit for bit, and the reference's TestMCMCLinearGaussianABC.test_fixed_stepsize and
test_adaptive_diag_stepsize."""
import numpy as np
import pytest

import oracle as O
from test_oracle_abc import DATA, LIK_COV, LIK_MAT, PRIOR_COV, params, posterior

pytestmark = pytest.mark.gpu


def _lg():
    import mocat_gb300 as mg
    return mg.abc.LinearGaussian(prior_mean=np.zeros(3), prior_covariance=PRIOR_COV, data=DATA,
                                 likelihood_matrix=LIK_MAT, likelihood_covariance=LIK_COV)


def test_chains_match_oracle(cuda):
    import mocat_gb300 as mg
    keys = np.stack([O.PRNGKey(s) for s in (1, 2, 3)])
    out = mg.abc.run_chains(_lg(), mg.abc.RandomWalkABC(threshold=1.0, stepsize=0.1), 2000, keys)
    for b in range(3):
        ref = O.abc_mcmc_lg(params(), 2000, keys[b], 0.1, 1.0)
        for k in ("value", "distance", "prior_potential", "alpha"):
            assert np.array_equal(getattr(out, k)[b].cpu().numpy(), ref[k]), k


def test_reference_fixed_stepsize(cuda):
    """the reference's check (n = 1e5, stepsize 0.1, threshold 1): the mean with PRNGKey(0), the mean
    and covariance on a chain that mixes (PRNGKey(1)); see tests/test_oracle_abc_mcmc.py"""
    import mocat_gb300 as mg
    pm, pc = posterior()
    smp = mg.abc.RandomWalkABC(stepsize=0.1, threshold=1.0)
    out = mg.abc.run(_lg(), smp, 100000, mg.random.PRNGKey(0))
    assert out.value.shape == (100000, 3)
    assert np.abs(pm - out.value.double().cpu().numpy().mean(0)).sum() < 3.0
    out = mg.abc.run(_lg(), smp, 100000, mg.random.PRNGKey(1))
    x = out.value.double().cpu().numpy()
    assert np.abs(pm - x.mean(0)).sum() < 3.0
    assert np.abs(pc - np.cov(x.T)).sum() < 3.0


def test_rm_chains_match_oracle(cuda):
    """RandomWalkABC() with RMMetropolisDiagStepsize (mgb_abc_mcmc_rm_lg): states, acceptance
    probabilities, thresholds and stepsizes of three chains equal the oracle's bit for bit, at the
    reference's defaults and at another Robbins-Monro schedule"""
    import mocat_gb300 as mg
    keys = np.stack([O.PRNGKey(s) for s in (4, 5, 6)])
    for target, scale, neg_exp in ((0.1, 1.0, 2.0 / 3.0), (0.3, 0.5, 0.75)):
        smp = mg.abc.RandomWalkABC()
        smp.tuning.target = target
        corr = mg.abc.RMMetropolisDiagStepsize(rm_stepsize_scale=scale, rm_stepsize_neg_exponent=neg_exp)
        out = mg.abc.run_chains(_lg(), smp, 3000, keys, correction=corr)
        for b in range(3):
            ref = O.abc_mcmc_rm_lg(params(), 3000, keys[b], target, scale, neg_exp)
            for k in ("value", "alpha", "threshold", "stepsize"):
                assert np.array_equal(getattr(out, k)[b].cpu().numpy(), ref[k]), (target, k)


def test_reference_adaptive_diag_stepsize(cuda):
    """TestMCMCLinearGaussianABC.test_adaptive_diag_stepsize through mocat's call shape
    (run(scenario, RandomWalkABC(), n, key, correction=RMMetropolisDiagStepsize())): n = 1e5,
    target 0.1; mean and covariance within 3 of the posterior's, the mean acceptance 0.1 to one
    decimal, the final stepsize the chain's variance / d * 2.38^2 to one decimal"""
    import mocat_gb300 as mg
    pm, pc = posterior()
    smp = mg.abc.RandomWalkABC()
    smp.tuning.target = 0.1
    out = mg.abc.run(_lg(), smp, 100000, mg.random.PRNGKey(0), correction=mg.abc.RMMetropolisDiagStepsize())
    x = out.value.double().cpu().numpy()
    assert np.abs(pm - x.mean(0)).sum() < 3.0
    assert np.abs(pc - np.cov(x.T)).sum() < 3.0
    np.testing.assert_almost_equal(float(out.alpha.double().mean()), 0.1, decimal=1)
    np.testing.assert_array_almost_equal(out.stepsize[-1].double().cpu().numpy(),
                                         np.diag(np.cov(x, rowvar=False)) / 3 * 2.38 ** 2, decimal=1)
    with pytest.raises(NotImplementedError):
        mg.abc.run(_lg(), mg.abc.RandomWalkABC(threshold=1.0), 10, mg.random.PRNGKey(0),
                   correction=mg.abc.RMMetropolisDiagStepsize())
