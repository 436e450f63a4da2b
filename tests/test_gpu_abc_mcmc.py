"""RandomWalkABC chains on the GPU (mocat_gb300.abc.run / run_chains with RandomWalkABC;
mgb_abc_mcmc_lg) vs the oracle bit for bit, and the reference's
TestMCMCLinearGaussianABC.test_fixed_stepsize."""
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
