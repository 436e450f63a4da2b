"""GPU ABC-SMC (mocat_gb300.abc) vs the oracle, and the reference's own
statistical check (tests/test_abc_linear_gaussian.py, TestMetSMCLinearGaussianABC).

Bit-exact: particles, distances, log-weights, stepsizes and every per-iteration
threshold, ESS, mean acceptance and resampling flag, for B posteriors at once.
"""
import numpy as np
import pytest

import oracle as O
from test_oracle_abc import DATA, LIK_COV, LIK_MAT, PRIOR_COV, params, posterior

pytestmark = pytest.mark.gpu


def _scenario(S0=PRIOR_COV, H=LIK_MAT, R=LIK_COV, data=DATA):
    import mocat_gb300 as mg
    return mg.abc.LinearGaussian(prior_mean=np.zeros(S0.shape[0]), prior_covariance=S0, data=data,
                                 likelihood_matrix=H, likelihood_covariance=R)


def _models():
    rng = np.random.default_rng(5)
    A = rng.standard_normal((2, 2))
    S2 = A @ A.T + 0.5 * np.eye(2)
    return {"d3dy2": (PRIOR_COV, LIK_MAT, LIK_COV, DATA),
            "d2dy2": (S2, np.array([[1.0, 0.3], [-0.2, 0.8]]), np.array([[0.1, 0.02], [0.02, 0.05]]),
                      np.array([0.7, -1.1])),
            "d1dy1": (np.array([[2.0]]), np.array([[1.0]]), np.array([[0.1]]), np.array([0.4]))}


@pytest.mark.parametrize("model", ["d3dy2", "d2dy2", "d1dy1"])
@pytest.mark.parametrize("case", ["adaptive", "schedule", "fixed_steps2"])
@pytest.mark.parametrize("N", [1000, 2500])
def test_matches_oracle(cuda, model, case, N):
    import mocat_gb300 as mg
    S0, H, R, data = _models()[model]
    sc = _scenario(S0, H, R, data)
    p = params(S0, H, R, data)
    if case == "adaptive":
        smp, kw = mg.abc.MetropolisedABCSMCSampler(ess_threshold_retain=0.8), dict(retain=0.8)
    elif case == "schedule":
        sch = np.linspace(6, 0.2, 8)
        smp, kw = mg.abc.MetropolisedABCSMCSampler(threshold_schedule=sch), dict(schedule=sch)
    else:
        smp = mg.abc.MetropolisedABCSMCSampler(mg.abc.RandomWalkABC(stepsize=0.05), mcmc_steps=2,
                                               ess_threshold_retain=0.7, max_iter=12)
        kw = dict(retain=0.7, stepsize=0.05, mcmc_steps=2, max_iter=12)
    keys = np.stack([O.PRNGKey(s) for s in (0, 7, 123)])
    out = mg.abc.run_batched(sc, smp, N, keys)
    for b in range(len(keys)):
        ref = O.abc_lg_run(p, N, keys[b], **kw)
        L = ref["iterations"] + 1
        assert int(out.iterations[b]) == ref["iterations"]
        assert np.array_equal(out.threshold[b, :L].cpu().numpy(), ref["threshold"])
        assert np.array_equal(out.ess[b, :L].cpu().numpy(), ref["ess"])
        assert np.array_equal(out.alpha[b, :L].cpu().numpy(), ref["alpha"])
        assert np.array_equal(out.resampled[b, :L].cpu().numpy(), ref["resampled"])
        assert np.array_equal(out.value[b].cpu().numpy(), ref["value"])
        assert np.array_equal(out.distance[b].cpu().numpy(), ref["distance"])
        assert np.array_equal(out.log_weight[b].cpu().numpy(), ref["log_weight"])
        assert np.array_equal(out.stepsize[b].cpu().numpy(), ref["stepsize"])
    assert bool(out.resampled.any())


@pytest.mark.parametrize("mode", ["adaptive", "schedule"])
def test_reference_statistical_check(cuda, mode):
    """n = 1000: posterior mean and covariance (absolute error sums) within 3 of the
    Kalman posterior, as the reference's test asserts"""
    import mocat_gb300 as mg
    sc = _scenario()
    if mode == "adaptive":
        smp = mg.abc.MetropolisedABCSMCSampler(ess_threshold_retain=0.8)
    else:
        smp = mg.abc.MetropolisedABCSMCSampler(threshold_schedule=np.linspace(10, 0.1, 10))
    out = mg.abc.run(sc, smp, 1000, mg.random.PRNGKey(0))
    pm, pc = posterior()
    assert out.value.shape == (out.iterations + 1, 1000, 3)
    x = out.value[-1].double().cpu().numpy()
    assert np.abs(pm - x.mean(0)).sum() < 3.0
    assert np.abs(pc - np.cov(x.T)).sum() < 3.0
    assert out.threshold.shape[0] == out.iterations + 1
    assert float(out.threshold[-1]) < float(out.threshold[0])


def test_many_posteriors_agree_statistically(cuda):
    """64 posteriors of 4096 particles in one batch: every one passes the reference's
    criterion, and they agree with each other.  (The ABC posterior is not the exact one:
    the terminal threshold is comparable to the data noise, and the reference's prior
    potential uses inv(chol(S0)) as its precision square root, which for a correlated
    prior is a different quadratic form; both are reproduced, not corrected.)"""
    import mocat_gb300 as mg
    keys = np.stack([O.PRNGKey(1000 + s) for s in range(64)])
    out = mg.abc.run_batched(_scenario(), mg.abc.MetropolisedABCSMCSampler(ess_threshold_retain=0.8), 4096, keys)
    pm, pc = posterior()
    x = out.value.double().cpu().numpy()
    means = x.mean(1)
    for b in range(64):
        assert np.abs(pm - means[b]).sum() < 3.0
        assert np.abs(pc - np.cov(x[b].T)).sum() < 3.0
    assert np.abs(means - means.mean(0)).max() < 0.3
    assert bool((out.iterations > 5).all())
