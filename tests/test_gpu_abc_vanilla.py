"""VanillaABC on the GPU (mocat_gb300.abc.run with VanillaABC; mgb_abc_vanilla_*) vs the oracle
bit for bit (linear-Gaussian and g-and-k scenarios, threshold and acceptance-rate forms), and
the reference's own checks (TestVanillaLinearGaussianABC, TestVanillaGK, TestVanillaGKOnlyA)."""
import numpy as np
import pytest

import oracle as O
from test_oracle_abc import DATA, LIK_COV, LIK_MAT, PRIOR_COV, params, posterior
from test_oracle_abc_gk import TRUE1, TRUE4, _unconstrain

pytestmark = pytest.mark.gpu


def _lg():
    import mocat_gb300 as mg
    return mg.abc.LinearGaussian(prior_mean=np.zeros(3), prior_covariance=PRIOR_COV, data=DATA,
                                 likelihood_matrix=LIK_MAT, likelihood_covariance=LIK_COV)


def _gk(onlyA):
    import mocat_gb300 as mg
    d = 1 if onlyA else 4
    true_u = _unconstrain(TRUE1 if onlyA else TRUE4).astype(np.float32)
    sc = (mg.abc.GKOnlyAThinOrder if onlyA else mg.abc.GKThinOrder)()
    sc.data = sc.likelihood_sample(true_u, mg.random.PRNGKey(0)).cpu().numpy()
    return sc, d, true_u


@pytest.mark.parametrize("kw", [dict(threshold=1.5), dict(acceptance_rate=0.05)])
def test_lg_matches_oracle(cuda, kw):
    import mocat_gb300 as mg
    key = O.PRNGKey(12)
    out = mg.abc.run(_lg(), mg.abc.VanillaABC(**kw), 5000, key)
    ref = O.abc_vanilla(5000, key, lg_params=params(), **kw)
    for k in ("value", "distance", "log_weight", "prior_potential"):
        assert np.array_equal(getattr(out, k).cpu().numpy(), ref[k]), k
    assert np.float32(out.threshold) == ref["threshold"]


@pytest.mark.parametrize("onlyA", [False, True])
def test_gk_matches_oracle(cuda, onlyA):
    import mocat_gb300 as mg
    sc, d, _ = _gk(onlyA)
    key = O.PRNGKey(3)
    out = mg.abc.run(sc, mg.abc.VanillaABC(acceptance_rate=0.2), 400, key)
    ref = O.abc_vanilla(400, key, acceptance_rate=0.2, gk=dict(d=d, data=sc.data))
    for k in ("value", "distance", "log_weight", "prior_potential"):
        assert np.array_equal(getattr(out, k).cpu().numpy(), ref[k]), k


def test_reference_lg_checks(cuda):
    import mocat_gb300 as mg
    pm, pc = posterior()
    for kw in (dict(threshold=5.0), dict(acceptance_rate=0.1)):
        smp = mg.abc.VanillaABC(**kw)
        out = mg.abc.run(_lg(), smp, 100000, mg.random.PRNGKey(0))
        acc = (out.log_weight > -np.inf).cpu().numpy()
        x = out.value.double().cpu().numpy()[acc]
        assert np.abs(pm - x.mean(0)).sum() < 10.0
        assert np.abs(pc - np.cov(x.T)).sum() < 10.0
        if "acceptance_rate" in kw:
            np.testing.assert_almost_equal(acc.mean(), 0.1, decimal=3)
            assert smp.parameters.threshold != np.inf


@pytest.mark.parametrize("onlyA", [False, True])
def test_reference_gk_checks(cuda, onlyA):
    """TestVanillaGK / TestVanillaGKOnlyA: n = 1e5, threshold 5 (A only: 1000) and acceptance
    rate 0.1: the accepted mean within 10 of the true parameters; acceptance 0.1 to 3 decimals"""
    import mocat_gb300 as mg
    sc, d, true_u = _gk(onlyA)
    for kw in (dict(threshold=1000.0 if onlyA else 5.0), dict(acceptance_rate=0.1)):
        smp = mg.abc.VanillaABC(**kw)
        out = mg.abc.run(sc, smp, 100000, mg.random.PRNGKey(0))
        acc = (out.log_weight > -np.inf).cpu().numpy()
        assert acc.any()
        x = out.value.double().cpu().numpy()[acc]
        assert np.abs(true_u - x.mean(0)).sum() < 10.0
        if "acceptance_rate" in kw:
            np.testing.assert_almost_equal(acc.mean(), 0.1, decimal=3)
            assert smp.parameters.threshold != np.inf
