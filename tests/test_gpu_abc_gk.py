"""g-and-k ABC on the GPU (mocat_gb300.abc.GKTransformedUniformPrior / GKOnlyATransformedUniformPrior,
mgb_abc_gk_*) vs the oracle: summaries of the simulator bit for bit, and the whole
MetropolisedABCSMCSampler run (particles, distances, log-weights, stepsizes, every
iteration's threshold, ESS, acceptance and resampling flag) bit for bit for B posteriors;
the adaptive RandomWalkABC chain bit for bit; and the reference's own checks
(tests/test_abc_gk.py TestMetSMCGK / TestMetSMCGKOnlyA, TestMCMCGK / TestMCMCGKOnlyA)."""
import numpy as np
import pytest
import torch

import oracle as O
from test_oracle_abc_gk import TRUE1, TRUE4, _unconstrain

pytestmark = pytest.mark.gpu


def _scenario(onlyA, data=None, n_raw=1000, n_sum=100):
    import mocat_gb300 as mg
    cls = mg.abc.GKOnlyAThinOrder if onlyA else mg.abc.GKThinOrder
    return cls(n_unsummarised_data=n_raw, num_thin=n_sum, data=data)


@pytest.mark.parametrize("onlyA", [False, True])
@pytest.mark.parametrize("n_raw,n_sum", [(1000, 100), (300, 17), (2048, 64)])
def test_simulator_bit_exact(cuda, onlyA, n_raw, n_sum):
    d = 1 if onlyA else 4
    rng = np.random.default_rng(n_raw)
    x = (rng.standard_normal((50, d)) * 0.8).astype(np.float32)
    keys = np.stack([O.PRNGKey(s) for s in range(50)])
    sc = _scenario(onlyA, n_raw=n_raw, n_sum=n_sum)
    got = sc.simulate_summaries(torch.from_numpy(x).cuda(), keys).cpu().numpy()
    ref, _ = O.gk_simulate(x, keys, d, n_raw=n_raw, n_sum=n_sum)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("onlyA", [False, True])
@pytest.mark.parametrize("mode", ["schedule", "adaptive"])
def test_smc_matches_oracle(cuda, onlyA, mode):
    import mocat_gb300 as mg
    d = 1 if onlyA else 4
    true_u = _unconstrain(TRUE1 if onlyA else TRUE4).astype(np.float32)
    data, _ = O.gk_simulate(true_u[None], O.PRNGKey(0)[None], d)
    sc = _scenario(onlyA, data=data[0])
    if mode == "schedule":
        sch = np.linspace(100.0, 10.0, 6)
        smp, kw = mg.abc.MetropolisedABCSMCSampler(threshold_schedule=sch, mcmc_steps=2), dict(schedule=sch,
                                                                                              mcmc_steps=2)
    else:
        smp = mg.abc.MetropolisedABCSMCSampler(ess_threshold_retain=0.7, termination_alpha=0.1, max_iter=12)
        kw = dict(retain=0.7, term_alpha=0.1, max_iter=12)
    N = 300
    keys = np.stack([O.PRNGKey(4), O.PRNGKey(77)])
    out = mg.abc.run_batched(sc, smp, N, keys)
    for b in range(2):
        ref = O.abc_gk_run(d, data[0], N, keys[b], **kw)
        L = ref["iterations"] + 1
        assert int(out.iterations[b]) == ref["iterations"]
        for k in ("threshold", "ess", "alpha", "resampled"):
            assert np.array_equal(getattr(out, k)[b, :L].cpu().numpy(), ref[k]), k
        for k in ("value", "distance", "log_weight", "stepsize"):
            assert np.array_equal(getattr(out, k)[b].cpu().numpy(), ref[k]), k


@pytest.mark.parametrize("onlyA", [False, True])
@pytest.mark.parametrize("mode", ["schedule", "adaptive"])
def test_reference_check(cuda, onlyA, mode):
    """TestMetSMCGK / TestMetSMCGKOnlyA: n = 1e3, |true - mean(final particles)|_1 < 3"""
    import mocat_gb300 as mg
    d = 1 if onlyA else 4
    true_u = _unconstrain(TRUE1 if onlyA else TRUE4).astype(np.float32)
    sc = _scenario(onlyA)
    sc.data = sc.likelihood_sample(true_u, mg.random.PRNGKey(0)).cpu().numpy()
    if mode == "schedule":
        smp = mg.abc.MetropolisedABCSMCSampler(threshold_schedule=np.linspace(100.0, 10.0, 10))
    else:
        smp = mg.abc.MetropolisedABCSMCSampler(ess_threshold_retain=0.8, termination_alpha=0.1)
    out = mg.abc.run(sc, smp, 1000, mg.random.PRNGKey(0))
    assert np.abs(true_u - out.value[-1].double().cpu().numpy().mean(0)).sum() < 3.0


@pytest.mark.parametrize("onlyA", [False, True])
def test_rm_chain_matches_oracle(cuda, onlyA):
    """RandomWalkABC() with RMMetropolisDiagStepsize on g-and-k (mgb_abc_mcmc_rm_gk, one CTA per
    chain): states, acceptance probabilities, thresholds and stepsizes of two chains equal the
    oracle's bit for bit"""
    import mocat_gb300 as mg
    d = 1 if onlyA else 4
    true_u = _unconstrain(TRUE1 if onlyA else TRUE4).astype(np.float32)
    data, _ = O.gk_simulate(true_u[None], O.PRNGKey(0)[None], d)
    sc = _scenario(onlyA, data=data[0])
    keys = np.stack([O.PRNGKey(31), O.PRNGKey(32)])
    smp = mg.abc.RandomWalkABC()
    scale = 0.1 if onlyA else 0.01
    out = mg.abc.run_chains(sc, smp, 300, keys, correction=mg.abc.RMMetropolisDiagStepsize(rm_stepsize_scale=scale))
    for b in range(2):
        ref = O.abc_mcmc_rm_gk(d, data[0], 300, keys[b], 0.1, scale)
        for k in ("value", "alpha", "threshold", "stepsize"):
            assert np.array_equal(getattr(out, k)[b].cpu().numpy(), ref[k]), k


@pytest.mark.parametrize("onlyA", [False, True])
def test_reference_mcmc_adaptive_diag_stepsize(cuda, onlyA):
    """TestMCMCGK / TestMCMCGKOnlyA.test_adaptive_diag_stepsize: n = 1e5 steps of RandomWalkABC() with
    RMMetropolisDiagStepsize(rm_stepsize_scale=0.01 (0.1 for A only)), target 0.1: |true - mean|_1 < 3
    and the mean acceptance 0.1 to one decimal"""
    import mocat_gb300 as mg
    true_u = _unconstrain(TRUE1 if onlyA else TRUE4).astype(np.float32)
    sc = _scenario(onlyA)
    sc.data = sc.likelihood_sample(true_u, mg.random.PRNGKey(0)).cpu().numpy()
    smp = mg.abc.RandomWalkABC()
    smp.tuning.target = 0.1
    corr = mg.abc.RMMetropolisDiagStepsize(rm_stepsize_scale=0.1 if onlyA else 0.01)
    out = mg.abc.run(sc, smp, 100000, mg.random.PRNGKey(0), correction=corr)
    assert out.value.shape == (100000, 1 if onlyA else 4)
    assert np.abs(true_u - out.value.double().cpu().numpy().mean(0)).sum() < 3.0
    np.testing.assert_almost_equal(float(out.alpha.double().mean()), 0.1, decimal=1)


@pytest.mark.parametrize("onlyA", [False, True])
def test_fixed_chain_matches_oracle(cuda, onlyA):
    """RandomWalkABC(stepsize, threshold) on g-and-k (mgb_abc_mcmc_gk, one CTA per chain): states,
    distances, prior potentials and acceptance probabilities of two chains equal the oracle's"""
    import mocat_gb300 as mg
    d = 1 if onlyA else 4
    true_u = _unconstrain(TRUE1 if onlyA else TRUE4).astype(np.float32)
    data, _ = O.gk_simulate(true_u[None], O.PRNGKey(0)[None], d)
    sc = _scenario(onlyA, data=data[0])
    keys = np.stack([O.PRNGKey(41), O.PRNGKey(42)])
    thr = 50.0
    out = mg.abc.run_chains(sc, mg.abc.RandomWalkABC(stepsize=0.05, threshold=thr), 300, keys)
    accepted = 0
    for b in range(2):
        ref = O.abc_mcmc_gk(d, data[0], 300, keys[b], 0.05, thr)
        accepted += int((ref["alpha"][1:] > 0).sum())
        for k in ("value", "distance", "prior_potential", "alpha"):
            assert np.array_equal(getattr(out, k)[b].cpu().numpy(), ref[k]), k
    assert accepted > 100  # the chains move
