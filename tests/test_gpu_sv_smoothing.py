"""Backward simulation, stitching and the online smoothers on the stochastic-volatility model
(dim 1; transition_potential of stochastic_volatility.py:78-85 with pq sqrt(t_new - t_prev))
vs the oracle bit for bit, full and rejection versions, on an uneven time grid; and the
bracketing checks of tests/test_ssm.py (FFBSi full and with max_rejections 2, both online
smoothers full and with maximum_rejections 10) on this model."""
import numpy as np
import pytest
import torch

import oracle as O

pytestmark = pytest.mark.gpu


def _setup(T=10, n=400, seed=1):
    import mocat_gb300 as mg
    ssm = mg.ssm.StochasticVolatility(dim=1, initial_covariance=0.3 ** 2 / (1 - 0.95 ** 2), transition_matrix=0.95,
                                      transition_covariance=0.09, likelihood_covariance_diag=1.0)
    t = np.cumsum(np.random.default_rng(seed).uniform(0.5, 1.5, T)).astype(np.float32)
    sim = ssm.simulate(t, mg.random.PRNGKey(seed))
    pf = mg.ssm.run_particle_filter_for_marginals(ssm, mg.ssm.BootstrapFilter(), sim.y, t, O.PRNGKey(seed + 1), n=n)
    return mg, ssm, t, pf


@pytest.mark.parametrize("max_rej", [0, 2, 12])
def test_backward_simulation_matches_oracle(cuda, max_rej):
    mg, ssm, t, pf = _setup()
    phi, pq = ssm.transition_constants()
    key = O.PRNGKey(9)
    out = mg.ssm.backward_simulation(ssm, pf, key, 250, maximum_rejections=max_rej)
    ref = O.ffbsi_sv(phi, pq, pf.value[..., 0].cpu().numpy(), pf.log_weight.cpu().numpy(), t, key, 250,
                     maximum_rejections=max_rej)
    assert np.array_equal(out.indices.cpu().numpy(), ref[1])
    assert np.array_equal(out.value[..., 0].cpu().numpy(), ref[0])
    if max_rej:
        assert np.array_equal(out.num_transition_evals.cpu().numpy(), ref[2])


@pytest.mark.parametrize("max_rej", [0, 3, 20])
def test_stitch_and_pairs_match_oracle(cuda, max_rej):
    mg, ssm, t, pf = _setup(seed=4)
    phi, pq = ssm.transition_constants()
    key = O.PRNGKey(2)
    x0, x1, lw1 = pf.value[4], pf.value[5], pf.log_weight[5]
    x0n, x1n, lwn = x0[:, 0].cpu().numpy(), x1[:, 0].cpu().numpy(), lw1.cpu().numpy()
    pot = mg.ssm._pair_potential(ssm, x0, x1, None, float(t[4]), float(t[5]))
    assert np.array_equal(pot.cpu().numpy(), O.transition_potential_pairs_sv(phi, pq, x0n, x1n, t[5] - t[4]))
    if max_rej:
        idx, ev = mg.ssm.rejection_stitching(ssm, x0, float(t[4]), x1, float(t[5]), lw1, key, max_rej)
        ri, rev = O.stitch_sv(phi, pq, x0n, x1n, lwn, t[5] - t[4], key, maximum_rejections=max_rej)
        assert ev == rev
    else:
        idx = mg.ssm.full_stitch(ssm, x0, float(t[4]), x1, float(t[5]), lw1, key)
        ri = O.stitch_sv(phi, pq, x0n, x1n, lwn, t[5] - t[4], key)
    assert np.array_equal(idx.cpu().numpy(), ri)


def test_bracketing_checks(cuda):
    import mocat_gb300 as mg
    ssm = mg.ssm.StochasticVolatility(dim=1)
    t = np.arange(20, dtype=np.float32)
    sim = ssm.simulate(t, mg.random.PRNGKey(0))
    x = sim.x[:, 0]
    pf = mg.ssm.run_particle_filter_for_marginals(ssm, mg.ssm.BootstrapFilter(), sim.y, t, mg.random.PRNGKey(0),
                                                  n=10000)
    for mr in (0, 2):
        bs = mg.ssm.backward_simulation(ssm, pf, mg.random.PRNGKey(0), 2000, maximum_rejections=mr)
        assert bool((x < bs.value.max(dim=1).values[:, 0]).all())
        assert bool((bs.value.min(dim=1).values[:, 0] < x).all())
    rkeys = mg.random.split(mg.random.PRNGKey(0), 20)
    for backward_sim in (False, True):
        for mr in (0, 10):
            bf = mg.ssm.BootstrapFilter()
            parts = mg.ssm.initiate_particles(ssm, bf, 2000, rkeys[0], sim.y[0], t=float(t[0]))
            for s in range(1, 20):
                parts = mg.ssm.propagate_particle_smoother(ssm, bf, parts, sim.y[s], float(t[s]), rkeys[s], 3,
                                                           backward_sim=backward_sim, maximum_rejections=mr)
            assert bool(torch.isfinite(parts.value).all())
            assert float((x > parts.value.max(dim=1).values[:, 0]).float().mean()) < 0.1
            assert float((x < parts.value.min(dim=1).values[:, 0]).float().mean()) < 0.1
