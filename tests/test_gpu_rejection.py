"""Backward simulation and stitching by rejection sampling (maximum_rejections > 0;
mocat/src/ssm/backward.py:54-214, online_smoothing.py:59-209) on the GPU.

Bit-exact against the oracle: sampled indices, trajectories and the per-step transition
evaluation counts, over settings that reach the bound resets and the final full draw.
The reference's own checks (tests/test_ssm.py _test_ffbsi_rejection with
max_rejections = 2, _test_online_smoothing_{pf,bs}_rejection with maximum_rejections = 10,
lag 3) on the 1-D and 5-D identity models and the non-linear benchmark."""
import numpy as np
import pytest
import torch

import oracle as O
from oracle import models

pytestmark = pytest.mark.gpu


def _lg(d, seed=0):
    import mocat_gb300 as mg
    F = models.random_stable_matrix(d, seed)
    Q = 0.3 * np.eye(d) + (0.05 * np.ones((d, d)) if d > 1 else 0)
    H, R = np.eye(d), 0.5 * np.eye(d)
    p = models.lg_params(np.zeros(d), np.eye(d), F, Q, H, R)
    ssm = mg.ssm.TimeHomogenousLinearGaussian(np.zeros(d), np.eye(d), F, Q, H, R)
    return p, ssm


@pytest.mark.parametrize("d,n,M,T", [(1, 300, 200, 8), (3, 257, 64, 6), (10, 512, 33, 5),
                                     (6, 257, 40, 5)])  # 6: run-time dimension
@pytest.mark.parametrize("max_rej,ibp,infl", [(2, 0.0, 1.01), (10, 0.0, 1.01), (25, 0.02, 1.3)])
def test_backward_simulation_rejection_matches_oracle(cuda, d, n, M, T, max_rej, ibp, infl):
    import mocat_gb300 as mg
    p, ssm = _lg(d, seed=d)
    _, y = models.simulate_lg(p, T, O.PRNGKey(1))
    pf = mg.ssm.run_particle_filter_for_marginals(ssm, mg.ssm.BootstrapFilter(), y, np.arange(T), O.PRNGKey(2), n=n)
    key = O.PRNGKey(3)
    out = mg.ssm.backward_simulation(ssm, pf, key, M, maximum_rejections=max_rej,
                                     transition_dens_bound_parameter=ibp, bound_inflation=infl)
    keep, _ = mg.ssm._transition_struct(ssm)
    ro, ri, rev = O.ffbsi_rejection_lg(keep["F"], keep["Pq"], keep["cq"], pf.value.cpu().numpy(),
                                       pf.log_weight.cpu().numpy(), key, M, max_rej, ibp, infl)
    assert np.array_equal(out.indices.cpu().numpy(), ri)
    assert np.array_equal(out.value.cpu().numpy(), ro)
    assert np.array_equal(out.num_transition_evals.cpu().numpy(), rev)
    assert rev[0] == 0 and (rev[1:] >= M).all()


@pytest.mark.parametrize("d,M", [(1, 1000), (2, 777), (5, 256), (7, 300)])  # 7: run-time dimension
@pytest.mark.parametrize("max_rej", [1, 3, 40])
def test_stitch_rejection_matches_oracle(cuda, d, M, max_rej):
    import mocat_gb300 as mg
    _, ssm = _lg(d, seed=10 + d)
    keep, _ = mg.ssm._transition_struct(ssm)
    rng = np.random.default_rng(d)
    x0 = rng.standard_normal((M, d)).astype(np.float32)
    x1 = (x0 @ keep["F"].T + 0.7 * rng.standard_normal((M, d))).astype(np.float32)
    lw1 = rng.standard_normal(M).astype(np.float32)
    key = O.PRNGKey(9)
    idx, ev = mg.ssm.rejection_stitching(ssm, torch.from_numpy(x0).cuda(), 0.0, torch.from_numpy(x1).cuda(), 1.0,
                                         torch.from_numpy(lw1).cuda(), key, max_rej)
    ri, rev = O.stitch_rejection_lg(keep["F"], keep["Pq"], keep["cq"], x0, x1, lw1, key, max_rej)
    assert np.array_equal(idx.cpu().numpy(), ri)
    assert ev == rev


def test_nl1d_rejection_matches_oracle(cuda):
    import mocat_gb300 as mg
    ssm = mg.ssm.NonLinear1DBenchmark()
    p, _ = ssm.derived()
    T = 8
    t = np.arange(T, dtype=np.float32)
    sim = ssm.simulate(t, mg.random.PRNGKey(4))
    pf = mg.ssm.run_particle_filter_for_marginals(ssm, mg.ssm.BootstrapFilter(), sim.y, t, O.PRNGKey(5), n=600)
    key = O.PRNGKey(6)
    for max_rej in (2, 12):
        out = mg.ssm.backward_simulation(ssm, pf, key, 300, maximum_rejections=max_rej)
        ro, ri, rev = O.ffbsi_rejection_nl1d(p, pf.value[..., 0].cpu().numpy(), pf.log_weight.cpu().numpy(), t, key,
                                             300, max_rej)
        assert np.array_equal(out.indices.cpu().numpy(), ri)
        assert np.array_equal(out.value[..., 0].cpu().numpy(), ro)
        assert np.array_equal(out.num_transition_evals.cpu().numpy(), rev)
    x0 = pf.value[3, :, 0].cpu().numpy()
    x1 = pf.value[4, :, 0].cpu().numpy()
    lw1 = pf.log_weight[4].cpu().numpy()
    idx, ev = mg.ssm.rejection_stitching(ssm, pf.value[3], float(t[3]), pf.value[4], float(t[4]), pf.log_weight[4],
                                         key, 10)
    ri, rev = O.stitch_rejection_nl1d(p, x0, x1, lw1, t[3], key, 10)
    assert np.array_equal(idx.cpu().numpy(), ri) and ev == rev


@pytest.mark.parametrize("model", ["eye1", "eye5", "nl1d"])
def test_reference_rejection_checks(cuda, model):
    """_test_ffbsi_rejection (filter n = 1e4, 2000 samples, max_rejections 2: the samples
    bracket every simulated state) and _test_online_smoothing_{pf,bs}_rejection (n = 2000,
    lag 3, maximum_rejections 10: the truth outside the particle range at under 10 % of times)"""
    import mocat_gb300 as mg
    if model == "nl1d":
        ssm = mg.ssm.NonLinear1DBenchmark()
    else:
        dim = 1 if model == "eye1" else 5
        e = np.eye(dim)
        ssm = mg.ssm.TimeHomogenousLinearGaussian(np.zeros(dim), e, e, e, e, e)
    t = np.arange(20, dtype=np.float32)
    sim = ssm.simulate(t, mg.random.PRNGKey(0))
    x = sim.x[:, 0]
    pf = mg.ssm.run_particle_filter_for_marginals(ssm, mg.ssm.BootstrapFilter(), sim.y, t, mg.random.PRNGKey(0),
                                                  n=10000)
    bs = mg.ssm.backward_simulation(ssm, pf, mg.random.PRNGKey(0), 2000, maximum_rejections=2)
    assert not hasattr(bs, "log_weight")
    assert bool((x < bs.value.max(dim=1).values[:, 0]).all())
    assert bool((bs.value.min(dim=1).values[:, 0] < x).all())
    rkeys = mg.random.split(mg.random.PRNGKey(0), 20)
    for backward_sim in (False, True):
        bf = mg.ssm.BootstrapFilter()
        parts = mg.ssm.initiate_particles(ssm, bf, 2000, rkeys[0], sim.y[0], t=float(t[0]))
        for s in range(1, 20):
            parts = mg.ssm.propagate_particle_smoother(ssm, bf, parts, sim.y[s], float(t[s]), rkeys[s], 3,
                                                       backward_sim=backward_sim, maximum_rejections=10)
        assert bool(torch.isfinite(parts.value).all())
        assert float((x > parts.value.max(dim=1).values[:, 0]).float().mean()) < 0.1
        assert float((x < parts.value.min(dim=1).values[:, 0]).float().mean()) < 0.1
        assert float(parts.num_transition_evals[-1]) > 0
