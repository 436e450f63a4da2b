"""The d-dimensional stochastic-volatility bootstrap filter on the GPU (run-time-dimension
kernels, mgb_pf_svd_*) against the oracle (o_svd_*): particles, log-weights and
resampling decisions bit for bit, log Z within 1e-5 relative, through the C-ABI and
through run_particle_filter_for_marginals / initiate_particles / propagate_particle_filter
on mocat_gb300.ssm.StochasticVolatility(dim > 1)."""
import numpy as np
import pytest
import torch

import oracle as O
from oracle import models

pytestmark = pytest.mark.gpu


def _model(d, seed, dense=True):
    import mocat_gb300 as mg
    rng = np.random.default_rng(seed)
    A = models.random_stable_matrix(d, seed) * 0.9
    Q = 0.2 * np.eye(d) + (0.05 * np.ones((d, d)) if dense else 0)
    R = rng.uniform(0.5, 2.0, d)
    S0 = 0.5 * np.eye(d)
    m0 = 0.1 * np.ones(d)
    p = models.svd_params(m0, S0, A, Q, R)
    sv = mg.ssm.StochasticVolatility(d, initial_mean=m0, initial_covariance=S0, transition_matrix=A,
                                     transition_covariance=Q, likelihood_covariance_diag=R)
    return p, sv


@pytest.mark.parametrize("d,dense", [(2, True), (3, False), (7, True), (32, False)])
@pytest.mark.parametrize("scheme", ["systematic", "multinomial"])
@pytest.mark.parametrize("n", [2000, 2001])
def test_run_matches_oracle(cuda, d, dense, scheme, n):
    import mocat_gb300 as mg
    p, sv = _model(d, 10 + d, dense)
    T = 20
    t = np.cumsum(np.r_[0.0, np.random.default_rng(d).uniform(0.5, 1.5, T - 1)]).astype(np.float32)
    _, y = models.simulate_svd(p, t, O.PRNGKey(0))
    ref = O.svd_run_hist(p, n, O.PRNGKey(3), y, t, 0.7, scheme)
    out = mg.ssm.run_particle_filter_for_marginals(sv, mg.ssm.BootstrapFilter(), y, t, O.PRNGKey(3), n=n,
                                                   ess_threshold=0.7, resampling=scheme)
    assert ref["resampled"].sum() >= 2
    assert np.array_equal(out.resampled.cpu().numpy(), ref["resampled"])
    assert np.array_equal(out.value.cpu().numpy(), ref["value"])
    assert np.array_equal(out.log_weight.cpu().numpy(), ref["log_weight"])
    np.testing.assert_allclose(out.ess.cpu().numpy(), ref["ess"], rtol=1e-5)
    assert abs(float(out.log_z) - ref["log_z"]) <= 1e-5 * abs(ref["log_z"])


def test_online_steps_match_oracle(cuda):
    import mocat_gb300 as mg
    from mocat_gb300.ssm import _step
    d, n = 5, 3001
    p, sv = _model(d, 3)
    t = np.array([0.0, 0.7, 1.9], np.float32)
    _, y = models.simulate_svd(p, t, O.PRNGKey(1))
    x0, lw0 = O.svd_init(p, n, O.PRNGKey(2), y[0])
    ip = mg.ssm.initiate_particles(sv, mg.ssm.BootstrapFilter(), n, O.PRNGKey(2), y[0], t[0])
    assert np.array_equal(ip.value[0].cpu().numpy(), x0)
    assert np.array_equal(ip.log_weight[0].cpu().numpy(), lw0)
    kt = O.split(O.PRNGKey(4), 1)[0]
    anc = np.sort(np.random.default_rng(0).integers(0, n, n)).astype(np.int32)
    for a, lwp in ((None, lw0), (anc, None)):
        xr, lr = O.svd_propagate(p, kt, y[1], float(np.float32(t[1]) - np.float32(t[0])), x0, a, lwp)
        _, s = sv.derived()
        xn, ln = _step(s, n, torch.from_numpy(kt.view(np.int32)).cuda().view(torch.uint32),
                       torch.from_numpy(y[1]).cuda(), torch.from_numpy(np.ascontiguousarray(x0.T)).cuda(),
                       None if a is None else torch.from_numpy(a).cuda(),
                       None if lwp is None else torch.from_numpy(lwp).cuda(), "mgb_pf_svd", t_prev=t[0], t_new=t[1])
        assert np.array_equal(xn.t().cpu().numpy(), xr)
        assert np.array_equal(ln.cpu().numpy(), lr)
    # the public online step: resample (ESS test) and propagate, as filtering.py:220-252
    pp = mg.ssm.propagate_particle_filter(sv, mg.ssm.BootstrapFilter(), ip, y[1], float(t[1]), O.PRNGKey(6),
                                          ess_threshold=0.0)
    xr, lr = O.svd_propagate(p, O.PRNGKey(6), y[1], float(np.float32(t[1]) - np.float32(t[0])), x0, None, lw0)
    assert np.array_equal(pp.value[1].cpu().numpy(), xr)
    assert np.array_equal(pp.log_weight[1].cpu().numpy(), lr)


def test_simulate_and_limits(cuda):
    import mocat_gb300 as mg
    p, sv = _model(4, 1)
    sim = sv.simulate(np.arange(30.0), mg.random.PRNGKey(0))
    assert sim.x.shape == (30, 4) and sim.y.shape == (30, 4)
    assert torch.isfinite(sim.y).all()
    with pytest.raises(NotImplementedError):  # above the run-time-dimension kernels' limit
        mg.ssm.initiate_particles(mg.ssm.StochasticVolatility(33), mg.ssm.BootstrapFilter(), 10, O.PRNGKey(0),
                                  np.zeros(33, np.float32))
    with pytest.raises(NotImplementedError):  # the smoothers and the batched filters take dim = 1
        sv.transition_constants()
