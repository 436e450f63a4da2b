"""One stochastic-volatility series through run_particle_filter_for_marginals (what a
mocat user calls per series; stochastic_volatility.py:15-108, filtering.py:255-324)
vs the oracle: particles, log-weights and resampling decisions bit for bit, on the
persistent single-launch path (systematic, even n) and the launch-per-step path
(multinomial, odd n), on unit and uneven time grids; log Z as the batched filters
give it for the same key; the bracketing check of tests/test_ssm.py."""
import numpy as np
import pytest

import oracle as O
from oracle import models

pytestmark = pytest.mark.gpu


def _setup(T=60, seed=0):
    import mocat_gb300 as mg
    ssm = mg.ssm.StochasticVolatility(dim=1, initial_covariance=0.3 ** 2 / (1 - 0.95 ** 2), transition_matrix=0.95,
                                      transition_covariance=0.09, likelihood_covariance_diag=1.0)
    p = models.sv_params()
    t = np.arange(T, dtype=np.float32)
    sim = ssm.simulate(t, mg.random.PRNGKey(seed))
    return mg, ssm, p, t, sim.y[:, 0].cpu().numpy()


@pytest.mark.parametrize("n,scheme,persistent", [(4096, "systematic", True), (4096, "systematic", False),
                                                 (1001, "multinomial", True), (2048, "categorical", False)])
def test_filter_matches_oracle(cuda, n, scheme, persistent):
    mg, ssm, p, t, y = _setup()
    key = O.PRNGKey(3)
    out = mg.ssm.run_particle_filter_for_marginals(ssm, mg.ssm.BootstrapFilter(), y, t, key, n=n,
                                                   ess_threshold=0.6, resampling=scheme, persistent=persistent)
    ref = O.sv_run_hist(p, n, key, y, t, ess_threshold=0.6, scheme=scheme)
    assert np.array_equal(out.resampled.cpu().numpy(), ref["resampled"])
    assert np.array_equal(out.value[..., 0].cpu().numpy(), ref["value"])
    assert np.array_equal(out.log_weight.cpu().numpy(), ref["log_weight"])
    np.testing.assert_allclose(float(out.log_z), ref["log_z"], rtol=1e-5)
    assert ref["resampled"].any()


def test_uneven_time_grid(cuda):
    """transition noise scaled by sqrt(t_t - t_{t-1}) per step"""
    mg, ssm, p, _, y = _setup(T=40)
    t = np.cumsum(np.random.default_rng(1).uniform(0.2, 2.5, 40)).astype(np.float32)
    key = O.PRNGKey(8)
    for persistent in (True, False):
        out = mg.ssm.run_particle_filter_for_marginals(ssm, mg.ssm.BootstrapFilter(), y, t, key, n=2048,
                                                       persistent=persistent)
        ref = O.sv_run_hist(p, 2048, key, y, t)
        assert np.array_equal(out.value[..., 0].cpu().numpy(), ref["value"])
        assert np.array_equal(out.log_weight.cpu().numpy(), ref["log_weight"])


def test_log_z_equals_batched(cuda):
    """the same series and key through the batched filters: same resampling count, log Z"""
    mg, ssm, p, t, y = _setup(T=80, seed=2)
    key = O.PRNGKey(5)
    out = mg.ssm.run_particle_filter_for_marginals(ssm, mg.ssm.BootstrapFilter(), y, t, key, n=4096,
                                                   resampling="multinomial", history=False)
    bt = mg.batched.run_particle_filters_batched(ssm, mg.ssm.BootstrapFilter(), [y], key[None], [4096],
                                                 resampling="multinomial")
    np.testing.assert_allclose(float(out.log_z), float(bt.log_z[0]), rtol=1e-5)
    assert int(out.resampled.sum()) == int(bt.resampled_count[0])


def test_propagate_matches_run(cuda):
    """initiate_particles + propagate_particle_filter step by step (dt from the particles'
    times) give the whole run's particles: init key split(key, 2)[1], step keys
    split(split(key, 2)[0], T - 1), resampling every step"""
    mg, ssm, p, _, y = _setup(T=12)
    t = np.cumsum(np.random.default_rng(3).uniform(0.5, 1.5, 12)).astype(np.float32)
    n = 512
    key = O.PRNGKey(9)
    pf = mg.ssm.BootstrapFilter()
    run = mg.ssm.run_particle_filter_for_marginals(ssm, pf, y, t, key, n=n, ess_threshold=2.0)
    k2 = O.split(key, 2)
    steps = O.split(k2[0], 11)
    parts = mg.ssm.initiate_particles(ssm, pf, n, k2[1], y[0], t[0])
    for s in range(1, 12):
        parts = mg.ssm.propagate_particle_filter(ssm, pf, parts, y[s], t[s], steps[s - 1], ess_threshold=2.0)
        assert np.array_equal(parts.value[-1, :, 0].cpu().numpy(), run.value[s, :, 0].cpu().numpy())
        assert np.array_equal(parts.log_weight[-1].cpu().numpy(), run.log_weight[s].cpu().numpy())


def test_bootstrap_brackets_truth(cuda):
    """the check of tests/test_ssm.py _test_bootstrap on this model (default parameters,
    PRNGKey(0), n = 2000): the truth within the particle range at every step"""
    import mocat_gb300 as mg
    ssm = mg.ssm.StochasticVolatility(dim=1)
    t = np.arange(20, dtype=np.float32)
    sim = ssm.simulate(t, mg.random.PRNGKey(0))
    pf = mg.ssm.run_particle_filter_for_marginals(ssm, mg.ssm.BootstrapFilter(), sim.y, t, mg.random.PRNGKey(0),
                                                  n=2000)
    x = sim.x[:, 0]
    assert bool((x < pf.value.max(dim=1).values[:, 0]).all())
    assert bool((pf.value.min(dim=1).values[:, 0] < x).all())
