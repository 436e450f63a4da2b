"""GPU bootstrap filter on the one-dimensional non-linear benchmark
(mocat/src/ssm/scenarios/nonlinear1d.py:16-80) vs the oracle.

Bit-exact: particles, log-weights, ancestors and resampling decisions; ESS and
log Z relative 1e-5 (float64 partial sums combined in a different order).
"""
import numpy as np
import pytest
import torch

import oracle as O

pytestmark = pytest.mark.gpu


def _setup(seed=0, T=30):
    import mocat_gb300 as mg
    ssm = mg.ssm.NonLinear1DBenchmark()
    p, _ = ssm.derived()
    t = np.arange(T, dtype=np.float32)
    sim = ssm.simulate(t, mg.random.PRNGKey(seed))
    y = sim.y.cpu().numpy().reshape(-1)
    return mg, ssm, p, t, y, sim


def _key(k):
    return torch.from_numpy(np.asarray(k, np.uint32).view(np.int32)).cuda().view(torch.uint32)


@pytest.mark.parametrize("n", [3000, 3001])
def test_init_and_step_bit_exact(cuda, n):
    mg, ssm, p, t, y, _ = _setup(1)
    from mocat_gb300.ssm import _step
    key = O.PRNGKey(1)
    x0, lw0 = O.nl_init(p, n, key, y[0])
    ip = mg.ssm.initiate_particles(ssm, mg.ssm.BootstrapFilter(), n, key, y[0])
    assert np.array_equal(ip.value[0, :, 0].cpu().numpy(), x0)
    assert np.array_equal(ip.log_weight[0].cpu().numpy(), lw0)
    kt = O.split(O.PRNGKey(2), 1)[0]
    anc = np.sort(np.random.default_rng(0).integers(0, n, n)).astype(np.int32)
    lw_in = np.random.default_rng(1).standard_normal(n).astype(np.float32)
    _, s = ssm.derived()
    for a, lwp, tp in ((None, lw_in, 0.0), (anc, None, 17.0), (None, None, 999.0)):
        xr, lr = O.nl_propagate(p, kt, y[1], tp, x0, a, lwp)
        xn, ln = _step(s, n, _key(kt), torch.from_numpy(y[1:2].copy()).cuda(),
                       torch.from_numpy(x0[None].copy()).cuda(), None if a is None else torch.from_numpy(a).cuda(),
                       None if lwp is None else torch.from_numpy(lwp).cuda(), "mgb_pf_nl1d", t_prev=tp)
        assert np.array_equal(xn[0].cpu().numpy(), xr)
        assert np.array_equal(ln.cpu().numpy(), lr)


@pytest.mark.parametrize("scheme", ["systematic", "multinomial", "categorical"])
@pytest.mark.parametrize("odd", [False, True])
def test_run_matches_oracle(cuda, scheme, odd):
    mg, ssm, p, t, y, _ = _setup(2)
    n = 2001 if odd else 2000
    key = O.PRNGKey(4)
    ref = O.nl_run(p, n, key, y, t, ess_threshold=0.6, scheme=scheme, history=True)
    out = mg.ssm.run_particle_filter_for_marginals(ssm, mg.ssm.BootstrapFilter(), y, t, key, n=n, ess_threshold=0.6,
                                                   resampling=scheme)
    assert ref["resampled"].sum() > 0
    assert np.array_equal(out.resampled.cpu().numpy(), ref["resampled"])
    assert np.array_equal(out.value[..., 0].cpu().numpy(), ref["value"])
    assert np.array_equal(out.log_weight.cpu().numpy(), ref["log_weight"])
    np.testing.assert_allclose(out.ess.cpu().numpy(), ref["ess"], rtol=1e-5)
    np.testing.assert_allclose(float(out.log_z), ref["log_z"], rtol=1e-5)


def test_run_large_matches_oracle(cuda):
    """2^18 particles, 40 steps, non-integer times: bit-exact final particles"""
    mg, ssm, p, _, _, _ = _setup(3, T=40)
    T, n = 40, 1 << 18
    t = (np.arange(T) * 0.37 + 0.1).astype(np.float32)
    y = (np.random.default_rng(3).standard_normal(T) * 3 + 4).astype(np.float32)
    key = O.PRNGKey(9)
    ref = O.nl_run(p, n, key, y, t, ess_threshold=0.5, scheme="systematic", history=True)
    out = mg.ssm.run_particle_filter_for_marginals(ssm, mg.ssm.BootstrapFilter(), y, t, key, n=n, history=False)
    assert np.array_equal(out.value[0, :, 0].cpu().numpy(), ref["value"][-1])
    assert np.array_equal(out.log_weight[0].cpu().numpy(), ref["log_weight"][-1])
    assert np.array_equal(out.resampled.cpu().numpy(), ref["resampled"])
    np.testing.assert_allclose(float(out.log_z), ref["log_z"], rtol=1e-6)


def test_propagate_and_resume(cuda):
    """propagate_particle_filter step by step (t_previous from the particles) and a run
    resumed from an initial sample give the oracle's particles"""
    mg, ssm, p, t, y, _ = _setup(4, T=8)
    n = 1024
    key = O.PRNGKey(5)
    pf = mg.ssm.BootstrapFilter()
    parts = mg.ssm.initiate_particles(ssm, pf, n, key, y[0], t[0])
    x, lw = O.nl_init(p, n, key, y[0])
    ess = O.lse_ess(lw)[3]
    for s in range(1, 8):
        ks = O.split(O.PRNGKey(100 + s), 1)[0]
        res = np.float32(ess) < np.float32(0.5 * n)
        anc = O.resample_systematic(lw, O.systematic_u_bits(ks))[0] if res else None
        x, lw = O.nl_propagate(p, ks, y[s], t[s - 1], x, anc, None if res else lw)
        ess = O.lse_ess(lw)[3]
        parts = mg.ssm.propagate_particle_filter(ssm, pf, parts, y[s], t[s], ks)
        assert np.array_equal(parts.value[-1, :, 0].cpu().numpy(), x)
        assert np.array_equal(parts.log_weight[-1].cpu().numpy(), lw)
    init = mg.ssm.initiate_particles(ssm, pf, n, key, y[0], t[0])
    rk = O.PRNGKey(11)
    out = mg.ssm.run_particle_filter_for_marginals(ssm, pf, y[1:], t[1:], rk, initial_sample=init)
    keys = O.split(rk, 7)
    x, lw = O.nl_init(p, n, key, y[0])
    ess, tp = O.lse_ess(lw)[3], t[0]
    for i in range(7):
        res = np.float32(ess) < np.float32(0.5 * n)
        anc = O.resample_systematic(lw, O.systematic_u_bits(keys[i]))[0] if res else None
        x, lw = O.nl_propagate(p, keys[i], y[i + 1], tp, x, anc, None if res else lw)
        ess, tp = O.lse_ess(lw)[3], t[i + 1]
    assert np.array_equal(out.value[-1, :, 0].cpu().numpy(), x)


def test_bootstrap_brackets_truth(cuda):
    """the reference's own check (tests/test_ssm.py _test_bootstrap): 20 steps, n = 2000,
    every latent state lies strictly between the particle minimum and maximum"""
    import mocat_gb300 as mg
    ssm = mg.ssm.NonLinear1DBenchmark()
    t = np.arange(20, dtype=np.float32)
    sim = ssm.simulate(t, mg.random.PRNGKey(0))
    assert sim.x.shape[0] == 20 and sim.y.shape[0] == 20
    assert np.array_equal(sim.t.cpu().numpy(), t)
    pf = mg.ssm.run_particle_filter_for_marginals(ssm, mg.ssm.BootstrapFilter(), sim.y, t, mg.random.PRNGKey(0),
                                                  n=2000)
    x = sim.x[:, 0]
    assert bool((x < pf.value.max(dim=1).values[:, 0]).all())
    assert bool((pf.value.min(dim=1).values[:, 0] < x).all())
