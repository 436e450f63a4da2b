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


# ------------------------------------------------ backward simulation, stitching

def test_ffbsi_bit_exact(cuda):
    """backward_simulation (maximum_rejections = 0) on the non-linear model: samples and
    indices equal the oracle's; times are non-integer so every step's drift differs"""
    mg, ssm, p, _, _, _ = _setup(5, T=12)
    T, n, M = 12, 700, 333
    t = (np.arange(T) * 0.61 + 0.2).astype(np.float32)
    y = (np.random.default_rng(5).standard_normal(T) * 3 + 3).astype(np.float32)
    pf = mg.ssm.run_particle_filter_for_marginals(ssm, mg.ssm.BootstrapFilter(), y, t, O.PRNGKey(6), n=n)
    key = O.PRNGKey(12)
    bs = mg.ssm.backward_simulation(ssm, pf, key, M)
    xs, idx = O.ffbsi_nl1d(p, pf.value[..., 0].cpu().numpy(), pf.log_weight.cpu().numpy(), t, key, M)
    assert np.array_equal(bs.indices.cpu().numpy(), idx)
    assert np.array_equal(bs.value[..., 0].cpu().numpy(), xs)
    assert bs.value.shape == (T, M, 1)


def test_stitch_and_pairs_bit_exact(cuda):
    mg, ssm, p, _, _, _ = _setup(6)
    rng = np.random.default_rng(6)
    M0, M1 = 90, 301
    x0 = (rng.standard_normal((M0, 1)) * 5).astype(np.float32)
    x1 = (rng.standard_normal((M1, 1)) * 5).astype(np.float32)
    lw = rng.standard_normal(M1).astype(np.float32)
    key = O.PRNGKey(13)
    for tp in (0.0, 3.0, 41.7):
        idx = mg.ssm.full_stitch(ssm, torch.from_numpy(x0).cuda(), tp, torch.from_numpy(x1).cuda(), tp + 1.0,
                                 torch.from_numpy(lw).cuda(), key)
        assert np.array_equal(idx.cpu().numpy(), O.stitch_nl1d(p, x0, x1, lw, tp, key))
        pp = mg.ssm._pair_potential(ssm, torch.from_numpy(x1[:M0]).cuda(), torch.from_numpy(x1[M1 - M0:]).cuda(),
                                    None, tp)
        assert np.array_equal(pp.cpu().numpy(), O.transition_potential_pairs_nl1d(p, x1[:M0], x1[M1 - M0:], tp))


def test_smoother_pf_variant_matches_oracle(cuda):
    """propagate_particle_smoother(backward_sim=False), lag 3, against an oracle-driven
    restatement (propagate from t_previous, systematic resampling, stitching at t)"""
    mg, ssm, p, t, y, _ = _setup(7, T=12)
    T, lag, n = 12, 3, 500
    keys = O.split(O.PRNGKey(8), T)
    bf = mg.ssm.BootstrapFilter()
    parts = mg.ssm.initiate_particles(ssm, bf, n, keys[0], y[0], t=float(t[0]))
    for s in range(1, T):
        parts = mg.ssm.propagate_particle_smoother(ssm, bf, parts, y[s], float(t[s]), keys[s], lag,
                                                   backward_sim=False)
    x0, lw = O.nl_init(p, n, keys[0], y[0])
    value = [x0]
    for s in range(1, T):
        key = keys[s]
        if O.lse_ess(lw)[3] < n - 1e-3:
            anc = O.resample_systematic(lw, O.systematic_u_bits(key))[0]
            value = [v[anc] for v in value]
        x_new, lw = O.nl_propagate(p, key, y[s], t[s - 1], value[-1])
        value.append(x_new)
        s1 = len(value) - lag - 1
        if s1 >= 0:
            nilw = lw + O.transition_potential_pairs_nl1d(p, value[s1], value[s1 + 1], t[s1])
            idx = O.stitch_nl1d(p, value[s1], value[s1 + 1], nilw, t[s1], key)
            value = value[:s1 + 1] + [v[idx] for v in value[s1 + 1:]]
            lw = np.zeros(n, np.float32)
    assert np.array_equal(parts.value[..., 0].cpu().numpy(), np.stack(value))


def test_backward_and_smoothers_bracket_truth(cuda):
    """the reference's checks (tests/test_ssm.py _test_ffbsi_full, _test_online_smoothing_*_full):
    backward samples bracket every simulated state; for the fixed-lag smoothers (lag 3,
    keys split(PRNGKey(0), 20)) the truth lies outside the particle range at under 10% of times"""
    import mocat_gb300 as mg
    ssm = mg.ssm.NonLinear1DBenchmark()
    t = np.arange(20, dtype=np.float32)
    sim = ssm.simulate(t, mg.random.PRNGKey(0))
    x = sim.x[:, 0]
    pf = mg.ssm.run_particle_filter_for_marginals(ssm, mg.ssm.BootstrapFilter(), sim.y, t, mg.random.PRNGKey(0),
                                                  n=10000)
    bs = mg.ssm.backward_simulation(ssm, pf, mg.random.PRNGKey(0), 2000)
    assert not hasattr(bs, "log_weight")
    assert bool((x < bs.value.max(dim=1).values[:, 0]).all())
    assert bool((bs.value.min(dim=1).values[:, 0] < x).all())
    rkeys = mg.random.split(mg.random.PRNGKey(0), 20)
    for backward_sim in (False, True):
        bf = mg.ssm.BootstrapFilter()
        parts = mg.ssm.initiate_particles(ssm, bf, 2000, rkeys[0], sim.y[0], t=float(t[0]))
        for s in range(1, 20):
            parts = mg.ssm.propagate_particle_smoother(ssm, bf, parts, sim.y[s], float(t[s]), rkeys[s], 3,
                                                       backward_sim=backward_sim)
        assert parts.value.shape == (20, 2000, 1)
        assert bool(torch.isfinite(parts.value).all())
        assert float((x > parts.value.max(dim=1).values[:, 0]).float().mean()) < 0.1
        assert float((x < parts.value.min(dim=1).values[:, 0]).float().mean()) < 0.1


@pytest.mark.parametrize("thr", [0.5, 2.0, 0.0])
def test_persistent_equals_launch_per_step(cuda, thr):
    """the persistent whole-filter kernel (k_pf_persist<NLModelP>) and the launch-per-step
    path give identical particles, log-weights and decisions; both equal the oracle"""
    mg, ssm, p, t, y, _ = _setup(8, T=25)
    n = 1 << 16
    key = O.PRNGKey(21)
    a = mg.ssm.run_particle_filter_for_marginals(ssm, mg.ssm.BootstrapFilter(), y, t, key, n=n, ess_threshold=thr)
    b = mg.ssm.run_particle_filter_for_marginals(ssm, mg.ssm.BootstrapFilter(), y, t, key, n=n, ess_threshold=thr,
                                                 persistent=False)
    ref = O.nl_run(p, n, key, y, t, ess_threshold=thr, scheme="systematic", history=True)
    for o in (a, b):
        assert np.array_equal(o.resampled.cpu().numpy(), ref["resampled"])
        assert np.array_equal(o.value[..., 0].cpu().numpy(), ref["value"])
        assert np.array_equal(o.log_weight.cpu().numpy(), ref["log_weight"])
        np.testing.assert_allclose(float(o.log_z), ref["log_z"], rtol=1e-6)
    np.testing.assert_allclose(a.ess.cpu().numpy(), b.ess.cpu().numpy(), rtol=1e-5)
