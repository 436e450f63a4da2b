"""GPU tempered SMC (MALA moves, adaptive temperatures) on logistic regression
vs the float64 restatement in oracle/smc.py fed the same jax.random draws.

The GPU evaluates potentials in float32, so an accept decision can flip where
the uniform lands within ~1e-6 of alpha; on these seeds none does, and the
test demands: the same number of iterations and resampling steps, temperatures
within 1e-4 relative, mean acceptance within 1e-4, log_norm_constant within
1e-4 relative, final particles within 1e-3.  The fp32 potential kernel itself
matches float64 within 1e-5 relative.  A statistical check against the exact
d = 2 log evidence (quadrature) covers the batched form at larger n.
"""
import numpy as np
import pytest
import torch

import oracle as O
from oracle import smc as osmc

pytestmark = pytest.mark.gpu


def _data(n, d, seed=0):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, d)).astype(np.float32)
    bt = rng.standard_normal(d)
    y = (rng.random(n) < 1 / (1 + np.exp(-X @ bt))).astype(np.float32)
    return X, y


@pytest.mark.parametrize("d", [2, 5, 50])
def test_potential_fp32_matches_float64(cuda, d):
    import mocat_gb300 as mg
    X, y = _data(3000, d)
    sc = mg.smc.LogisticRegression(X, y)
    beta = (np.random.default_rng(3).standard_normal((700, d)) * 0.3).astype(np.float32)
    lik, grad = sc.likelihood_potential_and_grad(torch.from_numpy(beta).cuda())
    ol, og = osmc.potential_grad(X, y, beta.astype(np.float64))
    np.testing.assert_allclose(lik.cpu().numpy(), ol, rtol=1e-5)
    np.testing.assert_allclose(grad.cpu().numpy(), og, rtol=1e-4, atol=1e-3)


@pytest.mark.parametrize("d,N,seed", [(2, 64, 0), (5, 128, 1), (3, 96, 2)])
def test_sampler_matches_restatement(cuda, d, N, seed):
    import mocat_gb300 as mg
    X, y = _data(200, d, seed)
    sc = mg.smc.LogisticRegression(X, y, prior_scale=1.0)
    sampler = mg.smc.MetropolisedSMCSampler(mg.smc.Underdamped(stepsize=0.15), mcmc_steps=3,
                                            ess_threshold_retain=0.6)
    keys = np.stack([O.PRNGKey(10 + seed), O.PRNGKey(20 + seed)])
    out = mg.smc.run_batched(sc, sampler, N, keys)
    for b in range(2):
        ref = osmc.run(X, y, 1.0, N, keys[b], stepsize=0.15, mcmc_steps=3, retain=0.6)
        L = int(out.iterations[b]) + 1
        assert L == len(ref["temperature"]), (L, len(ref["temperature"]))
        np.testing.assert_allclose(out.temperature[b, :L].cpu().numpy(), ref["temperature"], rtol=1e-4)
        assert np.array_equal(out.resampled[b, :L].cpu().numpy(), ref["resampled"])
        np.testing.assert_allclose(out.alpha[b, :L].cpu().numpy(), ref["alpha"], rtol=1e-4, atol=1e-5)
        np.testing.assert_allclose(out.log_norm_constant[b, :L].cpu().numpy(), ref["log_norm_constant"], rtol=1e-4)
        np.testing.assert_allclose(out.value[b].cpu().numpy(), ref["value"], atol=1e-3)


@pytest.mark.parametrize("N", [96, 95])  # even N: one cipher call per two outputs' draws
def test_categorical_resampling_matches_restatement(cuda, N):
    """resampling="categorical": the reference's random.categorical ancestors (O(N^2)
    Gumbel-max draws from the resampling key), against the restatement with the same draws"""
    import mocat_gb300 as mg
    d = 3
    X, y = _data(200, d, 5)
    sc = mg.smc.LogisticRegression(X, y, prior_scale=1.0)
    sampler = mg.smc.MetropolisedSMCSampler(mg.smc.Underdamped(stepsize=0.15), mcmc_steps=3,
                                            ess_threshold_retain=0.6, resampling="categorical")
    keys = np.stack([O.PRNGKey(41), O.PRNGKey(42)])
    out = mg.smc.run_batched(sc, sampler, N, keys)
    for b in range(2):
        ref = osmc.run(X, y, 1.0, N, keys[b], stepsize=0.15, mcmc_steps=3, retain=0.6, resampling="categorical")
        L = int(out.iterations[b]) + 1
        assert L == len(ref["temperature"]) and sum(ref["resampled"]) >= 2
        np.testing.assert_allclose(out.temperature[b, :L].cpu().numpy(), ref["temperature"], rtol=1e-4)
        assert np.array_equal(out.resampled[b, :L].cpu().numpy(), ref["resampled"])
        np.testing.assert_allclose(out.log_norm_constant[b, :L].cpu().numpy(), ref["log_norm_constant"], rtol=1e-4)
        np.testing.assert_allclose(out.value[b].cpu().numpy(), ref["value"], atol=1e-3)
    # and a different chain from the systematic default on the same keys
    sys_out = mg.smc.run_batched(sc, mg.smc.MetropolisedSMCSampler(mg.smc.Underdamped(stepsize=0.15), mcmc_steps=3,
                                                                   ess_threshold_retain=0.6), N, keys)
    assert not torch.equal(sys_out.value, out.value)


def test_batched_log_evidence_matches_quadrature(cuda):
    import mocat_gb300 as mg
    X, y = _data(100, 2)
    exact = osmc.log_evidence_2d(X, y, 1.0)
    sc = mg.smc.LogisticRegression(X, y)
    sampler = mg.smc.MetropolisedSMCSampler(mg.smc.Underdamped(stepsize=0.2), mcmc_steps=5,
                                            ess_threshold_retain=0.5)
    keys = np.stack([O.PRNGKey(s) for s in range(32)])
    out = mg.smc.run_batched(sc, sampler, 2048, keys)
    z = np.array([float(out.log_norm_constant[b, int(out.iterations[b])]) for b in range(32)])
    se = z.std() / np.sqrt(len(z))
    assert abs(z.mean() - exact) < 4 * se + 0.01, (z.mean(), exact, se)
    assert (out.temperature.max(1).values >= 1.0).all()


def test_single_posterior_run(cuda):
    import mocat_gb300 as mg
    X, y = _data(500, 5)
    sc = mg.smc.LogisticRegression(X, y)
    sampler = mg.smc.MetropolisedSMCSampler(mg.smc.Underdamped(stepsize=0.05), mcmc_steps=2)
    out = mg.smc.run(sc, sampler, 512, O.PRNGKey(7))
    assert float(out.temperature[-1]) == 1.0
    L = out.temperature.shape[0]
    assert out.value.shape == (L, 512, 5) and out.log_weight.shape == (L, 512)
    assert np.isfinite(out.log_norm_constant.cpu().numpy()).all()


@pytest.mark.parametrize("d,n_data,P", [(5, 1000, 256), (50, 3000, 700), (50, 20000, 4096), (2, 333, 130)])
def test_potential_bf16_tensor_cores(cuda, d, n_data, P):
    """tcgen05 path (bf16 X and beta, fp32 accumulation) against the fp32 kernel: the
    potential within 1e-2 relative plus bf16 rounding of the linear predictors,
    the gradient rows within 3e-2 (relative 2-norm)."""
    import mocat_gb300 as mg
    X, y = _data(n_data, d, seed=d)
    sc = mg.smc.LogisticRegression(X, y)
    beta = (np.random.default_rng(5).standard_normal((P, d)) * 0.3).astype(np.float32)
    bt = torch.from_numpy(beta).cuda()
    l32, g32 = sc.likelihood_potential_and_grad(bt, precision="fp32")
    l16, g16 = sc.likelihood_potential_and_grad(bt, precision="bf16")
    l32, g32, l16, g16 = (t.double().cpu().numpy() for t in (l32, g32, l16, g16))
    assert np.isfinite(l16).all() and np.isfinite(g16).all()
    rel = np.abs(l16 - l32) / np.abs(l32)
    assert rel.max() < 1e-2, rel.max()
    gr = np.linalg.norm(g16 - g32, axis=1) / np.linalg.norm(g32, axis=1)
    assert np.median(gr) < 3e-2 and gr.max() < 0.1, (np.median(gr), gr.max())


def test_sampler_bf16_close_to_fp32(cuda):
    import mocat_gb300 as mg
    X, y = _data(2000, 5)
    sc = mg.smc.LogisticRegression(X, y)
    sampler = mg.smc.MetropolisedSMCSampler(mg.smc.Underdamped(stepsize=0.02), mcmc_steps=3,
                                            ess_threshold_retain=0.5)
    keys = np.stack([O.PRNGKey(s) for s in range(8)])
    z32 = mg.smc.run_batched(sc, sampler, 1024, keys, precision="fp32")
    z16 = mg.smc.run_batched(sc, sampler, 1024, keys, precision="bf16")
    a = np.array([float(z32.log_norm_constant[b, int(z32.iterations[b])]) for b in range(8)])
    c = np.array([float(z16.log_norm_constant[b, int(z16.iterations[b])]) for b in range(8)])
    assert np.isfinite(c).all()
    assert abs(a.mean() - c.mean()) < 0.5 + 4 * (a.std() + c.std()) / np.sqrt(8), (a.mean(), c.mean())


def test_prior_scale_gradient_matches_quadrature(cuda):
    """d log Z / d s from the final weighted particles against central differences
    of the exact d = 2 log evidence."""
    import mocat_gb300 as mg
    X, y = _data(100, 2)
    h = 1e-3
    exact = (osmc.log_evidence_2d(X, y, 1.0 + h) - osmc.log_evidence_2d(X, y, 1.0 - h)) / (2 * h)
    sc = mg.smc.LogisticRegression(X, y)
    sampler = mg.smc.MetropolisedSMCSampler(mg.smc.Underdamped(stepsize=0.2), mcmc_steps=5,
                                            ess_threshold_retain=0.5)
    keys = np.stack([O.PRNGKey(100 + s) for s in range(16)])
    out = mg.smc.run_batched(sc, sampler, 4096, keys)
    g = out.grad_log_norm_constant_prior_scale.cpu().numpy()
    se = g.std() / np.sqrt(len(g))
    assert abs(g.mean() - exact) < 4 * se + 0.01, (g.mean(), exact, se)


COV = np.array([[1.0, 0.9], [0.9, 2.0]])


def _general_case(name):
    """(scenario, sampler, restatement kwargs, lik_fn, d) of the generalised moves"""
    import mocat_gb300 as mg
    if name.startswith("gauss"):
        sc = mg.smc.Gaussian(covariance=COV, prior_scale=7.0)
        ps = np.linalg.inv(np.linalg.cholesky(COV))
        fn, d = (lambda b: osmc.gaussian_potential_grad(np.zeros(2), ps, b)), 2
    else:
        d = 3 if name == "logreg_hmc" else 5
        X, y = _data(150, d, 7)
        sc = mg.smc.LogisticRegression(X, y, prior_scale=1.0)
        fn = (lambda X, y: (lambda b: osmc.potential_grad(X, y, b)))(X, y)
    if name == "gauss_rw_schedule":
        sch = np.arange(0.1, 1.01, 0.15).astype(np.float32)
        smp = mg.smc.MetropolisedSMCSampler(mg.smc.RandomWalk(stepsize=1.0), mcmc_steps=2, temperature_schedule=sch)
        kw = dict(stepsize=1.0, mcmc_steps=2, move="random_walk", schedule=sch)
    elif name == "gauss_ud_friction":
        smp = mg.smc.MetropolisedSMCSampler(mg.smc.Underdamped(stepsize=0.4, leapfrog_steps=3, friction=1.0),
                                            mcmc_steps=2, ess_threshold_retain=0.6)
        kw = dict(stepsize=0.4, mcmc_steps=2, retain=0.6, leapfrog_steps=3, friction=1.0)
    elif name == "logreg_hmc":
        smp = mg.smc.MetropolisedSMCSampler(mg.smc.Underdamped(stepsize=0.1, leapfrog_steps=2), mcmc_steps=2,
                                            ess_threshold_retain=0.6)
        kw = dict(stepsize=0.1, mcmc_steps=2, retain=0.6, leapfrog_steps=2)
    else:
        smp = mg.smc.MetropolisedSMCSampler(mg.smc.RandomWalk(stepsize=0.01), mcmc_steps=3, ess_threshold_retain=0.6)
        kw = dict(stepsize=0.01, mcmc_steps=3, retain=0.6, move="random_walk")
    return sc, smp, kw, fn, d


@pytest.mark.parametrize("name", ["gauss_rw_schedule", "gauss_ud_friction", "logreg_hmc", "logreg_rw"])
def test_general_moves_match_restatement(cuda, name):
    """RandomWalk moves, Underdamped with several leapfrog steps and a finite friction (momenta
    kept and resampled with the particles), temperature schedules and the Gaussian scenario,
    against the float64 restatement with the same draws (tolerances as above)"""
    import mocat_gb300 as mg
    sc, smp, kw, fn, d = _general_case(name)
    N = 64
    keys = np.stack([O.PRNGKey(31), O.PRNGKey(32)])
    out = mg.smc.run_batched(sc, smp, N, keys)
    for b in range(2):
        ref = osmc.run_general(fn, d, sc.prior_scale, N, keys[b], **kw)
        L = int(out.iterations[b]) + 1
        assert L == len(ref["temperature"]), (L, len(ref["temperature"]))
        np.testing.assert_allclose(out.temperature[b, :L].cpu().numpy(), ref["temperature"], rtol=1e-4)
        assert np.array_equal(out.resampled[b, :L].cpu().numpy(), ref["resampled"])
        np.testing.assert_allclose(out.alpha[b, :L].cpu().numpy(), ref["alpha"], rtol=1e-4, atol=1e-5)
        np.testing.assert_allclose(out.log_norm_constant[b, :L].cpu().numpy(), ref["log_norm_constant"], rtol=1e-4,
                                   atol=1e-5)
        np.testing.assert_allclose(out.value[b].cpu().numpy(), ref["value"], atol=1e-3)
    if "schedule" in kw:
        assert np.array_equal(out.temperature[0, :L].cpu().numpy(), kw["schedule"])


@pytest.mark.parametrize("move,schedule", [("rw", True), ("ud", True), ("rw", False), ("ud10", False)])
def test_reference_transport_checks(cuda, move, schedule):
    """TestMetropolisedSMC (tests/test_transport.py:121-170): n = 1e4, the correlated Gaussian
    with prior_sample 7 N(0, I) and prior_potential 0.5 |x / 49|^2; after a categorical resample
    of the final particles (PRNGKey(1)) the mean is 0 to 0 decimals and the covariance the
    posterior's to 1 decimal; log_norm_constant equals the tempered closed form to 0 decimals;
    a preschedule comes back as the temperatures"""
    import mocat_gb300 as mg
    sc = mg.smc.Gaussian(covariance=COV, prior_scale=49.0, prior_sample_scale=7.0)
    mv = {"rw": mg.smc.RandomWalk(stepsize=1.0), "ud": mg.smc.Underdamped(stepsize=1.0),
          "ud10": mg.smc.Underdamped(stepsize=1.0, leapfrog_steps=10)}[move]
    pre = np.arange(0.0, 1.1, 0.1).astype(np.float32)
    n = 10000
    out = mg.smc.run(sc, mg.smc.MetropolisedSMCSampler(mv), n, mg.random.PRNGKey(0),
                     temperature_schedule=pre if schedule else None)
    lw = out.log_weight[-1].cpu().numpy()
    idx = O.resample_gumbel(lw, O.PRNGKey(1), n)
    x = out.value[-1].cpu().numpy()[idx].astype(np.float64)
    post = np.linalg.inv(np.linalg.inv(COV) + np.eye(2) / 49.0)
    np.testing.assert_array_almost_equal(x.mean(0), np.zeros(2), decimal=0)
    np.testing.assert_array_almost_equal(np.cov(x.T), post, decimal=1)
    temps = out.temperature.cpu().numpy().astype(np.float64)
    lik_prec = np.linalg.inv(COV)
    dets = np.array([np.linalg.det(np.linalg.inv(lik_prec * t + np.eye(2) / 49.0)) for t in temps])
    np.testing.assert_array_almost_equal(out.log_norm_constant.cpu().numpy(), 0.5 * (np.log(dets) - 4 * np.log(7.0)),
                                         0)
    if schedule:
        assert np.array_equal(out.temperature.cpu().numpy(), pre[1:])
