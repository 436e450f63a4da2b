"""User-defined models and filters (the reference's plugin contract,
mocat/src/ssm/ssm.py:18-81 and filtering.py:20-139) through the generic GPU
driver: the plugin's vectorised methods propagate and weight, the library's
kernels split the keys, normalise, resample and gather.

A user model that restates the one-dimensional linear-Gaussian model in torch
(every operation a single rounding, as the oracle's d = 1 arithmetic) must give
the oracle's filter bit for bit: particles, log-weights, resampling decisions;
log Z within 1e-6.  The same model through initiate_particles /
propagate_particle_filter equals the fused kernels step for step.  A user
filter that overrides the vectorised proposal, on a model with a non-linear
transition, is checked against a float64 restatement of its weights and of
the reference's log Z recurrence.
"""
import numpy as np
import pytest
import torch

import oracle as O
from oracle import models

pytestmark = pytest.mark.gpu


def _user_lg1d(F, Q, H, R, m0, S0):
    """the user's model: the reference's TimeHomogenousLinearGaussian for d = 1, in torch"""
    import mocat_gb300 as mg
    one = np.eye(1)
    p = models.lg_params(np.full(1, m0), S0 * one, F * one, Q * one, H * one, R * one)
    f32 = np.float32

    class UserLG1D(mg.ssm.StateSpaceModel):
        dim, dim_obs = 1, 1

        def initial_sample(self, t, random_keys):
            e = mg.random.normal_keys(random_keys, 1)
            return e * f32(p["C0"][0, 0]) + f32(p["m0"][0])

        def transition_sample(self, x_previous, t_previous, t_new, random_keys):
            e = mg.random.normal_keys(random_keys, 1)
            return x_previous * f32(p["F"][0, 0]) + e * f32(p["Lq"][0, 0])

        def likelihood_potential(self, x, y, t):
            diff = y[0] - x[:, 0] * f32(p["H"][0, 0])
            v = diff * f32(p["P"][0, 0])
            return (v * v) * f32(0.5) + f32(p["c"])

    return UserLG1D(), p


@pytest.mark.parametrize("scheme", ["systematic", "multinomial"])
@pytest.mark.parametrize("n,T,thr", [(1000, 100, 0.5), (777, 60, 2.0), (4096, 40, 0.3)])
def test_user_model_equals_oracle_filter(cuda, scheme, n, T, thr):
    import mocat_gb300 as mg
    user, p = _user_lg1d(0.9, 1.0, 1.0, 0.25, 0.0, 1.0)
    _, y = models.simulate_lg(p, T, O.PRNGKey(0))
    key = O.PRNGKey(3)
    assert not mg.ssm._fused(user, mg.ssm.BootstrapFilter())
    out = mg.ssm.run_particle_filter_for_marginals(user, mg.ssm.BootstrapFilter(), y, np.arange(T), key, n=n,
                                                   ess_threshold=thr, resampling=scheme)
    ref = O.lg_run(p, n, key, y, thr, scheme, history=True)
    assert np.array_equal(out.resampled.cpu().numpy(), ref["resampled"])
    assert np.array_equal(out.value.cpu().numpy(), ref["value"])
    assert np.array_equal(out.log_weight.cpu().numpy(), ref["log_weight"])
    np.testing.assert_allclose(float(out.log_z), ref["log_z"], rtol=1e-6)
    np.testing.assert_allclose(out.ess.cpu().numpy(), ref["ess"], rtol=1e-5)


def test_user_model_online_steps_equal_the_fused_kernels(cuda):
    """initiate_particles + propagate_particle_filter with a user model follow the fused
    kernels' arithmetic (the reference's online path, filtering.py:173-252)"""
    import mocat_gb300 as mg
    user, p = _user_lg1d(0.8, 0.5, 1.0, 0.3, 0.1, 2.0)
    T, n = 12, 512
    _, y = models.simulate_lg(p, T, O.PRNGKey(1))
    pf = mg.ssm.BootstrapFilter()
    lg = mg.ssm.TimeHomogenousLinearGaussian(0.1 * np.ones(1), 2.0 * np.eye(1), 0.8 * np.eye(1), 0.5 * np.eye(1),
                                             np.eye(1), 0.3 * np.eye(1))
    a = mg.ssm.initiate_particles(user, pf, n, O.PRNGKey(5), y[0], 0.0)
    b = mg.ssm.initiate_particles(lg, pf, n, O.PRNGKey(5), y[0], 0.0)  # fused kernel
    assert torch.equal(a.value, b.value) and torch.equal(a.log_weight, b.log_weight)
    keys = mg.random.split(mg.random.PRNGKey(9), T)
    for t in range(1, T):
        a = mg.ssm.propagate_particle_filter(user, pf, a, y[t], float(t), keys[t], ess_threshold=0.5)
        b = mg.ssm.propagate_particle_filter(lg, pf, b, y[t], float(t), keys[t], ess_threshold=0.5)
    assert a.value.shape == (T, n, 1) and a.log_weight.shape == (T, n)
    assert torch.equal(a.value, b.value) and torch.equal(a.log_weight, b.log_weight)


def test_user_filter_and_nonlinear_model(cuda):
    """a user filter overriding the vectorised proposal (tempered likelihood weights) on a
    user model with a non-linear transition"""
    import mocat_gb300 as mg

    class NL(mg.ssm.StateSpaceModel):
        dim, dim_obs = 2, 1

        def initial_sample(self, t, random_keys):
            return mg.random.normal_keys(random_keys, 2)

        def transition_sample(self, x_previous, t_previous, t_new, random_keys):
            e = mg.random.normal_keys(random_keys, 2)
            return torch.stack([torch.sin(x_previous[:, 1]) + 0.3 * e[:, 0], 0.9 * x_previous[:, 0] + 0.3 * e[:, 1]], 1)

        def likelihood_potential(self, x, y, t):
            return 0.5 * ((y[0] - x[:, 0] * x[:, 1]) / 0.5) ** 2

    class Tempered(mg.ssm.ParticleFilter):
        def propose_and_intermediate_weight_vectorised(self, ssm_scenario, x_previous, t_previous, y_new, t_new,
                                                       random_keys):
            x_new = ssm_scenario.transition_sample(x_previous, t_previous, t_new, random_keys)
            return x_new, -0.5 * ssm_scenario.likelihood_potential(x_new, y_new, t_new)

    T, n = 30, 2048
    y = np.sin(np.arange(T, dtype=np.float32))[:, None]
    out = mg.ssm.run_particle_filter_for_marginals(NL(), Tempered(), y, np.arange(T), O.PRNGKey(4), n=n,
                                                   ess_threshold=0.5)
    x = out.value.double().cpu().numpy()
    lw = out.log_weight.double().cpu().numpy()
    res = out.resampled.cpu().numpy()
    assert res[1:].sum() > 0 and np.isfinite(float(out.log_z))
    for t in range(1, T):
        pot = 0.5 * ((y[t, 0] - x[t, :, 0] * x[t, :, 1]) / 0.5) ** 2
        carried = 0.0 if res[t] else lw[t - 1]
        np.testing.assert_allclose(lw[t], carried - 0.5 * pot, rtol=2e-5, atol=2e-5)
    lz, prev = 0.0, None
    for t in range(T):
        m = lw[t].max()
        lse = m + np.log(np.exp(lw[t] - m).sum())
        lz += lse - (np.log(n) if (t == 0 or res[t]) else prev)
        prev = lse
    np.testing.assert_allclose(float(out.log_z), lz, rtol=1e-6)
