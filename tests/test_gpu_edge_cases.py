"""Edge cases of the whole-filter runs against the oracle: tiny and ragged sizes,
non-finite observations (NaN and all-minus-infinity weights, which also disable
resampling since the ESS is NaN), and the persistent kernel's size limit
(n = 2^21 on the single-launch path, n = 2^21 + 2 on the launch-per-step path).
Particles and log-weights are compared bit for bit, NaN positions included."""
import numpy as np
import pytest

import oracle as O
from oracle import models

pytestmark = pytest.mark.gpu


def _lg(d):
    import mocat_gb300 as mg
    F = models.random_stable_matrix(d, 3)
    Q, H, R = 0.2 * np.eye(d), np.eye(d), 0.5 * np.eye(d)
    p = models.lg_params(np.zeros(d), np.eye(d), F, Q, H, R)
    return p, mg.ssm.TimeHomogenousLinearGaussian(np.zeros(d), np.eye(d), F, Q, H, R)


def _check(out, ref, exact_logz=False):
    assert np.array_equal(out.resampled.cpu().numpy(), ref["resampled"])
    assert np.array_equal(out.value.cpu().numpy(), ref["value"], equal_nan=True)
    assert np.array_equal(out.log_weight.cpu().numpy(), ref["log_weight"], equal_nan=True)
    lz, rz = float(out.log_z), float(ref["log_z"])
    if np.isfinite(rz):
        np.testing.assert_allclose(lz, rz, rtol=1e-5)
    else:
        assert (np.isnan(lz) and np.isnan(rz)) or lz == rz


@pytest.mark.parametrize("n", [1, 2, 3])
@pytest.mark.parametrize("T", [1, 2, 5])
def test_tiny_sizes_lg(cuda, n, T):
    import mocat_gb300 as mg
    p, ssm = _lg(2)
    _, y = models.simulate_lg(p, T, O.PRNGKey(1))
    for pers in (True, False):
        out = mg.ssm.run_particle_filter_for_marginals(ssm, mg.ssm.BootstrapFilter(), y, np.arange(T), O.PRNGKey(2),
                                                       n=n, ess_threshold=0.9, persistent=pers)
        ref = O.lg_run(p, n, O.PRNGKey(2), y, ess_threshold=0.9, history=True)
        _check(out, ref)


@pytest.mark.parametrize("n", [1, 2, 3])
@pytest.mark.parametrize("T", [1, 4])
def test_tiny_sizes_nl1d(cuda, n, T):
    import mocat_gb300 as mg
    ssm = mg.ssm.NonLinear1DBenchmark()
    p, _ = ssm.derived()
    t = np.arange(T, dtype=np.float32)
    y = (np.arange(T) * 0.7 + 1.0).astype(np.float32)
    for pers in (True, False):
        out = mg.ssm.run_particle_filter_for_marginals(ssm, mg.ssm.BootstrapFilter(), y, t, O.PRNGKey(3), n=n,
                                                       ess_threshold=0.9, persistent=pers)
        ref = O.nl_run(p, n, O.PRNGKey(3), y, t, ess_threshold=0.9, history=True)
        assert np.array_equal(out.value[..., 0].cpu().numpy(), ref["value"], equal_nan=True)
        assert np.array_equal(out.log_weight.cpu().numpy(), ref["log_weight"], equal_nan=True)
        assert np.array_equal(out.resampled.cpu().numpy(), ref["resampled"])


@pytest.mark.parametrize("kind", ["nan", "overflow"])
@pytest.mark.parametrize("persistent", [True, False])
def test_nonfinite_observations(cuda, kind, persistent):
    """a NaN observation makes every later log-weight NaN; a huge one makes every weight
    zero (log-weight -inf); either way the ESS is NaN, resampling stops, nothing faults,
    and the particles still equal the oracle's"""
    import mocat_gb300 as mg
    p, ssm = _lg(3)
    T, n = 8, 4096
    _, y = models.simulate_lg(p, T, O.PRNGKey(4))
    y = y.copy()
    y[3] = np.nan if kind == "nan" else 1e30
    out = mg.ssm.run_particle_filter_for_marginals(ssm, mg.ssm.BootstrapFilter(), y, np.arange(T), O.PRNGKey(5),
                                                   n=n, ess_threshold=0.5, persistent=persistent)
    ref = O.lg_run(p, n, O.PRNGKey(5), y, ess_threshold=0.5, history=True)
    _check(out, ref)
    assert not np.isfinite(float(out.log_z))
    assert not ref["resampled"][4:].any()


@pytest.mark.parametrize("n", [1 << 21, (1 << 21) + 2])
def test_persistent_size_limit(cuda, n):
    """the largest n of the single-launch path and the first n past it (launch per step)"""
    import mocat_gb300 as mg
    p, ssm = _lg(4)
    T = 3
    _, y = models.simulate_lg(p, T, O.PRNGKey(6))
    out = mg.ssm.run_particle_filter_for_marginals(ssm, mg.ssm.BootstrapFilter(), y, np.arange(T), O.PRNGKey(7),
                                                   n=n, ess_threshold=1.5, history=False)
    ref = O.lg_run(p, n, O.PRNGKey(7), y, ess_threshold=1.5, history=True)
    assert np.array_equal(out.resampled.cpu().numpy(), ref["resampled"])
    assert ref["resampled"][1:].all()
    assert np.array_equal(out.value[0].cpu().numpy(), ref["value"][-1])
    assert np.array_equal(out.log_weight[0].cpu().numpy(), ref["log_weight"][-1])
    np.testing.assert_allclose(float(out.log_z), ref["log_z"], rtol=1e-6)
