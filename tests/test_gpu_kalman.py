"""GPU Kalman filter and RTS smoother (mocat_gb300.ssm.run_kalman_filter_for_marginals,
run_kalman_smoother_for_marginals[_and_lag_ones]; mocat/src/ssm/linear_gaussian/kalman.py:16-104)
against the float64 oracle (oracle.kalman.filter_marginals / smoother_marginals), and the
reference's own checks (tests/test_ssm_linear_gaussian.py, TestKalman1D / TestKalman5D: the
simulated states lie within 3 (1-D) or 4 (5-D) marginal sds of the filter and smoother means).

The device path computes in float32 like the reference; the comparison against float64 is
relative to the scale of each output: |gpu - oracle| <= 2e-3 (1 + |oracle|) elementwise, and
the prediction-error log-likelihood to rtol 1e-4."""
import numpy as np
import pytest

import oracle as O
from oracle import kalman as K
from oracle import models

pytestmark = pytest.mark.gpu

TOL = 2e-3


def _spd(rng, d, scale):
    A = rng.standard_normal((d, d))
    return scale * (A @ A.T / d + 0.5 * np.eye(d))


def _model(d, dy, seed):
    import mocat_gb300 as mg
    rng = np.random.default_rng(seed)
    F = models.random_stable_matrix(d, seed)
    Q, S0, R = _spd(rng, d, 0.3), _spd(rng, d, 1.0), _spd(rng, dy, 0.5)
    H = rng.standard_normal((dy, d)) / np.sqrt(d)
    m0 = rng.standard_normal(d)
    ssm = mg.ssm.TimeHomogenousLinearGaussian(m0, S0, F, Q, H, R)
    return ssm, dict(F=F, Q=Q, H=H, R=R, m0=m0, C0=np.linalg.cholesky(S0))


def _close(gpu, ref, tol=TOL):
    g = gpu.double().cpu().numpy() if hasattr(gpu, "cpu") else np.asarray(gpu, np.float64)
    assert g.shape == ref.shape
    if g.size == 0:
        return
    err = np.abs(g - ref) / (1.0 + np.abs(ref))
    assert err.max() <= tol, err.max()


def _observations(ssm, T, seed):
    p, _ = ssm.derived()
    _, y = models.simulate_lg(p, T, O.PRNGKey(seed))
    return y


@pytest.mark.parametrize("d,dy", [(1, 1), (3, 1), (3, 3), (5, 5), (10, 1), (10, 10),
                                  (6, 6), (7, 3), (2, 4), (12, 12), (32, 5)])
def test_filter_and_smoother_match_oracle(cuda, d, dy):
    """compiled pairs and, for (6, 6), (7, 3), (2, 4), (12, 12), (32, 5), the run-time-dimension
    instance of the same kernels"""
    import mocat_gb300 as mg
    ssm, m = _model(d, dy, 10 * d + dy)
    T = 60
    y = _observations(ssm, T, d)
    fm, fc, ll = mg.ssm.run_kalman_filter_for_marginals(ssm, y, np.arange(T), return_log_likelihood=True)
    rm, rc, rll = K.filter_marginals(m["F"], m["Q"], m["H"], m["R"], m["m0"], m["C0"], y)
    _close(fm, rm)
    _close(fc, rc)
    np.testing.assert_allclose(float(ll), rll, rtol=1e-4)
    sm, sc, lag = mg.ssm.run_kalman_smoother_for_marginals_and_lag_ones(ssm, y, np.arange(T), (fm, fc))
    # the smoother's float64 oracle runs on the GPU's float32 filter output, so that each
    # kernel is checked on its own inputs
    rsm, rsc, rlag = K.smoother_marginals(m["F"], m["Q"], fm.double().cpu().numpy(), fc.double().cpu().numpy(),
                                          lag_ones=True)
    _close(sm, rsm)
    _close(sc, rsc)
    _close(lag, rlag)
    sm2, sc2 = mg.ssm.run_kalman_smoother_for_marginals(ssm, y, np.arange(T))
    assert np.array_equal(sm2.cpu().numpy(), sm.cpu().numpy())
    assert np.array_equal(sc2.cpu().numpy(), sc.cpu().numpy())
    # last step: smoothed = filtered
    assert np.array_equal(sm[-1].cpu().numpy(), fm[-1].cpu().numpy())


def test_batched_equals_single(cuda):
    """B observation sequences in one launch give bit for bit the single-sequence outputs"""
    import mocat_gb300 as mg
    ssm, _ = _model(4, 4, 1)
    T, B = 33, 5
    ys = np.stack([_observations(ssm, T, 100 + b) for b in range(B)])
    fm, fc, ll = mg.ssm.run_kalman_filter_for_marginals(ssm, ys, return_log_likelihood=True)
    sm, sc, lag = mg.ssm.run_kalman_smoother_for_marginals_and_lag_ones(ssm, ys, filter_output=(fm, fc))
    assert fm.shape == (B, T, 4) and fc.shape == (B, T, 4, 4) and ll.shape == (B,) and lag.shape == (B, T - 1, 4, 4)
    for b in range(B):
        f1, c1, l1 = mg.ssm.run_kalman_filter_for_marginals(ssm, ys[b], return_log_likelihood=True)
        s1, q1, g1 = mg.ssm.run_kalman_smoother_for_marginals_and_lag_ones(ssm, ys[b])
        for a, c in ((fm[b], f1), (fc[b], c1), (sm[b], s1), (sc[b], q1), (lag[b], g1)):
            assert np.array_equal(a.cpu().numpy(), c.cpu().numpy())
        assert float(ll[b]) == float(l1)


@pytest.mark.parametrize("T", [1, 2])
def test_short_sequences(cuda, T):
    import mocat_gb300 as mg
    ssm, m = _model(2, 1, 7)
    y = _observations(ssm, T, 3)
    fm, fc = mg.ssm.run_kalman_filter_for_marginals(ssm, y)
    rm, rc, _ = K.filter_marginals(m["F"], m["Q"], m["H"], m["R"], m["m0"], m["C0"], y)
    _close(fm, rm)
    _close(fc, rc)
    sm, sc, lag = mg.ssm.run_kalman_smoother_for_marginals_and_lag_ones(ssm, y, filter_output=(fm, fc))
    assert lag.shape == (T - 1, 2, 2)
    rsm, rsc, rlag = K.smoother_marginals(m["F"], m["Q"], fm.double().cpu().numpy(), fc.double().cpu().numpy(),
                                          lag_ones=True)
    _close(sm, rsm)
    _close(sc, rsc)
    _close(lag, rlag)


@pytest.mark.parametrize("dim,sds", [(1, 3), (5, 4)])
def test_reference_interval_check(cuda, dim, sds):
    """TestKalman1D / TestKalman5D: identity model, t = 0..19, simulated with PRNGKey(0)"""
    import mocat_gb300 as mg
    e = np.eye(dim)
    ssm = mg.ssm.TimeHomogenousLinearGaussian(np.zeros(dim), e, e, e, e, e)
    t = np.arange(20)
    sim = ssm.simulate(t, mg.random.PRNGKey(0))
    x = sim.x.cpu().numpy()
    for means, covs in (mg.ssm.run_kalman_filter_for_marginals(ssm, sim.y, t),
                        mg.ssm.run_kalman_smoother_for_marginals(ssm, sim.y, t)):
        mu = means.cpu().numpy()
        sd = np.sqrt(np.diagonal(covs.cpu().numpy(), axis1=-2, axis2=-1))
        assert (x < mu + sds * sd).all() and (mu - sds * sd < x).all()


def test_unsupported_model_raises(cuda):
    """above the run-time-dimension limit (d or dy > 32) the Kalman filter is refused on the host"""
    import mocat_gb300 as mg
    e = np.eye(33)
    ssm = mg.ssm.TimeHomogenousLinearGaussian(np.zeros(33), e, e, e, e, e)
    with pytest.raises(NotImplementedError):
        mg.ssm.run_kalman_filter_for_marginals(ssm, np.zeros((4, 33), np.float32))
