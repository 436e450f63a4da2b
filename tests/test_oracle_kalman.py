"""Kalman oracle (oracle.kalman.filter_marginals / smoother_marginals, restating
mocat/src/ssm/linear_gaussian/kalman.py:16-104) pinned against brute-force conditioning
of the joint Gaussian of (x_{0:T-1}, y_{0:T-1}), and against oracle.kalman.loglik."""
import numpy as np
import pytest

from oracle import kalman as K


def _model(d, dy, seed, diag_S0=True):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((d, d))
    F = 0.8 * A / np.abs(np.linalg.eigvals(A)).max()
    B = rng.standard_normal((d, d))
    Q = B @ B.T / d + 0.3 * np.eye(d)
    H = rng.standard_normal((dy, d))
    C = rng.standard_normal((dy, dy))
    R = C @ C.T / dy + 0.2 * np.eye(dy)
    S0 = np.diag(rng.uniform(0.5, 2.0, d)) if diag_S0 else (lambda M: M @ M.T + np.eye(d))(rng.standard_normal((d, d)))
    return F, Q, H, R, rng.standard_normal(d), S0


def _joint(F, Q, H, R, m0, P0, T):
    """mean and covariance of (x_0..x_{T-1}, y_0..y_{T-1}) with Var(x_0) = P0"""
    d, dy = F.shape[0], H.shape[0]
    mx = [m0]
    V = [P0]
    for t in range(1, T):
        mx.append(F @ mx[-1])
        V.append(F @ V[-1] @ F.T + Q)
    Cx = np.zeros((T * d, T * d))
    for s in range(T):
        for t in range(s, T):
            c = np.linalg.matrix_power(F, t - s) @ V[s]  # Cov(x_t, x_s)
            Cx[t * d:(t + 1) * d, s * d:(s + 1) * d] = c
            Cx[s * d:(s + 1) * d, t * d:(t + 1) * d] = c.T
    Hb = np.kron(np.eye(T), H)
    mean = np.concatenate([np.concatenate(mx), Hb @ np.concatenate(mx)])
    cov = np.block([[Cx, Cx @ Hb.T], [Hb @ Cx, Hb @ Cx @ Hb.T + np.kron(np.eye(T), R)]])
    return mean, cov


def _condition(mean, cov, nx, y, upto, dy):
    """mean and covariance of x given y_0..y_{upto}"""
    idx = np.arange(nx, nx + (upto + 1) * dy)
    Sxy = cov[:nx, idx]
    Syy = cov[np.ix_(idx, idx)]
    G = Sxy @ np.linalg.inv(Syy)
    return mean[:nx] + G @ (y[:upto + 1].ravel() - mean[idx]), cov[:nx, :nx] - G @ Sxy.T


@pytest.mark.parametrize("d,dy", [(1, 1), (2, 1), (3, 2)])
def test_filter_and_smoother_equal_joint_conditioning(d, dy):
    """with a diagonal initial covariance S0 the reference's t = 0 covariance is its square
    root diag(sqrt(S0)); the marginals are those of the joint Gaussian with that prior"""
    F, Q, H, R, m0, S0 = _model(d, dy, 10 * d + dy)
    T = 5
    C0 = np.linalg.cholesky(S0)
    y = np.random.default_rng(1).standard_normal((T, dy))
    fm, fc, _ = K.filter_marginals(F, Q, H, R, m0, C0, y)
    mean, cov = _joint(F, Q, H, R, m0, C0, T)
    for t in range(T):
        mu, P = _condition(mean, cov, T * d, y, t, dy)
        np.testing.assert_allclose(fm[t], mu[t * d:(t + 1) * d], atol=1e-10)
        np.testing.assert_allclose(fc[t], P[t * d:(t + 1) * d, t * d:(t + 1) * d], atol=1e-10)
    sm, sc, lag = K.smoother_marginals(F, Q, fm, fc, lag_ones=True)
    mu, P = _condition(mean, cov, T * d, y, T - 1, dy)
    for t in range(T):
        np.testing.assert_allclose(sm[t], mu[t * d:(t + 1) * d], atol=1e-10)
        np.testing.assert_allclose(sc[t], P[t * d:(t + 1) * d, t * d:(t + 1) * d], atol=1e-10)
    if d == 1:
        # kalman.py:83 forms the lag-one term with the FILTERED mean at t+1 where the exact
        # E[x_t x_{t+1} | y] = G P^s_{t+1} + mu^s_t mu^s_{t+1} has the predicted mean F mu^f_t:
        # the difference is G (F mu^f_t - mu^f_{t+1}) mu^s_{t+1}, reproduced as written
        for t in range(T - 1):
            exact = P[t, t + 1] + mu[t] * mu[t + 1]
            G = fc[t, 0, 0] * F[0, 0] / (F[0, 0] ** 2 * fc[t, 0, 0] + Q[0, 0])
            quirk = G * (F[0, 0] * fm[t, 0] - fm[t + 1, 0]) * sm[t + 1, 0]
            np.testing.assert_allclose(lag[t, 0, 0], exact + quirk, atol=1e-10)


def test_filter_loglik_equals_prediction_error_loglik():
    """with S0 = I (square root = covariance) the log-likelihood is oracle.kalman.loglik's,
    and that equals log N(y; joint mean, joint covariance)"""
    F, Q, H, R, m0, _ = _model(3, 2, 4)
    T = 6
    y = np.random.default_rng(2).standard_normal((T, 2))
    _, _, ll = K.filter_marginals(F, Q, H, R, m0, np.eye(3), y)
    np.testing.assert_allclose(ll, K.loglik(F, Q, H, R, m0, np.eye(3), y), rtol=1e-12)
    mean, cov = _joint(F, Q, H, R, m0, np.eye(3), T)
    Syy, e = cov[T * 3:, T * 3:], y.ravel() - mean[T * 3:]
    direct = -0.5 * (e.size * np.log(2 * np.pi) + np.linalg.slogdet(Syy)[1] + e @ np.linalg.solve(Syy, e))
    np.testing.assert_allclose(ll, direct, rtol=1e-10)
