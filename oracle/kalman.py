"""ORACLE (test infrastructure only): float64 Kalman filter log-likelihood and its exact gradient.

The reference's ``run_kalman_filter_for_marginals``
(mocat/src/ssm/linear_gaussian/kalman.py:16-57) returns filtered means and
covariances only; the prediction-error decomposition of log p(y_{0:T-1}) and
its gradient are new, written from the standard Kalman recursions:

    m_{0|-1} = m0,  P_{0|-1} = S0
    S_t = H P_{t|t-1} H' + R,  e_t = y_t - H m_{t|t-1}
    log p += -1/2 (dy log 2pi + log|S_t| + e_t' S_t^{-1} e_t)
    K_t = P_{t|t-1} H' S_t^{-1},  m_t = m_{t|t-1} + K_t e_t,  P_t = P_{t|t-1} - K_t H P_{t|t-1}
    m_{t+1|t} = F m_t,  P_{t+1|t} = F P_t F' + Q

The gradient w.r.t. theta = (F (d x d, row-major), log diag Q (d), log diag R (dy))
propagates the tangents (dm, dP) of every parameter direction through the same
recursion (forward-mode sensitivities), vectorised over directions.
(The reference quirk of using the initial covariance *square root* as the
covariance, kalman.py:20,26-28, only matters when S0 != I; this oracle uses S0.)

filter_marginals / smoother_marginals restate the reference's marginal filter and RTS
smoother as written, that quirk included, with the lag-one terms of kalman.py:60-94.
"""
import numpy as np

LOG2PI = np.log(2.0 * np.pi)


def loglik(F, Q, H, R, m0, S0, y):
    F, Q, H, R, m0, S0 = (np.asarray(a, np.float64) for a in (F, Q, H, R, m0, S0))
    y = np.asarray(y, np.float64).reshape(len(y), -1)
    m, P = m0.copy(), S0.copy()
    ll = 0.0
    dy = H.shape[0]
    for t in range(y.shape[0]):
        if t > 0:
            m = F @ m
            P = F @ P @ F.T + Q
        S = H @ P @ H.T + R
        e = y[t] - H @ m
        Si = np.linalg.inv(S)
        ll += -0.5 * (dy * LOG2PI + np.linalg.slogdet(S)[1] + e @ Si @ e)
        K = P @ H.T @ Si
        m = m + K @ e
        P = P - K @ H @ P
        P = 0.5 * (P + P.T)
    return ll


def loglik_and_grad(F, logq, H, logr, m0, S0, y):
    """(log p(y), d log p / d theta) with Q = diag(exp(logq)), R = diag(exp(logr)).

    theta order: F.ravel() (d*d), logq (d), logr (dy).
    """
    F, H, m0, S0 = (np.asarray(a, np.float64) for a in (F, H, m0, S0))
    logq, logr = np.asarray(logq, np.float64), np.asarray(logr, np.float64)
    y = np.asarray(y, np.float64).reshape(len(y), -1)
    d, dy = F.shape[0], H.shape[0]
    Q, R = np.diag(np.exp(logq)), np.diag(np.exp(logr))
    npar = d * d + d + dy
    dF = np.zeros((npar, d, d))
    dQ = np.zeros((npar, d, d))
    dR = np.zeros((npar, dy, dy))
    for i in range(d):
        for j in range(d):
            dF[i * d + j, i, j] = 1.0
    for i in range(d):
        dQ[d * d + i, i, i] = np.exp(logq[i])
    for i in range(dy):
        dR[d * d + d + i, i, i] = np.exp(logr[i])

    m, P = m0.copy(), S0.copy()
    dm = np.zeros((npar, d))
    dP = np.zeros((npar, d, d))
    ll = 0.0
    g = np.zeros(npar)
    for t in range(y.shape[0]):
        if t > 0:
            dm = np.einsum("pij,j->pi", dF, m) + dm @ F.T
            dP = (np.einsum("pij,jk,lk->pil", dF, P, F) + np.einsum("ij,pjk,lk->pil", F, dP, F)
                  + np.einsum("ij,jk,plk->pil", F, P, dF) + dQ)
            m = F @ m
            P = F @ P @ F.T + Q
        S = H @ P @ H.T + R
        e = y[t] - H @ m
        Si = np.linalg.inv(S)
        Sie = Si @ e
        ll += -0.5 * (dy * LOG2PI + np.linalg.slogdet(S)[1] + e @ Sie)
        dS = np.einsum("ij,pjk,lk->pil", H, dP, H) + dR
        de = -dm @ H.T
        g += -0.5 * (np.einsum("ij,pji->p", Si, dS) + 2.0 * de @ Sie - np.einsum("i,pij,j->p", Sie, dS, Sie))
        PHt = P @ H.T
        K = PHt @ Si
        dK = np.einsum("pij,kj->pik", dP, H) @ Si - np.einsum("ij,pjk,kl->pil", PHt @ Si, dS, Si)
        dm = dm + np.einsum("pij,j->pi", dK, e) + de @ K.T
        HP = H @ P
        dP = dP - np.einsum("pij,jk->pik", dK, HP) - np.einsum("ij,pjk->pik", K @ H, dP)
        dP = 0.5 * (dP + np.transpose(dP, (0, 2, 1)))
        m = m + K @ e
        P = P - K @ HP
        P = 0.5 * (P + P.T)
    return ll, g


def filter_marginals(F, Q, H, R, m0, C0, y):
    """run_kalman_filter_for_marginals (kalman.py:16-57) in float64, as the reference writes it:
    at t = 0 the initial covariance *square root* C0 stands in for the covariance; no
    symmetrisation.  Returns (means (T, d), covs (T, d, d), prediction-error log-likelihood)."""
    F, Q, H, R, m0, C0 = (np.asarray(a, np.float64) for a in (F, Q, H, R, m0, C0))
    y = np.asarray(y, np.float64).reshape(len(y), -1)
    dy = H.shape[0]
    mus, covs, ll = [], [], 0.0
    m, P = m0, C0
    for t in range(y.shape[0]):
        if t > 0:
            m = F @ m
            P = F @ P @ F.T + Q
        S = H @ P @ H.T + R
        Si = np.linalg.inv(S)
        e = y[t] - H @ m
        ll += -0.5 * (dy * LOG2PI + np.linalg.slogdet(S)[1] + e @ Si @ e)
        K = P @ H.T @ Si
        m = m + K @ e
        P = P - K @ H @ P
        mus.append(m)
        covs.append(P)
    return np.stack(mus), np.stack(covs), ll


def smoother_marginals(F, Q, means, covs, lag_ones=False):
    """run_kalman_smoother_for_marginals (kalman.py:60-104) in float64 from filter output;
    lag_ones=True also returns the lag-one terms of kalman.py:83, whose 1-D `@` products
    are dot products."""
    F, Q = np.asarray(F, np.float64), np.asarray(Q, np.float64)
    means, covs = np.asarray(means, np.float64), np.asarray(covs, np.float64)
    T, d = means.shape
    sm, sc = means.copy(), covs.copy()
    lag = np.zeros((max(T - 1, 0), d, d))
    for t in range(T - 2, -1, -1):
        A = F @ covs[t] @ F.T + Q
        G = covs[t] @ F.T @ np.linalg.inv(A)
        lag[t] = means[t] @ sm[t + 1] + G @ (sc[t + 1] + (sm[t + 1] - means[t + 1]) @ sm[t + 1])
        sm[t] = means[t] + G @ (sm[t + 1] - F @ means[t])
        sc[t] = covs[t] + G @ (sc[t + 1] - A) @ G.T
    return (sm, sc, lag) if lag_ones else (sm, sc)
