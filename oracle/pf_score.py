"""ORACLE (test infrastructure only): float64 restatement of the PaRIS score recursion.

Given a filter run's particles, its resampling ancestors and the backward
draws J (from o_lg_score), recompute the Fisher-identity statistics in
float64 from their definition

    tau_0^i = g_0(x_0^i)
    tau_t^i = (1/K) sum_k [tau_{t-1}^{J_k} + h_t(x_{t-1}^{J_k}, x_t^i)] + g_t(x_t^i)
    score   = sum_i W_{T-1}^i tau_{T-1}^i

with, for theta = (A, log q, log r) of x_t = A x_{t-1} + N(0, diag q),
y_t = x_t + N(0, diag r):

    h_t: dA_kl = e_k x_{t-1,l} / q_k,  dlog q_k = e_k^2 / (2 q_k) - 1/2,  e = x_t - A x_{t-1}
    g_t: dlog r_k = (y_k - x_k)^2 / (2 r_k) - 1/2.

This pins the float32 C restatement's arithmetic (o_score_step) independently
of its rounding: the two agree to float32 accumulation error.  The filter
itself follows mocat/src/ssm/filtering.py:255-324 (see oracle.c o_lg_run).
"""
import numpy as np


def score_from_draws(A, q, r, x_hist, lw_last, draws, y):
    """x_hist (T, n, d) float32 particles of every step; lw_last (n,) final
    log-weights; draws (T, n, K) source-particle indices of the backward draws
    (row 0 unused); y (T, d).  Returns the score (d*d + 2d,) in float64."""
    A, q, r = (np.asarray(a, np.float64) for a in (A, q, r))
    x_hist = np.asarray(x_hist, np.float64)
    y = np.asarray(y, np.float64).reshape(x_hist.shape[0], -1)
    T, n, d = x_hist.shape
    K = draws.shape[2]

    def g(x, yt):
        return -0.5 + (yt - x) ** 2 / (2.0 * r)

    tau = np.zeros((n, d * d + 2 * d))
    tau[:, d * d + d:] = g(x_hist[0], y[0])
    for t in range(1, T):
        xp, xn = x_hist[t - 1], x_hist[t]
        new = np.zeros_like(tau)
        for k in range(K):
            j = draws[t, :, k].astype(np.int64)
            e = xn - xp[j] @ A.T
            hA = (e / q)[:, :, None] * xp[j][:, None, :]
            new[:, :d * d] += tau[j, :d * d] + hA.reshape(n, -1)
            new[:, d * d:d * d + d] += tau[j, d * d:d * d + d] + (-0.5 + e * e / (2.0 * q))
            new[:, d * d + d:] += tau[j, d * d + d:]
        new /= K
        new[:, d * d + d:] += g(xn, y[t])
        tau = new
    lw = np.asarray(lw_last, np.float64)
    w = np.exp(lw - lw.max())
    return (w / w.sum()) @ tau
