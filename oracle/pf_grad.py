"""Differentiable float64 restatement of the bootstrap particle filter's log Z
with the resampling held fixed -- test infrastructure only (the checker of the
GPU adjoint, never part of the product path).

The filter is run_particle_filter_for_marginals (mocat/src/ssm/filtering.py:255-324)
with BootstrapFilter (:142-170) on a TimeHomogenousLinearGaussian model
(mocat/src/ssm/linear_gaussian/linear_gaussian.py:142-261) whose observation
matrix is the identity and whose covariances are diagonal:
    x_0 = C0 eps_0 + m0,             lw_0 = -pot(x_0, y_0)
    x_t = A x_{t-1}[a_t] + sqrt(q) eps_t,  lw_t = lw_res - pot(x_t, y_t)
    pot(x, y) = 0.5 sum_k (y_k - x_k)^2 / r_k + 0.5 sum_k log(2 pi r_k)
    log Z = sum_t [LSE(lw_t) - (log n if step t resampled (or t = 0) else LSE(lw_{t-1}))]
theta = (A, log q, log r).  The noise eps and the ancestors a_t come from the
oracle's float32 filter with the same key (common random numbers), so the
reference's jax.grad through run_particle_filter_for_marginals with the
ancestors treated as constants is restated by torch.autograd in float64.
"""
import math

import numpy as np
import torch


def tape(params, n, key, y, ess_threshold=0.5, scheme="systematic"):
    """Noise and ancestors of the oracle's float32 run: dict(eps (T, n, d), ancestors (T, n),
    resampled (T,), log_z) -- the common random numbers of the differentiable restatement."""
    import oracle as O
    y = np.asarray(y, np.float32).reshape(len(y), -1)
    T, d = y.shape[0], int(params["d"])
    run = O.lg_run_tape(params, n, key, y, ess_threshold, scheme)
    keys = O.lg_step_keys(key, T)
    eps = np.stack([O.lg_normals(keys[t], n, d) for t in range(T)])
    return dict(eps=eps, ancestors=run["ancestors"], resampled=run["resampled"], log_z=run["log_z"])


def log_z(A, log_q, log_r, m0, C0, y, eps, ancestors, resampled):
    """log Z as a differentiable function of (A, log_q, log_r) (torch float64 tensors)."""
    y = torch.as_tensor(np.asarray(y, np.float64))
    eps = torch.as_tensor(np.asarray(eps, np.float64))
    m0 = torch.as_tensor(np.asarray(m0, np.float64))
    C0 = torch.as_tensor(np.asarray(C0, np.float64))
    T, n, d = eps.shape
    r = torch.exp(log_r)
    sq = torch.exp(0.5 * log_q)
    c = 0.5 * torch.sum(math.log(2 * math.pi) + log_r)
    logn = math.log(n)

    def pot(x, yt):
        return 0.5 * torch.sum((yt - x) ** 2 / r, dim=1) + c

    x = eps[0] @ C0.T + m0
    lw = -pot(x, y[0])
    lz = torch.logsumexp(lw, 0) - logn
    for t in range(1, T):
        if resampled[t]:
            a = torch.as_tensor(np.asarray(ancestors[t], np.int64))
            xs, lres, lse_res = x[a], torch.zeros(n, dtype=torch.float64), logn
        else:
            xs, lres, lse_res = x, lw, torch.logsumexp(lw, 0)
        x = xs @ A.T + sq * eps[t]
        lw = lres - pot(x, y[t])
        lz = lz + torch.logsumexp(lw, 0) - lse_res
    return lz


def grad(A, log_q, log_r, m0, C0, y, tp):
    """(log Z, dlogZ/dA (d, d), dlogZ/dlog_q (d,), dlogZ/dlog_r (d,)) in float64."""
    A = torch.tensor(np.asarray(A, np.float64), requires_grad=True)
    lq = torch.tensor(np.asarray(log_q, np.float64), requires_grad=True)
    lr = torch.tensor(np.asarray(log_r, np.float64), requires_grad=True)
    lz = log_z(A, lq, lr, m0, C0, y, tp["eps"], tp["ancestors"], tp["resampled"])
    lz.backward()
    return float(lz.detach()), A.grad.numpy(), lq.grad.numpy(), lr.grad.numpy()
