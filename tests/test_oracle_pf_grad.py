"""The float64 differentiable restatement used to check the adjoint: its log Z
equals the oracle's float32 filter (same noise and ancestors), and its
autograd gradient equals central finite differences with common random
numbers.  CPU only."""
import numpy as np
import torch

import oracle as O
from oracle import models, pf_grad


def test_restatement_log_z_and_finite_differences():
    d, n, T = 3, 400, 25
    A = models.random_stable_matrix(d, 0)
    q, r = np.full(d, 0.1), np.full(d, 0.5)
    p = models.lg_params(np.zeros(d), np.eye(d), A, np.diag(q), np.eye(d), np.diag(r))
    _, y = models.simulate_lg(p, T, O.PRNGKey(0))
    tp = pf_grad.tape(p, n, O.PRNGKey(1), y, 0.7, "systematic")
    assert tp["resampled"].sum() > 2
    lz, gA, gq, gr = pf_grad.grad(A, np.log(q), np.log(r), np.zeros(d), np.eye(d), y, tp)
    assert abs(lz - tp["log_z"]) < 1e-5 * abs(lz)

    def f(A_, lq, lr):
        return float(pf_grad.log_z(torch.tensor(A_), torch.tensor(lq), torch.tensor(lr), np.zeros(d), np.eye(d), y,
                                   tp["eps"], tp["ancestors"], tp["resampled"]))

    h = 1e-5
    for (i, j) in [(0, 0), (1, 2), (2, 0)]:
        E = np.zeros((d, d))
        E[i, j] = h
        fd = (f(A + E, np.log(q), np.log(r)) - f(A - E, np.log(q), np.log(r))) / (2 * h)
        assert abs(fd - gA[i, j]) < 1e-5 * max(1.0, abs(fd))
    for k in range(d):
        e = np.zeros(d)
        e[k] = h
        fq = (f(A, np.log(q) + e, np.log(r)) - f(A, np.log(q) - e, np.log(r))) / (2 * h)
        fr = (f(A, np.log(q), np.log(r) + e) - f(A, np.log(q), np.log(r) - e)) / (2 * h)
        assert abs(fq - gq[k]) < 1e-5 * max(1.0, abs(fq))
        assert abs(fr - gr[k]) < 1e-5 * max(1.0, abs(fr))
