"""Backward simulation (full FFBSi, backward.py:217-245) on the GPU vs the oracle's
restatement: the sampled particle indices and trajectories are bit-exact (same
Gumbel draws, same transition-potential arithmetic, first maximum wins).  The
statistical check: smoothing means of a 1-D linear-Gaussian model against the
exact Rauch-Tung-Striebel smoother."""
import numpy as np
import pytest
import torch

import oracle as O
from oracle import models

pytestmark = pytest.mark.gpu


def _lg(d, seed=0):
    import mocat_gb300 as mg
    F = models.random_stable_matrix(d, seed)
    Q = 0.3 * np.eye(d) + (0.05 * np.ones((d, d)) if d > 1 else 0)
    H, R = np.eye(d), 0.5 * np.eye(d)
    p = models.lg_params(np.zeros(d), np.eye(d), F, Q, H, R)
    ssm = mg.ssm.TimeHomogenousLinearGaussian(np.zeros(d), np.eye(d), F, Q, H, R)
    return p, ssm, F, Q


@pytest.mark.parametrize("d,n,M,T", [(1, 300, 200, 12), (3, 257, 64, 10), (10, 512, 33, 6),
                                     (7, 300, 40, 6), (16, 200, 17, 4)])  # 7, 16: run-time dimension
def test_backward_simulation_matches_oracle(cuda, d, n, M, T):
    import mocat_gb300 as mg
    p, ssm, F, Q = _lg(d, seed=d)
    _, y = models.simulate_lg(p, T, O.PRNGKey(1))
    pf = mg.ssm.run_particle_filter_for_marginals(ssm, mg.ssm.BootstrapFilter(), y, np.arange(T), O.PRNGKey(2), n=n)
    key = O.PRNGKey(3)
    out = mg.ssm.backward_simulation(ssm, pf, key, n_samps=M)
    keep, _ = mg.ssm._transition_struct(ssm)
    ro, ri = O.ffbsi_lg(keep["F"], keep["Pq"], keep["cq"], pf.value.cpu().numpy(), pf.log_weight.cpu().numpy(),
                        key, M)
    assert np.array_equal(out.indices.cpu().numpy(), ri)
    assert np.array_equal(out.value.cpu().numpy(), ro)
    assert out.value.shape == (T, M, d)


def test_smoothing_means_match_rts(cuda):
    import mocat_gb300 as mg
    p, ssm, F, Q = _lg(1, seed=0)
    T = 30
    _, y = models.simulate_lg(p, T, O.PRNGKey(5))
    out = mg.ssm.forward_filtering_backward_simulation(ssm, mg.ssm.BootstrapFilter(), y, np.arange(T), 4096,
                                                       O.PRNGKey(6), n_pf=8192)
    # Rauch-Tung-Striebel smoother (float64)
    f, q, r = float(F[0, 0]), float(Q[0, 0]), 0.5
    m, P = 0.0, 1.0
    ms, Ps, mp, Pp = [], [], [], []
    for t in range(T):
        if t:
            m, P = f * m, f * f * P + q
        mp.append(m)
        Pp.append(P)
        k = P / (P + r)
        m, P = m + k * (float(y[t, 0]) - m), (1 - k) * P
        ms.append(m)
        Ps.append(P)
    sm, sP = ms[-1], Ps[-1]
    smooth = [sm]
    for t in range(T - 2, -1, -1):
        g = Ps[t] * f / Pp[t + 1]
        sm = ms[t] + g * (sm - mp[t + 1])
        smooth.append(sm)
    smooth = np.array(smooth[::-1])
    est = out.value[:, :, 0].double().mean(1).cpu().numpy()
    assert np.abs(est - smooth).max() < 0.1, np.abs(est - smooth).max()
