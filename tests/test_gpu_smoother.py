"""Online fixed-lag smoothing (online_smoothing.py) on the GPU vs the oracle.

The stitch kernel and the pair potentials are bit-exact with the oracle; the
particle-filter variant of propagate_particle_smoother, run for a dozen steps
with lag 3, reproduces an oracle-driven restatement (propagate, systematic
resampling, stitching) bit for bit.  The backward-simulation variant is run
for shape and consistency checks."""
import numpy as np
import pytest
import torch

import oracle as O
from oracle import models

pytestmark = pytest.mark.gpu


def _lg(d, seed=0):
    import mocat_gb300 as mg
    F = models.random_stable_matrix(d, seed)
    Q = 0.3 * np.eye(d)
    H, R = np.eye(d), 0.5 * np.eye(d)
    p = models.lg_params(np.zeros(d), np.eye(d), F, Q, H, R)
    ssm = mg.ssm.TimeHomogenousLinearGaussian(np.zeros(d), np.eye(d), F, Q, H, R)
    return p, ssm


@pytest.mark.parametrize("d,M0,M1", [(1, 100, 300), (3, 65, 257), (10, 40, 128),
                                     (12, 50, 129), (32, 20, 70)])  # 12, 32: run-time dimension
def test_stitch_and_pair_potential_bit_exact(cuda, d, M0, M1):
    import mocat_gb300 as mg
    _, ssm = _lg(d, d)
    rng = np.random.default_rng(d)
    x0 = rng.standard_normal((M0, d)).astype(np.float32)
    x1 = rng.standard_normal((M1, d)).astype(np.float32)
    lw = rng.standard_normal(M1).astype(np.float32)
    keep, _ = mg.ssm._transition_struct(ssm)
    key = O.PRNGKey(4)
    idx = mg.ssm.full_stitch(ssm, torch.from_numpy(x0).cuda(), 0.0, torch.from_numpy(x1).cuda(), 1.0,
                             torch.from_numpy(lw).cuda(), key)
    assert np.array_equal(idx.cpu().numpy(), O.stitch_lg(keep["F"], keep["Pq"], keep["cq"], x0, x1, lw, key))
    pp = mg.ssm._pair_potential(ssm, torch.from_numpy(x1[:M0]).cuda(), torch.from_numpy(x1[M1 - M0:]).cuda())
    ref = O.transition_potential_pairs(keep["F"], keep["Pq"], keep["cq"], x1[:M0], x1[M1 - M0:])
    assert np.array_equal(pp.cpu().numpy(), ref)


def _oracle_smoother_pf(p, keep, x0, lw0, y, keys, lag):
    n = x0.shape[0]
    value = [x0]
    lw = lw0.astype(np.float32)
    for t in range(1, len(y)):
        key = keys[t]
        lwd = lw.astype(np.float64)
        m = lwd.max()
        ess = np.exp(2 * (m + np.log(np.exp(lwd - m).sum())) - (2 * m + np.log(np.exp(2 * (lwd - m)).sum())))
        if ess < n - 1e-3:
            anc = O.resample_systematic(lw, int(O.random_bits(key, 1)[0]) >> 9)
            value = [v[anc] for v in value]
        x_new, lw = O.lg_propagate(p, key, y[t], value[-1], None, None)
        value.append(x_new)
        s1 = len(value) - lag - 1
        if s1 >= 0:
            nilw = lw + O.transition_potential_pairs(keep["F"], keep["Pq"], keep["cq"], value[s1], value[s1 + 1])
            idx = O.stitch_lg(keep["F"], keep["Pq"], keep["cq"], value[s1], value[s1 + 1], nilw, key)
            value = value[:s1 + 1] + [v[idx] for v in value[s1 + 1:]]
            lw = np.zeros(n, np.float32)
    return np.stack(value)


@pytest.mark.parametrize("d,n", [(1, 400), (3, 256), (6, 256)])  # 6: run-time dimension
def test_smoother_pf_variant_matches_oracle(cuda, d, n):
    import mocat_gb300 as mg
    p, ssm = _lg(d, 10 + d)
    T, lag = 12, 3
    _, y = models.simulate_lg(p, T, O.PRNGKey(7))
    keys = O.split(O.PRNGKey(8), T)
    bf = mg.ssm.BootstrapFilter()
    parts = mg.ssm.initiate_particles(ssm, bf, n, keys[0], y[0], t=0.0)
    for t in range(1, T):
        parts = mg.ssm.propagate_particle_smoother(ssm, bf, parts, y[t], float(t), keys[t], lag, backward_sim=False)
    keep, _ = mg.ssm._transition_struct(ssm)
    x0, lw0 = O.lg_init(p, n, keys[0], y[0])
    ref = _oracle_smoother_pf(p, keep, x0, lw0, y, keys, lag)
    assert np.array_equal(parts.value.cpu().numpy(), ref)
    assert parts.num_transition_evals.numel() == T


def test_smoother_bs_variant_runs(cuda):
    import mocat_gb300 as mg
    p, ssm = _lg(2, 3)
    T, lag, n = 10, 3, 256
    _, y = models.simulate_lg(p, T, O.PRNGKey(9))
    keys = O.split(O.PRNGKey(10), T)
    bf = mg.ssm.BootstrapFilter()
    parts = mg.ssm.initiate_particles(ssm, bf, n, keys[0], y[0], t=0.0)
    for t in range(1, T):
        parts = mg.ssm.propagate_particle_smoother(ssm, bf, parts, y[t], float(t), keys[t], lag, backward_sim=True)
    assert parts.value.shape == (T, n, 2)
    assert parts.marginal_filter.value.shape == (T, n, 2)
    assert torch.isfinite(parts.value).all()
    # the smoothed draws are particles of the marginal filter
    mf = parts.marginal_filter.value.cpu().numpy()
    sv = parts.value.cpu().numpy()
    for t in range(T - lag, T):
        rows = {tuple(r) for r in mf[t]}
        assert all(tuple(r) in rows for r in sv[t])
