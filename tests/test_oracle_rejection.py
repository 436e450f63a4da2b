"""Rejection-sampling backward simulation and stitching in the oracle
(oracle.ffbsi_rejection_*, oracle.stitch_rejection_*), pinned against a pure-Python
float32 restatement written in the reference's own structure (mocat/src/ssm/backward.py:54-214,
online_smoothing.py:59-175: prerun, while-loop of proposal rounds with bound resets,
full categorical for the items still unaccepted) on the pinned RNG, categorical and
transition-potential primitives."""
import numpy as np
import pytest

import oracle as O
from oracle import models

F32 = np.float32


def _argmax(v):
    """jnp.argmax over finite-or-inf values: first maximum (NaN entries skipped, as the kernels do)"""
    v = np.where(np.isnan(v), -np.inf, v)
    return int(np.argmax(v)) if np.isfinite(v).any() or (v == np.inf).any() else 0


def _nanmax(v):
    return F32(np.nan) if np.isnan(v).any() else F32(np.max(v))


def py_rejection(pot, n, Np, lw, key, max_rej, ibp, infl):
    """rejection_resampling / rejection_stitching; pot(i, js) -> float32 potentials of item i
    against pool entries js.  Returns (idx, evals, resets, finals)."""
    lw = lw.astype(F32)
    ibp, infl = F32(ibp), F32(infl)
    k3 = O.split(key, 3)
    g = O.gumbel(k3[0], (n, Np))
    idx = np.array([_argmax((g[i] + lw).astype(F32)) for i in range(n)])
    dens = np.array([O.expf(-pot(i, [idx[i]]))[0] for i in range(n)], F32)
    mx = _nanmax(dens)
    bound = F32(mx * infl) if mx > ibp else ibp
    with np.errstate(divide="ignore", invalid="ignore"):
        nya = O.uniform(k3[1], (n,)) > (dens / bound).astype(F32)
    keys = O.split(k3[2], n).copy()
    evals, it, resets = n, 1, 0
    while nya.sum() > 0 and it < max_rej:
        evals += int(nya.sum())
        new = np.zeros(n, bool)
        dens = np.zeros(n, F32)
        for i in range(n):
            if not nya[i]:
                continue
            kk = O.split(keys[i], 3)
            keys[i] = kk[0]
            j = _argmax((O.gumbel(kk[1], (Np,)) + lw).astype(F32))
            idx[i] = j
            dens[i] = O.expf(-pot(i, [j]))[0]
            with np.errstate(divide="ignore", invalid="ignore"):
                new[i] = O.uniform(kk[2], ()) > F32(dens[i] / bound)
        mx = _nanmax(dens)
        if mx > bound:
            bound = F32(mx * infl)
            new[:] = True
            resets += 1
        nya = new
        it += 1
    finals = int(nya.sum())
    for i in np.flatnonzero(nya):
        w = (lw - pot(i, np.arange(Np))).astype(F32)
        idx[i] = _argmax((O.gumbel(keys[i], (Np,)) + w).astype(F32))
    evals += Np * finals
    return idx, evals, resets, finals


def _lg(d, seed):
    rng = np.random.default_rng(seed)
    F = models.random_stable_matrix(d, seed)
    A = rng.standard_normal((d, d))
    Q = A @ A.T / d + 0.3 * np.eye(d)
    Pq = np.linalg.inv(np.linalg.cholesky(Q)).astype(F32)
    cq = F32((d * np.log(2 * np.pi) + np.log(np.linalg.det(Q))) / 2)
    return F.astype(F32), Pq, cq


def _lg_pot(F, Pq, cq, x0_rows, x1_rows):
    return O.transition_potential_pairs(F, Pq, cq, x0_rows, x1_rows)


CASES = [(3, 0.0, 1.01), (2, 0.0, 1.01), (40, 0.0, 1.01), (6, 0.05, 1.5)]


@pytest.mark.parametrize("max_rej,ibp,infl", CASES)
def test_stitch_rejection_lg_matches_restatement(max_rej, ibp, infl):
    F, Pq, cq = _lg(2, 1)
    rng = np.random.default_rng(2)
    M = 12
    x0 = rng.standard_normal((M, 2)).astype(F32)
    x1 = (x0 @ F.T + 0.8 * rng.standard_normal((M, 2))).astype(F32)
    lw1 = rng.standard_normal(M).astype(F32)
    key = O.PRNGKey(11)

    def pot(i, js):
        js = np.asarray(js)
        return _lg_pot(F, Pq, cq, np.repeat(x0[i:i + 1], js.size, 0), x1[js])
    ref, rev, resets, finals = py_rejection(pot, M, M, lw1, key, max_rej, ibp, infl)
    idx, ev = O.stitch_rejection_lg(F, Pq, cq, x0, x1, lw1, key, max_rej, ibp, infl)
    assert np.array_equal(idx, ref) and ev == rev


def test_restatement_exercises_every_branch():
    """the chosen inputs go through bound resets, and through the final full draw"""
    F, Pq, cq = _lg(2, 1)
    rng = np.random.default_rng(2)
    M = 12
    x0 = rng.standard_normal((M, 2)).astype(F32)
    x1 = (x0 @ F.T + 0.8 * rng.standard_normal((M, 2))).astype(F32)
    lw1 = rng.standard_normal(M).astype(F32)

    def pot(i, js):
        js = np.asarray(js)
        return _lg_pot(F, Pq, cq, np.repeat(x0[i:i + 1], js.size, 0), x1[js])
    seen_reset = seen_final = False
    for s in range(8):
        _, _, resets, finals = py_rejection(pot, M, M, lw1, O.PRNGKey(s), 40, 0.0, 1.01)
        seen_reset |= resets > 0
        _, _, _, finals2 = py_rejection(pot, M, M, lw1, O.PRNGKey(s), 2, 0.0, 1.01)
        seen_final |= finals2 > 0
    assert seen_reset and seen_final


@pytest.mark.parametrize("max_rej,ibp,infl", CASES[:3])
def test_ffbsi_rejection_lg_matches_restatement(max_rej, ibp, infl):
    F, Pq, cq = _lg(3, 4)
    rng = np.random.default_rng(5)
    T, N, M = 4, 9, 7
    x = rng.standard_normal((T, N, 3)).astype(F32)
    lw = rng.standard_normal((T, N)).astype(F32)
    key = O.PRNGKey(3)
    out, idx, ev = O.ffbsi_rejection_lg(F, Pq, cq, x, lw, key, M, max_rej, ibp, infl)
    tk = O.split(key, T)
    ri = np.empty((T, M), np.int64)
    rev = np.zeros(T, np.int64)
    ri[-1] = O.resample_gumbel(lw[-1], tk[-1], M)
    xs = x[-1][ri[-1]]
    for t in range(T - 2, -1, -1):
        def pot(i, js, t=t, xs=xs):
            js = np.asarray(js)
            return _lg_pot(F, Pq, cq, x[t][js], np.repeat(xs[i:i + 1], js.size, 0))
        ri[t], rev[t + 1], _, _ = py_rejection(pot, M, N, lw[t], tk[t], max_rej, ibp, infl)
        xs = x[t][ri[t]]
    assert np.array_equal(idx, ri) and np.array_equal(ev, rev)
    assert np.array_equal(out, np.stack([x[t][ri[t]] for t in range(T)]))


def test_rejection_nl1d_matches_restatement():
    import mocat_gb300 as mg
    p, _ = mg.ssm.NonLinear1DBenchmark().derived()
    rng = np.random.default_rng(8)
    M = 10
    x0 = (3 * rng.standard_normal(M)).astype(F32)
    x1 = (3 * rng.standard_normal(M)).astype(F32)
    lw1 = rng.standard_normal(M).astype(F32)
    t_prev = F32(4.0)
    key = O.PRNGKey(21)

    def pot(i, js):
        js = np.asarray(js)
        return O.transition_potential_pairs_nl1d(p, np.repeat(x0[i:i + 1], js.size), x1[js], t_prev)
    for max_rej in (2, 30):
        ref, rev, _, _ = py_rejection(pot, M, M, lw1, key, max_rej, 0.0, 1.01)
        idx, ev = O.stitch_rejection_nl1d(p, x0, x1, lw1, t_prev, key, max_rej)
        assert np.array_equal(idx, ref) and ev == rev
    T, N = 3, 8
    xh = (3 * rng.standard_normal((T, N))).astype(F32)
    lwh = rng.standard_normal((T, N)).astype(F32)
    tt = np.arange(T, dtype=F32)
    out, idx, ev = O.ffbsi_rejection_nl1d(p, xh, lwh, tt, key, 6, 20)
    tk = O.split(key, T)
    ri = np.empty((T, 6), np.int64)
    ri[-1] = O.resample_gumbel(lwh[-1], tk[-1], 6)
    for t in range(T - 2, -1, -1):
        xs = xh[t + 1][ri[t + 1]]

        def pot(i, js, t=t, xs=xs):
            js = np.asarray(js)
            return O.transition_potential_pairs_nl1d(p, xh[t][js], np.repeat(xs[i:i + 1], js.size), tt[t])
        ri[t], r, _, _ = py_rejection(pot, 6, N, lwh[t], tk[t], 20, 0.0, 1.01)
        assert ev[t + 1] == r
    assert np.array_equal(idx, ri) and ev[0] == 0
