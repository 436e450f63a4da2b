"""The oracle's Fisher-identity / PaRIS score (o_lg_score), on the CPU.

(1) Its float32 arithmetic equals the float64 restatement of the recursion
    (oracle/pf_score.py) fed the same particles and backward draws, within
    float32 accumulation error (1e-5 of the largest entry).
(2) Its filter is o_lg_run's: the same resampling steps and log Z.
(3) The backward draws are what the estimator defines: the first draw of
    every particle is its own ancestor (itself when the step did not resample),
    and with one draw the statistic is traced along the genealogy.
(4) It is consistent: against the exact Kalman score its error falls as n
    grows, at about the n^-1/2 rate (the fixed-ancestor pathwise gradient's
    does not fall).
"""
import numpy as np
import pytest

import oracle as O
from oracle import kalman, models, pf_score


def _model(d, seed):
    A = models.random_stable_matrix(d, seed)
    q = np.full(d, 0.2) * (1 + 0.1 * np.arange(d))
    r = np.full(d, 0.5) * (1 + 0.05 * np.arange(d))
    p = models.lg_params(np.zeros(d), np.eye(d), A, np.diag(q), np.eye(d), np.diag(r))
    return A, q, r, p


@pytest.mark.parametrize("scheme", ["systematic", "multinomial"])
@pytest.mark.parametrize("d,n,T,K,L,thr", [(1, 500, 30, 2, 8, 0.5), (3, 512, 30, 4, 3, 0.8), (3, 511, 25, 1, 0, 1.1),
                                           (10, 256, 20, 2, 5, 0.5), (2, 300, 40, 3, 2, 0.3)])
def test_float32_restatement_matches_float64_definition(scheme, d, n, T, K, L, thr):
    A, q, r, p = _model(d, d)
    _, y = models.simulate_lg(p, T, O.PRNGKey(d))
    key, skey = O.PRNGKey(7), O.PRNGKey(8)
    o = O.lg_score(p, n, key, skey, y, thr, scheme, K, L, draws=True)
    run = O.lg_run(p, n, key, y, thr, scheme, history=True)
    assert abs(o["log_z"] - run["log_z"]) <= 1e-12 * abs(run["log_z"])  # OpenMP-reduced float64 sums
    assert np.array_equal(o["resampled"], run["resampled"])
    ref = pf_score.score_from_draws(A, q, r, run["value"], run["log_weight"][-1], o["draws"], y)
    assert np.abs(ref - o["grad"]).max() <= 1e-5 * np.abs(ref).max()


def test_first_draw_is_the_ancestor_and_one_draw_traces_the_genealogy():
    d, n, T = 3, 700, 30
    A, q, r, p = _model(d, 1)
    _, y = models.simulate_lg(p, T, O.PRNGKey(2))
    key = O.PRNGKey(3)
    tape = O.lg_run_tape(p, n, key, y, 0.6, "systematic")
    res = tape["resampled"]
    assert 0 < res[1:].sum() < T - 1  # both kinds of step occur
    for K, L in ((1, 0), (3, 4)):
        o = O.lg_score(p, n, key, O.PRNGKey(4), y, 0.6, "systematic", K, L, draws=True)
        dr = o["draws"]
        for t in range(1, T):
            own = tape["ancestors"][t] if res[t] else np.arange(n)
            assert np.array_equal(dr[t, :, 0], own)
            assert dr[t].min() >= 0 and dr[t].max() < n
        if K > 1:  # the chain moves for some particles
            assert (dr[1:, :, 1] != dr[1:, :, 0]).mean() > 0.05


def test_more_proposals_move_the_chain_more():
    d, n, T = 3, 1000, 20
    A, q, r, p = _model(d, 5)
    _, y = models.simulate_lg(p, T, O.PRNGKey(6))
    moved = []
    for L in (1, 4, 16):
        dr = O.lg_score(p, n, O.PRNGKey(9), O.PRNGKey(10), y, 0.5, "systematic", 2, L, draws=True)["draws"]
        moved.append((dr[1:, :, 1] != dr[1:, :, 0]).mean())
    assert moved[0] < moved[1] < moved[2]


def test_error_against_the_kalman_score_falls_with_n():
    d, T = 2, 50
    A = models.random_stable_matrix(d, 3)
    q = np.full(d, 0.2) * (1 + 0.1 * np.arange(d))
    r = np.full(d, 0.5)
    p = models.lg_params(np.zeros(d), np.eye(d), A, np.diag(q), np.eye(d), np.diag(r))
    _, y = models.simulate_lg(p, T, O.PRNGKey(4))
    _, g = kalman.loglik_and_grad(A, np.log(q), np.eye(d), np.log(r), np.zeros(d), np.eye(d), y.astype(np.float64))

    def err(n):
        return np.mean([np.linalg.norm(O.lg_score(p, n, O.PRNGKey(10 + s), O.PRNGKey(20 + s), y, 0.5, "systematic",
                                                  2, 8)["grad"] - g) / np.linalg.norm(g) for s in range(6)])

    e_small, e_large = err(256), err(16384)
    # n^-1/2 predicts a factor 8 over this range; measured about 5.6
    assert e_large < 0.35 * e_small, (e_small, e_large)
    assert e_large < 0.15, e_large
