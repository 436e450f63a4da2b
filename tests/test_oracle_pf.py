"""Pins of the oracle's particle-system step (CPU).

* gaussian_potential against scipy's logpdf -- the cases of the reference's
  mocat/src/tests/test_utils.py:37-118;
* float64 Kalman log-likelihood gradient against finite differences;
* the particle filter's log-marginal-likelihood against the Kalman oracle;
* fixed-point systematic / multinomial resampling against exact big-integer
  restatements and against float64 inverse-CDF resampling (boundary ties
  counted);
* categorical against a brute-force argmax of the same Gumbel draws.
"""
import warnings

import numpy as np
import pytest
from scipy.stats import multivariate_normal

import oracle as O
from oracle import kalman, models
from oracle.potentials import gaussian_potential


def test_gaussian_potential_reference_cases():
    x = np.array([7.0])
    assert np.allclose(gaussian_potential(x), -multivariate_normal.logpdf(x, 0.0, 1.0))
    m = np.array([1.0])
    assert np.allclose(gaussian_potential(x, m), -multivariate_normal.logpdf(x, m, 1.0))
    prec = np.array([[2.0]])
    assert np.allclose(gaussian_potential(x, prec=prec[0]), -multivariate_normal.logpdf(x, 0, 1 / prec))
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        assert np.allclose(gaussian_potential(x, prec=prec), 0.5 * x ** 2 * prec)
    x = np.ones(5)
    prec = np.eye(5) * 2
    assert np.allclose(gaussian_potential(x, 3.0 * np.ones(5), prec=np.diag(prec), det_prec=2 ** 5),
                       -multivariate_normal.logpdf(x, 3.0 * np.ones(5), np.linalg.inv(prec)))
    sqrt_prec = np.arange(25).reshape(5, 5) / 100 + np.eye(5)
    prec = sqrt_prec @ sqrt_prec.T
    assert np.allclose(gaussian_potential(x, prec=prec, det_prec=np.linalg.det(prec)),
                       -multivariate_normal.logpdf(x, np.zeros(5), np.linalg.inv(prec)))
    x = np.ones((5, 2))
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        sp = np.array([[5.0, 0.0], [2.0, 3.0]])
        assert np.allclose(gaussian_potential(x, sqrt_prec=sp), np.repeat(0.5 * x[0] @ sp @ sp.T @ x[0], 5))


def test_lg_potential_matches_gaussian_potential():
    """The oracle's float32 LG weight equals -gaussian_potential(y, Hx, sqrt_prec=P, det_prec)."""
    d = 3
    rng = np.random.default_rng(0)
    R = np.diag([0.5, 0.7, 0.9])
    p = models.lg_params(np.zeros(d), np.eye(d), np.eye(d) * 0.9, np.eye(d), np.eye(d), R)
    x0, lw0 = O.lg_init(p, 64, O.PRNGKey(2), np.array([0.1, -0.3, 0.2], np.float32))
    ref = -gaussian_potential(np.array([0.1, -0.3, 0.2]), x0.astype(np.float64) @ p["H"].T.astype(np.float64),
                              sqrt_prec=np.linalg.inv(np.linalg.cholesky(R)), det_prec=1 / np.linalg.det(R))
    assert np.allclose(lw0, ref, rtol=1e-5, atol=1e-5)
    _ = rng


def test_kalman_gradient_finite_differences():
    d = 3
    F = models.random_stable_matrix(d, 0)
    logq, logr = np.log(0.1) * np.ones(d), np.log(0.5) * np.ones(d)
    p = models.lg_params(np.zeros(d), np.eye(d), F, np.diag(np.exp(logq)), np.eye(d), np.diag(np.exp(logr)))
    _, y = models.simulate_lg(p, 40, O.PRNGKey(0))
    ll, g = kalman.loglik_and_grad(F, logq, np.eye(d), logr, np.zeros(d), np.eye(d), y)
    th = np.concatenate([F.ravel(), logq, logr])

    def f(v):
        return kalman.loglik(v[:9].reshape(3, 3), np.diag(np.exp(v[9:12])), np.eye(3), np.diag(np.exp(v[12:])),
                             np.zeros(3), np.eye(3), y)

    eps = 1e-6
    fd = np.array([(f(th + eps * e) - f(th - eps * e)) / (2 * eps) for e in np.eye(th.size)])
    assert abs(ll - f(th)) < 1e-10
    assert np.max(np.abs(fd - g)) < 1e-5 * max(1.0, np.max(np.abs(g)))


@pytest.mark.parametrize("scheme", ["systematic", "multinomial"])
def test_pf_log_z_close_to_kalman(scheme):
    p = models.lg_params(np.zeros(1), np.eye(1), [[0.9]], np.eye(1), np.eye(1), [[0.25]])
    _, y = models.simulate_lg(p, 100, O.PRNGKey(0))
    kl = kalman.loglik(p["F64"], p["Q"], p["H64"], p["R"], p["m064"], p["S0"], y)
    r = O.lg_run(p, 20000, O.PRNGKey(1), y, ess_threshold=0.5, scheme=scheme)
    assert abs(r["log_z"] - kl) < 0.3, (r["log_z"], kl)
    assert r["resampled"].any()


def _exact_systematic(q, m23):
    n = len(q)
    C = np.cumsum(q.astype(object))
    Q = int(C[-1])
    out = np.empty(n, np.int64)
    i = 0
    for k in range(n):
        thr = ((k << 23) + m23) * Q // (n << 23)
        while C[i] <= thr:
            i += 1
        out[k] = i
    return out


@pytest.mark.parametrize("n", [1, 2, 7, 257, 3001])
def test_systematic_integer_math_exact(n):
    rng = np.random.default_rng(n)
    lw = (rng.standard_normal(n) * 3).astype(np.float32)
    q, ok = O.quantise(lw)
    assert ok
    for m in (0, 1, 4194304, (1 << 23) - 1):
        anc, _ = O.resample_systematic(lw, m)
        assert (anc == _exact_systematic(q, m)).all()


def test_systematic_vs_float64_ties_counted():
    """Same float32 weights, float64 cumulative sum vs exact 62-bit integer prefix:
    any disagreement is a boundary tie of the float64 scan; they are counted."""
    rng = np.random.default_rng(1)
    n = 100_000
    lw = (rng.standard_normal(n) * 2).astype(np.float32)
    m = 3_000_001
    anc, _ = O.resample_systematic(lw, m)
    w = O.expf(lw - lw.max()).astype(np.float64)
    c = np.cumsum(w)
    thr = (np.arange(n) + m * 2.0 ** -23) / n * c[-1]
    ref = np.searchsorted(c, thr, side="right")
    ties = int((anc != ref).sum())
    print(f"systematic n={n}: float64-scan boundary ties = {ties}")
    assert ties <= 1, ties
    assert (np.diff(anc) >= 0).all()
    # weights from a float64 exp differ from the float32 weights by ~1 ulp,
    # which moves a handful of boundaries: reported, bounded
    w64 = np.exp(lw.astype(np.float64) - lw.max())
    c64 = np.cumsum(w64)
    ref64 = np.searchsorted(c64, (np.arange(n) + m * 2.0 ** -23) / n * c64[-1], side="right")
    moved = int((anc != ref64).sum())
    print(f"systematic n={n}: boundaries moved by float64 exp = {moved}")
    assert moved <= n * 1e-3


def test_multinomial_distribution():
    n = 4096
    lw = np.log(np.linspace(0.1, 1.0, n)).astype(np.float32)
    counts = np.zeros(n)
    for s in range(40):
        anc, ok = O.resample_multinomial(lw, O.PRNGKey(s))
        assert ok and (np.diff(anc) >= 0).all()
        counts += np.bincount(anc, minlength=n)
    w = np.exp(lw.astype(np.float64))
    w /= w.sum()
    # mean offspring in quarters of the index range
    got = counts.reshape(4, -1).sum(1) / counts.sum()
    exp_ = w.reshape(4, -1).sum(1)
    assert np.allclose(got, exp_, atol=0.01)


def test_categorical_bruteforce():
    n = 50
    rng = np.random.default_rng(2)
    lw = rng.standard_normal(n).astype(np.float32)
    key = O.PRNGKey(9)
    anc = O.resample_gumbel(lw, key)
    g = O.gumbel(key, (n, n))
    assert (anc == np.argmax(g + lw[None, :], axis=1)).all()


def test_degenerate_weights():
    n = 10
    for lw in (np.full(n, -np.inf, np.float32), np.array([0.0] * 9 + [np.nan], np.float32)):
        anc, ok = O.resample_systematic(lw, 5)
        assert not ok and (anc == 0).all()
        anc, ok = O.resample_multinomial(lw, O.PRNGKey(0))
        assert not ok and (anc == 0).all()
