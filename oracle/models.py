"""ORACLE (test infrastructure only): scenario parameter derivation and simulation.

Restates, in float64 numpy rounded once to float32:
  * ``reset_covariance`` -- mocat/src/utils.py:247-262 (cholesky / inverse /
    determinant cached beside each covariance);
  * ``TimeHomogenousLinearGaussian.__init__`` -- mocat/src/ssm/linear_gaussian/
    linear_gaussian.py:160-209 (defaults to identities);
  * ``OptimalNonLinearGaussianParticleFilter.startup`` --
    mocat/src/ssm/nonlinear_gaussian.py:154-184 and ``kalman_gain``
    mocat/src/utils.py:476-484, for the linear transition function f(x) = F x;
  * ``StochasticVolatility`` -- mocat/src/ssm/scenarios/stochastic_volatility.py:25-108;
  * ``StateSpaceModel.simulate`` -- mocat/src/ssm/ssm.py:138-163 (keys =
    split(key, 2T): the first T drive the latent chain, the last T the
    observations).
"""
import numpy as np

from . import normal, split

LOG2PI = float(np.log(2.0 * np.pi))


def _mat(a, d=None):
    a = np.asarray(a, np.float64)
    if a.ndim == 0:
        a = np.eye(d or 1) * a
    elif a.ndim == 1:
        a = np.diag(a)
    return a


def lg_params(initial_mean=None, initial_covariance=None, transition_matrix=None, transition_covariance=None,
              likelihood_matrix=None, likelihood_covariance=None, dim=None):
    """float32 parameter block used by oracle.lg_* (and mirrored by the device path)."""
    for a in (initial_mean, initial_covariance, transition_covariance, likelihood_matrix, likelihood_covariance):
        if dim is None and a is not None and np.ndim(a) > 0:
            dim = np.shape(a)[-1]
    d = int(dim)
    m0 = np.zeros(d) if initial_mean is None else np.asarray(initial_mean, np.float64).reshape(d)
    S0 = np.eye(d) if initial_covariance is None else _mat(initial_covariance, d)
    F = np.eye(d) if transition_matrix is None else _mat(transition_matrix, d)
    Q = np.eye(d) if transition_covariance is None else _mat(transition_covariance, d)
    H = np.eye(d) if likelihood_matrix is None else _mat(likelihood_matrix, d)
    dy = H.shape[0]
    R = np.eye(dy) if likelihood_covariance is None else _mat(likelihood_covariance, dy)
    LR = np.linalg.cholesky(R)
    P = np.linalg.inv(LR)
    det_prec = 1.0 / np.linalg.det(R)
    f32 = lambda a: np.ascontiguousarray(a, np.float32)
    return dict(d=d, dy=dy, F=f32(F), Lq=f32(np.linalg.cholesky(Q)), H=f32(H), P=f32(P),
                c=np.float32((dy * LOG2PI - np.log(det_prec)) / 2.0), C0=f32(np.linalg.cholesky(S0)), m0=f32(m0),
                LR=f32(LR), Q=Q, R=R, S0=S0, F64=F, H64=H, m064=m0)


def opt_params(initial_mean=None, initial_covariance=None, transition_matrix=None, transition_covariance=None,
               likelihood_matrix=None, likelihood_covariance=None, dim=None):
    """Optimal-proposal constants (nonlinear_gaussian.py:154-184) for f(x) = F x."""
    p = lg_params(initial_mean, initial_covariance, transition_matrix, transition_covariance, likelihood_matrix,
                  likelihood_covariance, dim)
    S0, Q, R, H = p["S0"], p["Q"], p["R"], p["H64"]
    C0 = np.linalg.cholesky(S0)
    init_prec_sqrt = np.linalg.inv(C0)
    Lq = np.linalg.cholesky(Q)
    LR = np.linalg.cholesky(R)
    lik_prec_sqrt = np.linalg.inv(LR)

    def kalman_gain(cov_sqrt, inv_mat=None):
        if inv_mat is None:
            hc = H @ cov_sqrt
            inv_mat = np.linalg.inv(hc @ hc.T + LR @ LR.T)
        return cov_sqrt @ cov_sqrt.T @ H.T @ inv_mat

    K0 = kalman_gain(C0)
    a = H.T @ lik_prec_sqrt
    init_cond_prec = init_prec_sqrt @ init_prec_sqrt + a @ a.T
    C0c = np.linalg.inv(np.linalg.cholesky(init_cond_prec))
    hl = H @ Lq
    weight_precision = np.linalg.inv(hl @ hl.T + LR @ LR.T)
    K = kalman_gain(Lq, weight_precision)
    prop_cov = Q - K @ H @ Q
    S = np.linalg.cholesky(prop_cov)
    W = np.linalg.cholesky(weight_precision)
    wdet = np.linalg.det(weight_precision)
    f32 = lambda a: np.ascontiguousarray(a, np.float32)
    dy = H.shape[0]
    return dict(d=p["d"], dy=dy, F=p["F"], H=p["H"], K=f32(K), S=f32(S), W=f32(W),
                cw=np.float32((dy * LOG2PI - np.log(wdet)) / 2.0), K0=f32(K0), C0c=f32(C0c), m0=p["m0"])


def sv_params(phi=0.95, sigma=0.3, likelihood_variance=1.0, initial_variance=None, initial_mean=0.0, dt=1.0):
    """Scalar stochastic-volatility constants (d = 1)."""
    if initial_variance is None:
        initial_variance = sigma ** 2 / (1.0 - phi ** 2)
    r2 = 1.0 / likelihood_variance
    return dict(phi=np.float32(phi), bsig=np.float32(np.float32(sigma) * np.float32(np.sqrt(dt))),
                r2=np.float32(r2), cB=np.float32(0.5 * (LOG2PI - np.log(np.float32(r2)))),
                c0=np.float32(np.sqrt(initial_variance)), m0=np.float32(initial_mean),
                sqrtR=np.float32(np.sqrt(likelihood_variance)))


def svd_params(initial_mean=None, initial_covariance=None, transition_matrix=None, transition_covariance=None,
               likelihood_covariance_diag=None, dim=None):
    """float32 constants of the d-dimensional stochastic-volatility model
    (stochastic_volatility.py:25-108, diagonal likelihood covariance): A, Lq = chol(Q),
    C0 = chol(initial_covariance), m0, r2 = 1 / R (R = likelihood_covariance_diag) and
    cB = (d log 2 pi - sum log r2) / 2."""
    for a in (initial_mean, initial_covariance, transition_matrix, transition_covariance, likelihood_covariance_diag):
        if dim is None and a is not None and np.ndim(a) > 0:
            dim = np.shape(a)[-1]
    d = int(dim)
    m0 = np.zeros(d) if initial_mean is None else np.asarray(initial_mean, np.float64).reshape(d)
    S0 = np.eye(d) if initial_covariance is None else _mat(initial_covariance, d)
    A = np.eye(d) if transition_matrix is None else _mat(transition_matrix, d)
    Q = np.eye(d) if transition_covariance is None else _mat(transition_covariance, d)
    R = np.ones(d) if likelihood_covariance_diag is None else np.asarray(likelihood_covariance_diag, np.float64)
    R = np.diag(R) if R.ndim == 2 else R.reshape(d)
    f32 = lambda a: np.ascontiguousarray(a, np.float32)
    r2 = f32(1.0 / R)
    return dict(d=d, A=f32(A), Lq=f32(np.linalg.cholesky(Q)), C0=f32(np.linalg.cholesky(S0)), m0=f32(m0), r2=r2,
                cB=np.float32(0.5 * (d * LOG2PI - np.sum(np.log(r2.astype(np.float64))))), sqrtR=f32(np.sqrt(R)),
                Q=Q, R=R, S0=S0, A64=A)


def simulate_svd(p, t, key):
    """StateSpaceModel.simulate (ssm.py:138-163) for the d-dimensional stochastic-volatility
    model, float32 host arithmetic: x_0 = C0 e + m0, x_t = A x_{t-1} + (Lq e) sqrt(dt),
    y_t = sqrt(R) exp(x_t / 2) e'."""
    from . import split, normal
    t = np.asarray(t, np.float32).reshape(-1)
    T, d = t.size, p["d"]
    keys = split(key, 2 * T)
    f = np.float32
    x = np.empty((T, d), np.float32)
    y = np.empty((T, d), np.float32)
    for i in range(T):
        e = normal(keys[i], d)
        if i == 0:
            x[0] = (p["C0"] @ e).astype(np.float32) + p["m0"]
        else:
            sdt = f(np.sqrt(f(t[i] - t[i - 1])))
            x[i] = (p["A"] @ x[i - 1]).astype(np.float32) + ((p["Lq"] @ e).astype(np.float32) * sdt)
        ey = normal(keys[T + i], d)
        y[i] = (p["sqrtR"] * np.exp(f(0.5) * x[i]).astype(np.float32) * ey).astype(np.float32)
    return x, y


def simulate_lg(p, T, key):
    """StateSpaceModel.simulate (ssm.py:138-163) for the linear-Gaussian model, float32."""
    keys = split(key, 2 * T)
    d, dy = p["d"], p["dy"]
    x = np.empty((T, d), np.float32)
    y = np.empty((T, dy), np.float32)
    e = normal(keys[0], (d,))
    x[0] = (p["C0"] @ e).astype(np.float32) + p["m0"]
    for t in range(1, T):
        e = normal(keys[t], (d,))
        x[t] = (p["F"] @ x[t - 1]).astype(np.float32) + (p["Lq"] @ e).astype(np.float32)
    for t in range(T):
        e = normal(keys[T + t], (dy,))
        y[t] = (p["H"] @ x[t]).astype(np.float32) + (p["LR"] @ e).astype(np.float32)
    return x, y


def simulate_sv(p, T, key):
    """simulate for the scalar stochastic-volatility model."""
    keys = split(key, 2 * T)
    x = np.empty(T, np.float32)
    y = np.empty(T, np.float32)
    x[0] = normal(keys[0], (1,))[0] * p["c0"] + p["m0"]
    for t in range(1, T):
        x[t] = x[t - 1] * p["phi"] + normal(keys[t], (1,))[0] * p["bsig"]
    for t in range(T):
        y[t] = p["sqrtR"] * np.exp(np.float32(0.5) * x[t]) * normal(keys[T + t], (1,))[0]
    return x, y


def random_stable_matrix(d, seed, lo=0.5, hi=0.95):
    """Seeded QR of a N(0,1) matrix times diag(U(lo, hi)): spectral radius <= hi."""
    rng = np.random.default_rng(seed)
    q, _ = np.linalg.qr(rng.standard_normal((d, d)))
    return q @ np.diag(rng.uniform(lo, hi, d))
