"""Float64 restatement of the GPU tempered SMC sampler on logistic regression and the
Gaussian toy scenario -- test infrastructure only (the checker of mgb_smc_logreg_*,
never the product).

Follows mocat's MetropolisedSMCSampler (mocat/src/transport/smc.py:128-164,
193-226, 267-373) with Underdamped moves (any leapfrog_steps and friction; MALA for 1 and inf) or
RandomWalk moves (mocat/src/mcmc/standard_mcmc.py:20-153; utils.leapfrog mocat/src/utils.py:108-156;
Metropolis.correct mocat/src/mcmc/metropolis.py:48-70), regula-falsi
temperatures (utils.bisect mocat/src/utils.py:205-237) or a temperature schedule and the key schedule of
mocat.run (mocat/src/sample.py:110-148), with the same two choices as the GPU
sampler: systematic resampling (or, with resampling="categorical", the reference's
random.categorical) and no re-evaluation of the (deterministic) potentials at the
start of each MCMC block.  Draws come from the oracle's
jax.random restatement, so kernel and restatement see the same random numbers;
arithmetic is float64.

Also: exact log evidence of a d = 2 model by quadrature (the closed-form check
the reference's own SMC test makes, test_transport.py:49-55, for a model
without a closed form).
"""
import math

import numpy as np

import oracle as O


def softplus(z):
    return np.maximum(z, 0.0) + np.log1p(np.exp(-np.abs(z)))


def potential_grad(X, y, beta):
    """(lik (P,), grad (P, d)) in float64 for parameter rows beta (P, d)."""
    X = np.asarray(X, np.float64)
    y = np.asarray(y, np.float64)
    z = np.asarray(beta, np.float64) @ X.T
    lik = (softplus(z) - y * z).sum(1)
    r = 1.0 / (1.0 + np.exp(-z)) - y
    return lik, r @ X


def _split(key, num):
    return O.split(np.asarray(key, np.uint32), num)


def _logess(lw):
    m = np.max(lw)
    s1 = np.exp(lw - m).sum()
    s2 = np.exp(2 * (lw - m)).sum()
    return 2 * np.log(s1) - np.log(s2)


def _lse(lw):
    m = np.max(lw)
    return m + np.log(np.exp(lw - m).sum())


def _bisect(f, b0, b1, tol, max_iter):
    e0, e1 = f(b0), f(b1)
    incr = e1 > e0
    for _ in range(max_iter):
        if min(abs(e0), abs(e1)) < tol or (e0 < 0 and e1 < 0) or (e0 > 0 and e1 > 0):
            break
        npos = b0 - e0 * (b1 - b0) / (e1 - e0)
        ne = f(npos)
        if (ne > 0) if incr else (ne < 0):
            b1, e1 = npos, ne
        else:
            b0, e0 = npos, ne
    return b1 if abs(e1) < abs(e0) else b0


def gaussian_potential_grad(mean, prec_sqrt, beta):
    """toy_examples.Gaussian likelihood (mocat/src/scenarios/toy_examples.py:40-44) in float64:
    z = (x - mean) @ prec_sqrt^T, lik = |z|^2 / 2, grad = z @ prec_sqrt."""
    z = (np.asarray(beta, np.float64) - np.asarray(mean, np.float64)) @ np.asarray(prec_sqrt, np.float64).T
    return 0.5 * (z * z).sum(1), z @ np.asarray(prec_sqrt, np.float64)


def run(X, y, prior_scale, N, key, stepsize, mcmc_steps=5, retain=0.5, resample_thr=0.5, tol=1e-5,
        max_bisect=1000, max_temp=1.0, max_iter=1000, resampling="systematic"):
    """Logistic regression with MALA moves; see run_general."""
    return run_general(lambda b: potential_grad(X, y, b), np.asarray(X).shape[1], prior_scale, N, key, stepsize,
                       mcmc_steps=mcmc_steps, retain=retain, resample_thr=resample_thr, tol=tol,
                       max_bisect=max_bisect, max_temp=max_temp, max_iter=max_iter, resampling=resampling)


def run_general(lik_fn, d, prior_scale, N, key, stepsize, mcmc_steps=5, retain=0.5, resample_thr=0.5, tol=1e-5,
                max_bisect=1000, max_temp=1.0, max_iter=1000, move="underdamped", leapfrog_steps=1,
                friction=math.inf, sample_scale=None, schedule=None, resampling="systematic"):
    """lik_fn(beta (P, d)) -> (lik (P,), grad (P, d)).  move "underdamped" (leapfrog_steps, friction;
    standard_mcmc.py:72-153) or "random_walk" (standard_mcmc.py:20-64); schedule: the
    temperature_schedule without its leading 0 (max_temp, max_iter follow it).  Returns
    dict(temperature, log_norm_constant, ess, alpha, resampled (per iteration, entry 0 = after
    startup), value (N, d) final particles, accepts (list of (N,) bool per move))."""
    rw = move == "random_walk"
    if schedule is not None:
        schedule = np.asarray(schedule, np.float32)
        max_temp, max_iter = float(schedule[-1]), len(schedule)
    s2inv = np.float64(np.float32(1.0 / (prior_scale * prior_scale)))
    sscale = np.float32(prior_scale if sample_scale is None else sample_scale)
    msplit = 2 if rw else 3
    ek = _split(key, 2)
    e, sub = ek[0], ek[1]
    pk = _split(sub, N)
    beta = np.stack([(O.normal(pk[j], (d,)) * sscale).astype(np.float32) for j in range(N)])
    beta = beta.astype(np.float64)
    e = _split(e, 2 * N + 1)[2 * N]
    e = _split(e, msplit)[0]
    lik, glik = lik_fn(beta)
    ms = np.zeros((N, d))
    prior = lambda b: 0.5 * (b * b).sum(1) * s2inv
    gradU = lambda b, g, tau: b * s2inv + tau * g
    if not rw and math.isfinite(friction) and friction > 0:
        c1 = float(np.float32(math.exp(-friction * stepsize)))
        c2 = float(np.float32(math.sqrt(1.0 - math.exp(-2.0 * friction * stepsize))))
    else:
        c1, c2 = 0.0, 1.0

    def adapt(lw_res, ess_res, tau0, ell, it):
        if schedule is not None:
            tau1 = float(schedule[min(it, len(schedule) - 1)])
        else:
            target = math.log(ess_res * retain)
            f = lambda x: _logess(lw_res - (x - tau0) * ell) - target
            tau1 = _bisect(f, tau0, max_temp, tol, max_bisect)
        return tau1, lw_res - (tau1 - tau0) * ell

    tau, lw = adapt(np.zeros(N), float(N), 0.0, lik, 0)
    ess = math.exp(_logess(lw))
    logz = _lse(lw) - math.log(N)
    hist = dict(temperature=[tau], log_norm_constant=[logz], ess=[ess], alpha=[1.0], resampled=[False],
                accepts=[])
    it = 0
    while not (tau >= max_temp or it >= max_iter):
        res = ess <= resample_thr * N
        keys_all = _split(e, N + 2)
        pkeys = [_split(keys_all[j], msplit)[0] for j in range(N)]
        if res:
            if resampling == "categorical":  # random.categorical(key, lw, (N,)) (smc.py:61-71)
                anc = O.resample_gumbel(lw.astype(np.float32), keys_all[N])
            else:
                m23 = int(O.random_bits(keys_all[N], 1)[0]) >> 9
                anc = O.resample_systematic(lw.astype(np.float32), m23)
            beta, lik, glik, ms = beta[anc], lik[anc], glik[anc], ms[anc]
            lw_res, ess_res = np.zeros(N), float(N)
        else:
            lw_res, ess_res = lw, ess
        e = keys_all[N + 1]
        asum = np.zeros(N)
        for _ in range(mcmc_steps):
            U = prior(beta) + tau * lik
            if rw:
                noise = np.empty((N, d))
                for j in range(N):
                    kk = _split(pkeys[j], 3)
                    pkeys[j] = kk[0]
                    noise[j] = O.normal(kk[1], (d,))
                bn = beta + float(np.float32(math.sqrt(stepsize))) * noise
                ln, gn = lik_fn(bn)
                Un = prior(bn) + tau * ln
                with np.errstate(over="ignore", invalid="ignore"):
                    alpha = np.minimum(1.0, np.exp(-Un + U))
            else:
                mom = np.empty((N, d))
                for j in range(N):
                    kk = _split(pkeys[j], 2)
                    pkeys[j] = kk[0]
                    mom[j] = -ms[j] * c1 + c2 * O.normal(kk[1], (d,))
                p = mom
                bn, gn = beta, glik
                for _l in range(leapfrog_steps):
                    ph = p - stepsize / 2.0 * gradU(bn, gn, tau)
                    bn = bn + stepsize * ph
                    ln, gn = lik_fn(bn)
                    p = ph - stepsize / 2.0 * gradU(bn, gn, tau)
                Un = prior(bn) + tau * ln
                with np.errstate(over="ignore", invalid="ignore"):
                    alpha = np.minimum(1.0, np.exp(-Un + U - 0.5 * (p * p).sum(1) + 0.5 * (mom * mom).sum(1)))
            alpha = np.where(np.isnan(alpha), 0.0, alpha)
            u = np.empty(N)
            for j in range(N):
                k2 = pkeys[j] if rw else _split(pkeys[j], leapfrog_steps + 1)[0]
                kk = _split(k2, 2)
                pkeys[j] = kk[0]
                u[j] = O.uniform(kk[1], ())
            acc = u < alpha
            hist["accepts"].append(acc)
            beta = np.where(acc[:, None], bn, beta)
            lik = np.where(acc, ln, lik)
            glik = np.where(acc[:, None], gn, glik)
            if not rw:
                ms = np.where(acc[:, None], -p, mom)
            asum += alpha
        U = prior(beta) + tau * lik
        ell = (U - prior(beta)) / tau
        tau1, lw = adapt(lw_res, ess_res, tau, ell, it + 1)
        logz += _lse(lw) - (math.log(N) if res else _lse(lw_res))
        ess = math.exp(_logess(lw))
        tau = tau1
        it += 1
        for k, v in (("temperature", tau), ("log_norm_constant", logz), ("ess", ess),
                     ("alpha", asum.mean() / mcmc_steps), ("resampled", res)):
            hist[k].append(v)
    out = {k: np.asarray(v) for k, v in hist.items() if k != "accepts"}
    out["accepts"] = hist["accepts"]
    out["value"] = beta
    return out


def log_evidence_2d(X, y, prior_scale, half_width=None, grid=2001):
    """log integral of N(beta; 0, s^2 I) exp(-lik(beta)) d beta for d = 2 by a
    trapezoid grid around the posterior mode (float64)."""
    X = np.asarray(X, np.float64)
    assert X.shape[1] == 2
    # locate the mode by Newton steps
    b = np.zeros(2)
    for _ in range(50):
        z = X @ b
        s = 1.0 / (1.0 + np.exp(-z))
        g = X.T @ (s - y) + b / prior_scale ** 2
        Hm = (X * (s * (1 - s))[:, None]).T @ X + np.eye(2) / prior_scale ** 2
        b = b - np.linalg.solve(Hm, g)
    sd = np.sqrt(np.diag(np.linalg.inv(Hm)))
    hw = half_width if half_width is not None else 12.0 * sd
    g0 = np.linspace(b[0] - hw[0], b[0] + hw[0], grid)
    g1 = np.linspace(b[1] - hw[1], b[1] + hw[1], grid)
    B0, B1 = np.meshgrid(g0, g1, indexing="ij")
    pts = np.stack([B0.ravel(), B1.ravel()], 1)
    lik, _ = potential_grad(X, y, pts)
    logf = -lik - 0.5 * (pts * pts).sum(1) / prior_scale ** 2 - math.log(2 * math.pi * prior_scale ** 2)
    m = logf.max()
    w = np.exp(logf - m).reshape(grid, grid)
    integral = np.trapezoid(np.trapezoid(w, g1, axis=1), g0)
    return m + math.log(integral)
