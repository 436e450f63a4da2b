"""ABC-SMC oracle (oracle.abc_lg_run): pinned against an independent pure-Python
float32 restatement of MetropolisedABCSMCSampler + RandomWalkABC on the ABC
LinearGaussian scenario (mocat/src/abc/smc.py:101-245, abc/mcmc.py:59-103,
mcmc/metropolis.py:48-70, transport/smc.py:61-100, sample.py:110-148) built on
the pinned RNG and resampling primitives, and checked with the reference's own
statistical test (tests/test_abc_linear_gaussian.py, TestMetSMCLinearGaussianABC).
"""
import math
from fractions import Fraction

import numpy as np
import pytest

import oracle as O

F = np.float32
PRIOR_COV = np.array([[1.0, -0.6, 0.5], [-0.6, 0.7, 0.1], [0.5, -0.6, 3.0]])
DATA = np.array([1.4, -2.5])
LIK_MAT = np.array([[1.0, 0.5, 0.], [0.2, 0.3, 1.5]])
LIK_COV = np.array([[0.02, -0.01], [-0.01, 0.05]])


def params(S0=PRIOR_COV, H=LIK_MAT, R=LIK_COV, data=DATA, m0=None):
    d = S0.shape[0]
    C0 = np.linalg.cholesky(S0)
    p = dict(m0=np.zeros(d) if m0 is None else m0, C0=C0, P0=np.linalg.inv(C0), H=H, L=np.linalg.cholesky(R),
             data=data, c0=np.float32((d * math.log(2 * math.pi) + math.log(np.linalg.det(S0))) / 2))
    return {k: (np.asarray(v, np.float32) if k != "c0" else v) for k, v in p.items()}


def posterior(S0=PRIOR_COV, H=LIK_MAT, R=LIK_COV, data=DATA):
    K = S0 @ H.T @ np.linalg.inv(H @ S0 @ H.T + R)
    return K @ data, S0 - K @ H @ S0


def _normals(key, n):
    return np.asarray(O.normal(key, (n,)), np.float32)


def _block_sum(part):
    """the GPU's fixed-order float64 reduction of 1024 thread partials"""
    res = []
    for w in range(32):
        v = list(part[32 * w:32 * w + 32])
        for off in (16, 8, 4, 2, 1):
            v = [v[l] + (v[l + off] if l + off < 32 else v[l]) for l in range(32)]
        res.append(v[0])
    s = res[0]
    for r in res[1:]:
        s += r
    return s


def _strided_sum(vals, mask=None):
    """thread t's float32 sum of its values t, t + 1024, ... in index order, then the float64 tree"""
    part = [np.float32(0.0)] * 1024
    for i, v in enumerate(vals):
        if mask is None or mask[i]:
            part[i % 1024] = np.float32(part[i % 1024] + np.float32(v))
    return _block_sum([float(q) for q in part])


def _round_f32(q):
    """the float32 nearest to the rational q (ties to even)"""
    f = F(float(q))
    cands = [np.nextafter(f, F(-np.inf)), f, np.nextafter(f, F(np.inf))]
    return min(cands, key=lambda c: (abs(Fraction(float(c)) - q), int(np.asarray(c, np.float32).view(np.uint32)) & 1))


def _fma(a, b, c):
    """fmaf: a b + c with one rounding"""
    return _round_f32(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c)))


def _prior_pot_exact(p, x):
    d = x.size
    diff = [F(x[j] - p["m0"][j]) for j in range(d)]
    quad = F(0)
    for k in range(d):
        v = F(diff[0] * p["P0"][0, k])
        for j in range(1, d):
            v = _fma(diff[j], p["P0"][j, k], v)
        quad = F(v * v) if k == 0 else _fma(v, v, quad)
    return F(F(F(0.5) * quad) + p["c0"])


def _sim_dist(p, x, key):
    d, dy = x.size, p["data"].size
    e = _normals(key, dy)
    s = F(0)
    for r in range(dy):
        hx = F(p["H"][r, 0] * x[0])
        for k in range(1, d):
            hx = _fma(p["H"][r, k], x[k], hx)
        le = F(p["L"][r, 0] * e[0])
        for k in range(1, dy):
            le = _fma(p["L"][r, k], e[k], le)
        dv = F(F(hx + le) - p["data"][r])
        s = F(dv * dv) if r == 0 else F(s + F(dv * dv))
    return F(np.sqrt(s))


def _split1(key, num, i):
    return O.split(key, num)[i]


def _adapt(p, N, iter_, ess_prev, x, dist, lw, alpha, retain, schedule, term_alpha, max_iter):
    alive_prev = lw > -np.inf
    am = F(_strided_sum(alpha, alive_prev) / alive_prev.sum())
    if schedule is not None:
        thr = F(schedule[min(iter_, len(schedule) - 1)])
    else:
        q = F(F(F(retain) * F(ess_prev)) / F(N))
        pos = F(q * F(N - 1))
        lo, hi = F(math.floor(pos)), F(math.ceil(pos))
        hw = F(pos - lo)
        lwt = F(F(1) - hw)
        srt = np.sort(dist.view(np.uint32)).view(np.float32)
        vlo, vhi = srt[int(min(max(lo, 0), N - 1))], srt[int(min(max(hi, 0), N - 1))]
        thr = F(F(vlo * lwt) + F(vhi * hw))
    lw = np.where(dist > thr, F(-np.inf), F(0)).astype(np.float32)
    alive = int((lw == 0).sum())
    ess = F(np.asarray(O.expf(O.logf(F(alive)))).reshape(()))
    d = x.shape[1]
    step = np.empty(d, np.float32)
    for j in range(d):
        mean = _strided_sum(x[:, j]) / N
        mf = np.float32(mean)
        var = _strided_sum([np.float32(np.float32(v - mf) * np.float32(v - mf)) for v in x[:, j]]) / (N - 1)
        step[j] = F(F(F(var) / F(d)) * F(5.6644))
    active = not (alive == 0 or am <= F(term_alpha) or iter_ >= max_iter)
    return thr, F(ess), am, lw, step, active


def python_abc(p, N, key, retain=0.9, schedule=None, mcmc_steps=1, max_iter=10000, resample_thr=0.5,
               term_alpha=0.01):
    d = p["m0"].size
    e, sub = O.split(key, 2)
    x = np.zeros((N, d), np.float32)
    pk = O.split(sub, N)
    for i in range(N):
        ev = _normals(pk[i], d)
        for r in range(d):
            v = F(p["C0"][r, 0] * ev[0])
            for k in range(1, d):
                v = _fma(p["C0"][r, k], ev[k], v)
            x[i, r] = F(p["m0"][r] + v)
    pp = np.array([_prior_pot_exact(p, x[i]) for i in range(N)], np.float32)
    f = _split1(e, N + 1, N)
    sk = O.split(f, N + 1)
    dist = np.array([_sim_dist(p, x[i], sk[i]) for i in range(N)], np.float32)
    key_e = sk[N]
    alpha = np.ones(N, np.float32)
    lw = np.zeros(N, np.float32)
    if schedule is not None:
        max_iter = len(schedule)
    thr, ess, am, lw, step, active = _adapt(p, N, 0, F(N), x, dist, lw, alpha, retain, schedule, term_alpha,
                                            max_iter)
    hist = dict(threshold=[thr], ess=[ess], alpha=[am], resampled=[False])
    it = 0
    while active:
        it += 1
        res = ess < F(F(resample_thr) * F(N))
        ka = O.split(key_e, N + 2)
        if res:
            anc, _ = O.resample_systematic(lw, O.systematic_u_bits(ka[N]))
            x, dist, pp, alpha = x[anc].copy(), dist[anc].copy(), pp[anc].copy(), alpha[anc].copy()
            lw = np.zeros(N, np.float32)
            ess = F(N)
        sq = np.sqrt(step).astype(np.float32)
        for i in range(N):
            if not lw[i] > -np.inf:
                continue
            k = ka[i]
            asum = F(0)
            for s in range(mcmc_steps):
                k = O.split(k, 2)[0]
                kn, k1, _, k3 = O.split(k, 4)
                ev = _normals(k1, d)
                xp = np.array([F(x[i, j] + F(sq[j] * ev[j])) for j in range(d)], np.float32)
                ppn = _prior_pot_exact(p, xp)
                dn = _sim_dist(p, xp, k3)
                with np.errstate(over="ignore", invalid="ignore"):
                    a = F(F(O.expf(F(pp[i] - ppn)).reshape(())) * (F(1) if dn < thr else F(0)))
                a = F(0) if a != a else min(F(1), a)
                k, ku = O.split(kn, 2)
                u = F(np.asarray(O.uniform(ku, ())).reshape(()))
                if u < a:
                    x[i], pp[i], dist[i] = xp, ppn, dn
                asum = a if s == 0 else F(asum + a)
            alpha[i] = F(asum / F(mcmc_steps))
        thr, ess, am, lw, step, active = _adapt(p, N, it, ess, x, dist, lw, alpha, retain, schedule, term_alpha,
                                                max_iter)
        key_e = ka[N + 1]
        for k_, v in (("threshold", thr), ("ess", ess), ("alpha", am), ("resampled", bool(res))):
            hist[k_].append(v)
    return dict(value=x, log_weight=lw, distance=dist, stepsize=step, iterations=it,
                **{k: np.asarray(v) for k, v in hist.items()})


@pytest.mark.parametrize("case", ["adaptive", "schedule", "steps2"])
def test_oracle_matches_python_restatement(case):
    p = params()
    kw = dict(adaptive=dict(retain=0.6, max_iter=4), schedule=dict(schedule=np.linspace(6, 1, 4)),
              steps2=dict(retain=0.7, mcmc_steps=2, max_iter=3))[case]
    N = 40
    key = O.PRNGKey(3)
    ref = python_abc(p, N, key, **kw)
    out = O.abc_lg_run(p, N, key, **kw)
    assert out["iterations"] == ref["iterations"]
    for k in ("threshold", "ess", "alpha", "resampled"):
        assert np.array_equal(out[k], ref[k]), k
    for k in ("value", "log_weight", "distance", "stepsize"):
        assert np.array_equal(out[k], ref[k]), k
    assert out["resampled"].any()


def test_closed_form_resampling_of_zero_weights():
    """systematic resampling of 0 / -inf weights: output k takes the alive particle of rank
    floor((k 2^23 + m) A / (n 2^23)) -- the GPU's closed form equals the fixed-point fill"""
    rng = np.random.default_rng(0)
    for n in (7, 64, 1000, 4097):
        lw = np.where(rng.random(n) < 0.3, 0.0, -np.inf).astype(np.float32)
        lw[rng.integers(n)] = 0.0
        alive = np.flatnonzero(lw == 0)
        for m in (0, 1, 4194303, 8388607, int(rng.integers(1 << 23))):
            anc, _ = O.resample_systematic(lw, m)
            k = np.arange(n, dtype=np.uint64)
            r = ((k << np.uint64(23)) + np.uint64(m)) * np.uint64(alive.size) // (np.uint64(n) << np.uint64(23))
            assert np.array_equal(anc, alive[r.astype(np.int64)])


@pytest.mark.parametrize("mode", ["adaptive", "schedule"])
def test_reference_statistical_check(mode):
    """TestMetSMCLinearGaussianABC: n = 1000, posterior mean and covariance (absolute
    error sums) within 3 of the Kalman posterior"""
    p = params()
    kw = dict(retain=0.8) if mode == "adaptive" else dict(schedule=np.linspace(10, 0.1, 10))
    out = O.abc_lg_run(p, 1000, O.PRNGKey(0), **kw)
    pm, pc = posterior()
    x = out["value"].astype(np.float64)
    assert np.abs(pm - x.mean(0)).sum() < 3.0
    assert np.abs(pc - np.cov(x.T)).sum() < 3.0
