"""Oracle for the one-dimensional non-linear benchmark
(mocat/src/ssm/scenarios/nonlinear1d.py:16-80) checked against an independent
numpy float32 restatement of the bootstrap filter (filtering.py:255-324).  The
restatement uses the oracle's pinned RNG and resampling primitives only
(split / normal / resample_*), so what is checked here is the model arithmetic,
the key schedule and the ESS-triggered control flow.
"""
import math

import numpy as np
import pytest

import oracle as O

F = np.float32
PARAMS = dict(s0=F(math.sqrt(2.0)), tsd=F(math.sqrt(10.0)), lsd=F(1.0),
              c=F(F(np.log(F(2.0 * math.pi))) / F(2.0)))


def _drift(t):
    return F(8.0) * F(math.cos(float(F(1.2) * F(t))))


def _mean(x, drift):
    return (F(0.5) * x + (F(25.0) * x) / (F(1.0) + x * x)) + drift


def _potential(p, x, y):
    z = (F(y) - (x * x) / F(20.0)) / p["lsd"]
    return F(0.5) * (z * z) + p["c"]


def _normals(key, n):
    return np.array([O.normal(k, (1,))[0] for k in O.split(key, n)], np.float32)


def _numpy_run(p, n, key, y, t, thr, scheme):
    keys = O.lg_step_keys(key, len(y))
    with np.errstate(over="ignore"):
        x = _normals(keys[0], n) * p["s0"]
        lw = -_potential(p, x, y[0])
        xs, lws = [x], [lw]
        ess = O.lse_ess(lw)[3]
        res_flags = [False]
        for s in range(1, len(y)):
            kt = keys[s]
            res = F(ess) < F(thr) * F(n)
            if res:
                if scheme == "systematic":
                    anc, _ = O.resample_systematic(lw, O.systematic_u_bits(kt))
                elif scheme == "multinomial":
                    anc, _ = O.resample_multinomial(lw, kt)
                else:
                    anc = O.resample_gumbel(lw, kt)
                src, lres = x[anc], np.zeros(n, np.float32)
            else:
                src, lres = x, lw
            x = _mean(src, _drift(t[s - 1])) + _normals(kt, n) * p["tsd"]
            lw = lres - _potential(p, x, y[s])
            ess = O.lse_ess(lw)[3]
            xs.append(x)
            lws.append(lw)
            res_flags.append(bool(res))
    return np.stack(xs), np.stack(lws), np.array(res_flags)


@pytest.mark.parametrize("scheme", ["systematic", "multinomial", "categorical"])
def test_oracle_matches_numpy_restatement(scheme):
    rng = np.random.default_rng(0)
    T, n = 12, 257
    t = np.arange(T, dtype=np.float32)
    y = (rng.standard_normal(T) * 4 + 5).astype(np.float32)
    key = O.PRNGKey(7)
    xs, lws, res = _numpy_run(PARAMS, n, key, y, t, 0.7, scheme)
    ref = O.nl_run(PARAMS, n, key, y, t, ess_threshold=0.7, scheme=scheme, history=True)
    assert res.sum() > 0
    assert np.array_equal(ref["resampled"], res)
    assert np.array_equal(ref["value"], xs)
    assert np.array_equal(ref["log_weight"], lws)


def test_oracle_step_functions():
    rng = np.random.default_rng(1)
    n = 100
    key = O.PRNGKey(3)
    x0, lw0 = O.nl_init(PARAMS, n, key, F(2.5))
    assert np.array_equal(x0, _normals(key, n) * PARAMS["s0"])
    assert np.array_equal(lw0, -_potential(PARAMS, x0, 2.5))
    x0n, lw0n = O.nl_init(PARAMS, n, key)
    assert np.array_equal(x0n, x0) and not lw0n.any()
    kt = O.split(O.PRNGKey(4), 1)[0]
    anc = np.sort(rng.integers(0, n, n)).astype(np.int32)
    lwp = rng.standard_normal(n).astype(np.float32)
    x1, lw1 = O.nl_propagate(PARAMS, kt, 1.5, 7.0, x0, anc, lwp)
    want = _mean(x0[anc], _drift(7.0)) + _normals(kt, n) * PARAMS["tsd"]
    assert np.array_equal(x1, want)
    assert np.array_equal(lw1, lwp - _potential(PARAMS, want, 1.5))


def test_drift_matches_facade_formula():
    """the simulator's 8 cos(1.2 t) (numpy) equals the filters' (C) on the usual integer times"""
    from mocat_gb300.ssm import NonLinear1DBenchmark
    t = np.arange(0, 2000, dtype=np.float32)
    got = np.array([O.nl_drift(v) for v in t], np.float32)
    assert np.array_equal(got, NonLinear1DBenchmark.drift(t))
    assert np.array_equal(got, np.array([_drift(v) for v in t], np.float32))


def test_oracle_backward_pieces_match_numpy():
    """the oracle's non-linear transition potential and stitch follow the numpy arithmetic
    (Gumbel-max over split(key, M0)[j], first maximum)"""
    rng = np.random.default_rng(2)
    x0 = (rng.standard_normal(50) * 4).astype(np.float32)
    x1 = (rng.standard_normal(50) * 4).astype(np.float32)
    tp = 2.5
    want = []
    for a, b in zip(x0, x1):
        z = (b - _mean(a, _drift(tp))) / PARAMS["tsd"]
        want.append(F(0.5) * (z * z) + PARAMS["c"])
    assert np.array_equal(O.transition_potential_pairs_nl1d(PARAMS, x0, x1, tp), np.array(want, np.float32))
    lw1 = rng.standard_normal(50).astype(np.float32)
    key = O.PRNGKey(3)
    idx = O.stitch_nl1d(PARAMS, x0[:7], x1, lw1, tp, key)
    for j, k in enumerate(O.split(key, 7)):
        gum = O.gumbel(k, (50,))
        pot = O.transition_potential_pairs_nl1d(PARAMS, np.full(50, x0[j], np.float32), x1, tp)
        v = gum + (lw1 - pot)
        assert idx[j] == int(np.argmax(v))
