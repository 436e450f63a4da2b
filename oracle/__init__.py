"""ORACLE -- test infrastructure only.

CPU restatement of mocat's particle-system step.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may import
this package, and only as the checker (or the timed CPU baseline).  The
product package ``mocat_gb300`` never imports it.

Layers:
  * ``oracle.c`` / ``oracle_rng.h`` (compiled by ``oracle/Makefile`` into
    ``oracle/_build/liboracle.so``): jax.random restatement, particle-filter
    step and run, resampling, LSE/ESS -- see the C headers for the
    reference file:line each function follows.
  * ``models.py``: parameter derivation of the reference's scenario classes
    (``reset_covariance``, the optimal-proposal ``startup``), float64 -> float32.
  * ``kalman.py``: float64 Kalman log-likelihood and its exact gradient.
  * ``potentials.py``: numpy ``gaussian_potential``.
  * ``smc.py``: numpy tempered SMC sampler.

Parity status: the threefry2x32 core is pinned by the Random123 known-answer
vectors and jax's documented ``split(PRNGKey(0))`` output; everything else is
pinned by the reference's own tests (gaussian_potential vs scipy, bisect,
leapfrog golden values, SMC log-normalising-constant closed form) and by the
float64 Kalman oracle.  Bit parity of normals against XLA's erf_inv/log is
unpinned (no JAX in this environment).
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
vp = ctypes.c_void_p
i64 = ctypes.c_int64


def build():
    """Compile the C restatement (idempotent)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


class _LGModel(ctypes.Structure):
    _fields_ = [("d", ctypes.c_int), ("dy", ctypes.c_int), ("F", vp), ("Lq", vp), ("H", vp), ("P", vp),
                ("c", ctypes.c_float), ("C0", vp), ("m0", vp)]


class _OptModel(ctypes.Structure):
    _fields_ = [("d", ctypes.c_int), ("dy", ctypes.c_int), ("F", vp), ("H", vp), ("K", vp), ("S", vp), ("W", vp),
                ("cw", ctypes.c_float), ("K0", vp), ("C0c", vp), ("m0", vp)]


class _SVModel(ctypes.Structure):
    _fields_ = [("phi", ctypes.c_float), ("bsig", ctypes.c_float), ("r2", ctypes.c_float),
                ("cB", ctypes.c_float), ("c0", ctypes.c_float), ("m0", ctypes.c_float)]


class _SVDModel(ctypes.Structure):
    _fields_ = [("d", ctypes.c_int), ("A", vp), ("Lq", vp), ("C0", vp), ("m0", vp), ("r2", vp),
                ("cB", ctypes.c_float)]


class _NLModel(ctypes.Structure):
    _fields_ = [("s0", ctypes.c_float), ("tsd", ctypes.c_float), ("lsd", ctypes.c_float), ("c", ctypes.c_float)]


class _ABCModel(ctypes.Structure):
    _fields_ = [("d", ctypes.c_int), ("dy", ctypes.c_int), ("m0", vp), ("C0", vp), ("P0", vp),
                ("c0", ctypes.c_float), ("H", vp), ("L", vp), ("data", vp)]


class _ABCConfig(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int), ("mcmc_steps", ctypes.c_int), ("max_iter", ctypes.c_int),
                ("n_schedule", ctypes.c_int), ("adapt_stepsize", ctypes.c_int), ("retain", ctypes.c_float),
                ("resample_thr", ctypes.c_float), ("term_alpha", ctypes.c_float), ("stepsize", ctypes.c_float),
                ("schedule", vp)]


class _GKModel(ctypes.Structure):
    _fields_ = [("d", ctypes.c_int), ("n_raw", ctypes.c_int), ("n_sum", ctypes.c_int), ("c", ctypes.c_float),
                ("lo", ctypes.c_float), ("hi", ctypes.c_float), ("buffer", ctypes.c_float), ("data", ctypes.c_void_p)]


class _FFBSiModel(ctypes.Structure):
    _fields_ = [("d", ctypes.c_int), ("F", ctypes.c_void_p), ("Pq", ctypes.c_void_p), ("cq", ctypes.c_float),
                ("nl", ctypes.c_int), ("tsd", ctypes.c_float), ("c", ctypes.c_float), ("phi", ctypes.c_float),
                ("pq", ctypes.c_float)]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        L.o_threefry_block.argtypes = [ctypes.c_uint32, ctypes.c_uint32, u32p, u32p, i64, u32p, u32p]
        for nm in ("o_random_bits", "o_split"):
            getattr(L, nm).argtypes = [u32p, i64, u32p]
        for nm in ("o_uniform", "o_normal", "o_exponential", "o_gumbel"):
            getattr(L, nm).argtypes = [u32p, i64, f32p]
        for nm in ("o_math_logf", "o_math_expf", "o_math_erfinvf"):
            getattr(L, nm).argtypes = [f32p, i64, f32p]
        L.o_lse_ess.argtypes = [f32p, i64, f64p]
        L.o_weight_shift.argtypes = [i64]
        L.o_weight_shift.restype = ctypes.c_int
        L.o_exp_shift.argtypes = [i64]
        L.o_exp_shift.restype = ctypes.c_int
        L.o_quantise.argtypes = [f32p, i64, np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")]
        L.o_quantise.restype = ctypes.c_int
        L.o_resample_systematic.argtypes = [f32p, i64, ctypes.c_uint32, i32p]
        L.o_resample_systematic.restype = ctypes.c_int
        L.o_resample_multinomial.argtypes = [f32p, i64, u32p, i32p]
        L.o_resample_multinomial.restype = ctypes.c_int
        L.o_resample_gumbel.argtypes = [f32p, i64, i64, u32p, i32p]
        L.o_lg_init.argtypes = [ctypes.POINTER(_LGModel), i64, u32p, vp, f32p, f32p]
        L.o_lg_propagate.argtypes = [ctypes.POINTER(_LGModel), i64, u32p, f32p, f32p, vp, vp, f32p, f32p]
        L.o_lg_run.argtypes = [ctypes.POINTER(_LGModel), i64, i64, u32p, f32p, ctypes.c_float, ctypes.c_int,
                               f32p, i32p, vp, vp]
        L.o_lg_run.restype = ctypes.c_double
        L.o_lg_run_tape.argtypes = [ctypes.POINTER(_LGModel), i64, i64, u32p, f32p, ctypes.c_float, ctypes.c_int,
                                    f32p, i32p, i32p]
        L.o_lg_run_tape.restype = ctypes.c_double
        L.o_lg_score.argtypes = [ctypes.POINTER(_LGModel), i64, i64, u32p, u32p, f32p, ctypes.c_float, ctypes.c_int,
                                 ctypes.c_int, ctypes.c_int, f64p, f32p, i32p, vp]
        L.o_lg_score.restype = ctypes.c_double
        L.o_lg_step_keys.argtypes = [u32p, i64, u32p]
        L.o_lg_normals.argtypes = [u32p, i64, ctypes.c_int, f32p]
        L.o_opt_init.argtypes = [ctypes.POINTER(_OptModel), i64, u32p, f32p, f32p, f32p]
        L.o_opt_propagate.argtypes = [ctypes.POINTER(_OptModel), i64, u32p, f32p, f32p, vp, vp, f32p, f32p]
        L.o_opt_run.argtypes = [ctypes.POINTER(_OptModel), i64, i64, u32p, f32p, ctypes.c_float, ctypes.c_int,
                                f32p, i32p, vp, vp]
        L.o_opt_run.restype = ctypes.c_double
        L.o_sv_run.argtypes = [ctypes.POINTER(_SVModel), i64, i64, u32p, f32p, ctypes.c_float, ctypes.c_int,
                               vp, vp]
        L.o_sv_run.restype = ctypes.c_double
        L.o_sv_run_hist.argtypes = [ctypes.POINTER(_SVModel), i64, i64, u32p, f32p, vp, ctypes.c_float, ctypes.c_int,
                                    f32p, i32p, vp, vp]
        L.o_sv_run_hist.restype = ctypes.c_double
        L.o_sv_batch.argtypes = [ctypes.POINTER(_SVModel), i64, i64p, i64p, i64p, f32p, u32p, ctypes.c_float,
                                 ctypes.c_int, f64p]
        L.o_svd_init.argtypes = [ctypes.POINTER(_SVDModel), i64, u32p, vp, f32p, f32p]
        L.o_svd_propagate.argtypes = [ctypes.POINTER(_SVDModel), i64, u32p, f32p, ctypes.c_float, f32p, vp, vp, f32p,
                                      f32p]
        L.o_svd_run_hist.argtypes = [ctypes.POINTER(_SVDModel), i64, i64, u32p, f32p, vp, ctypes.c_float,
                                     ctypes.c_int, f32p, i32p, vp, vp]
        L.o_svd_run_hist.restype = ctypes.c_double
        L.o_nl_drift.argtypes = [ctypes.c_float]
        L.o_nl_drift.restype = ctypes.c_float
        L.o_nl_init.argtypes = [ctypes.POINTER(_NLModel), i64, u32p, vp, f32p, f32p]
        L.o_nl_propagate.argtypes = [ctypes.POINTER(_NLModel), i64, u32p, ctypes.c_float, ctypes.c_float, f32p, vp,
                                     vp, f32p, f32p]
        L.o_nl_run.argtypes = [ctypes.POINTER(_NLModel), i64, i64, u32p, f32p, f32p, ctypes.c_float, ctypes.c_int,
                               f32p, i32p, vp, vp]
        L.o_nl_run.restype = ctypes.c_double
        L.o_abc_lg_run.argtypes = [ctypes.POINTER(_ABCModel), ctypes.POINTER(_ABCConfig), u32p, f32p, f32p, f32p,
                                   f32p, f32p, f32p, f32p, i32p]
        L.o_abc_lg_run.restype = ctypes.c_int
        L.o_abc_gk_run.argtypes = [ctypes.POINTER(_GKModel), ctypes.POINTER(_ABCConfig), u32p, f32p, f32p, f32p,
                                   f32p, f32p, f32p, f32p, i32p]
        L.o_abc_gk_run.restype = ctypes.c_int
        L.o_gk_simulate.argtypes = [ctypes.POINTER(_GKModel), i64, f32p, u32p, vp, vp]
        L.o_abc_mcmc_rm_lg.argtypes = [ctypes.POINTER(_ABCModel), ctypes.c_int, u32p, ctypes.c_float, ctypes.c_float,
                                       ctypes.c_float, f32p, f32p, f32p, f32p]
        L.o_abc_mcmc_rm_gk.argtypes = [ctypes.POINTER(_GKModel), ctypes.c_int, u32p, ctypes.c_float, ctypes.c_float,
                                       ctypes.c_float, f32p, f32p, f32p, f32p]
        L.o_abc_mcmc_lg.argtypes = [ctypes.POINTER(_ABCModel), ctypes.c_int, u32p, ctypes.c_float, ctypes.c_float,
                                    f32p, f32p, f32p, f32p]
        L.o_abc_mcmc_gk.argtypes = [ctypes.POINTER(_GKModel), ctypes.c_int, u32p, ctypes.c_float, ctypes.c_float,
                                    f32p, f32p, f32p, f32p]
        for nm, mt in (("o_abc_vanilla_lg", _ABCModel), ("o_abc_vanilla_gk", _GKModel)):
            getattr(L, nm).argtypes = [ctypes.POINTER(mt), ctypes.c_int, u32p, ctypes.c_float, ctypes.c_float, f32p,
                                       f32p, f32p, f32p]
            getattr(L, nm).restype = ctypes.c_float
        L.o_ffbsi_nl1d.argtypes = [ctypes.POINTER(_NLModel), i64, i64, i64, f32p, f32p, f32p, u32p, f32p, i32p]
        L.o_stitch_nl1d.argtypes = [ctypes.POINTER(_NLModel), i64, i64, f32p, f32p, f32p, ctypes.c_float, u32p, i32p]
        L.o_transition_potential_pairs_nl1d.argtypes = [ctypes.POINTER(_NLModel), i64, f32p, f32p, ctypes.c_float,
                                                        f32p]
        L.o_ffbsi_lg.argtypes = [ctypes.POINTER(_FFBSiModel), i64, i64, i64, f32p, f32p, u32p, f32p, i32p]
        L.o_stitch_lg.argtypes = [ctypes.POINTER(_FFBSiModel), i64, i64, f32p, f32p, f32p, u32p, i32p]
        L.o_transition_potential_pairs.argtypes = [ctypes.POINTER(_FFBSiModel), i64, f32p, f32p, f32p]
        fl, i32 = ctypes.c_float, ctypes.c_int32
        L.o_ffbsi_sv.argtypes = [fl, fl, i64, i64, i64, f32p, f32p, f32p, u32p, f32p, i32p]
        L.o_stitch_sv.argtypes = [fl, fl, i64, i64, f32p, f32p, f32p, fl, u32p, i32p]
        L.o_transition_potential_pairs_sv.argtypes = [fl, fl, i64, f32p, f32p, fl, f32p]
        L.o_ffbsi_rejection_sv.argtypes = [fl, fl, i64, i64, i64, f32p, f32p, f32p, u32p, i32, fl, fl, f32p, i32p,
                                           i64p]
        L.o_stitch_rejection_sv.argtypes = [fl, fl, i64, f32p, f32p, f32p, fl, u32p, i32, fl, fl, i32p]
        L.o_stitch_rejection_sv.restype = i64
        L.o_ffbsi_rejection_lg.argtypes = [ctypes.POINTER(_FFBSiModel), i64, i64, i64, f32p, f32p, u32p, i32, fl, fl,
                                           f32p, i32p, i64p]
        L.o_ffbsi_rejection_nl1d.argtypes = [ctypes.POINTER(_NLModel), i64, i64, i64, f32p, f32p, f32p, u32p, i32, fl,
                                             fl, f32p, i32p, i64p]
        L.o_stitch_rejection_lg.argtypes = [ctypes.POINTER(_FFBSiModel), i64, f32p, f32p, f32p, u32p, i32, fl, fl,
                                            i32p]
        L.o_stitch_rejection_lg.restype = i64
        L.o_stitch_rejection_nl1d.argtypes = [ctypes.POINTER(_NLModel), i64, f32p, f32p, f32p, fl, u32p, i32, fl, fl,
                                              i32p]
        L.o_stitch_rejection_nl1d.restype = i64
        L.o_num_threads.restype = ctypes.c_int
        L.o_set_num_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def _u32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint32))


def _f32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32))


def _ptr(a):
    return None if a is None else a.ctypes.data


# ----------------------------------------------------------------- RNG layer

def threefry2x32(key, c0, c1):
    c0, c1 = _u32(np.atleast_1d(c0)), _u32(np.atleast_1d(c1))
    r0, r1 = np.empty_like(c0), np.empty_like(c1)
    key = _u32(key)
    lib().o_threefry_block(int(key[0]), int(key[1]), c0, c1, c0.size, r0, r1)
    return r0, r1


def PRNGKey(seed):
    """jax.random.PRNGKey for a 32-bit seed: [seed >> 32 (= 0), seed & 0xffffffff]."""
    s = int(seed)
    return np.array([(s >> 32) & 0xFFFFFFFF if s >= 0 else 0, s & 0xFFFFFFFF], dtype=np.uint32)


def random_bits(key, n):
    out = np.empty(int(n), np.uint32)
    lib().o_random_bits(_u32(key), out.size, out)
    return out


def split(key, num=2):
    out = np.empty((int(num), 2), np.uint32)
    lib().o_split(_u32(key), int(num), out.reshape(-1))
    return out


def _draw(fn, key, shape):
    shape = tuple(np.atleast_1d(shape)) if shape != () else ()
    n = int(np.prod(shape)) if shape else 1
    out = np.empty(n, np.float32)
    getattr(lib(), fn)(_u32(key), n, out)
    return out.reshape(shape)


def uniform(key, shape=()):
    return _draw("o_uniform", key, shape)


def normal(key, shape=()):
    return _draw("o_normal", key, shape)


def exponential(key, shape=()):
    return _draw("o_exponential", key, shape)


def gumbel(key, shape=()):
    return _draw("o_gumbel", key, shape)


def logf(x):
    x = _f32(x)
    out = np.empty_like(x)
    lib().o_math_logf(x.reshape(-1), x.size, out.reshape(-1))
    return out


def expf(x):
    x = _f32(x)
    out = np.empty_like(x)
    lib().o_math_expf(x.reshape(-1), x.size, out.reshape(-1))
    return out


def erfinvf(x):
    x = _f32(x)
    out = np.empty_like(x)
    lib().o_math_erfinvf(x.reshape(-1), x.size, out.reshape(-1))
    return out


# ------------------------------------------------------ weights / resampling

def lse_ess(lw):
    """(max, logsumexp(lw), logsumexp(2 lw), ess) in float64 (metrics.py:69-78)."""
    out = np.empty(4, np.float64)
    lw = _f32(lw)
    lib().o_lse_ess(lw, lw.size, out)
    return out


def quantise(lw):
    lw = _f32(lw)
    q = np.empty(lw.size, np.uint64)
    ok = lib().o_quantise(lw, lw.size, q)
    return q, bool(ok)


def weight_shift(n):
    return lib().o_weight_shift(int(n))


def systematic_u_bits(key):
    """23-bit mantissa m of u = uniform(key) = m 2^-23 (one draw, shape ())."""
    return int(random_bits(key, 1)[0]) >> 9


def resample_systematic(lw, m23):
    lw = _f32(lw)
    anc = np.empty(lw.size, np.int32)
    ok = lib().o_resample_systematic(lw, lw.size, int(m23), anc)
    return anc, bool(ok)


def resample_multinomial(lw, key):
    lw = _f32(lw)
    anc = np.empty(lw.size, np.int32)
    ok = lib().o_resample_multinomial(lw, lw.size, _u32(key), anc)
    return anc, bool(ok)


def resample_gumbel(lw, key, nout=None):
    """random.categorical(key, lw, shape=(nout,)) -- mocat's _resample (filtering.py:196-199)."""
    lw = _f32(lw)
    nout = lw.size if nout is None else int(nout)
    anc = np.empty(nout, np.int32)
    lib().o_resample_gumbel(lw, lw.size, nout, _u32(key), anc)
    return anc


SCHEMES = {"systematic": 0, "multinomial": 1, "categorical": 2}


# ----------------------------------------------------------- particle filters

def _lg_struct(p):
    keep = {k: _f32(v) for k, v in p.items() if isinstance(v, np.ndarray)}
    s = _LGModel(int(p["d"]), int(p["dy"]), _ptr(keep["F"]), _ptr(keep["Lq"]), _ptr(keep["H"]), _ptr(keep["P"]),
                 float(p["c"]), _ptr(keep["C0"]), _ptr(keep["m0"]))
    return s, keep


def lg_init(params, n, key, y0):
    s, keep = _lg_struct(params)
    x = np.empty((n, params["d"]), np.float32)
    lw = np.empty(n, np.float32)
    y0 = None if y0 is None else _f32(y0)
    lib().o_lg_init(ctypes.byref(s), n, _u32(key), _ptr(y0), x.reshape(-1), lw)
    return x, lw


def lg_propagate(params, key_t, y, x_prev, anc=None, lw_prev=None):
    s, keep = _lg_struct(params)
    x_prev = _f32(x_prev)
    n = x_prev.shape[0]
    x_new = np.empty_like(x_prev)
    lw_new = np.empty(n, np.float32)
    anc = None if anc is None else np.ascontiguousarray(anc, dtype=np.int32)
    lw_prev = None if lw_prev is None else _f32(lw_prev)
    lib().o_lg_propagate(ctypes.byref(s), n, _u32(key_t), _f32(y), x_prev.reshape(-1), _ptr(anc), _ptr(lw_prev),
                         x_new.reshape(-1), lw_new)
    return x_new, lw_new


def lg_run(params, n, key, y, ess_threshold=0.5, scheme="systematic", history=False):
    s, keep = _lg_struct(params)
    y = _f32(y).reshape(len(y), -1)
    T = y.shape[0]
    ess = np.empty(T, np.float32)
    res = np.empty(T, np.int32)
    xh = np.empty((T, n, params["d"]), np.float32) if history else None
    lh = np.empty((T, n), np.float32) if history else None
    logZ = lib().o_lg_run(ctypes.byref(s), n, T, _u32(key), y.reshape(-1), float(ess_threshold), SCHEMES[scheme],
                          ess, res, _ptr(xh), _ptr(lh))
    return dict(log_z=logZ, ess=ess, resampled=res.astype(bool), value=xh, log_weight=lh)


def lg_run_tape(params, n, key, y, ess_threshold=0.5, scheme="systematic"):
    """lg_run returning also the ancestors of every resampled step (T, n) (other rows -1)."""
    s, keep = _lg_struct(params)
    y = _f32(y).reshape(len(y), -1)
    T = y.shape[0]
    ess = np.empty(T, np.float32)
    res = np.empty(T, np.int32)
    anc = np.full((T, n), -1, np.int32)
    logZ = lib().o_lg_run_tape(ctypes.byref(s), n, T, _u32(key), y.reshape(-1), float(ess_threshold),
                               SCHEMES[scheme], ess, res, anc.reshape(-1))
    return dict(log_z=logZ, ess=ess, resampled=res.astype(bool), ancestors=anc)


def lg_score(params, n, key, smoothing_key, y, ess_threshold=0.5, scheme="systematic", backward_draws=2,
             mcmc_steps=8, draws=False):
    """Fisher-identity score of the bootstrap filter of lg_run(params, n, key, y, ...),
    smoothed by PaRIS with independent-Metropolis backward draws (o_lg_score).
    params: H = I, diagonal Lq and P.  Returns dict(log_z, grad (d*d + 2d, float64:
    dF row-major, d/dlog q, d/dlog r), ess, resampled, draws (T, n, K) or None)."""
    s, keep = _lg_struct(params)
    y = _f32(y).reshape(len(y), -1)
    T = y.shape[0]
    d = params["d"]
    grad = np.empty(d * d + 2 * d, np.float64)
    ess = np.empty(T, np.float32)
    res = np.empty(T, np.int32)
    dr = np.full((T, n, backward_draws), -1, np.int32) if draws else None
    logZ = lib().o_lg_score(ctypes.byref(s), n, T, _u32(key), _u32(smoothing_key), y.reshape(-1), float(ess_threshold),
                            SCHEMES[scheme], int(backward_draws), int(mcmc_steps), grad, ess, res, _ptr(dr))
    return dict(log_z=logZ, grad=grad, ess=ess, resampled=res.astype(bool), draws=dr)


def lg_step_keys(key, T):
    """(T, 2): row 0 the initial draw's key, row t the key of step t (filtering.py:267-278)."""
    out = np.empty((T, 2), np.uint32)
    lib().o_lg_step_keys(_u32(key), T, out.reshape(-1))
    return out


def lg_normals(key_t, n, d):
    """(n, d) bootstrap draws normal(split(k_t, n)[i], (d,))."""
    e = np.empty((n, d), np.float32)
    lib().o_lg_normals(_u32(key_t), n, d, e.reshape(-1))
    return e


def _opt_struct(p):
    keep = {k: _f32(v) for k, v in p.items() if isinstance(v, np.ndarray)}
    s = _OptModel(int(p["d"]), int(p["dy"]), _ptr(keep["F"]), _ptr(keep["H"]), _ptr(keep["K"]), _ptr(keep["S"]),
                  _ptr(keep["W"]), float(p["cw"]), _ptr(keep["K0"]), _ptr(keep["C0c"]), _ptr(keep["m0"]))
    return s, keep


def opt_init(params, n, key, y0):
    """initial_sample of the optimal-proposal filter (nonlinear_gaussian.py:198-209); weights 0."""
    s, keep = _opt_struct(params)
    x = np.empty((n, params["d"]), np.float32)
    lw = np.empty(n, np.float32)
    lib().o_opt_init(ctypes.byref(s), n, _u32(key), _f32(y0), x.reshape(-1), lw)
    return x, lw


def opt_propagate(params, key_t, y, x_prev, anc=None, lw_prev=None):
    """propose_and_intermediate_weight_vectorised (nonlinear_gaussian.py:264-281)."""
    s, keep = _opt_struct(params)
    x_prev = _f32(x_prev)
    n = x_prev.shape[0]
    x_new = np.empty_like(x_prev)
    lw_new = np.empty(n, np.float32)
    anc = None if anc is None else np.ascontiguousarray(anc, dtype=np.int32)
    lw_prev = None if lw_prev is None else _f32(lw_prev)
    lib().o_opt_propagate(ctypes.byref(s), n, _u32(key_t), _f32(y), x_prev.reshape(-1), _ptr(anc), _ptr(lw_prev),
                          x_new.reshape(-1), lw_new)
    return x_new, lw_new


def opt_run(params, n, key, y, ess_threshold=0.5, scheme="systematic", history=False):
    s, keep = _opt_struct(params)
    y = _f32(y).reshape(len(y), -1)
    T = y.shape[0]
    ess = np.empty(T, np.float32)
    res = np.empty(T, np.int32)
    xh = np.empty((T, n, params["d"]), np.float32) if history else None
    lh = np.empty((T, n), np.float32) if history else None
    logZ = lib().o_opt_run(ctypes.byref(s), n, T, _u32(key), y.reshape(-1), float(ess_threshold), SCHEMES[scheme],
                           ess, res, _ptr(xh), _ptr(lh))
    return dict(log_z=logZ, ess=ess, resampled=res.astype(bool), value=xh, log_weight=lh)


def _sv_struct(p):
    return _SVModel(*(float(p[k]) for k in ("phi", "bsig", "r2", "cB", "c0", "m0")))


def sv_run(params, n, key, y, ess_threshold=0.5, scheme="multinomial"):
    s = _sv_struct(params)
    y = _f32(y).reshape(-1)
    T = y.size
    ess = np.empty(T, np.float32)
    res = np.empty(T, np.int32)
    logZ = lib().o_sv_run(ctypes.byref(s), n, T, _u32(key), y, float(ess_threshold), SCHEMES[scheme],
                          ess.ctypes.data, res.ctypes.data)
    return dict(log_z=logZ, ess=ess, resampled=res.astype(bool))


def sv_run_hist(params, n, key, y, t=None, ess_threshold=0.5, scheme="systematic"):
    """run_particle_filter_for_marginals on StochasticVolatility (dim 1) with the history; params
    bsig is transition_covariance_sqrt and t (T,) the times (None: unit steps)."""
    s = _sv_struct(params)
    y = _f32(y).reshape(-1)
    T = y.size
    tt = None if t is None else _f32(t).reshape(-1)
    ess = np.empty(T, np.float32)
    res = np.empty(T, np.int32)
    xh = np.empty((T, n), np.float32)
    lh = np.empty((T, n), np.float32)
    logZ = lib().o_sv_run_hist(ctypes.byref(s), n, T, _u32(key), y, _ptr(tt), float(ess_threshold),
                               SCHEMES[scheme], ess, res, _ptr(xh), _ptr(lh))
    return dict(log_z=logZ, ess=ess, resampled=res.astype(bool), value=xh, log_weight=lh)


def _svd_struct(p):
    keep = [np.ascontiguousarray(p[k], np.float32) for k in ("A", "Lq", "C0", "m0", "r2")]
    s = _SVDModel(int(p["d"]), *[a.ctypes.data for a in keep], float(p["cB"]))
    return s, keep


def svd_init(params, n, key, y0):
    """initiate_particles for the d-dimensional stochastic-volatility model: x (n, d), lw (n,)"""
    s, keep = _svd_struct(params)
    d = int(params["d"])
    x = np.empty((n, d), np.float32)
    lw = np.empty(n, np.float32)
    y0 = None if y0 is None else _f32(y0).reshape(d)
    lib().o_svd_init(ctypes.byref(s), n, _u32(key), _ptr(y0), x, lw)
    return x, lw


def svd_propagate(params, kt, y, dt, x_prev, anc=None, lw_prev=None):
    """one bootstrap step of the d-dimensional stochastic-volatility model (x particle-major)"""
    s, keep = _svd_struct(params)
    x_prev = _f32(x_prev)
    n, d = x_prev.shape
    anc = None if anc is None else np.ascontiguousarray(anc, np.int32)
    lw_prev = None if lw_prev is None else _f32(lw_prev)
    xn = np.empty((n, d), np.float32)
    ln = np.empty(n, np.float32)
    lib().o_svd_propagate(ctypes.byref(s), n, _u32(kt), _f32(y).reshape(d), float(dt), x_prev, _ptr(anc),
                          _ptr(lw_prev), xn, ln)
    return xn, ln


def svd_run_hist(params, n, key, y, t=None, ess_threshold=0.5, scheme="systematic"):
    """run_particle_filter_for_marginals on the d-dimensional stochastic-volatility model with
    the history: value (T, n, d), log_weight (T, n), ess, resampled, log_z"""
    s, keep = _svd_struct(params)
    d = int(params["d"])
    y = _f32(y).reshape(-1, d)
    T = y.shape[0]
    tt = None if t is None else _f32(t).reshape(-1)
    ess = np.empty(T, np.float32)
    res = np.empty(T, np.int32)
    xh = np.empty((T, n, d), np.float32)
    lh = np.empty((T, n), np.float32)
    logZ = lib().o_svd_run_hist(ctypes.byref(s), n, T, _u32(key), y, _ptr(tt), float(ess_threshold),
                                SCHEMES[scheme], ess, res, _ptr(xh), _ptr(lh))
    return dict(log_z=logZ, ess=ess, resampled=res.astype(bool), value=xh, log_weight=lh)


def sv_batch(params, n, T, y_off, y, keys, ess_threshold=0.5, scheme="multinomial"):
    s = _sv_struct(params)
    n = np.ascontiguousarray(n, np.int64)
    T = np.ascontiguousarray(T, np.int64)
    y_off = np.ascontiguousarray(y_off, np.int64)
    out = np.empty(n.size, np.float64)
    lib().o_sv_batch(ctypes.byref(s), n.size, n, T, y_off, _f32(y), _u32(keys).reshape(-1), float(ess_threshold),
                     SCHEMES[scheme], out)
    return out


def _nl_struct(p):
    return _NLModel(*(float(p[k]) for k in ("s0", "tsd", "lsd", "c")))


def nl_drift(t):
    """8 cos(1.2 t) as the filters compute it (nonlinear1d.py:41-46)."""
    return np.float32(lib().o_nl_drift(float(np.float32(t))))


def nl_init(params, n, key, y0=None):
    """initiate_particles on NonLinear1DBenchmark: (x (n,), lw (n,))."""
    x = np.empty(n, np.float32)
    lw = np.empty(n, np.float32)
    y0 = None if y0 is None else _f32(y0).reshape(1)
    lib().o_nl_init(ctypes.byref(_nl_struct(params)), n, _u32(key), _ptr(y0), x, lw)
    return x, lw


def nl_propagate(params, key_t, y, t_prev, x_prev, anc=None, lw_prev=None):
    """One bootstrap step from t_prev: (x_new (n,), lw_new (n,))."""
    x_prev = _f32(x_prev).reshape(-1)
    n = x_prev.size
    x_new = np.empty(n, np.float32)
    lw_new = np.empty(n, np.float32)
    anc = None if anc is None else np.ascontiguousarray(anc, np.int32)
    lw_prev = None if lw_prev is None else _f32(lw_prev)
    lib().o_nl_propagate(ctypes.byref(_nl_struct(params)), n, _u32(key_t), float(np.float32(y)),
                         float(np.float32(t_prev)), x_prev, _ptr(anc), _ptr(lw_prev), x_new, lw_new)
    return x_new, lw_new


def nl_run(params, n, key, y, t, ess_threshold=0.5, scheme="systematic", history=False):
    """run_particle_filter_for_marginals with BootstrapFilter on NonLinear1DBenchmark."""
    y = _f32(y).reshape(-1)
    t = _f32(t).reshape(-1)
    T = y.size
    ess = np.empty(T, np.float32)
    res = np.empty(T, np.int32)
    xh = np.empty((T, n), np.float32) if history else None
    lh = np.empty((T, n), np.float32) if history else None
    logZ = lib().o_nl_run(ctypes.byref(_nl_struct(params)), n, T, _u32(key), y, t, float(ess_threshold),
                          SCHEMES[scheme], ess, res, _ptr(xh), _ptr(lh))
    return dict(log_z=logZ, ess=ess, resampled=res.astype(bool), value=xh, log_weight=lh)


def ffbsi_nl1d(params, x_hist, lw_hist, t, key, M):
    """backward_simulation_full on NonLinear1DBenchmark: x_hist, lw_hist (T, N), t (T,)
    -> (samples (T, M), indices (T, M))."""
    x_hist, lw_hist, t = _f32(x_hist), _f32(lw_hist), _f32(t).reshape(-1)
    T, N = lw_hist.shape
    out = np.empty((T, M), np.float32)
    idx = np.empty((T, M), np.int32)
    lib().o_ffbsi_nl1d(ctypes.byref(_nl_struct(params)), T, N, M, x_hist.reshape(-1), lw_hist.reshape(-1), t,
                       _u32(key), out.reshape(-1), idx.reshape(-1))
    return out, idx


def stitch_nl1d(params, x0, x1, lw1, t_prev, key):
    """full_stitch on NonLinear1DBenchmark, x0 (M0,) at t_prev, x1 (M1,) -> indices (M0,)."""
    x0, x1, lw1 = _f32(x0).reshape(-1), _f32(x1).reshape(-1), _f32(lw1).reshape(-1)
    idx = np.empty(x0.size, np.int32)
    lib().o_stitch_nl1d(ctypes.byref(_nl_struct(params)), x0.size, x1.size, x0, x1, lw1, float(np.float32(t_prev)),
                        _u32(key), idx)
    return idx


def transition_potential_pairs_nl1d(params, x0, x1, t_prev):
    x0, x1 = _f32(x0).reshape(-1), _f32(x1).reshape(-1)
    out = np.empty(x0.size, np.float32)
    lib().o_transition_potential_pairs_nl1d(ctypes.byref(_nl_struct(params)), x0.size, x0, x1,
                                            float(np.float32(t_prev)), out)
    return out


def abc_lg_run(params, N, key, mcmc_steps=1, max_iter=10000, retain=0.9, resample_thr=0.5, term_alpha=0.01,
               schedule=None, stepsize=None):
    """mocat.run(LinearGaussian ABC scenario, MetropolisedABCSMCSampler(...), N, key) restated with
    systematic resampling (one posterior).  params: m0, C0, P0, c0, H, L, data (float32).
    stepsize=None: the default sampler's variance-scaled stepsize; a float: fixed.
    Returns dict(value (N, d), log_weight, distance, stepsize, threshold, ess, alpha, resampled
    (iterations + 1 entries), iterations)."""
    keep = {k: _f32(params[k]) for k in ("m0", "C0", "P0", "H", "L", "data")}
    d, dy = keep["m0"].size, keep["data"].size
    md = _ABCModel(d, dy, keep["m0"].ctypes.data, keep["C0"].ctypes.data, keep["P0"].ctypes.data,
                   float(params["c0"]), keep["H"].ctypes.data, keep["L"].ctypes.data, keep["data"].ctypes.data)
    sch = None if schedule is None else _f32(schedule)
    if sch is not None:
        max_iter = sch.size
    cf = _ABCConfig(N, mcmc_steps, max_iter, 0 if sch is None else sch.size, 1 if stepsize is None else 0,
                    float(retain), float(resample_thr), float(term_alpha), 0.0 if stepsize is None else float(stepsize),
                    _ptr(sch))
    x = np.empty((N, d), np.float32)
    lw = np.empty(N, np.float32)
    dist = np.empty(N, np.float32)
    st = np.empty(d, np.float32)
    H = max_iter + 1
    ht, he, ha = np.zeros(H, np.float32), np.zeros(H, np.float32), np.zeros(H, np.float32)
    hr = np.zeros(H, np.int32)
    it = lib().o_abc_lg_run(ctypes.byref(md), ctypes.byref(cf), _u32(key), x.reshape(-1), lw, dist, st, ht, he, ha,
                            hr)
    L = it + 1
    return dict(value=x, log_weight=lw, distance=dist, stepsize=st, threshold=ht[:L], ess=he[:L], alpha=ha[:L],
                resampled=hr[:L].astype(bool), iterations=it)


def _gk_struct(d, n_raw, n_sum, data=None, c=0.8, lo=0.0, hi=10.0, buffer=1e-5):
    keep = None if data is None else _f32(data).reshape(-1)
    return _GKModel(int(d), int(n_raw), int(n_sum), float(c), float(lo), float(hi), float(buffer), _ptr(keep)), keep


def gk_simulate(x, keys, d, n_raw=1000, n_sum=100, data=None, **kw):
    """thinned order statistics (P, n_sum) of g-and-k simulations of parameter rows x (P, d) with
    keys (P, 2); with data also the distances (P,)."""
    x = _f32(x).reshape(-1, d)
    P = x.shape[0]
    s, keep = _gk_struct(d, n_raw, n_sum, data, **kw)
    summ = np.empty((P, n_sum), np.float32)
    dist = np.empty(P, np.float32) if data is not None else None
    lib().o_gk_simulate(ctypes.byref(s), P, x.reshape(-1), _u32(keys).reshape(-1), _ptr(summ), _ptr(dist))
    return summ, dist


def _abc_lg_struct(params):
    keep = {k: _f32(params[k]) for k in ("m0", "C0", "P0", "H", "L", "data")}
    md = _ABCModel(keep["m0"].size, keep["data"].size, keep["m0"].ctypes.data, keep["C0"].ctypes.data,
                   keep["P0"].ctypes.data, float(params["c0"]), keep["H"].ctypes.data, keep["L"].ctypes.data,
                   keep["data"].ctypes.data)
    return md, keep


def abc_vanilla(n, key, threshold=np.inf, acceptance_rate=None, lg_params=None, gk=None):
    """mocat.run(scenario, VanillaABC(threshold | acceptance_rate), n, key) on the ABC linear-Gaussian
    scenario (lg_params as abc_lg_run) or a g-and-k one (gk = dict(d, data, n_raw, n_sum)).
    Returns dict(value (n, d), prior_potential, distance, log_weight, threshold)."""
    if gk is not None:
        s, keep = _gk_struct(gk["d"], gk.get("n_raw", 1000), gk.get("n_sum", 100), gk["data"])
        fn, d = lib().o_abc_vanilla_gk, gk["d"]
    else:
        s, keep = _abc_lg_struct(lg_params)
        fn, d = lib().o_abc_vanilla_lg, s.d
    x = np.empty((n, d), np.float32)
    pp, dist, lw = (np.empty(n, np.float32) for _ in range(3))
    thr = fn(ctypes.byref(s), n, _u32(key), float(threshold), -1.0 if acceptance_rate is None else float(acceptance_rate),
             x.reshape(-1), pp, dist, lw)
    return dict(value=x, prior_potential=pp, distance=dist, log_weight=lw, threshold=np.float32(thr))


def abc_mcmc_lg(params, n, key, stepsize, threshold):
    """mocat.run(LinearGaussian ABC scenario, RandomWalkABC(stepsize, threshold), n, key): one chain;
    returns dict(value (n, d), distance, prior_potential, alpha (n))."""
    md, keep = _abc_lg_struct(params)
    x = np.empty((n, md.d), np.float32)
    dist, pp, al = (np.empty(n, np.float32) for _ in range(3))
    lib().o_abc_mcmc_lg(ctypes.byref(md), n, _u32(key), float(stepsize), float(threshold), x.reshape(-1), dist, pp, al)
    return dict(value=x, distance=dist, prior_potential=pp, alpha=al)


def abc_mcmc_rm_lg(params, n, key, target=0.1, scale=1.0, neg_exp=2.0 / 3.0):
    """RandomWalkABC() with RMMetropolisDiagStepsize(rm_stepsize_scale=scale) on the ABC linear-Gaussian
    scenario, one chain: dict(value (n, d), alpha (n), threshold (n), stepsize (n, d))."""
    md, keep = _abc_lg_struct(params)
    d = md.d
    x, st = np.empty((n, d), np.float32), np.empty((n, d), np.float32)
    al, th = np.empty(n, np.float32), np.empty(n, np.float32)
    lib().o_abc_mcmc_rm_lg(ctypes.byref(md), n, _u32(key), float(target), float(scale), float(np.float32(neg_exp)),
                           x.reshape(-1), al, th, st.reshape(-1))
    return dict(value=x, alpha=al, threshold=th, stepsize=st)


def abc_mcmc_gk(d, data, n, key, stepsize, threshold, n_raw=1000, n_sum=100):
    """RandomWalkABC(stepsize, threshold) on a g-and-k scenario, one chain: dict(value (n, d),
    distance, prior_potential, alpha (n))."""
    s, keep = _gk_struct(d, n_raw, n_sum, data)
    x = np.empty((n, d), np.float32)
    dist, pp, al = (np.empty(n, np.float32) for _ in range(3))
    lib().o_abc_mcmc_gk(ctypes.byref(s), n, _u32(key), float(stepsize), float(threshold), x.reshape(-1), dist, pp, al)
    return dict(value=x, distance=dist, prior_potential=pp, alpha=al)


def abc_mcmc_rm_gk(d, data, n, key, target=0.1, scale=1.0, neg_exp=2.0 / 3.0, n_raw=1000, n_sum=100):
    """RandomWalkABC() with RMMetropolisDiagStepsize(rm_stepsize_scale=scale) on a g-and-k scenario
    (d = 4 or 1, data: the n_sum summary values), one chain: dict(value (n, d), alpha, threshold (n),
    stepsize (n, d))."""
    s, keep = _gk_struct(d, n_raw, n_sum, data)
    x, st = np.empty((n, d), np.float32), np.empty((n, d), np.float32)
    al, th = np.empty(n, np.float32), np.empty(n, np.float32)
    lib().o_abc_mcmc_rm_gk(ctypes.byref(s), n, _u32(key), float(target), float(scale), float(np.float32(neg_exp)),
                           x.reshape(-1), al, th, st.reshape(-1))
    return dict(value=x, alpha=al, threshold=th, stepsize=st)


def abc_gk_run(d, data, N, key, n_raw=1000, n_sum=100, mcmc_steps=1, max_iter=10000, retain=0.9, resample_thr=0.5,
               term_alpha=0.01, schedule=None, stepsize=None):
    """mocat.run of MetropolisedABCSMCSampler on a g-and-k scenario (d = 4 or 1), one posterior;
    returns as abc_lg_run."""
    s, keep = _gk_struct(d, n_raw, n_sum, data)
    sch = None if schedule is None else _f32(schedule)
    if sch is not None:
        max_iter = sch.size
    cf = _ABCConfig(N, mcmc_steps, max_iter, 0 if sch is None else sch.size, 1 if stepsize is None else 0,
                    float(retain), float(resample_thr), float(term_alpha), 0.0 if stepsize is None else float(stepsize),
                    _ptr(sch))
    x = np.empty((N, d), np.float32)
    lw = np.empty(N, np.float32)
    dist = np.empty(N, np.float32)
    st = np.empty(d, np.float32)
    H = max_iter + 1
    ht, he, ha = np.zeros(H, np.float32), np.zeros(H, np.float32), np.zeros(H, np.float32)
    hr = np.zeros(H, np.int32)
    it = lib().o_abc_gk_run(ctypes.byref(s), ctypes.byref(cf), _u32(key), x.reshape(-1), lw, dist, st, ht, he, ha, hr)
    L = it + 1
    return dict(value=x, log_weight=lw, distance=dist, stepsize=st, threshold=ht[:L], ess=he[:L], alpha=ha[:L],
                resampled=hr[:L].astype(bool), iterations=it)


def ffbsi_lg(F, Pq, cq, x_hist, lw_hist, key, M):
    """backward_simulation_full (backward.py:217-245) for a linear-Gaussian transition:
    x_hist (T, N, d), lw_hist (T, N) -> (samples (T, M, d), indices (T, M))."""
    F, Pq = _f32(F), _f32(Pq)
    x_hist = _f32(x_hist)
    T, N, d = x_hist.shape
    s = _FFBSiModel(d, _ptr(F), _ptr(Pq), float(cq))
    out = np.empty((T, M, d), np.float32)
    idx = np.empty((T, M), np.int32)
    lib().o_ffbsi_lg(ctypes.byref(s), T, N, M, x_hist.reshape(-1), _f32(lw_hist).reshape(-1), _u32(key),
                     out.reshape(-1), idx.reshape(-1))
    return out, idx


def stitch_lg(F, Pq, cq, x0, x1, lw1, key):
    """full_stitch (online_smoothing.py:21-41): x0 (M0, d), x1 (M1, d) -> indices (M0,)."""
    F, Pq, x0, x1 = _f32(F), _f32(Pq), _f32(x0), _f32(x1)
    s = _FFBSiModel(x0.shape[1], _ptr(F), _ptr(Pq), float(cq))
    idx = np.empty(x0.shape[0], np.int32)
    lib().o_stitch_lg(ctypes.byref(s), x0.shape[0], x1.shape[0], x0.reshape(-1), x1.reshape(-1), _f32(lw1), _u32(key),
                      idx)
    return idx


def transition_potential_pairs(F, Pq, cq, x0, x1):
    F, Pq, x0, x1 = _f32(F), _f32(Pq), _f32(x0), _f32(x1)
    s = _FFBSiModel(x0.shape[1], _ptr(F), _ptr(Pq), float(cq))
    out = np.empty(x0.shape[0], np.float32)
    lib().o_transition_potential_pairs(ctypes.byref(s), x0.shape[0], x0.reshape(-1), x1.reshape(-1), out)
    return out


def ffbsi_rejection_lg(F, Pq, cq, x_hist, lw_hist, key, M, maximum_rejections, init_bound_param=0.0,
                       bound_inflation=1.01):
    """backward_simulation_rejection (backward.py:172-214) for a linear-Gaussian transition:
    x_hist (T, N, d), lw_hist (T, N) -> (samples (T, M, d), indices (T, M), evals (T,) int64)."""
    F, Pq = _f32(F), _f32(Pq)
    x_hist = _f32(x_hist)
    T, N, d = x_hist.shape
    s = _FFBSiModel(d, _ptr(F), _ptr(Pq), float(cq))
    out = np.empty((T, M, d), np.float32)
    idx = np.empty((T, M), np.int32)
    ev = np.empty(T, np.int64)
    lib().o_ffbsi_rejection_lg(ctypes.byref(s), T, N, M, x_hist.reshape(-1), _f32(lw_hist).reshape(-1), _u32(key),
                               int(maximum_rejections), float(np.float32(init_bound_param)),
                               float(np.float32(bound_inflation)), out.reshape(-1), idx.reshape(-1), ev)
    return out, idx, ev


def ffbsi_rejection_nl1d(params, x_hist, lw_hist, t, key, M, maximum_rejections, init_bound_param=0.0,
                         bound_inflation=1.01):
    """backward_simulation_rejection on NonLinear1DBenchmark: x_hist, lw_hist (T, N), t (T,)
    -> (samples (T, M), indices (T, M), evals (T,) int64)."""
    x_hist, lw_hist, t = _f32(x_hist), _f32(lw_hist), _f32(t).reshape(-1)
    T, N = lw_hist.shape
    out = np.empty((T, M), np.float32)
    idx = np.empty((T, M), np.int32)
    ev = np.empty(T, np.int64)
    lib().o_ffbsi_rejection_nl1d(ctypes.byref(_nl_struct(params)), T, N, M, x_hist.reshape(-1), lw_hist.reshape(-1),
                                 t, _u32(key), int(maximum_rejections), float(np.float32(init_bound_param)),
                                 float(np.float32(bound_inflation)), out.reshape(-1), idx.reshape(-1), ev)
    return out, idx, ev


def stitch_rejection_lg(F, Pq, cq, x0, x1, lw1, key, maximum_rejections, init_bound_param=0.0, bound_inflation=1.01):
    """rejection_stitching (online_smoothing.py:129-175): x0, x1 (M, d) -> (indices (M,), evals)."""
    F, Pq, x0, x1 = _f32(F), _f32(Pq), _f32(x0), _f32(x1)
    s = _FFBSiModel(x0.shape[1], _ptr(F), _ptr(Pq), float(cq))
    idx = np.empty(x0.shape[0], np.int32)
    ev = lib().o_stitch_rejection_lg(ctypes.byref(s), x0.shape[0], x0.reshape(-1), x1.reshape(-1), _f32(lw1),
                                     _u32(key), int(maximum_rejections), float(np.float32(init_bound_param)),
                                     float(np.float32(bound_inflation)), idx)
    return idx, int(ev)


def stitch_rejection_nl1d(params, x0, x1, lw1, t_prev, key, maximum_rejections, init_bound_param=0.0,
                          bound_inflation=1.01):
    """rejection_stitching on NonLinear1DBenchmark, x0 (M,) at t_prev, x1 (M,) -> (indices, evals)."""
    x0, x1, lw1 = _f32(x0).reshape(-1), _f32(x1).reshape(-1), _f32(lw1).reshape(-1)
    idx = np.empty(x0.size, np.int32)
    ev = lib().o_stitch_rejection_nl1d(ctypes.byref(_nl_struct(params)), x0.size, x0, x1, lw1,
                                       float(np.float32(t_prev)), _u32(key), int(maximum_rejections),
                                       float(np.float32(init_bound_param)), float(np.float32(bound_inflation)), idx)
    return idx, int(ev)


def ffbsi_sv(phi, pq, x_hist, lw_hist, t, key, M, maximum_rejections=0, init_bound_param=0.0, bound_inflation=1.01):
    """backward_simulation on StochasticVolatility (dim 1): x_hist, lw_hist (T, N), t (T,) -> (samples
    (T, M), indices (T, M)[, evals (T,) for maximum_rejections > 0])."""
    x_hist, lw_hist, t = _f32(x_hist), _f32(lw_hist), _f32(t).reshape(-1)
    T, N = lw_hist.shape
    out = np.empty((T, M), np.float32)
    idx = np.empty((T, M), np.int32)
    if maximum_rejections > 0:
        ev = np.empty(T, np.int64)
        lib().o_ffbsi_rejection_sv(float(phi), float(pq), T, N, M, x_hist.reshape(-1), lw_hist.reshape(-1), t,
                                   _u32(key), int(maximum_rejections), float(np.float32(init_bound_param)),
                                   float(np.float32(bound_inflation)), out.reshape(-1), idx.reshape(-1), ev)
        return out, idx, ev
    lib().o_ffbsi_sv(float(phi), float(pq), T, N, M, x_hist.reshape(-1), lw_hist.reshape(-1), t, _u32(key),
                     out.reshape(-1), idx.reshape(-1))
    return out, idx


def stitch_sv(phi, pq, x0, x1, lw1, dt, key, maximum_rejections=0, init_bound_param=0.0, bound_inflation=1.01):
    """full_stitch / rejection_stitching on StochasticVolatility: x0 (M0,), x1 (M1,) -> indices
    [(, evals) for maximum_rejections > 0]"""
    x0, x1, lw1 = _f32(x0).reshape(-1), _f32(x1).reshape(-1), _f32(lw1).reshape(-1)
    idx = np.empty(x0.size, np.int32)
    if maximum_rejections > 0:
        ev = lib().o_stitch_rejection_sv(float(phi), float(pq), x0.size, x0, x1, lw1, float(np.float32(dt)),
                                         _u32(key), int(maximum_rejections), float(np.float32(init_bound_param)),
                                         float(np.float32(bound_inflation)), idx)
        return idx, int(ev)
    lib().o_stitch_sv(float(phi), float(pq), x0.size, x1.size, x0, x1, lw1, float(np.float32(dt)), _u32(key), idx)
    return idx


def transition_potential_pairs_sv(phi, pq, x0, x1, dt):
    x0, x1 = _f32(x0).reshape(-1), _f32(x1).reshape(-1)
    out = np.empty(x0.size, np.float32)
    lib().o_transition_potential_pairs_sv(float(phi), float(pq), x0.size, x0, x1, float(np.float32(dt)), out)
    return out


def num_threads():
    return lib().o_num_threads()


def set_num_threads(k):
    lib().o_set_num_threads(int(k))
