"""Parameter gradients of the bootstrap particle filter: a hand-written adjoint of the
log Z estimate, and a consistent score estimate by Fisher's identity.

mocat obtains parameter gradients by jax.grad through
run_particle_filter_for_marginals (mocat/src/ssm/filtering.py:255-324); here the
gradient of the log Z estimate with the ancestors and resampling decisions
held fixed comes from one call into the C library (mgb_pf_lg_grad): a taped
forward filter, then a backward pass that recomputes segments of
``ckpt_every`` steps from checkpoints.

The model is TimeHomogenousLinearGaussian with the identity likelihood matrix
and diagonal transition / likelihood covariances; theta = (A, log diag Q,
log diag R).

* ``log_z_and_grad(ssm_scenario, y, random_key, n, ...)``: log Z and the three
  gradient blocks for a scenario object.
* ``log_z_and_score(...)``: the score d log p(y) / d theta by Fisher's identity,
  smoothed along the same filter by PaRIS (mgb_pf_lg_score); its error falls as n
  grows, which the fixed-ancestor gradient's does not.
* ``ParticleFilterLogZ``: a torch.autograd.Function whose forward is the
  filter's log Z and whose backward is the adjoint, so that
  ``particle_filter_log_z(A, log_q, log_r, ...)`` composes with torch code.
"""
import ctypes
import math

import numpy as np
import torch

from . import _dev, _lib
from ._lib import call
from .core import cdict
from .resampling import SCHEMES
from .ssm import RUN_LAUNCH_PER_STEP, TimeHomogenousLinearGaussian, _f32

LOG2PI = math.log(2.0 * math.pi)
SUPPORTED_D = (1, 2, 3, 4, 5, 8, 10)


def _diag_model(A, log_q, log_r, C0, m0):
    """(float32 arrays kept alive, C-ABI struct) for theta = (A, log q, log r)."""
    A = np.asarray(A, np.float64)
    d = A.shape[0]
    lq = np.asarray(log_q, np.float64).reshape(d)
    lr = np.asarray(log_r, np.float64).reshape(d)
    keep = dict(F=_f32(A), Lq=_f32(np.diag(np.exp(0.5 * lq))), H=_f32(np.eye(d)), P=_f32(np.diag(np.exp(-0.5 * lr))),
                C0=_f32(C0), m0=_f32(np.asarray(m0, np.float64).reshape(d)))
    c = np.float32(0.5 * (d * LOG2PI + lr.sum()))
    s = _lib.LGModel(d, d, keep["F"].ctypes.data, keep["Lq"].ctypes.data, keep["H"].ctypes.data,
                     keep["P"].ctypes.data, keep["C0"].ctypes.data, keep["m0"].ctypes.data, float(c))
    return keep, s


def _grad_call(s, d, y, key, n, ess_threshold, resampling, ckpt_every, persistent=True):
    dev = _dev.device()
    y2 = _dev.as_f32(y).reshape(-1, d).contiguous()
    T = y2.shape[0]
    key = _dev.as_key(key)
    if d not in SUPPORTED_D:
        raise NotImplementedError(f"adjoint for d = {d} not compiled (supported {SUPPORTED_D})")
    ws = _dev.workspace(_lib.lib().mgb_pf_lg_grad_workspace(n, T, d, ckpt_every), dev)
    logz = torch.empty(1, dtype=torch.float64, device=dev)
    grad = torch.empty(d * d + 2 * d, dtype=torch.float32, device=dev)
    res = torch.empty(T, dtype=torch.int32, device=dev)
    call("mgb_pf_lg_grad", ctypes.byref(s), n, T, _dev.ptr(key), _dev.ptr(y2), float(ess_threshold),
         SCHEMES[resampling] | (0 if persistent else RUN_LAUNCH_PER_STEP), int(ckpt_every), _dev.ptr(ws),
         ws.numel(), _dev.ptr(logz), _dev.ptr(grad),
         _dev.ptr(res), _dev.stream_ptr())
    return logz[0], grad, res


def log_z_and_grad(ssm_scenario, y, random_key, n, ess_threshold=0.5, resampling="systematic", ckpt_every=32,
                   persistent=True, estimator="pathwise", backward_draws=2, mcmc_steps=8, smoothing_key=None):
    """log Z of run_particle_filter_for_marginals(ssm_scenario, BootstrapFilter(), y, ..., n=n)
    and a gradient with respect to (transition_matrix, log diag transition_covariance,
    log diag likelihood_covariance).

    estimator="pathwise": the gradient of the log Z estimate with the ancestors and
    resampling decisions held fixed (what jax.grad through the reference's filter
    computes); it does not converge to the score d log p(y) / d theta as n grows,
    because it drops the resampling's dependence on theta.  persistent=False runs the
    taped forward pass one launch per phase instead of one persistent launch (same
    gradient; log Z within 1e-6, its float partial sums grouped differently).

    estimator="fisher": log_z_and_score (the consistent Fisher-identity estimate,
    smoothed by PaRIS), with backward_draws, mcmc_steps and smoothing_key as there.

    Returns cdict(log_z, grad_transition_matrix (d, d), grad_log_transition_covariance_diag (d,),
    grad_log_likelihood_covariance_diag (d,), resampled (T,))."""
    if estimator == "fisher":
        return log_z_and_score(ssm_scenario, y, random_key, n, backward_draws=backward_draws, mcmc_steps=mcmc_steps,
                               smoothing_key=smoothing_key, ess_threshold=ess_threshold, resampling=resampling)
    if estimator != "pathwise":
        raise ValueError(f"estimator must be 'pathwise' or 'fisher', not {estimator!r}")
    if not isinstance(ssm_scenario, TimeHomogenousLinearGaussian):
        raise NotImplementedError(f"{ssm_scenario.__class__.__name__}: no adjoint kernel for this model")
    _, s = ssm_scenario.derived()
    d = ssm_scenario.dim
    lz, g, res = _grad_call(s, d, y, random_key, n, ess_threshold, resampling, ckpt_every, persistent)
    return cdict(log_z=lz, grad_transition_matrix=g[:d * d].reshape(d, d),
                 grad_log_transition_covariance_diag=g[d * d:d * d + d],
                 grad_log_likelihood_covariance_diag=g[d * d + d:], resampled=res.bool())


def default_smoothing_key(random_key):
    """split(random_key, 3)[2]: the smoothing draws' key when none is given (the
    filter itself uses split(random_key, 2), so the streams do not overlap)."""
    from .random import split
    return split(_dev.as_key(random_key), 3)[2].contiguous()


def log_z_and_score(ssm_scenario, y, random_key, n, backward_draws=2, mcmc_steps=8, smoothing_key=None,
                    ess_threshold=0.5, resampling="systematic", return_draws=False):
    """The score d log p(y) / d theta, theta = (transition_matrix, log diag
    transition_covariance, log diag likelihood_covariance), by Fisher's identity along
    the bootstrap filter run_particle_filter_for_marginals(ssm_scenario, BootstrapFilter(),
    y, ..., random_key, n=n) (same particles and log Z), smoothed by PaRIS: every particle
    carries the smoothed complete-data score forward, averaged over `backward_draws` draws
    per step (its own ancestor, then an independent-Metropolis chain over the step's
    particles with `mcmc_steps` uniform proposals per draw).  The estimate is consistent:
    its error falls as n grows (about n^-1/2 once n is large), unlike the fixed-ancestor
    pathwise gradient.  One library call (mgb_pf_lg_score), no host synchronisation.

    smoothing_key seeds the backward draws (default: default_smoothing_key(random_key)).
    Returns cdict(log_z, grad_transition_matrix (d, d), grad_log_transition_covariance_diag (d,),
    grad_log_likelihood_covariance_diag (d,), resampled (T,), grad (d*d + 2d,)) and, with
    return_draws, draws (T, n, backward_draws): the source particle of every backward draw."""
    if not isinstance(ssm_scenario, TimeHomogenousLinearGaussian):
        raise NotImplementedError(f"{ssm_scenario.__class__.__name__}: no score kernel for this model")
    _, s = ssm_scenario.derived()
    d = ssm_scenario.dim
    if d not in SUPPORTED_D:
        raise NotImplementedError(f"score for d = {d} not compiled (supported {SUPPORTED_D})")
    dev = _dev.device()
    y2 = _dev.as_f32(y).reshape(-1, d).contiguous()
    T = y2.shape[0]
    key = _dev.as_key(random_key)
    skey = default_smoothing_key(key) if smoothing_key is None else _dev.as_key(smoothing_key)
    ws = _dev.workspace(_lib.lib().mgb_pf_lg_score_workspace(n, T, d), dev)
    logz = torch.empty(1, dtype=torch.float64, device=dev)
    grad = torch.empty(d * d + 2 * d, dtype=torch.float32, device=dev)
    res = torch.empty(T, dtype=torch.int32, device=dev)
    draws = torch.full((T, n, int(backward_draws)), -1, dtype=torch.int32, device=dev) if return_draws else None
    call("mgb_pf_lg_score", ctypes.byref(s), n, T, _dev.ptr(key), _dev.ptr(skey), _dev.ptr(y2), float(ess_threshold),
         SCHEMES[resampling], int(backward_draws), int(mcmc_steps), _dev.ptr(ws), ws.numel(), _dev.ptr(logz),
         _dev.ptr(grad), _dev.ptr(res), _dev.ptr(draws), _dev.stream_ptr())
    out = cdict(log_z=logz[0], grad_transition_matrix=grad[:d * d].reshape(d, d),
                grad_log_transition_covariance_diag=grad[d * d:d * d + d],
                grad_log_likelihood_covariance_diag=grad[d * d + d:], resampled=res.bool(), grad=grad)
    if return_draws:
        out.draws = draws
    return out


def log_z_and_grad_many(ssm_scenario, y, random_keys, n, ess_threshold=0.5, resampling="systematic",
                        ckpt_every=32, max_concurrent=8):
    """log_z_and_grad for B keys at once: each evaluation runs on its own CUDA stream,
    enqueued from its own host thread (the C library releases the interpreter lock),
    so the kernels of different evaluations overlap on the GPU.  The forward passes run
    one launch per phase (log_z_and_grad(..., persistent=False) gives the same values).

    Returns cdict(log_z (B,), grad (B, d*d + 2d)) in the layout of mgb_pf_lg_grad."""
    import threading
    if not isinstance(ssm_scenario, TimeHomogenousLinearGaussian):
        raise NotImplementedError(f"{ssm_scenario.__class__.__name__}: no adjoint kernel for this model")
    keys = np.asarray(random_keys.cpu() if isinstance(random_keys, torch.Tensor) else random_keys,
                      np.uint32).reshape(-1, 2)
    B, d = keys.shape[0], ssm_scenario.dim
    _, s = ssm_scenario.derived()
    dev = _dev.device()
    y2 = _dev.as_f32(y).reshape(-1, d).contiguous()
    T = y2.shape[0]
    nws = _lib.lib().mgb_pf_lg_grad_workspace(n, T, d, ckpt_every)
    logz = torch.empty(B, dtype=torch.float64, device=dev)
    grad = torch.empty((B, d * d + 2 * d), dtype=torch.float32, device=dev)
    keys_dev = torch.from_numpy(keys.view(np.int32).copy()).to(dev).view(torch.uint32)
    lanes = min(B, max_concurrent)
    ws = [_dev.workspace(nws, dev) for _ in range(lanes)]
    streams = [torch.cuda.Stream(dev) for _ in range(lanes)]
    cur = torch.cuda.current_stream(dev)
    for st in streams:
        st.wait_stream(cur)
    errors = []

    def lane(j):
        try:
            with torch.cuda.stream(streams[j]):
                for b in range(j, B, lanes):
                    # launch per phase: the concurrent gradients overlap on the GPU, which one
                    # whole-GPU persistent forward launch per gradient would prevent
                    call("mgb_pf_lg_grad", ctypes.byref(s), n, T, _dev.ptr(keys_dev[b]), _dev.ptr(y2),
                         float(ess_threshold), SCHEMES[resampling] | RUN_LAUNCH_PER_STEP, int(ckpt_every),
                         _dev.ptr(ws[j]), ws[j].numel(),
                         _dev.ptr(logz[b:b + 1]), _dev.ptr(grad[b]), None,
                         ctypes.c_void_p(streams[j].cuda_stream))
        except Exception as e:  # re-raised on the calling thread
            errors.append(e)

    threads = [threading.Thread(target=lane, args=(j,)) for j in range(lanes)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    if errors:
        raise errors[0]
    for st in streams:
        cur.wait_stream(st)
    return cdict(log_z=logz, grad=grad)


def log_z_and_score_batched(ssm_scenario, y, random_keys, n, backward_draws=2, mcmc_steps=8, smoothing_keys=None,
                            ess_threshold=0.5):
    """log_z_and_score for B filter keys in one library call (mgb_pf_lg_score_batch): every
    per-step kernel runs all B filters, one per grid row, so filters too small to fill the
    GPU share each launch.  Systematic resampling, even n; the same values as B calls of
    log_z_and_score (smoothing_keys default to default_smoothing_key of each filter key).

    Returns cdict(log_z (B,), grad (B, d*d + 2d)) in the layout of mgb_pf_lg_score."""
    if not isinstance(ssm_scenario, TimeHomogenousLinearGaussian):
        raise NotImplementedError(f"{ssm_scenario.__class__.__name__}: no score kernel for this model")
    d = ssm_scenario.dim
    if d not in SUPPORTED_D:
        raise NotImplementedError(f"score for d = {d} not compiled (supported {SUPPORTED_D})")
    _, s = ssm_scenario.derived()
    dev = _dev.device()
    keys = _dev.as_key(random_keys).reshape(-1, 2).contiguous()
    B = keys.shape[0]
    skeys = (torch.stack([default_smoothing_key(keys[b]) for b in range(B)]).contiguous() if smoothing_keys is None
             else _dev.as_key(smoothing_keys).reshape(-1, 2).contiguous())
    y2 = _dev.as_f32(y).reshape(-1, d).contiguous()
    T = y2.shape[0]
    ws = _dev.workspace(_lib.lib().mgb_pf_lg_score_batch_workspace(n, T, d, B), dev)
    logz = torch.empty(B, dtype=torch.float64, device=dev)
    grad = torch.empty((B, d * d + 2 * d), dtype=torch.float32, device=dev)
    call("mgb_pf_lg_score_batch", ctypes.byref(s), n, T, B, _dev.ptr(keys), _dev.ptr(skeys), _dev.ptr(y2),
         float(ess_threshold), int(backward_draws), int(mcmc_steps), _dev.ptr(ws), ws.numel(), _dev.ptr(logz),
         _dev.ptr(grad), _dev.stream_ptr())
    return cdict(log_z=logz, grad=grad)


def log_z_and_score_many(ssm_scenario, y, random_keys, n, backward_draws=2, mcmc_steps=8, smoothing_keys=None,
                         ess_threshold=0.5, resampling="systematic", max_concurrent=8):
    """log_z_and_score for B filter keys at once: each evaluation runs on its own CUDA
    stream, enqueued from its own host thread (the C library releases the interpreter
    lock), so the launches of different evaluations overlap on the GPU.  The same values
    as B calls of log_z_and_score (smoothing_keys default to default_smoothing_key of
    each filter key).

    Returns cdict(log_z (B,), grad (B, d*d + 2d)) in the layout of mgb_pf_lg_score."""
    import threading
    if not isinstance(ssm_scenario, TimeHomogenousLinearGaussian):
        raise NotImplementedError(f"{ssm_scenario.__class__.__name__}: no score kernel for this model")
    d = ssm_scenario.dim
    if d not in SUPPORTED_D:
        raise NotImplementedError(f"score for d = {d} not compiled (supported {SUPPORTED_D})")
    _, s = ssm_scenario.derived()
    dev = _dev.device()
    keys = _dev.as_key(random_keys).reshape(-1, 2).contiguous()
    B = keys.shape[0]
    skeys = (torch.stack([default_smoothing_key(keys[b]) for b in range(B)]) if smoothing_keys is None
             else _dev.as_key(smoothing_keys).reshape(-1, 2).contiguous())
    y2 = _dev.as_f32(y).reshape(-1, d).contiguous()
    T = y2.shape[0]
    nws = _lib.lib().mgb_pf_lg_score_workspace(n, T, d)
    logz = torch.empty(B, dtype=torch.float64, device=dev)
    grad = torch.empty((B, d * d + 2 * d), dtype=torch.float32, device=dev)
    lanes = min(B, max_concurrent)
    ws = [_dev.workspace(nws, dev) for _ in range(lanes)]
    streams = [torch.cuda.Stream(dev) for _ in range(lanes)]
    cur = torch.cuda.current_stream(dev)
    for st in streams:
        st.wait_stream(cur)
    errors = []

    def lane(j):
        try:
            for b in range(j, B, lanes):
                call("mgb_pf_lg_score", ctypes.byref(s), n, T, _dev.ptr(keys[b]), _dev.ptr(skeys[b]), _dev.ptr(y2),
                     float(ess_threshold), SCHEMES[resampling], int(backward_draws), int(mcmc_steps),
                     _dev.ptr(ws[j]), ws[j].numel(), _dev.ptr(logz[b:b + 1]), _dev.ptr(grad[b]), None, None,
                     ctypes.c_void_p(streams[j].cuda_stream))
        except Exception as e:  # re-raised on the calling thread
            errors.append(e)

    threads = [threading.Thread(target=lane, args=(j,)) for j in range(lanes)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    if errors:
        raise errors[0]
    for st in streams:
        cur.wait_stream(st)
    return cdict(log_z=logz, grad=grad)


class ParticleFilterLogZ(torch.autograd.Function):
    """forward: log Z of the bootstrap filter for theta = (A, log q, log r);
    backward: the adjoint (ancestors held fixed), computed in the same library call."""

    @staticmethod
    def forward(ctx, A, log_q, log_r, y, random_key, n, C0, m0, ess_threshold, resampling, ckpt_every):
        d = A.shape[0]
        _, s = _diag_model(A.detach().cpu().numpy(), log_q.detach().cpu().numpy(), log_r.detach().cpu().numpy(),
                           C0, m0)
        lz, g, _ = _grad_call(s, d, y, random_key, n, ess_threshold, resampling, ckpt_every)
        ctx.save_for_backward(g)
        ctx.d = d
        ctx.devs = (A.device, log_q.device, log_r.device)
        return lz.to(A.device)

    @staticmethod
    def backward(ctx, gout):
        (g,) = ctx.saved_tensors
        d = ctx.d
        gout = gout.to(g.device, torch.float32)
        gA = (gout * g[:d * d]).reshape(d, d).to(ctx.devs[0])
        gq = (gout * g[d * d:d * d + d]).to(ctx.devs[1])
        gr = (gout * g[d * d + d:]).to(ctx.devs[2])
        return gA, gq, gr, None, None, None, None, None, None, None, None


def particle_filter_log_z(A, log_q, log_r, y, random_key, n, initial_covariance=None, initial_mean=None,
                          ess_threshold=0.5, resampling="systematic", ckpt_every=32):
    """Differentiable log Z (torch) of the bootstrap filter for
    x_t = A x_{t-1} + N(0, diag(exp(log_q))), y_t = x_t + N(0, diag(exp(log_r)))."""
    d = A.shape[0]
    S0 = np.eye(d) if initial_covariance is None else np.asarray(initial_covariance, np.float64)
    C0 = np.linalg.cholesky(S0)
    m0 = np.zeros(d) if initial_mean is None else np.asarray(initial_mean, np.float64)
    return ParticleFilterLogZ.apply(A, log_q, log_r, y, random_key, int(n), C0, m0, float(ess_threshold), resampling,
                                    int(ckpt_every))
