"""State-space models and particle filters with mocat's call signatures
(mocat/src/ssm/ssm.py, linear_gaussian/linear_gaussian.py,
scenarios/stochastic_volatility.py, filtering.py), running on the GPU.

Differences from the reference, by design:
  * ``resampling=`` selects the scheme; the default ``"systematic"`` is O(n).
    ``"categorical"`` reproduces the reference's ``random.categorical``
    (Gumbel-max, O(n^2)), ``"multinomial"`` is an O(n) inverse-CDF draw.
  * The filter output cdict additionally carries ``log_z`` (log-marginal
    likelihood from the log-weights) and ``resampled`` (per-step flags).
  * ``history=False`` keeps only the final particles (the (T, n, d) history
    of a 2^20-particle, 1000-step filter would be 42 GB).
"""
import ctypes
import math

import numpy as np
import torch

from . import _dev, _lib
from . import random as mrandom
from ._lib import call
from .core import cdict
from .metrics import ess_log_weight
from .resampling import SCHEMES, resample

LOG2PI = math.log(2.0 * math.pi)
RUN_LAUNCH_PER_STEP = 0x100  # MGB_RUN_LAUNCH_PER_STEP
LG_SUPPORTED = {(1, 1), (2, 1), (3, 1), (4, 1), (5, 1), (8, 1), (10, 1),
                (2, 2), (3, 3), (4, 4), (5, 5), (8, 8), (10, 10)}
LG_RUNTIME_MAX = 32  # bootstrap filter at other (d, dy): run-time-dimension kernels, d, dy <= 32


def _np(a):
    if isinstance(a, torch.Tensor):
        a = a.detach().cpu().numpy()
    return np.asarray(a, dtype=np.float64)


def _as_matrix(a, d):
    a = _np(a)
    if a.ndim == 0:
        return np.eye(d) * float(a)
    if a.ndim == 1:
        return np.diag(a)
    return a


def _f32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32))


class StateSpaceModel:
    """Plugin interface of mocat/src/ssm/ssm.py:18-81."""
    name = None
    dim = None
    dim_obs = None

    def __init__(self, name=None, **kwargs):
        if name is not None:
            self.name = name
        for k, v in kwargs.items():
            setattr(self, k, v)

    def __repr__(self):
        return f"mocat_gb300.StateSpaceModel.{self.__class__.__name__}"


class TimeHomogenousLinearGaussian(StateSpaceModel):
    """x_t ~ N(F x_{t-1}, Q), y_t ~ N(H x_t, R) (linear_gaussian.py:142-261).

    Cached derived quantities follow reset_covariance (mocat/src/utils.py:247-262):
    covariance square roots are Cholesky factors, precision square roots their
    inverses, precision determinants 1 / det(covariance).
    """
    name = "Time-homogenous Linear Gaussian"
    _PARAMS = ("initial_mean", "initial_covariance", "transition_matrix", "transition_covariance",
               "likelihood_matrix", "likelihood_covariance")

    def __init__(self, initial_mean=None, initial_covariance=None, transition_matrix=None,
                 transition_covariance=None, likelihood_matrix=None, likelihood_covariance=None, name=None, **kwargs):
        super().__init__(name=name, **kwargs)
        if "dim" not in kwargs:
            for a in (initial_mean, initial_covariance, transition_covariance, likelihood_matrix,
                      likelihood_covariance):
                if a is not None and np.ndim(_np(a)) > 0:
                    self.dim = _np(a).shape[-1]
                    break
        if self.dim is None:
            raise AttributeError(f"Could not find dimension for {self.__class__.__name__}")
        d = self.dim
        self.initial_mean = np.zeros(d) if initial_mean is None else _np(initial_mean).reshape(d)
        self.initial_covariance = np.eye(d) if initial_covariance is None else _as_matrix(initial_covariance, d)
        self.transition_matrix = np.eye(d) if transition_matrix is None else _as_matrix(transition_matrix, d)
        self.transition_covariance = (np.eye(d) if transition_covariance is None
                                      else _as_matrix(transition_covariance, d))
        self.likelihood_matrix = np.eye(d) if likelihood_matrix is None else _as_matrix(likelihood_matrix, d)
        self.dim_obs = self.likelihood_matrix.shape[0]
        self.likelihood_covariance = (np.eye(self.dim_obs) if likelihood_covariance is None
                                      else _as_matrix(likelihood_covariance, self.dim_obs))

    def __setattr__(self, key, value):
        self.__dict__[key] = value
        if key in self._PARAMS:
            self.__dict__.pop("_derived", None)
            self.__dict__.pop("_transition", None)

    # derived float32 parameters and the C-ABI model struct
    def derived(self):
        if "_derived" not in self.__dict__:
            R = self.likelihood_covariance
            LR = np.linalg.cholesky(R)
            det_prec = 1.0 / np.linalg.det(R)
            p = dict(d=self.dim, dy=self.dim_obs, F=_f32(self.transition_matrix),
                     Lq=_f32(np.linalg.cholesky(self.transition_covariance)), H=_f32(self.likelihood_matrix),
                     P=_f32(np.linalg.inv(LR)), c=np.float32((self.dim_obs * LOG2PI - np.log(det_prec)) / 2.0),
                     C0=_f32(np.linalg.cholesky(self.initial_covariance)), m0=_f32(self.initial_mean), LR=_f32(LR))
            s = _lib.LGModel(p["d"], p["dy"], p["F"].ctypes.data, p["Lq"].ctypes.data, p["H"].ctypes.data,
                             p["P"].ctypes.data, p["C0"].ctypes.data, p["m0"].ctypes.data, float(p["c"]))
            self.__dict__["_derived"] = (p, s)
        return self.__dict__["_derived"]

    def transition_function(self, x_previous, t_previous, t_new):
        """F x on the batch (n, d) (the mean of transition_sample, linear_gaussian.py:86-94)"""
        return x_previous @ torch.as_tensor(np.asarray(self.transition_matrix, np.float32), device=x_previous.device).T

    def gpu_supported(self):
        """(d, dy) has compiled kernels for every path, the gradients included"""
        return (self.dim, self.dim_obs) in LG_SUPPORTED

    def gpu_runtime_supported(self):
        """the bootstrap and optimal-proposal filters, the Kalman filter / smoothers and the
        particle smoothers (backward simulation, stitching, rejection sampling) run on the
        GPU: compiled kernels, or the run-time-dimension kernels (the same operations; one
        launch per phase for the bootstrap filter) for d, dy <= 32.  The gradients need a
        compiled pair (gpu_supported)."""
        return self.gpu_supported() or (self.dim <= LG_RUNTIME_MAX and self.dim_obs <= LG_RUNTIME_MAX)

    def simulate(self, t_all, random_key):
        """StateSpaceModel.simulate (ssm.py:138-163): split(key, 2T), first T keys drive
        the latent chain, the last T the observations.  Draws on the GPU."""
        p, _ = self.derived()
        T = len(t_all)
        keys = mrandom.split(random_key, 2 * T)
        d, dy = p["d"], p["dy"]
        ex = _normal_keys(keys[:T], d).cpu().numpy()
        ey = _normal_keys(keys[T:], dy).cpu().numpy()
        x = np.empty((T, d), np.float32)
        y = np.empty((T, dy), np.float32)
        x[0] = (p["C0"] @ ex[0]).astype(np.float32) + p["m0"]
        for t in range(1, T):
            x[t] = (p["F"] @ x[t - 1]).astype(np.float32) + (p["Lq"] @ ex[t]).astype(np.float32)
        for t in range(T):
            y[t] = (p["H"] @ x[t]).astype(np.float32) + (p["LR"] @ ey[t]).astype(np.float32)
        dev = _dev.device()
        return cdict(x=torch.from_numpy(x).to(dev), y=torch.from_numpy(y).to(dev),
                     t=torch.as_tensor(np.asarray(t_all), device=dev), name=f"{self.name} simulation")


class NonLinearGaussian(StateSpaceModel):
    """x_t ~ N(f(x_{t-1}, t_previous, t_new), Q), y_t ~ N(H x_t, R), Q, H, R time-homogeneous
    (mocat/src/ssm/nonlinear_gaussian.py:19-131).  Subclass it and implement
    transition_function(x_previous, t_previous, t_new) on the whole particle batch: x_previous
    is an (n, d) float32 CUDA tensor, the result (n, d).  The filters then run through the
    generic driver (the library's key, normal, logsumexp / ESS, resampling and gather kernels,
    the model's arithmetic in torch); OptimalNonLinearGaussianParticleFilter uses the
    transition function and the constants of its startup."""
    dim = None

    def __init__(self, initial_mean=None, initial_covariance=None, transition_covariance=None,
                 likelihood_matrix=None, likelihood_covariance=None, name=None):
        super().__init__(name=name)
        d = self.dim
        if d is None:
            for a in (initial_mean, initial_covariance, transition_covariance, likelihood_matrix,
                      likelihood_covariance):
                if a is not None and np.ndim(a) > 0:
                    d = int(np.shape(a)[-1])
                    break
        if d is None:
            raise AttributeError(f"Could not find dimension for {self.__class__.__name__}")
        self.dim = d
        self.initial_mean = np.zeros(d) if initial_mean is None else _np(initial_mean).reshape(d)
        self.initial_covariance = np.eye(d) if initial_covariance is None else _as_matrix(initial_covariance, d)
        self.transition_covariance = (np.eye(d) if transition_covariance is None
                                      else _as_matrix(transition_covariance, d))
        self.likelihood_matrix = np.eye(d) if likelihood_matrix is None else np.atleast_2d(_np(likelihood_matrix))
        self.dim_obs = self.likelihood_matrix.shape[0]
        self.likelihood_covariance = (np.eye(self.dim_obs) if likelihood_covariance is None
                                      else _as_matrix(likelihood_covariance, self.dim_obs))

    def __setattr__(self, key, value):
        self.__dict__[key] = value
        if key in ("initial_mean", "initial_covariance", "transition_covariance", "likelihood_matrix",
                   "likelihood_covariance"):
            self.__dict__.pop("_consts", None)

    def constants(self):
        """float32 CUDA tensors: m0, C0 = chol(initial_covariance), Lq = chol(Q), H,
        P = inv(chol(R)) (the likelihood precision square root) and c = (dy log 2 pi -
        log det(R^-1)) / 2, as reset_covariance (utils.py:247-262) derives them"""
        if "_consts" not in self.__dict__:
            dev = _dev.device()
            R = self.likelihood_covariance
            P = np.linalg.inv(np.linalg.cholesky(R))
            t = lambda a: torch.as_tensor(np.asarray(a, np.float32), device=dev)
            self.__dict__["_consts"] = dict(
                m0=t(self.initial_mean), C0=t(np.linalg.cholesky(self.initial_covariance)),
                Lq=t(np.linalg.cholesky(self.transition_covariance)), H=t(self.likelihood_matrix), P=t(P),
                c=float(np.float32((self.dim_obs * LOG2PI + np.log(np.linalg.det(R))) / 2.0)))
        return self.__dict__["_consts"]

    def transition_function(self, x_previous, t_previous, t_new):
        raise NotImplementedError(f"{self.__class__.__name__} nonlinear transition_function not implemented")

    def initial_sample(self, t, random_keys):
        """normal(key_i, (d,)) @ C0^T + m0 (nonlinear_gaussian.py:87-91)"""
        c = self.constants()
        return mrandom.normal_keys(random_keys, self.dim) @ c["C0"].T + c["m0"]

    def transition_sample(self, x_previous, t_previous, t_new, random_keys):
        """f(x) + normal(key_i, (d,)) @ transition_covariance_sqrt (:106-112; the reference
        multiplies by the Cholesky factor itself, not its transpose)"""
        c = self.constants()
        return (self.transition_function(x_previous, t_previous, t_new)
                + mrandom.normal_keys(random_keys, self.dim) @ c["Lq"])

    def likelihood_potential(self, x, y, t):
        """gaussian_potential(y, x H^T, sqrt_prec = P) = 0.5 |(y - H x) P|^2 + c (:114-120)"""
        c = self.constants()
        v = (_dev.as_f32(y).reshape(1, -1) - x @ c["H"].T) @ c["P"]
        return 0.5 * (v * v).sum(-1) + c["c"]


class StochasticVolatility(StateSpaceModel):
    """x_t ~ N(A x_{t-1}, Q dt), y_t ~ N(0, R exp(x_t)) elementwise
    (mocat/src/ssm/scenarios/stochastic_volatility.py:15-108).  dim = 1 runs the
    scalar kernels (single series, batches of many series, smoothers); dim 2..32 the
    bootstrap filter on run-time-dimension kernels.  likelihood_covariance_diag is the
    diagonal of R (a matrix argument is reduced to its diagonal); the reference's
    default, an identity matrix, drops the potential's normalising constant there,
    which only shifts log Z."""
    name = "Stochastic Volatility"
    _PARAMS = ("initial_mean", "initial_covariance", "transition_matrix", "transition_covariance",
               "likelihood_covariance_diag")

    def __init__(self, dim=1, initial_mean=None, initial_covariance=None, transition_matrix=None,
                 transition_covariance=None, likelihood_covariance_diag=None, name=None):
        super().__init__(name=name)
        self.dim = dim
        self.dim_obs = dim
        self.initial_mean = np.zeros(dim) if initial_mean is None else _np(initial_mean).reshape(dim)
        self.initial_covariance = np.eye(dim) if initial_covariance is None else _as_matrix(initial_covariance, dim)
        self.transition_matrix = np.eye(dim) if transition_matrix is None else _as_matrix(transition_matrix, dim)
        self.transition_covariance = (np.eye(dim) if transition_covariance is None
                                      else _as_matrix(transition_covariance, dim))
        lcd = np.ones(dim) if likelihood_covariance_diag is None else _np(likelihood_covariance_diag)
        self.likelihood_covariance_diag = np.diag(lcd) if lcd.ndim == 2 else lcd.reshape(dim)

    def __setattr__(self, key, value):
        self.__dict__[key] = value
        if key in self._PARAMS:
            self.__dict__.pop("_derived", None)

    def derived(self, dt=1.0):
        """float32 constants of the d = 1 kernels and the C-ABI struct:
        phi = A, bsig = sqrt(Q) sqrt(dt), r2 = 1 / R, cB = (log 2 pi - log r2) / 2,
        c0 = sqrt(initial_covariance), m0 = initial_mean.  dim > 1: the constants of the
        run-time-dimension kernels (mgb_svd_model): A, Lq = chol(Q), C0 = chol(initial
        covariance), m0, r2 = 1 / R, cB = (d log 2 pi - sum log r2) / 2."""
        if self.dim != 1:
            if "_derived" not in self.__dict__:
                d = self.dim
                f32 = lambda a: np.ascontiguousarray(a, np.float32)
                r2 = f32(1.0 / np.asarray(self.likelihood_covariance_diag, np.float64))
                p = dict(d=d, A=f32(self.transition_matrix), Lq=f32(np.linalg.cholesky(self.transition_covariance)),
                         C0=f32(np.linalg.cholesky(self.initial_covariance)), m0=f32(self.initial_mean), r2=r2,
                         cB=np.float32(0.5 * (d * LOG2PI - np.sum(np.log(r2.astype(np.float64))))),
                         sqrtR=f32(np.sqrt(self.likelihood_covariance_diag)))
                s = _lib.SVDModel(d, p["A"].ctypes.data, p["Lq"].ctypes.data, p["C0"].ctypes.data,
                                  p["m0"].ctypes.data, p["r2"].ctypes.data, float(p["cB"]))
                self.__dict__["_derived"] = (p, s)
            return self.__dict__["_derived"]
        if "_derived" not in self.__dict__ or self.__dict__["_derived"][0]["dt"] != dt:
            r2 = np.float32(1.0 / float(self.likelihood_covariance_diag[0]))
            p = dict(dt=dt, phi=np.float32(self.transition_matrix[0, 0]),
                     bsig=np.float32(np.float32(np.sqrt(self.transition_covariance[0, 0])) * np.float32(np.sqrt(dt))),
                     r2=r2, cB=np.float32(0.5 * (LOG2PI - np.log(r2))),
                     c0=np.float32(np.sqrt(self.initial_covariance[0, 0])), m0=np.float32(self.initial_mean[0]),
                     sqrtR=np.float32(np.sqrt(float(self.likelihood_covariance_diag[0]))))
            s = _lib.SVModel(*(float(p[k]) for k in ("phi", "bsig", "r2", "cB", "c0", "m0")))
            self.__dict__["_derived"] = (p, s)
        return self.__dict__["_derived"]

    def transition_constants(self):
        """(phi, pq) of the transition potential, float32: transition_matrix and
        transition_precision_sqrt = inv(chol(transition_covariance)) (utils.py:247-262)"""
        if self.dim != 1:
            raise NotImplementedError("StochasticVolatility: the smoothing kernels take dim = 1")
        f = np.float32
        return f(self.transition_matrix[0, 0]), f(f(1.0) / f(np.sqrt(f(self.transition_covariance[0, 0]))))

    def simulate(self, t_all, random_key):
        """StateSpaceModel.simulate (ssm.py:138-163) with this model's samplers
        (stochastic_volatility.py:71-108): x_0 = e c0 + m0, x_t = phi x_{t-1} + (e sqrt(Q))
        sqrt(t_t - t_{t-1}), y_t = sqrt(R) exp(x_t / 2) e; normals drawn on the GPU
        (dim > 1: x_0 = C0 e + m0, x_t = A x_{t-1} + (Lq e) sqrt(dt))."""
        if self.dim != 1:
            return self._simulate_d(t_all, random_key)
        p, _ = self.derived()
        f = np.float32
        t = np.asarray(t_all.cpu() if isinstance(t_all, torch.Tensor) else t_all, np.float32).reshape(-1)
        T = t.size
        keys = mrandom.split(random_key, 2 * T)
        ex = _normal_keys(keys[:T], 1).cpu().numpy()[:, 0]
        ey = _normal_keys(keys[T:], 1).cpu().numpy()[:, 0]
        sq = f(np.sqrt(f(self.transition_covariance[0, 0])))
        x = np.empty(T, np.float32)
        x[0] = f(ex[0] * p["c0"]) + p["m0"]
        for i in range(1, T):
            x[i] = f(x[i - 1] * p["phi"]) + f(f(ex[i] * sq) * f(np.sqrt(f(t[i] - t[i - 1]))))
        y = (f(p["sqrtR"]) * np.exp(f(0.5) * x).astype(np.float32) * ey).astype(np.float32)
        dev = _dev.device()
        return cdict(x=torch.from_numpy(x[:, None]).to(dev), y=torch.from_numpy(y[:, None]).to(dev),
                     t=torch.as_tensor(t, device=dev), name=f"{self.name} simulation")

    def _simulate_d(self, t_all, random_key):
        p, _ = self.derived()
        f = np.float32
        d = self.dim
        t = np.asarray(t_all.cpu() if isinstance(t_all, torch.Tensor) else t_all, np.float32).reshape(-1)
        T = t.size
        keys = mrandom.split(random_key, 2 * T)
        ex = _normal_keys(keys[:T], d).cpu().numpy()
        ey = _normal_keys(keys[T:], d).cpu().numpy()
        x = np.empty((T, d), np.float32)
        x[0] = (p["C0"] @ ex[0]).astype(np.float32) + p["m0"]
        for i in range(1, T):
            sdt = f(np.sqrt(f(t[i] - t[i - 1])))
            x[i] = (p["A"] @ x[i - 1]).astype(np.float32) + (p["Lq"] @ ex[i]).astype(np.float32) * sdt
        y = (p["sqrtR"] * np.exp(f(0.5) * x).astype(np.float32) * ey).astype(np.float32)
        dev = _dev.device()
        return cdict(x=torch.from_numpy(x).to(dev), y=torch.from_numpy(y).to(dev), t=torch.as_tensor(t, device=dev),
                     name=f"{self.name} simulation")


class NonLinear1DBenchmark(StateSpaceModel):
    """x_0 ~ N(0, initial_sd^2), x_t ~ N(0.5 x + 25 x / (1 + x^2) + 8 cos(1.2 t_prev), transition_sd^2),
    y_t ~ N(x_t^2 / 20, likelihood_sd^2) (mocat/src/ssm/scenarios/nonlinear1d.py:16-80).
    The likelihood potential's normaliser is log(2 pi) / 2 whatever likelihood_sd is, as in
    the reference (gaussian_potential of the standardised residual)."""
    name = "1D Non-linear Benchmark"
    dim = 1
    dim_obs = 1
    _PARAMS = ("initial_sd", "transition_sd", "likelihood_sd")

    def __init__(self, initial_sd=math.sqrt(2.0), transition_sd=math.sqrt(10.0), likelihood_sd=1.0, name=None):
        super().__init__(name=name)
        self.initial_sd = float(initial_sd)
        self.transition_sd = float(transition_sd)
        self.likelihood_sd = float(likelihood_sd)

    def __setattr__(self, key, value):
        self.__dict__[key] = value
        if key in self._PARAMS:
            self.__dict__.pop("_derived", None)

    def derived(self):
        if "_derived" not in self.__dict__:
            p = dict(s0=np.float32(self.initial_sd), tsd=np.float32(self.transition_sd),
                     lsd=np.float32(self.likelihood_sd),
                     c=np.float32(np.float32(np.log(np.float32(2.0 * math.pi))) / np.float32(2.0)))
            s = _lib.NL1DModel(float(p["s0"]), float(p["tsd"]), float(p["lsd"]), float(p["c"]))
            self.__dict__["_derived"] = (p, s)
        return self.__dict__["_derived"]

    def gpu_supported(self):
        return True

    @staticmethod
    def drift(t):
        """8 cos(1.2 t) as the kernels form it: 8 * float32(cos(float64(1.2f * t)))."""
        a = np.float32(1.2) * np.asarray(t, np.float32)
        return (np.float32(8.0) * np.cos(a.astype(np.float64)).astype(np.float32)).astype(np.float32)

    def transition_mean(self, x, t_previous):
        x = np.asarray(x, np.float32)
        f = np.float32
        return (f(0.5) * x + (f(25.0) * x) / (f(1.0) + x * x)) + self.drift(t_previous)

    def simulate(self, t_all, random_key):
        """StateSpaceModel.simulate (ssm.py:138-163): split(key, 2T); the first T keys
        drive the latent chain, the last T the observations."""
        p, _ = self.derived()
        t_np = np.asarray(t_all.cpu() if isinstance(t_all, torch.Tensor) else t_all, np.float32).reshape(-1)
        T = t_np.size
        keys = mrandom.split(random_key, 2 * T)
        ex = _normal_keys(keys[:T], 1).cpu().numpy()[:, 0]
        ey = _normal_keys(keys[T:], 1).cpu().numpy()[:, 0]
        x = np.empty(T, np.float32)
        x[0] = ex[0] * p["s0"]
        for i in range(1, T):
            x[i] = self.transition_mean(x[i - 1], t_np[i - 1]) + ex[i] * p["tsd"]
        y = (x * x) / np.float32(20.0) + ey * p["lsd"]
        dev = _dev.device()
        return cdict(x=torch.from_numpy(x[:, None].copy()).to(dev), y=torch.from_numpy(y[:, None].copy()).to(dev),
                     t=torch.as_tensor(t_np, device=dev), name=f"{self.name} simulation")


def _normal_keys(keys, d):
    keys = _dev.as_key(keys)
    out = torch.empty((keys.shape[0], d), dtype=torch.float32, device=keys.device)
    call("mgb_normal_keys", _dev.ptr(keys), keys.shape[0], d, _dev.ptr(out), _dev.stream_ptr())
    return out


class ParticleFilter:
    """Plugin interface of mocat/src/ssm/filtering.py:20-139.

    The built-in models run on fused CUDA kernels.  Any other model or filter runs
    through the generic driver (run_particle_filter_for_marginals and friends), which
    calls the two vectorised methods below with the whole particle batch as torch
    tensors on the GPU and does the rest (keys, logsumexp / ESS, resampling, gather,
    log Z) with the library's kernels.  Where the reference vmaps a per-particle
    method, the GPU plugin receives the batch: a model's initial_sample(t, random_keys),
    transition_sample(x_previous, t_previous, t_new, random_keys) and
    likelihood_potential(x, y, t) take x of shape (n, d) and random_keys of shape (n, 2)
    (uint32, jax's key layout; mocat_gb300.random.normal_keys draws from them) and
    return (n, d) / (n,) float32 CUDA tensors.  A filter may instead override the two
    vectorised methods."""
    name = "Particle Filter"

    def __init__(self, name=None):
        if name is not None:
            self.name = name

    def __repr__(self):
        return f"mocat_gb300.ParticleFilter.{self.__class__.__name__}"

    def startup(self, ssm_scenario):
        pass

    def initial_sample_and_weight_vectorised(self, ssm_scenario, y, t, random_keys):
        """filtering.py:65-78 with the batch: (x (n, d), log_weight (n,))."""
        x = ssm_scenario.initial_sample(t, random_keys)
        if y is None:
            return x, torch.zeros(x.shape[0], dtype=torch.float32, device=x.device)
        return x, -ssm_scenario.likelihood_potential(x, y, t)

    def propose_and_intermediate_weight_vectorised(self, ssm_scenario, x_previous, t_previous, y_new, t_new,
                                                   random_keys):
        """filtering.py:124-139 for the bootstrap proposal (filtering.py:142-170): the
        transition's draw, weighted by the likelihood."""
        x_new = ssm_scenario.transition_sample(x_previous, t_previous, t_new, random_keys)
        return x_new, -ssm_scenario.likelihood_potential(x_new, y_new, t_new)


class BootstrapFilter(ParticleFilter):
    """Propose from the transition, weight by the likelihood (filtering.py:142-170)."""
    name = "Bootstrap Filter"


class OptimalNonLinearGaussianParticleFilter(ParticleFilter):
    """Optimal proposal for linear-Gaussian observations
    (mocat/src/ssm/nonlinear_gaussian.py:134-281): fused kernels for a linear transition
    f(x) = F x (a TimeHomogenousLinearGaussian scenario); a NonLinearGaussian scenario runs
    the vectorised methods below through the generic driver.  startup computes the
    reference's constants (:154-184) in float64 and keeps float32 copies."""
    name = "Optimal Non-linear Gaussian Particle Filter"

    def _t(self, name):
        return torch.as_tensor(np.asarray(self._consts[name], np.float32), device=_dev.device())

    def initial_sample_and_weight_vectorised(self, ssm_scenario, y, t, random_keys):
        """(:223-229, initial_sample :205-215): mean m0 + K0 (y - H m0), one (n, d) normal
        draw from the first particle key, times the conditioned covariance square root
        (not transposed, as the reference); zero log-weights"""
        if getattr(self, "_consts", None) is None:
            self.startup(ssm_scenario)
        n = random_keys.shape[0]
        m0, H, K0 = self._t("m064"), self._t("H64"), self._t("K0")
        mean = m0 + K0 @ (_dev.as_f32(y).reshape(-1) - H @ m0)
        e = mrandom.normal(random_keys[0], (n, ssm_scenario.dim))
        return mean + e @ self._t("C0c"), torch.zeros(n, dtype=torch.float32, device=e.device)

    def propose_and_intermediate_weight_vectorised(self, ssm_scenario, x_previous, t_previous, y_new, t_new,
                                                   random_keys):
        """(:264-281): mx = f(x), x_new = mx + (y - mx H^T) K^T + normal(keys[0], (n, d)) S^T,
        log-weight -(0.5 |(y - mx H^T) W|^2 + cw)"""
        if getattr(self, "_consts", None) is None:
            self.startup(ssm_scenario)
        H, K, S, W = self._t("H64"), self._t("K"), self._t("S"), self._t("W")
        mx = ssm_scenario.transition_function(x_previous, t_previous, t_new)
        r = _dev.as_f32(y_new).reshape(1, -1) - mx @ H.T
        e = mrandom.normal(random_keys[0], tuple(x_previous.shape))
        x_new = mx + r @ K.T + e @ S.T
        v = r @ W
        return x_new, -(0.5 * (v * v).sum(-1) + float(self._consts["cw"]))

    def startup(self, ssm_scenario):
        lg = isinstance(ssm_scenario, TimeHomogenousLinearGaussian)
        p = ssm_scenario.derived()[0] if lg else None
        S0 = ssm_scenario.initial_covariance
        Q = ssm_scenario.transition_covariance
        H = ssm_scenario.likelihood_matrix
        R = ssm_scenario.likelihood_covariance
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

        self.initial_kalman_gain = kalman_gain(C0)
        a = H.T @ lik_prec_sqrt
        init_cond_prec = init_prec_sqrt @ init_prec_sqrt + a @ a.T
        self.initial_conditioned_precision_sqrt = np.linalg.cholesky(init_cond_prec)
        self.initial_conditioned_covariance_sqrt = np.linalg.inv(self.initial_conditioned_precision_sqrt)
        hl = H @ Lq
        weight_precision = np.linalg.inv(hl @ hl.T + LR @ LR.T)
        self.proposal_kalman_gain = kalman_gain(Lq, weight_precision)
        prop_cov = Q - self.proposal_kalman_gain @ H @ Q
        self.proposal_covariance_sqrt = np.linalg.cholesky(prop_cov)
        self.weight_precision_sqrt = np.linalg.cholesky(weight_precision)
        self.weight_precision_det = np.linalg.det(weight_precision)
        dy = H.shape[0]
        c = dict(d=ssm_scenario.dim, dy=dy, K=_f32(self.proposal_kalman_gain),
                 S=_f32(self.proposal_covariance_sqrt), W=_f32(self.weight_precision_sqrt),
                 cw=np.float32((dy * LOG2PI - np.log(self.weight_precision_det)) / 2.0),
                 K0=_f32(self.initial_kalman_gain), C0c=_f32(self.initial_conditioned_covariance_sqrt),
                 H64=_f32(H), m064=_f32(ssm_scenario.initial_mean))
        self._consts = c
        if not lg:
            self._struct = None
            return
        c.update(F=p["F"], H=p["H"], m0=p["m0"])
        self._struct = _lib.OptModel(c["d"], c["dy"], c["F"].ctypes.data, c["H"].ctypes.data, c["K"].ctypes.data,
                                     c["S"].ctypes.data, c["W"].ctypes.data, float(c["cw"]), c["K0"].ctypes.data,
                                     c["C0c"].ctypes.data, c["m0"].ctypes.data)


def _overrides(obj, base, names):
    return any(getattr(type(obj), m, None) is not getattr(base, m, None) for m in names)


def _fused(ssm_scenario, particle_filter):
    """True when a fused kernel runs this model / filter pair: a built-in model (or a
    subclass that keeps its plugin methods) with a built-in filter (or a subclass that
    keeps its vectorised methods).  False routes the pair to the generic driver."""
    pf_base = next((b for b in (OptimalNonLinearGaussianParticleFilter, BootstrapFilter)
                    if isinstance(particle_filter, b)), None)
    if pf_base is None or _overrides(particle_filter, pf_base, ("initial_sample_and_weight_vectorised",
                                                                  "propose_and_intermediate_weight_vectorised")):
        return False
    for base in (TimeHomogenousLinearGaussian, StochasticVolatility, NonLinear1DBenchmark):
        if isinstance(ssm_scenario, base):
            return not _overrides(ssm_scenario, base, ("initial_sample", "transition_sample", "likelihood_potential"))
    return False


def _check_lg(ssm_scenario, particle_filter):
    if isinstance(ssm_scenario, StochasticVolatility):
        if type(particle_filter) is not BootstrapFilter:
            raise NotImplementedError(f"{particle_filter.__class__.__name__}: no fused GPU kernel for this model")
        if not 1 <= ssm_scenario.dim <= LG_RUNTIME_MAX:
            raise NotImplementedError(f"StochasticVolatility: the GPU kernels take dim 1..{LG_RUNTIME_MAX}")
        return
    if isinstance(ssm_scenario, NonLinear1DBenchmark):
        if type(particle_filter) is not BootstrapFilter:
            raise NotImplementedError(f"{particle_filter.__class__.__name__}: no fused GPU kernel for this model")
        return
    if not isinstance(ssm_scenario, TimeHomogenousLinearGaussian):
        raise NotImplementedError(f"{ssm_scenario.__class__.__name__}: no fused GPU kernel for this model")
    if not isinstance(particle_filter, (BootstrapFilter, OptimalNonLinearGaussianParticleFilter)):
        raise NotImplementedError(f"{particle_filter.__class__.__name__}: no fused GPU kernel for this filter")
    if not ssm_scenario.gpu_runtime_supported():
        raise NotImplementedError(f"(d, dy) = ({ssm_scenario.dim}, {ssm_scenario.dim_obs}) above the "
                                  f"run-time-dimension limit ({LG_RUNTIME_MAX})")


def _kernels(ssm_scenario, particle_filter):
    """(C-ABI prefix, model struct) of the fused kernels for this scenario / filter pair."""
    if isinstance(ssm_scenario, NonLinear1DBenchmark):
        return "mgb_pf_nl1d", ssm_scenario.derived()[1]
    if isinstance(ssm_scenario, StochasticVolatility):
        if ssm_scenario.dim != 1:
            return "mgb_pf_svd", ssm_scenario.derived()[1]
        # bsig of the dt = 1 struct is transition_covariance_sqrt; the kernels scale it by sqrt(dt)
        return "mgb_pf_sv", ssm_scenario.derived(1.0)[1]
    if isinstance(particle_filter, OptimalNonLinearGaussianParticleFilter):
        if getattr(particle_filter, "_struct", None) is None:
            particle_filter.startup(ssm_scenario)
        return "mgb_pf_opt", particle_filter._struct
    return "mgb_pf_lg", ssm_scenario.derived()[1]


def _y2(y, dy):
    y = _dev.as_f32(y)
    return y.reshape(-1, dy).contiguous()


def initiate_particles(ssm_scenario, particle_filter, n, random_key, y=None, t=None):
    """filtering.py:173-193: particles (1, n, d), log-weights (1, n), ess (1,)."""
    if not _fused(ssm_scenario, particle_filter):
        return _initiate_generic(ssm_scenario, particle_filter, n, random_key, y, t)
    _check_lg(ssm_scenario, particle_filter)
    particle_filter.startup(ssm_scenario)
    prefix, s = _kernels(ssm_scenario, particle_filter)
    d = ssm_scenario.dim
    dev = _dev.device()
    key = _dev.as_key(random_key)
    x = torch.empty((d, n), dtype=torch.float32, device=dev)
    lw = torch.empty(n, dtype=torch.float32, device=dev)
    yd = None if y is None else _y2(y, ssm_scenario.dim_obs).reshape(-1)
    call(prefix + "_init", ctypes.byref(s), n, _dev.ptr(key), _dev.ptr(yd), _dev.ptr(x), _dev.ptr(lw),
         _dev.stream_ptr())
    return cdict(value=x.t().contiguous()[None], log_weight=lw[None],
                 t=torch.atleast_1d(torch.as_tensor(0.0 if t is None else t, device=dev)),
                 y=None if y is None else yd[None], ess=ess_log_weight(lw).reshape(1).float())


def resample_particles(particles, random_key, resample_full=True, resampling="systematic"):
    """filtering.py:202-217 (gather of the value history by the latest weights)."""
    out = particles.copy()
    lw = particles.log_weight if particles.log_weight.dim() == 1 else particles.log_weight[-1]
    n = lw.numel()
    anc = resample(lw, random_key, resampling).long()
    if particles.log_weight.dim() == 1:
        # x[..., idx, :]: every time slice of a (T, n, d) value along the particle axis
        out.value = particles.value[..., anc, :]
        out.log_weight = torch.zeros(n, device=lw.device)
    elif resample_full:
        out.value = particles.value[:, anc]
        out.log_weight = particles.log_weight.clone()
        out.log_weight[-1] = 0.0
    else:
        out.value = particles.value.clone()
        out.value[-1] = particles.value[-1][anc]
        out.log_weight = particles.log_weight.clone()
        out.log_weight[-1] = 0.0
    return out


def _step(s, n, key, y_t, x_prev_soa, anc, lw_prev, prefix="mgb_pf_lg", t_prev=None, t_new=None):
    x_new = torch.empty_like(x_prev_soa)
    lw_new = torch.empty(n, dtype=torch.float32, device=x_prev_soa.device)
    # the non-linear model's transition depends on t_previous, the stochastic-volatility
    # model's on t_new - t_previous (float32, as the reference's time arrays)
    if prefix == "mgb_pf_nl1d":
        tp = (float(t_prev),)
    elif prefix in ("mgb_pf_sv", "mgb_pf_svd"):
        tp = (float(np.float32(float(t_new)) - np.float32(float(t_prev))),)
    else:
        tp = ()
    call(prefix + "_propagate", ctypes.byref(s), n, _dev.ptr(key), _dev.ptr(y_t), *tp, _dev.ptr(x_prev_soa),
         _dev.ptr(anc), _dev.ptr(lw_prev), _dev.ptr(x_new), _dev.ptr(lw_new), _dev.stream_ptr())
    return x_new, lw_new


def propagate_particle_filter(ssm_scenario, particle_filter, particles, y_new, t_new, random_key,
                              ess_threshold=0.5, resample_full=True, resampling="systematic"):
    """filtering.py:220-252: resample if ess < threshold n, then propagate and append."""
    if not _fused(ssm_scenario, particle_filter):
        return _propagate_generic(ssm_scenario, particle_filter, particles, y_new, t_new, random_key, ess_threshold,
                                  resample_full, resampling)
    _check_lg(ssm_scenario, particle_filter)
    prefix, s = _kernels(ssm_scenario, particle_filter)
    n = particles.value.shape[1]
    key = _dev.as_key(random_key)
    if float(particles.ess[-1]) < ess_threshold * n:
        particles = resample_particles(particles, key, resample_full, resampling)
    x_prev = particles.value[-1].t().contiguous()
    lw_prev = particles.log_weight[-1].contiguous()
    y_t = _y2(y_new, ssm_scenario.dim_obs).reshape(-1)
    x_new, lw_new = _step(s, n, key, y_t, x_prev, None, lw_prev, prefix, t_prev=particles.t[-1], t_new=t_new)
    out = particles.copy()
    out.value = torch.cat([particles.value, x_new.t()[None]], 0)
    out.log_weight = torch.cat([particles.log_weight, lw_new[None]], 0)
    out.y = torch.cat([particles.y, y_t[None]], 0) if particles.y is not None else y_t[None]
    out.t = torch.cat([particles.t, torch.atleast_1d(torch.as_tensor(t_new, device=out.t.device)).to(out.t.dtype)])
    out.ess = torch.cat([particles.ess, ess_log_weight(lw_new).reshape(1).float()])
    return out


def run_particle_filter_for_marginals(ssm_scenario, particle_filter, y, t, random_key, n=None, initial_sample=None,
                                      ess_threshold=0.5, resampling="systematic", history=True, persistent=True):
    """filtering.py:255-324 on the GPU.

    Returns cdict(value (T, n, d), log_weight (T, n), ess (T,), t, y, log_z, resampled)
    (value/log_weight only the final step, shape (1, n, d) / (1, n), when history=False).
    persistent=False forces one kernel launch per phase and step instead of the
    single persistent launch (bootstrap filter on the linear-Gaussian or the
    non-linear benchmark model, systematic resampling, even n <= 2^21); results
    are the same.  A model or filter without a fused kernel runs through the
    generic driver (ParticleFilter's vectorised plugin methods, the library's
    logsumexp / resampling / gather kernels); persistent is then ignored.

    resampling defaults to "systematic", a deliberate deviation: the reference
    draws ancestors with random.categorical (filtering.py:199), which is
    resampling="categorical" here (the same Gumbel-max draws, O(n^2) per step,
    small n only).  Systematic resampling has lower variance and is O(n), but
    gives different ancestors from the reference's on the same key.
    """
    if not _fused(ssm_scenario, particle_filter):
        return _run_generic(ssm_scenario, particle_filter, y, t, random_key, n, initial_sample, ess_threshold,
                            resampling, history)
    _check_lg(ssm_scenario, particle_filter)
    particle_filter.startup(ssm_scenario)
    prefix, s = _kernels(ssm_scenario, particle_filter)
    d, dy = ssm_scenario.dim, ssm_scenario.dim_obs
    dev = _dev.device()
    y2 = _y2(y, dy)
    key = _dev.as_key(random_key)
    sc = SCHEMES[resampling]
    if initial_sample is not None:
        return _run_from(ssm_scenario, s, initial_sample, y2, t, key, ess_threshold, resampling, prefix)
    T = y2.shape[0]
    nl = prefix in ("mgb_pf_nl1d", "mgb_pf_sv", "mgb_pf_svd")
    if nl:
        t32 = _dev.as_f32(t).reshape(-1).contiguous()
        if t32.numel() != T:
            raise ValueError(f"t has {t32.numel()} entries for {T} observations")
        wsa = (n, T, d, sc) if prefix == "mgb_pf_svd" else (n, T, sc)
        ws = _dev.workspace(getattr(_lib.lib(), prefix + "_workspace")(*wsa), dev)
    else:
        ws = _dev.workspace(getattr(_lib.lib(), prefix + "_workspace")(n, T, d, sc), dev)
    logz = torch.empty(1, dtype=torch.float64, device=dev)
    ess = torch.empty(T, dtype=torch.float32, device=dev)
    res = torch.empty(T, dtype=torch.int32, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    xh = torch.empty((T, d, n) if history else (1, d, n), dtype=torch.float32, device=dev)
    lh = torch.empty((T, n) if history else (1, n), dtype=torch.float32, device=dev)
    out = _lib.PFOutputs(logz.data_ptr(), ess.data_ptr(), res.data_ptr(), xh.data_ptr() if history else None,
                         lh.data_ptr() if history else None, None if history else xh.data_ptr(),
                         None if history else lh.data_ptr(), err.data_ptr(), None)
    if nl:
        call(prefix + "_run", ctypes.byref(s), n, T, _dev.ptr(key), _dev.ptr(y2), _dev.ptr(t32),
             float(ess_threshold), sc | (0 if persistent else RUN_LAUNCH_PER_STEP), _dev.ptr(ws), ws.numel(),
             ctypes.byref(out), _dev.stream_ptr())
    else:
        flags = 0 if (persistent or prefix != "mgb_pf_lg") else RUN_LAUNCH_PER_STEP
        call(prefix + "_run", ctypes.byref(s), n, T, _dev.ptr(key), _dev.ptr(y2), float(ess_threshold), sc | flags,
             _dev.ptr(ws), ws.numel(), ctypes.byref(out), _dev.stream_ptr())
    e = int(err.item())
    if e & 1:
        raise _lib.MGBError(5, "run_particle_filter_for_marginals")
    tt = torch.as_tensor(np.asarray(t if not isinstance(t, torch.Tensor) else t.cpu()), device=dev)
    return cdict(value=xh.permute(0, 2, 1), log_weight=lh, ess=ess, t=tt, y=y2, log_z=logz[0],
                 resampled=res.bool(), degenerate=bool(e & 2))


# ---------------------------------------------------------------- generic driver
def _lse_ess(lw):
    """(LSE, ESS) of log-weights on the device (mgb_lse_ess), as float64 device scalars."""
    n = lw.numel()
    ws = _dev.workspace(_lib.lib().mgb_lse_ess_workspace(n), lw.device)
    out = torch.empty(4, dtype=torch.float64, device=lw.device)
    call("mgb_lse_ess", _dev.ptr(lw), n, _dev.ptr(out), _dev.ptr(ws), ws.numel(), _dev.stream_ptr())
    return out[1], out[3]


def _plugin_xw(x, lw, n, where):
    """the plugin's (x, log_weight) as contiguous float32 device tensors (n, d), (n,)."""
    if not isinstance(x, torch.Tensor) or not x.is_cuda or not isinstance(lw, torch.Tensor) or not lw.is_cuda:
        raise _lib.MGBError(1, f"{where}: the plugin must return CUDA tensors (no host path)")
    x = x.to(torch.float32)
    if x.dim() == 1:
        x = x[:, None]
    lw = lw.to(torch.float32).reshape(-1)
    if x.shape[0] != n or lw.numel() != n:
        raise ValueError(f"{where}: plugin returned {tuple(x.shape)} / {tuple(lw.shape)} for n = {n}")
    return x.contiguous(), lw.contiguous()


def _gather(x, anc):
    out = torch.empty_like(x)
    call("mgb_gather_rows", _dev.ptr(x), x.shape[1], _dev.ptr(anc), x.shape[0], _dev.ptr(out), _dev.stream_ptr())
    return out


def _initiate_generic(ssm_scenario, particle_filter, n, random_key, y=None, t=None):
    particle_filter.startup(ssm_scenario)
    dev = _dev.device()
    sub_keys = mrandom.split(_dev.as_key(random_key), n)
    yd = None if y is None else _dev.as_f32(y).reshape(-1)
    x, lw = _plugin_xw(*particle_filter.initial_sample_and_weight_vectorised(ssm_scenario, yd, t, sub_keys), n,
                       "initial_sample_and_weight_vectorised")
    _, ess = _lse_ess(lw)
    return cdict(value=x[None], log_weight=lw[None],
                 t=torch.atleast_1d(torch.as_tensor(0.0 if t is None else t, device=dev)),
                 y=None if yd is None else yd[None], ess=ess.float().reshape(1))


def _generic_step(ssm_scenario, particle_filter, x, lw, ess, n, key, y_t, t_prev, t_new, ess_threshold, resampling):
    """One body of the reference's scan (filtering.py:280-311): resample on the
    previous ESS, propagate with split(k_t, n), add the carried log-weight."""
    res = bool(np.float32(float(ess)) < np.float32(ess_threshold) * np.float32(n))
    if res:
        anc = resample(lw, key, resampling)
        x_res, lw_res = _gather(x, anc), torch.zeros_like(lw)
    else:
        x_res, lw_res = x, lw
    keys = mrandom.split(key, n)
    x_new, lw_inc = _plugin_xw(*particle_filter.propose_and_intermediate_weight_vectorised(
        ssm_scenario, x_res, t_prev, y_t, t_new, keys), n, "propose_and_intermediate_weight_vectorised")
    return x_new, lw_res + lw_inc, res


def _propagate_generic(ssm_scenario, particle_filter, particles, y_new, t_new, random_key, ess_threshold=0.5,
                       resample_full=True, resampling="systematic"):
    n = particles.value.shape[1]
    key = _dev.as_key(random_key)
    if float(particles.ess[-1]) < ess_threshold * n:
        particles = resample_particles(particles, key, resample_full, resampling)
    x_prev = particles.value[-1].contiguous()
    lw_prev = particles.log_weight[-1].contiguous()
    y_t = _dev.as_f32(y_new).reshape(-1)
    keys = mrandom.split(key, n)
    x_new, lw_inc = _plugin_xw(*particle_filter.propose_and_intermediate_weight_vectorised(
        ssm_scenario, x_prev, particles.t[-1], y_t, t_new, keys), n, "propose_and_intermediate_weight_vectorised")
    lw_new = lw_prev + lw_inc
    out = particles.copy()
    out.value = torch.cat([particles.value, x_new[None]], 0)
    out.log_weight = torch.cat([particles.log_weight, lw_new[None]], 0)
    out.y = torch.cat([particles.y, y_t[None]], 0) if particles.y is not None else y_t[None]
    out.t = torch.cat([particles.t, torch.atleast_1d(torch.as_tensor(t_new, device=out.t.device)).to(out.t.dtype)])
    out.ess = torch.cat([particles.ess, ess_log_weight(lw_new).reshape(1).float()])
    return out


def _run_generic(ssm_scenario, particle_filter, y, t, random_key, n=None, initial_sample=None, ess_threshold=0.5,
                 resampling="systematic", history=True):
    """run_particle_filter_for_marginals (filtering.py:255-324) for a user model or filter:
    the key schedule, ESS trigger, key reuse (k_t resamples and seeds split(k_t, n)) and
    log-weight carry of the reference; the plugin's vectorised methods propagate and weight."""
    particle_filter.startup(ssm_scenario)
    dev = _dev.device()
    y2 = _dev.as_f32(y)
    if y2.dim() == 1:
        y2 = y2[:, None]
    t_np = np.asarray(t.cpu() if isinstance(t, torch.Tensor) else t, np.float32).reshape(-1)
    key = _dev.as_key(random_key)
    if initial_sample is None:
        k2 = mrandom.split(key)
        key, sub = k2[0].contiguous(), k2[1].contiguous()
        initial_sample = _initiate_generic(ssm_scenario, particle_filter, n, sub, y2[0], float(t_np[0]))
        y2, t_np = y2[1:], t_np[1:]
    x = initial_sample.value[-1].contiguous()
    lw = initial_sample.log_weight[-1].contiguous()
    n = lw.numel()
    lse_prev, ess = _lse_ess(lw)
    logz = lse_prev - math.log(n)
    t_prev = float(initial_sample.t[-1])
    Tp = y2.shape[0]
    keys = mrandom.split(key, Tp) if Tp else None
    xs, lws, esss, resd = [x], [lw], [ess.float()], [False]
    for i in range(Tp):
        x, lw, res = _generic_step(ssm_scenario, particle_filter, x, lw, ess, n, keys[i].contiguous(),
                                   y2[i].contiguous(), t_prev, float(t_np[i]), ess_threshold, resampling)
        lse, ess = _lse_ess(lw)
        logz = logz + lse - (math.log(n) if res else lse_prev)
        lse_prev = lse
        t_prev = float(t_np[i])
        if history:
            xs.append(x)
            lws.append(lw)
        esss.append(ess.float())
        resd.append(res)
    value = torch.stack(xs) if history else x[None]
    log_weight = torch.stack(lws) if history else lw[None]
    tt = torch.cat([initial_sample.t.to(torch.float32), torch.as_tensor(t_np, device=dev)])
    yy = torch.cat([initial_sample.y, y2]) if initial_sample.y is not None else y2
    return cdict(value=value, log_weight=log_weight, ess=torch.stack(esss), t=tt, y=yy, log_z=logz.reshape(()),
                 resampled=torch.tensor(resd, device=dev))


def _run_from(ssm_scenario, s, initial_sample, y2, t, key, ess_threshold, resampling, prefix="mgb_pf_lg"):
    """Resume from given particles (filtering.py:266-275 with initial_sample set)."""
    x = initial_sample.value[-1].t().contiguous()
    lw = initial_sample.log_weight[-1].contiguous()
    n = lw.numel()
    ess = float(initial_sample.ess[-1])
    T = y2.shape[0]
    keys = mrandom.split(key, T)
    vals, lws, esss, resd = [], [], [], []
    logz = 0.0
    lse_prev = float(torch.logsumexp(lw.double(), 0))
    # t_previous of step i: the initial sample's last time, then t[i - 1] (filtering.py:295-303)
    t_np = np.asarray(t.cpu() if isinstance(t, torch.Tensor) else t, np.float32).reshape(-1)
    t_prev = float(initial_sample.t[-1]) if initial_sample.t is not None else 0.0
    for i in range(T):
        res = ess < ess_threshold * n
        anc = resample(lw, keys[i], resampling) if res else None
        t_new = float(t_np[i]) if i < t_np.size else t_prev
        x, lw = _step(s, n, keys[i], y2[i], x, anc, None if res else lw, prefix, t_prev=t_prev, t_new=t_new)
        t_prev = t_new
        lse = float(torch.logsumexp(lw.double(), 0))
        logz += lse - (math.log(n) if res else lse_prev)
        lse_prev = lse
        ess = float(ess_log_weight(lw))
        vals.append(x.t())
        lws.append(lw)
        esss.append(ess)
        resd.append(res)
    dev = lw.device
    return cdict(value=torch.stack(vals), log_weight=torch.stack(lws), ess=torch.tensor(esss, device=dev),
                 t=torch.as_tensor(np.asarray(t if not isinstance(t, torch.Tensor) else t.cpu()), device=dev),
                 y=y2, log_z=torch.tensor(logz, dtype=torch.float64, device=dev),
                 resampled=torch.tensor(resd, device=dev))


def _kalman_struct(ssm_scenario):
    """float32 F, Q, H, R, m0 and the initial covariance square root (the reference's t = 0 covariance)"""
    keep = dict(F=_f32(ssm_scenario.transition_matrix), Q=_f32(ssm_scenario.transition_covariance),
                H=_f32(ssm_scenario.likelihood_matrix), R=_f32(ssm_scenario.likelihood_covariance),
                m0=_f32(ssm_scenario.initial_mean), C0=_f32(np.linalg.cholesky(ssm_scenario.initial_covariance)))
    s = _lib.KalmanModel(ssm_scenario.dim, ssm_scenario.dim_obs,
                         *[keep[k].ctypes.data for k in ("F", "Q", "H", "R", "m0", "C0")])
    return keep, s


def _check_kalman(ssm_scenario):
    if not isinstance(ssm_scenario, TimeHomogenousLinearGaussian):
        raise NotImplementedError(f"{ssm_scenario.__class__.__name__}: the Kalman filter takes a linear-Gaussian model")
    # compiled pairs, or the run-time-dimension instance for d, dy <= 32
    if not ssm_scenario.gpu_runtime_supported():
        raise NotImplementedError(f"(d, dy) = ({ssm_scenario.dim}, {ssm_scenario.dim_obs}) not compiled")


def run_kalman_filter_for_marginals(lgssm_scenario, y, t=None, return_log_likelihood=False):
    """kalman.py:16-57 on the GPU: (means (T, d), covs (T, d, d)) filtered marginals.  y may carry a
    leading batch axis (B, T, dy): B sequences of the same model in one launch, outputs (B, T, ...).
    return_log_likelihood=True appends the prediction-error log-likelihood (float64, (B,) or scalar)."""
    _check_kalman(lgssm_scenario)
    d, dy = lgssm_scenario.dim, lgssm_scenario.dim_obs
    yy = _dev.as_f32(y)
    if yy.dim() == 1:
        yy = yy.reshape(-1, dy)
    batched = yy.dim() == 3
    yy = (yy if batched else yy[None]).contiguous()
    B, T = yy.shape[0], yy.shape[1]
    dev = yy.device
    means = torch.empty((B, T, d), dtype=torch.float32, device=dev)
    covs = torch.empty((B, T, d, d), dtype=torch.float32, device=dev)
    ll = torch.empty(B, dtype=torch.float64, device=dev)
    _, s = _kalman_struct(lgssm_scenario)
    call("mgb_kalman_filter", ctypes.byref(s), B, T, _dev.ptr(yy), _dev.ptr(means), _dev.ptr(covs), _dev.ptr(ll),
         _dev.stream_ptr())
    out = (means, covs, ll) if batched else (means[0], covs[0], ll[0])
    return out if return_log_likelihood else out[:2]


def run_kalman_smoother_for_marginals_and_lag_ones(lgssm_scenario, y, t=None, filter_output=None):
    """kalman.py:60-94 on the GPU: (means, covs, lag_ones) smoothed marginals and the lag-one
    terms (T-1, d, d), in the batched form of run_kalman_filter_for_marginals."""
    _check_kalman(lgssm_scenario)
    if filter_output is None:
        filter_output = run_kalman_filter_for_marginals(lgssm_scenario, y, t)
    fm, fc = (_dev.as_f32(a) for a in filter_output[:2])
    batched = fm.dim() == 3
    fm = (fm if batched else fm[None]).contiguous()
    fc = (fc if batched else fc[None]).contiguous()
    B, T, d = fm.shape
    sm, sc = torch.empty_like(fm), torch.empty_like(fc)
    lag = torch.empty((B, max(T - 1, 0), d, d), dtype=torch.float32, device=fm.device)
    _, s = _kalman_struct(lgssm_scenario)
    call("mgb_kalman_smoother", ctypes.byref(s), B, T, _dev.ptr(fm), _dev.ptr(fc), _dev.ptr(sm), _dev.ptr(sc),
         _dev.ptr(lag) if T > 1 else None, _dev.stream_ptr())
    return (sm, sc, lag) if batched else (sm[0], sc[0], lag[0])


def run_kalman_smoother_for_marginals(lgssm_scenario, y, t=None, filter_output=None):
    """kalman.py:97-104 on the GPU: (means, covs) smoothed marginals (the batched form as
    run_kalman_filter_for_marginals)."""
    _check_kalman(lgssm_scenario)
    if filter_output is None:
        filter_output = run_kalman_filter_for_marginals(lgssm_scenario, y, t)
    fm, fc = (_dev.as_f32(a) for a in filter_output[:2])
    batched = fm.dim() == 3
    fm = (fm if batched else fm[None]).contiguous()
    fc = (fc if batched else fc[None]).contiguous()
    B, T = fm.shape[0], fm.shape[1]
    sm, sc = torch.empty_like(fm), torch.empty_like(fc)
    _, s = _kalman_struct(lgssm_scenario)
    call("mgb_kalman_smoother", ctypes.byref(s), B, T, _dev.ptr(fm), _dev.ptr(fc), _dev.ptr(sm), _dev.ptr(sc), None,
         _dev.stream_ptr())
    return (sm, sc) if batched else (sm[0], sc[0])


def _transition_struct(ssm_scenario):
    """F, transition_precision_sqrt = inv(chol(Q)), and the normaliser of the transition
    potential, computed as reset_covariance does (mocat/src/utils.py:247-262)."""
    if "_transition" not in ssm_scenario.__dict__:
        Q = ssm_scenario.transition_covariance
        Pq = np.linalg.inv(np.linalg.cholesky(Q))
        det_prec = 1.0 / np.linalg.det(Q)
        d = ssm_scenario.dim
        keep = dict(F=_f32(ssm_scenario.transition_matrix), Pq=_f32(Pq),
                    cq=np.float32((d * LOG2PI - np.log(det_prec)) / 2.0))
        s = _lib.LGTransition(d, keep["F"].ctypes.data, keep["Pq"].ctypes.data, float(keep["cq"]))
        ssm_scenario.__dict__["_transition"] = (keep, s)
    return ssm_scenario.__dict__["_transition"]


def _bsim_output(marginal_particles, out, evals, idx):
    """backward.py:207-214 / :240-245: a copy of the filter output with the value replaced by the
    backward trajectories, num_transition_evals added and log_weight removed (the sampled
    indices are kept as well)"""
    res = cdict(**{k: v for k, v in marginal_particles.__dict__.items() if k != "log_weight"})
    res.value = out.permute(0, 2, 1)
    res.num_transition_evals = evals
    res.indices = idx
    return res


def backward_simulation(ssm_scenario, marginal_particles, random_key, n_samps=None, maximum_rejections=0,
                        transition_dens_bound_parameter=0.0, bound_inflation=1.01):
    """backward.py:248-270: n_samps trajectories drawn backwards through the filter's particles,
    by the full categorical (maximum_rejections = 0, backward_simulation_full :217-245) or by
    rejection sampling (backward_simulation_rejection :172-214).  Returns cdict(value
    (T, n_samps, d), t, num_transition_evals (T,), indices)."""
    nl = isinstance(ssm_scenario, NonLinear1DBenchmark)
    sv = isinstance(ssm_scenario, StochasticVolatility)
    if not nl and not sv and not isinstance(ssm_scenario, TimeHomogenousLinearGaussian):
        raise NotImplementedError(f"{ssm_scenario.__class__.__name__}: no backward-simulation kernel for this model")
    if sv and ssm_scenario.dim != 1:
        raise NotImplementedError("StochasticVolatility: the GPU kernels take dim = 1")
    if not nl and not sv and not ssm_scenario.gpu_runtime_supported():
        raise NotImplementedError(f"d = {ssm_scenario.dim} above the run-time-dimension limit ({LG_RUNTIME_MAX})")
    value = marginal_particles.value
    T, n, d = value.shape
    M = n if n_samps is None else int(n_samps)
    x = _dev.as_f32(value).permute(0, 2, 1).contiguous()
    lw = _dev.as_f32(marginal_particles.log_weight).reshape(T, n).contiguous()
    key = _dev.as_key(random_key)
    dev = x.device
    out = torch.empty((T, d, M), dtype=torch.float32, device=dev)
    idx = torch.empty((T, M), dtype=torch.int32, device=dev)
    tt = None
    if nl or sv:
        tt = _dev.as_f32(marginal_particles.t).reshape(-1).contiguous()
        if tt.numel() != T:
            raise ValueError(f"marginal_particles.t has {tt.numel()} entries for {T} steps")
    if sv:
        th = np.ascontiguousarray(tt.cpu().numpy(), np.float32)
        phi, pq = ssm_scenario.transition_constants()
    if maximum_rejections > 0:
        cfg = _lib.RejectionConfig(int(maximum_rejections), float(transition_dens_bound_parameter),
                                   float(bound_inflation))
        ws = _dev.workspace(_lib.lib().mgb_ffbsi_rejection_workspace(n, M, T, d), dev)
        evals = torch.empty(T, dtype=torch.int64, device=dev)
        if sv:
            call("mgb_ffbsi_rejection_sv", float(phi), float(pq), ctypes.byref(cfg), T, n, M, _dev.ptr(x),
                 _dev.ptr(lw), th.ctypes.data, _dev.ptr(key), _dev.ptr(out), _dev.ptr(idx), _dev.ptr(evals),
                 _dev.ptr(ws), ws.numel(), _dev.stream_ptr())
        elif nl:
            call("mgb_ffbsi_rejection_nl1d", ctypes.byref(ssm_scenario.derived()[1]), ctypes.byref(cfg), T, n, M,
                 _dev.ptr(x), _dev.ptr(lw), _dev.ptr(tt), _dev.ptr(key), _dev.ptr(out), _dev.ptr(idx), _dev.ptr(evals),
                 _dev.ptr(ws), ws.numel(), _dev.stream_ptr())
        else:
            _, s = _transition_struct(ssm_scenario)
            call("mgb_ffbsi_rejection_lg", ctypes.byref(s), ctypes.byref(cfg), T, n, M, _dev.ptr(x), _dev.ptr(lw),
                 _dev.ptr(key), _dev.ptr(out), _dev.ptr(idx), _dev.ptr(evals), _dev.ptr(ws), ws.numel(),
                 _dev.stream_ptr())
        return _bsim_output(marginal_particles, out, evals, idx)
    ws = _dev.workspace(_lib.lib().mgb_ffbsi_workspace(n, T, d), dev)
    if sv:
        call("mgb_ffbsi_sv", float(phi), float(pq), T, n, M, _dev.ptr(x), _dev.ptr(lw), th.ctypes.data,
             _dev.ptr(key), _dev.ptr(out), _dev.ptr(idx), _dev.ptr(ws), ws.numel(), _dev.stream_ptr())
    elif nl:
        call("mgb_ffbsi_nl1d", ctypes.byref(ssm_scenario.derived()[1]), T, n, M, _dev.ptr(x), _dev.ptr(lw),
             _dev.ptr(tt), _dev.ptr(key), _dev.ptr(out), _dev.ptr(idx), _dev.ptr(ws), ws.numel(), _dev.stream_ptr())
    else:
        _, s = _transition_struct(ssm_scenario)
        call("mgb_ffbsi_lg", ctypes.byref(s), T, n, M, _dev.ptr(x), _dev.ptr(lw), _dev.ptr(key), _dev.ptr(out),
             _dev.ptr(idx), _dev.ptr(ws), ws.numel(), _dev.stream_ptr())
    evals = torch.full((T,), float(n * M), device=dev)
    evals[0] = 0.0
    return _bsim_output(marginal_particles, out, evals, idx)


def forward_filtering_backward_simulation(ssm_scenario, particle_filter, y, t, n_samps, random_key, n_pf=None,
                                          ess_threshold=0.5, maximum_rejections=0, transition_dens_bound_parameter=0.0,
                                          bound_inflation=1.01, resampling="systematic"):
    """backward.py:272-315: (pf_key, bsi_key) = split(key); filter with n_pf particles, then
    backward_simulation of n_samps trajectories."""
    keys = mrandom.split(_dev.as_key(random_key), 2)
    n_pf = n_samps if n_pf is None else n_pf
    pf = run_particle_filter_for_marginals(ssm_scenario, particle_filter, y, t, keys[0], n=n_pf,
                                           ess_threshold=ess_threshold, resampling=resampling)
    out = backward_simulation(ssm_scenario, pf, keys[1], n_samps, maximum_rejections,
                              transition_dens_bound_parameter, bound_inflation)
    out.log_z = pf.log_z
    return out


def _dt(t_prev, t_new):
    return float(np.float32(float(t_new)) - np.float32(float(t_prev)))


def _pair_potential(ssm_scenario, x0, x1, lw=None, t_prev=0.0, t_new=None):
    """lw_i + transition_potential(x0_i at t_prev -> x1_i at t_new) for particle-major (M, d) rows."""
    x0t = _dev.as_f32(x0).t().contiguous()
    x1t = _dev.as_f32(x1).t().contiguous()
    M = x0t.shape[1]
    out = torch.empty(M, dtype=torch.float32, device=x0t.device)
    lwd = None if lw is None else _dev.as_f32(lw).reshape(-1).contiguous()
    if isinstance(ssm_scenario, StochasticVolatility):
        phi, pq = ssm_scenario.transition_constants()
        call("mgb_transition_potential_pairs_sv", float(phi), float(pq), M, _dev.ptr(x0t), _dev.ptr(x1t),
             _dt(t_prev, t_new), _dev.ptr(lwd), _dev.ptr(out), _dev.stream_ptr())
        return out
    if isinstance(ssm_scenario, NonLinear1DBenchmark):
        call("mgb_transition_potential_pairs_nl1d", ctypes.byref(ssm_scenario.derived()[1]), M, _dev.ptr(x0t),
             _dev.ptr(x1t), float(t_prev), _dev.ptr(lwd), _dev.ptr(out), _dev.stream_ptr())
        return out
    _, s = _transition_struct(ssm_scenario)
    call("mgb_transition_potential_pairs", ctypes.byref(s), M, _dev.ptr(x0t), _dev.ptr(x1t), _dev.ptr(lwd),
         _dev.ptr(out), _dev.stream_ptr())
    return out


def full_stitch(ssm_scenario, x0_all, t, x1_all, tplus1, x1_log_weight, random_key):
    """online_smoothing.py:33-41: for each x0_j a categorical draw over the x1_i with
    log-weights x1_log_weight - transition_potential(x0_j -> x1_i); keys split(key, len(x0))."""
    x0t = _dev.as_f32(x0_all).t().contiguous()
    x1t = _dev.as_f32(x1_all).t().contiguous()
    M0, M1 = x0t.shape[1], x1t.shape[1]
    lw = _dev.as_f32(x1_log_weight).reshape(-1).contiguous()
    idx = torch.empty(M0, dtype=torch.int32, device=x0t.device)
    if isinstance(ssm_scenario, StochasticVolatility):
        phi, pq = ssm_scenario.transition_constants()
        call("mgb_stitch_sv", float(phi), float(pq), M0, M1, _dev.ptr(x0t), _dev.ptr(x1t), _dev.ptr(lw),
             _dt(t, tplus1), _dev.ptr(_dev.as_key(random_key)), _dev.ptr(idx), _dev.stream_ptr())
        return idx
    if isinstance(ssm_scenario, NonLinear1DBenchmark):
        call("mgb_stitch_nl1d", ctypes.byref(ssm_scenario.derived()[1]), M0, M1, _dev.ptr(x0t), _dev.ptr(x1t),
             _dev.ptr(lw), float(t), _dev.ptr(_dev.as_key(random_key)), _dev.ptr(idx), _dev.stream_ptr())
        return idx
    _, s = _transition_struct(ssm_scenario)
    call("mgb_stitch_lg", ctypes.byref(s), M0, M1, _dev.ptr(x0t), _dev.ptr(x1t), _dev.ptr(lw),
         _dev.ptr(_dev.as_key(random_key)), _dev.ptr(idx), _dev.stream_ptr())
    return idx


def rejection_stitching(ssm_scenario, x0_all, t, x1_all, tplus1, x1_log_weight, random_key, maximum_rejections,
                        init_bound_param=0.0, bound_inflation=1.01):
    """online_smoothing.py:129-175: for each x0_i an index into x1_all by rejection sampling
    against exp(-transition_potential), the full categorical for those still unaccepted after
    maximum_rejections rounds.  Returns (indices (M,), transition evaluations)."""
    x0t = _dev.as_f32(x0_all).t().contiguous()
    x1t = _dev.as_f32(x1_all).t().contiguous()
    M, d = x1t.shape[1], x1t.shape[0]
    if x0t.shape[1] != M:
        raise ValueError(f"rejection stitching pairs x0_all ({x0t.shape[1]}) with x1_all ({M}) one to one")
    lw = _dev.as_f32(x1_log_weight).reshape(-1).contiguous()
    dev = x0t.device
    idx = torch.empty(M, dtype=torch.int32, device=dev)
    evals = torch.empty(1, dtype=torch.int64, device=dev)
    cfg = _lib.RejectionConfig(int(maximum_rejections), float(init_bound_param), float(bound_inflation))
    ws = _dev.workspace(_lib.lib().mgb_stitch_rejection_workspace(M, d), dev)
    key = _dev.as_key(random_key)
    if isinstance(ssm_scenario, StochasticVolatility):
        phi, pq = ssm_scenario.transition_constants()
        call("mgb_stitch_rejection_sv", float(phi), float(pq), ctypes.byref(cfg), M, _dev.ptr(x0t), _dev.ptr(x1t),
             _dev.ptr(lw), _dt(t, tplus1), _dev.ptr(key), _dev.ptr(idx), _dev.ptr(evals), _dev.ptr(ws), ws.numel(),
             _dev.stream_ptr())
    elif isinstance(ssm_scenario, NonLinear1DBenchmark):
        call("mgb_stitch_rejection_nl1d", ctypes.byref(ssm_scenario.derived()[1]), ctypes.byref(cfg), M,
             _dev.ptr(x0t), _dev.ptr(x1t), _dev.ptr(lw), float(t), _dev.ptr(key), _dev.ptr(idx), _dev.ptr(evals),
             _dev.ptr(ws), ws.numel(), _dev.stream_ptr())
    else:
        _, s = _transition_struct(ssm_scenario)
        call("mgb_stitch_rejection_lg", ctypes.byref(s), ctypes.byref(cfg), M, _dev.ptr(x0t), _dev.ptr(x1t),
             _dev.ptr(lw), _dev.ptr(key), _dev.ptr(idx), _dev.ptr(evals), _dev.ptr(ws), ws.numel(),
             _dev.stream_ptr())
    return idx, int(evals.item())


def fixed_lag_stitching(ssm_scenario, early_block, t, recent_block, recent_block_log_weight, tplus1, random_key,
                        maximum_rejections=0, init_bound_param=0.0, bound_inflation=1.01):
    """online_smoothing.py:178-209: returns (stitched value, transition evaluations); full
    stitching for maximum_rejections = 0, rejection stitching otherwise."""
    x0_fixed_all = early_block[-1]
    x0_vary_all, x1_vary_all = recent_block[0], recent_block[1]
    nilw = _pair_potential(ssm_scenario, x0_vary_all, x1_vary_all, recent_block_log_weight, t, tplus1)
    if maximum_rejections > 0:
        inds, evals = rejection_stitching(ssm_scenario, x0_fixed_all, t, x1_vary_all, tplus1, nilw, random_key,
                                          maximum_rejections, init_bound_param, bound_inflation)
        return torch.cat([early_block, recent_block[1:, inds.long()]], 0), evals
    inds = full_stitch(ssm_scenario, x0_fixed_all, t, x1_vary_all, tplus1, nilw, random_key).long()
    return torch.cat([early_block, recent_block[1:, inds]], 0), len(x0_fixed_all) ** 2


def _check_smoother(ssm_scenario, particle_filter):
    _check_lg(ssm_scenario, particle_filter)
    if isinstance(ssm_scenario, StochasticVolatility) and ssm_scenario.dim != 1:
        raise NotImplementedError("StochasticVolatility: the smoothing kernels take dim = 1")
    if isinstance(ssm_scenario, TimeHomogenousLinearGaussian) and not ssm_scenario.gpu_runtime_supported():
        raise NotImplementedError(f"(d, dy) = ({ssm_scenario.dim}, {ssm_scenario.dim_obs}) above the "
                                  f"run-time-dimension limit ({LG_RUNTIME_MAX})")
    if not isinstance(particle_filter, BootstrapFilter):
        raise NotImplementedError("the online smoother runs the bootstrap filter")


def propagate_particle_smoother_pf(ssm_scenario, particle_filter, particles, y_new, t_new, random_key, lag,
                                   maximum_rejections=0, init_bound_param=0.0, bound_inflation=1.01,
                                   resampling="systematic"):
    """online_smoothing.py:212-282: resample unless unweighted, propagate, append, then
    stitch the block that leaves the lag window.  The same key drives the resampling,
    the proposal and the stitch, as in the reference."""
    _check_smoother(ssm_scenario, particle_filter)
    prefix, s = _kernels(ssm_scenario, particle_filter)
    key = _dev.as_key(random_key)
    n = particles.value.shape[1]
    out = particles.copy()
    if not hasattr(out, "num_transition_evals"):
        out.num_transition_evals = torch.zeros(1, device=particles.value.device)
    lw_last = particles.log_weight if particles.log_weight.dim() == 1 else particles.log_weight[-1]
    if float(ess_log_weight(lw_last)) < n - 1e-3:
        out = resample_particles(out, key, True, resampling)
    x_prev = out.value[-1].t().contiguous()
    y_t = _y2(y_new, ssm_scenario.dim_obs).reshape(-1)
    x_new, lw = _step(s, n, key, y_t, x_prev, None, None, prefix, t_prev=out.t[-1], t_new=t_new)
    dev = x_new.device
    out.value = torch.cat([out.value, x_new.t()[None]], 0)
    out.y = torch.cat([out.y, y_t[None]], 0) if getattr(out, "y", None) is not None else y_t[None]
    out.t = torch.cat([out.t, torch.atleast_1d(torch.as_tensor(t_new, device=dev)).to(out.t.dtype)])
    out.ess = ess_log_weight(lw).reshape(1).float()
    len_t = out.t.numel()
    s1 = len_t - lag - 1
    nte = 0
    if s1 >= 0:
        out.value, nte = fixed_lag_stitching(ssm_scenario, out.value[:s1 + 1], out.t[s1], out.value[s1:], lw,
                                             out.t[s1 + 1], key, maximum_rejections, init_bound_param,
                                             bound_inflation)
    out.num_transition_evals = torch.cat([out.num_transition_evals,
                                          torch.tensor([float(nte)], device=dev)])
    out.log_weight = torch.zeros(n, device=dev) if s1 >= 0 else lw
    return out


def propagate_particle_smoother_bs(ssm_scenario, particle_filter, particles, y_new, t_new, random_key, lag,
                                   ess_threshold=0.5, maximum_rejections=0, init_bound_param=0.0,
                                   bound_inflation=1.01, resampling="systematic"):
    """online_smoothing.py:285-366: propagate the marginal filter, then backward-simulate
    the last lag + 1 steps and stitch them onto the fixed block."""
    _check_smoother(ssm_scenario, particle_filter)
    key = _dev.as_key(random_key)
    n = particles.value.shape[1]
    out = particles.copy()
    if not hasattr(out, "num_transition_evals"):
        out.num_transition_evals = torch.zeros(1, device=particles.value.device)
    if not hasattr(out, "marginal_filter"):
        out.marginal_filter = cdict(value=particles.value, log_weight=particles.log_weight, y=particles.y,
                                    t=particles.t, ess=particles.ess)
    split_keys = mrandom.split(key, 4)
    out.marginal_filter = propagate_particle_filter(ssm_scenario, particle_filter, out.marginal_filter, y_new, t_new,
                                                    split_keys[1], ess_threshold, False, resampling)
    dev = out.marginal_filter.value.device
    y_t = _y2(y_new, ssm_scenario.dim_obs).reshape(-1)
    out.y = torch.cat([out.y, y_t[None]], 0) if getattr(out, "y", None) is not None else y_t[None]
    out.t = torch.cat([out.t, torch.atleast_1d(torch.as_tensor(t_new, device=dev)).to(out.t.dtype)])
    out.log_weight = torch.zeros(n, device=dev)
    out.ess = out.marginal_filter.ess[-1:]
    len_t = out.t.numel()
    s1 = len_t - lag - 1
    if s1 >= 0:
        bsim = backward_simulation(ssm_scenario, out.marginal_filter[s1:], split_keys[2], n, maximum_rejections,
                                   init_bound_param, bound_inflation)
        out.value, snte = fixed_lag_stitching(ssm_scenario, out.value[:s1 + 1], out.t[s1], bsim.value,
                                              torch.zeros(n, device=dev), out.t[s1 + 1], key, maximum_rejections,
                                              init_bound_param, bound_inflation)
        nte = snte + float(bsim.num_transition_evals.sum())
    else:
        bsim = backward_simulation(ssm_scenario, out.marginal_filter, split_keys[2], n, maximum_rejections,
                                   init_bound_param, bound_inflation)
        out.value, nte = bsim.value, float(bsim.num_transition_evals.sum())
    out.num_transition_evals = torch.cat([out.num_transition_evals, torch.tensor([float(nte)], device=dev)])
    return out


def propagate_particle_smoother(ssm_scenario, particle_filter, particles, y_new, t_new, random_key, lag,
                                backward_sim=True, ess_threshold=0.5, maximum_rejections=0, init_bound_param=0.0,
                                bound_inflation=1.01, resampling="systematic"):
    """Online fixed-lag particle smoothing (online_smoothing.py:369-386)."""
    if backward_sim:
        return propagate_particle_smoother_bs(ssm_scenario, particle_filter, particles, y_new, t_new, random_key,
                                              lag, ess_threshold, maximum_rejections, init_bound_param,
                                              bound_inflation, resampling)
    return propagate_particle_smoother_pf(ssm_scenario, particle_filter, particles, y_new, t_new, random_key, lag,
                                          maximum_rejections, init_bound_param, bound_inflation, resampling)
