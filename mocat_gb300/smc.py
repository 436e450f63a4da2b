"""Tempered SMC sampler (mocat/src/transport/smc.py:100-373) with Underdamped / MALA / HMC
or RandomWalk moves (mocat/src/mcmc/standard_mcmc.py:20-153) and the Metropolis correction
(mocat/src/mcmc/metropolis.py:48-70), adaptive or scheduled temperatures, driven as
mocat.run (mocat/src/sample.py:110-148), running on the GPU for B independent posteriors
at once, on Bayesian logistic regression or the Gaussian toy scenario.

    scenario = LogisticRegression(X, y, prior_scale=1.0)
    sampler = MetropolisedSMCSampler(Underdamped(stepsize=0.01), mcmc_steps=5, ess_threshold_retain=0.5)
    out = run(scenario, sampler, n=16384, random_key=PRNGKey(0))             # one posterior
    outs = run_batched(scenario, sampler, n=16384, random_keys=keys)          # B posteriors
    run(Gaussian(covariance=S, prior_scale=49.0, prior_sample_scale=7.0),
        MetropolisedSMCSampler(RandomWalk(stepsize=1.0)), 10000, key, temperature_schedule=sched)

Differences from the reference, by design:
  * resampling (ess <= ess_threshold_resample n) is systematic, O(n), by default;
    MetropolisedSMCSampler(..., resampling="categorical") draws the reference's
    random.categorical instead (smc.py:61-71: O(n^2) Gumbel-max draws);
  * run() returns the reference's stacked chain for value and log_weight; run_batched
    keeps the final particles of every posterior (chain=True adds the stacked chain);
  * ``precision="bf16"`` evaluates the likelihood potential and its gradient on
    the tensor cores (bf16 operands, float32 accumulation); "fp32" on the CUDA cores.
"""
import ctypes
import math

import numpy as np
import torch

from . import _dev, _lib
from ._lib import call
from .core import Scenario, cdict

PRECISIONS = {"fp32": 0, "bf16": 1}
SUPPORTED_D = (2, 3, 5, 10, 20, 50)
MAX_N = 24576  # MGB_SMC_MAX_N


class LogisticRegression(Scenario):
    """beta ~ N(0, prior_scale^2 I), y_i ~ Bernoulli(sigmoid(x_i . beta)).

    prior_potential = |beta|^2 / (2 s^2); likelihood_potential = sum_i softplus(x_i . beta) - y_i x_i . beta."""
    name = "Logistic Regression"

    def __init__(self, X, y, prior_scale=1.0, name=None):
        X = torch.as_tensor(np.asarray(X.cpu() if isinstance(X, torch.Tensor) else X, np.float32))
        y = torch.as_tensor(np.asarray(y.cpu() if isinstance(y, torch.Tensor) else y, np.float32)).reshape(-1)
        if X.ndim != 2 or X.shape[0] != y.shape[0]:
            raise ValueError("X must be (n_data, d) and y (n_data,)")
        self.dim = X.shape[1]
        self.prior_scale = float(prior_scale)
        dev = _dev.device()
        self.X = X.contiguous().to(dev)
        self.y = y.contiguous().to(dev)
        self._Xbf16 = None
        super().__init__(name=name)

    @property
    def n_data(self):
        return self.X.shape[0]

    def Xbf16(self):
        """(n_data, 64) bf16 copy of X, zero-padded to 64 features (tensor-core operand)."""
        if self._Xbf16 is None:
            if self.dim > 64:
                raise NotImplementedError("the tensor-core path takes d <= 64")
            xb = torch.zeros((self.n_data, 64), dtype=torch.bfloat16, device=self.X.device)
            xb[:, :self.dim] = self.X.to(torch.bfloat16)
            self._Xbf16 = xb.contiguous()
        return self._Xbf16

    def prior_potential(self, x, random_key=None):
        x = _dev.as_f32(x)
        return 0.5 * (x * x).sum(-1) / self.prior_scale ** 2

    def likelihood_potential_and_grad(self, x, random_key=None, precision="fp32"):
        """(likelihood potential (P,), gradient (P, d)) for parameter rows x (P, d) on the GPU."""
        x = _dev.as_f32(x)
        squeeze = x.ndim == 1
        x = x.reshape(-1, self.dim).contiguous()
        P = x.shape[0]
        pr = PRECISIONS[precision]
        ws = _dev.workspace(_lib.lib().mgb_logreg_workspace(P, self.n_data, self.dim, pr))
        lik = torch.empty(P, dtype=torch.float32, device=x.device)
        grad = torch.empty((P, self.dim), dtype=torch.float32, device=x.device)
        xb = self.Xbf16() if pr == 1 else None
        call("mgb_logreg_potential_grad", _dev.ptr(self.X), _dev.ptr(self.y), self.n_data, self.dim, _dev.ptr(x), P,
             _dev.ptr(lik), _dev.ptr(grad), pr, _dev.ptr(xb), _dev.ptr(ws), ws.numel(), _dev.stream_ptr())
        return (lik[0], grad[0]) if squeeze else (lik, grad)

    def likelihood_potential(self, x, random_key=None):
        return self.likelihood_potential_and_grad(x)[0]


class Underdamped:
    """Underdamped Langevin proposal (standard_mcmc.py:72-153): leapfrog_steps leapfrog steps of
    the tempered potential, momenta refreshed by the OU solution with the given friction
    (infinite friction: fresh momenta, i.e. HMC, and MALA for one leapfrog step)."""
    name = "Underdamped"

    def __init__(self, stepsize=None, leapfrog_steps=1, friction=math.inf):
        self.stepsize = stepsize
        self.leapfrog_steps = int(leapfrog_steps)
        self.friction = float(friction)


class RandomWalk:
    """Random-walk proposal x + sqrt(stepsize) N(0, I) (standard_mcmc.py:20-64)."""
    name = "Random Walk"

    def __init__(self, stepsize=None):
        self.stepsize = stepsize


class Gaussian(Scenario):
    """toy_examples.Gaussian (mocat/src/scenarios/toy_examples.py:17-51): likelihood potential
    0.5 |(x - mean) @ precision_sqrt^T|^2 with precision_sqrt = inv(chol(covariance)).  The GPU
    sampler's prior is N(0, prior_scale^2 I) in the potential (prior_scale = inf: flat) and draws
    prior_sample_scale N(0, I) (defaults to prior_scale), covering a scenario whose prior_sample
    and prior_potential are set separately."""
    name = "Gaussian"

    def __init__(self, dim=None, mean=None, covariance=None, prior_scale=1.0, prior_sample_scale=None, name=None):
        if covariance is not None:
            cov = np.asarray(covariance.cpu() if isinstance(covariance, torch.Tensor) else covariance, np.float64)
            d = cov.shape[-1] if cov.ndim else (int(dim) if dim is not None else 1)
        else:
            d = int(dim) if dim is not None else (np.asarray(mean).shape[-1] if mean is not None else 1)
            cov = np.ones(d)
        if cov.ndim < 2:
            cov = np.diag(np.broadcast_to(cov, (d,)))
        self.dim = d
        self.mean = np.zeros(d) if mean is None else np.asarray(mean, np.float64).reshape(d)
        self.covariance = cov
        self.precision_sqrt = np.linalg.inv(np.linalg.cholesky(cov))
        self.prior_scale = float(prior_scale)
        self.prior_sample_scale = self.prior_scale if prior_sample_scale is None else float(prior_sample_scale)
        self._dc = None
        super().__init__(name=name)

    def device_constants(self):
        """(mean, precision_sqrt) as float32 device tensors, uploaded on first use"""
        if self._dc is None:
            dev = _dev.device()
            self._dc = (torch.as_tensor(self.mean.astype(np.float32), device=dev).contiguous(),
                        torch.as_tensor(self.precision_sqrt.astype(np.float32), device=dev).contiguous())
        return self._dc

    def prior_potential(self, x, random_key=None):
        x = _dev.as_f32(x)
        return 0.5 * (x * x).sum(-1) / self.prior_scale ** 2

    def likelihood_potential(self, x, random_key=None):
        m, ps = self.device_constants()
        z = (_dev.as_f32(x) - m) @ ps.T
        return 0.5 * (z * z).sum(-1)


class MetropolisedSMCSampler:
    """Tempered SMC with MCMC moves (smc.py:229-373), adaptive temperatures or a
    temperature_schedule (its leading 0 removed; max_temperature and max_iter follow it,
    smc.py:113-125, :243-245)."""
    name = "Metropolised SMC Sampler"

    def __init__(self, mcmc_sampler, mcmc_correction="sampler_default", mcmc_steps=1, max_iter=int(1e4),
                 temperature_schedule=None, max_temperature=1.0, ess_threshold_retain=0.9,
                 ess_threshold_resample=0.5, bisection_tol=1e-5, max_bisection_iter=1000, resampling="systematic"):
        if isinstance(mcmc_sampler, type):
            mcmc_sampler = mcmc_sampler()
        if mcmc_correction not in ("sampler_default", "Metropolis"):
            raise NotImplementedError("the GPU sampler uses the Metropolis correction")
        if not isinstance(mcmc_sampler, (Underdamped, RandomWalk)) or mcmc_sampler.stepsize is None:
            raise NotImplementedError("the GPU sampler moves with Underdamped(stepsize, ...) or RandomWalk(stepsize)")
        if isinstance(mcmc_sampler, Underdamped) and mcmc_sampler.leapfrog_steps < 1:
            raise ValueError("leapfrog_steps must be >= 1")
        self.mcmc_sampler = mcmc_sampler
        self.mcmc_steps = int(mcmc_steps)
        self.max_iter = int(max_iter)
        self.max_temperature = float(max_temperature)
        self.ess_threshold_retain = float(ess_threshold_retain)
        self.ess_threshold_resample = float(ess_threshold_resample)
        self.bisection_tol = float(bisection_tol)
        self.max_bisection_iter = int(max_bisection_iter)
        if resampling not in ("systematic", "categorical"):
            raise NotImplementedError(f"resampling {resampling!r}: the GPU sampler resamples 'systematic' or "
                                      "'categorical'")
        self.resampling = resampling
        self.temperature_schedule = None
        self.set_schedule(temperature_schedule)

    def set_schedule(self, temperature_schedule):
        """TemperedSMCSampler.__setattr__ (smc.py:113-125, :261-265)"""
        if temperature_schedule is None:
            self.temperature_schedule = None
            return
        sch = np.asarray(temperature_schedule.cpu() if isinstance(temperature_schedule, torch.Tensor)
                         else temperature_schedule, np.float32).reshape(-1)
        if sch.size and sch[0] == 0.0:
            sch = sch[1:]
        if sch.size == 0:
            raise ValueError("empty temperature schedule")
        self.temperature_schedule = sch
        self.max_temperature = float(sch[-1])
        self.max_iter = int(sch.size)


class BatchedSMC:
    """B posteriors of one scenario advanced together; ``init()`` then ``step()`` until
    ``done()``, or ``run()``.  The workspace stays on the device between calls."""

    def __init__(self, scenario, sampler, n, random_keys, precision="fp32", max_iter=None):
        gauss = isinstance(scenario, Gaussian)
        if not gauss and not isinstance(scenario, LogisticRegression):
            raise NotImplementedError(f"{scenario.__class__.__name__}: no GPU SMC kernel for this scenario")
        if scenario.dim not in SUPPORTED_D:
            raise NotImplementedError(f"d = {scenario.dim} not compiled (supported {SUPPORTED_D})")
        if not 2 <= n <= MAX_N:
            raise NotImplementedError(f"n must be in [2, {MAX_N}]")
        keys = _dev.as_key(random_keys).reshape(-1, 2).contiguous()
        self.scenario, self.sampler = scenario, sampler
        self.B, self.n = keys.shape[0], int(n)
        mi = sampler.max_iter if max_iter is None else int(max_iter)
        mv = sampler.mcmc_sampler
        rw = isinstance(mv, RandomWalk)
        sch = sampler.temperature_schedule
        self._sched = None if sch is None else torch.as_tensor(sch, device=keys.device).contiguous()
        fr = 0.0 if rw or not math.isfinite(mv.friction) else float(mv.friction)
        self.cfg = _lib.SMCConfig(self.B, self.n, scenario.dim, sampler.mcmc_steps, mv.stepsize,
                                  scenario.prior_scale, sampler.ess_threshold_retain, sampler.ess_threshold_resample,
                                  sampler.bisection_tol, sampler.max_bisection_iter, sampler.max_temperature,
                                  min(mi, 100000), PRECISIONS[precision], 1 if rw else 0,
                                  1 if rw else mv.leapfrog_steps, fr,
                                  getattr(scenario, "prior_sample_scale", scenario.prior_scale),
                                  0 if sch is None else len(sch), _dev.ptr(self._sched), 1 if gauss else 0,
                                  _dev.ptr(scenario.device_constants()[0]) if gauss else None,
                                  _dev.ptr(scenario.device_constants()[1]) if gauss else None,
                                  2 if getattr(sampler, "resampling", "systematic") == "categorical" else 0)
        self.keys = keys
        self.Xb = scenario.Xbf16() if precision == "bf16" and not gauss else None
        self.ws = _dev.workspace(_lib.lib().mgb_smc_logreg_workspace(ctypes.byref(self.cfg), self._n_data()))
        self.views = _lib.SMCViews()
        call("mgb_smc_logreg_views", ctypes.byref(self.cfg), _dev.ptr(self.ws), ctypes.byref(self.views))
        self.iterations = 0

    def _n_data(self):
        return self.scenario.n_data if isinstance(self.scenario, LogisticRegression) else 1

    def _args(self):
        sc = self.scenario
        if isinstance(sc, Gaussian):
            return (ctypes.byref(self.cfg), None, None, None, 1)
        return (ctypes.byref(self.cfg), _dev.ptr(sc.X), _dev.ptr(sc.y), _dev.ptr(self.Xb), sc.n_data)

    def _tensor(self, name, shape, dtype):
        n = int(np.prod(shape))
        ptr = getattr(self.views, name)
        store = self.ws.view(torch.uint8)
        off = ptr - self.ws.data_ptr()
        nbytes = n * torch.tensor([], dtype=dtype).element_size()
        return store[off:off + nbytes].view(dtype).reshape(shape)

    def init(self):
        call("mgb_smc_logreg_init", *self._args(), _dev.ptr(self.keys), _dev.ptr(self.ws), self.ws.numel(),
             _dev.stream_ptr())
        self.iterations = 0

    def step(self):
        call("mgb_smc_logreg_step", *self._args(), _dev.ptr(self.ws), self.ws.numel(), _dev.stream_ptr())
        self.iterations += 1

    def done(self):
        return not bool(self._tensor("active", (self.B,), torch.int32).any())

    def run(self, chain=False):
        """to termination; chain=True also records value, log_weight after the startup and
        every iteration (the reference's stacked chain), as result().chain_*"""
        self._chain = {k: [] for k in ('value', 'log_weight')} if chain else None
        self.init()
        if chain:
            self._snap()
        while not self.done() and self.iterations < self.cfg.max_iter:
            self.step()
            if chain:
                self._snap()
        out = self.result()
        if chain:
            for k, v in self._chain.items():
                out.__dict__["chain_" + k] = torch.stack(v)
        return out

    def _d(self):
        return self.cfg.d

    def _snap(self):
        self._chain["value"].append(self._tensor("value", (self.B, self.n, self._d()), torch.float32).clone())
        self._chain["log_weight"].append(self._tensor("log_weight", (self.B, self.n), torch.float32).clone())

    def prior_scale_grad(self):
        """(B,) d log Z / d prior_scale at the current particles (Fisher identity)."""
        out = torch.empty(self.B, dtype=torch.float64, device=self.ws.device)
        call("mgb_smc_logreg_prior_scale_grad", ctypes.byref(self.cfg), _dev.ptr(self.ws), _dev.ptr(out),
             _dev.stream_ptr())
        return out

    def result(self):
        B, n, d, H = self.B, self.n, self.cfg.d, self.views.hist_len
        it = self._tensor("iter", (B,), torch.int32).clone()
        L = int(it.max()) + 1
        return cdict(value=self._tensor("value", (B, n, d), torch.float32).clone(),
                     log_weight=self._tensor("log_weight", (B, n), torch.float32).clone(),
                     likelihood_potential=self._tensor("likelihood_potential", (B, n), torch.float32).clone(),
                     temperature=self._tensor("hist_temperature", (B, H), torch.float32)[:, :L].clone(),
                     log_norm_constant=self._tensor("hist_log_norm_constant", (B, H), torch.float64)[:, :L].clone(),
                     ess=self._tensor("hist_ess", (B, H), torch.float32)[:, :L].clone(),
                     alpha=self._tensor("hist_alpha", (B, H), torch.float32)[:, :L].clone(),
                     resampled=self._tensor("hist_resampled", (B, H), torch.int32)[:, :L].bool(),
                     iterations=it, grad_log_norm_constant_prior_scale=self.prior_scale_grad())


def run_batched(scenario, sampler, n, random_keys, precision="fp32", temperature_schedule=None, chain=False):
    """mocat.run(scenario, sampler, n, key) for each of B keys, in one batch.  Fields carry a
    leading B axis; per-iteration arrays are padded past each posterior's last iteration.
    temperature_schedule (a run() keyword in the reference) sets the sampler's schedule;
    chain=True adds chain_value (L, B, n, d) and chain_log_weight (L, B, n)."""
    if temperature_schedule is not None:
        sampler.set_schedule(temperature_schedule)
    return BatchedSMC(scenario, sampler, n, random_keys, precision).run(chain)


def run(scenario, sampler, n, random_key, precision="fp32", temperature_schedule=None):
    """mocat.run (sample.py:110-148) for MetropolisedSMCSampler on a LogisticRegression or
    Gaussian scenario, with the reference's stacked layout: value (L, n, d) and log_weight (L, n)
    after the startup and every iteration, temperature, log_norm_constant, ess, alpha (L,)."""
    out = run_batched(scenario, sampler, n, _dev.as_key(random_key).reshape(1, 2), precision, temperature_schedule,
                      chain=True)
    L = int(out.iterations[0]) + 1
    return cdict(value=out.chain_value[:L, 0], log_weight=out.chain_log_weight[:L, 0],
                 likelihood_potential=out.likelihood_potential[0], temperature=out.temperature[0, :L],
                 log_norm_constant=out.log_norm_constant[0, :L], ess=out.ess[0, :L], alpha=out.alpha[0, :L],
                 resampled=out.resampled[0, :L])
