"""Likelihood-free SMC (ABC-SMC) on the GPU with mocat's names
(mocat/src/abc/abc.py, abc/mcmc.py, abc/smc.py, abc/scenarios/linear_gaussian.py, abc/scenarios/gk.py).

    scenario = LinearGaussian(prior_mean, prior_covariance, data, likelihood_matrix, likelihood_covariance)
    sampler = MetropolisedABCSMCSampler(ess_threshold_retain=0.8)           # RandomWalkABC moves
    out = run(scenario, sampler, n=1000, random_key=PRNGKey(0))             # one posterior
    outs = run_batched(scenario, sampler, n=1000, random_keys=keys)         # B posteriors

Differences from the reference, by design:
  * resampling (ess < ess_threshold_resample n) is systematic, O(n), instead of
    random.categorical;
  * run() returns the reference's stacked chain for value, log_weight and distance;
    run_batched keeps the final particles of every posterior (chain=True adds the chain);
  * the stepsize variance and the mean acceptance are float64 sums in a fixed
    order.
"""
import ctypes
import math

import numpy as np
import torch

from . import _dev, _lib
from ._lib import call
from .core import Scenario, cdict

SUPPORTED = {(1, 1), (2, 1), (2, 2), (3, 2), (3, 3), (5, 5), (10, 10)}
MAX_N = 65536  # MGB_ABC_MAX_N


def _arr(a, shape=None):
    a = np.asarray(a.cpu() if isinstance(a, torch.Tensor) else a, np.float64)
    return a if shape is None else a.reshape(shape)


class ABCScenario(Scenario):
    """Scenario whose likelihood can be simulated but not evaluated (abc/abc.py:15-39)."""
    data = None

    def potential(self, x, random_key=None):
        raise TypeError(f"{self.name} abc_scenario potential is intractable")

    def likelihood_potential(self, x, random_key=None):
        raise TypeError(f"{self.name} abc_scenario likelihood_potential is intractable")

    def distance_function(self, simulated_data):
        d = torch.as_tensor(simulated_data) - torch.as_tensor(np.asarray(self.data, np.float32),
                                                                 device=torch.as_tensor(simulated_data).device)
        return torch.sqrt((d * d).sum(-1))


class LinearGaussian(ABCScenario):
    """x ~ N(prior_mean, prior_covariance), data ~ N(likelihood_matrix x, likelihood_covariance)
    (abc/scenarios/linear_gaussian.py).  Square roots follow reset_covariance
    (mocat/src/utils.py:247-262): Cholesky factors and their inverses."""
    name = "Linear Gaussian"

    def __init__(self, prior_mean=0.0, prior_covariance=1.0, data=0.0, likelihood_matrix=1.0,
                 likelihood_covariance=1.0, name=None):
        super().__init__(name=name)
        m0 = _arr(prior_mean)
        self.dim = m0.size if m0.ndim else None
        for a in (prior_covariance, likelihood_matrix, likelihood_covariance):
            if self.dim is None and np.ndim(_arr(a)) > 0:
                self.dim = _arr(a).shape[-1]
        if self.dim is None:
            raise AttributeError(f"Could not find dimension for {self.__class__.__name__}")
        d = self.dim
        self.prior_mean = np.ones(d) * m0 if m0.ndim == 0 else m0.reshape(d)
        S0 = _arr(prior_covariance)
        self.prior_covariance = np.eye(d) * S0 if S0.ndim == 0 else S0
        H = _arr(likelihood_matrix)
        self.likelihood_matrix = np.eye(d) * H if H.ndim == 0 else H
        self.dim_obs = self.likelihood_matrix.shape[0]
        R = _arr(likelihood_covariance)
        self.likelihood_covariance = np.eye(self.dim_obs) * R if R.ndim == 0 else R
        self.data = np.ones(self.dim_obs) * _arr(data) if np.ndim(data) == 0 else _arr(data).reshape(self.dim_obs)

    def derived(self):
        """float32 constants of the kernels and the C-ABI model struct"""
        d = self.dim
        C0 = np.linalg.cholesky(self.prior_covariance)
        keep = dict(m0=self.prior_mean, C0=C0, P0=np.linalg.inv(C0), H=self.likelihood_matrix,
                    L=np.linalg.cholesky(self.likelihood_covariance), data=self.data)
        keep = {k: np.ascontiguousarray(np.asarray(v, np.float32)) for k, v in keep.items()}
        keep["c0"] = np.float32((d * math.log(2 * math.pi) + math.log(np.linalg.det(self.prior_covariance))) / 2)
        s = _lib.ABCModel(d, self.dim_obs, keep["m0"].ctypes.data, keep["C0"].ctypes.data, keep["P0"].ctypes.data,
                          float(keep["c0"]), keep["H"].ctypes.data, keep["L"].ctypes.data, keep["data"].ctypes.data)
        return keep, s

    def prior_sample(self, random_key):
        from . import random as mrandom
        e = mrandom.normal(random_key, (self.dim,)).cpu().numpy().astype(np.float64)
        return self.prior_mean + np.linalg.cholesky(self.prior_covariance) @ e


class GKTransformedUniformPrior(ABCScenario):
    """g-and-k distribution with a N(0, I) prior on unconstrained parameters
    (abc/scenarios/gk.py:81-116, constrain lo + Phi(x) (hi - lo)), summarised by thinned
    order statistics as the reference's GK tests do (tests/test_abc_gk.py GKThinOrder):
    the sorted n_unsummarised_data draws at ranks floor(j n / num_thin).  Simulations run
    on the GPU, one CTA per parameter row (mgb_abc_gk_simulate)."""
    name = "GK_fewN"
    dim = 4
    c = 0.8
    prior_mins = 0.0
    prior_maxs = 10.0
    buffer = 1e-5

    def __init__(self, n_unsummarised_data=1000, num_thin=100, data=None, name=None):
        super().__init__(name=name)
        self.n_unsummarised_data = int(n_unsummarised_data)
        self.num_thin = int(num_thin)
        self.data = None if data is None else _arr(data).reshape(-1)

    def constrain(self, unconstrained_x):
        x = torch.as_tensor(np.asarray(unconstrained_x, np.float64))
        return (self.prior_mins + torch.special.ndtr(x) * (self.prior_maxs - self.prior_mins)).numpy()

    def unconstrain(self, constrained_x):
        x = torch.as_tensor(np.asarray(constrained_x, np.float64))
        return torch.special.ndtri((x - self.prior_mins) / (self.prior_maxs - self.prior_mins)).numpy()

    def model(self, data_dev=None):
        return _lib.GKModel(self.dim, self.n_unsummarised_data, self.num_thin, self.c, self.prior_mins,
                            self.prior_maxs, self.buffer, data_dev)

    def prior_potential(self, x, random_key=None):
        x = _arr(x)
        return 0.5 * (x ** 2).sum(-1)

    def prior_sample(self, random_key):
        from . import random as mrandom
        return mrandom.normal(random_key, (self.dim,)).cpu().numpy().astype(np.float64)

    def simulate_summaries(self, x, random_keys):
        """likelihood_sample for parameter rows x (P, d) with keys (P, 2): (P, num_thin) on the GPU"""
        xs = _dev.as_f32(x).reshape(-1, self.dim).contiguous()
        keys = _dev.as_key(random_keys).reshape(-1, 2).contiguous()
        out = torch.empty((xs.shape[0], self.num_thin), dtype=torch.float32, device=xs.device)
        call("mgb_abc_gk_simulate", ctypes.byref(self.model()), xs.shape[0], _dev.ptr(xs), _dev.ptr(keys),
             _dev.ptr(out), None, _dev.stream_ptr())
        return out

    def likelihood_sample(self, x, random_key):
        return self.simulate_summaries(_arr(x).reshape(1, -1), _dev.as_key(random_key).reshape(1, 2))[0]


class GKOnlyATransformedUniformPrior(GKTransformedUniformPrior):
    """the A-only g-and-k scenario (abc/scenarios/gk.py:138-175): B = 1, g = 2, and the exponent
    of (1 + z^2) is c, as the reference writes it"""
    name = "GK_fewN only A"
    dim = 1


GKThinOrder = GKTransformedUniformPrior
GKOnlyAThinOrder = GKOnlyATransformedUniformPrior


class RandomWalkABC:
    """Random-walk ABC MCMC kernel (abc/mcmc.py:59-103): x + sqrt(stepsize) eps, accepted with
    probability min(1, exp(prior_potential_old - prior_potential_new) [distance_new < threshold])."""
    name = "Random Walk ABC"

    def __init__(self, threshold=None, stepsize=None):
        self.threshold = threshold
        self.stepsize = stepsize
        # the Robbins-Monro target of RMMetropolisDiagStepsize (abc/mcmc.py:44-48)
        self.tuning = cdict(parameter="threshold", target=0.1, metric="alpha", monotonicity="increasing")


class RMMetropolisDiagStepsize:
    """The adaptive correction of RandomWalkABC chains (abc/mcmc.py:105-140 over RMMetropolis,
    mcmc/metropolis.py:73-160): after every Metropolis step, a log Robbins-Monro update of the
    threshold towards sampler.tuning.target acceptance, and the per-dimension stepsize set to
    2.38^2 / d times a running estimate of the posterior variances; rm step = scale iter^-neg_exp."""

    def __init__(self, super_correction=None, adapt_cut_off=math.inf, rm_stepsize_scale=1.0,
                 rm_stepsize_neg_exponent=2.0 / 3.0, log_update=True):
        if super_correction not in (None, "Metropolis"):
            raise NotImplementedError("the GPU chain uses the Metropolis correction underneath")
        if adapt_cut_off != math.inf or not log_update:
            raise NotImplementedError("the GPU chain adapts at every step with the log update")
        self.rm_stepsize_scale = float(rm_stepsize_scale)
        self.rm_stepsize_neg_exponent = float(rm_stepsize_neg_exponent)


class VanillaABC:
    """Importance (rejection) ABC from the prior (abc/importance.py:97-118) run as mocat.run runs
    it: a chain of n prior draws with sequential keys, log_weight 0 where the distance is below
    the threshold, else -inf; with acceptance_rate the threshold becomes the acceptance_rate
    quantile of the chain's distances (clean_chain_ar) and is written back to
    parameters.threshold."""
    name = "Vanilla ABC"

    def __init__(self, threshold=math.inf, acceptance_rate=None):
        self.parameters = cdict(threshold=float(threshold))
        if acceptance_rate is not None:
            self.parameters.acceptance_rate = float(acceptance_rate)


def _run_vanilla(scenario, sampler, n, random_key):
    gk = isinstance(scenario, GKTransformedUniformPrior)
    if not gk and not isinstance(scenario, LinearGaussian):
        raise NotImplementedError(f"{scenario.__class__.__name__}: no GPU ABC kernel for this scenario")
    if not gk and (scenario.dim, scenario.dim_obs) not in SUPPORTED:
        raise NotImplementedError(f"(d, dy) = ({scenario.dim}, {scenario.dim_obs}) not compiled")
    if not 2 <= n <= 0x7FFFFFFF:
        raise ValueError("n must be at least 2")
    key = _dev.as_key(random_key).reshape(2).contiguous()
    dev = key.device
    d = scenario.dim
    x = torch.empty((n, d), dtype=torch.float32, device=dev)
    pp, dist, lw = (torch.empty(n, dtype=torch.float32, device=dev) for _ in range(3))
    thr = torch.empty(1, dtype=torch.float32, device=dev)
    ws = _dev.workspace(_lib.lib().mgb_abc_vanilla_workspace(n), dev)
    rate = getattr(sampler.parameters, "acceptance_rate", None)
    args = (n, _dev.ptr(key), float(sampler.parameters.threshold), -1.0 if rate is None else float(rate),
            _dev.ptr(ws), ws.numel(), _dev.ptr(x), _dev.ptr(pp), _dev.ptr(dist), _dev.ptr(lw), _dev.ptr(thr),
            _dev.stream_ptr())
    if gk:
        if scenario.data is None or np.size(scenario.data) != scenario.num_thin:
            raise ValueError("the g-and-k scenario needs data: num_thin summary values")
        data = torch.as_tensor(np.asarray(scenario.data, np.float32), device=dev).contiguous()
        call("mgb_abc_vanilla_gk", ctypes.byref(scenario.model(_dev.ptr(data))), *args)
    else:
        _keep, model = scenario.derived()
        call("mgb_abc_vanilla_lg", ctypes.byref(model), *args)
    t = float(thr.item())
    if rate is not None:
        sampler.parameters.threshold = t
    return cdict(value=x, log_weight=lw, distance=dist, prior_potential=pp, threshold=t)


class MetropolisedABCSMCSampler:
    """ABC-SMC with MCMC moves (abc/smc.py:101-245).  mcmc_sampler=None is the reference's
    default: RandomWalkABC with the stepsize re-set after every iteration to the particles'
    per-dimension variance / d * 2.38^2; RandomWalkABC(stepsize=s) keeps s fixed."""
    name = "ABC SMC"

    def __init__(self, mcmc_sampler=None, mcmc_correction="sampler_default", mcmc_steps=1, threshold_schedule=None,
                 max_iter=int(1e4), ess_threshold_retain=0.9, ess_threshold_resample=0.5, termination_alpha=0.01):
        if isinstance(mcmc_sampler, type):
            mcmc_sampler = mcmc_sampler()
        if mcmc_sampler is not None and not isinstance(mcmc_sampler, RandomWalkABC):
            raise NotImplementedError("the GPU sampler moves with RandomWalkABC")
        if mcmc_correction not in ("sampler_default", "Metropolis"):
            raise NotImplementedError("the GPU sampler uses the Metropolis correction")
        if mcmc_sampler is not None and mcmc_sampler.stepsize is None:
            raise NotImplementedError("RandomWalkABC needs a stepsize when given explicitly")
        self.mcmc_sampler = mcmc_sampler
        self.mcmc_steps = int(mcmc_steps)
        self.threshold_schedule = None if threshold_schedule is None else _arr(threshold_schedule).reshape(-1)
        self.max_iter = len(self.threshold_schedule) if self.threshold_schedule is not None else int(max_iter)
        self.ess_threshold_retain = float(ess_threshold_retain)
        self.ess_threshold_resample = float(ess_threshold_resample)
        self.termination_alpha = float(termination_alpha)


class BatchedABCSMC:
    """B posteriors of one ABC scenario advanced together on the GPU; ``init()`` then
    ``step()`` until ``done()``, or ``run()``."""

    def __init__(self, scenario, sampler, n, random_keys):
        self.gk = isinstance(scenario, GKTransformedUniformPrior)
        if not self.gk and not isinstance(scenario, LinearGaussian):
            raise NotImplementedError(f"{scenario.__class__.__name__}: no GPU ABC kernel for this scenario")
        if not self.gk and (scenario.dim, scenario.dim_obs) not in SUPPORTED:
            raise NotImplementedError(f"(d, dy) = ({scenario.dim}, {scenario.dim_obs}) not compiled")
        if self.gk and (scenario.data is None or np.size(scenario.data) != scenario.num_thin):
            raise ValueError("the g-and-k scenario needs data: num_thin summary values")
        if not 2 <= n <= MAX_N:
            raise NotImplementedError(f"n must be in [2, {MAX_N}]")
        keys = _dev.as_key(random_keys).reshape(-1, 2).contiguous()
        self.scenario, self.sampler = scenario, sampler
        self.keys = keys
        self.B, self.n = keys.shape[0], int(n)
        if self.gk:
            self._data = torch.as_tensor(np.asarray(scenario.data, np.float32), device=keys.device).contiguous()
            self.model = scenario.model(_dev.ptr(self._data))
        else:
            self._keep, self.model = scenario.derived()
        sch = sampler.threshold_schedule
        self._sch = None if sch is None else np.ascontiguousarray(sch, np.float32)
        fixed = sampler.mcmc_sampler is not None
        self.cfg = _lib.ABCConfig(self.B, self.n, sampler.mcmc_steps, min(sampler.max_iter, 100000),
                                  sampler.ess_threshold_retain, sampler.ess_threshold_resample,
                                  sampler.termination_alpha, 0 if fixed else 1,
                                  float(sampler.mcmc_sampler.stepsize) if fixed else 0.0,
                                  0 if self._sch is None else self._sch.size,
                                  None if self._sch is None else self._sch.ctypes.data)
        d = scenario.dim
        wsf = _lib.lib().mgb_abc_gk_workspace if self.gk else _lib.lib().mgb_abc_smc_workspace
        self.ws = _dev.workspace(wsf(ctypes.byref(self.cfg), d))
        self._pref = "mgb_abc_gk_smc" if self.gk else "mgb_abc_smc"
        self.views = _lib.ABCViews()
        call("mgb_abc_smc_views", ctypes.byref(self.cfg), d, _dev.ptr(self.ws), ctypes.byref(self.views))
        self.iterations = 0

    def _tensor(self, name, shape, dtype):
        n = int(np.prod(shape))
        off = getattr(self.views, name) - self.ws.data_ptr()
        nbytes = n * torch.tensor([], dtype=dtype).element_size()
        return self.ws.view(torch.uint8)[off:off + nbytes].view(dtype).reshape(shape)

    def init(self):
        call(self._pref + "_init", ctypes.byref(self.cfg), ctypes.byref(self.model), _dev.ptr(self.keys),
             _dev.ptr(self.ws), self.ws.numel(), _dev.stream_ptr())
        self.iterations = 0

    def step(self):
        call(self._pref + "_step", ctypes.byref(self.cfg), ctypes.byref(self.model), _dev.ptr(self.ws),
             self.ws.numel(), _dev.stream_ptr())
        self.iterations += 1

    def done(self):
        return not bool(self._tensor("active", (self.B,), torch.int32).any())

    def run(self, chain=False):
        """to termination; chain=True also records value, log_weight, distance after the startup and
        every iteration (the reference's stacked chain), as result().chain_*"""
        self._chain = {k: [] for k in ('value', 'log_weight', 'distance')} if chain else None
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
        return self.scenario.dim

    def _snap(self):
        self._chain["value"].append(self._tensor("value", (self.B, self.n, self._d()), torch.float32).clone())
        self._chain["log_weight"].append(self._tensor("log_weight", (self.B, self.n), torch.float32).clone())
        self._chain["distance"].append(self._tensor("distance", (self.B, self.n), torch.float32).clone())

    def result(self):
        B, n, d, H = self.B, self.n, self.scenario.dim, self.views.hist_len
        it = self._tensor("iter", (B,), torch.int32).clone()
        L = int(it.max()) + 1
        return cdict(value=self._tensor("value", (B, n, d), torch.float32).clone(),
                     log_weight=self._tensor("log_weight", (B, n), torch.float32).clone(),
                     distance=self._tensor("distance", (B, n), torch.float32).clone(),
                     prior_potential=self._tensor("prior_potential", (B, n), torch.float32).clone(),
                     stepsize=self._tensor("stepsize", (B, d), torch.float32).clone(),
                     threshold=self._tensor("hist_threshold", (B, H), torch.float32)[:, :L].clone(),
                     ess=self._tensor("hist_ess", (B, H), torch.float32)[:, :L].clone(),
                     alpha=self._tensor("hist_alpha", (B, H), torch.float32)[:, :L].clone(),
                     resampled=self._tensor("hist_resampled", (B, H), torch.int32)[:, :L].bool(),
                     iterations=it)


def run_batched(scenario, sampler, n, random_keys, chain=False):
    """mocat.run(scenario, sampler, n, key) for each of B keys, in one batch.  Per-iteration
    arrays are padded past each posterior's last iteration; chain=True adds chain_value
    (L, B, n, d), chain_log_weight and chain_distance (L, B, n)."""
    return BatchedABCSMC(scenario, sampler, n, random_keys).run(chain)


def _gk_chains(scenario, sampler, n, random_keys, correction):
    """RandomWalkABC chains on a g-and-k scenario, one CTA per chain (run_chains)"""
    rm = isinstance(correction, RMMetropolisDiagStepsize)
    name = getattr(correction, "__name__", type(correction).__name__)
    if not rm and correction is not None and correction != "Metropolis" and name != "Metropolis":
        raise NotImplementedError(f"{name}: no GPU chain for this correction")
    if scenario.data is None or np.size(scenario.data) != scenario.num_thin:
        raise ValueError("the g-and-k scenario needs data: num_thin summary values")
    keys = _dev.as_key(random_keys).reshape(-1, 2).contiguous()
    B, d, dev = keys.shape[0], scenario.dim, keys.device
    data = torch.as_tensor(np.asarray(scenario.data, np.float32), device=dev).contiguous()
    model = scenario.model(_dev.ptr(data))
    x = torch.empty((B, n, d), dtype=torch.float32, device=dev)
    if rm:
        if sampler.stepsize is not None or sampler.threshold is not None:
            raise NotImplementedError("the adaptive GPU chain starts from the sampler's defaults "
                                      "(threshold and stepsize unset)")
        st = torch.empty((B, n, d), dtype=torch.float32, device=dev)
        al, th = (torch.empty((B, n), dtype=torch.float32, device=dev) for _ in range(2))
        call("mgb_abc_mcmc_rm_gk", ctypes.byref(model), B, n, _dev.ptr(keys), float(sampler.tuning.target),
             correction.rm_stepsize_scale, correction.rm_stepsize_neg_exponent, _dev.ptr(x), _dev.ptr(al),
             _dev.ptr(th), _dev.ptr(st), _dev.stream_ptr())
        return cdict(value=x, alpha=al, threshold=th, stepsize=st)
    if sampler.stepsize is None or sampler.threshold is None:
        raise NotImplementedError("RandomWalkABC chains need a fixed stepsize and threshold")
    dist, pp, al = (torch.empty((B, n), dtype=torch.float32, device=dev) for _ in range(3))
    call("mgb_abc_mcmc_gk", ctypes.byref(model), B, n, _dev.ptr(keys), float(sampler.stepsize),
         float(sampler.threshold), _dev.ptr(x), _dev.ptr(dist), _dev.ptr(pp), _dev.ptr(al), _dev.stream_ptr())
    return cdict(value=x, distance=dist, prior_potential=pp, alpha=al)


def run_chains(scenario, sampler, n, random_keys, correction=None):
    """RandomWalkABC run as an MCMC sampler (abc/mcmc.py:16-100, mocat.run) for B independent
    chains, one per key.  With the Metropolis correction (correction=None): fixed stepsize and
    threshold; value (B, n, d), distance, prior_potential, alpha (B, n).  With
    correction=RMMetropolisDiagStepsize(): the adaptive chain from the sampler's defaults
    (threshold and stepsize unset); value (B, n, d), alpha, threshold (B, n), stepsize (B, n, d).
    Linear-Gaussian and g-and-k scenarios (one CTA per chain on g-and-k)."""
    if isinstance(scenario, GKTransformedUniformPrior):
        return _gk_chains(scenario, sampler, n, random_keys, correction)
    if not isinstance(scenario, LinearGaussian):
        raise NotImplementedError(f"{scenario.__class__.__name__}: no GPU ABC-MCMC kernel for this scenario")
    if (scenario.dim, scenario.dim_obs) not in SUPPORTED:
        raise NotImplementedError(f"(d, dy) = ({scenario.dim}, {scenario.dim_obs}) not compiled")
    if isinstance(correction, RMMetropolisDiagStepsize):
        if sampler.stepsize is not None or sampler.threshold is not None:
            raise NotImplementedError("the adaptive GPU chain starts from the sampler's defaults "
                                      "(threshold and stepsize unset)")
        keys = _dev.as_key(random_keys).reshape(-1, 2).contiguous()
        B, d, dev = keys.shape[0], scenario.dim, keys.device
        x = torch.empty((B, n, d), dtype=torch.float32, device=dev)
        st = torch.empty((B, n, d), dtype=torch.float32, device=dev)
        al, th = (torch.empty((B, n), dtype=torch.float32, device=dev) for _ in range(2))
        _keep, model = scenario.derived()
        call("mgb_abc_mcmc_rm_lg", ctypes.byref(model), B, n, _dev.ptr(keys), float(sampler.tuning.target),
             correction.rm_stepsize_scale, correction.rm_stepsize_neg_exponent, _dev.ptr(x), _dev.ptr(al),
             _dev.ptr(th), _dev.ptr(st), _dev.stream_ptr())
        return cdict(value=x, alpha=al, threshold=th, stepsize=st)
    name = getattr(correction, "__name__", type(correction).__name__)
    if correction is not None and correction != "Metropolis" and name != "Metropolis":
        raise NotImplementedError(f"{name}: no GPU chain for this correction")
    if sampler.stepsize is None or sampler.threshold is None:
        raise NotImplementedError("RandomWalkABC chains need a fixed stepsize and threshold")
    keys = _dev.as_key(random_keys).reshape(-1, 2).contiguous()
    B, d, dev = keys.shape[0], scenario.dim, keys.device
    x = torch.empty((B, n, d), dtype=torch.float32, device=dev)
    dist, pp, al = (torch.empty((B, n), dtype=torch.float32, device=dev) for _ in range(3))
    _keep, model = scenario.derived()
    call("mgb_abc_mcmc_lg", ctypes.byref(model), B, n, _dev.ptr(keys), float(sampler.stepsize),
         float(sampler.threshold), _dev.ptr(x), _dev.ptr(dist), _dev.ptr(pp), _dev.ptr(al), _dev.stream_ptr())
    return cdict(value=x, distance=dist, prior_potential=pp, alpha=al)


def run(scenario, sampler, n, random_key, correction=None):
    """mocat.run (sample.py:110-148) for MetropolisedABCSMCSampler, VanillaABC or RandomWalkABC (an MCMC
    chain) on an ABC scenario.
    ABC-SMC returns the reference's stacked layout: value (L, n, d), log_weight and distance
    (L, n) after the startup and every iteration, threshold, ess, alpha, resampled (L,)."""
    if isinstance(sampler, VanillaABC):
        return _run_vanilla(scenario, sampler, n, random_key)
    if isinstance(sampler, RandomWalkABC):
        out = run_chains(scenario, sampler, n, _dev.as_key(random_key).reshape(1, 2), correction)
        return cdict(**{k: v[0] for k, v in out.__dict__.items()})
    out = run_batched(scenario, sampler, n, _dev.as_key(random_key).reshape(1, 2), chain=True)
    L = int(out.iterations[0]) + 1
    return cdict(value=out.chain_value[:L, 0], log_weight=out.chain_log_weight[:L, 0],
                 distance=out.chain_distance[:L, 0], prior_potential=out.prior_potential[0],
                 stepsize=out.stepsize[0], threshold=out.threshold[0, :L], ess=out.ess[0, :L], alpha=out.alpha[0, :L],
                 resampled=out.resampled[0, :L], iterations=int(out.iterations[0]))
