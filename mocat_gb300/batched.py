"""Many independent particle filters in one persistent launch.

mocat filters one series per call (run_particle_filter_for_marginals,
mocat/src/ssm/filtering.py:255-324); for B stochastic-volatility series
(mocat/src/ssm/scenarios/stochastic_volatility.py) of uneven length T_b and
particle count n_b, ``run_particle_filters_batched`` returns what B such calls
would give for log Z, with one kernel launch (mgb_pf_sv_batch_run).  Launch
shapes come from a planner and an autotuner in the C library.

``BatchedFilters`` keeps the batch resident on the device so that the launch
can be re-run or captured in a CUDA graph (``enqueue``).
"""
import ctypes

import numpy as np
import torch

from . import _dev, _lib
from ._lib import call
from .core import cdict
from .resampling import SCHEMES
from .ssm import BootstrapFilter, StochasticVolatility

DEFAULT_LAUNCH = (512, 16)  # threads per CTA, particles per thread
MAX_N = 8192  # MGB_SV_BATCH_MAX_N


def _flat_obs(ys):
    """(y_flat float32, offsets int64, lengths int32) from a list of 1-D series."""
    ys = [np.asarray(y.detach().cpu() if isinstance(y, torch.Tensor) else y, dtype=np.float32).reshape(-1)
          for y in ys]
    T = np.array([y.size for y in ys], dtype=np.int32)
    off = np.zeros(len(ys), dtype=np.int64)
    if len(ys) > 1:
        off[1:] = np.cumsum(T[:-1].astype(np.int64))
    return np.concatenate(ys) if ys else np.zeros(0, np.float32), off, T


class BatchedFilters:
    """B bootstrap filters of a StochasticVolatility (dim 1) scenario.

    ns: particle counts (B,), 2 <= n_b <= 8192; ys: B observation series
    (length T_b >= 1) or a flat array with ``lengths``; random_keys: (B, 2)
    jax-style keys, one per filter.  ``resampling`` is "multinomial" or
    "systematic"; a filter resamples at step t when ess_{t-1} < ess_threshold n_b.
    ``launch`` = (threads, particles per thread) or None to autotune
    (``tune=True``, probes of ``probe_steps`` steps) or take the default.
    ``pin_y=True`` keeps a pinned host copy of the observations so that
    ``run(copy_in=True)`` measures the host-to-device path.
    """

    def __init__(self, ssm_scenario, particle_filter, ns, ys, random_keys, ess_threshold=0.5,
                 resampling="multinomial", launch=None, tune=False, probe_steps=128, lengths=None, pin_y=False):
        if not isinstance(ssm_scenario, StochasticVolatility):
            raise NotImplementedError(f"{ssm_scenario.__class__.__name__}: no batched GPU kernel for this model")
        if ssm_scenario.dim != 1:
            raise NotImplementedError("batched stochastic-volatility filters take dim = 1")
        if not isinstance(particle_filter, BootstrapFilter):
            raise NotImplementedError(f"{particle_filter.__class__.__name__}: no batched GPU kernel for this filter")
        if resampling not in ("multinomial", "systematic"):
            raise NotImplementedError(f"batched filters resample 'multinomial' or 'systematic', not {resampling!r}")
        particle_filter.startup(ssm_scenario)
        _, self._model = ssm_scenario.derived()
        dev = _dev.device()
        if lengths is None:
            y_flat, off, T = _flat_obs(ys)
        else:
            T = np.asarray(lengths, dtype=np.int32)
            off = np.zeros(T.size, np.int64)
            off[1:] = np.cumsum(T[:-1].astype(np.int64))
            y_flat = np.asarray(ys.detach().cpu() if isinstance(ys, torch.Tensor) else ys, np.float32).reshape(-1)
        n = np.ascontiguousarray(np.asarray(ns, dtype=np.int32).reshape(-1))
        B = n.size
        if T.size != B or B < 1:
            raise ValueError("ns and ys must describe the same, non-empty set of filters")
        if y_flat.size != int(T.astype(np.int64).sum()):
            raise ValueError("observations do not match the series lengths")
        keys = _dev.as_key(random_keys, dev).reshape(B, 2)
        self.B, self.n_host, self.T_host = B, n, np.ascontiguousarray(T)
        self.scheme = SCHEMES[resampling]
        self.ess_threshold = float(ess_threshold)
        self.n = torch.from_numpy(n).to(dev)
        self.T = torch.from_numpy(self.T_host).to(dev)
        self.y_off = torch.from_numpy(off).to(dev)
        self.y_host = torch.from_numpy(np.ascontiguousarray(y_flat))
        if pin_y:
            self.y_host = self.y_host.pin_memory()
        self.y = self.y_host.to(dev)
        self.keys = keys
        self.counter = torch.zeros(1, dtype=torch.int32, device=dev)
        self.log_z = torch.empty(B, dtype=torch.float64, device=dev)
        self.resampled_count = torch.empty(B, dtype=torch.int32, device=dev)
        self.tuned_ms = None
        if launch is None and tune:
            launch = self.autotune(probe_steps)
        self.set_launch(launch or DEFAULT_LAUNCH)

    def autotune(self, probe_steps=128):
        """(threads, particles per thread) of the fastest candidate launch on this batch."""
        ws = _dev.workspace(_lib.lib().mgb_pf_sv_batch_autotune_workspace(self.B))
        best = _lib.SVLaunch()
        ms = ctypes.c_float()
        call("mgb_pf_sv_batch_autotune", ctypes.byref(self._model), self.B, self.n_host.ctypes.data,
             self.T_host.ctypes.data, _dev.ptr(self.n), _dev.ptr(self.T), _dev.ptr(self.y_off), _dev.ptr(self.y),
             _dev.ptr(self.keys), self.ess_threshold, self.scheme, int(probe_steps), _dev.ptr(ws), ws.numel(),
             ctypes.byref(best), ctypes.byref(ms), _dev.stream_ptr())
        self.tuned_ms = ms.value
        return int(best.threads), int(best.ppt)

    def set_launch(self, launch):
        threads, ppt = launch
        self.launch = _lib.SVLaunch(int(threads), int(ppt), 0, 0, 0)
        order = np.empty(self.B, np.int32)
        bundles = np.empty(4 * self.B, np.int32)
        call("mgb_pf_sv_batch_plan", self.B, self.n_host.ctypes.data, self.T_host.ctypes.data,
             ctypes.byref(self.launch), order.ctypes.data, bundles.ctypes.data)
        dev = self.n.device
        self.order = torch.from_numpy(order).to(dev)
        self.bundles = torch.from_numpy(bundles[:4 * self.launch.nbundles].copy()).to(dev)
        self.plan = dict(threads=int(threads), ppt=int(ppt), nbundles=int(self.launch.nbundles),
                         smem_bytes=int(self.launch.smem_bytes))

    def enqueue(self):
        """Enqueue the batched run on the current stream (CUDA-graph capturable)."""
        call("mgb_pf_sv_batch_run", ctypes.byref(self._model), self.B, _dev.ptr(self.n), _dev.ptr(self.T),
             _dev.ptr(self.y_off), _dev.ptr(self.y), _dev.ptr(self.keys), ctypes.byref(self.launch),
             _dev.ptr(self.order), _dev.ptr(self.bundles), self.ess_threshold, self.scheme, _dev.ptr(self.counter),
             _dev.ptr(self.log_z), _dev.ptr(self.resampled_count), None, _dev.stream_ptr())

    def run(self, copy_in=False):
        """Run all filters; copy_in=True first copies the observations from the host copy."""
        if copy_in:
            self.y.copy_(self.y_host, non_blocking=True)
        self.enqueue()
        return cdict(log_z=self.log_z, resampled_count=self.resampled_count, n=self.n, T=self.T)

    @property
    def particle_steps(self):
        return int((self.n_host.astype(np.int64) * self.T_host.astype(np.int64)).sum())


def synthetic_sv_batch(B, seed=0, t_range=(50, 2000), log2n_range=(9, 13), phi=0.95, sigma=0.3):
    """Seeded synthetic stochastic-volatility series: T_b ~ U{t_range}, n_b = 2^U{log2n_range},
    x_0 ~ N(0, sigma^2 / (1 - phi^2)), x_t = phi x_{t-1} + sigma eps, y_t = exp(x_t / 2) eta,
    filter keys PRNGKey-style {0, seed * B + b}.  Returns (ns, y_flat, lengths, keys)."""
    rng = np.random.default_rng(seed)
    T = rng.integers(t_range[0], t_range[1] + 1, B).astype(np.int32)
    ns = (1 << rng.integers(log2n_range[0], log2n_range[1] + 1, B)).astype(np.int32)
    Tmax = int(T.max())
    x = rng.standard_normal(B) * (sigma / np.sqrt(1.0 - phi * phi))
    Y = np.empty((B, Tmax), np.float32)
    for t in range(Tmax):
        if t:
            x = phi * x + sigma * rng.standard_normal(B)
        Y[:, t] = np.exp(0.5 * x) * rng.standard_normal(B)
    y_flat = np.concatenate([Y[b, :T[b]] for b in range(B)]).astype(np.float32)
    keys = np.stack([np.zeros(B, np.uint32), (seed * B + np.arange(B)).astype(np.uint32)], 1)
    return ns, y_flat, T, keys


def run_particle_filters_batched(ssm_scenario, particle_filter, ys, random_keys, ns, ess_threshold=0.5,
                                 resampling="multinomial", launch=None, tune=False):
    """B independent run_particle_filter_for_marginals calls (filtering.py:255-324) in one launch.

    Returns cdict(log_z (B,) float64, resampled_count (B,) int32, n, T)."""
    bf = BatchedFilters(ssm_scenario, particle_filter, ns, ys, random_keys, ess_threshold, resampling, launch, tune)
    return bf.run()
