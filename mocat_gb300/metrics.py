"""ESS from log-weights (mocat/src/metrics.py:69-78), computed on the GPU."""
import torch

from .core import cdict
from .resampling import lse_ess


def _lw(log_weight):
    if isinstance(log_weight, cdict) and hasattr(log_weight, "log_weight"):
        log_weight = log_weight.log_weight
    if not isinstance(log_weight, torch.Tensor):
        raise TypeError("log_weight must be a tensor or cdict with log_weight attribute")
    return log_weight


def log_ess_log_weight(log_weight):
    """2 logsumexp(lw) - logsumexp(2 lw) (float64 scalar tensor on the device)."""
    o = lse_ess(_lw(log_weight))
    return 2.0 * o[1] - o[2]


def ess_log_weight(log_weight):
    return torch.exp(log_ess_log_weight(log_weight))
