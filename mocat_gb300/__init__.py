"""mocat_gb300: mocat's particle-system step on GB300 (sm_103a).

Propagate -> weight -> logsumexp/ESS -> resample -> gather as hand-written
CUDA kernels behind a C ABI (include/mocat_gb300.h, libmocatgb.so), with
Python classes and functions that keep mocat's names and call signatures.
PyTorch supplies device memory and streams only.
"""
from . import abc
from . import adjoint
from . import batched
from . import smc
from . import random
from . import ssm
from .core import Scenario, cdict, load_cdict, save_cdict, static_cdict
from .metrics import ess_log_weight, log_ess_log_weight
from .resampling import gather_rows, lse_ess, resample

__version__ = "0.1.0"

__all__ = ["abc", "adjoint", "batched", "smc", "random", "ssm", "Scenario", "cdict", "static_cdict", "save_cdict", "load_cdict", "ess_log_weight",
           "log_ess_log_weight", "resample", "gather_rows", "lse_ess"]
