"""ctypes binding of the C ABI declared in include/mocat_gb300.h.

The library is loaded from the package's own build folder; there is no CPU
fallback: if it is missing, every entry point raises.
"""
import ctypes
import os
import re

from .build import LIB

_lib = None


class MGBError(RuntimeError):
    def __init__(self, status, where=""):
        self.status = status
        super().__init__(f"mocat_gb300: {where} failed with status {status} ({status_string(status)})")


class LGModel(ctypes.Structure):
    _fields_ = [("d", ctypes.c_int32), ("dy", ctypes.c_int32),
                ("F", ctypes.c_void_p), ("Lq", ctypes.c_void_p), ("H", ctypes.c_void_p), ("P", ctypes.c_void_p),
                ("C0", ctypes.c_void_p), ("m0", ctypes.c_void_p), ("c", ctypes.c_float)]


class PFOutputs(ctypes.Structure):
    _fields_ = [("log_z", ctypes.c_void_p), ("ess", ctypes.c_void_p), ("resampled", ctypes.c_void_p),
                ("x_hist", ctypes.c_void_p), ("lw_hist", ctypes.c_void_p), ("x_final", ctypes.c_void_p),
                ("lw_final", ctypes.c_void_p), ("err", ctypes.c_void_p), ("trace", ctypes.c_void_p)]


class OptModel(ctypes.Structure):
    _fields_ = [("d", ctypes.c_int32), ("dy", ctypes.c_int32), ("F", ctypes.c_void_p), ("H", ctypes.c_void_p),
                ("K", ctypes.c_void_p), ("S", ctypes.c_void_p), ("W", ctypes.c_void_p), ("cw", ctypes.c_float),
                ("K0", ctypes.c_void_p), ("C0c", ctypes.c_void_p), ("m0", ctypes.c_void_p)]


class NL1DModel(ctypes.Structure):
    _fields_ = [("initial_sd", ctypes.c_float), ("transition_sd", ctypes.c_float), ("likelihood_sd", ctypes.c_float),
                ("c", ctypes.c_float)]


class ABCModel(ctypes.Structure):
    _fields_ = [("d", ctypes.c_int32), ("dy", ctypes.c_int32), ("m0", ctypes.c_void_p), ("C0", ctypes.c_void_p),
                ("P0", ctypes.c_void_p), ("c0", ctypes.c_float), ("H", ctypes.c_void_p), ("L", ctypes.c_void_p),
                ("data", ctypes.c_void_p)]


class GKModel(ctypes.Structure):
    _fields_ = [("d", ctypes.c_int32), ("n_unsummarised", ctypes.c_int32), ("n_summary", ctypes.c_int32),
                ("c", ctypes.c_float), ("prior_min", ctypes.c_float), ("prior_max", ctypes.c_float),
                ("buffer", ctypes.c_float), ("data_dev", ctypes.c_void_p)]


class ABCConfig(ctypes.Structure):
    _fields_ = [("B", ctypes.c_int32), ("N", ctypes.c_int32), ("mcmc_steps", ctypes.c_int32),
                ("max_iter", ctypes.c_int32), ("ess_threshold_retain", ctypes.c_float),
                ("ess_threshold_resample", ctypes.c_float), ("termination_alpha", ctypes.c_float),
                ("adapt_stepsize", ctypes.c_int32), ("stepsize", ctypes.c_float), ("n_schedule", ctypes.c_int32),
                ("schedule", ctypes.c_void_p)]


class ABCViews(ctypes.Structure):
    _fields_ = [(k, ctypes.c_void_p) for k in ("value", "distance", "log_weight", "prior_potential", "alpha",
                                                "stepsize", "threshold", "ess", "alpha_mean", "iter", "active",
                                                "hist_threshold", "hist_ess", "hist_alpha", "hist_resampled")] + \
               [("hist_len", ctypes.c_int32)]


class KalmanModel(ctypes.Structure):
    _fields_ = [("d", ctypes.c_int32), ("dy", ctypes.c_int32)] + \
               [(k, ctypes.c_void_p) for k in ("F", "Q", "H", "R", "m0", "C0")]


class LGTransition(ctypes.Structure):
    _fields_ = [("d", ctypes.c_int32), ("F", ctypes.c_void_p), ("Pq", ctypes.c_void_p), ("cq", ctypes.c_float)]


class RejectionConfig(ctypes.Structure):
    _fields_ = [("maximum_rejections", ctypes.c_int32), ("init_bound_param", ctypes.c_float),
                ("bound_inflation", ctypes.c_float)]


class SVModel(ctypes.Structure):
    _fields_ = [("phi", ctypes.c_float), ("bsig", ctypes.c_float), ("r2", ctypes.c_float), ("cB", ctypes.c_float),
                ("c0", ctypes.c_float), ("m0", ctypes.c_float)]


class SVDModel(ctypes.Structure):
    _fields_ = [("d", ctypes.c_int32), ("A", ctypes.c_void_p), ("Lq", ctypes.c_void_p), ("C0", ctypes.c_void_p),
                ("m0", ctypes.c_void_p), ("r2", ctypes.c_void_p), ("cB", ctypes.c_float)]


class SVLaunch(ctypes.Structure):
    _fields_ = [("threads", ctypes.c_int32), ("ppt", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32),
                ("nbundles", ctypes.c_int32), ("smem_bytes", ctypes.c_int64)]


class SMCConfig(ctypes.Structure):
    _fields_ = [("B", ctypes.c_int32), ("N", ctypes.c_int32), ("d", ctypes.c_int32), ("mcmc_steps", ctypes.c_int32),
                ("stepsize", ctypes.c_float), ("prior_scale", ctypes.c_float),
                ("ess_threshold_retain", ctypes.c_float), ("ess_threshold_resample", ctypes.c_float),
                ("bisection_tol", ctypes.c_float), ("max_bisection_iter", ctypes.c_int32),
                ("max_temperature", ctypes.c_float), ("max_iter", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("move", ctypes.c_int32), ("leapfrog_steps", ctypes.c_int32), ("friction", ctypes.c_float),
                ("prior_sample_scale", ctypes.c_float), ("n_schedule", ctypes.c_int32),
                ("schedule_dev", ctypes.c_void_p), ("likelihood", ctypes.c_int32),
                ("gauss_mean_dev", ctypes.c_void_p), ("gauss_prec_sqrt_dev", ctypes.c_void_p),
                ("resampling", ctypes.c_int32)]


class SMCViews(ctypes.Structure):
    _fields_ = [(k, ctypes.c_void_p) for k in ("value", "log_weight", "likelihood_potential", "temperature", "ess",
                                               "log_norm_constant", "iter", "active", "hist_temperature",
                                               "hist_log_norm_constant", "hist_ess", "hist_alpha",
                                               "hist_resampled")] + [("hist_len", ctypes.c_int32)]


_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int
_F = ctypes.c_float
_SZ = ctypes.c_size_t

_SIGNATURES = {
    "mgb_status_string": ([_I32], ctypes.c_char_p),
    "mgb_version": ([], _I32),
    "mgb_random_bits": ([_P, _I64, _P, _P], _I32),
    "mgb_split": ([_P, _I64, _P, _P], _I32),
    "mgb_uniform": ([_P, _I64, _P, _P], _I32),
    "mgb_normal": ([_P, _I64, _P, _P], _I32),
    "mgb_exponential": ([_P, _I64, _P, _P], _I32),
    "mgb_gumbel": ([_P, _I64, _P, _P], _I32),
    "mgb_normal_keys": ([_P, _I64, _I64, _P, _P], _I32),
    "mgb_math_eval": ([_I32, _P, _I64, _P, _P], _I32),
    "mgb_lse_ess_workspace": ([_I64], _SZ),
    "mgb_lse_ess": ([_P, _I64, _P, _P, _SZ, _P], _I32),
    "mgb_resample_workspace": ([_I64, _I32], _SZ),
    "mgb_resample": ([_P, _I64, _I32, _P, _P, _P, _SZ, _P, _P], _I32),
    "mgb_resample_systematic_u": ([_P, _I64, ctypes.c_uint32, _P, _P, _SZ, _P, _P], _I32),
    "mgb_resample_systematic_u_noalloc": ([_P, _I64, ctypes.c_uint32, _P, _P, _P], _I32),
    "mgb_gather_rows": ([_P, _I64, _P, _I64, _P, _P], _I32),
    "mgb_pf_lg_init": ([ctypes.POINTER(LGModel), _I64, _P, _P, _P, _P, _P], _I32),
    "mgb_pf_lg_propagate": ([ctypes.POINTER(LGModel), _I64, _P, _P, _P, _P, _P, _P, _P, _P], _I32),
    "mgb_pf_lg_workspace": ([_I64, _I64, ctypes.c_int32, _I32], _SZ),
    "mgb_pf_lg_run": ([ctypes.POINTER(LGModel), _I64, _I64, _P, _P, _F, _I32, _P, _SZ, ctypes.POINTER(PFOutputs), _P],
                      _I32),
    "mgb_pf_lg_grad_workspace": ([_I64, _I64, ctypes.c_int32, ctypes.c_int32], _SZ),
    "mgb_pf_lg_grad": ([ctypes.POINTER(LGModel), _I64, _I64, _P, _P, _F, _I32, ctypes.c_int32, _P, _SZ, _P, _P, _P, _P],
                       _I32),
    "mgb_wait_selftest_workspace": ([], _SZ),
    "mgb_wait_selftest": ([ctypes.c_int, ctypes.c_int32, _P, _SZ, _P], _I32),
    "mgb_pf_lg_score_batch_workspace": ([_I64, _I64, ctypes.c_int32, _I64], _SZ),
    "mgb_pf_lg_score_batch": ([ctypes.POINTER(LGModel), _I64, _I64, _I64, _P, _P, _P, _F, ctypes.c_int32,
                               ctypes.c_int32, _P, _SZ, _P, _P, _P], _I32),
    "mgb_pf_lg_score_workspace": ([_I64, _I64, ctypes.c_int32], _SZ),
    "mgb_pf_lg_score": ([ctypes.POINTER(LGModel), _I64, _I64, _P, _P, _P, _F, _I32, ctypes.c_int32, ctypes.c_int32, _P,
                         _SZ, _P, _P, _P, _P, _P], _I32),
    "mgb_stitch_lg": ([ctypes.POINTER(LGTransition), _I64, _I64, _P, _P, _P, _P, _P, _P], _I32),
    "mgb_transition_potential_pairs": ([ctypes.POINTER(LGTransition), _I64, _P, _P, _P, _P, _P], _I32),
    "mgb_ffbsi_workspace": ([_I64, _I64, ctypes.c_int32], _SZ),
    "mgb_ffbsi_lg": ([ctypes.POINTER(LGTransition), _I64, _I64, _I64, _P, _P, _P, _P, _P, _P, _SZ, _P], _I32),
    "mgb_pf_opt_init": ([ctypes.POINTER(OptModel), _I64, _P, _P, _P, _P, _P], _I32),
    "mgb_pf_opt_propagate": ([ctypes.POINTER(OptModel), _I64, _P, _P, _P, _P, _P, _P, _P, _P], _I32),
    "mgb_pf_opt_workspace": ([_I64, _I64, ctypes.c_int32, _I32], _SZ),
    "mgb_pf_opt_run": ([ctypes.POINTER(OptModel), _I64, _I64, _P, _P, _F, _I32, _P, _SZ, ctypes.POINTER(PFOutputs),
                        _P], _I32),
    "mgb_pf_svd_init": ([ctypes.POINTER(SVDModel), _I64, _P, _P, _P, _P, _P], _I32),
    "mgb_pf_svd_propagate": ([ctypes.POINTER(SVDModel), _I64, _P, _P, _F, _P, _P, _P, _P, _P, _P], _I32),
    "mgb_pf_svd_workspace": ([_I64, _I64, ctypes.c_int32, ctypes.c_int], _SZ),
    "mgb_pf_svd_run": ([ctypes.POINTER(SVDModel), _I64, _I64, _P, _P, _P, _F, ctypes.c_int, _P, _SZ,
                        ctypes.POINTER(PFOutputs), _P], _I32),
    "mgb_pf_sv_init": ([ctypes.POINTER(SVModel), _I64, _P, _P, _P, _P, _P], _I32),
    "mgb_pf_sv_propagate": ([ctypes.POINTER(SVModel), _I64, _P, _P, _F, _P, _P, _P, _P, _P, _P], _I32),
    "mgb_pf_sv_workspace": ([_I64, _I64, ctypes.c_int], _SZ),
    "mgb_pf_sv_run": ([ctypes.POINTER(SVModel), _I64, _I64, _P, _P, _P, _F, ctypes.c_int, _P, _SZ,
                       ctypes.POINTER(PFOutputs), _P], _I32),
    "mgb_pf_nl1d_init": ([ctypes.POINTER(NL1DModel), _I64, _P, _P, _P, _P, _P], _I32),
    "mgb_pf_nl1d_propagate": ([ctypes.POINTER(NL1DModel), _I64, _P, _P, _F, _P, _P, _P, _P, _P, _P], _I32),
    "mgb_pf_nl1d_workspace": ([_I64, _I64, _I32], _SZ),
    "mgb_pf_nl1d_run": ([ctypes.POINTER(NL1DModel), _I64, _I64, _P, _P, _P, _F, _I32, _P, _SZ,
                         ctypes.POINTER(PFOutputs), _P], _I32),
    "mgb_ffbsi_nl1d": ([ctypes.POINTER(NL1DModel), _I64, _I64, _I64, _P, _P, _P, _P, _P, _P, _P, _SZ, _P], _I32),
    "mgb_stitch_nl1d": ([ctypes.POINTER(NL1DModel), _I64, _I64, _P, _P, _P, _F, _P, _P, _P], _I32),
    "mgb_ffbsi_sv": ([_F, _F, _I64, _I64, _I64, _P, _P, _P, _P, _P, _P, _P, _SZ, _P], _I32),
    "mgb_stitch_sv": ([_F, _F, _I64, _I64, _P, _P, _P, _F, _P, _P, _P], _I32),
    "mgb_transition_potential_pairs_sv": ([_F, _F, _I64, _P, _P, _F, _P, _P, _P], _I32),
    "mgb_ffbsi_rejection_sv": ([_F, _F, ctypes.POINTER(RejectionConfig), _I64, _I64, _I64, _P, _P, _P, _P, _P, _P,
                                _P, _P, _SZ, _P], _I32),
    "mgb_stitch_rejection_sv": ([_F, _F, ctypes.POINTER(RejectionConfig), _I64, _P, _P, _P, _F, _P, _P, _P, _P, _SZ,
                                 _P], _I32),
    "mgb_ffbsi_rejection_workspace": ([_I64, _I64, _I64, ctypes.c_int32], _SZ),
    "mgb_stitch_rejection_workspace": ([_I64, ctypes.c_int32], _SZ),
    "mgb_ffbsi_rejection_lg": ([ctypes.POINTER(LGTransition), ctypes.POINTER(RejectionConfig), _I64, _I64, _I64, _P,
                                _P, _P, _P, _P, _P, _P, _SZ, _P], _I32),
    "mgb_ffbsi_rejection_nl1d": ([ctypes.POINTER(NL1DModel), ctypes.POINTER(RejectionConfig), _I64, _I64, _I64, _P,
                                  _P, _P, _P, _P, _P, _P, _P, _SZ, _P], _I32),
    "mgb_stitch_rejection_lg": ([ctypes.POINTER(LGTransition), ctypes.POINTER(RejectionConfig), _I64, _P, _P, _P, _P,
                                 _P, _P, _P, _SZ, _P], _I32),
    "mgb_stitch_rejection_nl1d": ([ctypes.POINTER(NL1DModel), ctypes.POINTER(RejectionConfig), _I64, _P, _P, _P, _F,
                                   _P, _P, _P, _P, _SZ, _P], _I32),
    "mgb_transition_potential_pairs_nl1d": ([ctypes.POINTER(NL1DModel), _I64, _P, _P, _F, _P, _P, _P], _I32),
    "mgb_abc_gk_workspace": ([ctypes.POINTER(ABCConfig), ctypes.c_int32], _SZ),
    "mgb_abc_gk_smc_init": ([ctypes.POINTER(ABCConfig), ctypes.POINTER(GKModel), _P, _P, _SZ, _P], _I32),
    "mgb_abc_gk_smc_step": ([ctypes.POINTER(ABCConfig), ctypes.POINTER(GKModel), _P, _SZ, _P], _I32),
    "mgb_abc_gk_simulate": ([ctypes.POINTER(GKModel), _I64, _P, _P, _P, _P, _P], _I32),
    "mgb_abc_mcmc_lg": ([ctypes.POINTER(ABCModel), _I64, _I64, _P, _F, _F, _P, _P, _P, _P, _P], _I32),
    "mgb_abc_mcmc_rm_lg": ([ctypes.POINTER(ABCModel), _I64, _I64, _P, _F, _F, _F, _P, _P, _P, _P, _P], _I32),
    "mgb_abc_mcmc_rm_gk": ([ctypes.POINTER(GKModel), _I64, _I64, _P, _F, _F, _F, _P, _P, _P, _P, _P], _I32),
    "mgb_abc_mcmc_gk": ([ctypes.POINTER(GKModel), _I64, _I64, _P, _F, _F, _P, _P, _P, _P, _P], _I32),
    "mgb_abc_vanilla_workspace": ([_I64], _SZ),
    "mgb_abc_vanilla_lg": ([ctypes.POINTER(ABCModel), _I64, _P, _F, _F, _P, _SZ, _P, _P, _P, _P, _P, _P], _I32),
    "mgb_abc_vanilla_gk": ([ctypes.POINTER(GKModel), _I64, _P, _F, _F, _P, _SZ, _P, _P, _P, _P, _P, _P], _I32),
    "mgb_abc_smc_workspace": ([ctypes.POINTER(ABCConfig), ctypes.c_int32], _SZ),
    "mgb_abc_smc_views": ([ctypes.POINTER(ABCConfig), ctypes.c_int32, _P, ctypes.POINTER(ABCViews)], _I32),
    "mgb_abc_smc_init": ([ctypes.POINTER(ABCConfig), ctypes.POINTER(ABCModel), _P, _P, _SZ, _P], _I32),
    "mgb_abc_smc_step": ([ctypes.POINTER(ABCConfig), ctypes.POINTER(ABCModel), _P, _SZ, _P], _I32),
    "mgb_kalman_filter": ([ctypes.POINTER(KalmanModel), _I64, _I64, _P, _P, _P, _P, _P], _I32),
    "mgb_kalman_smoother": ([ctypes.POINTER(KalmanModel), _I64, _I64, _P, _P, _P, _P, _P, _P], _I32),
    "mgb_logreg_workspace": ([_I64, _I64, ctypes.c_int32, _I32], _SZ),
    "mgb_logreg_potential_grad": ([_P, _P, _I64, ctypes.c_int32, _P, _I64, _P, _P, _I32, _P, _P, _SZ, _P], _I32),
    "mgb_smc_logreg_workspace": ([ctypes.POINTER(SMCConfig), _I64], _SZ),
    "mgb_smc_logreg_views": ([ctypes.POINTER(SMCConfig), _P, ctypes.POINTER(SMCViews)], _I32),
    "mgb_smc_logreg_init": ([ctypes.POINTER(SMCConfig), _P, _P, _P, _I64, _P, _P, _SZ, _P], _I32),
    "mgb_smc_logreg_prior_scale_grad": ([ctypes.POINTER(SMCConfig), _P, _P, _P], _I32),
    "mgb_smc_logreg_step": ([ctypes.POINTER(SMCConfig), _P, _P, _P, _I64, _P, _SZ, _P], _I32),
    "mgb_pf_sv_batch_plan": ([_I64, _P, _P, ctypes.POINTER(SVLaunch), _P, _P], _I32),
    "mgb_pf_sv_batch_run": ([ctypes.POINTER(SVModel), _I64, _P, _P, _P, _P, _P, ctypes.POINTER(SVLaunch), _P, _P, _F,
                             _I32, _P, _P, _P, _P, _P], _I32),
    "mgb_pf_sv_batch_autotune_workspace": ([_I64], _SZ),
    "mgb_pf_sv_batch_autotune": ([ctypes.POINTER(SVModel), _I64, _P, _P, _P, _P, _P, _P, _P, _F, _I32, ctypes.c_int32,
                                  _P, _SZ, ctypes.POINTER(SVLaunch), ctypes.POINTER(ctypes.c_float), _P], _I32),
}


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise MGBError(-1, f"loading {LIB} (not built; run __graft_entry__.build())")
        L = ctypes.CDLL(LIB)
        for name, (args, res) in _SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def status_string(status):
    try:
        return lib().mgb_status_string(int(status)).decode()
    except MGBError:
        return "library not loaded"


def call(name, *args):
    st = getattr(lib(), name)(*args)
    if st != 0:
        raise MGBError(st, name)
    return st


def header_symbols(header=None):
    """Names of the functions declared in include/mocat_gb300.h."""
    header = header or os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                                    "mocat_gb300.h")
    text = open(header).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mgb_[a-z0-9_]+)\s*\(", text)))
