"""C ABI checks that need no GPU: the library loads, exports every function
include/mocat_gb300.h declares, and rejects bad arguments before touching
the device."""
import ctypes

import pytest

from mocat_gb300 import _lib


@pytest.fixture(scope="module")
def L():
    return _lib.lib()


def test_exports_every_declared_symbol(L):
    names = _lib.header_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # every declared symbol has a ctypes signature in the binding
    assert set(names) <= set(_lib._SIGNATURES), set(names) - set(_lib._SIGNATURES)


def test_status_strings(L):
    assert _lib.status_string(0) == "ok"
    assert "workspace" in _lib.status_string(4)
    assert L.mgb_version() >= 100


def test_bad_arguments_rejected_on_host(L):
    null = None
    assert L.mgb_split(null, 5, null, null) == 1
    assert L.mgb_normal(null, 5, null, null) == 1
    assert L.mgb_random_bits(null, -1, null, null) == 1
    assert L.mgb_lse_ess(null, 0, null, null, 0, null) == 1
    assert L.mgb_resample(null, 0, 0, null, null, null, 0, null, null) == 1
    assert L.mgb_resample_systematic_u(ctypes.c_void_p(16), 4, 1 << 23, ctypes.c_void_p(16), ctypes.c_void_p(16),
                                       1 << 20, null, null) == 1
    assert L.mgb_gather_rows(null, 0, null, 1, null, null) == 1
    m = _lib.LGModel(10, 10, None, None, None, None, None, None, 0.0)
    assert L.mgb_pf_lg_run(ctypes.byref(m), 16, 4, null, null, 0.5, 0, null, 0, null, null) == 1


def test_workspace_too_small_rejected_on_host(L):
    import numpy as np
    d = 10
    arrs = [np.eye(d, dtype=np.float32) for _ in range(5)] + [np.zeros(d, np.float32)]
    m = _lib.LGModel(d, d, *[a.ctypes.data for a in arrs], 1.0)
    need = L.mgb_pf_lg_workspace(1 << 20, 1000, d, 0)
    assert need > (1 << 20) * 4 * 2 * d
    p = ctypes.c_void_p(256)
    assert L.mgb_pf_lg_run(ctypes.byref(m), 1 << 20, 1000, p, p, 0.5, 0, p, need - 1, None, None) == 4
    assert L.mgb_resample_workspace(1000, 1) > L.mgb_resample_workspace(1000, 0)


def test_noalloc_array_holds_the_largest_allowed_size(L):
    """the fixed 256 KiB array of mgb_resample_systematic_u_noalloc holds the
    scratch of n = MGB_NOALLOC_MAX_N (a host-only size query)"""
    max_n = 1 << 24  # MGB_NOALLOC_MAX_N
    assert L.mgb_resample_workspace(max_n, 0) <= 256 * 1024


def test_unsupported_dimension_rejected_on_host(L):
    """dimensions above the run-time-dimension kernels' limit (32) are refused before any
    device call, for the whole filter and the online init / propagate entry points"""
    import numpy as np
    d = 33
    arrs = [np.eye(d, dtype=np.float32) for _ in range(5)] + [np.zeros(d, np.float32)]
    m = _lib.LGModel(d, d, *[a.ctypes.data for a in arrs], 1.0)
    p = ctypes.c_void_p(256)
    need = L.mgb_pf_lg_workspace(1000, 10, d, 0)
    assert L.mgb_pf_lg_run(ctypes.byref(m), 1000, 10, p, p, 0.5, 0, p, need, None, None) == 2
    assert L.mgb_pf_lg_init(ctypes.byref(m), 1000, p, p, p, p, None) == 2
    assert L.mgb_pf_lg_propagate(ctypes.byref(m), 1000, p, p, p, None, None, p, p, None) == 2
    m1 = _lib.LGModel(5, 33, *[a.ctypes.data for a in arrs], 1.0)  # dy above the limit
    assert L.mgb_pf_lg_init(ctypes.byref(m1), 1000, p, p, p, p, None) == 2
    # the particle smoothers: the same limit on the transition's d
    tr = _lib.LGTransition(d, arrs[0].ctypes.data, arrs[1].ctypes.data, 0.0)
    assert L.mgb_ffbsi_lg(ctypes.byref(tr), 4, 64, 16, p, p, p, p, p, p, 1 << 30, None) == 2
    assert L.mgb_stitch_lg(ctypes.byref(tr), 16, 64, p, p, p, p, p, None) == 2
    assert L.mgb_transition_potential_pairs(ctypes.byref(tr), 16, p, p, None, p, None) == 2
    cfg = _lib.RejectionConfig(5, 0.0, 1.01)
    assert L.mgb_ffbsi_rejection_lg(ctypes.byref(tr), ctypes.byref(cfg), 4, 64, 16, p, p, p, p, p, p, p, 1 << 30,
                                    None) == 2
    assert L.mgb_stitch_rejection_lg(ctypes.byref(tr), ctypes.byref(cfg), 16, p, p, p, p, p, p, p, 1 << 30,
                                     None) == 2


def test_new_entry_points_reject_bad_arguments_on_host(L):
    """Kalman, rejection samplers, stochastic-volatility filter and smoothing, SMC moves, ABC
    (g-and-k, VanillaABC, RandomWalkABC chains): argument checks run before any device call"""
    import numpy as np
    null = None
    p = ctypes.c_void_p(256)
    # Kalman: null model, then (d, dy) above the run-time-dimension limit (32)
    assert L.mgb_kalman_filter(null, 1, 4, p, p, p, null, null) == 1
    e = np.eye(33, dtype=np.float32)
    km = _lib.KalmanModel(33, 33, *([e.ctypes.data] * 5), np.zeros(33, np.float32).ctypes.data)
    assert L.mgb_kalman_filter(ctypes.byref(km), 1, 4, p, p, p, null, null) == 2
    assert L.mgb_kalman_smoother(ctypes.byref(km), 1, 4, p, p, p, p, null, null) == 2
    # rejection samplers: maximum_rejections must be >= 1
    F = np.eye(2, dtype=np.float32)
    tr = _lib.LGTransition(2, F.ctypes.data, F.ctypes.data, 0.0)
    cfg = _lib.RejectionConfig(0, 0.0, 1.01)
    assert L.mgb_stitch_rejection_lg(ctypes.byref(tr), ctypes.byref(cfg), 16, p, p, p, p, p, p, p, 1 << 20,
                                     null) == 1
    cfg.maximum_rejections = 5
    assert L.mgb_ffbsi_rejection_lg(ctypes.byref(tr), ctypes.byref(cfg), 0, 16, 16, p, p, p, p, p, p, p, 1 << 20,
                                    null) == 1
    assert L.mgb_ffbsi_sv(1.0, 1.0, 0, 16, 16, p, p, p, p, p, p, p, 1 << 20, null) == 1
    # stochastic-volatility filter: an unknown resampling scheme
    sv = _lib.SVModel(0.95, 0.3, 1.0, 0.9, 1.0, 0.0)
    assert L.mgb_pf_sv_run(ctypes.byref(sv), 64, 8, p, p, p, 0.5, 7, p, 1 << 30, null, null) == 2
    # SMC: an unknown move
    sc = _lib.SMCConfig(1, 64, 2, 1, 0.1, 1.0, 0.5, 0.5, 1e-5, 100, 1.0, 10, 0, 9)
    assert L.mgb_smc_logreg_init(ctypes.byref(sc), p, p, null, 10, p, p, 1 << 30, null) == 1
    # g-and-k ABC: d must be 1 or 4
    acfg = _lib.ABCConfig(1, 64, 1, 10, 0.8, 0.5, 0.01, 1, 0.0, 0, None)
    gk = _lib.GKModel(3, 1000, 100, 0.8, 0.0, 10.0, 1e-5, 256)
    assert L.mgb_abc_gk_smc_init(ctypes.byref(acfg), ctypes.byref(gk), p, p, 1 << 30, null) == 1
    assert L.mgb_abc_gk_simulate(ctypes.byref(gk), 4, p, p, p, null, null) == 1
    # VanillaABC: too small a workspace; RandomWalkABC chains: a negative stepsize
    d3 = np.eye(3, dtype=np.float32)
    v3 = np.zeros(3, np.float32)
    am = _lib.ABCModel(3, 2, v3.ctypes.data, d3.ctypes.data, d3.ctypes.data, 0.0, d3.ctypes.data, d3.ctypes.data,
                       v3.ctypes.data)
    need = L.mgb_abc_vanilla_workspace(1000)
    assert need > 0
    assert L.mgb_abc_vanilla_lg(ctypes.byref(am), 1000, p, 1.0, -1.0, p, need - 1, p, p, p, p, p, null) == 4
    assert L.mgb_abc_mcmc_lg(ctypes.byref(am), 1, 100, p, -0.1, 1.0, p, p, p, p, null) == 1
    # the adaptive chain: a non-positive Robbins-Monro scale, a negative exponent
    assert L.mgb_abc_mcmc_rm_lg(ctypes.byref(am), 1, 100, p, 0.1, 0.0, 2.0 / 3.0, p, p, p, p, null) == 1
    assert L.mgb_abc_mcmc_rm_lg(ctypes.byref(am), 1, 100, p, 0.1, 1.0, -1.0, p, p, p, p, null) == 1


def test_score_entry_points_reject_bad_arguments_on_host(L):
    """mgb_pf_lg_score / mgb_pf_lg_score_batch / mgb_wait_selftest: every argument check runs
    before any device call (1 = bad argument, 2 = unsupported configuration)"""
    import numpy as np
    d = 3
    eye = np.eye(d, dtype=np.float32)
    arrs = [eye, eye, eye, eye, eye, np.zeros(d, np.float32)]
    m = _lib.LGModel(d, d, *[a.ctypes.data for a in arrs], 1.0)
    p = ctypes.c_void_p(256)
    big = 1 << 30
    args = lambda K, L_, T=20, n=1024: (ctypes.byref(m), n, T, p, p, p, 0.5, 0, K, L_, p, big, None, p, None, None,
                                        None)
    assert L.mgb_pf_lg_score(*args(0, 8)) == 1             # no backward draw
    assert L.mgb_pf_lg_score(*args(5, 8)) == 1             # more than 4 draws
    assert L.mgb_pf_lg_score(*args(3, 2049)) == 1          # (K - 1) L > 4096
    assert L.mgb_pf_lg_score(*args(2, 8, T=(1 << 20) + 1)) == 1
    assert L.mgb_pf_lg_score(*args(2, 8, n=1)) == 1
    full = np.full((d, d), 0.1, np.float32)                # a non-diagonal transition covariance
    m2 = _lib.LGModel(d, d, eye.ctypes.data, full.ctypes.data, eye.ctypes.data, eye.ctypes.data, eye.ctypes.data,
                      arrs[5].ctypes.data, 1.0)
    assert L.mgb_pf_lg_score(ctypes.byref(m2), 1024, 20, p, p, p, 0.5, 0, 2, 8, p, big, None, p, None, None,
                             None) == 2
    m3 = _lib.LGModel(d, 1, *[a.ctypes.data for a in arrs], 1.0)  # dy != d
    assert L.mgb_pf_lg_score(ctypes.byref(m3), 1024, 20, p, p, p, 0.5, 0, 2, 8, p, big, None, p, None, None,
                             None) == 2
    bargs = lambda B, n=1024, K=2: (ctypes.byref(m), n, 20, B, p, p, p, 0.5, K, 8, p, big, None, p, None)
    assert L.mgb_pf_lg_score_batch(*bargs(0)) == 1
    assert L.mgb_pf_lg_score_batch(*bargs(4, K=0)) == 1
    assert L.mgb_pf_lg_score_batch(*bargs(4, n=1023)) == 2  # even n only
    assert L.mgb_pf_lg_score_batch_workspace(1024, 20, d, 4) == 4 * L.mgb_pf_lg_score_batch_workspace(1024, 20, d, 1)
    assert L.mgb_wait_selftest(2, 64, p, 256, None) == 1
    assert L.mgb_wait_selftest(0, 0, p, 256, None) == 1
