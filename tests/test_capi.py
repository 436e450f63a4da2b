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


def test_unsupported_dimension_rejected_on_host(L):
    import numpy as np
    d = 7
    arrs = [np.eye(d, dtype=np.float32) for _ in range(5)] + [np.zeros(d, np.float32)]
    m = _lib.LGModel(d, d, *[a.ctypes.data for a in arrs], 1.0)
    p = ctypes.c_void_p(256)
    need = L.mgb_pf_lg_workspace(1000, 10, d, 0)
    assert L.mgb_pf_lg_run(ctypes.byref(m), 1000, 10, p, p, 0.5, 0, p, need, None, None) == 2
