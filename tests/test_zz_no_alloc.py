"""The allocation-free systematic resampling entry point.

Callers such as an XLA custom call or a node of a framework-built CUDA graph
receive their buffers and cannot allocate device memory of their own; for
them mgb_resample_systematic_u_noalloc keeps its scratch in a fixed array
inside the library.  These tests call it through the C ABI and check that two
calls in a row (a large then a smaller problem, so the second call starts from
the first call's leftover scratch) give exactly the ancestors of the
workspace-based mgb_resample_systematic_u.  Ancestors are integer results, so
the tolerance is zero.

The file name sorts last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

MAX_N = 1 << 24  # MGB_NOALLOC_MAX_N


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _with_workspace(L, lw, m23):
    n = lw.numel()
    ws = torch.empty(L.mgb_resample_workspace(n, 0), dtype=torch.uint8, device=lw.device)
    anc = torch.empty(n, dtype=torch.int32, device=lw.device)
    err = torch.zeros(1, dtype=torch.int32, device=lw.device)
    st = L.mgb_resample_systematic_u(_ptr(lw), n, m23, _ptr(anc), _ptr(ws), ws.numel(), _ptr(err),
                                     ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    return anc, err


def _noalloc(L, lw, m23):
    n = lw.numel()
    anc = torch.empty(n, dtype=torch.int32, device=lw.device)
    err = torch.zeros(1, dtype=torch.int32, device=lw.device)
    st = L.mgb_resample_systematic_u_noalloc(_ptr(lw), n, m23, _ptr(anc), _ptr(err),
                                             ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    return anc, err


def test_noalloc_matches_workspace_path_two_calls(cuda):
    from mocat_gb300 import _lib
    L = _lib.lib()
    rng = np.random.default_rng(123)
    cases = [(1 << 22, 4_000_001, 2.0), (50_001, 77, 5.0)]
    for n, m23, scale in cases:
        lw = torch.from_numpy((rng.standard_normal(n) * scale).astype(np.float32)).to(cuda)
        got, gerr = _noalloc(L, lw, m23)
        ref, rerr = _with_workspace(L, lw, m23)
        torch.cuda.synchronize()
        assert torch.equal(got, ref), n
        assert int(gerr.item()) == int(rerr.item()) == 0


def test_noalloc_at_the_largest_allowed_size(cuda):
    """n = MGB_NOALLOC_MAX_N fills the fixed array the most; then a small call
    starts from its leftover scratch"""
    from mocat_gb300 import _lib
    L = _lib.lib()
    rng = np.random.default_rng(7)
    cases = [(MAX_N, 123_457, 3.0), (1000, 5, 1.0)]
    for n, m23, scale in cases:
        lw = torch.from_numpy((rng.standard_normal(n) * scale).astype(np.float32)).to(cuda)
        got, gerr = _noalloc(L, lw, m23)
        ref, rerr = _with_workspace(L, lw, m23)
        torch.cuda.synchronize()
        assert torch.equal(got, ref), n
        assert int(gerr.item()) == int(rerr.item()) == 0


def test_noalloc_rejects_oversize_on_host(cuda):
    from mocat_gb300 import _lib
    L = _lib.lib()
    p = ctypes.c_void_p(256)
    assert L.mgb_resample_systematic_u_noalloc(p, MAX_N + 1, 0, p, None, None) == 2
