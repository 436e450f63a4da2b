"""Bounded device waits.  Each spin wait of the library's kernels (the
persistent filter's grid barrier, the decoupled-lookback tile scan) gives up
after a fixed number of polls, raises bit 1 of the error word and lets the
kernel finish.  mgb_wait_selftest drives each wait, with the library's own
wait code and a small poll limit, on a wait nothing will satisfy (a barrier
one block short; a lookback whose predecessor never publishes): the call must
come back with MGB_ERR_DEVICE_TIMEOUT, the context must stay usable, and the
next ordinary filter run must be bit-exact with the oracle."""
import ctypes

import numpy as np
import pytest
import torch

import oracle as O
from oracle import models

pytestmark = pytest.mark.gpu

TIMEOUT = 5  # MGB_ERR_DEVICE_TIMEOUT


def _filter_matches_oracle():
    import mocat_gb300 as mg
    d, n, T = 3, 4096, 40
    A = models.random_stable_matrix(d, 1)
    p = models.lg_params(np.zeros(d), np.eye(d), A, 0.2 * np.eye(d), np.eye(d), 0.5 * np.eye(d))
    _, y = models.simulate_lg(p, T, O.PRNGKey(1))
    ssm = mg.ssm.TimeHomogenousLinearGaussian(np.zeros(d), np.eye(d), A, 0.2 * np.eye(d), np.eye(d), 0.5 * np.eye(d))
    key = O.PRNGKey(2)
    out = mg.ssm.run_particle_filter_for_marginals(ssm, mg.ssm.BootstrapFilter(), y, np.arange(T), key, n=n)
    ref = O.lg_run(p, n, key, y, history=True)
    assert np.array_equal(out.value.cpu().numpy(), ref["value"])
    assert np.array_equal(out.log_weight.cpu().numpy(), ref["log_weight"])


@pytest.mark.parametrize("which", [0, 1])
@pytest.mark.parametrize("polls", [1, 64, 4096])
def test_wait_runs_out_and_reports(cuda, which, polls):
    from mocat_gb300 import _lib
    L = _lib.lib()
    ws = torch.zeros(L.mgb_wait_selftest_workspace(), dtype=torch.uint8, device=cuda)
    st = L.mgb_wait_selftest(which, polls, ctypes.c_void_p(ws.data_ptr()), ws.numel(),
                             ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == TIMEOUT
    assert int(ws[:4].view(torch.int32).item()) & 1  # the error word's timeout bit
    torch.cuda.synchronize()  # the context is still usable
    _filter_matches_oracle()


def test_bad_arguments(cuda):
    from mocat_gb300 import _lib
    L = _lib.lib()
    ws = torch.zeros(256, dtype=torch.uint8, device=cuda)
    p = ctypes.c_void_p(ws.data_ptr())
    assert L.mgb_wait_selftest(2, 64, p, 256, None) == 1
    assert L.mgb_wait_selftest(0, 0, p, 256, None) == 1
    assert L.mgb_wait_selftest(0, (1 << 22) + 1, p, 256, None) == 1
    assert L.mgb_wait_selftest(0, 64, p, 255, None) == 1
