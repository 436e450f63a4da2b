"""Host-side planner of the batched stochastic-volatility launch (no GPU):
every filter is scheduled exactly once, bundles hold filters of one slot size
within the CTA's particle capacity and named-barrier limit, bundles come
longest first, and bad sizes are rejected."""
import ctypes

import numpy as np
import pytest

from mocat_gb300 import _lib


def _plan(ns, T, threads=512, ppt=16):
    ns = np.ascontiguousarray(ns, np.int32)
    T = np.ascontiguousarray(T, np.int32)
    B = ns.size
    l = _lib.SVLaunch(threads, ppt, 0, 0, 0)
    order = np.full(B, -1, np.int32)
    bundles = np.full(4 * B, -1, np.int32)
    st = _lib.lib().mgb_pf_sv_batch_plan(B, ns.ctypes.data, T.ctypes.data, ctypes.byref(l), order.ctypes.data,
                                         bundles.ctypes.data)
    return st, l, order, bundles[:4 * max(l.nbundles, 0)].reshape(-1, 4)


def _slot(n):
    s = 64
    while s < n + (n & 1):
        s <<= 1
    return s


@pytest.mark.parametrize("threads,ppt", [(512, 16), (256, 32), (1024, 8), (256, 4)])
def test_plan_covers_every_filter_once(threads, ppt):
    rng = np.random.default_rng(0)
    cap = threads * ppt
    ns = rng.integers(2, min(cap, 8192) + 1, 700)
    T = rng.integers(1, 2001, 700)
    st, l, order, bd = _plan(ns, T, threads, ppt)
    assert st == 0
    assert sorted(order.tolist()) == list(range(700))
    seen = np.zeros(700, int)
    smem = 0
    costs = []
    for first, count, slot, _ in bd:
        members = order[first:first + count]
        seen[members] += 1
        assert all(_slot(ns[m]) == slot for m in members)
        G = max(32, slot // ppt)
        assert count * slot <= cap and count * G <= threads
        assert count <= (16 if G == 32 else 15)
        smem = max(smem, count * (24 * slot + 16))
        costs.append(slot / G * T[members].max())
    assert (seen == 1).all()
    assert l.smem_bytes == smem <= 227 * 1024
    assert all(a >= b for a, b in zip(costs, costs[1:]))


def test_plan_rejects_bad_sizes():
    assert _plan([1, 64], [5, 5])[0] == 1          # n < 2
    assert _plan([8193], [5])[0] == 1              # n > 8192
    assert _plan([64, 64], [5, 0])[0] == 1         # T < 1
    assert _plan([4096], [5], 256, 8)[0] == 2      # larger than a CTA's capacity
    assert _plan([64], [5], 384, 16)[0] == 1       # unsupported CTA size
    assert _plan([64], [5], 512, 12)[0] == 1       # ppt not a power of two
