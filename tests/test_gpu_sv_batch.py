"""Batched stochastic-volatility filters (one persistent launch) vs the oracle.

Each filter must reproduce the oracle's o_sv_run (the bootstrap filter of
run_particle_filter_for_marginals on StochasticVolatility, d = 1): the same
resampling decisions at every step (count compared exactly) and log Z within
1e-5 relative.  Log-weight sums are float partials per warp, so log Z is not
bit-exact; particles and ancestors are, which the exact resample counts over
hundreds of steps depend on.
"""
import numpy as np
import pytest
import torch

import oracle as O
from oracle import models

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def _scenario():
    import mocat_gb300 as mg
    return mg.ssm.StochasticVolatility(dim=1, initial_covariance=0.3 ** 2 / (1 - 0.95 ** 2), transition_matrix=0.95,
                                       transition_covariance=0.09, likelihood_covariance_diag=1.0)


def _oracle(p, ns, y_flat, T, keys, thr, scheme):
    off = np.zeros(len(ns), np.int64)
    off[1:] = np.cumsum(np.asarray(T[:-1], np.int64))
    logz, nres = [], []
    for b in range(len(ns)):
        r = O.sv_run(p, int(ns[b]), keys[b], y_flat[off[b]:off[b] + T[b]], thr, scheme)
        logz.append(r["log_z"])
        nres.append(int(r["resampled"].sum()))
    return np.array(logz), np.array(nres)


def _mixed_batch(seed=0, B=40, tmax=150):
    from mocat_gb300.batched import synthetic_sv_batch
    ns, y, T, keys = synthetic_sv_batch(B, seed, t_range=(1, tmax), log2n_range=(6, 13))
    # uneven sizes: odd, non-powers of two, tiny
    extra = [2, 3, 5, 63, 100, 255, 1000, 3001, 5000, 8191]
    ns[:len(extra)] = extra
    T[0], T[1] = 1, 2
    off = np.concatenate([[0], np.cumsum(T.astype(np.int64))])
    rng = np.random.default_rng(seed + 99)
    y = rng.standard_normal(int(off[-1])).astype(np.float32) * 1.5
    return ns, y, T, keys


def _run(ns, y, T, keys, thr, scheme, launch):
    import mocat_gb300 as mg
    sc = _scenario()
    bf = mg.batched.BatchedFilters(sc, mg.ssm.BootstrapFilter(), ns, y, keys, ess_threshold=thr, resampling=scheme,
                                   launch=launch, lengths=T)
    out = bf.run()
    torch.cuda.synchronize()
    return out.log_z.cpu().numpy(), out.resampled_count.cpu().numpy(), bf


@pytest.mark.parametrize("scheme", ["multinomial", "systematic"])
@pytest.mark.parametrize("launch", [(512, 16), (256, 32), (1024, 8)])
def test_mixed_batch_matches_oracle(cuda, scheme, launch):
    ns, y, T, keys = _mixed_batch()
    p, _ = _scenario().derived()
    lz, nr, _ = _run(ns, y, T, keys, 0.5, scheme, launch)
    olz, onr = _oracle(p, ns, y, T, keys, 0.5, scheme)
    assert np.array_equal(nr, onr), np.nonzero(nr != onr)
    np.testing.assert_allclose(lz, olz, rtol=RTOL, atol=0)


@pytest.mark.parametrize("thr", [0.0, 0.9, 2.0])
def test_thresholds(cuda, thr):
    """0 never resamples, 2 resamples at every step after the first."""
    ns, y, T, keys = _mixed_batch(seed=3, B=24, tmax=60)
    p, _ = _scenario().derived()
    lz, nr, _ = _run(ns, y, T, keys, thr, "multinomial", (512, 16))
    olz, onr = _oracle(p, ns, y, T, keys, thr, "multinomial")
    assert np.array_equal(nr, onr)
    if thr == 0.0:
        assert nr.sum() == 0
    if thr == 2.0:
        assert np.array_equal(nr, T - 1)
    np.testing.assert_allclose(lz, olz, rtol=RTOL, atol=0)


def test_small_launch_shape_rejects_large_filters(cuda):
    import mocat_gb300 as mg
    ns, y, T, keys = _mixed_batch()
    with pytest.raises(mg._lib.MGBError):
        _run(ns, y, T, keys, 0.5, "multinomial", (256, 8))  # 2048 particles per CTA < 8191


def test_graph_replay_and_determinism(cuda):
    ns, y, T, keys = _mixed_batch(seed=5)
    lz, nr, bf = _run(ns, y, T, keys, 0.5, "multinomial", (512, 16))
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        bf.enqueue()
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    bf.log_z.zero_()
    with torch.cuda.graph(g):
        bf.enqueue()
    for _ in range(2):
        bf.log_z.zero_()
        g.replay()
        torch.cuda.synchronize()
        assert np.array_equal(bf.log_z.cpu().numpy(), lz)
        assert np.array_equal(bf.resampled_count.cpu().numpy(), nr)


def test_autotune_picks_a_valid_cached_shape(cuda):
    import mocat_gb300 as mg
    ns, y, T, keys = _mixed_batch(seed=7)
    sc = _scenario()
    bf = mg.batched.BatchedFilters(sc, mg.ssm.BootstrapFilter(), ns, y, keys, lengths=T, tune=True, probe_steps=32)
    assert bf.plan["threads"] * bf.plan["ppt"] >= 8191
    assert bf.tuned_ms is not None and bf.tuned_ms > 0
    first = bf.autotune(32)
    assert first == (bf.plan["threads"], bf.plan["ppt"])  # cached
    out = bf.run()
    p, _ = sc.derived()
    olz, onr = _oracle(p, ns, y, T, keys, 0.5, "multinomial")
    assert np.array_equal(out.resampled_count.cpu().numpy(), onr)
    np.testing.assert_allclose(out.log_z.cpu().numpy(), olz, rtol=RTOL, atol=0)


def test_full_size_batch_sampled_parity(cuda):
    """The 4096-series workload (T ~ U{50..2000}, n = 2^U{9..13}): every log Z finite,
    and 24 filters spread over the batch checked against the oracle."""
    import mocat_gb300 as mg
    ns, y, T, keys = mg.batched.synthetic_sv_batch(4096, seed=0)
    sc = _scenario()
    p, _ = sc.derived()
    lz, nr, bf = _run(ns, y, T, keys, 0.5, "multinomial", (512, 16))
    assert np.isfinite(lz).all()
    assert (nr > 0).all() and (nr < T).all()
    off = np.concatenate([[0], np.cumsum(T.astype(np.int64))])
    pick = np.unique(np.concatenate([np.argsort(-(ns.astype(np.int64) * T))[:4],
                                     np.random.default_rng(1).choice(4096, 20, replace=False)]))
    for b in pick:
        r = O.sv_run(p, int(ns[b]), keys[b], y[off[b]:off[b + 1]], 0.5, "multinomial")
        assert int(r["resampled"].sum()) == nr[b], b
        np.testing.assert_allclose(lz[b], r["log_z"], rtol=RTOL, atol=0)
