"""GPU logsumexp / ESS, resampling and gather vs the oracle.

Ancestors are integer work: bit-exact with the weights and uniforms fed in.
LSE / ESS are float64 reductions of float32 exponentials: relative 1e-6.
"""
import numpy as np
import pytest
import torch

import oracle as O

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 7, 255, 2047, 2048, 2049, 4097, 100_003, 1 << 20]


def _lw(n, seed, scale=3.0):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(n) * scale).astype(np.float32)


@pytest.mark.parametrize("n", SIZES)
def test_lse_ess(cuda, n):
    from mocat_gb300 import lse_ess
    lw = _lw(n, n)
    got = lse_ess(torch.from_numpy(lw).cuda()).cpu().numpy()
    ref = O.lse_ess(lw)
    assert got[0] == ref[0]
    assert np.allclose(got[1:], ref[1:], rtol=1e-6, atol=1e-6), (got, ref)


def test_lse_ess_edge_cases(cuda):
    from mocat_gb300 import lse_ess
    for lw in (np.full(5, -np.inf, np.float32), np.array([0, np.nan, 1], np.float32),
               np.array([0, np.inf], np.float32), np.zeros(3, np.float32)):
        got = lse_ess(torch.from_numpy(lw).cuda()).cpu().numpy()
        ref = O.lse_ess(lw)
        assert np.allclose(got[1:], ref[1:], equal_nan=True), (lw, got, ref)


@pytest.mark.parametrize("n", SIZES)
def test_systematic_bit_exact(cuda, n):
    from mocat_gb300.resampling import resample, resample_systematic_u
    lw = _lw(n, n + 1)
    lwd = torch.from_numpy(lw).cuda()
    for m in (0, 12345, (1 << 23) - 1):
        got = resample_systematic_u(lwd, m).cpu().numpy()
        ref, ok = O.resample_systematic(lw, m)
        assert ok and np.array_equal(got, ref), (n, m, np.flatnonzero(got != ref)[:10])
    key = O.PRNGKey(n)
    got = resample(lwd, key, "systematic").cpu().numpy()
    ref, _ = O.resample_systematic(lw, O.systematic_u_bits(key))
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("n", SIZES)
def test_multinomial_bit_exact(cuda, n):
    from mocat_gb300.resampling import resample
    lw = _lw(n, n + 2)
    key = O.PRNGKey(n + 3)
    got = resample(torch.from_numpy(lw).cuda(), key, "multinomial").cpu().numpy()
    ref, ok = O.resample_multinomial(lw, key)
    assert ok and np.array_equal(got, ref), (n, np.flatnonzero(got != ref)[:10])


@pytest.mark.parametrize("n", [1, 2, 5, 64, 1000, 4096, 4097])  # even n: the row-pair kernel
def test_categorical_bit_exact(cuda, n):
    from mocat_gb300.resampling import resample
    lw = _lw(n, n + 4)
    key = O.PRNGKey(n + 5)
    got = resample(torch.from_numpy(lw).cuda(), key, "categorical").cpu().numpy()
    ref = O.resample_gumbel(lw, key)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("scheme", ["systematic", "multinomial"])
def test_resample_edge_weights(cuda, scheme):
    from mocat_gb300.resampling import resample
    n = 5000
    cases = {
        "one_hot": np.where(np.arange(n) == 4321, 0.0, -np.inf).astype(np.float32),
        "heavy": np.where(np.arange(n) < 3, 50.0, 0.0).astype(np.float32),
        "underflow": np.concatenate([[0.0], np.full(n - 1, -200.0)]).astype(np.float32),
        "equal": np.zeros(n, np.float32),
        "all_neg_inf": np.full(n, -np.inf, np.float32),
        "nan": np.concatenate([np.zeros(n - 1), [np.nan]]).astype(np.float32),
    }
    key = O.PRNGKey(11)
    for name, lw in cases.items():
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        got = resample(torch.from_numpy(lw).cuda(), key, scheme, err=err).cpu().numpy()
        if scheme == "systematic":
            ref, ok = O.resample_systematic(lw, O.systematic_u_bits(key))
        else:
            ref, ok = O.resample_multinomial(lw, key)
        assert np.array_equal(got, ref), name
        assert bool(int(err.item()) & 2) == (not ok), name


def test_systematic_large_properties(cuda):
    """n = 2^22: sorted ancestors, offspring counts within floor/ceil of n w_i."""
    from mocat_gb300.resampling import resample_systematic_u
    n = 1 << 22
    lw = _lw(n, 99, 1.0)
    anc = resample_systematic_u(torch.from_numpy(lw).cuda(), 777).cpu().numpy()
    assert (np.diff(anc) >= 0).all() and anc.min() >= 0 and anc.max() < n
    q, _ = O.quantise(lw)
    w = q.astype(np.float64) / q.astype(np.float64).sum()
    cnt = np.bincount(anc, minlength=n)
    assert (cnt >= np.floor(n * w) - 1).all() and (cnt <= np.ceil(n * w) + 1).all()


@pytest.mark.parametrize("width", [1, 3, 4, 10, 50])
def test_gather_rows(cuda, width):
    from mocat_gb300 import gather_rows
    rng = np.random.default_rng(width)
    x = rng.standard_normal((3000, width)).astype(np.float32)
    anc = rng.integers(0, 3000, 2500).astype(np.int32)
    got = gather_rows(torch.from_numpy(x).cuda(), torch.from_numpy(anc).cuda()).cpu().numpy()
    assert np.array_equal(got, x[anc])
