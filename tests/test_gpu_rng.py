"""GPU jax.random draws and float maths vs the oracle: bit-exact."""
import numpy as np
import pytest
import torch

import oracle as O

pytestmark = pytest.mark.gpu


def _np(t):
    t = t.contiguous().cpu()
    return t.view(torch.int32).numpy().view(np.uint32) if t.dtype == torch.uint32 else t.numpy()


@pytest.mark.parametrize("n", [1, 2, 3, 10, 1001, 1 << 16])
def test_bits_and_draws_bit_exact(cuda, n):
    import mocat_gb300.random as R
    for seed in (0, 1701):
        key = R.PRNGKey(seed)
        okey = O.PRNGKey(seed)
        assert (_np(R.random_bits(key, (n,))) == O.random_bits(okey, n)).all()
        assert np.array_equal(_np(R.uniform(key, (n,))), O.uniform(okey, (n,)))
        assert np.array_equal(_np(R.normal(key, (n,))), O.normal(okey, (n,)))
        assert np.array_equal(_np(R.exponential(key, (n,))), O.exponential(okey, (n,)))
        assert np.array_equal(_np(R.gumbel(key, (n,))), O.gumbel(okey, (n,)))


def test_split_and_known_values(cuda):
    import mocat_gb300.random as R
    assert _np(R.split(R.PRNGKey(0))).tolist() == [[4146024105, 967050713], [2718843009, 1272950319]]
    assert np.float32(_np(R.normal(R.PRNGKey(0)))) == np.float32(-0.20584226)
    for num in (1, 3, 1000, 65537):
        assert (_np(R.split(R.PRNGKey(5), num)) == O.split(O.PRNGKey(5), num)).all()


def test_math_bit_exact(cuda):
    import ctypes
    from mocat_gb300 import _dev, _lib
    rng = np.random.default_rng(0)
    xs = {
        0: np.concatenate([np.exp(rng.uniform(-87, 88, 100000)), rng.uniform(1e-7, 1, 100000)]).astype(np.float32),
        1: np.concatenate([rng.uniform(-110, 89, 100000), [-np.inf, 0.0, -0.0, 1e-30]]).astype(np.float32),
        2: rng.uniform(-0.9999999, 0.9999999, 200000).astype(np.float32),
    }
    fns = {0: O.logf, 1: O.expf, 2: O.erfinvf}
    for op, x in xs.items():
        xd = torch.from_numpy(x).cuda()
        out = torch.empty_like(xd)
        _lib.call("mgb_math_eval", op, _dev.ptr(xd), x.size, _dev.ptr(out), _dev.stream_ptr())
        got = out.cpu().numpy()
        ref = fns[op](x)
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), op
    _ = ctypes


def test_normal_keys(cuda):
    from mocat_gb300.ssm import _normal_keys
    import mocat_gb300.random as R
    keys = R.split(R.PRNGKey(3), 17)
    got = _np(_normal_keys(keys, 10))
    okeys = O.split(O.PRNGKey(3), 17)
    ref = np.stack([O.normal(k, (10,)) for k in okeys])
    assert np.array_equal(got, ref)
