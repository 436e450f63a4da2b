"""jax.random on the GPU (threefry2x32, jax's non-partitionable counter layout).

Keys are uint32 device tensors of shape (2,) (PRNGKey(seed) = [0, seed]);
draws match jax.random's raw bits, and its uniform / normal / exponential /
gumbel constructions (normal = sqrt(2) erfinv(u), erfinv by Giles' single
precision method).  Used by the reference at mocat/src/ssm/filtering.py:181,
199, 267, 278, 294 and mocat/src/transport/smc.py:65, 82, 140.
"""
import math

import numpy as np
import torch

from . import _dev
from ._lib import call


def PRNGKey(seed):
    s = int(seed)
    hi = (s >> 32) & 0xFFFFFFFF if s >= 0 else 0
    return _dev.as_key(np.array([hi, s & 0xFFFFFFFF], dtype=np.uint64).astype(np.uint32))


def _shape(shape):
    if shape is None or shape == ():
        return ()
    return tuple(int(s) for s in (shape if isinstance(shape, (tuple, list)) else (shape,)))


def split(key, num=2):
    key = _dev.as_key(key)
    out = torch.empty((int(num), 2), dtype=torch.uint32, device=key.device)
    call("mgb_split", _dev.ptr(key), int(num), _dev.ptr(out), _dev.stream_ptr())
    return out


def _draw(fn, key, shape, dtype):
    key = _dev.as_key(key)
    shape = _shape(shape)
    n = int(np.prod(shape)) if shape else 1
    out = torch.empty(n, dtype=dtype, device=key.device)
    call(fn, _dev.ptr(key), n, _dev.ptr(out), _dev.stream_ptr())
    return out.reshape(shape)


def random_bits(key, shape=()):
    return _draw("mgb_random_bits", key, shape, torch.uint32)


def normal_keys(keys, d):
    """normal(keys[i], (d,)) for every key of a (n, 2) key array, as one (n, d) draw:
    the batched form of the per-particle draws of a vmapped plugin method."""
    keys = _dev.as_key(keys).reshape(-1, 2).contiguous()
    out = torch.empty((keys.shape[0], int(d)), dtype=torch.float32, device=keys.device)
    call("mgb_normal_keys", _dev.ptr(keys), keys.shape[0], int(d), _dev.ptr(out), _dev.stream_ptr())
    return out


def uniform(key, shape=(), minval=0.0, maxval=1.0):
    u = _draw("mgb_uniform", key, shape, torch.float32)
    if minval == 0.0 and maxval == 1.0:
        return u
    lo = torch.tensor(minval, dtype=torch.float32, device=u.device)
    hi = torch.tensor(maxval, dtype=torch.float32, device=u.device)
    return torch.maximum(lo, u * (hi - lo) + lo)


def normal(key, shape=()):
    return _draw("mgb_normal", key, shape, torch.float32)


def exponential(key, shape=()):
    return _draw("mgb_exponential", key, shape, torch.float32)


def gumbel(key, shape=()):
    return _draw("mgb_gumbel", key, shape, torch.float32)


def categorical(key, logits, shape=None):
    """random.categorical for 1-D logits with shape=(n,) (n = len(logits)): Gumbel-max."""
    from .resampling import resample
    lw = _dev.as_f32(logits)
    if lw.dim() != 1:
        raise ValueError("categorical: 1-D logits only")
    if shape is not None and _shape(shape) != (lw.numel(),):
        raise ValueError("categorical: shape must equal (len(logits),)")
    return resample(lw, key, scheme="categorical")
