"""Device plumbing: PyTorch provides memory and streams; compute goes through the C ABI."""
import ctypes

import numpy as np
import torch

from . import _lib


def device():
    if not torch.cuda.is_available():
        raise _lib.MGBError(-1, "locating a CUDA device (mocat_gb300 runs on the GPU only)")
    return torch.device("cuda", torch.cuda.current_device())


def stream_ptr(dev=None):
    return ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


def ptr(t):
    if t is None:
        return None
    if not t.is_cuda:
        raise _lib.MGBError(1, "passing a host tensor where device memory is required")
    return ctypes.c_void_p(t.data_ptr())


def as_f32(x, dev=None):
    """float32 contiguous device tensor from a tensor / array / scalar."""
    dev = dev or device()
    if isinstance(x, torch.Tensor):
        return x.to(device=dev, dtype=torch.float32).contiguous()
    return torch.as_tensor(np.ascontiguousarray(np.asarray(x, dtype=np.float32)), device=dev)


def as_key(key, dev=None):
    """uint32 (..., 2) device tensor from a key (tensor, numpy array or sequence)."""
    dev = dev or device()
    if isinstance(key, torch.Tensor):
        if key.dtype == torch.uint32:
            return key.to(dev).contiguous()
        key = key.cpu().numpy()
    a = np.ascontiguousarray(np.asarray(key).astype(np.uint32))
    return torch.from_numpy(a.view(np.int32)).to(dev).view(torch.uint32)


def key_to_numpy(key):
    k = key.contiguous()
    return k.view(torch.int32).cpu().numpy().view(np.uint32) if k.dtype == torch.uint32 else np.asarray(k.cpu())


def workspace(nbytes, dev=None):
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=dev or device())
