"""Weight normalisation, resampling and gather on the GPU.

* ``lse_ess(lw)``: (max, logsumexp(lw), logsumexp(2 lw), ess) in float64 --
  log_ess_log_weight / ess_log_weight of mocat/src/metrics.py:69-78.
* ``resample(lw, key, scheme)``: ancestors for the reference's ``_resample``
  (mocat/src/ssm/filtering.py:196-199; SMCSampler.resample
  mocat/src/transport/smc.py:61-71).  ``scheme``:
    - ``"systematic"``: u = uniform(key), thresholds (k + u)/n;
    - ``"multinomial"``: inverse CDF at n sorted uniforms built from n+1
      exponential spacings drawn with ``key``;
    - ``"categorical"``: the reference's own ``random.categorical(key, lw,
      (n,))`` (Gumbel-max, O(n^2); n <= 46340).
* ``gather_rows(x, ancestors)``: x[ancestors] for a particle-major float32
  array (cdict.__getitem__, mocat/src/core.py:46-56).
"""
import torch

from . import _dev
from ._lib import call

SCHEMES = {"systematic": 0, "multinomial": 1, "categorical": 2}


def lse_ess(lw):
    lw = _dev.as_f32(lw).reshape(-1)
    n = lw.numel()
    ws = _dev.workspace(_lib_ws("mgb_lse_ess_workspace", n), lw.device)
    out = torch.empty(4, dtype=torch.float64, device=lw.device)
    call("mgb_lse_ess", _dev.ptr(lw), n, _dev.ptr(out), _dev.ptr(ws), ws.numel(), _dev.stream_ptr())
    return out


def _lib_ws(fn, *args):
    from ._lib import lib
    return getattr(lib(), fn)(*args)


def resample(lw, key, scheme="systematic", err=None):
    lw = _dev.as_f32(lw).reshape(-1)
    n = lw.numel()
    sc = SCHEMES[scheme]
    ws = _dev.workspace(_lib_ws("mgb_resample_workspace", n, sc), lw.device)
    anc = torch.empty(n, dtype=torch.int32, device=lw.device)
    key = _dev.as_key(key, lw.device)
    call("mgb_resample", _dev.ptr(lw), n, sc, _dev.ptr(key), _dev.ptr(anc), _dev.ptr(ws), ws.numel(),
         _dev.ptr(err), _dev.stream_ptr())
    return anc


def resample_systematic_u(lw, m23, err=None):
    """Systematic resampling with u = m23 * 2^-23 fed in."""
    lw = _dev.as_f32(lw).reshape(-1)
    n = lw.numel()
    ws = _dev.workspace(_lib_ws("mgb_resample_workspace", n, 0), lw.device)
    anc = torch.empty(n, dtype=torch.int32, device=lw.device)
    call("mgb_resample_systematic_u", _dev.ptr(lw), n, int(m23), _dev.ptr(anc), _dev.ptr(ws), ws.numel(),
         _dev.ptr(err), _dev.stream_ptr())
    return anc


def gather_rows(x, ancestors):
    """out[k] = x[ancestors[k]] for a float32 device tensor of shape (n, ...)."""
    anc = ancestors.to(device=x.device, dtype=torch.int32).contiguous()
    xc = x.contiguous()
    width = int(xc[0].numel()) if xc.dim() > 1 else 1
    out = torch.empty((anc.numel(),) + tuple(xc.shape[1:]), dtype=xc.dtype, device=xc.device)
    call("mgb_gather_rows", _dev.ptr(xc), width, _dev.ptr(anc), anc.numel(), _dev.ptr(out), _dev.stream_ptr())
    return out
