"""``cdict`` container and ``Scenario`` base (mocat/src/core.py).

``cdict.__getitem__`` with an index tensor gathers every array field
(mocat/src/core.py:46-56); float32 fields on the GPU go through the
library's row gather kernel.
"""
import copy
import pickle
from pathlib import Path

import numpy as np
import torch


class cdict:
    def __init__(self, **kwargs):
        self.__dict__.update(kwargs)

    def copy(self):
        return cdict(**self.__dict__)

    def deepcopy(self):
        return copy.deepcopy(self)

    def __repr__(self):
        return f"mocat_gb300.cdict({self.__dict__.__repr__()})"

    def save(self, path, overwrite=False):
        save_cdict(self, path, overwrite)

    def __getitem__(self, item):
        if isinstance(item, str):
            return self.__dict__[item]
        out = self.copy()
        for key, attr in out.__dict__.items():
            if isinstance(attr, torch.Tensor) and attr.dim() > 0:
                out.__dict__[key] = _index(attr, item)
            elif isinstance(attr, np.ndarray) and attr.ndim > 0:
                out.__dict__[key] = attr[item]
            elif isinstance(attr, cdict) and not isinstance(attr, static_cdict):
                out.__dict__[key] = attr[item]
        return out

    def __add__(self, other):
        out = self.copy()
        if other is None:
            return out
        for key, attr in out.__dict__.items():
            if hasattr(other, key):
                o = other.__dict__[key]
                if isinstance(attr, torch.Tensor) or isinstance(o, torch.Tensor):
                    a = torch.atleast_1d(torch.as_tensor(attr))
                    b = torch.atleast_1d(torch.as_tensor(o, device=a.device))
                    out.__dict__[key] = torch.cat([a, b], 0)
                elif (isinstance(attr, cdict) and not isinstance(attr, static_cdict) and isinstance(o, cdict)
                      and not isinstance(o, static_cdict)) or key == "time":
                    out.__dict__[key] = attr + o
        return out

    @property
    def is_empty(self):
        return self.__dict__ == {}

    def keys(self):
        return self.__dict__.keys()

    def __iter__(self):
        return self.__dict__.__iter__()


class static_cdict(cdict):
    pass


def _index(t, item):
    if (isinstance(item, torch.Tensor) and item.dim() == 1 and item.dtype in (torch.int32, torch.int64)
            and t.is_cuda and t.dtype == torch.float32 and t.dim() >= 1):
        from .resampling import gather_rows
        return gather_rows(t, item)
    return t[item]


def save_cdict(in_cdict, path, overwrite=False):
    path = Path(path)
    if path.suffix != ".cdict":
        path = path.with_suffix(".cdict")
    path.parent.mkdir(parents=True, exist_ok=True)
    if path.exists():
        if overwrite:
            path.unlink()
        else:
            raise RuntimeError(f"File {path} already exists.")
    host = cdict(**{k: (v.cpu() if isinstance(v, torch.Tensor) else v) for k, v in in_cdict.__dict__.items()})
    with open(path, "wb") as f:
        pickle.dump(host, f)


def load_cdict(path):
    path = Path(path)
    if not path.is_file():
        raise ValueError(f"Not a file: {path}")
    if path.suffix != ".cdict":
        raise ValueError(f"Not a .cdict file: {path}")
    with open(path, "rb") as f:
        return pickle.load(f)


class Scenario:
    """Target for the SMC samplers: prior_potential, likelihood_potential,
    prior_sample and a temperature (mocat/src/core.py:146-261)."""
    name = None
    dim = None
    temperature = 1.0

    def __init__(self, name=None, **kwargs):
        if name is not None:
            self.name = name
        for k, v in kwargs.items():
            if hasattr(self, k):
                self.__dict__[k] = v

    def __repr__(self):
        return f"mocat_gb300.Scenario.{self.__class__.__name__}"
