"""``cdict`` container and ``Scenario`` base (mocat/src/core.py).

``cdict.__getitem__`` with an index tensor gathers every array field
(mocat/src/core.py:46-56); float32 fields on the GPU go through the
library's row gather kernel.
"""
import contextlib
import copy
import pickle
import sys
import types
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

    def save(self, path, overwrite=False, reference_format=False):
        save_cdict(self, path, overwrite, reference_format)

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


REFERENCE_CORE = "mocat.src.core"  # module path of the reference's cdict in its pickles


def _host(v):
    if isinstance(v, torch.Tensor):
        return v.detach().cpu()
    if isinstance(v, cdict):
        return type(v)(**{k: _host(x) for k, x in v.__dict__.items()})
    return v


@contextlib.contextmanager
def _reference_classes():
    """(cdict, static_cdict) classes importable as mocat.src.core.* while pickling, from
    stub modules registered for the duration (the reference's own classes need jax)"""
    names = ("mocat", "mocat.src", REFERENCE_CORE)
    saved = {n: sys.modules.get(n) for n in names}
    mods = {n: types.ModuleType(n) for n in names}
    C = type("cdict", (), {"__module__": REFERENCE_CORE})
    S = type("static_cdict", (C,), {"__module__": REFERENCE_CORE})
    mods[REFERENCE_CORE].cdict, mods[REFERENCE_CORE].static_cdict = C, S
    mods["mocat"].src, mods["mocat.src"].core = mods["mocat.src"], mods[REFERENCE_CORE]
    sys.modules.update(mods)
    try:
        yield C, S
    finally:
        for n, m in saved.items():
            if m is None:
                sys.modules.pop(n, None)
            else:
                sys.modules[n] = m


class _ReferencePickler(pickle.Pickler):
    """writes cdicts as mocat.src.core.cdict instances and tensors as numpy arrays"""

    def __init__(self, f, classes):
        super().__init__(f, protocol=4)
        self.classes = classes

    def reducer_override(self, obj):
        if isinstance(obj, cdict):
            cls = self.classes[1] if isinstance(obj, static_cdict) else self.classes[0]
            # unpickling calls cls() (the reference's cdict(**kwargs) with none) and then
            # fills __dict__ from the state
            return cls, (), dict(obj.__dict__)
        if isinstance(obj, torch.Tensor):
            return obj.detach().cpu().numpy().__reduce__()
        return NotImplemented


def _jax_array_from_state(*args):
    """a jax array pickles as (reconstructor, (fun, args, numpy state, aval state)): the
    numpy array's own reduce plus jax's abstract-value fields; rebuild the numpy array"""
    if len(args) >= 3 and callable(args[0]) and isinstance(args[1], tuple):
        arr = args[0](*args[1])
        arr.__setstate__(args[2])
        return arr
    for a in args:
        if isinstance(a, np.ndarray):
            return a
    raise pickle.UnpicklingError("unrecognised jax array in a .cdict file")


class _CompatUnpickler(pickle.Unpickler):
    """reads .cdict files of this package and of the reference (mocat.src.core classes,
    jax arrays as numpy arrays)"""

    def find_class(self, module, name):
        if module == REFERENCE_CORE and name in ("cdict", "static_cdict"):
            return cdict if name == "cdict" else static_cdict
        if module.split(".")[0] in ("jax", "jaxlib"):
            return _jax_array_from_state
        return super().find_class(module, name)


def _to_tensors(c):
    for k, v in c.__dict__.items():
        if isinstance(v, np.ndarray) and v.dtype != object:
            c.__dict__[k] = torch.from_numpy(np.ascontiguousarray(v))
        elif isinstance(v, cdict):
            _to_tensors(v)
    return c


def save_cdict(in_cdict, path, overwrite=False, reference_format=False):
    """core.py:91-105.  reference_format=True writes the reference's own pickle layout
    (mocat.src.core.cdict, numpy arrays), which mocat's load_cdict reads."""
    path = Path(path)
    if path.suffix != ".cdict":
        path = path.with_suffix(".cdict")
    path.parent.mkdir(parents=True, exist_ok=True)
    if path.exists():
        if overwrite:
            path.unlink()
        else:
            raise RuntimeError(f"File {path} already exists.")
    host = _host(in_cdict)
    with open(path, "wb") as f:
        if reference_format:
            with _reference_classes() as classes:
                _ReferencePickler(f, classes).dump(host)
        else:
            pickle.dump(host, f)


def load_cdict(path):
    """core.py:108-121: a .cdict written by this package or by mocat; arrays come back as
    CPU tensors (the reference converts to its own array type in the same place)."""
    path = Path(path)
    if not path.is_file():
        raise ValueError(f"Not a file: {path}")
    if path.suffix != ".cdict":
        raise ValueError(f"Not a .cdict file: {path}")
    with open(path, "rb") as f:
        data = _CompatUnpickler(f).load()
    return _to_tensors(data) if isinstance(data, cdict) else data


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
