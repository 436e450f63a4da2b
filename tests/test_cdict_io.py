""".cdict files (mocat/src/core.py:34-37, 91-121): this package's own pickles, the
reference's pickle layout written by save_cdict(..., reference_format=True), and
files in the layout mocat writes (mocat.src.core.cdict holding jax arrays)."""
import pickle
import sys
import types

import numpy as np
import pytest
import torch

import mocat_gb300 as mg
from mocat_gb300.core import cdict, static_cdict


def _sample():
    return cdict(value=torch.randn(5, 3), log_weight=torch.zeros(5), ess=torch.tensor([5.0]), name="run",
                 summary=static_cdict(sampler="Bootstrap Filter", n=5),
                 nested=cdict(t=torch.arange(4, dtype=torch.float32)))


def _same(a, b):
    assert set(a.__dict__) == set(b.__dict__)
    for k, v in a.__dict__.items():
        w = b.__dict__[k]
        if isinstance(v, torch.Tensor):
            assert torch.equal(torch.as_tensor(w), v), k
        elif isinstance(v, cdict):
            assert type(w) is type(v), k
            _same(v, w)
        else:
            assert v == w, k


class _RefModules:
    """stand-ins for the reference's modules, as mocat's own load_cdict would see them"""

    def __enter__(self):
        self.names = ("mocat", "mocat.src", "mocat.src.core", "jax", "jax._src", "jax._src.array")
        self.saved = {n: sys.modules.get(n) for n in self.names}
        m = {n: types.ModuleType(n) for n in self.names}

        class RefCdict:  # the reference's cdict: __init__(**kwargs), state in __dict__
            def __init__(self, **kw):
                self.__dict__.update(kw)
        RefCdict.__module__, RefCdict.__qualname__, RefCdict.__name__ = "mocat.src.core", "cdict", "cdict"

        class RefStatic(RefCdict):
            pass
        RefStatic.__module__, RefStatic.__qualname__, RefStatic.__name__ = "mocat.src.core", "static_cdict", \
            "static_cdict"

        def _reconstruct_array(fun, args, arr_state, aval_state):
            a = fun(*args)
            a.__setstate__(arr_state)
            return a
        _reconstruct_array.__module__, _reconstruct_array.__qualname__ = "jax._src.array", "_reconstruct_array"
        m["mocat.src.core"].cdict, m["mocat.src.core"].static_cdict = RefCdict, RefStatic
        m["jax._src.array"]._reconstruct_array = _reconstruct_array
        m["mocat"].src, m["mocat.src"].core = m["mocat.src"], m["mocat.src.core"]
        m["jax"]._src, m["jax._src"].array = m["jax._src"], m["jax._src.array"]
        sys.modules.update(m)
        self.RefCdict, self.RefStatic, self.reconstruct = RefCdict, RefStatic, _reconstruct_array
        return self

    def __exit__(self, *a):
        for n, mod in self.saved.items():
            if mod is None:
                sys.modules.pop(n, None)
            else:
                sys.modules[n] = mod


def test_own_format_round_trip(tmp_path):
    c = _sample()
    mg.save_cdict(c, tmp_path / "a")
    _same(c, mg.load_cdict(tmp_path / "a.cdict"))
    with pytest.raises(RuntimeError):
        mg.save_cdict(c, tmp_path / "a")
    mg.save_cdict(c, tmp_path / "a", overwrite=True)
    with pytest.raises(ValueError):
        mg.load_cdict(tmp_path / "missing.cdict")


def test_reference_format_is_readable_by_the_reference(tmp_path):
    c = _sample()
    c.save(tmp_path / "r", reference_format=True)
    raw = (tmp_path / "r.cdict").read_bytes()
    assert b"mocat.src.core" in raw and b"mocat_gb300" not in raw and b"torch" not in raw
    assert "mocat.src.core" not in sys.modules  # the stub modules are gone after the dump
    with _RefModules() as ref:
        with open(tmp_path / "r.cdict", "rb") as f:
            got = pickle.load(f)  # what mocat's load_cdict does before converting arrays
        assert type(got) is ref.RefCdict and type(got.summary) is ref.RefStatic
        assert isinstance(got.value, np.ndarray) and got.value.dtype == np.float32
        assert np.array_equal(got.value, c.value.numpy()) and np.array_equal(got.nested.t, c.nested.t.numpy())
        assert got.name == "run" and got.summary.n == 5
    _same(c, mg.load_cdict(tmp_path / "r.cdict"))


def test_reads_files_written_by_the_reference(tmp_path):
    """a file in the layout mocat's save_cdict produces: its cdict class holding jax arrays,
    each pickled as (reconstructor, (numpy reduce function, args, numpy state, aval state))"""
    vals = dict(value=np.random.default_rng(0).standard_normal((4, 2)).astype(np.float32),
                log_weight=np.zeros(4, np.float32), t=np.arange(4, dtype=np.int32))
    with _RefModules() as ref:
        class JaxLike:  # stands in for a jax Array: pickles through jax's reconstructor
            def __init__(self, a):
                self.a = a

            def __reduce__(self):
                fun, args, state = self.a.__reduce__()
                return ref.reconstruct, (fun, args, state, {"weak_type": False})
        obj = ref.RefCdict(**{k: JaxLike(v) for k, v in vals.items()}, name="pf",
                           summary=ref.RefStatic(sampler="Bootstrap Filter"))
        with open(tmp_path / "ref.cdict", "wb") as f:
            pickle.dump(obj, f)
    got = mg.load_cdict(tmp_path / "ref.cdict")
    assert type(got) is cdict and type(got.summary) is static_cdict
    for k, v in vals.items():
        assert isinstance(got.__dict__[k], torch.Tensor)
        assert np.array_equal(got.__dict__[k].numpy(), v)
    assert got.name == "pf" and got.summary.sampler == "Bootstrap Filter"
