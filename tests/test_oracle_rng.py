"""Pins of the oracle's jax.random restatement (CPU).

* threefry2x32-20 against the Random123 known-answer vectors (the three
  vectors jax's own random tests use), kept in tests/golden/known_answers.json;
* jax's counter layout against jax's documented outputs: split(PRNGKey(0)),
  random_bits(PRNGKey(1701), (3,)) (odd length: the zero-pad path),
  normal(PRNGKey(0)) and uniform(PRNGKey(0));
* the float maths against float64 references (accuracy bounds).
"""
import json
import os

import numpy as np
import pytest
import scipy.special as sp

import oracle as O

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))


@pytest.mark.parametrize("case", GOLDEN["threefry2x32_20"]["cases"])
def test_threefry_known_answers(case):
    r0, r1 = O.threefry2x32(tuple(case["key"]), case["counter"][0], case["counter"][1])
    assert [int(r0[0]), int(r1[0])] == case["expect"]


def test_prngkey_layout():
    assert O.PRNGKey(0).tolist() == [0, 0]
    assert O.PRNGKey(42).tolist() == [0, 42]


def test_split_matches_jax_docs():
    assert O.split(O.PRNGKey(0)).tolist() == GOLDEN["jax_random_documented"]["split_PRNGKey0"]


def test_random_bits_odd_length():
    assert O.random_bits(O.PRNGKey(1701), 3).tolist() == GOLDEN["jax_random_documented"]["random_bits_PRNGKey1701_3"]


def test_normal_uniform_scalar_values():
    g = GOLDEN["jax_random_documented"]
    assert np.float32(O.normal(O.PRNGKey(0))) == np.float32(g["normal_PRNGKey0"])
    assert np.float32(O.uniform(O.PRNGKey(0))) == np.float32(g["uniform_PRNGKey0"])


def test_split_num_consistent_with_bits():
    key = O.PRNGKey(7)
    ks = O.split(key, 5)
    bits = O.random_bits(key, 10)
    assert (ks.reshape(-1) == bits).all()


def test_erfinv_accuracy():
    x = np.linspace(-0.9999999, 0.9999999, 400001).astype(np.float32)
    got = O.erfinvf(x).astype(np.float64)
    ref = sp.erfinv(x.astype(np.float64))
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-30)
    assert rel.max() < 5e-7


def test_log_exp_accuracy():
    x = np.exp(np.linspace(-87, 88, 200001)).astype(np.float32)
    x = x[np.isfinite(x) & (x > 1.2e-38)]
    lg = O.logf(x).astype(np.float64)
    ref = np.log(x.astype(np.float64))
    assert np.max(np.abs(lg - ref) / np.maximum(np.abs(ref), 1.0)) < 3e-7
    z = np.linspace(-87, 88, 200001).astype(np.float32)
    ez = O.expf(z).astype(np.float64)
    rz = np.exp(z.astype(np.float64))
    assert np.max(np.abs(ez - rz) / rz) < 2e-7
    assert O.expf(np.array([-np.inf, -200.0, np.nan], np.float32))[:2].tolist() == [0.0, 0.0]


def test_normal_moments():
    z = O.normal(O.PRNGKey(3), (1 << 20,)).astype(np.float64)
    assert abs(z.mean()) < 5e-3 and abs(z.std() - 1) < 5e-3
    e = O.exponential(O.PRNGKey(4), (1 << 20,)).astype(np.float64)
    assert abs(e.mean() - 1) < 5e-3 and e.min() >= 0 and np.isfinite(e).all()
    g = O.gumbel(O.PRNGKey(5), (1 << 20,)).astype(np.float64)
    assert abs(g.mean() - 0.5772156649) < 5e-3
