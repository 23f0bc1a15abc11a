"""Pins the PRNG oracle (CPU only).

The known-answer values are published ones, restated from the public record in
``tests/golden/published_known_answers.json``:

* Random123 threefry2x32_20 known-answer vectors (zero key/counter, all-ones, and the
  pi-digits key/counter), the same triples JAX's own test suite checks;
* outputs printed in the JAX documentation for ``PRNGKey(0)`` (legacy-mode ``split``,
  ``normal(key, (1,))``, ``uniform(key, (3,))``; partitionable-mode ``split``).
"""

import json
import os

import numpy as np
import pytest

from oracle import coracle, models
from oracle import threefry as t

with open(os.path.join(os.path.dirname(__file__), "golden", "published_known_answers.json")) as _f:
    GOLDEN = json.load(_f)

KAT = [(tuple(int(v, 16) for v in r["key"]), tuple(int(v, 16) for v in r["counter"]),
        tuple(int(v, 16) for v in r["output"])) for r in GOLDEN["threefry2x32_20"]]
JAX0 = GOLDEN["jax_prngkey0"]


@pytest.mark.parametrize("key,ctr,expect", KAT)
def test_threefry_kat_numpy(key, ctr, expect):
    y0, y1 = t.threefry2x32(key[0], key[1], ctr[0], ctr[1])
    assert (int(y0), int(y1)) == expect


@pytest.mark.parametrize("key,ctr,expect", KAT)
def test_threefry_kat_c(key, ctr, expect):
    y0, y1 = coracle.threefry(np.array(key, np.uint32), [ctr[0]], [ctr[1]])
    assert (int(y0[0]), int(y1[0])) == expect


def test_prngkey_layout():
    assert t.PRNGKey(0).tolist() == [0, 0]
    assert t.PRNGKey(42).tolist() == [0, 42]
    assert t.PRNGKey(2**33 + 5).tolist() == [2, 5]


def test_kat_count():
    assert len(KAT) == 3


def test_jax_doc_values_legacy():
    k = t.PRNGKey(0)
    assert t.split(k, 2, t.LEGACY).tolist() == JAX0["legacy_split_2"]
    np.testing.assert_allclose(t.normal(k, (1,), t.LEGACY), JAX0["legacy_normal_1"], rtol=1e-6)
    np.testing.assert_allclose(t.uniform(k, (3,), mode=t.LEGACY), JAX0["legacy_uniform_3"],
                               rtol=1e-6)


def test_jax_doc_values_partitionable():
    k = t.PRNGKey(0)
    assert t.split(k, 2).tolist() == JAX0["partitionable_split_2"]


def test_partitionable_bits_prefix_stable():
    # in partitionable mode word i does not depend on the requested shape
    k = t.PRNGKey(7)
    a = t.bits(k, (5,))
    b = t.bits(k, (37,))
    assert np.array_equal(a, b[:5])


def test_legacy_odd_padding():
    k = t.PRNGKey(3)
    b = t.bits(k, (5,), t.LEGACY)
    y0, y1 = t.threefry2x32(k[0], k[1], np.array([0, 1, 2], np.uint32), np.array([3, 4, 0], np.uint32))
    assert b.tolist() == [y0[0], y0[1], y0[2], y1[0], y1[1]]


def test_uniform_is_exact_grid():
    b = np.arange(0, 2**32, 2**20 + 12345, dtype=np.uint64).astype(np.uint32)
    u = t.bits_to_unit_float(b)
    assert np.array_equal(u.astype(np.float64), (b >> 9).astype(np.float64) * 2.0**-23)


def test_normal_giles_vs_f64():
    b = np.random.RandomState(0).randint(0, 2**32, size=20000, dtype=np.uint64).astype(np.uint32)
    a32 = t.normal_from_bits(b).astype(np.float64)
    a64 = t.normal_from_bits_f64(b)
    # Giles' float32 polynomial is ~5e-6 relative in the tails (|z| ~ 3.8), inside the
    # 1e-5 relative tolerance of FP32 results
    assert np.max(np.abs(a32 - a64) / np.maximum(np.abs(a64), 1e-3)) < 1e-5


def test_bernoulli_threshold_exact():
    b = np.arange(0, 2**32, 4099, dtype=np.uint64).astype(np.uint32)
    u = t.bits_to_unit_float(b)
    p = np.float32(0.05)
    thr = int(np.ceil(np.float64(p) * 2**23))
    assert np.array_equal(u < p, (b >> 9) < thr)


def test_randint_range_and_span_one():
    k = t.PRNGKey(11)
    r = t.randint(k, (1000,), 0, 256)
    assert r.min() >= 0 and r.max() < 256
    assert np.all(t.randint(k, (10,), 5, 5) == 5)


def test_keychain_numpy_vs_c():
    rng, _ = models.model_keys(3, 2)
    a, ra = models.keychain(rng, 17, 2)
    b, rb = coracle.keychain(rng, 17, 2)
    assert np.array_equal(a, b) and np.array_equal(ra, rb)


def test_randomwalk_numpy_vs_c():
    x, y, m = models.randomwalk_run(0, 2000, 10)
    r = coracle.randomwalk_run(0, 2000, 10)
    # float32 states: identical up to last-ulp differences of log1pf implementations
    d = np.abs(x - r["x"])
    d = np.minimum(d, 1 - d)
    assert d.max() < 1e-6
    np.testing.assert_allclose(m, r["means"], rtol=1e-6)


def test_randomwalk_f32_vs_f64_oracle():
    r = coracle.randomwalk_run(0, 5000, 50, f64=True)
    d = np.abs(r["x"].astype(np.float64) - r["x64"])
    d = np.minimum(d, 1 - d)
    assert d.max() < 1e-5
    np.testing.assert_allclose(r["means"], r["means64"], rtol=1e-5)
