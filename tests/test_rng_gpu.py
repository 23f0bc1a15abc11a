"""K1 parity: device jax.random vs the NumPy oracle (bit-exact bits/keys/uniform/bernoulli/
randint; normal within the 1e-5 FP32 tolerance), both threefry modes."""

import numpy as np
import pytest
import torch

from oracle import threefry as t

pytestmark = pytest.mark.gpu

MODES = [(True, t.PARTITIONABLE), (False, t.LEGACY)]


@pytest.fixture(autouse=True)
def _restore_mode(cuda):
    import jaxabm_gb300.random as jr
    yield
    jr.set_partitionable(True)


def _keys(n, seed=0):
    rs = np.random.RandomState(seed)
    return rs.randint(0, 2**32, size=(n, 2), dtype=np.uint64).astype(np.uint32)


def _dev_keys(a):
    from jaxabm_gb300 import _dev
    return _dev.keys_from_numpy(a)


def _u32(tns):
    return tns.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("part,mode", MODES)
@pytest.mark.parametrize("num", [1, 2, 3, 7, 1000])
def test_split(part, mode, num):
    import jaxabm_gb300.random as jr
    jr.set_partitionable(part)
    keys = _keys(5, num)
    out = _u32(jr.split(_dev_keys(keys), num))
    ref = np.stack([t.split(k, num, mode) for k in keys])
    assert np.array_equal(out, ref)


@pytest.mark.parametrize("part,mode", MODES)
@pytest.mark.parametrize("count", [1, 2, 5, 64, 4097])
def test_bits_uniform_bernoulli(part, mode, count):
    import jaxabm_gb300.random as jr
    jr.set_partitionable(part)
    keys = _keys(3, count)
    dk = _dev_keys(keys)
    b = _u32(jr.bits(dk, (count,)))
    rb = np.stack([t.bits(k, (count,), mode) for k in keys])
    assert np.array_equal(b, rb)
    u = jr.uniform(dk, (count,), -2.5, 7.0).cpu().numpy()
    assert np.array_equal(u, t.uniform_from_bits(rb, -2.5, 7.0))
    be = jr.bernoulli(dk, 0.05, (count,)).cpu().numpy()
    assert np.array_equal(be, t.bits_to_unit_float(rb) < np.float32(0.05))


@pytest.mark.parametrize("part,mode", MODES)
def test_normal_tolerance(part, mode):
    import jaxabm_gb300.random as jr
    jr.set_partitionable(part)
    keys = _keys(4, 9)
    n = jr.normal(_dev_keys(keys), (5000,)).cpu().numpy().astype(np.float64)
    rb = np.stack([t.bits(k, (5000,), mode) for k in keys])
    ref32 = t.normal_from_bits(rb).astype(np.float64)
    ref64 = t.normal_from_bits_f64(rb)
    # FP32 tolerance 1e-5 relative (floor 1e-3 absolute scale near zero)
    assert np.max(np.abs(n - ref32) / np.maximum(np.abs(ref32), 1e-3)) < 1e-5
    assert np.max(np.abs(n - ref64) / np.maximum(np.abs(ref64), 1e-3)) < 1e-5


def test_scalar_shapes_and_doc_values():
    import jaxabm_gb300.random as jr
    k = jr.PRNGKey(0)
    jr.set_partitionable(False)
    assert _u32(jr.split(k)).tolist() == [[4146024105, 967050713], [2718843009, 1272950319]]
    np.testing.assert_allclose(jr.normal(k, (1,)).cpu().numpy(), [-0.20584226], rtol=1e-6)
    np.testing.assert_allclose(jr.uniform(k, (3,)).cpu().numpy(),
                               [0.9653214, 0.31468165, 0.63302994], rtol=1e-6)
    jr.set_partitionable(True)
    assert _u32(jr.split(k)).tolist() == [[1797259609, 2579123966], [928981903, 3453687069]]
    assert jr.uniform(k).shape == ()


@pytest.mark.parametrize("part,mode", MODES)
@pytest.mark.parametrize("lo,hi", [(0, 256), (0, 7), (-5, 1000003), (3, 3)])
def test_randint(part, mode, lo, hi):
    import jaxabm_gb300.random as jr
    jr.set_partitionable(part)
    keys = _keys(2, hi)
    out = jr.randint(_dev_keys(keys), (333,), lo, hi).cpu().numpy()
    ref = np.stack([t.randint(k, (333,), lo, hi, mode) for k in keys])
    assert np.array_equal(out, ref)


def test_keychain_matches_oracle():
    import jaxabm_gb300.random as jr
    from oracle import models
    rng, _ = models.model_keys(5, 3)
    d = _dev_keys(rng)
    ck, uk = jr.keychain(d, 40, 3, update_keys=True)
    ref, ref_rng = models.keychain(rng, 40, 3)
    assert np.array_equal(_u32(ck), ref)
    assert np.array_equal(_u32(d), ref_rng)
    # update key = split(step_key after the collections)[1]
    r = rng.copy()
    k = t.split(r, 2)
    sk = k[1]
    for _ in range(3):
        sk = t.split(sk, 2)[0]
    assert np.array_equal(_u32(uk)[0], t.split(sk, 2)[1])


def test_bad_mode_rejected():
    from jaxabm_gb300 import _lib, _dev
    keys = _dev_keys(_keys(1))
    out = torch.empty((1, 2, 2), dtype=torch.int32, device="cuda")
    st = _lib.load().abm_rng_split(_dev.ptr(keys), 1, 2, _dev.ptr(out), 7, None)
    assert st == _lib.ABM_ERR_BADARG


@pytest.mark.parametrize("nkeys,count", [(3000, 1), (1500, 3), (40, 700)])
def test_many_keys(nkeys, count):
    """Per-agent draws (many keys, few elements each: the flat launch) and many keys with
    many elements each (the 2-D launch) match the oracle."""
    import jaxabm_gb300.random as jr
    jr.set_partitionable(True)
    keys = _keys(nkeys, count + 11)
    dk = _dev_keys(keys)
    b = _u32(jr.bits(dk, (count,)))
    rb = np.stack([t.bits(k, (count,), t.PARTITIONABLE) for k in keys])
    assert np.array_equal(b, rb)
    s = _u32(jr.split(dk, count))
    rs = np.stack([t.split(k, count, t.PARTITIONABLE) for k in keys])
    assert np.array_equal(s, rs)


@pytest.mark.parametrize("partitionable", [True, False])
@pytest.mark.parametrize("n,width,height,seed", [(58_982, 256, 256, 1), (1000, 7, 13, 0),
                                                 (5, 1 << 20, 3, 42)])
def test_grid_position_agents_matches_oracle(cuda, partitionable, n, width, height, seed):
    """Grid.position_agents without positions (jaxabm/agentpy.py:496-527): x = randint(
    PRNGKey(seed), (n,), 0, width) with the unsplit key and y = randint(split(key)[1], (n,),
    0, height), equal to the oracle's randint; positions may coincide, as in the
    reference."""
    import jaxabm_gb300 as jx
    from oracle import threefry as tf
    mode = tf.PARTITIONABLE if partitionable else tf.LEGACY
    jx.random.set_partitionable(partitionable)
    try:
        class M(jx.Model):
            def setup(self):
                self.walkers = self.add_agents(n, jx.RandomWalker, name="walkers")
                self.grid = jx.Grid(self, (width, height))

        m = M({"seed": seed})
        m.setup()
        m.grid.position_agents(m.walkers)
        pos = m.walkers.collection._states["position"].cpu().numpy()
    finally:
        jx.random.set_partitionable(True)
    key = tf.PRNGKey(seed)
    x = tf.randint(key, (n,), 0, width, mode)
    y = tf.randint(tf.split(key, 2, mode)[1], (n,), 0, height, mode)
    assert pos.shape == (n, 2)
    assert np.array_equal(pos[:, 0], x) and np.array_equal(pos[:, 1], y)
    assert pos[:, 0].min() >= 0 and pos[:, 0].max() < width
    assert pos[:, 1].min() >= 0 and pos[:, 1].max() < height
