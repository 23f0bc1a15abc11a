"""K6 compaction and K7 reductions vs NumPy (bit-exact indices, stable order)."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 15, 16, 17, 4095, 4096, 4097, 100_003, 1 << 20])
@pytest.mark.parametrize("density", [0.0, 0.01, 0.5, 1.0])
def test_select_indices(cuda, n, density):
    from jaxabm_gb300.select import select_indices
    rs = np.random.RandomState(n)
    m = rs.rand(n) < density
    idx, c = select_indices(torch.from_numpy(m).cuda())
    ref = np.nonzero(m)[0]
    assert c == len(ref)
    assert np.array_equal(idx.cpu().numpy(), ref)


def test_select_unaligned_mask(cuda):
    from jaxabm_gb300.select import select_indices
    m = torch.from_numpy(np.random.RandomState(1).rand(5001) < 0.3).cuda()
    sub = m[3:]  # data pointer not 16-byte aligned: scalar path
    idx, c = select_indices(sub)
    assert np.array_equal(idx.cpu().numpy(), np.nonzero(sub.cpu().numpy())[0])


def test_compact_states_rows(cuda):
    from jaxabm_gb300.select import compact_states
    n = 3001
    rs = np.random.RandomState(2)
    st = {"a": torch.from_numpy(rs.rand(n).astype(np.float32)).cuda(),
          "b": torch.from_numpy(rs.randint(0, 100, size=(n, 3)).astype(np.int8)).cuda(),
          "c": torch.from_numpy(rs.randint(0, 9, size=(n, 2)).astype(np.int64)).cuda()}
    mask = st["a"] > 0.5
    out, c = compact_states(st, mask)
    mk = mask.cpu().numpy()
    for k in st:
        assert np.array_equal(out[k].cpu().numpy(), st[k].cpu().numpy()[mk])
    assert c == mk.sum()


def test_agent_collection_filter_and_aggregate(cuda):
    import jaxabm_gb300 as jx
    m = jx.JaxModel(config=jx.ModelConfig(seed=1))
    coll = jx.AgentCollection(jx.agentpy.AgentWrapper(jx.RandomWalker), 5000)
    m.add_agent_collection("w", coll)
    m.initialize()
    f = coll.filter(lambda s: s["x"] > 0.5)
    x = coll.states["x"].cpu().numpy()
    assert f.num_agents == int((x > 0.5).sum())
    assert np.array_equal(f.states["x"].cpu().numpy(), x[x > 0.5])
    np.testing.assert_allclose(float(coll.aggregate("x")), x.astype(np.float64).mean(), rtol=1e-6)
    with pytest.raises(ValueError):
        coll.aggregate("nope")


@pytest.mark.parametrize("op", [0, 1, 2, 3])
def test_reduce(cuda, op):
    from jaxabm_gb300.select import reduce
    x = np.random.RandomState(op).randn(123_457).astype(np.float32)
    out = float(reduce(torch.from_numpy(x).cuda(), op))
    ref = [x.astype(np.float64).sum(), x.astype(np.float64).mean(), x.min(), x.max()][op]
    np.testing.assert_allclose(out, ref, rtol=1e-6)


@pytest.mark.parametrize("where", [0, 5, 77_777, 123_456])
def test_reduce_propagates_nan(cuda, where):
    """A NaN anywhere makes sum, mean, min and max NaN, as jnp.sum / mean / min / max do."""
    from jaxabm_gb300.select import reduce
    x = np.random.RandomState(1).randn(123_457).astype(np.float32)
    x[where] = np.nan
    d = torch.from_numpy(x).cuda()
    for op in range(4):
        assert np.isnan(float(reduce(d, op))), op
    x[where] = 0.5  # without the NaN: ordinary results again
    d = torch.from_numpy(x).cuda()
    assert float(reduce(d, 2)) == x.min() and float(reduce(d, 3)) == x.max()


def test_select_agentlist_api(cuda):
    import jaxabm_gb300 as jx

    class M(jx.Model):
        def setup(self):
            self.walkers = self.add_agents(2000, jx.RandomWalker, name="walkers")

    m = M({"steps": 3, "seed": 4})
    m.run()
    sel = m.walkers.select(lambda s: s["y"] < 0.25)
    y = m.walkers.y.cpu().numpy()
    assert len(sel) == int((y < 0.25).sum())
    assert np.array_equal(sel.y.cpu().numpy(), y[y < 0.25])


@pytest.mark.parametrize("n", [1, 15, 4096, 4097, 100_003, 1 << 20])
def test_select_where_matches_numpy(cuda, n):
    """Predicate programs over float32, int32, int8 and bool attributes select exactly the
    indices numpy's boolean evaluation does (float32 compares in float32)."""
    from jaxabm_gb300.select import select_where
    rs = np.random.RandomState(n)
    h = {"x": rs.rand(n).astype(np.float32), "i": rs.randint(-5, 6, n).astype(np.int32),
         "k": rs.randint(0, 3, n).astype(np.int8), "f": rs.rand(n) < 0.3}
    st = {k: torch.from_numpy(v).cuda() for k, v in h.items()}
    conds = [
        (lambda s: s["x"] > 0.5, lambda s: s["x"] > np.float32(0.5)),
        (lambda s: (s["x"] >= 0.2) & (s["x"] < 0.6), lambda s: (s["x"] >= np.float32(0.2))
         & (s["x"] < np.float32(0.6))),
        (lambda s: ~(s["k"] == 2) | (s["i"] <= -3), lambda s: ~(s["k"] == 2) | (s["i"] <= -3)),
        (lambda s: s["f"], lambda s: s["f"]),
        (lambda s: (s["i"] != 0) & s["f"] & (0.1 < s["x"]),
         lambda s: (s["i"] != 0) & s["f"] & (s["x"] > np.float32(0.1))),
        (lambda s: s["x"] > 2.0, lambda s: s["x"] > 2.0),  # nothing selected
        (lambda s: s["x"] >= 0.0, lambda s: s["x"] >= 0.0),  # everything selected
    ]
    from jaxabm_gb300 import select as sel
    for cond, ref in conds:
        idx, c = select_where(st, cond)
        assert sel.last_path == "predicate"
        want = np.nonzero(ref(h))[0]
        assert c == len(want) and np.array_equal(idx.cpu().numpy(), want)


def test_select_uses_predicate_path_and_falls_back(cuda):
    """AgentList.select runs simple conditions as predicate programs and anything else
    through an eager mask; both give numpy's selection."""
    import jaxabm_gb300 as jx
    from jaxabm_gb300 import select as sel

    class M(jx.Model):
        def setup(self):
            self.walkers = self.add_agents(5000, jx.RandomWalker, name="walkers")

    m = M({"steps": 2, "seed": 3})
    m.run()
    x, y = m.walkers.x.cpu().numpy(), m.walkers.y.cpu().numpy()
    a = m.walkers.select(lambda s: (s["x"] < 0.3) | (s["y"] > 0.8))
    assert sel.last_path == "predicate"
    keep = (x < np.float32(0.3)) | (y > np.float32(0.8))
    assert len(a) == keep.sum() and np.array_equal(a.x.cpu().numpy(), x[keep])
    b = m.walkers.select(lambda s: (s["x"] + s["y"]) > 1.0)
    assert sel.last_path == "mask"
    keep = (x + y) > 1.0
    assert len(b) == keep.sum() and np.array_equal(b.y.cpu().numpy(), y[keep])


def test_select_where_rejects_bad_programs(cuda):
    from jaxabm_gb300 import _lib
    from jaxabm_gb300.select import ATTR_DTYPE, OP_DTYPE
    x = torch.rand(100, device="cuda")
    attrs = np.array([(x.data_ptr(), 0, 0)], dtype=ATTR_DTYPE)
    idx = torch.empty(100, dtype=torch.int32, device="cuda")
    cnt = torch.empty(1, dtype=torch.int64, device="cuda")
    ws = torch.empty(4096, dtype=torch.uint8, device="cuda")
    L = _lib.load()
    for prog in ([(7, 0, 0.0)], [(3, 0, 0.5), (3, 0, 0.2)], [(3, 1, 0.5)], [(12, 0, 0.0)]):
        ops = np.array(prog, dtype=OP_DTYPE)
        assert L.abm_select_where(attrs.ctypes.data, 1, ops.ctypes.data, len(prog), 100,
                                  idx.data_ptr(), cnt.data_ptr(), ws.data_ptr(), ws.numel(),
                                  None) == _lib.ABM_ERR_BADARG, prog
