"""API behaviour of the host layer, mirroring the reference's unit tests
(tests/unit/test_model.py, test_agent.py, test_api.py, test_core.py of JaxABM).  Nothing
here launches a kernel: these run without a GPU."""

import os
import pickle

import numpy as np
import pytest

import jaxabm_gb300 as jx
from jaxabm_gb300 import registry
from jaxabm_gb300.agentpy import AgentWrapper


class Plain(jx.Agent):
    """Unregistered agent: allowed to exist, rejected at initialisation."""

    def setup(self):
        return {"x": 1.0}

    def step(self, model_state):
        return {"x": self._state["x"] + 1}


def test_model_config_defaults():
    c = jx.ModelConfig()
    assert (c.seed, c.steps, c.track_history, c.collect_interval) == (0, 100, True, 1)
    c = jx.ModelConfig(seed=42, steps=20, track_history=False, collect_interval=5)
    assert (c.seed, c.steps, c.track_history, c.collect_interval) == (42, 20, False, 5)


def test_agent_collection_validates_size():
    with pytest.raises(ValueError):
        jx.AgentCollection(AgentWrapper(jx.RandomWalker), 0)
    with pytest.raises(ValueError):
        jx.AgentCollection(AgentWrapper(jx.RandomWalker), -3)
    with pytest.raises(ValueError):
        jx.AgentCollection(AgentWrapper(jx.RandomWalker), 2.5)


def test_agent_collection_init_requires_model_config():
    coll = jx.AgentCollection(AgentWrapper(jx.RandomWalker), 10)
    with pytest.raises(TypeError):
        coll.init(None, {"seed": 0})


def test_update_before_init_raises():
    coll = jx.AgentCollection(AgentWrapper(jx.RandomWalker), 10)
    with pytest.raises(ValueError):
        coll.update({}, None, jx.ModelConfig())


def test_unregistered_agent_rejected_before_any_launch():
    m = jx.JaxModel(config=jx.ModelConfig(seed=1))
    m.add_agent_collection("p", jx.AgentCollection(AgentWrapper(Plain), 10))
    with pytest.raises(jx.UnregisteredAgentError):
        m.initialize()
    assert not m._is_initialized
    with pytest.raises(jx.UnregisteredAgentError):
        registry.lookup(Plain)


def test_unregistered_error_is_type_error():
    assert issubclass(jx.UnregisteredAgentError, TypeError)


def test_subclass_of_registered_agent():
    class SameWalker(jx.RandomWalker):
        pass

    class OtherWalker(jx.RandomWalker):
        def step(self, model_state=None, key=None):
            return {}

    assert registry.lookup(SameWalker) is registry.lookup(jx.RandomWalker)
    with pytest.raises(jx.UnregisteredAgentError):
        registry.lookup(OtherWalker)


def test_register_and_unregister():
    class K(registry.StepKernel):
        name = "k"

    registry.register_step(Plain, K())
    try:
        assert registry.lookup(Plain).name == "k"
    finally:
        registry.unregister_step(Plain)
    with pytest.raises(TypeError):
        registry.register_step(Plain, object())


def test_model_errors():
    m = jx.JaxModel()
    with pytest.raises(ValueError):
        m.initialize()  # no collections
    with pytest.raises(RuntimeError):
        m.step()  # not initialised


def test_model_env_state_and_model_state():
    m = jx.JaxModel(params={"a": 1})
    m.add_env_state("price", 1.5)
    m.add_env_state("counter", 0)
    coll = jx.AgentCollection(AgentWrapper(jx.RandomWalker), 5)
    m.add_agent_collection("walkers", coll)
    s = m.model_state()
    assert s["time_step"] == 0 and s["env"] == {"price": 1.5, "counter": 0}
    assert "agents_walkers" in s and s["agents_walkers"] is None
    assert m.agent_collections == {"walkers": coll}
    assert m.state["env"] == {"price": 1.5, "counter": 0}


def test_wrapper_init_state_and_update():
    class A(jx.Agent):
        def setup(self):
            return {"v": 1}

        def step(self, model_state):
            return {"v": self._state["v"] + model_state["inc"]}

    w = AgentWrapper(A, {"p": 3})
    assert w.agent_instance.p == {"p": 3}
    assert w.init_state(jx.ModelConfig(), None) == {"v": 1}
    assert w.update({"v": 1}, {"inc": 2}, jx.ModelConfig(), None) == {"v": 3}


def test_wrapper_rejects_non_dict():
    class Bad(jx.Agent):
        def setup(self):
            return 5

        def step(self, model_state):
            return [1]

    class NoneAgent(jx.Agent):
        def setup(self):
            return None

        def step(self, model_state):
            return None

    w = AgentWrapper(Bad)
    with pytest.raises(ValueError):
        w.init_state(jx.ModelConfig(), None)
    with pytest.raises(ValueError):
        w.update({}, {}, jx.ModelConfig(), None)
    w2 = AgentWrapper(NoneAgent)
    assert w2.init_state(jx.ModelConfig(), None) == {}
    assert w2.update({"a": 1}, {}, jx.ModelConfig(), None) == {"a": 1}


def test_agent_attribute_proxy():
    a = Plain()
    a.speed = 3
    assert a.speed == 3 and a._state == {"speed": 3}
    with pytest.raises(AttributeError):
        _ = a.missing


def test_model_add_agents_names_and_lazy_instances():
    class M(jx.Model):
        def setup(self):
            pass

    m = M({"steps": 5, "seed": 3})
    lst = m.add_agents(1000, jx.RandomWalker)
    assert lst.name == "randomwalkers" and len(lst) == 1000
    named = m.add_agents(10, jx.RandomWalker, name="w", sigma=0.5)
    assert named.params == {"sigma": 0.5}
    a = m.get_agent("w", 3)
    assert a.id == 3 and a.p == {"sigma": 0.5} and a.model is m
    assert m.get_agent("w", 10) is None and m.get_agent("nope", 0) is None
    assert len(m._agent_instances["randomwalkers"]._made) == 0  # no 1000 objects up front


def test_model_defaults_and_record():
    m = jx.Model()
    assert m.p == {} and m.seed == 0 and m.steps == 100
    m = jx.Model({"seed": 7, "steps": 3})
    assert m.seed == 7 and m.steps == 3
    assert jx.Model({"seed": 7}, seed=9).seed == 9
    m.record("x", 1)
    m.record("x", 2)
    assert m._recorded_data == {"x": [1, 2]}


def test_environment_state():
    m = jx.Model()
    m.env.add_state("temp", 25.0)
    m.env.rate = 0.1
    assert m.env.temp == 25.0 and m.env.rate == 0.1
    assert m.env.state == {"temp": 25.0, "rate": 0.1}
    with pytest.raises(AttributeError):
        _ = m.env.nothing


def test_network_edges_and_neighbors():
    m = jx.Model()
    net = jx.Network(m)
    net.add_edge(0, 1)
    net.add_edge(1, 2)
    net.add_edge(3, 3)
    e = m.env.network_edges
    assert e.tolist() == [[0, 1], [1, 0], [1, 2], [2, 1], [3, 3]]
    assert net.get_neighbors(1).tolist() == [0, 2]
    d = jx.Network(jx.Model(), directed=True)
    d.add_edge(0, 1)
    d.add_edge(0, 2)
    assert d.get_neighbors(0).tolist() == [1, 2] and d.get_neighbors(1).tolist() == []
    net.add_edges([[4, 5], [5, 6]])
    assert net.get_neighbors(5).tolist() == [4, 6]


def test_grid_env_state():
    m = jx.Model()
    g = jx.Grid(m, (10, 20), periodic=True)
    assert m.env.grid_shape == (10, 20) and m.env.grid_periodic is True
    assert g.shape == (10, 20)


def test_results_roundtrip(tmp_path):
    data = {"step": [1, 2, 3], "mean_x": [0.5, 0.51, 0.52],
            "agents.walkers.x": np.arange(4, dtype=np.float32)}
    r = jx.Results(data)
    assert r.variables.walkers.x[2] == 2.0 and len(r.variables.walkers.x) == 4
    p = str(tmp_path / "r.pkl")
    r.save(p)
    r2 = jx.Results.load(p)
    assert r2["mean_x"] == [0.5, 0.51, 0.52]
    assert np.array_equal(r2["agents.walkers.x"], data["agents.walkers.x"])


def test_format_time_and_convert():
    assert jx.format_time(5.0) == "5.00s"
    assert jx.format_time(75.5) == "1m 15.50s"
    assert jx.format_time(3725) == "1h 2m 5.00s"
    import torch
    out = jx.convert_to_numpy({"a": [torch.tensor([1, 2])], "b": (torch.tensor(3.0),)})
    assert isinstance(out["a"][0], np.ndarray) and out["b"][0] == 3.0


def test_library_required(monkeypatch, tmp_path):
    from jaxabm_gb300 import _lib
    with pytest.raises(RuntimeError):
        _lib.load(str(tmp_path / "missing.so"))


def test_status_errors_raise():
    from jaxabm_gb300 import _lib
    with pytest.raises(_lib.AbmError) as e:
        _lib.check(_lib.ABM_ERR_WORKSPACE, "abm_x")
    assert "workspace too small" in str(e.value) and e.value.status == _lib.ABM_ERR_WORKSPACE


def test_server_work_and_order_tables():
    """Host tables of the SIR server: tiles of each resident request in slot order, padded
    with the inactive row; the resident kernel's order lists live requests largest first
    (ties in admission order), then every other row once."""
    import numpy as np
    from jaxabm_gb300.serving import order_table, work_table
    table, k = work_table([3, 0, 5], [8192 * 2 + 1, 10, 8192], dummy=9, capacity=8, tile=8192)
    assert k == 5
    assert table[:5].tolist() == [[3, 0, 8192, 0], [3, 8192, 16384, 0], [3, 16384, 16385, 0],
                                  [0, 0, 10, 0], [5, 0, 8192, 0]]
    assert (table[5:, 0] == 9).all() and (table[5:, 1:] == 0).all()
    empty, k0 = work_table([], [], dummy=2, capacity=3)
    assert k0 == 0 and (empty[:, 0] == 2).all()
    order = order_table([4, 1, 6], [100, 300, 100], total=8)
    assert order.tolist() == [1, 4, 6, 0, 2, 3, 5, 7]
    assert sorted(order.tolist()) == list(range(8))
    import pytest
    with pytest.raises(ValueError):
        work_table([0], [8192 * 5], dummy=1, capacity=4)


def test_schelling_threshold_fraction():
    from jaxabm_gb300.schelling import threshold_fraction
    assert threshold_fraction(0.375) == (3, 8)
    assert threshold_fraction(0.5) == (1, 2)
    assert threshold_fraction(0.3) == (3, 10)
    assert threshold_fraction((5, 8)) == (5, 8)
    assert threshold_fraction(0) == (0, 1) and threshold_fraction(1) == (1, 1)
    # decisions depend on the threshold only through same/occ with occ <= 8
    for t in (0.1, 0.3, 0.37, 0.51, 0.74, 0.999):
        num, den = threshold_fraction(t)
        for occ in range(1, 9):
            for same in range(occ + 1):
                assert (den * same < num * occ) == (same / occ < t), (t, same, occ)
    with pytest.raises(ValueError):
        threshold_fraction((1, 0))


def test_select_condition_compiler():
    """Conditions made of attribute comparisons with numbers and &, |, ~ become postfix
    predicate programs (a reflected comparison `c < s[a]` is `s[a] > c`; a bool attribute
    alone is `!= 0`); anything else is left to eager evaluation (None)."""
    import torch
    from jaxabm_gb300.select import (SELECT_AND, SELECT_EQ, SELECT_GT, SELECT_LE, SELECT_NE,
                                     SELECT_NOT, SELECT_OR, compile_condition)
    st = {"x": torch.zeros(10), "k": torch.zeros(10, dtype=torch.int8),
          "f": torch.zeros(10, dtype=torch.bool), "d": torch.zeros(10, dtype=torch.float64),
          "m": torch.zeros((10, 2))}
    assert compile_condition(lambda s: (s["x"] > 0.5) & ~(s["k"] == 2), st) == (
        [(SELECT_GT, 0, 0.5), (SELECT_EQ, 1, 2.0), (SELECT_NOT, 0, 0.0), (SELECT_AND, 0, 0.0)],
        ["x", "k"])
    assert compile_condition(lambda s: 0.25 < s["x"], st) == ([(SELECT_GT, 0, 0.25)], ["x"])
    assert compile_condition(lambda s: s["f"], st) == ([(SELECT_NE, 0, 0.0)], ["f"])
    assert compile_condition(lambda s: (s["x"] > 0.1) | (s["x"] <= 0.9), st) == (
        [(SELECT_GT, 0, 0.1), (SELECT_LE, 0, 0.9), (SELECT_OR, 0, 0.0)], ["x"])
    for cond in (lambda s: s["x"] * 2 > 1, lambda s: s["d"] > 1, lambda s: s["m"] > 0,
                 lambda s: (s["x"] > 0.1) and (s["x"] < 0.5), lambda s: s["x"] > s["x"],
                 lambda s: torch.ones(10, dtype=torch.bool), lambda s: s.get("x"),
                 lambda s: s["nope"] > 0):
        assert compile_condition(cond, st) is None
    many = lambda s: ((s["x"] > 0) & (s["x"] > 1) & (s["x"] > 2) & (s["x"] > 3) & (s["x"] > 4)
                      & (s["x"] > 5) & (s["x"] > 6) & (s["x"] > 7) & (s["x"] > 8))  # 17 ops
    assert compile_condition(many, st) is None


def test_state_snapshot_and_restore_helpers():
    """The copy and in-place restore behind Model.state_dict / load_state_dict (CPU
    tensors stand in for device ones)."""
    import torch
    from jaxabm_gb300.model import _restore, _snapshot
    grid = torch.arange(12, dtype=torch.int8)
    view = grid.view(3, 4)
    env = {"grid": view, "shape": (3, 4), "nested": {"a": torch.ones(2)}, "k": 7}
    snap = _snapshot(env)
    view.add_(1)
    env["nested"]["a"].mul_(5)
    assert torch.equal(snap["grid"], torch.arange(12, dtype=torch.int8).view(3, 4))
    assert torch.equal(snap["nested"]["a"], torch.ones(2))
    out = _restore(env, snap)
    assert out is env and env["grid"] is view  # same shape: written in place
    assert torch.equal(grid, torch.arange(12, dtype=torch.int8))
    assert torch.equal(env["nested"]["a"], torch.ones(2)) and env["k"] == 7
    other = {"grid": torch.zeros(5, dtype=torch.int8)}
    _restore(other, snap)  # other shape: replaced by a copy
    assert other["grid"].shape == (3, 4) and other["grid"] is not snap["grid"]
    assert _restore(None, {"x": 1}) == {"x": 1}


def test_state_dict_requires_initialized_model():
    m = jx.JaxModel()
    with pytest.raises(RuntimeError):
        m.state_dict()


def test_nvtx_ranges_pair_up(monkeypatch):
    """With tracing on, every range is pushed and popped, also when the body raises; with
    tracing off nothing is pushed."""
    import torch
    from jaxabm_gb300 import trace
    log = []
    monkeypatch.setattr(torch.cuda.nvtx, "range_push", lambda name: log.append(("push", name)))
    monkeypatch.setattr(torch.cuda.nvtx, "range_pop", lambda: log.append(("pop",)))
    was = trace.tracing()
    try:
        trace.set_tracing(False)
        with trace.nvtx_range("off"):
            pass
        assert log == []
        jx.set_tracing(True)
        with trace.nvtx_range("Model.run"):
            with trace.nvtx_range("abm_sir_run"):
                pass
        with pytest.raises(KeyError):
            with trace.nvtx_range("fails"):
                raise KeyError("x")
        assert log == [("push", "Model.run"), ("push", "abm_sir_run"), ("pop",), ("pop",),
                       ("push", "fails"), ("pop",)]
    finally:
        trace.set_tracing(was)
