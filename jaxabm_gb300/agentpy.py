"""AgentPy-like API (mirrors jaxabm/agentpy.py:40-1152): Agent, AgentList, Environment,
Grid, Network, Results and Model, backed by SoA CUDA tensors and registered step kernels.

Differences from the reference that a user can observe, all deliberate:

* ``Agent.setup``/``Agent.step`` may take an optional ``key`` argument: the per-agent key
  ``split(coll_key, N)[i]`` of the protocol (jaxabm/agent.py:156), which the reference's
  ``AgentWrapper.update`` drops (jaxabm/agentpy.py:199-227).
* ``Model.add_agents`` creates agent objects lazily (on ``get_agent``/iteration) instead of
  ``n`` Python objects up front (jaxabm/agentpy.py:968-974).
* ``Model.run`` puts the final agent states into ``Results`` as ``agents.<name>.<var>``;
  the reference intends this (jaxabm/agentpy.py:1103-1106) but its state never holds them.
* ``Network`` takes CSR adjacency directly (``from_csr``/``add_edges``) besides the O(E)
  ``add_edge``.
"""

import inspect
import itertools
import pickle
import time
from typing import Any, Dict, List, Optional, Tuple, Type, Union

import numpy as np
import torch

from . import _dev
from . import random as jrandom
from .agent import AgentCollection, AgentType
from .core import ModelConfig, verbose
from .model import Model as JaxModel
from .select import compact_where
from .utils import convert_to_numpy, format_time


def _accepts_key(fn) -> bool:
    try:
        return "key" in inspect.signature(fn).parameters
    except (TypeError, ValueError):
        return False


class Agent:
    """Base class for agents (jaxabm/agentpy.py:40-154)."""

    def __init__(self):
        self.id = None
        self.model = None
        self.p = {}
        self._state = {}

    def setup(self) -> Dict[str, Any]:
        return {}

    def step(self, model_state: Optional[Dict[str, Any]] = None) -> Dict[str, Any]:
        return self._state

    def update_state(self, new_state: Dict[str, Any]) -> None:
        if self.model is not None and hasattr(self.model, "_update_agent_state"):
            self.model._update_agent_state(self, new_state)
        else:
            self._state.update(new_state)

    def __getattr__(self, name: str) -> Any:
        state = self.__dict__.get("_state")
        if state and name in state:
            return state[name]
        raise AttributeError(f"'{self.__class__.__name__}' object has no attribute '{name}'")

    def __setattr__(self, name: str, value: Any) -> None:
        if name in ("id", "model", "p", "_state"):
            super().__setattr__(name, value)
        else:
            if "_state" not in self.__dict__:
                super().__setattr__("_state", {})
            self.update_state({name: value})


class AgentWrapper(AgentType):
    """Adapter from an Agent class to the AgentType protocol (jaxabm/agentpy.py:157-227)."""

    def __init__(self, agent_class: Type[Agent], params: Optional[Dict[str, Any]] = None):
        self.agent_class = agent_class
        self.params = params or {}
        self.agent_instance = agent_class()
        if params:
            self.agent_instance.p = params

    def init_state(self, model_config: ModelConfig, key=None) -> Dict[str, Any]:
        setup = self.agent_instance.setup
        state = setup(key=key) if _accepts_key(setup) else setup()
        if not isinstance(state, dict):
            if state is None:
                return {}
            raise ValueError(f"Agent.setup() must return a dictionary, got {type(state)}")
        return state

    def update(self, state: Dict[str, Any], model_state: Dict[str, Any],
               model_config: ModelConfig, key=None) -> Dict[str, Any]:
        self.agent_instance._state = state
        step = self.agent_instance.step
        new_state = step(model_state, key=key) if _accepts_key(step) else step(model_state)
        if not isinstance(new_state, dict):
            if new_state is None:
                return state
            raise ValueError(f"Agent.step() must return a dictionary, got {type(new_state)}")
        return new_state


class AgentList:
    """Container of agents of one class (jaxabm/agentpy.py:230-378)."""

    def __init__(self, model: "Model", n: int, agent_class: Type[Agent], **kwargs):
        self.model = model
        self.n = n
        self.agent_class = agent_class
        self.params = kwargs
        self.agent_type = AgentWrapper(agent_class, kwargs)
        self.collection = AgentCollection(agent_type=self.agent_type, num_agents=n)
        self.name = None

    @property
    def states(self) -> Dict[str, Any]:
        jm = getattr(self.model, "_jax_model", None)
        if jm is not None and jm._is_initialized and self.name:
            agent_states = jm.state.get("agents", {})
            if self.name in agent_states and agent_states[self.name] is not None:
                # a selected sub-list owns its own compacted collection
                if self.collection.states is None or self.collection is jm.agent_collections.get(self.name):
                    return agent_states[self.name]
        states = self.collection.states
        return states if states is not None else {}

    def __getattr__(self, name: str) -> Any:
        if name.startswith("__") or name in ("model", "n", "agent_class", "params", "agent_type",
                                              "collection", "name"):
            raise AttributeError(name)
        states = self.states
        if name in states:
            return states[name]
        raise AttributeError(f"'AgentList' object has no attribute '{name}'")

    def __len__(self) -> int:
        return self.n

    def select(self, condition) -> "AgentList":
        """Agents satisfying ``condition(states)`` (jaxabm/agentpy.py:316-345).  A condition
        made of attribute comparisons with numbers and &, |, ~ runs as a predicate program
        inside the compaction kernels; any other condition is evaluated into a mask."""
        states = self.states
        new_states, count = compact_where(states, condition)
        filtered = AgentList.__new__(AgentList)
        filtered.model = self.model
        filtered.n = count
        filtered.agent_class = self.agent_class
        filtered.params = self.params
        filtered.agent_type = self.agent_type
        coll = AgentCollection.__new__(AgentCollection)
        coll.agent_type = self.agent_type
        coll.num_agents = count
        coll.model_config = self.collection.model_config
        coll._key = self.collection._key
        coll._states = new_states
        coll._env = self.collection._env
        coll._last_metrics = None
        filtered.collection = coll
        filtered.name = None
        return filtered

    def __iter__(self):
        if self.name and self.model is not None and self.name in getattr(
                self.model, "_agent_instances", {}):
            yield from self.model._agent_instances[self.name]
            return
        states = self.states
        if not states:
            return
        host = {k: convert_to_numpy(v) for k, v in states.items()}
        num = len(next(iter(host.values())))
        for i in range(num):
            agent = self.agent_class()
            agent.model = self.model
            agent.id = i
            agent.p = self.params
            agent._state = {k: host[k][i] for k in host}
            yield agent


class _LazyAgents:
    """Agent objects of a collection, created on first access (not n up front)."""

    def __init__(self, model, name, n, agent_class, params):
        self._model, self._name, self._n = model, name, n
        self._cls, self._params = agent_class, params
        self._made: Dict[int, Agent] = {}

    def __len__(self):
        return self._n

    def __getitem__(self, i):
        if i < 0:
            i += self._n
        if not 0 <= i < self._n:
            raise IndexError(i)
        a = self._made.get(i)
        if a is None:
            a = self._cls()
            a.id = i
            a.model = self._model
            a.p = self._params
            self._made[i] = a
        return a

    def __iter__(self):
        for i in range(self._n):
            yield self[i]

    def __contains__(self, agent):
        return isinstance(agent, Agent) and self._made.get(agent.id) is agent

    def index(self, agent):
        if agent in self:
            return agent.id
        raise ValueError("agent not in list")


class Environment:
    """Environment state container (jaxabm/agentpy.py:381-462)."""

    def __init__(self, model: "Model"):
        object.__setattr__(self, "model", model)
        object.__setattr__(self, "state", {})

    def add_state(self, name: str, value: Any) -> None:
        self.state[name] = value
        jm = getattr(self.model, "_jax_model", None)
        if jm is not None:
            jm.add_env_state(name, value)

    def __getattr__(self, name: str) -> Any:
        state = self.__dict__.get("state", {})
        if name in state:
            return state[name]
        jm = getattr(self.__dict__.get("model"), "_jax_model", None)
        if jm is not None and jm.state:
            env = jm.state.get("env", {})
            if name in env:
                return env[name]
        raise AttributeError(f"'Environment' object has no attribute '{name}'")

    def __setattr__(self, name: str, value: Any) -> None:
        if name in ("model", "state"):
            object.__setattr__(self, name, value)
            return
        self.state[name] = value
        jm = getattr(self.__dict__.get("model"), "_jax_model", None)
        if jm is not None:
            jm.add_env_state(name, value)


class Grid:
    """2-D grid (jaxabm/agentpy.py:465-527).  ``shape`` is (width, height); a cell (x, y)
    has the flat index ``x * height + y``."""

    def __init__(self, model: "Model", shape: Tuple[int, int], periodic: bool = False):
        self.model = model
        self.shape = tuple(int(s) for s in shape)
        self.periodic = periodic
        self.model.env.add_state("grid_shape", self.shape)
        self.model.env.add_state("grid_periodic", periodic)

    def position_agents(self, agents: AgentList, positions=None) -> None:
        """Place agents: given positions, else ``x = randint(PRNGKey(seed), (n,), 0, width)``
        and ``y = randint(split(key)[1], (n,), 0, height)`` (jaxabm/agentpy.py:496-527)."""
        n = len(agents)
        width, height = self.shape
        if positions is None:
            key = jrandom.PRNGKey(self.model.p.get("seed", 0))
            x = jrandom.randint(key, (n,), 0, width)
            sub = jrandom.split(key)[1].contiguous()
            y = jrandom.randint(sub, (n,), 0, height)
            positions = torch.stack([x, y], dim=1)
        elif not isinstance(positions, torch.Tensor):
            positions = torch.as_tensor(np.asarray(positions), dtype=torch.int32,
                                        device=_dev.device())
        coll = agents.collection
        if coll._states is None:
            coll._states = {}
        coll._states = dict(coll._states)
        coll._states["position"] = positions


def csr_from_edges(edges, n):
    """Device CSR (row_ptr int32[n+1], col int32[E]) of an (E, 2) edge array over nodes
    0..n-1, stable by source (``abm_csr_from_edges``: a radix sort on the device)."""
    from . import _lib
    e = np.ascontiguousarray(np.asarray(edges, dtype=np.int32).reshape(-1, 2))
    dev = _dev.device()
    E = e.shape[0]
    if n <= 0:
        if E:
            raise ValueError("edges given for a network without nodes")
        return (torch.zeros(1, dtype=torch.int32, device=dev),
                torch.zeros(0, dtype=torch.int32, device=dev))
    src = torch.from_numpy(np.ascontiguousarray(e[:, 0])).to(dev)
    dst = torch.from_numpy(np.ascontiguousarray(e[:, 1])).to(dev)
    rp = torch.empty(n + 1, dtype=torch.int32, device=dev)
    col = torch.empty(max(E, 1), dtype=torch.int32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    ws = _dev.workspace(_lib.load().abm_csr_workspace_bytes(E, n))
    _lib.call("abm_csr_from_edges", _dev.ptr(src), _dev.ptr(dst), E, n, _dev.ptr(rp),
              _dev.ptr(col), _dev.ptr(status), _dev.ptr(ws), ws.numel(), _dev.stream_handle())
    if int(status.item()) != 0:
        raise ValueError(f"an edge endpoint lies outside 0..{n - 1}")
    return rp, col[:E]


class Network:
    """Agent network (jaxabm/agentpy.py:530-615), held as an int32 edge list in the
    environment plus CSR adjacency (``network_row_ptr``/``network_col``) for kernels."""

    def __init__(self, model: "Model", directed: bool = False):
        self.model = model
        self.directed = directed
        self._edges = np.zeros((0, 2), dtype=np.int32)
        self.model.env.add_state("network_directed", directed)
        self.model.env.add_state("network_edges", self._edges)

    def add_edge(self, from_agent: Union[Agent, int], to_agent: Union[Agent, int]) -> None:
        """Append (from, to), and the reverse edge when undirected (jaxabm/agentpy.py:559-582)."""
        fid = from_agent.id if isinstance(from_agent, Agent) else int(from_agent)
        tid = to_agent.id if isinstance(to_agent, Agent) else int(to_agent)
        rows = [[fid, tid]]
        if not self.directed and fid != tid:
            rows.append([tid, fid])
        self.add_edges(np.asarray(rows, dtype=np.int32), symmetric=False)

    def add_edges(self, edges, symmetric: Optional[bool] = None) -> None:
        """Bulk append of an (E, 2) edge array; undirected networks add reverse edges."""
        e = np.asarray(edges, dtype=np.int32).reshape(-1, 2)
        if symmetric is None:
            symmetric = not self.directed
        if symmetric:
            rev = e[e[:, 0] != e[:, 1]][:, ::-1]
            e = np.concatenate([e, rev], axis=0)
        self._edges = np.concatenate([self._edges, e], axis=0)
        self.model.env.add_state("network_edges", self._edges)
        self._csr = None

    def from_csr(self, row_ptr, col) -> None:
        """Adopt CSR adjacency directly (row i's neighbours are col[row_ptr[i]:row_ptr[i+1]])."""
        dev = _dev.device()
        rp = torch.as_tensor(np.asarray(row_ptr), dtype=torch.int32).to(dev)
        cl = torch.as_tensor(np.asarray(col), dtype=torch.int32).to(dev)
        self._csr = (rp, cl)
        self.model.env.add_state("network_row_ptr", rp)
        self.model.env.add_state("network_col", cl)

    def csr(self):
        """(row_ptr, col) device tensors; built on the device from the edge list (stable by
        source: a row keeps its edges in the order they were added) when the network was
        given as edges."""
        if getattr(self, "_csr", None) is None:
            e = self._edges
            n = int(e.max()) + 1 if e.size else 0
            rp, col = csr_from_edges(e, n)
            self._csr = (rp, col)
            self.model.env.add_state("network_row_ptr", rp)
            self.model.env.add_state("network_col", col)
        return self._csr

    def get_neighbors(self, agent: Union[Agent, int]):
        """Neighbour ids (jaxabm/agentpy.py:584-615): outgoing when directed, else the
        sorted unique union of both directions."""
        aid = agent.id if isinstance(agent, Agent) else int(agent)
        e = self._edges
        if self.directed:
            return e[e[:, 0] == aid, 1]
        return np.unique(np.concatenate([e[e[:, 0] == aid, 1], e[e[:, 1] == aid, 0]]))


class Results:
    """Simulation results (jaxabm/agentpy.py:618-806)."""

    class VariableContainer:
        def __init__(self, data: Dict[str, Any]):
            self._data = data
            types = {k.split(".")[1] for k in data if k.startswith("agents.")}
            for t in types:
                setattr(self, t, self.AgentContainer(data, t))

        class AgentContainer:
            def __init__(self, data, agent_type):
                self._data = data
                self._agent_type = agent_type
                self._variables = set()
                for key in data:
                    if key.startswith(f"agents.{agent_type}."):
                        var = key.split(".")[-1]
                        self._variables.add(var)
                        setattr(self, var, self.VariableSeries(data[key], var))

            class VariableSeries:
                def __init__(self, values, name):
                    self._values = values
                    self._name = name

                def plot(self, ax=None, **kwargs):
                    import matplotlib.pyplot as plt
                    if ax is None:
                        _, ax = plt.subplots()
                    vals = self._values
                    if len(vals) and hasattr(vals[0], "shape") and len(vals[0].shape) > 0:
                        ax.plot(np.mean(np.array(vals), axis=1), **kwargs)
                        ax.set_ylabel(f"Mean {self._name}")
                    else:
                        ax.plot(vals, **kwargs)
                        ax.set_ylabel(self._name)
                    ax.set_xlabel("Time")
                    return ax

                def __getitem__(self, key):
                    return self._values[key]

                def __len__(self):
                    return len(self._values)

    def __init__(self, data: Dict[str, Any]):
        self._data = convert_to_numpy(data)
        self.variables = self.VariableContainer(self._data)

    def __getitem__(self, key):
        return self._data[key]

    def keys(self):
        return self._data.keys()

    @property
    def data(self) -> Dict[str, Any]:
        return self._data

    def plot(self, variables: Optional[List[str]] = None, ax=None, **kwargs):
        import matplotlib.pyplot as plt
        if ax is None:
            _, ax = plt.subplots()
        if variables is None:
            for key, values in self._data.items():
                if isinstance(values, list) and all(isinstance(v, (int, float, np.number))
                                                    for v in values):
                    ax.plot(values, label=key, **kwargs)
        else:
            for var in variables:
                if var in self._data:
                    ax.plot(self._data[var], label=var, **kwargs)
        ax.legend()
        ax.set_xlabel("Time")
        return ax

    def save(self, filename: str) -> None:
        with open(filename, "wb") as f:
            pickle.dump(self._data, f)

    @classmethod
    def load(cls, filename: str) -> "Results":
        with open(filename, "rb") as f:
            return cls(pickle.load(f))


class Model:
    """Base class of AgentPy-like models (jaxabm/agentpy.py:809-1152)."""

    def __init__(self, parameters: Optional[Dict[str, Any]] = None, seed: Optional[int] = None):
        self.p = parameters or {}
        self.seed = seed if seed is not None else self.p.get("seed", 0)
        self.steps = self.p.get("steps", 100)
        self.env = Environment(self)
        self._recorded_data: Dict[str, List[Any]] = {}
        self._agent_lists: Dict[str, AgentList] = {}
        self._jax_model: Optional[JaxModel] = None
        self._current_env_state: Dict[str, Any] = {}
        self._current_agent_states: Dict[str, Any] = {}
        self._running = False
        self._agent_instances: Dict[str, _LazyAgents] = {}

    def setup(self) -> None:
        pass

    def step(self) -> None:
        pass

    def end(self) -> None:
        pass

    def update_state(self, env_state, agent_states, model_params, key):
        """Per-step environment hook (jaxabm/agentpy.py:895-924): runs ``self.step()``."""
        self._current_env_state = dict(env_state)
        self._current_agent_states = agent_states
        self.step()
        new_env_state = dict(env_state)
        new_env_state.update(self.env.state)
        return new_env_state

    def compute_metrics(self, env_state, agent_states, model_params) -> Dict[str, Any]:
        return {}

    def add_agents(self, n: int, agent_class: Type[Agent], name: Optional[str] = None,
                   **kwargs) -> AgentList:
        agent_list = AgentList(self, n, agent_class, **kwargs)
        if name is None:
            name = agent_class.__name__.lower() + "s"
        self._agent_lists[name] = agent_list
        agent_list.name = name
        self._agent_instances[name] = _LazyAgents(self, name, n, agent_class, kwargs)
        return agent_list

    def _update_agent_state(self, agent: Agent, new_state: Dict[str, Any]) -> None:
        """Write an agent's attribute change into the SoA tensors (jaxabm/agentpy.py:978-1011)."""
        for name, agents in self._agent_instances.items():
            if agent in agents:
                index = agents.index(agent)
                coll = self._agent_lists[name].collection
                if coll.states is not None:
                    for k, v in new_state.items():
                        if k in coll.states and isinstance(coll.states[k], torch.Tensor):
                            coll.states[k][index] = v
                agent._state.update(new_state)
                return
        agent._state.update(new_state)

    def get_agent(self, collection_name: str, agent_id: int) -> Optional[Agent]:
        agents = self._agent_instances.get(collection_name)
        if agents is not None and 0 <= agent_id < len(agents):
            return agents[agent_id]
        return None

    def record(self, name: str, value: Any) -> None:
        self._recorded_data.setdefault(name, []).append(value)

    def _hooks(self):
        cls = type(self)
        has_step = cls.step is not Model.step
        has_update = cls.update_state is not Model.update_state
        has_metrics = cls.compute_metrics is not Model.compute_metrics
        return (self.update_state if (has_step or has_update) else None,
                self.compute_metrics if has_metrics else None)

    def core_model(self) -> JaxModel:
        """Run ``setup()`` and return the core :class:`JaxModel` that :meth:`run` drives
        (its collections and environment are this model's), e.g. to step it piecewise or
        to checkpoint it with ``state_dict()`` (jaxabm/agentpy.py:1040-1075)."""
        config = ModelConfig(steps=self.steps, collect_interval=1, seed=self.seed)
        self.setup()
        update_fn, metrics_fn = self._hooks()
        self._dynamic_state_update = update_fn is not None
        self._jax_model = JaxModel(params=self.p, config=config, update_state_fn=update_fn,
                                   metrics_fn=metrics_fn)
        for name, agent_list in self._agent_lists.items():
            self._jax_model.add_agent_collection(name, agent_list.collection)
        for name, value in self.env.state.items():
            self._jax_model.add_env_state(name, value)
        return self._jax_model

    def run(self, steps: Optional[int] = None) -> Results:
        """Set up, run and collect results (jaxabm/agentpy.py:1040-1114)."""
        if steps is not None:
            self.steps = steps
        self._running = True
        self.core_model()
        start = time.time()
        results_dict = self._jax_model.run()
        simulation_time = time.time() - start
        self.end()
        self._running = False
        results_dict.update(self._recorded_data)
        for name, states in self._jax_model.state.get("agents", {}).items():
            for state_name, values in (states or {}).items():
                results_dict[f"agents.{name}.{state_name}"] = values
        results = Results(results_dict)
        self.simulation_time = simulation_time
        if verbose():
            print(f"Simulation executed in {format_time(simulation_time)}")
        return results

    def batch_run(self, parameter_ranges: Dict[str, List[Any]], repetitions: int = 1):
        """Every parameter combination, ``repetitions`` runs each (jaxabm/agentpy.py:1116-1152):
        run ``r`` of a combination is ``self.__class__(params, seed=self.seed + r)``.  The
        reference runs them one after another; here models of a batchable family (SIR,
        random walk, Schelling, opinion; no Python hooks) run as one batched ensemble
        (:func:`jaxabm_gb300.batching.run_ensemble`), each result equal to that model's own
        ``run()``; other models run one by one."""
        from .batching import run_ensemble
        names = list(parameter_ranges.keys())
        keys, models = [], []
        for values in itertools.product(*parameter_ranges.values()):
            params = dict(self.p)
            params.update(zip(names, values))
            for r in range(repetitions):
                keys.append(tuple(values))
                models.append(self.__class__(params, seed=self.seed + r))
        runs = run_ensemble(models) if self._hooks() == (None, None) else None
        if runs is None:
            runs = [m.run() for m in models]
        results = {}
        for values, res in zip(keys, runs):
            results.setdefault(values, []).append(res)
        return results
