"""Agent types and SoA agent collections (mirrors jaxabm/agent.py:19-243).

An :class:`AgentCollection` holds its agents' state as a structure of arrays: one CUDA
tensor per attribute, shape ``(num_agents, ...)``.  Initialisation and updates run on the
step kernel registered for the collection's agent class (see :mod:`.registry`); an
unregistered class raises :class:`UnregisteredAgentError` in :meth:`AgentCollection.init`.
"""

from typing import Any, Callable, Dict, Optional, Protocol

import torch

from .core import ModelConfig
from .registry import lookup
from .trace import nvtx_range

AgentState = Dict[str, Any]


class AgentType(Protocol):
    """Protocol of agent types (jaxabm/agent.py:19-51).

    ``init_state(model_config, key)`` and ``update(state, model_state, model_config, key)``
    describe one agent.  In this engine the registered kernel of the class executes them
    for all agents at once; the methods document the semantics.
    """

    def init_state(self, model_config: Any, key: Any) -> AgentState:
        ...

    def update(self, state: AgentState, model_state: Dict[str, Any], model_config: Any,
               key: Any) -> AgentState:
        ...


class AgentCollection:
    """Collection of agents of one type (jaxabm/agent.py:54-243)."""

    def __init__(self, agent_type: AgentType, num_agents: int):
        if not isinstance(num_agents, int) or isinstance(num_agents, bool) or num_agents <= 0:
            raise ValueError("num_agents must be a positive integer")
        self.agent_type = agent_type
        self.num_agents = num_agents
        self.model_config: Optional[ModelConfig] = None
        self._key = None
        self._states: Optional[Dict[str, torch.Tensor]] = None
        self._env: Dict[str, Any] = {}
        self._last_metrics = None

    # -- kernel binding -----------------------------------------------------------------
    @property
    def kernel(self):
        return lookup(self.agent_type)

    def _param_source(self) -> dict:
        src = {}
        wrapped = getattr(self.agent_type, "params", None)
        if isinstance(wrapped, dict):
            src.update(wrapped)
        for k in self.kernel.params:
            if k not in src and hasattr(self.agent_type, k) and not callable(
                    getattr(self.agent_type, k)):
                src[k] = getattr(self.agent_type, k)
        return src

    @property
    def params(self) -> dict:
        return self.kernel.resolve_params(self._param_source())

    def bind_env(self, env: Dict[str, Any]) -> None:
        """Give the collection the model environment its kernel reads (graph, grid)."""
        self._env = env if env is not None else {}

    # -- reference API ------------------------------------------------------------------
    def init(self, key: Any, model_config: ModelConfig) -> None:
        """Initialise all agents from ``key`` (jaxabm/agent.py:92-130): agent ``i`` gets
        ``split(key, num_agents)[i]`` inside the registered init kernel."""
        if not isinstance(model_config, ModelConfig):
            raise TypeError("model_config must be a ModelConfig instance.")
        if not isinstance(self.num_agents, int) or self.num_agents <= 0:
            raise ValueError("Number of agents must be a positive integer.")
        kernel = self.kernel  # raises UnregisteredAgentError before any launch
        self._key = key
        self.model_config = model_config
        self._states = kernel.init(self.num_agents, key, self.params, self._env)

    def update(self, model_state: Dict[str, Any], key: Any, model_config: ModelConfig) -> None:
        """One synchronous update of every agent (jaxabm/agent.py:132-179)."""
        if self._states is None:
            raise ValueError("Agent collection not initialized. Call init() first.")
        if self.model_config is None:
            raise RuntimeError("Model config not set for AgentCollection. Ensure "
                               "Model.initialize() was called.")
        with nvtx_range(f"AgentCollection.update {self.kernel.name}"):
            self._states, self._last_metrics = self.kernel.step(self._states, key, self.params,
                                                                self._env)

    def run_steps(self, coll_keys: torch.Tensor):
        """``coll_keys.shape[0]`` updates as one fused launch sequence; returns the
        per-step metrics tensor [T, m] (or None)."""
        if self._states is None:
            raise ValueError("Agent collection not initialized. Call init() first.")
        with nvtx_range(f"AgentCollection.run_steps {self.kernel.name}"):
            self._states, metrics = self.kernel.run(self._states, coll_keys, self.params,
                                                    self._env)
        return metrics

    def get_states(self) -> Dict[str, Any]:
        return self._states

    @property
    def states(self) -> Dict[str, torch.Tensor]:
        return self._states

    def aggregate(self, variable: str, fn: Callable = None) -> Any:
        """``fn(states[variable])``; default: the mean (jaxabm/agent.py:198-211)."""
        if self._states is None or variable not in self._states:
            raise ValueError(f"Variable {variable} not found in agent states")
        if fn is None:
            from .select import mean
            return mean(self._states[variable])
        return fn(self._states[variable])

    def filter(self, condition: Callable[[Dict[str, Any]], Any]) -> "AgentCollection":
        """Agents whose ``condition(states)`` mask is true, in ascending id order
        (jaxabm/agent.py:213-243); compaction runs in the warp-ballot kernels, with simple
        conditions evaluated inside them (``select.compact_where``)."""
        from .select import compact_where
        new_states, count = compact_where({k: self._states[k] for k in self._states},
                                          condition)
        filtered = AgentCollection.__new__(AgentCollection)
        filtered.agent_type = self.agent_type
        filtered.num_agents = count
        filtered.model_config = self.model_config
        filtered._key = self._key
        filtered._states = new_states
        filtered._env = self._env
        filtered._last_metrics = None
        return filtered
