"""Core simulation runtime (mirrors jaxabm/model.py:18-342).

``Model.run`` keeps the reference semantics: the key chain of ``initialize``/``step``
(jaxabm/model.py:118-168), synchronous agent updates, environment update, metrics, and
history every ``collect_interval`` steps.  What changes is where the loop runs:

* fused path: when no Python hook (``update_state_fn``/``metrics_fn``) has to see each
  step, the whole key chain is generated by one kernel and every collection runs all its
  steps in its registered kernel; the per-step metrics the kernels reduce are copied to
  the host once, at the end;
* per-step path: with Python hooks, ``step()`` runs one kernel step per collection and
  calls the hooks with the device tensors, like the reference's Python loop.
"""

import time
from typing import Any, Callable, Dict, List, Optional

import torch

from . import random as jrandom
from .agent import AgentCollection
from .trace import nvtx_range
from .core import ModelConfig, verbose


def _metric_value(v):
    if isinstance(v, torch.Tensor) and v.numel() == 1:
        return v.reshape(()).item()
    return v


def _snapshot(d: Dict[str, Any]) -> Dict[str, Any]:
    """Copy of a state dict: tensors cloned on their device, nested dicts copied, other
    values shared (ints, floats, tuples and the like are immutable)."""
    out = {}
    for k, v in (d or {}).items():
        if isinstance(v, torch.Tensor):
            out[k] = v.detach().clone()
        elif isinstance(v, dict):
            out[k] = _snapshot(v)
        else:
            out[k] = v
    return out


def _restore(dst: Dict[str, Any], src: Dict[str, Any]) -> Dict[str, Any]:
    """Write snapshot ``src`` into ``dst``: a tensor of the same shape and dtype is
    overwritten in place (views of it, such as a grid, stay valid), anything else is
    replaced by a copy; keys missing from ``src`` are dropped."""
    out = {}
    for k, v in src.items():
        cur = dst.get(k) if dst is not None else None
        if isinstance(v, torch.Tensor):
            if (isinstance(cur, torch.Tensor) and cur.shape == v.shape and cur.dtype == v.dtype
                    and cur.device == v.device):
                cur.copy_(v)
                out[k] = cur
            else:
                out[k] = v.detach().clone()
        elif isinstance(v, dict):
            out[k] = _restore(cur if isinstance(cur, dict) else {}, v)
        else:
            out[k] = v
    if dst is not None:
        dst.clear()
        dst.update(out)
        return dst
    return out


class Model:
    """Core model class (jaxabm/model.py:18-342)."""

    def __init__(self, params: Optional[Dict[str, Any]] = None,
                 config: Optional[ModelConfig] = None,
                 update_state_fn: Optional[Callable] = None,
                 metrics_fn: Optional[Callable] = None):
        self.config = config or ModelConfig()
        self._rng = None  # PRNGKey(config.seed) on the device, created by initialize()
        self._agent_collections: Dict[str, AgentCollection] = {}
        self._env_state: Dict[str, Any] = {}
        self._state: Optional[Dict[str, Any]] = None
        self._params = params or {}
        self._update_state_fn = update_state_fn
        self._metrics_fn = metrics_fn
        self._time_step = 0
        self._history: List[Dict[str, Any]] = []
        self._is_initialized = False
        self.last_run_seconds = None

    # -- construction -----------------------------------------------------------------
    def add_agent_collection(self, name: str, agent_collection: AgentCollection) -> None:
        if self._is_initialized:
            raise RuntimeError("Cannot add agent collections after model is initialized")
        self._agent_collections[name] = agent_collection

    def add_env_state(self, name: str, value: Any) -> None:
        if self._is_initialized and self._state is not None:
            self._state.setdefault("env", {})[name] = value
        if self._env_state is None:
            self._env_state = {}
        self._env_state[name] = value

    def model_state(self) -> Dict[str, Any]:
        state = {"time_step": self._time_step, "env": self._env_state}
        for name, collection in self._agent_collections.items():
            state[f"agents_{name}"] = collection.states
        return state

    # -- lifecycle ----------------------------------------------------------------------
    def initialize(self) -> None:
        """keys = split(PRNGKey(seed), C + 1); rng = keys[0]; collection i initialises
        from keys[i + 1] (jaxabm/model.py:118-144)."""
        if not self._agent_collections:
            raise ValueError("No agent collections added to model")
        # resolve every kernel first: an unregistered class fails before any launch
        for collection in self._agent_collections.values():
            _ = collection.kernel
        keys = jrandom.split(jrandom.PRNGKey(self.config.seed), len(self._agent_collections) + 1)
        self._rng = keys[0].clone()
        for i, collection in enumerate(self._agent_collections.values()):
            if getattr(collection, "model_config", None) is None:
                collection.model_config = self.config
            collection.bind_env(self._env_state)
            collection.init(keys[i + 1].clone(), self.config)
        self._is_initialized = True
        self._state = {"env": self._env_state.copy()}

    def _fusable(self) -> bool:
        if self._update_state_fn is not None or self._metrics_fn is not None:
            return False
        return all(c.kernel.independent for c in self._agent_collections.values())

    def _kernel_metrics(self, rows: Dict[str, Any]) -> Dict[str, Any]:
        out = {}
        single = len(self._agent_collections) == 1
        for name, row in rows.items():
            if row is None:
                continue
            kernel = self._agent_collections[name].kernel
            for j, m in enumerate(kernel.metrics):
                out[m if single else f"{name}.{m}"] = row[j]
        return out

    def step(self) -> Dict[str, Any]:
        """One step (jaxabm/model.py:146-216)."""
        with nvtx_range("Model.step"):
            return self._step()

    def _step(self) -> Dict[str, Any]:
        if not self._is_initialized:
            raise RuntimeError("Model must be initialized before stepping. Call initialize() first.")
        want_update = self._update_state_fn is not None
        ck = jrandom.keychain(self._rng, 1, len(self._agent_collections), update_keys=want_update)
        if want_update:
            ck, uk = ck
        current_model_state = self.model_state()
        rows = {}
        for c, (name, collection) in enumerate(self._agent_collections.items()):
            collection.update(current_model_state, ck[0, c], self.config)
            rows[name] = collection._last_metrics
        updated_agent_states = {n: c.states for n, c in self._agent_collections.items()}
        if want_update:
            self._env_state = self._update_state_fn(self._env_state, updated_agent_states,
                                                    self._params, uk[0])
            for collection in self._agent_collections.values():
                collection.bind_env(self._env_state)
        metrics = self._kernel_metrics(rows)
        if self._metrics_fn is not None:
            metrics.update(self._metrics_fn(self._env_state, updated_agent_states, self._params))
        self._time_step += 1
        if self.config.track_history and self._time_step % self.config.collect_interval == 0:
            self._history.append({"time_step": self._time_step, "metrics": metrics})
        return metrics

    def _run_fused(self, steps: int) -> None:
        ncoll = len(self._agent_collections)
        coll_keys = jrandom.keychain(self._rng, steps, ncoll)
        per_coll = {}
        for c, (name, collection) in enumerate(self._agent_collections.items()):
            per_coll[name] = collection.run_steps(coll_keys[:, c].contiguous())
        host = {n: (m.cpu() if m is not None else None) for n, m in per_coll.items()}
        interval = self.config.collect_interval
        for t in range(steps):
            self._time_step += 1
            if self.config.track_history and self._time_step % interval == 0:
                rows = {n: (m[t] if m is not None else None) for n, m in host.items()}
                self._history.append({"time_step": self._time_step,
                                      "metrics": self._kernel_metrics(rows)})

    def run(self, steps: Optional[int] = None) -> Dict[str, List[Any]]:
        """Run ``steps`` steps and return ``{'step': [...], metric: [...]}``
        (jaxabm/model.py:218-262)."""
        with nvtx_range("Model.run"):
            return self._run(steps)

    def _run(self, steps: Optional[int]) -> Dict[str, List[Any]]:
        if not self._is_initialized:
            self.initialize()
        steps_to_run = steps if steps is not None else self.config.steps
        if self.config.track_history:
            self._history = []
        start = time.time()
        if steps_to_run > 0 and self._fusable():
            self._run_fused(steps_to_run)
        else:
            for _ in range(steps_to_run):
                self.step()
        torch.cuda.synchronize()
        elapsed = time.time() - start
        self.last_run_seconds = elapsed
        if verbose():
            sps = steps_to_run / elapsed if elapsed > 0 else float("inf")
            print(f"Ran {steps_to_run} steps in {elapsed:.2f}s ({sps:.1f} steps/sec)")
        if self.config.track_history and self._history:
            out = {"step": [h["time_step"] for h in self._history]}
            for name in self._history[0]["metrics"].keys():
                vals = [h["metrics"][name] for h in self._history]
                if all(isinstance(v, torch.Tensor) and v.numel() == 1 for v in vals):
                    out[name] = torch.stack([v.reshape(()) for v in vals]).cpu().tolist()
                else:
                    out[name] = [_metric_value(v) for v in vals]
            return out
        return {}

    # -- checkpoint / resume ------------------------------------------------------------
    def state_dict(self) -> Dict[str, Any]:
        """Everything a later :meth:`run` depends on, copied: the step counter, the model
        key, the environment (its tensors, e.g. a Schelling grid, cloned on the device),
        every collection's SoA tensors and key, and the collected history.  A model that
        loads it continues bit for bit like this one (the reference persists only
        ``Results``, jaxabm/agentpy.py:783-806)."""
        if not self._is_initialized:
            raise RuntimeError("Model must be initialized before its state can be saved")
        return {
            "time_step": self._time_step,
            "rng": self._rng.detach().clone(),
            "env": _snapshot(self._env_state),
            "collections": {
                name: {"states": _snapshot(c.states),
                       "key": c._key.detach().clone() if isinstance(c._key, torch.Tensor)
                       else c._key}
                for name, c in self._agent_collections.items()},
            "history": list(self._history),
        }

    def load_state_dict(self, state: Dict[str, Any]) -> None:
        """Resume from :meth:`state_dict` of a model with the same collections (names and
        agent counts); initialises this model first when needed.  Tensors are written in
        place where shapes match, so buffers that kernels or views hold stay valid."""
        if not self._is_initialized:
            self.initialize()
        saved = state["collections"]
        if set(saved) != set(self._agent_collections):
            raise ValueError(f"state has collections {sorted(saved)}, model has "
                             f"{sorted(self._agent_collections)}")
        for name, c in self._agent_collections.items():
            st = saved[name]["states"]
            cur = c.states or {}
            for k, v in st.items():
                have = cur.get(k)
                if (isinstance(v, torch.Tensor) and isinstance(have, torch.Tensor)
                        and v.shape != have.shape):
                    raise ValueError(f"collection {name!r}: state {k!r} has shape "
                                     f"{tuple(v.shape)}, the model's {tuple(have.shape)}")
        self._rng.copy_(state["rng"])
        self._time_step = int(state["time_step"])
        _restore(self._env_state, state["env"])
        for name, c in self._agent_collections.items():
            c._states = _restore(c._states, saved[name]["states"])
            key = saved[name]["key"]
            c._key = key.detach().clone() if isinstance(key, torch.Tensor) else key
            c.bind_env(self._env_state)
        self._history = list(state.get("history", []))
        self._state = {"env": self._env_state.copy()}

    # -- accessors ----------------------------------------------------------------------
    @property
    def agent_collections(self) -> Dict[str, AgentCollection]:
        return self._agent_collections

    @property
    def state(self) -> Dict[str, Any]:
        if self._state is None:
            self._state = {"env": self._env_state.copy()}
        if self._is_initialized:
            self._state["agents"] = {n: c.states for n, c in self._agent_collections.items()}
        return self._state

    def jit_step(self) -> Callable:
        """Pure step function ``(env_state, agent_states, params, key) ->
        (env_state, agent_states, metrics, key)`` over the registered kernels
        (jaxabm/model.py:287-342)."""
        def _step_fn(env_state, agent_states, params, key):
            updated = {}
            rows = {}
            for name, states in agent_states.items():
                collection = self._agent_collections[name]
                ks = jrandom.split(key)
                key, sub = ks[0].clone(), ks[1].clone()
                updated[name], rows[name] = collection.kernel.step(
                    states, sub, collection.params, env_state)
            if self._update_state_fn:
                ks = jrandom.split(key)
                key, update_key = ks[0].clone(), ks[1].clone()
                env_state = self._update_state_fn(env_state, updated, params, update_key)
            metrics = self._kernel_metrics(rows)
            if self._metrics_fn:
                metrics.update(self._metrics_fn(env_state, updated, params))
            return env_state, updated, metrics, key
        return _step_fn
