"""Random-walk agents: the quick-start model with ``jax.random`` noise.

Agent semantics (partitionable ``jax.random``; agent ``i`` holds the key
``split(coll_key, N)[i]`` of ``AgentCollection.update``, jaxabm/agent.py:156)::

    setup(key):  kx, ky = split(key); x = uniform(kx); y = uniform(ky)
    step(model_state, key):  kx, ky = split(key)
                             x = (x + sigma * normal(kx)) % 1.0; y likewise with ky

with per-step metrics ``mean_x``/``mean_y`` (the reference computes these in a Python
``compute_metrics``/``record``, examples/models/random_walk.py:112-139).  All steps of a
run execute in one launch of ``abm_randomwalk_run``.
"""

import torch

from . import _dev
from . import _lib
from . import random as jrandom
from .agentpy import Agent, Model
from .registry import StepKernel, register_step


class RandomWalkKernel(StepKernel):
    name = "randomwalk"
    attributes = ("x", "y")
    metrics = ("mean_x", "mean_y")
    params = {"sigma": 0.01}

    def init(self, n, init_key, params, env):
        x = _dev.empty((n,), torch.float32)
        y = _dev.empty((n,), torch.float32)
        _lib.call("abm_randomwalk_init", _dev.ptr(x), _dev.ptr(y), n, _dev.ptr(init_key),
                  _dev.stream_handle())
        return {"x": x, "y": y}

    def run(self, states, coll_keys, params, env):
        coll_keys = coll_keys.reshape(-1, 2).contiguous()
        steps = coll_keys.shape[0]
        x, y = states["x"], states["y"]
        n = x.shape[0]
        means = _dev.empty((steps, 2), torch.float32)
        ws = _dev.workspace(_lib.load().abm_randomwalk_workspace_bytes(n, steps))
        _lib.call("abm_randomwalk_run", _dev.ptr(x), _dev.ptr(y), n, _dev.ptr(coll_keys), steps,
                  float(params["sigma"]), _dev.ptr(means), _dev.ptr(ws), ws.numel(),
                  _dev.stream_handle())
        return states, means

    def step(self, states, coll_key, params, env):
        states, means = self.run(states, coll_key.reshape(1, 2), params, env)
        return states, means[0]


class RandomWalker(Agent):
    """Random-walk agent on the unit torus (registered: runs on ``abm_randomwalk_*``).

    The Python methods restate the semantics for one agent with the device samplers;
    models never call them (the registered kernel runs every agent)."""

    def setup(self, key=None):
        ks = jrandom.split(key)
        return {"x": jrandom.uniform(ks[0]), "y": jrandom.uniform(ks[1])}

    def step(self, model_state=None, key=None):
        sigma = self.p.get("sigma", 0.01)
        ks = jrandom.split(key)
        x = torch.remainder(self._state["x"] + sigma * jrandom.normal(ks[0]), 1.0)
        y = torch.remainder(self._state["y"] + sigma * jrandom.normal(ks[1]), 1.0)
        return {"x": x, "y": y}


register_step(RandomWalker, RandomWalkKernel())


class RandomWalkModel(Model):
    """N random walkers (parameters ``n``, ``sigma``, ``steps``, ``seed``); records
    ``mean_x``/``mean_y`` every step."""

    def setup(self):
        self.walkers = self.add_agents(int(self.p.get("n", 10_000)), RandomWalker,
                                       name="walkers", sigma=float(self.p.get("sigma", 0.01)))
