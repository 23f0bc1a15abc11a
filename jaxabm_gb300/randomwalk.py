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

import numpy as np
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


def ensemble_member(model):
    """``(n, sigma, seed, steps)`` of a ``RandomWalkModel`` that can run as a batch member
    (no Python hooks, the class's own ``setup``), else None."""
    if not isinstance(model, RandomWalkModel) or model._hooks() != (None, None) \
            or type(model).setup is not RandomWalkModel.setup:
        return None
    p = model.p
    return (int(p.get("n", 10_000)), float(p.get("sigma", 0.01)), int(model.seed),
            int(model.steps))


def run_ensemble(models):
    """Random-walk models run as batches of one launch sequence each (members of one size and
    step count together: ``abm_randomwalk_init_batch`` / ``abm_randomwalk_run_batch``);
    returns one ``Results`` per model, equal to that model's own ``run()`` (keys ``step``,
    ``mean_x``, ``mean_y``, ``agents.walkers.x``, ``agents.walkers.y``), or None unless
    every model is a batchable ``RandomWalkModel``."""
    from .agentpy import Results
    specs = [ensemble_member(m) for m in models]
    if any(s is None for s in specs):
        return None
    out = [None] * len(models)
    groups = {}
    for k, (n, _, _, steps) in enumerate(specs):
        groups.setdefault((n, steps), []).append(k)
    for (n, steps), idx in groups.items():
        M = len(idx)
        seeds = np.array([specs[k][2] for k in idx], dtype=np.uint64)
        keys = np.stack([(seeds >> np.uint64(32)).astype(np.uint32),
                         (seeds & np.uint64(0xFFFFFFFF)).astype(np.uint32)], axis=1)
        pair = jrandom.split(_dev.keys_from_numpy(keys), 2)  # Model.initialize, one collection
        rng, init = pair[:, 0].contiguous(), pair[:, 1].contiguous()
        x = _dev.empty((M, n), torch.float32)
        y = _dev.empty((M, n), torch.float32)
        _lib.call("abm_randomwalk_init_batch", _dev.ptr(x), _dev.ptr(y), n, M, _dev.ptr(init),
                  _dev.stream_handle())
        if steps > 0:
            ck = jrandom.keychain(rng, steps, 1).reshape(M, steps, 2).contiguous()
            sig = torch.tensor([specs[k][1] for k in idx], dtype=torch.float32,
                               device=x.device)
            means = _dev.empty((M, steps, 2), torch.float32)
            ws = _dev.workspace(_lib.load().abm_randomwalk_batch_workspace_bytes(n, steps, M))
            _lib.call("abm_randomwalk_run_batch", _dev.ptr(x), _dev.ptr(y), n, M, _dev.ptr(ck),
                      steps, _dev.ptr(sig), _dev.ptr(means), _dev.ptr(ws), ws.numel(),
                      _dev.stream_handle())
            host_means = means.cpu().numpy()
        hx, hy = x.cpu().numpy(), y.cpu().numpy()
        for j, k in enumerate(idx):
            data = {"agents.walkers.x": hx[j], "agents.walkers.y": hy[j]}
            if steps > 0:
                data = {"step": list(range(1, steps + 1)),
                        "mean_x": host_means[j, :, 0].tolist(),
                        "mean_y": host_means[j, :, 1].tolist(), **data}
            out[k] = Results(data)
    return out
