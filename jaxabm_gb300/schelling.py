"""Schelling segregation on a torus Grid: registered agent and model.

Agent semantics (partitionable ``jax.random``; agent ``i`` holds
``agent_key = split(coll_key, N)[i]``, jaxabm/agent.py:156), all agents reading the
pre-step grid::

    occ, same = occupied Moore-8 neighbours, and those of the agent's type
    unhappy    = 8 * same < 3 * occ                        (fewer than 37.5% alike)
    if unhappy: idx = min(floor(uniform(agent_key) * e), e - 1) into the ascending list of
                the e empty cells; claim that cell; the lowest claiming id moves

The reference's Schelling example leaves both the neighbourhood rule and the move as
placeholders (examples/models/schelling_model.py:54-68); its setup -- types split 50/50
by id, positions from ``numpy.random.RandomState(seed).shuffle`` of the cells
(schelling_model.py:89-93,147-170) -- is kept.  Steps run in ``abm_schelling_run``.
"""

import numpy as np
import torch

from . import _dev
from . import _lib
from .agentpy import Agent, Grid, Model
from .registry import StepKernel, register_step


def initial_layout(width, height, density=0.9, ratio=0.5, seed=1):
    """(positions int32[n], types int8[n]): ``n = int(density * W * H)`` agents on the first
    ``n`` cells of a ``RandomState(seed)`` shuffle of the cells (index ``x * H + y``);
    the first ``int(n * ratio)`` agents have type 0, the rest type 1."""
    C = int(width) * int(height)
    n = int(density * C)
    cells = np.arange(C, dtype=np.int64)
    np.random.RandomState(int(seed)).shuffle(cells)
    pos = cells[:n].astype(np.int32)
    n0 = int(n * ratio)
    types = np.concatenate([np.zeros(n0, np.int8), np.ones(n - n0, np.int8)])
    return pos, types


class SchellingKernel(StepKernel):
    name = "schelling"
    attributes = ("position", "type")
    metrics = ("unhappy", "moved")
    params = {}
    independent = True

    def init(self, n, init_key, params, env):
        W, H = env["grid_shape"]
        layout = env.get("schelling_layout")
        if layout is None:
            raise ValueError("Schelling agents need env['schelling_layout'] = (positions, types)")
        pos, types = layout
        if len(pos) != n:
            raise ValueError(f"layout has {len(pos)} positions for {n} agents")
        dev = _dev.device()
        p = torch.as_tensor(np.asarray(pos, dtype=np.int32)).to(dev)
        t = torch.as_tensor(np.asarray(types, dtype=np.int8)).to(dev)
        grid = torch.empty(W * H, dtype=torch.int8, device=dev)
        cell_agent = torch.empty(W * H, dtype=torch.int32, device=dev)
        status = torch.zeros(1, dtype=torch.int32, device=dev)
        _lib.call("abm_schelling_place", _dev.ptr(p), _dev.ptr(t), n, W, H, _dev.ptr(grid),
                  _dev.ptr(cell_agent), _dev.ptr(status), _dev.stream_handle())
        if int(status.item()) != 0:
            raise ValueError("Schelling layout: position out of range or two agents on one cell")
        env["grid"] = grid.view(W, H)
        return {"position": p, "type": t, "_cell_agent": cell_agent}

    def run(self, states, coll_keys, params, env):
        coll_keys = coll_keys.reshape(-1, 2).contiguous()
        steps = coll_keys.shape[0]
        W, H = env["grid_shape"]
        p, t, ca = states["position"], states["type"], states["_cell_agent"]
        n = p.numel()
        grid = env["grid"]
        stats = torch.empty((steps, 2), dtype=torch.int32, device=p.device)
        ws = _dev.workspace(_lib.load().abm_schelling_workspace_bytes(n, W, H))
        _lib.call("abm_schelling_run", _dev.ptr(p), _dev.ptr(t), n, W, H, _dev.ptr(grid),
                  _dev.ptr(ca), _dev.ptr(coll_keys), steps, _dev.ptr(stats), _dev.ptr(ws),
                  ws.numel(), _dev.stream_handle())
        return states, stats

    def step(self, states, coll_key, params, env):
        states, stats = self.run(states, coll_key.reshape(1, 2), params, env)
        return states, stats[0]


class SchellingAgent(Agent):
    """Schelling agent on a torus Grid (registered: runs on ``abm_schelling_*``)."""

    def setup(self):
        return {"type": 0, "position": 0}


register_step(SchellingAgent, SchellingKernel())


class SchellingModel(Model):
    """Parameters: ``width``/``height`` (256), ``density`` (0.9), ``ratio`` (0.5),
    ``steps`` (200), ``seed`` (1).  Records ``unhappy`` and ``moved`` every step."""

    def setup(self):
        W = int(self.p.get("width", 256))
        H = int(self.p.get("height", W))
        self.grid = Grid(self, (W, H), periodic=True)
        pos, types = initial_layout(W, H, float(self.p.get("density", 0.9)),
                                    float(self.p.get("ratio", 0.5)), int(self.seed))
        self.env.add_state("schelling_layout", (pos, types))
        self.agents = self.add_agents(len(pos), SchellingAgent, name="agents")
