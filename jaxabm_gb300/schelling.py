"""Schelling segregation on a torus Grid: registered agent and model.

Agent semantics (partitionable ``jax.random``; agent ``i`` holds
``agent_key = split(coll_key, N)[i]``, jaxabm/agent.py:156), all agents reading the
pre-step grid::

    occ, same = occupied Moore-8 neighbours, and those of the agent's type
    unhappy    = same / occ < threshold   (as den * same < num * occ, threshold = num/den
                                           exactly; the workload's 37.5 % is 3/8)
    if unhappy: idx = min(floor(uniform(agent_key) * e), e - 1) into the ascending list of
                the e empty cells; claim that cell; the lowest claiming id moves

The reference's Schelling example leaves both the neighbourhood rule and the move as
placeholders (examples/models/schelling_model.py:54-68); its setup -- types split 50/50
by id, positions from ``numpy.random.RandomState(seed).shuffle`` of the cells
(schelling_model.py:89-93,147-170) -- is kept.  Steps run in ``abm_schelling_run``.
"""

from fractions import Fraction

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


def threshold_fraction(threshold):
    """(num, den) of a similarity threshold: an exact fraction for a (num, den) pair or a
    number (a float is taken at its exact value when that has a small denominator, e.g.
    0.375 -> 3/8, else at the nearest fraction with a denominator of at most 10^6; the
    unhappiness test compares same/occ with occ <= 8, so the decisions are those of the
    float itself unless it lies within 1e-12 of a fraction k/occ)."""
    if isinstance(threshold, (tuple, list)):
        num, den = (int(v) for v in threshold)
    else:
        f = Fraction(float(threshold)).limit_denominator(10 ** 6)
        num, den = f.numerator, f.denominator
    if den <= 0 or num < 0 or num > (1 << 27) or den > (1 << 27):
        raise ValueError(f"bad Schelling threshold {threshold!r}")
    return num, den


class SchellingKernel(StepKernel):
    name = "schelling"
    attributes = ("position", "type")
    metrics = ("unhappy", "moved")
    params = {"threshold": 0.375}
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
        num, den = threshold_fraction(params["threshold"])
        _lib.call("abm_schelling_run", _dev.ptr(p), _dev.ptr(t), n, W, H, _dev.ptr(grid),
                  _dev.ptr(ca), _dev.ptr(coll_keys), steps, num, den, _dev.ptr(stats),
                  _dev.ptr(ws), ws.numel(), _dev.stream_handle())
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
    ``threshold`` (similarity threshold, 0.375 = 3/8; a number or a (num, den) pair),
    ``steps`` (200), ``seed`` (1).  Records ``unhappy`` and ``moved`` every step."""

    def setup(self):
        W = int(self.p.get("width", 256))
        H = int(self.p.get("height", W))
        self.grid = Grid(self, (W, H), periodic=True)
        pos, types = initial_layout(W, H, float(self.p.get("density", 0.9)),
                                    float(self.p.get("ratio", 0.5)), int(self.seed))
        self.env.add_state("schelling_layout", (pos, types))
        self.agents = self.add_agents(len(pos), SchellingAgent, name="agents",
                                      threshold=self.p.get("threshold", 0.375))


# numpy view of abm_schelling_member (include/jaxabm_gb300.h), 72 bytes
MEMBER_DTYPE = np.dtype([("pos", "<u8"), ("type", "<u8"), ("grid", "<u8"), ("cell_agent", "<u8"),
                         ("coll_keys", "<u8"), ("stats", "<u8"), ("workspace", "<u8"),
                         ("n", "<i8"), ("thr_num", "<i4"), ("thr_den", "<i4")])
assert MEMBER_DTYPE.itemsize == 72
CLUSTER_MAX_CELLS = 1 << 18


def ensemble_member(model):
    """``(W, H, density, ratio, threshold, seed, steps)`` of a ``SchellingModel`` that can run
    as a batch member, else None."""
    if not isinstance(model, SchellingModel) or model._hooks() != (None, None) \
            or type(model).setup is not SchellingModel.setup:
        return None
    p = model.p
    W = int(p.get("width", 256))
    H = int(p.get("height", W))
    return (W, H, float(p.get("density", 0.9)), float(p.get("ratio", 0.5)),
            threshold_fraction(p.get("threshold", 0.375)), int(model.seed), int(model.steps))


def run_ensemble(models):
    """Schelling models of one grid shape and step count run in one launch, one
    thread-block cluster per model (``abm_schelling_run_batch``; grids of up to 2^18
    cells); returns one ``Results`` per model equal to its own ``run()`` (keys ``step``,
    ``unhappy``, ``moved`` and the final ``agents.agents.*`` states), or None unless every
    model is a batchable ``SchellingModel``."""
    from . import random as jrandom
    from .agentpy import Results
    specs = [ensemble_member(m) for m in models]
    if any(s is None for s in specs) or any(s[0] * s[1] > CLUSTER_MAX_CELLS for s in specs):
        return None
    out = [None] * len(models)
    groups = {}
    for k, s in enumerate(specs):
        groups.setdefault((s[0], s[1], s[6]), []).append(k)
    dev = _dev.device()
    L = _lib.load()
    for (W, H, steps), idx in groups.items():
        M = len(idx)
        layouts = [initial_layout(W, H, specs[k][2], specs[k][3], specs[k][5]) for k in idx]
        ns = [len(pos) for pos, _ in layouts]
        seeds = np.array([specs[k][5] for k in idx], dtype=np.uint64)
        keys = np.stack([(seeds >> np.uint64(32)).astype(np.uint32),
                         (seeds & np.uint64(0xFFFFFFFF)).astype(np.uint32)], axis=1)
        rng = jrandom.split(_dev.keys_from_numpy(keys), 2)[:, 0].contiguous()
        ck = (jrandom.keychain(rng, steps, 1).reshape(M, steps, 2).contiguous() if steps > 0
              else None)
        states, tables = [], np.zeros(M, dtype=MEMBER_DTYPE)
        stats = torch.zeros((M, max(steps, 1), 2), dtype=torch.int32, device=dev)
        status = torch.zeros(M, dtype=torch.int32, device=dev)
        for j, (pos, types) in enumerate(layouts):
            p = torch.from_numpy(pos).to(dev)
            t = torch.from_numpy(types).to(dev)
            grid = torch.empty(W * H, dtype=torch.int8, device=dev)
            ca = torch.empty(W * H, dtype=torch.int32, device=dev)
            ws = _dev.workspace(L.abm_schelling_workspace_bytes(ns[j], W, H))
            _lib.call("abm_schelling_place", _dev.ptr(p), _dev.ptr(t), ns[j], W, H,
                      _dev.ptr(grid), _dev.ptr(ca), _dev.ptr(status[j:]), _dev.stream_handle())
            states.append((p, t, grid, ca, ws))
            num, den = specs[idx[j]][4]
            tables[j] = (p.data_ptr(), t.data_ptr(), grid.data_ptr(), ca.data_ptr(),
                         ck[j].data_ptr() if ck is not None else 0, stats[j].data_ptr(),
                         ws.data_ptr(), ns[j], num, den)
        if int(status.max().item()) != 0:
            raise ValueError("Schelling layout: position out of range or two agents on one cell")
        if steps > 0:
            d_tab = torch.from_numpy(tables.view(np.uint8).copy()).to(dev)
            _lib.call("abm_schelling_run_batch", _dev.ptr(d_tab), M, W, H, steps,
                      _dev.stream_handle())
        host_stats = stats.cpu().numpy()
        for j, k in enumerate(idx):
            p, t, grid, ca, _ = states[j]
            data = {"agents.agents.position": p.cpu().numpy(),
                    "agents.agents.type": t.cpu().numpy(),
                    "agents.agents._cell_agent": ca.cpu().numpy()}
            if steps > 0:
                data = {"step": list(range(1, steps + 1)),
                        "unhappy": host_stats[j, :steps, 0].tolist(),
                        "moved": host_stats[j, :steps, 1].tolist(), **data}
            out[k] = Results(data)
    return out
