"""SIR contagion on a Network: registered agent, model and network builders.

Agent semantics (partitionable ``jax.random``; agent ``i`` holds
``agent_key = split(coll_key, N)[i]``, jaxabm/agent.py:156)::

    k_inf, k_rec = split(agent_key)
    S: becomes I if, for some CSR slot k of its row whose neighbour is I,
       uniform(k_inf, (deg,))[k] < beta            (a bernoulli(beta) draw per I-edge)
    I: becomes R if uniform(k_rec) < gamma
    R: stays R

with the compartments' counts ``S``, ``I``, ``R`` recorded after every step.  The step runs
in ``abm_sir_run``/``abm_sir_steps``: one byte per agent holds its compartment and its
number of infected neighbours, so only agents that can change (susceptible agents with an
infected neighbour, infected agents) read their CSR row or draw, and each change updates
its neighbours' counts.
"""

import ctypes

import numpy as np
import torch

from . import _dev
from . import _lib
from .agentpy import Agent, Model, Network
from .registry import StepKernel, register_step

SUSCEPTIBLE, INFECTED, RECOVERED = 0, 1, 2


def _np_ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def barabasi_albert(n, m=4, seed=0):
    """Barabasi-Albert graph as symmetric CSR (row_ptr int32[n+1], col int32[2*m*(n-m)]),
    built by the library's native generator."""
    L = _lib.load()
    e = L.abm_graph_ba_num_edges(int(n), int(m))
    if e < 0:
        raise ValueError(f"bad Barabasi-Albert size n={n}, m={m}")
    row_ptr = np.empty(int(n) + 1, dtype=np.int32)
    col = np.empty(int(e), dtype=np.int32)
    _lib.check(L.abm_graph_barabasi_albert(int(n), int(m), int(seed) & (2**64 - 1),
                                           _np_ptr(row_ptr), _np_ptr(col), int(e)),
               "abm_graph_barabasi_albert")
    return row_ptr, col


def random_regular(n, d=16, seed=0):
    """Simple d-regular graph as symmetric CSR (library's native generator)."""
    L = _lib.load()
    row_ptr = np.empty(int(n) + 1, dtype=np.int32)
    col = np.empty(int(n) * int(d), dtype=np.int32)
    _lib.check(L.abm_graph_random_regular(int(n), int(d), int(seed) & (2**64 - 1),
                                          _np_ptr(row_ptr), _np_ptr(col), col.size),
               "abm_graph_random_regular")
    return row_ptr, col


def initial_states(n, fraction=0.001, seed=0):
    """int8 compartments with ``max(1, int(fraction * n))`` infected agents chosen by a
    seeded permutation (``numpy.random.RandomState(seed).permutation(n)``)."""
    k = max(1, int(fraction * n))
    st = np.zeros(int(n), dtype=np.int8)
    st[np.random.RandomState(int(seed)).permutation(int(n))[:k]] = INFECTED
    return st


class SIRKernel(StepKernel):
    name = "sir"
    attributes = ("state",)
    metrics = ("S", "I", "R")
    params = {"beta": 0.05, "gamma": 0.1, "initial_infected": 0.001, "infection_seed": 0}

    def init(self, n, init_key, params, env):
        rp = env.get("network_row_ptr")
        if rp is None:
            raise ValueError("SIR agents need a Network with CSR adjacency (Network.from_csr)")
        if rp.numel() != n + 1:
            raise ValueError(f"network has {rp.numel() - 1} nodes for {n} agents")
        init = env.get("sir_initial_state")
        if init is None:
            init = initial_states(n, params["initial_infected"], params["infection_seed"])
        st = torch.as_tensor(np.asarray(init, dtype=np.int8)).to(_dev.device())
        return {"state": st.contiguous()}

    def run(self, states, coll_keys, params, env):
        coll_keys = coll_keys.reshape(-1, 2).contiguous()
        steps = coll_keys.shape[0]
        st = states["state"].contiguous()
        n = st.numel()
        rp, col = env["network_row_ptr"], env["network_col"]
        counts = torch.empty((steps, 3), dtype=torch.int32, device=st.device)
        e = col.numel()
        ws = _dev.workspace(_lib.load().abm_sir_run_workspace_bytes(n, e))
        _lib.call("abm_sir_run", _dev.ptr(rp), _dev.ptr(col), n, e, _dev.ptr(st),
                  _dev.ptr(coll_keys), steps, float(params["beta"]), float(params["gamma"]),
                  _dev.ptr(counts), _dev.ptr(ws), ws.numel(), _dev.stream_handle())
        return {"state": st}, counts

    def step(self, states, coll_key, params, env):
        states, counts = self.run(states, coll_key.reshape(1, 2), params, env)
        return states, counts[0]


class SIRAgent(Agent):
    """SIR agent on a Network (registered: runs on ``abm_sir_*``)."""

    def setup(self):
        return {"state": SUSCEPTIBLE}


register_step(SIRAgent, SIRKernel())


class SIRModel(Model):
    """SIR on a Barabasi-Albert network.

    Parameters: ``n`` (agents), ``m`` (BA attachment), ``beta``, ``gamma``,
    ``initial_infected`` (fraction), ``steps``, ``seed`` (model key, graph and initial
    infections), optional ``row_ptr``/``col`` (CSR) to skip graph generation."""

    def setup(self):
        n = int(self.p.get("n", 1 << 20))
        if "row_ptr" in self.p:
            rp, col = self.p["row_ptr"], self.p["col"]
        else:
            rp, col = barabasi_albert(n, int(self.p.get("m", 4)), int(self.p.get("graph_seed", self.seed)))
        self.network = Network(self)
        self.network.from_csr(rp, col)
        self.agents = self.add_agents(n, SIRAgent, name="people",
                                      beta=float(self.p.get("beta", 0.05)),
                                      gamma=float(self.p.get("gamma", 0.1)),
                                      initial_infected=float(self.p.get("initial_infected", 0.001)),
                                      infection_seed=int(self.p.get("infection_seed", self.seed)))

    def ensemble_member(self, graph_cache=None):
        """This model as one member of an SIR ensemble: ``(row_ptr, col, initial states,
        beta, gamma, seed, steps)`` built from its parameters exactly as ``setup`` and
        ``run`` would, or None when it cannot run batched (a subclass with Python hooks or
        its own ``setup``).  ``graph_cache`` shares generated graphs between members."""
        if self._hooks() != (None, None) or type(self).setup is not SIRModel.setup:
            return None
        p, seed = self.p, int(self.seed)
        n = int(p.get("n", 1 << 20))
        if "row_ptr" in p:
            g = (np.asarray(p["row_ptr"], np.int32), np.asarray(p["col"], np.int32))
        else:
            key = (n, int(p.get("m", 4)), int(p.get("graph_seed", seed)))
            if graph_cache is None:
                graph_cache = {}
            if key not in graph_cache:
                graph_cache[key] = barabasi_albert(*key)
            g = graph_cache[key]
        init = initial_states(n, float(p.get("initial_infected", 0.001)),
                              int(p.get("infection_seed", seed)))
        return (g[0], g[1], init, float(p.get("beta", 0.05)), float(p.get("gamma", 0.1)),
                seed, int(self.steps))


def run_ensemble(models):
    """Run SIR models as one batched launch sequence (``ensemble.SIRBatch``: every member and
    step in one CUDA-graph replay) and return one ``Results`` per model, each equal to that
    model's own ``run()`` (keys ``step``, ``S``, ``I``, ``R``, ``agents.people.state``).
    Members with different step counts run as one batch per step count.  Returns None
    unless every model is a batchable ``SIRModel`` (``ensemble_member``)."""
    from .agentpy import Results
    from .ensemble import SIRBatch
    cache, members = {}, []
    for m in models:
        spec = m.ensemble_member(cache) if isinstance(m, SIRModel) else None
        if spec is None:
            return None
        members.append(spec)
    out = [None] * len(members)
    by_steps = {}
    for k, spec in enumerate(members):
        by_steps.setdefault(spec[6], []).append(k)
    for steps, idx in by_steps.items():
        grp = [members[k] for k in idx]
        if steps == 0:
            for k, spec in zip(idx, grp):
                out[k] = Results({"agents.people.state": np.asarray(spec[2], np.int8).copy()})
            continue
        batch = SIRBatch([(s[0], s[1]) for s in grp], [s[2] for s in grp],
                         [s[3] for s in grp], [s[4] for s in grp], [s[5] for s in grp], steps)
        batch.run()
        counts = batch.counts.reshape(len(grp), steps, 3).cpu().numpy()
        for j, k in enumerate(idx):
            data = {"step": list(range(1, steps + 1)),
                    "S": counts[j, :, 0].tolist(), "I": counts[j, :, 1].tolist(),
                    "R": counts[j, :, 2].tolist(),
                    "agents.people.state": batch.final_state(j).cpu().numpy()}
            out[k] = Results(data)
    return out
