"""Batched SIR ensembles: many independent SIR models stepped by one launch sequence.

The reference runs ensembles as serial Python loops of ``model.run()``
(``Model.batch_run``, jaxabm/agentpy.py:1116-1152; ``SensitivityAnalysis.run``,
jaxabm/analysis.py:97-165).  Here every member is an *instance*: its CSR, per-agent words
and per-step counts live in packed device buffers, a device descriptor
(``abm_sir_instance``) points into them, and ``abm_sir_steps`` advances all live instances
over a persistent grid of (instance, 8192-agent tile) work items.  The whole multi-step
launch sequence is captured once in a CUDA graph and replayed.

Each instance follows exactly the single-model key chain (``PRNGKey(seed)`` ->
``initialize`` -> ``Model.step``), so its result is identical to running it alone.
"""

import math
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import torch

from . import _dev
from . import _lib
from . import random as jrandom
from .sir import barabasi_albert, initial_states
from .trace import nvtx_range

TILE = 8192  # agents per work item (abm_sir_tile_agents)

# numpy view of abm_sir_instance (include/jaxabm_gb300.h), 152 bytes
INSTANCE_DTYPE = np.dtype([
    ("row_ptr", "<u8"), ("adj", "<u8"), ("words", "<u8"), ("hub_counts", "<u8"),
    ("comp", "<u8"), ("counts", "<u8"), ("done_flag", "<u8"), ("coll_keys", "<u8"),
    ("rng", "<u4", (2,)),
    ("n", "<i4"), ("t", "<i4"), ("steps", "<i4"), ("beta", "<f4"), ("gamma", "<f4"),
    ("num_s", "<i4"), ("num_i", "<i4"), ("num_r", "<i4"), ("step_si", "<i4"),
    ("step_ir", "<i4"), ("edges_scanned", "<u8"), ("edges_pushed", "<u8"),
    ("candidates", "<u8"), ("coll", "<u4", (2,)), ("draws", "<u8"),
])
assert INSTANCE_DTYPE.itemsize == 152

# bits of the status word of the pack and resident entry points (ABM_SIR_STATUS_*)
STATUS_OVERSIZE = 1
STATUS_BAD_COMPARTMENT = 2
STATUS_BAD_COLUMN = 4


def raise_status(bits, where="SIR batch"):
    """Raise the error a status word reports (no-op for 0): ``AbmError`` with
    ABM_ERR_BADARG for an oversize instance or a compartment outside 0..2, ABM_ERR_BOUNDS
    for a CSR column outside its instance."""
    bits = int(bits)
    if not bits:
        return
    msgs = []
    if bits & STATUS_OVERSIZE:
        msgs.append("an instance has more agents than the resident call's max_agents")
    if bits & STATUS_BAD_COMPARTMENT:
        msgs.append("an initial compartment is outside 0..2 (S, I, R); it was run as R")
    if bits & STATUS_BAD_COLUMN:
        msgs.append("a CSR column points outside its instance; it was run as a self-loop")
    code = _lib.ABM_ERR_BOUNDS if bits == STATUS_BAD_COLUMN else _lib.ABM_ERR_BADARG
    raise _lib.AbmError(code, where, "; ".join(msgs))


WORDS = INSTANCE_DTYPE.itemsize // 4
RNG_WORD = INSTANCE_DTYPE.fields["rng"][1] // 4  # int32 column of rng[0]
STEPS_WORD = INSTANCE_DTYPE.fields["steps"][1] // 4  # int32 column of steps


def check_layout():
    size = _lib.load().abm_sir_instance_size()
    if size != INSTANCE_DTYPE.itemsize:
        raise RuntimeError(f"abm_sir_instance is {size} bytes, host layout expects "
                           f"{INSTANCE_DTYPE.itemsize}")
    tile = _lib.load().abm_sir_tile_agents()
    if tile != TILE:
        raise RuntimeError(f"SIR kernels take {tile}-agent tiles, host layout expects {TILE}")


def tiles_for(inst, n):
    b = np.arange(0, n, TILE, dtype=np.int64)
    out = np.zeros((b.size, 4), dtype=np.int32)
    out[:, 0] = inst
    out[:, 1] = b
    out[:, 2] = np.minimum(b + TILE, n)
    return out


def model_rngs(seeds):
    """Device rng after ``Model.initialize`` for each seed: split(PRNGKey(s), 2)[0]."""
    seeds = np.asarray(seeds, dtype=np.uint64)
    keys = np.zeros((seeds.size, 2), dtype=np.uint32)
    keys[:, 0] = (seeds >> np.uint64(32)).astype(np.uint32)
    keys[:, 1] = (seeds & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    dk = _dev.keys_from_numpy(keys)
    return jrandom.split(dk, 2)[:, 0].contiguous()


def changes_workspace(max_agents, max_tiles, device=None):
    """Zeroed list workspace of ``abm_sir_steps`` for ``max_agents`` live agents in at most
    ``max_tiles`` work items."""
    nbytes = _lib.load().abm_sir_changes_bytes(int(max_agents), int(max_tiles))
    return torch.zeros(max(nbytes, 32), dtype=torch.uint8, device=device or _dev.device())


def launch_struct(cfg):
    """Host ``abm_sir_launch`` for (sweep, candidates, push) grid sizes (None: defaults)."""
    if cfg is None:
        return None
    a = np.zeros(4, dtype=np.int32)
    a[:3] = [int(v) for v in cfg]
    return a


def default_launch():
    a = np.zeros(4, dtype=np.int32)
    _lib.call("abm_sir_default_launch", a.ctypes.data)
    return tuple(int(v) for v in a[:3])


def changes_overflowed(ws):
    return int(ws[4:8].view(torch.int32).item()) != 0


def word_bytes(n):
    """Bytes of an instance's word array: one per agent, padded to a multiple of 16."""
    return (int(n) + 15) // 16 * 16


def pack_words(state_i8, row_ptr, col, adj, words, hub_counts, comp, stream=None):
    """Per-agent words of one instance (compartment, hub mark, infected-neighbour count),
    the hub counts, the 2-bit compartments and the hub-tagged columns ``adj`` (may be
    ``col`` itself)."""
    n = state_i8.numel()
    scratch = torch.zeros(4, dtype=torch.int32, device=words.device)
    _lib.call("abm_sir_pack", _dev.ptr(state_i8), _dev.ptr(row_ptr), _dev.ptr(col), n,
              _dev.ptr(adj), _dev.ptr(words), _dev.ptr(hub_counts), _dev.ptr(comp),
              _dev.ptr(scratch), _dev.ptr(scratch[3:]), _dev.stream_handle(stream))
    return scratch


def unpack_words(words, n=None, stream=None):
    n = words.numel() if n is None else int(n)
    out = torch.empty(n, dtype=torch.int8, device=words.device)
    _lib.call("abm_sir_unpack", _dev.ptr(words), n, _dev.ptr(out), _dev.stream_handle(stream))
    return out


def chunk_ranges(nbytes, chunks):
    """Index ranges [a, b) covering 0..len(nbytes) in order, for copying and running a batch
    in ``chunks`` pieces: range c ends where the cumulative bytes first reach 2^(c+1-chunks)
    of the total (the first range ~1/2^(chunks-1) of the bytes, each next one doubling),
    every range holds at least one instance, and empty ranges are dropped."""
    nbytes = np.asarray(nbytes, dtype=np.float64)
    k = nbytes.size
    if k == 0:
        return []
    chunks = max(1, int(chunks))
    cum = np.cumsum(nbytes) / float(nbytes.sum())
    bounds, start = [], 0
    for c in range(chunks):
        if start >= k:
            break
        frac = 1.0 / (1 << (chunks - 1 - c))
        stop = min(k, max(start + 1, int(np.searchsorted(cum, frac - 1e-12)) + 1))
        bounds.append((start, stop))
        start = stop
    if start < k:
        bounds.append((start, k))
    return bounds


# Fixed cost of one step of a member on the resident path (its three barriers and the
# dependent loads of its phases), counted in list entries: per-member device times give
# ~10 us per active step against ~10 ns of CTA time per list entry, and replays of the
# 4,096-member ensemble are fastest with 4,096-16,384 here (65,536 puts large members too
# late and is slower than ordering by size).
STEP_COST_ENTRIES = 4096


def excess_degrees(row_ptrs):
    """<k^2>/<k> - 1 of each CSR graph: the mean number of further neighbours of an agent
    reached along an edge, the branching factor of a contagion on the graph."""
    out = np.zeros(len(row_ptrs), dtype=np.float64)
    for j, rp in enumerate(row_ptrs):
        deg = np.diff(np.asarray(rp, dtype=np.int64)).astype(np.float64)
        tot = deg.sum()
        out[j] = (deg * deg).sum() / tot - 1.0 if tot > 0 else 0.0
    return out


def predicted_costs(n, num_s, num_i, betas, gammas, k_exc, steps):
    """Predicted resident-path time of each member, in list entries, from a mean-field SIR
    recursion on its excess degree k: per step an S agent is infected with probability
    1 - (1 - beta i)^k and an infected one recovers with probability gamma; a member is
    active while its expected infected count is at least 1/2, and an active step costs
    ``STEP_COST_ENTRIES`` plus its expected list entries (infected agents and susceptible
    agents with an infected neighbour).  Used only to order the members (longest first),
    which never changes results: a long-lived epidemic on a small graph can take longer
    than a quick one on a large graph, and started last it would run alone at the end."""
    n = np.maximum(np.asarray(n, dtype=np.float64), 1.0)
    i = np.asarray(num_i, dtype=np.float64) / n
    s = np.asarray(num_s, dtype=np.float64) / n
    beta = np.asarray(betas, dtype=np.float64)
    gamma = np.asarray(gammas, dtype=np.float64)
    k = np.maximum(np.asarray(k_exc, dtype=np.float64), 0.0)
    cost = np.zeros_like(n)
    alive = np.ones(n.shape, dtype=bool)
    for _ in range(int(steps)):
        alive &= i * n >= 0.5
        if not alive.any():
            break
        cost += np.where(alive, STEP_COST_ENTRIES + n * (i + s * (1.0 - (1.0 - i) ** k)), 0.0)
        new_i = s * (1.0 - (1.0 - beta * i) ** k)
        new_r = gamma * i
        s = s - new_i
        i = i + new_i - new_r
    return cost


def member_costs(graphs, init_states, betas, gammas, steps):
    """:func:`predicted_costs` of SIR members given as host (row_ptr, col) graphs and int8
    compartments."""
    num_s = np.array([int((np.asarray(st) == 0).sum()) for st in init_states], dtype=np.int64)
    num_i = np.array([int((np.asarray(st) == 1).sum()) for st in init_states], dtype=np.int64)
    n = np.array([len(rp) - 1 for rp, _ in graphs], dtype=np.int64)
    return predicted_costs(n, num_s, num_i, betas, gammas,
                           excess_degrees([rp for rp, _ in graphs]), steps)


class SIRBatch:
    """A fixed set of SIR instances packed into device buffers.

    Args:
        graphs: list of (row_ptr, col) host CSR arrays
        init_states: list of int8 host compartment arrays
        betas, gammas: per-instance parameters
        seeds: per-instance model seeds (key chain of ``Model.initialize``/``step``)
        steps: number of steps every instance runs
        resident: run on the resident path (``abm_sir_steps_resident``: one CTA per
            instance at a time, all of its steps, words in shared memory) -- None picks it
            when every instance fits, False keeps the per-step grid kernels
            (``abm_sir_steps``), True requires it.  Both give identical results.
    """

    def __init__(self, graphs, init_states, betas, gammas, seeds, steps, resident=None):
        check_layout()
        dev = _dev.device()
        k = len(graphs)
        self.k = k
        self.steps = int(steps)
        self.n = np.array([len(rp) - 1 for rp, _ in graphs], dtype=np.int64)
        self.e = np.array([len(c) for _, c in graphs], dtype=np.int64)
        rp_off = np.concatenate([[0], np.cumsum(self.n + 1)])
        col_off = np.concatenate([[0], np.cumsum(self.e)])
        # word arrays (one byte per agent) start 16-byte aligned and are padded to 16 bytes
        w_off = np.concatenate([[0], np.cumsum((self.n + 15) // 16 * 16)])
        cnt_off = np.arange(k + 1, dtype=np.int64) * self.steps * 3
        h_rp = np.empty(rp_off[-1], dtype=np.int32)
        h_col = np.empty(col_off[-1], dtype=np.int32)
        h_st = np.zeros(w_off[-1], dtype=np.int8)
        for i, ((rp, col), st) in enumerate(zip(graphs, init_states)):
            h_rp[rp_off[i]:rp_off[i + 1]] = rp
            h_col[col_off[i]:col_off[i + 1]] = col
            h_st[w_off[i]:w_off[i] + self.n[i]] = st
        self.h_state0 = h_st
        self.row_ptr = torch.from_numpy(h_rp).to(dev)
        self.col = torch.from_numpy(h_col).to(dev)
        self.state8 = torch.from_numpy(h_st).to(dev)
        self.words = torch.empty(int(w_off[-1]), dtype=torch.uint8, device=dev)
        self.hub_counts = torch.zeros(int(w_off[-1]), dtype=torch.int32, device=dev)
        self.comp = torch.zeros(int(w_off[-1]) // 16, dtype=torch.int32, device=dev)
        self.counts = torch.zeros(int(cnt_off[-1]), dtype=torch.int32, device=dev)
        self._offsets = (rp_off, col_off, w_off, cnt_off)
        sizes = np.array([[int((st == c).sum()) for c in (0, 1, 2)] for st in init_states],
                         dtype=np.int32).reshape(k, 3)
        self.s0 = sizes[:, 0].astype(np.int64)
        desc = np.zeros(k, dtype=INSTANCE_DTYPE)
        desc["row_ptr"] = self.row_ptr.data_ptr() + 4 * rp_off[:-1]
        desc["adj"] = self.col.data_ptr() + 4 * col_off[:-1]
        desc["words"] = self.words.data_ptr() + w_off[:-1]
        desc["hub_counts"] = self.hub_counts.data_ptr() + 4 * w_off[:-1]
        desc["comp"] = self.comp.data_ptr() + w_off[:-1] // 4
        desc["counts"] = self.counts.data_ptr() + 4 * cnt_off[:-1]
        desc["n"] = self.n
        desc["steps"] = self.steps
        desc["beta"] = np.asarray(betas, dtype=np.float32)
        desc["gamma"] = np.asarray(gammas, dtype=np.float32)
        desc["num_s"], desc["num_i"], desc["num_r"] = sizes[:, 0], sizes[:, 1], sizes[:, 2]
        self.desc = torch.from_numpy(desc.view(np.int32).reshape(k, WORDS).copy()).to(dev)
        self.rng0 = model_rngs(seeds)
        self.desc[:, RNG_WORD:RNG_WORD + 2] = self.rng0
        self.desc0 = self.desc.clone()
        self.work = torch.from_numpy(
            np.concatenate([tiles_for(i, int(n)) for i, n in enumerate(self.n)])).to(dev)
        self._status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.pack()
        bad = int(self._status.item())
        if bad & STATUS_BAD_COMPARTMENT:
            raise ValueError("initial compartments must be 0 (S), 1 (I) or 2 (R)")
        if bad & STATUS_BAD_COLUMN:
            raise ValueError("a CSR column points outside its instance (0..n-1)")
        self.words0 = self.words.clone()
        self.hub_counts0 = self.hub_counts.clone()
        self.comp0 = self.comp.clone()
        self.changes = None  # list workspace of the grid path, allocated on first use
        self.launch_cfg = None  # (sweep, candidates, push) grid sizes; None = defaults
        self._graph = None
        self._graph_states = None
        self._graph_steps = None
        self._from_states = False  # the next resident run builds its words from state8
        self._words0_stale = False  # inputs were loaded after the step-0 words were saved
        # resident path: instances longest first by predicted time (mean-field cost model),
        # one change list per resident CTA
        L = _lib.load()
        self.max_n = int(self.n.max())
        self.cost = predicted_costs(self.n, sizes[:, 0], sizes[:, 1], betas, gammas,
                                    excess_degrees([rp for rp, _ in graphs]), self.steps)
        self.order = torch.from_numpy(np.argsort(-self.cost, kind="stable").astype(np.int32)).to(dev)
        self.res_grid = int(L.abm_sir_resident_grid(self.max_n)) if resident is not False else 0
        self.resident_ok = self.res_grid > 0
        if resident and not self.resident_ok:
            raise ValueError(f"an instance of {self.max_n} agents does not fit the resident path "
                             f"(at most {L.abm_sir_resident_max_agents()})")
        if self.resident_ok:
            self.res_scratch = torch.empty(L.abm_sir_resident_scratch_bytes(self.max_n,
                                                                            self.res_grid),
                                           dtype=torch.uint8, device=dev)
            self.res_status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.mode = "resident" if self.resident_ok else "grid"
        if self.mode == "grid":
            self._ensure_changes()

    def _ensure_changes(self):
        """The grid path's list workspace (16 bytes per agent: change and candidate lists),
        allocated when the batch first takes that path (before any graph capture)."""
        if self.changes is None:
            if torch.cuda.is_current_stream_capturing():
                raise RuntimeError("select the grid path before capturing a graph")
            self.changes = changes_workspace(int(self.n.sum()), self.work.shape[0])

    def set_mode(self, mode):
        """``"resident"`` or ``"grid"`` (drops the captured graph)."""
        if mode not in ("resident", "grid"):
            raise ValueError(f"unknown SIR batch mode {mode!r}")
        if mode == "resident" and not self.resident_ok:
            raise ValueError("this batch cannot run on the resident path")
        if mode == "grid" and self.mode != "grid":
            # the grid kernels need their list workspace, packed words and hub-tagged columns
            self._ensure_changes()
            self.pack()
            self.words0.copy_(self.words)
            self.hub_counts0.copy_(self.hub_counts)
            self.comp0.copy_(self.comp)
            self._words0_stale = False
        self.mode = mode
        self._graph = None
        self._graph_states = None

    def pack(self, stream=None):
        """Words, hub counts and 2-bit compartments of every instance from the int8
        compartments in ``state8``; tags the hub entries of ``col`` in place (three
        launches)."""
        _lib.call("abm_sir_pack_batch", _dev.ptr(self.desc), _dev.ptr(self.work),
                  self.work.shape[0], _dev.ptr(self.state8), _dev.ptr(self.words),
                  _dev.ptr(self._status), _dev.stream_handle(stream))

    def load_host(self, h_row_ptr, h_col, h_state8, stream=None):
        """Inputs from (pinned) host buffers laid out like ``row_ptr``/``col``/``state8``:
        copy them in and rewind every instance to step 0.  The instances keep their sizes
        and the S/I/R totals given at construction, so the loaded compartments must have the
        same totals per instance (other agents may be infected).  The grid path rebuilds the
        words, hub counts and column tags here; the resident kernel builds each instance's
        words itself at step 0."""
        self.row_ptr.copy_(h_row_ptr, non_blocking=True)
        self.col.copy_(h_col, non_blocking=True)
        self.state8.copy_(h_state8, non_blocking=True)
        self.rewind_loaded(stream)

    def rewind_loaded(self, stream=None):
        """After new inputs were copied into ``row_ptr``/``col``/``state8``: rebuild what the
        path needs (the grid path packs here; the resident kernel builds the words itself
        at step 0) and rewind every instance to step 0."""
        if self.mode != "resident":
            self.pack(stream)
        self._from_states = self.mode == "resident"
        self._words0_stale = True  # the saved step-0 words belong to the earlier inputs
        self.desc.copy_(self.desc0, non_blocking=True)

    def _chunk_plan(self, chunks):
        """Index ranges of the overlapped host run (a small first range, so the kernels
        start early, then ranges of growing byte counts), each with its own order (longest
        predicted time first), resident grid, scratch and stream."""
        if getattr(self, "_chunks", None) is not None:
            if self._chunks[0] == chunks:
                return self._chunks[1]
            # the old plan's scratch may still be in use on its streams: finish them before
            # it is released to the allocator
            torch.cuda.synchronize()
            self._chunks = None
        L = _lib.load()
        dev = self.row_ptr.device
        bounds = chunk_ranges(4 * (self.n + 1) + 4 * self.e + self.n, chunks)
        order = np.concatenate([a + np.argsort(-self.cost[a:b], kind="stable")
                                for a, b in bounds]).astype(np.int32)
        d_order = torch.from_numpy(order).to(dev)
        plan = []
        for a, b in bounds:
            max_n = int(self.n[a:b].max())
            grid = min(self.res_grid, b - a)
            scratch = torch.empty(L.abm_sir_resident_scratch_bytes(max_n, grid),
                                  dtype=torch.uint8, device=dev)
            plan.append({"range": (a, b), "max_n": max_n, "grid": grid, "scratch": scratch,
                         "stream": torch.cuda.Stream(), "event": torch.cuda.Event()})
        self._chunks = (chunks, (plan, d_order, torch.cuda.Stream()))
        return self._chunks[1]

    def run_from_host(self, h_row_ptr, h_col, h_state8, h_counts=None, chunks=8):
        """Every step of every instance from page-locked host inputs (laid out like
        ``row_ptr``/``col``/``state8``), with the host-to-device copies overlapping the
        kernels (resident path).  The instances are split into ``chunks`` index ranges --
        the first small, so that kernels start after a few percent of the bytes -- and each
        range runs as its own resident launch on its own stream as soon as its copies have
        landed, while the later ranges are still being copied; with ``h_counts`` (page-
        locked, laid out like ``counts``) each range's counts are copied back as soon as it
        finishes.  Launches of different ranges share the GPU, so order the instances
        longest first (:func:`member_costs`) for the shortest run.  Returns after enqueueing; the results equal
        :meth:`load_host` followed by :meth:`run`."""
        if self.mode != "resident":
            raise ValueError("run_from_host needs the resident path")
        with nvtx_range("SIRBatch.run_from_host"):
            self._run_from_host(h_row_ptr, h_col, h_state8, h_counts, int(chunks))

    def _run_from_host(self, h_row_ptr, h_col, h_state8, h_counts, chunks):
        plan, d_order, copy = self._chunk_plan(chunks)
        rp_off, col_off, w_off, cnt_off = self._offsets
        cur = torch.cuda.current_stream()
        self.res_status.zero_()
        copy.wait_stream(cur)
        with torch.cuda.stream(copy):
            self.desc.copy_(self.desc0, non_blocking=True)
            for c in plan:
                a, b = c["range"]
                self.row_ptr[rp_off[a]:rp_off[b]].copy_(h_row_ptr[rp_off[a]:rp_off[b]],
                                                        non_blocking=True)
                self.col[col_off[a]:col_off[b]].copy_(h_col[col_off[a]:col_off[b]],
                                                      non_blocking=True)
                self.state8[w_off[a]:w_off[b]].copy_(h_state8[w_off[a]:w_off[b]],
                                                     non_blocking=True)
                c["event"].record(copy)
        for c in plan:
            a, b = c["range"]
            s = c["stream"]
            s.wait_event(c["event"])
            _lib.call("abm_sir_steps_resident", _dev.ptr(self.desc), b - a,
                      _dev.ptr(d_order) + 4 * a, c["max_n"], self.steps, c["grid"],
                      _dev.ptr(self.state8), _dev.ptr(self.words), _dev.ptr(c["scratch"]),
                      c["scratch"].numel(), _dev.ptr(self.res_status), s.cuda_stream)
            if h_counts is not None:
                with torch.cuda.stream(s):
                    h_counts[cnt_off[a]:cnt_off[b]].copy_(self.counts[cnt_off[a]:cnt_off[b]],
                                                          non_blocking=True)
        for c in plan:
            cur.wait_stream(c["stream"])
        cur.wait_stream(copy)
        self._from_states = False
        self._words0_stale = True  # the saved step-0 words belong to the earlier inputs

    @property
    def agent_steps(self):
        return int(self.n.sum()) * self.steps

    def reset(self):
        """Back to step 0 (words, counters, key chains) without reallocating: the packed
        words of step 0 are copied back (device to device), so the next run starts from
        them.  After :meth:`load_host` brought other inputs, the words of step 0 are
        rebuilt from them instead (the grid path packs again; the resident kernel builds
        them at step 0).  The status words are cleared, except what a pack of the loaded
        inputs reports about them."""
        if self.resident_ok:
            self.res_status.zero_()
        if self._words0_stale:
            self.desc.copy_(self.desc0)
            if self.mode == "resident":
                self._from_states = True
                return
            self.pack()
            self.words0.copy_(self.words)
            self.hub_counts0.copy_(self.hub_counts)
            self.comp0.copy_(self.comp)
            self._words0_stale = False
            self._from_states = False
            return
        self.words.copy_(self.words0)
        self.hub_counts.copy_(self.hub_counts0)
        self.comp.copy_(self.comp0)
        self.desc.copy_(self.desc0)
        self._from_states = False

    def launch(self, nsteps, stream=None, from_states=None):
        """Enqueue ``nsteps`` steps of every live instance (C ABI ``abm_sir_steps_resident``
        or ``abm_sir_steps``).  On the resident path, ``from_states`` (default: after
        :meth:`load_host`) has the kernel build the words of instances at step 0 from
        ``state8`` instead of reading the packed words."""
        if self.mode == "resident":
            if from_states is None:
                from_states = self._from_states
                self._from_states = False
            st = _dev.ptr(self.state8) if from_states else None
            wb = _dev.ptr(self.words) if from_states else None
            _lib.call("abm_sir_steps_resident", _dev.ptr(self.desc), self.k, _dev.ptr(self.order),
                      self.max_n, int(nsteps), self.res_grid, st, wb, _dev.ptr(self.res_scratch),
                      self.res_scratch.numel(), _dev.ptr(self.res_status),
                      _dev.stream_handle(stream))
            return
        self._ensure_changes()
        _lib.call("abm_sir_steps", _dev.ptr(self.desc), self.k, _dev.ptr(self.work),
                  self.work.shape[0], None, int(nsteps), self._launch_ptr(), _dev.ptr(self.changes),
                  self.changes.numel(), _dev.stream_handle(stream))

    def _launch_ptr(self):
        self._launch_buf = launch_struct(self.launch_cfg)  # kept alive for the call
        return None if self._launch_buf is None else self._launch_buf.ctypes.data

    def set_launch(self, cfg):
        """Use grid sizes ``cfg`` = (sweep, candidates, push); drops the captured graph."""
        self.launch_cfg = None if cfg is None else tuple(int(v) for v in cfg)
        self._graph = None
        self._graph_states = None

    def capture(self, nsteps):
        """Capture ``nsteps`` steps into a CUDA graph (replayed by :meth:`replay`); on the
        resident path a second graph builds the words from ``state8`` (used after
        :meth:`load_host`)."""
        def one(from_states):
            torch.cuda.synchronize()
            s = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())
            g = torch.cuda.CUDAGraph()
            with torch.cuda.stream(s):
                with torch.cuda.graph(g, stream=s):
                    self.launch(nsteps, s, from_states=from_states)
            torch.cuda.current_stream().wait_stream(s)
            torch.cuda.synchronize()
            return g
        self._graph = one(False)
        self._graph_states = one(True) if self.mode == "resident" else None
        self._graph_steps = nsteps
        return self._graph

    def replay(self):
        with nvtx_range("SIRBatch.replay"):
            if self._from_states and self._graph_states is not None:
                self._graph_states.replay()
                self._from_states = False
            else:
                self._graph.replay()

    def run(self, use_graph=True, check=True):
        """All ``steps`` steps of every instance; with ``check`` (default) waits for them
        and raises on bad inputs (:meth:`check`)."""
        if use_graph:
            if self._graph is None or self._graph_steps != self.steps:
                self.capture(self.steps)
            self.replay()
        else:
            self.launch(self.steps)
        if check:
            self.check()

    def status(self):
        """Status bits (``STATUS_*``) the inputs and runs since the last :meth:`reset`
        raised (synchronises with the device)."""
        bits = int(self._status.item())
        if self.resident_ok:
            bits |= int(self.res_status.item())
        return bits

    def check(self):
        """Raise if a list overflowed or an input was bad (oversize instance, compartment
        outside 0..2, CSR column outside its instance); each kind has its own message."""
        if self.changes is not None and changes_overflowed(self.changes):
            raise RuntimeError("SIR change list overflowed (workspace smaller than live agents)")
        raise_status(self.status())

    def final_state(self, i):
        w_off = self._offsets[2]
        return unpack_words(self.words[w_off[i]:w_off[i] + int(self.n[i])])

    def counts_of(self, i):
        c = self._offsets[3]
        return self.counts[c[i]:c[i + 1]].reshape(self.steps, 3)

    def launches_per_run(self):
        if self.mode == "resident":
            return 1  # one launch for every step of every instance
        # prepare, then per step sweep, candidates, push and (more than 256 instances)
        # finalize, and a work-list compaction every 8 steps
        per_step = 3 if self.k <= 256 else 4
        return per_step * self.steps + 1 + (self.steps + 7) // 8

    def edge_stats(self):
        """(CSR slots read by decide, CSR slots read by push, compartment changes,
        decision candidates) since the last reset, summed over instances."""
        d = self.desc.cpu().numpy().view(INSTANCE_DTYPE).reshape(-1)
        changes = int((d["num_i"] + 2 * d["num_r"]).sum() - (self.h_state0 == 1).sum()
                      - 2 * (self.h_state0 == 2).sum())
        return (int(d["edges_scanned"].sum()), int(d["edges_pushed"].sum()), changes,
                int(d["candidates"].sum()))

    def threefry_blocks(self):
        """Threefry2x32-20 blocks the completed run evaluated, from its counters:
        2 per susceptible decision (the infection key split(split(coll_key, i)[0])), 1 per
        infection draw, 3 per recovery decision (key and draw), 3 per instance-step for the
        key chain (step key, collection key, next rng).  Recovery decisions are the
        infected agents at the start of every step, read from the counts."""
        d = self.desc.cpu().numpy().view(INSTANCE_DTYPE).reshape(-1)
        counts = self.counts.reshape(self.k, self.steps, 3).cpu().numpy().astype(np.int64)
        i0 = np.array([(self.h_state0[o:o + n] == 1).sum() for o, n in
                       zip(self._offsets[2][:-1], self.n)], dtype=np.int64)
        i_before = np.concatenate([i0[:, None], counts[:, :-1, 1]], axis=1)
        rec = int(i_before.sum())
        sus = int(d["candidates"].sum()) - rec
        blocks = 2 * sus + int(d["draws"].sum()) + 3 * rec + 3 * int(d["t"].sum())
        return {"blocks": blocks, "susceptible_decisions": sus, "recovery_decisions": rec,
                "infection_draws": int(d["draws"].sum())}

    def live_agent_steps(self):
        """Agent-steps whose words the sweep reads: steps of an instance that start with at
        least one infected agent (the others cannot change and are skipped)."""
        counts = self.counts.reshape(self.k, self.steps, 3).cpu().numpy().astype(np.int64)
        i0 = np.array([(self.h_state0[o:o + n] == 1).sum() for o, n in
                       zip(self._offsets[2][:-1], self.n)], dtype=np.int64)
        i_before = np.concatenate([i0[:, None], counts[:, :-1, 1]], axis=1)
        return int(((i_before > 0).sum(axis=1) * self.n).sum())

    def algorithmic_bytes_resident(self):
        """HBM bytes the resident path must move (after the run completed): each instance's
        words read and written once and its 2-bit copy written (2.25 B per agent); per
        decision a 4-byte list entry written and read and 8 bytes of row offsets (an
        infected agent reads none, so this over-counts); per CSR slot read by a decision
        or pushed its 4-byte column (neighbour states and counts live in shared memory);
        per change a 4-byte entry written and read and 8 bytes of row offsets; S/I/R counts
        12 B per instance and step."""
        scanned, pushed, changes, cands = self.edge_stats()
        words = int(((self.n + 15) // 16 * 16).sum())
        return int(2.25 * words + 16 * cands + 4 * scanned + 16 * changes + 4 * pushed
                   + 12 * self.k * self.steps)

    def algorithmic_bytes(self):
        """Bytes the run must move (after it completed), each datum at its own size: per
        live agent-step its 1-byte word; per decision candidate 8 bytes (a susceptible
        candidate's row offsets; an infected one reads nothing more, so this over-counts);
        per CSR slot read by a decision 5 bytes (4-byte column + neighbour word); per slot
        pushed 6 bytes (column + count read and write); per compartment change 26 bytes
        (8-byte list entry written and read, 8-byte row offsets, own word read and
        write)."""
        scanned, pushed, changes, cands = self.edge_stats()
        return int(self.live_agent_steps() + 8 * cands + 5 * scanned + 6 * pushed
                   + 26 * changes)


# ---- the batched-ensemble workload (4,096 SIR instances) -------------------------------

def ensemble_spec(count=4096, n_lo=1_000, n_hi=100_000, seed=2, rate=200.0):
    """Per-instance sizes, parameters, seeds and Poisson arrival times.

    Sizes are log-uniform in [n_lo, n_hi] (``RandomState(seed)``); (beta, gamma) come from a
    scrambled 2-D Sobol sequence seeded with ``seed``, scaled to [0.01, 0.2] x [0.05, 0.3];
    arrivals are a Poisson stream of ``rate`` requests/s (exponential gaps,
    ``RandomState(seed + 1)``)."""
    from scipy.stats import qmc
    rs = np.random.RandomState(seed)
    n = np.rint(np.exp(rs.uniform(math.log(n_lo), math.log(n_hi), size=count))).astype(np.int64)
    try:
        sob = qmc.Sobol(d=2, scramble=True, rng=np.random.default_rng(seed))
    except TypeError:  # older SciPy spells the argument `seed`
        sob = qmc.Sobol(d=2, scramble=True, seed=seed)
    u = sob.random(count)
    beta = (0.01 + 0.19 * u[:, 0]).astype(np.float32)
    gamma = (0.05 + 0.25 * u[:, 1]).astype(np.float32)
    gaps = np.random.RandomState(seed + 1).exponential(1.0 / rate, size=count)
    arrivals = np.cumsum(gaps) - gaps[0]
    seeds = np.arange(count, dtype=np.int64)
    return {"n": n, "beta": beta, "gamma": gamma, "arrival_s": arrivals, "seed": seeds}


def partition_members(sizes, world):
    """Member indices of each of ``world`` ranks: the members split so that every member
    belongs to exactly one rank and the ranks' agent totals are balanced (largest member
    first, each to the rank with the fewest agents so far; ties to the lower rank).  Each
    rank's list is in ascending member order."""
    sizes = np.asarray(sizes, dtype=np.int64)
    world = int(world)
    if world < 1:
        raise ValueError("world must be at least 1")
    load = np.zeros(world, dtype=np.int64)
    owner = np.empty(sizes.size, dtype=np.int64)
    for i in np.argsort(-sizes, kind="stable"):
        r = int(np.argmin(load))
        owner[i] = r
        load[r] += sizes[i]
    return [np.flatnonzero(owner == r) for r in range(world)]


def rank_spec(count=4096, rank=0, world=1):
    """This rank's share of the first ``count`` members of the ensemble specification in a
    ``world``-rank run: the members are partitioned across the ranks, balanced by agents
    (:func:`partition_members`), so every member runs on exactly one GPU and the ranks need
    no collective.  Adds ``member``, the members' indices in the full specification."""
    spec = ensemble_spec(4096 if count <= 4096 else count)
    spec = {k: v[:count].copy() for k, v in spec.items()}
    mine = partition_members(spec["n"], world)[int(rank)]
    out = {k: v[mine].copy() for k, v in spec.items()}
    out["member"] = mine
    return out


def build_instances(spec, m=4, initial_infected=0.001, workers=None):
    """Host CSR graphs and initial compartments of every instance (native generator,
    threads across instances)."""
    def one(i):
        n = int(spec["n"][i])
        s = int(spec["seed"][i])
        g = barabasi_albert(n, m, s)
        return g, initial_states(n, initial_infected, s)
    with ThreadPoolExecutor(max_workers=workers) as ex:
        res = list(ex.map(one, range(len(spec["n"]))))
    return [r[0] for r in res], [r[1] for r in res]
