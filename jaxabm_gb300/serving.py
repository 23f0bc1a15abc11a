"""Continuous-batching server for SIR simulation requests.

Requests (a network, initial compartments, beta, gamma, seed, steps) arrive over time.
The server keeps every admitted request resident on the device as one instance of the
batched SIR step (``abm_sir_steps_resident``, or ``abm_sir_steps`` on the grid path) and
advances all of them together, ``steps_per_tick`` steps per tick:

* admission: a request is admitted when a descriptor slot is free, its tiles fit the work
  list, and its buffers fit the free device memory (``torch.cuda.mem_get_info``) minus a
  reserve; otherwise it waits in the queue (first come, first served).  Everything that
  fits at a tick is admitted as one group (one allocation per buffer kind, one pack
  launch);
* every tick replays ONE captured CUDA graph over a fixed-capacity work list; admitting or
  retiring requests only rewrites device tables (descriptor rows, work items), so the graph
  is never re-captured.  It is captured, and replayed once over the empty tables, when
  the server is constructed, so the first request does not wait for that set-up;
* completion: the finalize kernel raises the request's done flag in pinned host memory
  after its last step; the host sees it without synchronising, enqueues the copy of the
  per-step counts and frees the slot.

Every request's draws depend only on its own key chain, so its result is identical alone
and in any mix.
"""

import collections
import time

import numpy as np
import torch

from . import _dev
from . import _lib
from .trace import nvtx_range
from .ensemble import (INSTANCE_DTYPE, RNG_WORD, STATUS_BAD_COLUMN, STATUS_BAD_COMPARTMENT,
                       STEPS_WORD, TILE, changes_overflowed, changes_workspace, check_layout,
                       launch_struct, model_rngs, raise_status, unpack_words, word_bytes)


def work_table(slots, sizes, dummy, capacity, tile=TILE):
    """Work items (slot, begin, end, 0) of the requests at ``slots`` with ``sizes`` agents,
    ``tile`` agents each, in the given order, padded to ``capacity`` rows with the inactive
    row ``dummy``: returns (int32[capacity, 4], number of items)."""
    slots = np.asarray(slots, dtype=np.int64)
    sizes = np.asarray(sizes, dtype=np.int64)
    tiles = (sizes + tile - 1) // tile
    k = int(tiles.sum())
    if k > capacity:
        raise ValueError(f"{k} work items exceed the capacity {capacity}")
    out = np.zeros((capacity, 4), dtype=np.int32)
    out[:, 0] = dummy
    if k:
        owner = np.repeat(np.arange(slots.size), tiles)
        first = np.repeat(np.cumsum(tiles) - tiles, tiles)
        begin = (np.arange(k) - first) * tile
        out[:k, 0] = slots[owner]
        out[:k, 1] = begin
        out[:k, 2] = np.minimum(begin + tile, sizes[owner])
    return out, k


def order_table(slots, sizes, total):
    """Every descriptor row 0..total-1 once: the given slots first, largest request first
    (ties in the given order), then the other rows in index order."""
    slots = np.asarray(slots, dtype=np.int64)
    sizes = np.asarray(sizes, dtype=np.int64)
    live = slots[np.argsort(-sizes, kind="stable")]
    rest = np.ones(int(total), dtype=bool)
    rest[slots] = False
    return np.concatenate([live, np.nonzero(rest)[0]]).astype(np.int32)


class _Group:
    """Device buffers shared by the requests admitted together; every request of the group
    holds it, so the buffers are freed once the last of them has retired.  ``h_status`` is
    a pinned copy of the group's pack status (bad compartments or columns), written on the
    server stream right after the pack; ``h_counts`` is the group's pinned result buffer
    (every request's per-step counts at its offset)."""
    __slots__ = ("bufs", "h_status", "h_counts")

    def __init__(self, bufs, h_status, h_counts):
        self.bufs = bufs
        self.h_status = h_status
        self.h_counts = h_counts


def _host_span(a, dtype):
    """(array, address, bytes) of host array ``a`` as a contiguous ``dtype`` array: ``a``
    itself when it already is one (numpy or CPU tensor), else a converted copy, which the
    caller keeps alive until the copies that read it were issued."""
    if isinstance(a, torch.Tensor):
        if a.is_cuda:
            raise ValueError("request arrays must be host arrays")
        want = {np.int32: torch.int32, np.int8: torch.int8}[dtype]
        if a.dtype != want or not a.is_contiguous():
            a = a.to(want).contiguous()
        return a, a.data_ptr(), a.numel() * a.element_size()
    a = np.ascontiguousarray(a, dtype=dtype)
    return a, a.ctypes.data, a.nbytes


def copy_segments(dst, src, nbytes, to_device, stream, pinned=False):
    """Many copies in one call (address lists as numpy uint64).  With ``pinned`` (every
    host side is page-locked) one ``abm_copy_segments_kernel`` launch does them all from a
    page-locked segment table, which is returned and must stay alive until the stream has
    run the copy; otherwise ``abm_copy_segments`` issues one copy call per segment (None is
    returned)."""
    dst = np.ascontiguousarray(dst, dtype=np.uint64).reshape(-1)
    src = np.ascontiguousarray(src, dtype=np.uint64).reshape(-1)
    nbytes = np.ascontiguousarray(nbytes, dtype=np.uint64).reshape(-1)
    if pinned and dst.size:
        table = torch.empty((dst.size, 3), dtype=torch.int64, pin_memory=True)
        t = table.numpy().view(np.uint64)
        t[:, 0], t[:, 1], t[:, 2] = dst, src, nbytes
        st = _lib.load().abm_copy_segments_kernel(table.data_ptr(), dst.size, stream.cuda_stream)
        if st == _lib.ABM_OK:
            return table
        if st != _lib.ABM_ERR_BADARG:  # BADARG: memory the kernel may not touch; copy below
            _lib.check(st, "abm_copy_segments_kernel")
    _lib.call("abm_copy_segments", dst.size, dst.ctypes.data, src.ctypes.data, nbytes.ctypes.data,
              1 if to_device else 0, stream.cuda_stream)
    return None


def input_error(req):
    """The error of a request whose inputs the pack flagged (compartment outside 0..2 or a
    CSR column outside 0..n-1), found on the host for that request alone; None if its own
    inputs are fine (another request of its admission group was flagged)."""
    st = np.asarray(req.state, dtype=np.int8)
    col = np.asarray(req.col, dtype=np.int64)
    bits = 0
    if st.size and (st.min() < 0 or st.max() > 2):
        bits |= STATUS_BAD_COMPARTMENT
    if col.size and (col.min() < 0 or col.max() >= req.n):
        bits |= STATUS_BAD_COLUMN
    if not bits:
        return None
    try:
        raise_status(bits, f"request {req.rid}")
    except _lib.AbmError as err:
        return err


class Request:
    """One simulation request: a CSR network (``row_ptr`` int32[n+1], ``col`` int32[E]),
    initial int8 compartments ``state``, parameters, model seed and steps.  Arrays are host
    arrays (numpy or CPU tensors; page-locked tensors copy asynchronously, and a request
    whose three arrays are page-locked is copied by the server's gather kernel), int32 /
    int8 and contiguous; their contents must stay unchanged until the request is admitted
    (their addresses are taken when the request is made or an array is replaced)."""
    __slots__ = ("rid", "_row_ptr", "_col", "_state", "beta", "gamma", "seed", "steps",
                 "arrival", "admitted", "finished", "_counts", "final_state", "_slot",
                 "_bufs", "_event", "keep_state", "error", "_n", "_e", "cancelled", "_spans",
                 "_pinned")

    def __init__(self, rid, row_ptr, col, state, beta, gamma, seed, steps, arrival=None,
                 keep_state=False):
        self.rid = rid
        self._row_ptr, self._col, self._state = row_ptr, col, state
        self._refresh()
        self.beta, self.gamma, self.seed, self.steps = float(beta), float(gamma), int(seed), int(steps)
        self.arrival = arrival
        self.admitted = None
        self.finished = None
        self._counts = None  # (page-locked result buffer, offset) once retired
        self.final_state = None
        self.keep_state = keep_state
        self.error = None  # AbmError when the request's inputs were bad (set at harvest)
        self.cancelled = False
        self._slot = None
        self._bufs = None
        self._event = None

    def _refresh(self):
        """Sizes, and the (array, address, bytes) of each input (a converted copy when the
        given array is not a contiguous int32 / int8 one) with whether all three are
        page-locked; redone whenever an input array is replaced."""
        self._n = len(self._row_ptr) - 1
        self._e = len(self._col)
        self._spans = (_host_span(self._row_ptr, np.int32), _host_span(self._col, np.int32),
                       _host_span(self._state, np.int8))
        self._pinned = all(isinstance(a[0], torch.Tensor) and a[0].is_pinned()
                           for a in self._spans)

    @property
    def row_ptr(self):
        return self._row_ptr

    @row_ptr.setter
    def row_ptr(self, v):
        self._row_ptr = v
        self._refresh()

    @property
    def col(self):
        return self._col

    @col.setter
    def col(self, v):
        self._col = v
        self._refresh()

    @property
    def state(self):
        return self._state

    @state.setter
    def state(self, v):
        self._state = v
        self._refresh()

    @property
    def n(self):
        return self._n

    @property
    def counts(self):
        """Per-step S/I/R counts int32[steps, 3] (a view into the admission group's
        page-locked result buffer), or None before the request has retired."""
        c = self._counts
        if c is None or isinstance(c, torch.Tensor):
            return c
        buf, c0 = c
        self._counts = buf[c0:c0 + 3 * self.steps].view(self.steps, 3)
        return self._counts

    def device_bytes(self):
        n, e = self._n, self._e
        # CSR; int8 compartments, word bytes, hub counts and 2-bit compartments (each padded
        # to 16 agents); per-step counts
        return 4 * (n + 1) + 4 * e + 6 * word_bytes(n) + word_bytes(n) // 4 + 12 * self.steps

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.arrival


class SIRServer:
    """Continuous-batching SIR server on the current CUDA device.

    Args:
        max_slots: concurrently resident requests
        max_tiles: capacity of the work list (8192-agent tiles of resident requests)
        steps_per_tick: steps every resident request advances per tick
        reserve_bytes: device memory kept free at admission
        grid: (sweep, candidates, push) persistent grid sizes, or None for the defaults
        path: ``"grid"`` (the per-step kernels over the work list: every step of a request
            is spread over the whole GPU, so ticks are short and latency low), ``"resident"``
            (one CTA per request for all steps of a tick: highest throughput when many
            requests are resident, longer ticks for large requests) or ``"auto"`` (resident
            when it can hold ``max_request_agents``)
        max_request_agents: largest request the resident path accepts (larger requests are
            rejected at submission on that path)
    """

    def __init__(self, max_slots=512, max_tiles=65536, steps_per_tick=16,
                 reserve_bytes=1 << 30, grid=None, path="grid", max_request_agents=100_000):
        check_layout()
        dev = _dev.device()
        if path not in ("auto", "resident", "grid"):
            raise ValueError(f"unknown server path {path!r}")
        L = _lib.load()
        self.max_request_agents = int(max_request_agents)
        self.res_grid = (int(L.abm_sir_resident_grid(self.max_request_agents))
                         if path != "grid" else 0)
        if path == "resident" and self.res_grid <= 0:
            raise ValueError(f"the resident path cannot hold requests of "
                             f"{self.max_request_agents} agents")
        self.resident = self.res_grid > 0
        if self.resident:
            self.res_scratch = torch.empty(
                L.abm_sir_resident_scratch_bytes(self.max_request_agents, self.res_grid),
                dtype=torch.uint8, device=dev)
            self.res_status = torch.zeros(1, dtype=torch.int32, device=dev)
            # instances in the order the resident CTAs take them: live requests largest first
            self.order = torch.arange(int(max_slots) + 1, dtype=torch.int32, device=dev)
            self.h_order = torch.arange(int(max_slots) + 1, dtype=torch.int32).pin_memory()
        self.max_slots = int(max_slots)
        self.max_tiles = int(max_tiles)
        self.steps_per_tick = int(steps_per_tick)
        self.reserve = int(reserve_bytes)
        self.grid = None if grid is None else tuple(int(v) for v in grid)
        words = INSTANCE_DTYPE.itemsize // 4
        self.dummy = self.max_slots  # inactive descriptor row (t = steps = 0)
        self.desc = torch.zeros((self.max_slots + 1, words), dtype=torch.int32, device=dev)
        self.h_desc = torch.zeros((self.max_slots + 1, words), dtype=torch.int32).pin_memory()
        self.h_work = torch.zeros((self.max_tiles, 4), dtype=torch.int32).pin_memory()
        self.h_work[:, 0] = self.dummy
        self.work = torch.zeros((self.max_tiles, 4), dtype=torch.int32, device=dev)
        self.work.copy_(self.h_work)
        self.changes = changes_workspace(self.max_tiles * TILE, self.max_tiles)
        # number of live work items, read by the kernels on every replay
        self.live = torch.zeros(1, dtype=torch.int32, device=dev)
        self.h_live = torch.zeros(1, dtype=torch.int32).pin_memory()
        self.done = torch.zeros(self.max_slots, dtype=torch.int32).pin_memory()
        self.stream = torch.cuda.Stream()
        self.free_slots = list(range(self.max_slots - 1, -1, -1))
        self.active = {}  # slot -> Request
        self.queue = collections.deque()
        self.retiring = []
        self.completed = []
        self.cancelled = []  # requests withdrawn by cancel()
        self._cancelling = []  # (slot, event): slots freed once their in-flight ticks ran
        self.ticks = 0
        self.launches = 0
        self._work_dirty = False
        self._graph = None
        self._tiles_used = 0
        self._work_event = None
        self._in_flight = collections.deque()  # events of replayed ticks
        self._tables = []  # (event, page-locked segment table) of harvest copies in flight
        self.max_ticks_in_flight = 2
        # warm start: the tick graph is captured and replayed once over the empty tables,
        # and the device operations of an admission (key split, row staging, descriptor
        # scatter, pinned copies) run once on the inactive row with its own contents, so
        # every kernel is loaded and every launch set up before the first request arrives
        self._capture()
        with torch.cuda.stream(self.stream):
            self._graph.replay()
            h_row = torch.empty((1, words), dtype=torch.int32, pin_memory=True)
            h_row.copy_(self.desc[self.dummy:self.dummy + 1], non_blocking=True)
            self.stream.synchronize()
            d_row = h_row.to(dev, non_blocking=True)
            keep = d_row[:, RNG_WORD:RNG_WORD + 2].clone()
            d_row[:, RNG_WORD:RNG_WORD + 2] = model_rngs([0])
            d_row[:, RNG_WORD:RNG_WORD + 2] = keep
            self.desc.index_copy_(0, torch.as_tensor([self.dummy], device=dev), d_row)
        self.stream.synchronize()

    # -- graph ------------------------------------------------------------------------
    def _launch(self):
        if self.resident:
            _lib.call("abm_sir_steps_resident", _dev.ptr(self.desc), self.max_slots + 1,
                      _dev.ptr(self.order), self.max_request_agents, self.steps_per_tick,
                      self.res_grid, None, None, _dev.ptr(self.res_scratch),
                      self.res_scratch.numel(), _dev.ptr(self.res_status),
                      self.stream.cuda_stream)
            return
        _lib.call("abm_sir_steps", _dev.ptr(self.desc), self.max_slots + 1, _dev.ptr(self.work),
                  self.max_tiles, _dev.ptr(self.live), self.steps_per_tick, self._launch_ptr(),
                  _dev.ptr(self.changes),
                  self.changes.numel(), self.stream.cuda_stream)

    def _launch_ptr(self):
        self._launch_buf = launch_struct(self.grid)  # kept alive for the call
        return None if self._launch_buf is None else self._launch_buf.ctypes.data

    def _capture(self):
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(self.stream):
            with torch.cuda.graph(g, stream=self.stream):
                self._launch()
        torch.cuda.synchronize()
        self._graph = g

    # -- request lifecycle --------------------------------------------------------------
    def submit(self, req: Request) -> None:
        if self.resident and req.n > self.max_request_agents:
            raise ValueError(f"request {req.rid} has {req.n} agents; this server's resident "
                             f"path holds at most {self.max_request_agents}")
        if req.arrival is None:
            req.arrival = time.perf_counter()
        self.queue.append(req)

    def _tiles(self, req):
        return (req._n + TILE - 1) // TILE

    @staticmethod
    def free_bytes():
        """Device memory available to new requests: free in the driver plus what the caching
        allocator holds but does not use."""
        free, _ = torch.cuda.mem_get_info()
        return free + torch.cuda.memory_reserved() - torch.cuda.memory_allocated()

    def check(self):
        """Raise if the change list overflowed or the resident kernel reported a bad
        instance (bad inputs of single requests are reported on the request: ``error``)."""
        if changes_overflowed(self.changes):
            raise RuntimeError("SIR change list overflowed")
        if self.resident:
            raise_status(int(self.res_status.item()), "SIR server (resident path)")

    def _admit(self):
        """Admit the longest prefix of the queue that fits (free slots, work-list tiles,
        free device memory minus the reserve) as one group: one allocation per buffer kind,
        one host-to-device copy per input array, one descriptor scatter, one key-split
        launch and one pack launch for the whole group."""
        if not self.queue or not self.free_slots:
            return 0
        room = self.free_bytes() - self.reserve
        tiles_left = self.max_tiles - self._tiles_used
        picked, need = [], 0
        for req in self.queue:
            t, b = self._tiles(req), req.device_bytes()
            if len(picked) == len(self.free_slots) or t > tiles_left or need + b > room:
                break
            picked.append(req)
            tiles_left -= t
            need += b
        if not picked:
            return 0
        for _ in picked:
            self.queue.popleft()
        g = len(picked)
        dev, s = self.desc.device, self.stream
        n = np.fromiter((r._n for r in picked), dtype=np.int64, count=g)
        e = np.fromiter((r._e for r in picked), dtype=np.int64, count=g)
        steps = np.fromiter((r.steps for r in picked), dtype=np.int64, count=g)
        wb = (n + 15) // 16 * 16
        rp_off = np.concatenate([[0], np.cumsum(n + 1)])
        col_off = np.concatenate([[0], np.cumsum(e)])
        w_off = np.concatenate([[0], np.cumsum(wb)])
        c_off = np.concatenate([[0], np.cumsum(3 * steps)])
        slots = [self.free_slots.pop() for _ in range(g)]
        with torch.cuda.stream(s):
            rp = torch.empty(int(rp_off[-1]), dtype=torch.int32, device=dev)
            col = torch.empty(int(col_off[-1]), dtype=torch.int32, device=dev)
            st8 = torch.empty(int(w_off[-1]), dtype=torch.int8, device=dev)
            words = torch.empty(int(w_off[-1]), dtype=torch.uint8, device=dev)
            hubs = torch.empty(int(w_off[-1]), dtype=torch.int32, device=dev)
            comp = torch.empty(int(w_off[-1]) // 16, dtype=torch.int32, device=dev)
            counts = torch.zeros(int(c_off[-1]), dtype=torch.int32, device=dev)
            # every request's three arrays in one call: one gather-kernel launch when all
            # are page-locked, else one cudaMemcpyAsync each (the requests keep their
            # converted copies alive; a copy from pageable memory has read its source when
            # the call returns)
            src = np.fromiter((a[1] for r in picked for a in r._spans), dtype=np.uint64,
                              count=3 * g).reshape(g, 3)
            nbytes = np.fromiter((a[2] for r in picked for a in r._spans), dtype=np.uint64,
                                 count=3 * g).reshape(g, 3)
            if np.any(nbytes[:, 0] != 4 * (n + 1)) or np.any(nbytes[:, 1] != 4 * e) \
                    or np.any(nbytes[:, 2] != n):
                raise ValueError("a request's row_ptr, col and state disagree in size")
            dst = np.stack([rp.data_ptr() + 4 * rp_off[:-1], col.data_ptr() + 4 * col_off[:-1],
                            st8.data_ptr() + w_off[:-1]], axis=1).astype(np.uint64)
            table = copy_segments(dst, src, nbytes, True, s,
                                  pinned=all(r._pinned for r in picked))
            rngs = model_rngs([r.seed for r in picked])
        rows = np.zeros(g, dtype=INSTANCE_DTYPE)
        rows["row_ptr"] = rp.data_ptr() + 4 * rp_off[:-1]
        rows["adj"] = col.data_ptr() + 4 * col_off[:-1]
        rows["words"] = words.data_ptr() + w_off[:-1]
        rows["hub_counts"] = hubs.data_ptr() + 4 * w_off[:-1]
        rows["comp"] = comp.data_ptr() + w_off[:-1] // 4
        rows["counts"] = counts.data_ptr() + 4 * c_off[:-1]
        rows["done_flag"] = self.done.data_ptr() + 4 * np.asarray(slots, dtype=np.int64)
        rows["n"] = n
        rows["steps"] = steps
        rows["beta"] = [r.beta for r in picked]
        rows["gamma"] = [r.gamma for r in picked]
        # num_s / num_i / num_r stay 0 here: abm_sir_count_batch adds them on the device
        work, _ = work_table(slots, n, self.dummy, int(((n + TILE - 1) // TILE).sum()))
        self.done.numpy()[np.asarray(slots, dtype=np.int64)] = 0
        h_rows = torch.empty((g, INSTANCE_DTYPE.itemsize // 4), dtype=torch.int32,
                             pin_memory=True)
        h_rows.numpy()[:] = rows.view(np.int32).reshape(g, -1)
        h_work = torch.empty(work.shape, dtype=torch.int32, pin_memory=True)
        h_work.numpy()[:] = work
        h_counts = torch.empty(int(c_off[-1]), dtype=torch.int32, pin_memory=True)
        status = torch.zeros(1, dtype=torch.int32, device=dev)
        with torch.cuda.stream(s):
            d_rows = h_rows.to(dev, non_blocking=True)
            d_rows[:, RNG_WORD:RNG_WORD + 2] = rngs
            self.desc.index_copy_(0, torch.as_tensor(slots, device=dev), d_rows)
            d_work = h_work.to(dev, non_blocking=True)
            _lib.call("abm_sir_count_batch", _dev.ptr(self.desc), _dev.ptr(d_work),
                      work.shape[0], _dev.ptr(st8), _dev.ptr(words), s.cuda_stream)
            _lib.call("abm_sir_pack_batch", _dev.ptr(self.desc), _dev.ptr(d_work), work.shape[0],
                      _dev.ptr(st8), _dev.ptr(words), _dev.ptr(status), s.cuda_stream)
            h_status = torch.zeros(1, dtype=torch.int32).pin_memory()
            h_status.copy_(status, non_blocking=True)
            # staging buffers stay alive until the copies and the pack have run
            done_ev = torch.cuda.Event()
            done_ev.record(s)
        group = _Group((rp, col, st8, words, hubs, comp, counts, h_rows, h_work, d_work,
                        status, done_ev, table), h_status, h_counts)
        now = time.perf_counter()
        for req, slot, w0, c0 in zip(picked, slots, w_off[:-1].tolist(), c_off[:-1].tolist()):
            req._slot = slot
            req._bufs = (group, w0, c0)
            req.admitted = now
            self.active[slot] = req
        self._tiles_used += int(((n + TILE - 1) // TILE).sum())
        self._work_dirty = True
        return g

    def _rebuild_work(self):
        # the pinned staging buffers may still feed the previous rebuild's copies
        if self._work_event is not None:
            self._work_event.synchronize()
        slots = np.fromiter(self.active.keys(), dtype=np.int64, count=len(self.active))
        sizes = np.fromiter((r.n for r in self.active.values()), dtype=np.int64,
                            count=len(self.active))
        table, k = work_table(slots, sizes, self.dummy, self.max_tiles)
        self.h_work.numpy()[:] = table
        if self.resident:
            self.h_order.numpy()[:] = order_table(slots, sizes, self.max_slots + 1)
        with torch.cuda.stream(self.stream):
            self.work[:max(k, 1)].copy_(self.h_work[:max(k, 1)], non_blocking=True)
            self.h_live[0] = k
            self.live.copy_(self.h_live, non_blocking=True)
            if self.resident:
                self.order.copy_(self.h_order, non_blocking=True)
            self._work_event = torch.cuda.Event()
            self._work_event.record(self.stream)
        self._work_dirty = False

    def _harvest(self):
        """Retire requests whose done flag is up: their counts (and final states when kept)
        are copied into their group's pinned result buffer, all of them in one call."""
        slots = np.fromiter(self.active.keys(), dtype=np.int64, count=len(self.active))
        finished = slots[self.done.numpy()[slots] == 1].tolist()
        if finished:
            nf = len(finished)
            dst = np.empty(nf, dtype=np.uint64)
            src = np.empty(nf, dtype=np.uint64)
            nbytes = np.empty(nf, dtype=np.uint64)
            retired = []
            with torch.cuda.stream(self.stream):
                for k, slot in enumerate(finished):
                    req = self.active.pop(slot)
                    group, w0, c0 = req._bufs
                    h_counts = group.h_counts
                    req._counts = (h_counts, c0)  # the view is made on first access
                    dst[k] = h_counts.data_ptr() + 4 * c0
                    src[k] = group.bufs[6].data_ptr() + 4 * c0
                    nbytes[k] = 12 * req.steps
                    if req.keep_state:
                        words_dev = group.bufs[3]
                        req.final_state = torch.empty(req.n, dtype=torch.int8, pin_memory=True)
                        st = unpack_words(words_dev[w0:w0 + req.n], req.n, self.stream)
                        req.final_state.copy_(st, non_blocking=True)
                    # the request's last step ran after its group's pack, so the pinned
                    # status copy is in place
                    if int(group.h_status[0]):
                        req.error = input_error(req)
                    retired.append(req)
                    self._tiles_used -= (req._n + TILE - 1) // TILE
                self.free_slots.extend(finished)
                # every result buffer is page-locked: one gather-kernel launch; its segment
                # table stays referenced until the copy has run
                table = copy_segments(dst, src, nbytes, False, self.stream, pinned=True)
                ev = torch.cuda.Event()
                ev.record(self.stream)
                self._tables.append((ev, table))
            for req in retired:
                req._event = ev
            self.retiring.extend(retired)
            self._work_dirty = True
        self._tables = [(ev, t) for ev, t in self._tables if not ev.query()]
        still, seen = [], {}  # one query per copy event (shared by a harvest's requests)
        now = None
        for req in self.retiring:
            done = seen.get(id(req._event))
            if done is None:
                done = seen[id(req._event)] = req._event.query()
            if done:
                if now is None:
                    now = time.perf_counter()
                req.finished = now
                req._bufs = None
                self.completed.append(req)
            else:
                still.append(req)
        self.retiring = still

    def tick(self) -> None:
        """Admit what fits, advance every resident request by steps_per_tick steps, and
        harvest completions."""
        with nvtx_range("SIRServer.tick"):
            self._tick()

    def _tick(self) -> None:
        self._free_cancelled_slots()
        self._harvest()
        self._admit()
        if self._work_dirty:
            self._rebuild_work()
        if self.active:
            if self._graph is None:
                self._capture()
            with torch.cuda.stream(self.stream):
                self._graph.replay()
                ev = torch.cuda.Event()
                ev.record(self.stream)
            self._in_flight.append(ev)
            while len(self._in_flight) > self.max_ticks_in_flight:
                self._in_flight.popleft().synchronize()
            self.ticks += 1
            if self.resident:
                self.launches += 1
            else:
                per_step = 3 if self.max_slots + 1 <= 256 else 4
                self.launches += (per_step * self.steps_per_tick + 1
                                  + (self.steps_per_tick + 7) // 8)

    def cancel(self, rid) -> bool:
        """Withdraw request ``rid``: a queued request is dropped; an admitted one stops at
        the next tick -- its descriptor's step count is set to 0 on the server stream, so no
        kernel advances it any more, and its slot is reused once the ticks already enqueued
        have run (their last writes to the slot are then done).  Returns whether ``rid``
        was queued or running; cancelled requests go to ``cancelled`` without results."""
        for req in list(self.queue):
            if req.rid == rid:
                self.queue.remove(req)
                req.cancelled = True
                self.cancelled.append(req)
                return True
        for slot, req in list(self.active.items()):
            if req.rid == rid:
                del self.active[slot]
                with torch.cuda.stream(self.stream):
                    self.desc[slot, STEPS_WORD] = 0
                    ev = torch.cuda.Event()
                    ev.record(self.stream)
                req.cancelled = True
                req._bufs = None
                self.cancelled.append(req)
                self._cancelling.append((slot, ev))
                self._tiles_used -= self._tiles(req)
                self._work_dirty = True
                return True
        return False

    def _free_cancelled_slots(self):
        still = []
        for slot, ev in self._cancelling:
            if ev.query():
                self.done.numpy()[slot] = 0
                self.free_slots.append(slot)
            else:
                still.append((slot, ev))
        self._cancelling = still

    def idle(self) -> bool:
        return not (self.queue or self.active or self.retiring)

    def drain(self, timeout_s=600.0) -> None:
        t0 = time.perf_counter()
        while not self.idle():
            self.tick()
            if not self.active and self.retiring:
                self.stream.synchronize()
            if time.perf_counter() - t0 > timeout_s:
                raise TimeoutError("requests still pending after drain timeout")

    def serve(self, requests, arrival_offsets, timeout_s=600.0):
        """Replay a request stream in real time: request i is submitted at
        start + arrival_offsets[i]; returns when all have completed."""
        order = np.argsort(arrival_offsets, kind="stable")
        t0 = time.perf_counter()
        k = 0
        while k < len(order) or not self.idle():
            now = time.perf_counter() - t0
            while k < len(order) and arrival_offsets[order[k]] <= now:
                req = requests[order[k]]
                req.arrival = t0 + float(arrival_offsets[order[k]])
                self.queue.append(req)
                k += 1
            self.tick()
            if self.idle() and k < len(order):
                time.sleep(max(0.0, min(0.002, arrival_offsets[order[k]] - now)))
            elif not self.active and self.retiring:
                self.stream.synchronize()
            if time.perf_counter() - t0 > timeout_s:
                raise TimeoutError("stream not finished before timeout")
        return time.perf_counter() - t0

    def latencies(self):
        return np.array([r.latency for r in self.completed], dtype=np.float64)
