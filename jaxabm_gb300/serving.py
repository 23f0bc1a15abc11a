"""Continuous-batching server for SIR simulation requests.

Requests (a network, initial compartments, beta, gamma, seed, steps) arrive over time.
The server keeps every admitted request resident on the device as one instance of the
batched SIR step (``abm_sir_steps``) and advances all of them together, ``steps_per_tick``
steps per tick:

* admission: a request is admitted when a descriptor slot is free, its tiles fit the work
  list, and its buffers fit the free device memory (``torch.cuda.mem_get_info``) minus a
  reserve; otherwise it waits in the queue (first come, first served);
* every tick replays ONE captured CUDA graph over a fixed-capacity work list; admitting or
  retiring requests only rewrites device tables (descriptor rows, work items), so the graph
  is never re-captured;
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
from .ensemble import (INSTANCE_DTYPE, RNG_WORD, TILE, changes_overflowed, changes_workspace,
                       check_layout, launch_struct, model_rngs, pack_words, unpack_words,
                       word_bytes)


class Request:
    __slots__ = ("rid", "row_ptr", "col", "state", "beta", "gamma", "seed", "steps",
                 "arrival", "admitted", "finished", "counts", "final_state", "_slot",
                 "_bufs", "_event", "keep_state")

    def __init__(self, rid, row_ptr, col, state, beta, gamma, seed, steps, arrival=None,
                 keep_state=False):
        self.rid = rid
        self.row_ptr, self.col, self.state = row_ptr, col, state
        self.beta, self.gamma, self.seed, self.steps = float(beta), float(gamma), int(seed), int(steps)
        self.arrival = arrival
        self.admitted = None
        self.finished = None
        self.counts = None
        self.final_state = None
        self.keep_state = keep_state
        self._slot = None
        self._bufs = None
        self._event = None

    @property
    def n(self):
        return len(self.row_ptr) - 1

    def device_bytes(self):
        n, e = self.n, len(self.col)
        # CSR, int8 compartments, word bytes (padded to 16), hub counts, per-step counts
        return 4 * (n + 1) + 4 * e + n + (n + 15) // 16 * 16 + 4 * n + 12 * self.steps

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
    """

    def __init__(self, max_slots=512, max_tiles=65536, steps_per_tick=16,
                 reserve_bytes=1 << 30, grid=None):
        check_layout()
        dev = _dev.device()
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
        self.ticks = 0
        self.launches = 0
        self._work_dirty = False
        self._graph = None
        self._tiles_used = 0
        self._work_event = None
        self._in_flight = collections.deque()  # events of replayed ticks
        self.max_ticks_in_flight = 2

    # -- graph ------------------------------------------------------------------------
    def _launch(self):
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
        if req.arrival is None:
            req.arrival = time.perf_counter()
        self.queue.append(req)

    def _tiles(self, req):
        return (req.n + TILE - 1) // TILE

    @staticmethod
    def free_bytes():
        """Device memory available to new requests: free in the driver plus what the caching
        allocator holds but does not use."""
        free, _ = torch.cuda.mem_get_info()
        return free + torch.cuda.memory_reserved() - torch.cuda.memory_allocated()

    def check(self):
        if changes_overflowed(self.changes):
            raise RuntimeError("SIR change list overflowed")

    def _try_admit(self, req) -> bool:
        if not self.free_slots or self._tiles_used + self._tiles(req) > self.max_tiles:
            return False
        if self.free_bytes() - self.reserve < req.device_bytes():
            return False
        slot = self.free_slots.pop()
        dev = self.desc.device
        s = self.stream
        with torch.cuda.stream(s):
            rp = torch.as_tensor(req.row_ptr).to(dev, non_blocking=True)
            col = torch.as_tensor(req.col).to(dev, non_blocking=True)
            st8 = torch.as_tensor(req.state).to(dev, non_blocking=True)
            st = torch.empty(word_bytes(req.n), dtype=torch.uint8, device=dev)
            hubs = torch.empty(req.n, dtype=torch.int32, device=dev)
            pack_words(st8, rp, col, col, st, hubs, s)
            counts = torch.zeros(req.steps * 3, dtype=torch.int32, device=dev)
            rng = model_rngs([req.seed])
        host_state = np.asarray(req.state)
        row = np.zeros(1, dtype=INSTANCE_DTYPE)
        row["row_ptr"] = rp.data_ptr()
        row["adj"] = col.data_ptr()
        row["words"] = st.data_ptr()
        row["hub_counts"] = hubs.data_ptr()
        row["counts"] = counts.data_ptr()
        row["done_flag"] = self.done.data_ptr() + 4 * slot
        row["n"] = req.n
        row["t"] = 0
        row["steps"] = req.steps
        row["beta"] = req.beta
        row["gamma"] = req.gamma
        row["num_s"] = int((host_state == 0).sum())
        row["num_i"] = int((host_state == 1).sum())
        row["num_r"] = int((host_state == 2).sum())
        self.done[slot] = 0
        self.h_desc[slot] = torch.from_numpy(row.view(np.int32).copy())
        with torch.cuda.stream(s):
            self.desc[slot].copy_(self.h_desc[slot], non_blocking=True)
            self.desc[slot, RNG_WORD:RNG_WORD + 2] = rng[0]
        req._slot = slot
        req._bufs = (rp, col, st, hubs, counts)
        req.admitted = time.perf_counter()
        self.active[slot] = req
        self._tiles_used += self._tiles(req)
        self._work_dirty = True
        return True

    def _rebuild_work(self):
        # the pinned staging buffers may still feed the previous rebuild's copies
        if self._work_event is not None:
            self._work_event.synchronize()
        w = self.h_work
        w[:, 0] = self.dummy
        w[:, 1:] = 0
        k = 0
        for slot, req in self.active.items():
            b = torch.arange(0, req.n, TILE, dtype=torch.int32)
            m = b.numel()
            w[k:k + m, 0] = slot
            w[k:k + m, 1] = b
            w[k:k + m, 2] = torch.clamp(b + TILE, max=req.n)
            k += m
        with torch.cuda.stream(self.stream):
            self.work[:max(k, 1)].copy_(w[:max(k, 1)], non_blocking=True)
            self.h_live[0] = k
            self.live.copy_(self.h_live, non_blocking=True)
            self._work_event = torch.cuda.Event()
            self._work_event.record(self.stream)
        self._work_dirty = False

    def _harvest(self):
        """Retire requests whose done flag is up: enqueue their result copies."""
        finished = [slot for slot in self.active if int(self.done[slot]) == 1]
        for slot in finished:
            req = self.active.pop(slot)
            rp, col, st, hubs, counts = req._bufs
            with torch.cuda.stream(self.stream):
                req.counts = torch.empty((req.steps, 3), dtype=torch.int32).pin_memory()
                req.counts.copy_(counts.view(req.steps, 3), non_blocking=True)
                if req.keep_state:
                    req.final_state = torch.empty(req.n, dtype=torch.int8).pin_memory()
                    req.final_state.copy_(unpack_words(st, req.n, self.stream), non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(self.stream)
            req._event = ev
            self.retiring.append(req)
            self._tiles_used -= self._tiles(req)
            self.free_slots.append(slot)
            self._work_dirty = True
        still = []
        for req in self.retiring:
            if req._event.query():
                req.finished = time.perf_counter()
                req._bufs = None
                self.completed.append(req)
            else:
                still.append(req)
        self.retiring = still

    def tick(self) -> None:
        """Admit what fits, advance every resident request by steps_per_tick steps, and
        harvest completions."""
        self._harvest()
        while self.queue and self._try_admit(self.queue[0]):
            self.queue.popleft()
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
            self.launches += 4 * self.steps_per_tick + 1 + (self.steps_per_tick + 7) // 8

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
