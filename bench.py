"""Benchmark of the agent-step engine on one GB300: agent-steps/s, plain vs batched+served.

Default workload: the batched and served SIR ensemble -- 4,096 SIR instances on
Barabasi-Albert graphs (m=4), agent counts log-uniform in [1e3, 1e5], (beta, gamma) from a
scrambled Sobol sequence (seed 2), 365 steps each.  One bench step = the whole ensemble
(all instances, all 365 steps) in one captured CUDA-graph launch; inputs (~3 GB of CSR)
are larger than L2.  Reported beside it: ``e2e`` (same step through the public batch API
with pinned host buffers: inputs H2D, counts D2H), ``plain`` (one simulation per launch
sequence, the JaxModel.run path, on a sample of the instances), ``served`` (the Poisson
request stream at 200 requests/s replayed in real time through the continuous-batching
server: p50/p99 latency and throughput), and ``cpu_baseline`` (the C/OpenMP oracle on a
sample of the instances, host cores).

Prints ONE JSON line on rank 0.  ``--impl reference`` times the CPU port of the same
workload (the reference itself runs on JAX, which the GPU host does not have), built from
``oracle/`` alone: its inputs come from the oracle's own generators, and its timed steps
together run every member of the ensemble once.

The GPU line carries ``parity``: the oracle's results on the first 1,024 members and the
largest one (from the oracle's own inputs) compared bit for bit with the batched replay;
any mismatch makes the run exit non-zero after printing the line.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402
import torch  # noqa: E402

L2_BYTES = 129 * 1024 * 1024


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.proc = None
        self.dev = device_index

    def start(self):
        try:
            uuid = str(torch.cuda.get_device_properties(self.dev).uuid)
            sel = ["-i", uuid if uuid.startswith("GPU-") else "GPU-" + uuid]
        except Exception:
            sel = []
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"] + sel, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sms, maxs, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sms.append(float(parts[0]))
                maxs.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sms:
            return None
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": max(maxs),
                "reasons": sorted(reasons), "samples": len(sms)}


def _dist():
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def _barrier(world):
    if world > 1:
        torch.distributed.barrier()


def _reduce(v, world, op):
    if world == 1:
        return v
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    torch.distributed.all_reduce(t, op=op)
    return float(t.item())


# --------------------------------------------------------------------------------------
# SIR ensemble (default workload)
# --------------------------------------------------------------------------------------

ENSEMBLE_NAME = "sir_ensemble_4096_ba_m4_n1e3_1e5_t365"


def ensemble_config(sizes, steps, world, m=4):
    """The ``config`` of both arms, from the member sizes alone (a BA(m) graph of n nodes
    has 2 m (n - m) directed edges)."""
    n = np.asarray(sizes, dtype=np.int64)
    e = 2 * m * (n - m)
    return {"workload": ENSEMBLE_NAME, "instances": int(n.size), "steps_per_instance": int(steps),
            "agents": int(n.sum()), "directed_edges": int(e.sum()),
            "l2": "inputs larger than L2 (CSR %.2f GB)" % (e.sum() * 4 / 1e9),
            "parallelism": f"members partitioned across {world} rank(s), balanced by agents"}


class SIREnsembleBench:
    name = ENSEMBLE_NAME

    def __init__(self, rank, world=1, count=4096, steps=365, grids=None, path="auto"):
        from jaxabm_gb300 import ensemble
        self.ensemble = ensemble
        self.T = steps
        spec = ensemble.rank_spec(count, rank, world)  # this rank's share of the members
        self.spec = spec
        self.count = len(spec["n"])
        self.full_sizes = ensemble.ensemble_spec(4096 if count <= 4096 else count)["n"][:count]
        t0 = time.perf_counter()
        self.graphs, self.inits = ensemble.build_instances(spec)
        self.build_s = time.perf_counter() - t0
        # --grids pins the per-step grid kernels; --path resident / grid pins the path
        self.resident = {"auto": None, "resident": True, "grid": False}[path]
        if grids is not None:
            self.resident = False
        # batch members longest first by predicted device time (batch position pos[k] holds
        # this rank's member k): the resident kernel takes them in that order anyway, and
        # the end-to-end leg's index-range copies then land in the order the kernel needs
        self.costs = ensemble.member_costs(self.graphs, self.inits, spec["beta"],
                                           spec["gamma"], steps)
        self.perm = np.argsort(-self.costs, kind="stable")
        self.pos = np.empty_like(self.perm)
        self.pos[self.perm] = np.arange(self.perm.size)
        self.batch = self._make_batch()
        from jaxabm_gb300 import autotune
        t0 = time.perf_counter()
        if grids is not None:
            self.batch.set_launch(grids)
            self.launch = tuple(grids)
            self.picked_by = "--grids"
        elif self.resident:
            self.launch = ensemble.default_launch()
            self.picked_by = "--path resident"
        else:
            self.launch = autotune.tune_sir_batch(self.batch)
            self.picked_by = "jaxabm_gb300.autotune"
        self.tune_s = time.perf_counter() - t0
        self.batch.capture(steps)
        self.units_per_step = self.batch.agent_steps
        self.launches_per_step = self.batch.launches_per_run()
        # pinned host copies of the packed inputs for the end-to-end leg
        b = self.batch
        self.h_rp = torch.from_numpy(b.row_ptr.cpu().numpy()).pin_memory()
        self.h_col = torch.from_numpy(b.col.cpu().numpy()).pin_memory()
        self.h_state = torch.from_numpy(b.h_state0).pin_memory()
        self.h_counts = torch.empty(b.counts.numel(), dtype=torch.int32).pin_memory()

    def _make_batch(self):
        p, spec = self.perm, self.spec
        return self.ensemble.SIRBatch([self.graphs[i] for i in p], [self.inits[i] for i in p],
                                      spec["beta"][p], spec["gamma"][p], spec["seed"][p], self.T,
                                      resident=self.resident)

    def reset(self):
        self.batch.reset()

    def step(self, stream, dom=None):
        if dom:
            dom[0].record(stream)
        self.batch.replay()
        if dom:
            dom[1].record(stream)

    def e2e_step(self, stream):
        b = self.batch
        if b.mode == "resident":
            # copies of later index ranges overlap the kernels of earlier ones
            b.run_from_host(self.h_rp, self.h_col, self.h_state, self.h_counts)
            return
        b.load_host(self.h_rp, self.h_col, self.h_state)
        b.replay()
        self.h_counts.copy_(b.counts, non_blocking=True)

    def e2e_pipelined(self, steps):
        """End to end with two input sets: while step k replays, step k+1's inputs are
        copied from the same pinned host buffers on a second stream (the copy waits until
        that input set's previous replay is done); every step still copies its 3.2 GB in and
        its counts out inside the timed region.  Returns ms per step."""
        if getattr(self, "_b2", None) is None:
            self._b2 = self._make_batch()
            self._b2.set_launch(self.batch.launch_cfg)
            self._b2.set_mode(self.batch.mode)
            self._b2.capture(self.T)
        batches = [self.batch, self._b2]
        comp = torch.cuda.current_stream()
        copy = torch.cuda.Stream()
        ready = [torch.cuda.Event() for _ in range(2)]
        free = [torch.cuda.Event() for _ in range(2)]
        for ev in free:
            ev.record(comp)

        def issue_copy(k):
            b = batches[k % 2]
            copy.wait_event(free[k % 2])
            with torch.cuda.stream(copy):
                b.row_ptr.copy_(self.h_rp, non_blocking=True)
                b.col.copy_(self.h_col, non_blocking=True)
                b.state8.copy_(self.h_state, non_blocking=True)
            ready[k % 2].record(copy)

        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(comp)
        issue_copy(0)
        for k in range(steps):
            if k + 1 < steps:
                issue_copy(k + 1)
            b = batches[k % 2]
            comp.wait_event(ready[k % 2])
            b.rewind_loaded()
            b.replay()
            self.h_counts.copy_(b.counts, non_blocking=True)
            free[k % 2].record(comp)
        e1.record(comp)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    @property
    def e2e_bytes(self):
        h2d = (self.h_rp.numel() + self.h_col.numel()) * 4 + self.h_state.numel()
        return h2d, self.h_counts.numel() * 4

    def final_replay(self):
        """One more replay from step 0 after the timed legs: its status is checked (bad
        inputs raise), its counters give the work of a replay, and its results are what
        the parity check compares."""
        self.batch.reset()
        self.batch.replay()
        torch.cuda.synchronize()
        self.batch.check()

    def algorithmic_bytes(self):
        """HBM bytes of the last replay's work (after :meth:`final_replay`)."""
        scanned, pushed, changes, cands = self.batch.edge_stats()
        self.work_stats = {"live_agent_steps": self.batch.live_agent_steps(),
                           "decision_candidates": cands, "csr_slots_scanned": scanned,
                           "csr_slots_pushed": pushed, "compartment_changes": changes}
        self.work_stats.update(self.batch.threefry_blocks())
        if self.batch.mode == "resident":
            return self.batch.algorithmic_bytes_resident()
        return self.batch.algorithmic_bytes()

    def plain(self, sample=48):
        """One simulation per call (abm_sir_run, the JaxModel.run path), on the first
        ``sample`` instances, each from device-resident inputs, one after another."""
        from jaxabm_gb300 import _dev, _lib
        import jaxabm_gb300.random as jr
        L = _lib.load()
        units, secs = 0, 0.0
        for i in range(min(sample, self.count)):
            rp, col = self.graphs[i]
            n = len(rp) - 1
            drp = torch.from_numpy(rp).cuda()
            dcol = torch.from_numpy(col).cuda()
            buf = torch.from_numpy(self.inits[i]).cuda()
            counts = torch.empty((self.T, 3), dtype=torch.int32, device="cuda")
            ws = torch.empty(L.abm_sir_run_workspace_bytes(n, len(col)), dtype=torch.uint8,
                             device="cuda")
            rng = self.ensemble.model_rngs([int(self.spec["seed"][i])])[0].contiguous()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ck = jr.keychain(rng, self.T, 1).reshape(self.T, 2).contiguous()
            _lib.call("abm_sir_run", _dev.ptr(drp), _dev.ptr(dcol), n, len(col), _dev.ptr(buf),
                      _dev.ptr(ck),
                      self.T, float(self.spec["beta"][i]), float(self.spec["gamma"][i]),
                      _dev.ptr(counts), _dev.ptr(ws), ws.numel(), None)
            torch.cuda.synchronize()
            secs += time.perf_counter() - t0
            units += n * self.T
        return {"value": units / secs, "unit": "agent-steps/s",
                "sample": f"first {min(sample, self.count)} instances, one simulation per "
                          f"call (abm_sir_run, the JaxModel.run path: the key chain, the "
                          f"pack, then one resident launch of one CTA for all steps)"}

    def served(self, burst=False):
        """The request stream through the continuous-batching server: the Poisson arrivals
        at 200 requests/s replayed in real time (latency under the stream's own load), or,
        with ``burst``, every request submitted at once (the server's capacity)."""
        from jaxabm_gb300.serving import Request, SIRServer
        reqs = []
        for i in range(self.count):
            rp, col = self.graphs[i]
            reqs.append(Request(i, torch.from_numpy(rp).pin_memory(),
                                torch.from_numpy(col).pin_memory(),
                                torch.from_numpy(self.inits[i]).pin_memory(),
                                self.spec["beta"][i], self.spec["gamma"][i],
                                int(self.spec["seed"][i]), self.T))
        # a real-time stream is served on the per-step grid kernels (every step of a request
        # spread over the whole GPU: shortest ticks); a burst on the resident kernel (one CTA
        # per request: highest throughput)
        path = "resident" if burst else "grid"
        srv = SIRServer(max_slots=4096, max_tiles=1 << 17, steps_per_tick=32, path=path)
        arrivals = np.zeros(self.count) if burst else self.spec["arrival_s"]
        torch.cuda.synchronize()
        wall = srv.serve(reqs, arrivals)
        lat = srv.latencies()
        units = sum(r.n for r in reqs) * self.T
        # spot-check a few results against the batched run (bit-identical by design)
        self.batch.reset()
        self.batch.replay()
        torch.cuda.synchronize()
        same = all(np.array_equal(r.counts.numpy(),
                                  self.batch.counts_of(int(self.pos[r.rid])).cpu().numpy())
                   for r in sorted(srv.completed, key=lambda r: r.rid)[:: max(1, self.count // 16)])
        return {"value": units / wall, "unit": "agent-steps/s",
                "p50_ms": float(np.percentile(lat, 50) * 1e3),
                "p99_ms": float(np.percentile(lat, 99) * 1e3),
                "requests": len(lat),
                "arrivals": "all at t=0" if burst else "Poisson, 200 requests/s, real time",
                "wall_s": wall, "ticks": srv.ticks, "steps_per_tick": srv.steps_per_tick,
                "path": path, "results_match_batched": bool(same),
                "note": ("the server's capacity: every request submitted at t=0" if burst else
                         "bounded by the arrival rate: the stream offers "
                         f"{units / float(np.max(arrivals)):.3g} agent-steps/s")}

    def oracle_check(self, threads, sample=1024):
        """The C/OpenMP oracle on this rank's first ``sample`` members and its largest one,
        each from the oracle's own inputs (``oracle.workloads``), timed on the host cores
        (``cpu_baseline``) and compared bit for bit with the last replay's per-step counts
        and final compartments (``parity``)."""
        from oracle import coracle, models, workloads
        coracle.set_threads(threads)
        ospec = workloads.sir_ensemble_spec(4096 if len(self.full_sizes) <= 4096
                                            else len(self.full_sizes))
        local = list(range(min(sample, self.count)))
        big = int(np.argmax(self.spec["n"]))
        if big not in local:
            local.append(big)
        members = [int(self.spec["member"][k]) for k in local]
        inputs = workloads.sir_members(ospec, members)
        b = self.batch
        counts = b.counts.reshape(b.k, self.T, 3).cpu().numpy()
        words = self.ensemble.unpack_words(b.words).cpu().numpy()
        w_off = b._offsets[2]
        rngs = np.stack([models.model_keys(int(ospec["seed"][i]), 1)[0] for i in members])
        t0 = time.perf_counter()
        states, ref_counts, _ = coracle.sir_run_many(
            [(rp, col) for rp, col, _ in inputs], [st0 for _, _, st0 in inputs], rngs, self.T,
            ospec["beta"][members], ospec["gamma"][members])
        secs = time.perf_counter() - t0
        units = sum(len(st0) for _, _, st0 in inputs) * self.T
        bad = []
        for j, (k, i) in enumerate(zip(local, members)):
            q = int(self.pos[k])  # the member's batch position
            gpu_state = words[w_off[q]:w_off[q] + len(states[j])]
            if not (np.array_equal(ref_counts[j], counts[q])
                    and np.array_equal(states[j], gpu_state)):
                bad.append(i)
        desc = (f"members {members[0]}..{members[min(sample, self.count) - 1]} (first "
                f"{min(sample, self.count)} of this rank) and the largest ({members[-1]}, "
                f"{int(self.spec['n'][big])} agents), {self.T} steps each, C/OpenMP oracle "
                f"(host threads take whole members) on the oracle's own inputs")
        cpu = {"value": units / secs, "unit": "agent-steps/s", "cores": threads, "kind": "port",
               "sample": desc}
        parity = {"instances_checked": len(local), "mismatches": len(bad),
                  "mismatched_members": bad[:16], "compared": "all per-step S/I/R counts and "
                  "final compartments, bit for bit", "sample": desc}
        return cpu, parity


def _time_ms(fn, reps=3, warmup=1):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(reps):
        fn()
    e.record()
    e.synchronize()
    return s.elapsed_time(e) / reps


def model_lines():
    """Single-model throughput of the other workload models (device-resident inputs)."""
    from jaxabm_gb300 import _dev, _lib, opinion, schelling, sir
    import jaxabm_gb300.random as jr
    L = _lib.load()
    out = {}

    # quick-start random walk: N = 10,000, 100 steps, PRNGKey(0)
    n, T = 10_000, 100
    x = torch.rand(n, device="cuda")
    y = torch.rand(n, device="cuda")
    rng = jr.split(jr.PRNGKey(0), 2)[0].contiguous()
    ck = torch.empty((T, 1, 2), dtype=torch.int32, device="cuda")
    means = torch.empty((T, 2), device="cuda")
    ws = torch.empty(L.abm_randomwalk_workspace_bytes(n, T), dtype=torch.uint8, device="cuda")

    def rw():
        _lib.call("abm_keychain", _dev.ptr(rng), 1, 1, T, _dev.ptr(ck), None, None)
        _lib.call("abm_randomwalk_run", _dev.ptr(x), _dev.ptr(y), n, _dev.ptr(ck), T, 0.01,
                  _dev.ptr(means), _dev.ptr(ws), ws.numel(), None)
    ms = _time_ms(rw, reps=20)
    out["randomwalk_n10000_t100"] = {"agent_steps_per_s": n * T / (ms / 1e3), "ms_per_run": ms,
                                     "launches_per_run": 3}

    # Schelling 256 x 256 torus, density 0.9, 200 steps, seed 1
    W = H = 256
    pos0, types = schelling.initial_layout(W, H, 0.9, 0.5, 1)
    n = len(pos0)
    T = 200
    p = torch.from_numpy(pos0).cuda()
    t8 = torch.from_numpy(types).cuda()
    grid = torch.empty(W * H, dtype=torch.int8, device="cuda")
    ca = torch.empty(W * H, dtype=torch.int32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    stats = torch.empty((T, 2), dtype=torch.int32, device="cuda")
    ws = torch.empty(L.abm_schelling_workspace_bytes(n, W, H), dtype=torch.uint8, device="cuda")
    rng = jr.split(jr.PRNGKey(1), 2)[0].contiguous()
    ck = jr.keychain(rng.clone(), T, 1).reshape(T, 2).contiguous()
    p0 = p.clone()

    def sch():
        p.copy_(p0)
        _lib.call("abm_schelling_place", _dev.ptr(p), _dev.ptr(t8), n, W, H, _dev.ptr(grid),
                  _dev.ptr(ca), _dev.ptr(status), None)
        _lib.call("abm_schelling_run", _dev.ptr(p), _dev.ptr(t8), n, W, H, _dev.ptr(grid),
                  _dev.ptr(ca), _dev.ptr(ck), T, 3, 8, _dev.ptr(stats), _dev.ptr(ws), ws.numel(),
                  None)
    ms = _time_ms(sch, reps=3)
    out["schelling_256x256_t200"] = {"agent_steps_per_s": n * T / (ms / 1e3), "ms_per_run": ms,
                                     "launches_per_run": 3}

    # SIR, one model: N = 2^20 Barabasi-Albert m=4, 365 steps (the plain engine)
    n, T = 1 << 20, 365
    rp, col = sir.barabasi_albert(n, 4, 0)
    drp, dcol = torch.from_numpy(rp).cuda(), torch.from_numpy(col).cuda()
    st0 = torch.from_numpy(sir.initial_states(n, 0.001, 0)).cuda()
    st = st0.clone()
    counts = torch.empty((T, 3), dtype=torch.int32, device="cuda")
    ws = torch.empty(L.abm_sir_run_workspace_bytes(n, len(col)), dtype=torch.uint8,
                     device="cuda")
    rng = jr.split(jr.PRNGKey(0), 2)[0].contiguous()
    ck = jr.keychain(rng.clone(), T, 1).reshape(T, 2).contiguous()

    def sir1():
        st.copy_(st0)
        _lib.call("abm_sir_run", _dev.ptr(drp), _dev.ptr(dcol), n, len(col), _dev.ptr(st),
                  _dev.ptr(ck), T,
                  0.05, 0.1, _dev.ptr(counts), _dev.ptr(ws), ws.numel(), None)
    ms = _time_ms(sir1, reps=3)
    out["sir_ba_n1048576_t365"] = {"agent_steps_per_s": n * T / (ms / 1e3), "ms_per_run": ms,
                                   "launches_per_run": 3 * T + 6 + (T + 7) // 8,
                                   "path": "abm_sir_run, kernels launched one by one"}
    # the same model as a one-instance batch, its 365 steps replayed from one CUDA graph
    from jaxabm_gb300 import ensemble
    b1 = ensemble.SIRBatch([(rp, col)], [sir.initial_states(n, 0.001, 0)], [0.05], [0.1], [0],
                           T)
    b1.capture(T)

    def sir_graph():
        b1.reset()
        b1.replay()
    ms = _time_ms(sir_graph, reps=3)
    out["sir_ba_n1048576_t365_graph"] = {
        "agent_steps_per_s": n * T / (ms / 1e3), "ms_per_run": ms,
        "launches_per_run": b1.launches_per_run(),
        "path": "SIRBatch of one instance, CUDA-graph replay (reset included)"}
    del b1

    # opinion calibration: N = 2^18, 16-regular, 64 instances, 200 steps, checkpoints every 20
    n, B, T = 1 << 18, 64, 200
    rp, col = sir.random_regular(n, 16, 0)
    o0 = opinion.initial_opinions(n, 0)
    pr = opinion.calibration_params(B)
    batch = opinion.OpinionBatch(rp, col, o0, pr[:, 0], pr[:, 1], pr[:, 2])
    target = np.array([0.5, 0.3, 0.2, 0.15])
    ms_f = _time_ms(lambda: batch.forward(T), reps=2)

    def fwd_adj():
        batch.forward(T, 20)
        batch.backward(target)
    ms_fa = _time_ms(fwd_adj, reps=1)
    # the forward's work: one exact sigmoid and update per CSR slot, instance and step;
    # compulsory bytes per step: the opinions read once and written once, the CSR once
    evals = len(col) * B * T
    fwd_bytes = (2 * 4 * n * B + 4 * (len(col) + n + 1)) * T
    hbm, _ = _peaks()
    out["opinion_n262144_b64_t200"] = {
        "instance_agent_steps_per_s_forward": n * B * T / (ms_f / 1e3), "ms_forward": ms_f,
        "ms_forward_plus_adjoint": ms_fa,
        "instance_agent_steps_per_s_forward_plus_adjoint": n * B * T / (ms_fa / 1e3),
        "forward": {"edge_instance_evaluations_per_s": evals / (ms_f / 1e3),
                    "bound": "fp32 issue (table-driven exponential, IEEE reciprocal and "
                             "division per evaluation); the neighbour rows are L2 hits",
                    "hbm_frac_of_compulsory_bytes": fwd_bytes / (ms_f / 1e3) / 1e9 / hbm}}

    # sensitivity analysis: 256 Latin-hypercube samples of (beta, gamma) for an SIR model of
    # 10,000 agents (BA m=4, its own graph per sample seed), 365 steps; host wall time of the
    # whole analysis (graphs, packing, one batched replay, results) against the same
    # models run one by one (8 of them timed, scaled to 256)
    import time

    import jaxabm_gb300 as jx

    def sa_factory(params=None, config=None):
        p = {"n": 10_000, "m": 4, "steps": 365}
        p.update(params or {})
        return jx.SIRModel(p, seed=config.seed)
    ranges = {"beta": (0.01, 0.2), "gamma": (0.05, 0.3)}
    sa = jx.SensitivityAnalysis(sa_factory, ranges, ["I", "R"], num_samples=256, seed=0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sa.run(verbose=False)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    host = sa.samples.cpu().numpy()
    t0 = time.perf_counter()
    for i in range(8):
        sa_factory(params={"beta": float(host[i, 0]), "gamma": float(host[i, 1])},
                   config=jx.ModelConfig(seed=1000 + i)).run()
    torch.cuda.synchronize()
    serial = (time.perf_counter() - t0) / 8 * 256
    out["sensitivity_sir_256_samples_n10000_t365"] = {
        "wall_s": wall, "batched": sa.batched, "serial_wall_s_estimate": serial,
        "speedup": serial / wall, "agent_steps_per_s": 256 * 10_000 * 365 / wall,
        "note": "host clock around SensitivityAnalysis.run (graph generation and packing "
                "included); serial = each sample's model.run() alone, 8 timed"}
    del sa

    hbm, _ = _peaks()
    # Network CSR on the device: the 8,388,576 directed edges of BA(2^20, m=4) in shuffled
    # order -> row_ptr/col (stable radix sort by source)
    rp, col = sir.barabasi_albert(1 << 20, 4, 0)
    nn = len(rp) - 1
    perm = np.random.RandomState(0).permutation(len(col))
    esrc = torch.from_numpy(np.repeat(np.arange(nn), np.diff(rp)).astype(np.int32)[perm]).cuda()
    edst = torch.from_numpy(col[perm]).cuda()
    E = len(col)
    crp = torch.empty(nn + 1, dtype=torch.int32, device="cuda")
    ccol = torch.empty(E, dtype=torch.int32, device="cuda")
    cst = torch.zeros(1, dtype=torch.int32, device="cuda")
    ws = torch.empty(L.abm_csr_workspace_bytes(E, nn), dtype=torch.uint8, device="cuda")

    def csr():
        _lib.call("abm_csr_from_edges", _dev.ptr(esrc), _dev.ptr(edst), E, nn, _dev.ptr(crp),
                  _dev.ptr(ccol), _dev.ptr(cst), _dev.ptr(ws), ws.numel(), None)
    ms = _time_ms(csr, reps=5)
    out["csr_from_edges_ba_n1048576"] = {"edges_per_s": E / (ms / 1e3), "ms": ms,
                                         "launches_per_call": 3 * 3 + 2}
    del esrc, edst, ccol, ws

    # K6 compaction of a 2^28-entry mask (half set, larger than L2) into int32 indices
    n = 1 << 28
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    mask = (torch.rand(n, device="cuda", generator=g) < 0.5).view(torch.uint8)
    idx = torch.empty(n, dtype=torch.int32, device="cuda")
    count = torch.zeros(1, dtype=torch.int64, device="cuda")
    ws = torch.empty(L.abm_select_workspace_bytes(n), dtype=torch.uint8, device="cuda")

    def sel():
        _lib.call("abm_select_indices", _dev.ptr(mask), n, _dev.ptr(idx), _dev.ptr(count),
                  _dev.ptr(ws), ws.numel(), None)
    ms = _time_ms(sel, reps=5)
    k = int(count.item())
    alg = n + 4 * k  # mask read once, indices written once
    out["select_mask_268435456"] = {
        "entries_per_s": n / (ms / 1e3), "ms": ms, "selected": k, "launches_per_call": 3,
        "roofline": {"bound": "hbm", "achieved": alg / (ms / 1e3) / 1e9, "peak": hbm,
                     "unit": "GB/s", "frac": alg / (ms / 1e3) / 1e9 / hbm,
                     "algorithmic_bytes": alg,
                     "note": "1 B mask read + 4 B per selected index written; the kernels "
                             "read the mask twice (count pass, scatter pass)"}}
    del mask, idx, ws

    # K1 sampler: jax.random.uniform(PRNGKey(0), (2^28,)) -- one threefry per element
    out_u = torch.empty(n, dtype=torch.float32, device="cuda")
    key = jr.PRNGKey(0)

    def uni():
        _lib.call("abm_rng_uniform", _dev.ptr(key), 1, n, 0.0, 1.0, _dev.ptr(out_u), 1, None)
    ms = _time_ms(uni, reps=5)
    out["rng_uniform_268435456"] = {
        "samples_per_s": n / (ms / 1e3), "ms": ms,
        "roofline": {"bound": "alu", "achieved": 4 * n / (ms / 1e3) / 1e9, "peak": hbm,
                     "unit": "GB/s written", "frac": 4 * n / (ms / 1e3) / 1e9 / hbm,
                     "note": "one threefry2x32-20 block per sample; HBM fraction of the "
                             "4-byte writes"}}
    return out


WORKLOADS = {"sir_ensemble": SIREnsembleBench}
DEFAULT_WORKLOAD = "sir_ensemble"


def sampler_block_rate(reps=5):
    """Measured threefry2x32-20 block rate of the K1 sampler (jax.random.uniform over 2^28
    elements, one block per element, ALU-bound): the issue-side peak of the SIR kernels,
    whose work is dominated by the same blocks."""
    from jaxabm_gb300 import _dev, _lib
    import jaxabm_gb300.random as jr
    n = 1 << 28
    out = torch.empty(n, dtype=torch.float32, device="cuda")
    key = jr.PRNGKey(0)

    def uni():
        _lib.call("abm_rng_uniform", _dev.ptr(key), 1, n, 0.0, 1.0, _dev.ptr(out), 1, None)
    ms = _time_ms(uni, reps=reps, warmup=2)
    del out
    return n / (ms / 1e3), ms


def run_ours(args):
    world, rank, local = _dist()
    if world > 1:
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    import jaxabm_gb300 as jx
    jx.set_verbose(False)
    jx.build()
    grids = None if not args.grids else tuple(int(v) for v in args.grids.split(","))
    wl = WORKLOADS[args.workload](rank, world, count=args.instances, grids=grids,
                                  path=args.path)
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        wl.reset()
        wl.step(stream)
    torch.cuda.synchronize()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    clocks.start()
    _barrier(world)
    torch.cuda.synchronize()
    for i in range(args.steps):
        wl.reset()
        wl.step(stream, (starts[i], ends[i]))
    torch.cuda.synchronize()
    _barrier(world)
    clk = clocks.stop()
    wl.batch.check()  # a bad input of the timed replays raises here
    ms_local = sum(s.elapsed_time(e) for s, e in zip(starts, ends)) / args.steps
    ms = _reduce(ms_local, world, torch.distributed.ReduceOp.MAX if world > 1 else None)

    # end-to-end through the batch API with pinned host buffers
    for _ in range(2):
        wl.e2e_step(stream)
    torch.cuda.synchronize()
    _barrier(world)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        wl.e2e_step(stream)
    e1.record(stream)
    torch.cuda.synchronize()
    _barrier(world)
    e2e_ms = _reduce(e0.elapsed_time(e1) / args.steps, world,
                     torch.distributed.ReduceOp.MAX if world > 1 else None)

    e2e_pipe_ms = _reduce(wl.e2e_pipelined(args.steps), world,
                          torch.distributed.ReduceOp.MAX if world > 1 else None)
    units = _reduce(wl.units_per_step, world, torch.distributed.ReduceOp.SUM if world > 1 else None)
    value = units / (ms / 1e3)
    hbm_peak, peak_kind = _peaks()
    wl.final_replay()
    alg_bytes = wl.algorithmic_bytes()
    achieved = alg_bytes / (ms_local / 1e3) / 1e9
    blocks = wl.work_stats["blocks"]
    block_peak, sampler_ms = sampler_block_rate()
    # the per-unit figure of a whole-graph pass (every agent reads its row each step:
    # 4 B column + 1 B neighbour state per CSR slot, 6 B per agent), which the frontier
    # formulation does not move; its rate can exceed the HBM peak for that reason
    dense_bytes = int((5 * wl.batch.e.sum() + 6 * wl.batch.n.sum()) * wl.T)
    dense = {"bytes_per_step": dense_bytes,
             "achieved": dense_bytes / (ms_local / 1e3) / 1e9, "unit": "GB/s",
             "frac": dense_bytes / (ms_local / 1e3) / 1e9 / hbm_peak,
             "note": "bytes a dense pass over every agent and CSR slot would move per "
                     "replay (5 B per slot + 6 B per agent and step); not the bound"}
    h2d, d2h = wl.e2e_bytes
    out = {
        "metric": "agent-steps/s", "value": value, "unit": "agent-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "int8",
        "data": "synthetic",
        "config": ensemble_config(wl.full_sizes, wl.T, world),
        "e2e": {"value": units / (e2e_ms / 1e3), "unit": "agent-steps/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "path": ("SIRBatch.run_from_host: page-locked inputs copied in 8 index "
                         "ranges, each range's resident launch starting when its copies "
                         "land, its counts copied back when it ends"
                         if wl.batch.mode == "resident" else
                         "SIRBatch.load_host + replay + counts copy")},
        "e2e_pipelined": {"value": units / (e2e_pipe_ms / 1e3), "unit": "agent-steps/s",
                          "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                          "note": "two input sets: step k+1's host-to-device copies run on a "
                                  "second stream during step k's replay"},
        "gpu_launches": wl.launches_per_step * args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": None,
                     "traffic_note": "DRAM bytes come from ncu captures only (not measurable "
                                     "in-run); the committed profile summaries give them",
                     "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"
                     if peak_kind == "measured" else "fallback",
                     "kernel": ("sir_resident_kernel: one launch runs every step of every "
                                "instance (one CTA per instance at a time, words in shared "
                                "memory); bound by the latency of each warp's dependent work "
                                "(threefry chains, row loads) at 2 CTAs per SM, not by HBM"
                                if wl.batch.mode == "resident" else
                                "SIR step sequence (sweep + candidates + push + finalize per "
                                "step; 365 steps in one CUDA-graph replay), timed as a unit"),
                     "algorithmic_bytes_per_step": alg_bytes,
                     "work_per_step": wl.work_stats,
                     "dense_equivalent": dense},
        "roofline_issue": {"bound": "threefry2x32-20 blocks (ALU issue)",
                           "achieved": blocks / (ms_local / 1e3), "peak": block_peak,
                           "unit": "blocks/s", "frac": blocks / (ms_local / 1e3) / block_peak,
                           "blocks_per_step": blocks,
                           "peak_kind": "measured in this run: the K1 sampler "
                                        "(jax.random.uniform, 2^28 elements, one block each, "
                                        f"{sampler_ms:.3f} ms)"},
        "clocks": clk,
    }
    if not args.quick:
        out["plain"] = wl.plain()
        out["plain"]["batched_over_plain"] = value / out["plain"]["value"]
        out["served"] = wl.served()
        out["served"]["served_over_plain"] = out["served"]["value"] / out["plain"]["value"]
        out["served_burst"] = wl.served(burst=True)
        out["served_burst"]["served_over_plain"] = (out["served_burst"]["value"]
                                                    / out["plain"]["value"])
        wl.final_replay()  # the served legs replay the batch: the parity check reads a fresh run
    parity = None
    if rank == 0 and not args.no_parity:
        cpu, parity = wl.oracle_check(os.cpu_count() or 1)
        if world == 1:
            out["cpu_baseline"] = cpu
        out["parity"] = parity
    if not args.quick or args.models:
        out["models"] = model_lines()
    out["setup_s"] = {"graph_build": wl.build_s, "autotune": wl.tune_s}
    out["launch"] = {"path": wl.batch.mode, "sweep": wl.launch[0], "candidates": wl.launch[1],
                     "push": wl.launch[2], "picked_by": wl.picked_by}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    if parity is not None and parity["mismatches"]:
        sys.exit(3)


def run_reference(args):
    """The reference's CPU path on the same workload: the C/OpenMP port of the SIR step
    (the reference itself needs JAX, absent on this host) on all host cores, with inputs
    from the oracle's own generators.  The members are split into ``--steps`` runs of
    nearly equal agent totals; timed step k runs run k, so the timed steps together run
    every member once (warm-up step w runs run w mod steps, untimed)."""
    world, rank, _ = _dist()
    if rank != 0:
        return
    from oracle import coracle, models, workloads
    cores = os.cpu_count() or 1
    coracle.set_threads(cores)
    T = 365
    spec = workloads.sir_ensemble_spec(4096 if args.instances <= 4096 else args.instances)
    count = args.instances
    sizes = spec["n"][:count]
    runs = workloads.balanced_slices(sizes, args.steps)
    t0 = time.perf_counter()
    members = workloads.sir_members(spec, range(count))
    build_s = time.perf_counter() - t0

    rngs = np.stack([models.model_keys(int(spec["seed"][i]), 1)[0] for i in range(count)])

    def one_step(k):
        idx = runs[k]
        coracle.sir_run_many([members[i][:2] for i in idx], [members[i][2] for i in idx],
                             rngs[idx], T, spec["beta"][idx], spec["gamma"][idx])
        return int(sizes[idx].sum()) * T

    for w in range(args.warmup):
        one_step(w % args.steps)
    units, secs = 0, 0.0
    for k in range(args.steps):
        t0 = time.perf_counter()
        units += one_step(k)
        secs += time.perf_counter() - t0
    value = units / secs
    ms = 1e3 * secs / args.steps
    out = {"metric": "agent-steps/s", "value": value, "unit": "agent-steps/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "int8",
           "data": "synthetic", "impl": "reference",
           "config": ensemble_config(sizes, T, world),
           "cpu_baseline": {"value": value, "unit": "agent-steps/s", "cores": cores,
                            "kind": "port",
                            "sample": f"all {count} members over the {args.steps} timed steps "
                                      f"(step k runs the k-th of {args.steps} runs of nearly "
                                      f"equal agent totals), {T} steps each; C/OpenMP port of "
                                      f"the reference's SIR step (host threads take whole "
                                      f"members) on the oracle's own inputs (the reference "
                                      f"needs JAX, absent on this host)"},
           "e2e": {"value": value, "unit": "agent-steps/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0},
           "setup_s": {"input_build": build_s}}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--quick", action="store_true",
                    help="only the batched value and e2e (no plain/served/cpu legs)")
    ap.add_argument("--models", action="store_true",
                    help="with --quick: also time the single-model workloads")
    ap.add_argument("--instances", type=int, default=4096,
                    help="ensemble members (the first K of the 4,096-member specification); "
                         "smaller values are for profiling captures")
    ap.add_argument("--path", default="auto", choices=["auto", "resident", "grid"],
                    help="SIR ensemble path: the autotuner's choice, the resident "
                         "per-instance kernel, or the per-step grid kernels")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the oracle parity check (profiling captures)")
    ap.add_argument("--grids", default=None,
                    help="fixed sweep,candidates,push grid sizes instead of the autotuner "
                         "(profiling captures: keeps the launch sequence short)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
