"""Benchmark of the agent-step engine on one GB300 (agent-steps/s).

Prints ONE JSON line on rank 0.  ``--impl reference`` times the CPU oracle port of the
same workload on the host cores instead (the reference runs on JAX, which is not
available on the GPU host).
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
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def _barrier(world):
    if world > 1:
        torch.distributed.barrier()


def _max_over_ranks(v, world):
    if world == 1:
        return v
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def _sum_over_ranks(v, world):
    if world == 1:
        return v
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.SUM)
    return float(t.item())


# --------------------------------------------------------------------------------------
# workloads
# --------------------------------------------------------------------------------------

class RandomWalkBench:
    """Quick-start random walk: N=10,000 agents, 100 steps, PRNGKey(0); one bench step is
    one full 100-step run (1e6 agent-steps)."""

    name = "randomwalk_n10000_t100"

    def __init__(self, rank, n=10_000, steps=100, sigma=0.01):
        from jaxabm_gb300 import _dev, _lib
        import jaxabm_gb300.random as jr
        from oracle import models
        self._lib, self._dev, self.jr = _lib, _dev, jr
        self.n, self.T, self.sigma = n, steps, sigma
        rng, (ik,) = models.model_keys(rank, 1)
        self.rng0 = rng
        self.x = torch.empty(n, dtype=torch.float32, device="cuda")
        self.y = torch.empty(n, dtype=torch.float32, device="cuda")
        _lib.call("abm_randomwalk_init", _dev.ptr(self.x), _dev.ptr(self.y), n,
                  _dev.ptr(_dev.keys_from_numpy(ik)), None)
        self.x0 = self.x.clone()
        self.y0 = self.y.clone()
        self.rng = _dev.keys_from_numpy(rng)
        self.ck = torch.empty((steps, 1, 2), dtype=torch.int32, device="cuda")
        self.means = torch.empty((steps, 2), dtype=torch.float32, device="cuda")
        wsb = _lib.load().abm_randomwalk_workspace_bytes(n, steps)
        self.ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
        self.launches_per_step = 3
        self.units_per_step = n * steps
        self.bytes_per_unit = 16  # read + write x, y per agent-step (keys live in registers)
        self.h_x = torch.empty(n, dtype=torch.float32).pin_memory()
        self.h_y = torch.empty(n, dtype=torch.float32).pin_memory()
        self.h_x.copy_(self.x0.cpu())
        self.h_y.copy_(self.y0.cpu())
        self.h_means = torch.empty((steps, 2), dtype=torch.float32).pin_memory()

    def reset(self):
        self.x.copy_(self.x0)
        self.y.copy_(self.y0)

    def step(self, stream, dom_events=None):
        L, D = self._lib, self._dev
        s = stream.cuda_stream
        L.call("abm_keychain", D.ptr(self.rng), 1, 1, self.T, D.ptr(self.ck), None, s)
        if dom_events:
            dom_events[0].record(stream)
        L.call("abm_randomwalk_run", D.ptr(self.x), D.ptr(self.y), self.n, D.ptr(self.ck), self.T,
               self.sigma, D.ptr(self.means), D.ptr(self.ws), self.ws.numel(), s)
        if dom_events:
            dom_events[1].record(stream)

    def e2e_step(self, stream):
        """Same step through the C ABI with host buffers: H2D of the states, run, D2H of
        the per-step means."""
        self.x.copy_(self.h_x, non_blocking=True)
        self.y.copy_(self.h_y, non_blocking=True)
        self.step(stream)
        self.h_means.copy_(self.means, non_blocking=True)

    @property
    def e2e_bytes(self):
        return 8 * self.n, 8 * self.T

    def cpu_baseline(self, threads):
        from oracle import coracle
        coracle.set_threads(threads)
        n, T = self.n, self.T
        reps = 0
        t0 = time.perf_counter()
        while True:
            coracle.randomwalk_run(0, n, T, self.sigma)
            reps += 1
            if time.perf_counter() - t0 > 10.0 or reps >= 200:
                break
        dt = time.perf_counter() - t0
        return {"value": reps * n * T / dt, "unit": "agent-steps/s", "cores": threads,
                "kind": "port", "sample": f"{reps} full runs of N={n}, T={T} (C oracle, OpenMP)"}


WORKLOADS = {"randomwalk": RandomWalkBench}
DEFAULT_WORKLOAD = "randomwalk"


def _flush_l2(buf):
    buf.add_(1)


def run_ours(args):
    world, rank, local = _dist()
    if world > 1:
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    import jaxabm_gb300 as jx
    jx.set_verbose(False)
    jx.build()
    wl = WORKLOADS[args.workload](rank)
    stream = torch.cuda.current_stream()
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        wl.reset()
        wl.step(stream)
    torch.cuda.synchronize()

    # device-resident timed region: per-step events, L2 flushed between steps
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    dom = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    clocks = ClockSampler(local)
    clocks.start()
    _barrier(world)
    torch.cuda.synchronize()
    for i in range(args.steps):
        wl.reset()
        _flush_l2(flush)
        starts[i].record(stream)
        wl.step(stream, dom[i])
        ends[i].record(stream)
    torch.cuda.synchronize()
    _barrier(world)
    clk = clocks.stop()
    ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends)) / args.steps
    dom_ms = sum(a.elapsed_time(b) for a, b in dom) / args.steps
    ms = _max_over_ranks(ms, world)

    # end-to-end through the C ABI with host buffers
    for _ in range(2):
        wl.e2e_step(stream)
    torch.cuda.synchronize()
    _barrier(world)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        wl.e2e_step(stream)
    e1.record(stream)
    torch.cuda.synchronize()
    _barrier(world)
    e2e_ms = _max_over_ranks(e0.elapsed_time(e1) / args.steps, world)

    units = _sum_over_ranks(wl.units_per_step, world)
    value = units / (ms / 1e3)
    hbm_peak, peak_kind = _peaks()
    achieved = wl.units_per_step * wl.bytes_per_unit / (dom_ms / 1e3) / 1e9
    h2d, d2h = wl.e2e_bytes
    out = {
        "metric": "agent-steps/s", "value": value, "unit": "agent-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": wl.name, "l2": "flushed between timed steps (256 MiB write)",
                   "parallelism": f"replicas{world}"},
        "e2e": {"value": units / (e2e_ms / 1e3), "unit": "agent-steps/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": wl.launches_per_step * args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": None, "peak_kind": peak_kind},
        "clocks": clk,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = wl.cpu_baseline(os.cpu_count() or 1)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_reference(args):
    world, rank, _ = _dist()
    if rank != 0:
        return
    sys.path.insert(0, ROOT)
    from oracle import coracle
    cores = os.cpu_count() or 1
    coracle.set_threads(cores)
    wl_cls = WORKLOADS[args.workload]
    name = wl_cls.name
    times = []
    n, T = 10_000, 100
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        coracle.randomwalk_run(0, n, T)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
    ms = 1e3 * sum(times) / len(times)
    value = n * T / (ms / 1e3)
    out = {"metric": "agent-steps/s", "value": value, "unit": "agent-steps/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic", "impl": "reference",
           "config": {"workload": name, "parallelism": "host cores"},
           "cpu_baseline": {"value": value, "unit": "agent-steps/s", "cores": cores,
                            "kind": "port",
                            "sample": f"full N={n}, T={T} runs (C oracle, OpenMP)"},
           "e2e": {"value": value, "unit": "agent-steps/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
