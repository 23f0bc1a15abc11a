"""Project-written autotuner for the launch schedules of the batched SIR step.

It first times the resident path (one CTA per instance, all steps in one launch) when the
instances fit it, then tunes the per-step grid kernels, and keeps the faster of the two.
The per-step kernels (sweep, candidates, push) run over persistent grids whose best size
depends on the GPU and the workload (number of instances, agents, how much of a step is
random gathering).  The tuner measures CUDA-graph replays of the actual batch for
candidate grid sizes by coordinate descent (one kernel at a time, the others fixed),
keeps the fastest, and caches the choice in a JSON file keyed by GPU and workload.

Results never depend on the choice: the model is integer-valued and every kernel's work
is order-free (commutative integer atomics, per-agent decisions), so any configuration
produces bit-identical compartments and counts (tests/test_autotune.py,
test_results_identical_under_any_launch).
"""

import json
import math
import os
import time

import torch

from . import ensemble

PER_SM_CHOICES = (1, 2, 3, 4, 6, 8)
KERNELS = ("sweep", "candidates", "push")


def default_cache_path():
    return os.environ.get(
        "JAXABM_GB300_AUTOTUNE_CACHE",
        os.path.join(os.path.expanduser("~"), ".cache", "jaxabm_gb300", "autotune.json"))


def _bucket(x):
    """Power-of-two bucket, so similar workloads share a cache entry."""
    return 1 << max(0, int(math.ceil(math.log2(max(int(x), 1)))))


def workload_key(gpu_name, sm_count, instances, agents, steps):
    return (f"{gpu_name}|sms={sm_count}|sir|instances~{_bucket(instances)}"
            f"|agents~{_bucket(agents)}|steps={int(steps)}")


def load_cache(path):
    if not os.path.exists(path):
        return {}
    try:
        with open(path) as f:
            data = json.load(f)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def store_cache(path, key, entry):
    data = load_cache(path)
    data[key] = entry
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def candidate_grids(default, sm_count, kernel_index):
    """Grid sizes to try for one kernel: multiples of the SM count up to 8 CTAs per SM,
    plus the default."""
    out = {int(default[kernel_index])}
    for p in PER_SM_CHOICES:
        out.add(p * sm_count)
    return sorted(out)


def time_replay(batch, reps=1, warmup=1):
    """Mean milliseconds of a full replay of ``batch`` with its current launch config."""
    batch.capture(batch.steps)
    for _ in range(warmup):
        batch.reset()
        batch.replay()
    torch.cuda.synchronize()
    total = 0.0
    for _ in range(reps):
        batch.reset()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        batch.replay()
        e.record()
        e.synchronize()
        total += s.elapsed_time(e)
    return total / reps


def tune_sir_batch(batch, cache_path=None, reps=1, force=False, log=None):
    """Pick (sweep, candidates, push) grid sizes for ``batch``; applies and returns them.

    The cached choice is used when present (unless ``force``).  The batch is left reset
    with a fresh graph for the chosen configuration."""
    cache_path = cache_path or default_cache_path()
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    key = workload_key(props.name, props.multi_processor_count, batch.k, int(batch.n.sum()),
                       batch.steps)
    if not force:
        hit = load_cache(cache_path).get(key)
        if hit and "grids" in hit:
            batch.set_launch(hit["grids"])
            if batch.resident_ok:
                batch.set_mode(hit.get("mode", "grid"))
            return tuple(hit["grids"])
    resident_ms = None
    if batch.resident_ok:
        batch.set_mode("resident")
        resident_ms = time_replay(batch, reps)
        if log:
            log(f"autotune resident: {resident_ms:.2f} ms")
        batch.set_mode("grid")
    default = ensemble.default_launch()
    best = list(default)
    batch.set_launch(best)
    best_ms = time_replay(batch, reps)
    tried = {tuple(best): best_ms}
    t0 = time.perf_counter()
    for ki in range(len(KERNELS)):
        for g in candidate_grids(default, props.multi_processor_count, ki):
            cfg = list(best)
            cfg[ki] = g
            if tuple(cfg) in tried:
                continue
            batch.set_launch(cfg)
            ms = time_replay(batch, reps)
            tried[tuple(cfg)] = ms
            if log:
                log(f"autotune {KERNELS[ki]}={g}: {ms:.2f} ms")
            if ms < best_ms:
                best, best_ms = cfg, ms
    batch.set_launch(best)
    mode = "resident" if resident_ms is not None and resident_ms <= best_ms else "grid"
    if batch.resident_ok:
        batch.set_mode(mode)
    batch.reset()
    store_cache(cache_path, key, {"grids": list(best), "ms": best_ms, "mode": mode,
                                  "resident_ms": resident_ms,
                                  "default": list(default), "default_ms": tried[tuple(default)],
                                  "configs_tried": len(tried),
                                  "seconds": time.perf_counter() - t0})
    return tuple(best)
