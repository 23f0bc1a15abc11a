"""Autotuner bookkeeping (CPU) and result invariance under launch choices (GPU)."""

import numpy as np
import pytest
import torch

from jaxabm_gb300 import autotune


def test_cache_roundtrip(tmp_path):
    p = str(tmp_path / "sub" / "tune.json")
    assert autotune.load_cache(p) == {}
    autotune.store_cache(p, "k1", {"grids": [1, 2, 3]})
    autotune.store_cache(p, "k2", {"grids": [4, 5, 6]})
    c = autotune.load_cache(p)
    assert c["k1"]["grids"] == [1, 2, 3] and c["k2"]["grids"] == [4, 5, 6]
    (tmp_path / "bad.json").write_text("{not json")
    assert autotune.load_cache(str(tmp_path / "bad.json")) == {}


def test_workload_key_buckets():
    a = autotune.workload_key("GB300", 152, 4096, 87_421_729, 365)
    b = autotune.workload_key("GB300", 152, 4000, 80_000_000, 365)
    c = autotune.workload_key("GB300", 152, 4096, 87_421_729, 200)
    assert a == b and a != c


def test_candidate_grids():
    g = autotune.candidate_grids((760, 912, 1216), 152, 1)
    assert 912 in g and 152 in g and 1216 in g and g == sorted(g)


@pytest.mark.gpu
def test_results_identical_under_any_launch(cuda, tmp_path):
    from jaxabm_gb300 import ensemble, sir
    sizes, seeds = [5000, 1200, 20_000], [1, 2, 3]
    graphs = [sir.barabasi_albert(n, 4, s) for n, s in zip(sizes, seeds)]
    inits = [sir.initial_states(n, 0.002, s) for n, s in zip(sizes, seeds)]
    b = ensemble.SIRBatch(graphs, inits, [0.1, 0.2, 0.05], [0.1, 0.1, 0.2], seeds, 40)
    assert b.mode == "resident"
    b.run()
    torch.cuda.synchronize()
    results = [(b.counts.cpu().numpy().copy(), [b.final_state(i).cpu().numpy() for i in range(3)])]
    b.set_mode("grid")
    for cfg in (None, (1, 1, 1), (152, 304, 152 * 8), (7, 3, 5)):
        b.set_launch(cfg)
        b.reset()
        b.run()
        torch.cuda.synchronize()
        results.append((b.counts.cpu().numpy().copy(),
                        [b.final_state(i).cpu().numpy() for i in range(3)]))
    for c, st in results[1:]:
        assert np.array_equal(c, results[0][0])
        for a, r in zip(st, results[0][1]):
            assert np.array_equal(a, r)
    cache = str(tmp_path / "tune.json")
    cfg = autotune.tune_sir_batch(b, cache_path=cache)
    assert len(cfg) == 3 and all(v > 0 for v in cfg)
    entry = list(autotune.load_cache(cache).values())[0]
    assert entry["mode"] in ("resident", "grid") and b.mode == entry["mode"]
    b.run()
    torch.cuda.synchronize()
    assert np.array_equal(b.counts.cpu().numpy(), results[0][0])
    # second call is served from the cache
    assert autotune.tune_sir_batch(b, cache_path=cache) == cfg
