"""SIR parity: bit-exact compartments and per-step S/I/R counts vs the C oracle, through the
C ABI (plain single-model run and batched instances) and the jx.Model API."""

import numpy as np
import pytest
import torch

from oracle import coracle, models

pytestmark = pytest.mark.gpu


def _graph(kind, n, seed=0):
    from jaxabm_gb300 import sir
    if kind == "ba":
        return sir.barabasi_albert(n, 4, seed)
    if kind == "ba2":
        return sir.barabasi_albert(n, 2, seed)
    if kind == "star":  # one hub of degree n-1 (warp-cooperative path), leaves of degree 1
        rp = np.zeros(n + 1, np.int32)
        rp[1] = n - 1
        rp[2:] = n - 1 + np.arange(1, n)
        col = np.concatenate([np.arange(1, n), np.zeros(n - 1)]).astype(np.int32)
        return rp, col
    if kind == "rr":
        return sir.random_regular(n, 16, seed)
    if kind == "clique":  # n = 64: every row 63 long, every agent a hub (count in hub_counts)
        # n = 63: every row 62 long, the longest row whose count lives in the agent's byte
        rp = (np.arange(n + 1) * (n - 1)).astype(np.int32)
        col = np.concatenate([np.delete(np.arange(n), i) for i in range(n)]).astype(np.int32)
        return rp, col
    raise ValueError(kind)


def _run_abi(rp, col, st0, seed, steps, beta, gamma):
    from jaxabm_gb300 import _dev, _lib
    import jaxabm_gb300.random as jr
    rng, _ = models.model_keys(seed, 1)
    ck = jr.keychain(_dev.keys_from_numpy(rng), steps, 1).reshape(steps, 2).contiguous()
    n = st0.size
    buf = torch.from_numpy(st0).cuda()
    drp = torch.from_numpy(rp).cuda()
    dcol = torch.from_numpy(col).cuda()
    counts = torch.empty((steps, 3), dtype=torch.int32, device="cuda")
    wsb = _lib.load().abm_sir_run_workspace_bytes(n, len(col))
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    _lib.call("abm_sir_run", _dev.ptr(drp), _dev.ptr(dcol), n, len(col), _dev.ptr(buf),
              _dev.ptr(ck), steps,
              beta, gamma, _dev.ptr(counts), _dev.ptr(ws), wsb, None)
    torch.cuda.synchronize()
    fin = buf.cpu().numpy()
    return fin, counts.cpu().numpy()


@pytest.mark.parametrize("kind,n,steps,beta,gamma,frac", [
    ("ba2", 200, 30, 0.3, 0.1, 0.01),
    ("ba", 5000, 60, 0.05, 0.1, 0.01),
    ("ba", 30000, 40, 0.02, 0.05, 0.3),   # many hubs with many infected neighbours
    ("star", 3000, 25, 0.02, 0.05, 0.01),
    ("clique", 64, 20, 0.01, 0.2, 0.01),
    ("clique", 64, 12, 0.002, 0.02, 0.6),
    ("clique", 63, 12, 0.002, 0.02, 0.6),  # byte counts near their 62 limit
    ("rr", 4096, 40, 0.1, 0.2, 0.01),
])
def test_sir_abi_bit_exact(cuda, kind, n, steps, beta, gamma, frac):
    from jaxabm_gb300 import sir
    rp, col = _graph(kind, n)
    st0 = sir.initial_states(n, frac, 1)
    fin, counts = _run_abi(rp, col, st0, 7, steps, beta, gamma)
    rng, _ = models.model_keys(7, 1)
    ref_st, ref_counts, _ = coracle.sir_run(rp, col, st0, rng, steps, beta, gamma)
    assert np.array_equal(fin, ref_st)
    assert np.array_equal(counts, ref_counts)


def test_sir_full_config_bit_exact(cuda):
    """N = 2^20 Barabasi-Albert (m=4), 0.1% infected, beta 0.05, gamma 0.1, 365 steps."""
    from jaxabm_gb300 import sir
    n = 1 << 20
    rp, col = sir.barabasi_albert(n, 4, 0)
    st0 = sir.initial_states(n, 0.001, 0)
    fin, counts = _run_abi(rp, col, st0, 0, 365, 0.05, 0.1)
    rng, _ = models.model_keys(0, 1)
    ref_st, ref_counts, _ = coracle.sir_run(rp, col, st0, rng, 365, 0.05, 0.1)
    assert np.array_equal(counts, ref_counts)
    assert np.array_equal(fin, ref_st)
    # size-independent properties: conservation and monotone R
    assert np.all(counts.sum(axis=1) == n)
    assert np.all(np.diff(counts[:, 2]) >= 0) and np.all(np.diff(counts[:, 0]) <= 0)


def test_sir_model_api(cuda):
    import jaxabm_gb300 as jx
    from jaxabm_gb300 import sir
    n = 20_000
    model = jx.SIRModel({"n": n, "steps": 50, "seed": 3, "beta": 0.08, "gamma": 0.15})
    res = model.run()
    rp, col = sir.barabasi_albert(n, 4, 3)
    st0 = sir.initial_states(n, 0.001, 3)
    rng, _ = models.model_keys(3, 1)
    ref_st, ref_counts, _ = coracle.sir_run(rp, col, st0, rng, 50, 0.08, 0.15)
    assert np.array_equal(np.array([res["S"], res["I"], res["R"]]).T, ref_counts)
    assert np.array_equal(res["agents.people.state"], ref_st)
    # select the infected through the warp-ballot compaction
    inf = model.agents.select(lambda s: s["state"] == 1)
    assert len(inf) == int((ref_st == 1).sum())


@pytest.mark.parametrize("use_graph", [False, True])
@pytest.mark.parametrize("path", ["resident", "grid"])
def test_sir_batched_equals_alone(cuda, use_graph, path):
    """Each instance of a batch is bit-identical to the instance run alone, on both paths."""
    from jaxabm_gb300 import ensemble, sir
    sizes = [300, 1000, 4097, 257, 256, 70_000]
    seeds = [11, 12, 13, 14, 15, 16]
    betas = [0.2, 0.05, 0.1, 0.15, 0.01, 0.06]
    gammas = [0.05, 0.1, 0.3, 0.2, 0.1, 0.08]
    graphs = [sir.barabasi_albert(n, 4, s) for n, s in zip(sizes, seeds)]
    inits = [sir.initial_states(n, 0.002, s) for n, s in zip(sizes, seeds)]
    steps = 45
    b = ensemble.SIRBatch(graphs, inits, betas, gammas, seeds, steps,
                          resident=(path == "resident"))
    assert b.mode == path
    b.run(use_graph=use_graph)
    torch.cuda.synchronize()
    b.check()
    for i in range(len(sizes)):
        rng, _ = models.model_keys(seeds[i], 1)
        ref_st, ref_counts, ref_rng = coracle.sir_run(graphs[i][0], graphs[i][1], inits[i], rng,
                                                      steps, betas[i], gammas[i])
        assert np.array_equal(b.counts_of(i).cpu().numpy(), ref_counts), i
        assert np.array_equal(b.final_state(i).cpu().numpy(), ref_st), i
        d = b.desc[i].cpu().numpy().view(np.uint32)
        assert np.array_equal(d[ensemble.RNG_WORD:ensemble.RNG_WORD + 2], ref_rng)
    # replay after reset reproduces the run
    c0 = b.counts.clone()
    b.reset()
    b.run(use_graph=use_graph)
    torch.cuda.synchronize()
    assert torch.equal(c0, b.counts)


def test_sir_bad_args(cuda):
    from jaxabm_gb300 import _lib
    L = _lib.load()
    assert L.abm_sir_steps(None, 1, None, 0, None, 1, 0, None, 0, None) == _lib.ABM_ERR_BADARG
    assert L.abm_sir_run(None, None, 10, 0, None, None, 1, 0.1, 0.1, None, None, 0, None) == \
        _lib.ABM_ERR_BADARG


def test_sir_batch_run_matches_serial(cuda):
    """SIRModel.batch_run runs every combination and repetition in one batched launch
    sequence; each result equals the same model run alone (the reference's serial loop)."""
    import jaxabm_gb300 as jx
    base = {"n": 3000, "steps": 30, "m": 3}
    model = jx.SIRModel(dict(base), seed=5)
    res = model.batch_run({"beta": [0.05, 0.2], "gamma": [0.1, 0.3]}, repetitions=2)
    assert len(res) == 4 and all(len(v) == 2 for v in res.values())
    for (beta, gamma), runs in res.items():
        for r, got in enumerate(runs):
            p = dict(base, beta=beta, gamma=gamma)
            ref = jx.SIRModel(p, seed=5 + r).run()
            for key in ("S", "I", "R"):
                assert list(got[key]) == list(ref[key]), (beta, gamma, r, key)
            assert np.array_equal(got["agents.people.state"], ref["agents.people.state"])


def test_sir_repack_is_idempotent(cuda):
    """Packing a batch again (its columns already carry hub tags) gives the same words,
    hub counts and results; a graph with hubs (BA m=8, n=3000) exercises the tags."""
    from jaxabm_gb300 import ensemble, sir
    sizes, seeds = [3000, 1500], [21, 22]
    graphs = [sir.barabasi_albert(n, 8, s) for n, s in zip(sizes, seeds)]
    inits = [sir.initial_states(n, 0.01, s) for n, s in zip(sizes, seeds)]
    b = ensemble.SIRBatch(graphs, inits, [0.08, 0.15], [0.1, 0.2], seeds, 25)
    w0, h0, c0 = b.words.clone(), b.hub_counts.clone(), b.col.clone()
    assert (c0 < 0).any()  # some columns point at hubs (bit 31 set)
    b.pack()
    torch.cuda.synchronize()
    assert torch.equal(b.words, w0) and torch.equal(b.col, c0)
    hubs = (w0 >> 2) == 63
    assert torch.equal(b.hub_counts[hubs.nonzero()], h0[hubs.nonzero()])
    b.run()
    torch.cuda.synchronize()
    for i in range(2):
        rng, _ = models.model_keys(seeds[i], 1)
        ref_st, ref_counts, _ = coracle.sir_run(graphs[i][0], graphs[i][1], inits[i], rng, 25,
                                                [0.08, 0.15][i], [0.1, 0.2][i])
        assert np.array_equal(b.counts_of(i).cpu().numpy(), ref_counts)
        assert np.array_equal(b.final_state(i).cpu().numpy(), ref_st)


def test_sir_resident_edge_cases_match_oracle(cuda):
    """Resident path on instances that stress it: hubs (BA m=8, a star, a 64-clique where
    every agent is a hub), rows longer than 96 slots (draw-first), tiny instances (5 and 17
    agents: one partial chunk), an instance without infected agents, and stepping in three
    calls (10 + 7 + the rest).  Compartments, counts, key chains and the 2-bit compartment
    copy equal the oracle's."""
    from jaxabm_gb300 import ensemble, sir
    graphs = [sir.barabasi_albert(3000, 8, 1), _graph("star", 700), _graph("clique", 64),
              sir.barabasi_albert(5, 2, 3), sir.barabasi_albert(17, 4, 4),
              sir.barabasi_albert(2000, 4, 5), sir.barabasi_albert(40_000, 4, 6)]
    n = [len(rp) - 1 for rp, _ in graphs]
    fr = [0.01, 0.02, 0.1, 0.4, 0.2, 0.0, 0.001]
    inits = [sir.initial_states(k, f, 30 + i) if f > 0 else np.zeros(k, np.int8)
             for i, (k, f) in enumerate(zip(n, fr))]
    seeds = [40 + i for i in range(len(graphs))]
    betas = [0.05, 0.3, 0.02, 0.5, 0.2, 0.1, 0.07]
    gammas = [0.1, 0.2, 0.05, 0.3, 0.1, 0.1, 0.1]
    steps = 60
    b = ensemble.SIRBatch(graphs, inits, betas, gammas, seeds, steps, resident=True)
    b.launch(10)
    b.launch(7)
    b.launch(steps)
    torch.cuda.synchronize()
    b.check()
    d = b.desc.cpu().numpy().view(ensemble.INSTANCE_DTYPE).reshape(-1)
    for i in range(len(graphs)):
        rng, _ = models.model_keys(seeds[i], 1)
        ref_st, ref_counts, ref_rng = coracle.sir_run(graphs[i][0], graphs[i][1], inits[i], rng,
                                                      steps, betas[i], gammas[i])
        assert np.array_equal(b.counts_of(i).cpu().numpy(), ref_counts), i
        assert np.array_equal(b.final_state(i).cpu().numpy(), ref_st), i
        assert np.array_equal(d["rng"][i], ref_rng), i
        assert d["t"][i] == steps
        w = b._offsets[2]
        comp = b.comp[w[i] // 16:w[i + 1] // 16].cpu().numpy().view(np.uint32)
        unpacked = (comp[:, None] >> (2 * np.arange(16, dtype=np.uint32))) & 3
        assert np.array_equal(unpacked.reshape(-1)[:n[i]], ref_st.astype(np.uint32)), i


def test_sir_resident_rejects_oversize_instance(cuda):
    """An instance larger than the resident call's max_agents is left untouched and sets the
    status word; the host picks the grid path for batches that do not fit."""
    from jaxabm_gb300 import _dev, _lib, ensemble, sir
    graphs = [sir.barabasi_albert(3000, 4, 1), sir.barabasi_albert(800, 4, 2)]
    inits = [sir.initial_states(3000, 0.01, 1), sir.initial_states(800, 0.01, 2)]
    b = ensemble.SIRBatch(graphs, inits, [0.1, 0.1], [0.1, 0.1], [1, 2], 20, resident=True)
    L = _lib.load()
    grid = L.abm_sir_resident_grid(1000)
    assert grid > 0
    scratch = torch.empty(L.abm_sir_resident_scratch_bytes(1000, grid), dtype=torch.uint8,
                          device=cuda)
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    _lib.call("abm_sir_steps_resident", _dev.ptr(b.desc), 2, None, 1000, 20, grid, None, None,
              _dev.ptr(scratch), scratch.numel(), _dev.ptr(status), None)
    torch.cuda.synchronize()
    assert int(status.item()) == 1
    d = b.desc.cpu().numpy().view(ensemble.INSTANCE_DTYPE).reshape(-1)
    assert d["t"][0] == 0 and d["t"][1] == 20
    with pytest.raises(_lib.AbmError):
        _lib.call("abm_sir_steps_resident", _dev.ptr(b.desc), 2, None, 1000, 20, grid, None,
                  None, _dev.ptr(scratch), 16, _dev.ptr(status), None)
    big = L.abm_sir_resident_max_agents() + 16
    g = [sir.barabasi_albert(big, 2, 3)]
    b2 = ensemble.SIRBatch(g, [sir.initial_states(big, 0.001, 3)], [0.1], [0.1], [3], 2)
    assert b2.mode == "grid" and not b2.resident_ok
    with pytest.raises(ValueError):
        ensemble.SIRBatch(g, [sir.initial_states(big, 0.001, 3)], [0.1], [0.1], [3], 2,
                          resident=True)


def test_sir_resident_builds_words_from_untagged_inputs(cuda):
    """The resident kernel builds each instance's words at step 0 from the int8
    compartments, so inputs copied in from the host (columns without hub tags, no pack)
    give the oracle's results; an out-of-range column (replaced by a self-loop) or
    compartment (stored as R) makes run() raise, each with its own code and message."""
    from jaxabm_gb300 import _lib
    from jaxabm_gb300 import ensemble, sir
    graphs = [sir.barabasi_albert(3000, 8, 7), _graph("star", 500), sir.barabasi_albert(900, 4, 8)]
    n = [len(rp) - 1 for rp, _ in graphs]
    inits = [sir.initial_states(k, 0.02, 50 + i) for i, k in enumerate(n)]
    seeds, betas, gammas, steps = [61, 62, 63], [0.06, 0.3, 0.1], [0.1, 0.2, 0.15], 40
    b = ensemble.SIRBatch(graphs, inits, betas, gammas, seeds, steps, resident=True)
    h_rp = torch.from_numpy(np.concatenate([rp for rp, _ in graphs]).astype(np.int32))
    h_col = torch.from_numpy(np.concatenate([c for _, c in graphs]).astype(np.int32))
    h_st = torch.from_numpy(b.h_state0.copy())
    assert (b.col.cpu() < 0).any()  # the packed columns carry hub tags; the host copy does not
    b.load_host(h_rp, h_col, h_st)
    b.run()
    torch.cuda.synchronize()
    b.check()
    for i in range(3):
        rng, _ = models.model_keys(seeds[i], 1)
        ref_st, ref_counts, _ = coracle.sir_run(graphs[i][0], graphs[i][1], inits[i], rng, steps,
                                                betas[i], gammas[i])
        assert np.array_equal(b.counts_of(i).cpu().numpy(), ref_counts), i
        assert np.array_equal(b.final_state(i).cpu().numpy(), ref_st), i
    bad_col = h_col.clone()
    bad_col[5] = 10_000_000
    bad_col[7] = -3
    b.load_host(h_rp, bad_col, h_st)
    with pytest.raises(_lib.AbmError, match="CSR column points outside") as err:
        b.run()
    assert err.value.status == _lib.ABM_ERR_BOUNDS
    assert b.status() == ensemble.STATUS_BAD_COLUMN
    b.reset()
    assert b.status() == 0
    bad_st = h_st.clone()
    bad_st[3] = 7
    b.load_host(h_rp, h_col, bad_st)
    with pytest.raises(_lib.AbmError, match="compartment is outside 0..2") as err:
        b.run()
    assert err.value.status == _lib.ABM_ERR_BADARG
    assert b.status() == ensemble.STATUS_BAD_COMPARTMENT
    # good inputs again: the status is cleared and the run equals the oracle
    b.load_host(h_rp, h_col, h_st)
    b.reset()
    b.run()
    for i in range(3):
        rng, _ = models.model_keys(seeds[i], 1)
        _, ref_counts, _ = coracle.sir_run(graphs[i][0], graphs[i][1], inits[i], rng, steps,
                                           betas[i], gammas[i])
        assert np.array_equal(b.counts_of(i).cpu().numpy(), ref_counts), i


def test_sir_grid_path_reports_bad_inputs(cuda):
    """The grid path's pack reports a bad column and a bad compartment of loaded inputs;
    run() raises with the matching code, and the construction rejects both up front."""
    from jaxabm_gb300 import _lib, ensemble, sir
    graphs = [sir.barabasi_albert(800, 4, 3), sir.barabasi_albert(500, 4, 4)]
    inits = [sir.initial_states(800, 0.02, 1), sir.initial_states(500, 0.02, 2)]
    b = ensemble.SIRBatch(graphs, inits, [0.1, 0.1], [0.1, 0.1], [1, 2], 10, resident=False)
    h_rp = torch.from_numpy(np.concatenate([rp for rp, _ in graphs]).astype(np.int32))
    h_col = torch.from_numpy(np.concatenate([c for _, c in graphs]).astype(np.int32))
    bad_col = h_col.clone()
    bad_col[-1] = 500  # the second instance has agents 0..499
    b.load_host(h_rp, bad_col, torch.from_numpy(b.h_state0.copy()))
    with pytest.raises(_lib.AbmError) as err:
        b.run()
    assert err.value.status == _lib.ABM_ERR_BOUNDS
    bad = [inits[0].copy(), inits[1]]
    bad[0][10] = -1
    with pytest.raises(ValueError, match="compartments"):
        ensemble.SIRBatch(graphs, bad, [0.1, 0.1], [0.1, 0.1], [1, 2], 10, resident=False)
    g2 = [graphs[0], (graphs[1][0], np.where(graphs[1][1] == 3, 9999, graphs[1][1]))]
    with pytest.raises(ValueError, match="CSR column"):
        ensemble.SIRBatch(g2, inits, [0.1, 0.1], [0.1, 0.1], [1, 2], 10, resident=False)


@pytest.mark.parametrize("path", ["resident", "grid"])
def test_sir_reset_after_load_host_keeps_loaded_inputs(cuda, path):
    """Inputs loaded from the host (other infected agents, the same S/I/R totals) are what
    a reset() rewinds to, on both paths: the run after the reset equals the oracle on the
    loaded compartments."""
    from jaxabm_gb300 import ensemble, sir
    sizes, seeds = [2500, 900], [71, 72]
    graphs = [sir.barabasi_albert(k, 4, s) for k, s in zip(sizes, seeds)]
    first = [sir.initial_states(k, 0.01, s) for k, s in zip(sizes, seeds)]
    other = [sir.initial_states(k, 0.01, s + 100) for k, s in zip(sizes, seeds)]
    assert all((a == 1).sum() == (b == 1).sum() for a, b in zip(first, other))
    betas, gammas, steps = [0.1, 0.15], [0.1, 0.2], 30
    b = ensemble.SIRBatch(graphs, first, betas, gammas, seeds, steps,
                          resident=(path == "resident"))
    w_off = b._offsets[2]
    h_st = np.zeros(int(w_off[-1]), dtype=np.int8)
    for i, st in enumerate(other):
        h_st[w_off[i]:w_off[i] + len(st)] = st
    h_rp = torch.from_numpy(np.concatenate([rp for rp, _ in graphs]).astype(np.int32))
    h_col = torch.from_numpy(np.concatenate([c for _, c in graphs]).astype(np.int32))
    b.load_host(h_rp, h_col, torch.from_numpy(h_st))
    b.run()
    b.reset()
    b.run()
    torch.cuda.synchronize()
    b.check()
    for i in range(2):
        rng, _ = models.model_keys(seeds[i], 1)
        ref_st, ref_counts, _ = coracle.sir_run(graphs[i][0], graphs[i][1], other[i], rng, steps,
                                                betas[i], gammas[i])
        assert np.array_equal(b.counts_of(i).cpu().numpy(), ref_counts), (path, i)
        assert np.array_equal(b.final_state(i).cpu().numpy(), ref_st), (path, i)


@pytest.mark.parametrize("path", ["resident", "grid"])
def test_sir_headline_ensemble_slice_matches_oracle(cuda, path):
    """Members of the 4,096-instance benchmark ensemble (the first 64 and the largest, member
    2461 with 99,619 agents; BA m=4, Sobol (beta, gamma), 365 steps): the GPU runs them as
    one batch from the package's inputs, the C oracle runs each alone from the oracle's own
    inputs; every per-step S/I/R count and every final compartment is bit-identical."""
    from jaxabm_gb300 import ensemble
    from oracle import workloads
    spec = ensemble.ensemble_spec(4096)
    idx = list(range(64)) + [int(np.argmax(spec["n"]))]
    sub = {k: v[idx] for k, v in spec.items()}
    graphs, inits = ensemble.build_instances(sub)
    b = ensemble.SIRBatch(graphs, inits, sub["beta"], sub["gamma"], sub["seed"], 365,
                          resident=(path == "resident"))
    assert b.mode == path
    b.run()
    counts = b.counts.reshape(len(idx), 365, 3).cpu().numpy()
    ospec = workloads.sir_ensemble_spec(4096)
    members = workloads.sir_members(ospec, idx)
    for k, i in enumerate(idx):
        rp, col, st0 = members[k]
        assert np.array_equal(rp, graphs[k][0]) and np.array_equal(st0, inits[k])
        rng, _ = models.model_keys(int(ospec["seed"][i]), 1)
        ref_st, ref_counts, _ = coracle.sir_run(rp, col, st0, rng, 365, float(ospec["beta"][i]),
                                                float(ospec["gamma"][i]))
        assert np.array_equal(counts[k], ref_counts), (path, i)
        assert np.array_equal(b.final_state(k).cpu().numpy(), ref_st), (path, i)
    assert int(b.n.max()) == int(spec["n"].max()) == 99_619


@pytest.mark.parametrize("chunks", [1, 3, 8])
def test_sir_run_from_host_overlapped_equals_oracle(cuda, chunks):
    """run_from_host: index ranges copied on one stream while earlier ranges run, each as
    its own resident launch; every member's counts (copied back per range) and final
    compartments equal its own oracle run, for any number of ranges, and the batch's
    replay afterwards gives the same."""
    from jaxabm_gb300 import ensemble, sir
    sizes = [9000, 6000, 4000, 2500, 1500, 900, 700, 300, 120, 64, 40]
    seeds = list(range(31, 31 + len(sizes)))
    graphs = [sir.barabasi_albert(n, 4, s) for n, s in zip(sizes, seeds)]
    inits = [sir.initial_states(n, 0.01, s + 7) for n, s in zip(sizes, seeds)]
    betas = [0.04 + 0.01 * i for i in range(len(sizes))]
    gammas = [0.08 + 0.005 * i for i in range(len(sizes))]
    steps = 40
    b = ensemble.SIRBatch(graphs, inits, betas, gammas, seeds, steps, resident=True)
    h_rp = torch.from_numpy(b.row_ptr.cpu().numpy()).pin_memory()
    h_col = torch.from_numpy(b.col.cpu().numpy()).pin_memory()
    h_st = torch.from_numpy(b.h_state0).pin_memory()
    h_counts = torch.zeros(b.counts.numel(), dtype=torch.int32).pin_memory()
    for _ in range(2):  # twice: the second run starts over from the loaded inputs
        b.run_from_host(h_rp, h_col, h_st, h_counts, chunks=chunks)
        torch.cuda.synchronize()
        b.check()
        hc = h_counts.numpy().reshape(len(sizes), steps, 3)
        for i in range(len(sizes)):
            rng, _ = models.model_keys(seeds[i], 1)
            ref_st, ref_counts, _ = coracle.sir_run(graphs[i][0], graphs[i][1], inits[i], rng,
                                                    steps, betas[i], gammas[i])
            assert np.array_equal(hc[i], ref_counts), (chunks, i)
            assert np.array_equal(b.final_state(i).cpu().numpy(), ref_st), (chunks, i)
    b.reset()
    b.run()
    assert np.array_equal(b.counts.cpu().numpy(), h_counts.numpy())


def test_sir_run_from_host_needs_the_resident_path(cuda):
    from jaxabm_gb300 import ensemble, sir
    g = [sir.barabasi_albert(500, 4, 1)]
    st = [sir.initial_states(500, 0.02, 1)]
    b = ensemble.SIRBatch(g, st, [0.1], [0.1], [1], 10, resident=False)
    with pytest.raises(ValueError):
        b.run_from_host(torch.zeros(1), torch.zeros(1), torch.zeros(1))


def test_sir_resident_member_order_never_changes_results(cuda):
    """The resident kernel takes members in the batch's order (longest predicted time
    first); any other order -- reversed, shuffled -- gives bit-identical counts and final
    compartments, since each member runs alone on its CTA."""
    from jaxabm_gb300 import ensemble
    spec = ensemble.ensemble_spec(4096)
    idx = list(range(0, 4096, 97))
    sub = {k: v[idx] for k, v in spec.items()}
    graphs, inits = ensemble.build_instances(sub)
    b = ensemble.SIRBatch(graphs, inits, sub["beta"], sub["gamma"], sub["seed"], 365,
                          resident=True)
    order0 = b.order.cpu().numpy()
    assert np.array_equal(order0, np.argsort(-b.cost, kind="stable"))
    b.run()
    ref_counts = b.counts.cpu().numpy().copy()
    ref_states = [b.final_state(k).cpu().numpy().copy() for k in range(len(idx))]
    rs = np.random.RandomState(5)
    for order in (order0[::-1], rs.permutation(len(idx))):
        b.order.copy_(torch.from_numpy(np.ascontiguousarray(order, dtype=np.int32)))
        b.reset()
        b.run()
        assert np.array_equal(b.counts.cpu().numpy(), ref_counts)
        for k in range(len(idx)):
            assert np.array_equal(b.final_state(k).cpu().numpy(), ref_states[k])
