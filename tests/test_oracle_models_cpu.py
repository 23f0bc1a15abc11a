"""The C oracle's SIR and Schelling (the GPU parity checkers) against independent, direct
NumPy statements of the rules (oracle/models.py) on small cases: bit-exact compartments,
positions, per-step counts and key chains.  No GPU."""

import numpy as np
import pytest

from oracle import coracle, models


def _ba(n, m, seed):
    """Small Barabasi-Albert-like graph (seeded, symmetric CSR) built here in NumPy."""
    rs = np.random.RandomState(seed)
    edges = set()
    for i in range(m, n):
        targets = rs.choice(i, size=min(m, i), replace=False)
        for j in targets:
            edges.add((i, int(j)))
    return _csr(n, edges)


def _csr(n, undirected):
    rows = [[] for _ in range(n)]
    for a, b in undirected:
        rows[a].append(b)
        rows[b].append(a)
    rp = np.zeros(n + 1, dtype=np.int32)
    rp[1:] = np.cumsum([len(r) for r in rows])
    col = np.array([c for r in rows for c in sorted(r)], dtype=np.int32)
    return rp, col


def _star(n):
    return _csr(n, {(0, i) for i in range(1, n)})


def _clique(n):
    return _csr(n, {(a, b) for a in range(n) for b in range(a + 1, n)})


CASES = [
    ("ba", lambda: _ba(80, 3, 1), 0.05, 0.2, 0.1, 25, 3),
    ("ba_dense", lambda: _ba(60, 6, 2), 0.1, 0.3, 0.15, 20, 4),
    ("star", lambda: _star(40), 0.1, 0.3, 0.1, 20, 5),
    ("clique64", lambda: _clique(64), 0.05, 0.05, 0.2, 15, 6),
    ("isolated", lambda: _csr(30, {(0, 1), (2, 3)}), 0.2, 0.5, 0.1, 10, 7),
]


@pytest.mark.parametrize("name,make,frac,beta,gamma,steps,seed", CASES,
                         ids=[c[0] for c in CASES])
def test_c_oracle_sir_equals_numpy_statement(name, make, frac, beta, gamma, steps, seed):
    rp, col = make()
    n = len(rp) - 1
    rs = np.random.RandomState(seed)
    st0 = np.zeros(n, dtype=np.int8)
    st0[rs.permutation(n)[:max(1, int(frac * n))]] = 1
    rng, _ = models.model_keys(seed, 1)
    ref_st, ref_counts, ref_rng = models.sir_run(rp, col, st0, rng, steps, beta, gamma)
    c_st, c_counts, c_rng = coracle.sir_run(rp, col, st0, rng, steps, beta, gamma)
    assert np.array_equal(c_counts, ref_counts)
    assert np.array_equal(c_st, ref_st)
    assert np.array_equal(c_rng, ref_rng)
    assert (ref_counts.sum(axis=1) == n).all()
    if name != "isolated":  # the epidemic spreads, so the comparison covers infections
        assert ref_counts[-1, 0] < (st0 == 0).sum()


@pytest.mark.parametrize("W,H,density,seed,steps", [(12, 10, 0.8, 1, 8), (9, 9, 0.5, 2, 10),
                                                   (16, 7, 0.9, 3, 6), (5, 5, 0.96, 4, 5)])
def test_c_oracle_schelling_equals_numpy_statement(W, H, density, seed, steps):
    """The C oracle's Schelling step (the GPU tests' checker) against the direct NumPy
    statement of the rule: positions and (unhappy, moved) per step, bit for bit."""
    rs = np.random.RandomState(seed)
    n = int(density * W * H)
    pos = rs.permutation(W * H)[:n].astype(np.int32)
    types = (np.arange(n) >= n // 2).astype(np.int8)
    rng, _ = models.model_keys(seed, 1)
    ck, _ = models.keychain(rng, steps, 1)
    ck = ck.reshape(steps, 2)
    ref_pos, ref_stats = models.schelling_run(pos, types, W, H, ck)
    c_pos, c_stats = coracle.schelling_run(pos, types, W, H, ck)
    assert np.array_equal(c_stats, ref_stats)
    assert np.array_equal(c_pos, ref_pos)
    assert ref_stats[:, 1].sum() > 0  # agents moved, so claims were compared


def test_golden_small_cases():
    """The committed small-case vectors (tests/golden/oracle_small_cases.npz, written by
    tests/golden/make_oracle_fixtures.py from the NumPy statements) are reproduced by the
    NumPy statements and by the C oracle."""
    import importlib.util
    import os
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    spec = importlib.util.spec_from_file_location("make_oracle_fixtures",
                                                  os.path.join(here, "make_oracle_fixtures.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    g = np.load(os.path.join(here, "oracle_small_cases.npz"))
    fresh = mk.cases()
    assert set(g.files) == set(fresh)
    for k in g.files:
        if k.startswith("rw_"):  # floating point: libm may differ across machines
            np.testing.assert_allclose(fresh[k], g[k], rtol=1e-6, atol=1e-6, err_msg=k)
        else:
            assert np.array_equal(g[k], fresh[k]), k
    rng, _ = models.model_keys(int(g["sir_seed"]), 1)
    st, counts, r = coracle.sir_run(g["sir_row_ptr"], g["sir_col"], g["sir_state0"], rng,
                                    int(g["sir_steps"]), float(g["sir_beta"]),
                                    float(g["sir_gamma"]))
    assert np.array_equal(st, g["sir_state"]) and np.array_equal(counts, g["sir_counts"])
    assert np.array_equal(r, g["sir_rng"])
    assert counts[-1, 0] < (g["sir_state0"] == 0).sum()
    pos, stats = coracle.schelling_run(g["sch_pos0"], g["sch_types"], int(g["sch_W"]),
                                       int(g["sch_H"]), g["sch_coll_keys"])
    assert np.array_equal(pos, g["sch_pos"]) and np.array_equal(stats, g["sch_stats"])
    rw = coracle.randomwalk_run(0, 100, 5)
    d = np.abs(rw["x"].astype(np.float64) - g["rw_x"])
    assert np.minimum(d, 1 - d).max() < 1e-6
    np.testing.assert_allclose(rw["means"], g["rw_means"], rtol=1e-6)
