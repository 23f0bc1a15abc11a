"""Host-side network builders and ensemble specification (CPU only)."""

import numpy as np
import pytest
import scipy.sparse as sp

from jaxabm_gb300 import ensemble, sir


def _check_simple_symmetric(rp, col):
    n = len(rp) - 1
    a = sp.csr_matrix((np.ones(col.size, np.int32), col, rp), shape=(n, n))
    assert (a != a.T).nnz == 0
    assert a.diagonal().sum() == 0
    assert a.max() == 1
    for i in range(0, n, max(1, n // 50)):
        row = col[rp[i]:rp[i + 1]]
        assert np.all(np.diff(row) > 0)


@pytest.mark.parametrize("n,m", [(10, 2), (1000, 4), (50_000, 4), (3000, 7)])
def test_barabasi_albert(lib, n, m):
    rp, col = sir.barabasi_albert(n, m, 5)
    assert col.size == 2 * m * (n - m)
    _check_simple_symmetric(rp, col)
    deg = np.diff(rp)
    assert deg.min() >= 1 and deg[m + 1:].min() >= m
    # deterministic in the seed
    rp2, col2 = sir.barabasi_albert(n, m, 5)
    assert np.array_equal(col, col2)
    assert not np.array_equal(col, sir.barabasi_albert(n, m, 6)[1])


def test_barabasi_albert_bad_sizes(lib):
    with pytest.raises(ValueError):
        sir.barabasi_albert(3, 4)


@pytest.mark.parametrize("n,d", [(40, 4), (1000, 16), (1 << 16, 16)])
def test_random_regular(lib, n, d):
    rp, col = sir.random_regular(n, d, 3)
    assert np.all(np.diff(rp) == d)
    _check_simple_symmetric(rp, col)


def test_initial_states():
    st = sir.initial_states(1 << 20, 0.001, 0)
    assert (st == 1).sum() == 1048 and (st == 0).sum() == (1 << 20) - 1048
    assert (sir.initial_states(500, 0.001, 0) == 1).sum() == 1


def test_instance_layout(lib):
    ensemble.check_layout()
    assert ensemble.INSTANCE_DTYPE.itemsize == lib.abm_sir_instance_size()


def test_tiles_cover_instance(lib):
    assert ensemble.TILE == lib.abm_sir_tile_agents()
    t = ensemble.tiles_for(3, 20000)
    assert t[0].tolist() == [3, 0, 8192, 0] and t[-1].tolist() == [3, 16384, 20000, 0]
    assert (t[:, 2] - t[:, 1]).sum() == 20000
    assert ensemble.tiles_for(0, 1000).tolist() == [[0, 0, 1000, 0]]


def test_ensemble_spec():
    s = ensemble.ensemble_spec(4096)
    assert s["n"].min() >= 1000 and s["n"].max() <= 100_000
    assert 15_000 < s["n"].mean() < 28_000
    assert s["beta"].min() >= 0.01 and s["beta"].max() <= 0.2
    assert s["gamma"].min() >= 0.05 and s["gamma"].max() <= 0.3
    assert s["arrival_s"][0] == 0.0 and np.all(np.diff(s["arrival_s"]) >= 0)
    assert 15.0 < s["arrival_s"][-1] < 26.0
    assert np.array_equal(s["n"], ensemble.ensemble_spec(4096)["n"])


def test_chunk_ranges_cover_in_order():
    """The index ranges of SIRBatch.run_from_host: contiguous, in order, each non-empty,
    covering every instance once; the first holds about 1/2^(chunks-1) of the bytes."""
    from jaxabm_gb300.ensemble import chunk_ranges
    rng = np.random.default_rng(3)
    for k, chunks in [(1, 8), (3, 8), (11, 3), (4096, 8), (50, 1), (7, 7)]:
        nbytes = np.sort(rng.integers(100, 10_000, k))[::-1]
        r = chunk_ranges(nbytes, chunks)
        assert r[0][0] == 0 and r[-1][1] == k
        assert all(a < b for a, b in r)
        assert all(r[i][1] == r[i + 1][0] for i in range(len(r) - 1))
        assert len(r) <= max(1, chunks)
        if k >= 4096:
            first = nbytes[r[0][0]:r[0][1]].sum() / nbytes.sum()
            assert first <= 2.0 / (1 << (chunks - 1)) + nbytes[0] / nbytes.sum()
    assert chunk_ranges([], 4) == []


def test_excess_degrees():
    """<k^2>/<k> - 1: k - 1 on a k-regular graph; on a star (centre degree n-1, n-1 leaves
    of degree 1) ((n-1)^2 + (n-1)) / (2(n-1)) - 1 = n/2 - 1; 0 without edges."""
    n, k = 64, 6
    rp = np.arange(n + 1, dtype=np.int32) * k
    star = np.concatenate([[0, n - 1], n - 1 + np.arange(1, n)]).astype(np.int32)
    e = ensemble.excess_degrees([rp, star, np.zeros(5, np.int32)])
    assert e[0] == pytest.approx(k - 1)
    assert e[1] == pytest.approx(n / 2 - 1)
    assert e[2] == 0.0


def test_predicted_costs_order_members():
    """The resident path's member order: no infected agent costs nothing; at equal
    parameters a larger member costs more; a slow epidemic on a small graph outlasts (and
    out-costs) a quick one on a graph six times larger."""
    n = np.array([10_000, 20_000, 5_000, 30_000, 5_000])
    num_i = np.array([10, 20, 5, 30, 0])
    num_s = n - num_i
    beta = np.array([0.05, 0.05, 0.011, 0.2, 0.05])
    gamma = np.array([0.1, 0.1, 0.067, 0.3, 0.1])
    k = np.full(5, 20.0)
    c = ensemble.predicted_costs(n, num_s, num_i, beta, gamma, k, 365)
    assert c[4] == 0.0
    assert c[1] > c[0] > 0
    assert c[2] > c[3]
    # at least one active step's fixed cost for every member with an infected agent
    assert np.all(c[:4] >= ensemble.STEP_COST_ENTRIES)
