"""The oracle's own workload inputs (CPU only): its network generators equal the library's,
the Barabasi-Albert graphs have Barabasi-Albert degree statistics, and its statement of the
4,096-member ensemble equals the package's."""

import numpy as np
import pytest

from oracle import workloads as ow


@pytest.mark.parametrize("n,m,seed", [(10, 2, 5), (1000, 4, 5), (50_000, 4, 5), (3000, 7, 1),
                                      (99_984, 4, 17), (6, 5, 0)])
def test_barabasi_albert_equals_library(lib, n, m, seed):
    from jaxabm_gb300 import sir
    a, b = ow.barabasi_albert(n, m, seed), sir.barabasi_albert(n, m, seed)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


@pytest.mark.parametrize("n,d,seed", [(40, 4, 3), (1000, 16, 3), (1 << 16, 16, 0), (200, 6, 9)])
def test_random_regular_equals_library(lib, n, d, seed):
    from jaxabm_gb300 import sir
    a, b = ow.random_regular(n, d, seed), sir.random_regular(n, d, seed)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_barabasi_albert_degree_statistics():
    """Preferential attachment, not some other generator: the degree CCDF follows the
    Barabasi-Albert law P(K >= k) = m (m + 1) / (k (k + 1)) (within 3 % up to k = 64, 6 %
    at k = 128), and node i's degree grows as m sqrt(n / i) with its age."""
    n, m = 400_000, 4
    rp, col = ow.barabasi_albert(n, m, 0)
    deg = np.diff(rp)
    assert col.size == 2 * m * (n - m) and deg[m + 1:].min() == m
    for k, tol in [(5, 0.03), (6, 0.03), (8, 0.03), (12, 0.03), (16, 0.03), (24, 0.03),
                   (32, 0.03), (64, 0.03), (128, 0.06)]:
        emp = (deg >= k).mean()
        assert abs(emp / (m * (m + 1) / (k * (k + 1))) - 1) < tol, k
    for lo, hi in [(100, 200), (1000, 2000), (n // 2, n)]:
        expect = m * np.sqrt(n / np.arange(lo, hi)).mean()
        assert abs(deg[lo:hi].mean() / expect - 1) < 0.1, (lo, hi)
    # a uniform-attachment graph of the same size would have a thin (exponential) tail
    assert (deg >= 128).sum() > 300


def test_random_regular_is_simple_and_regular():
    rp, col = ow.random_regular(5000, 16, 4)
    assert np.all(np.diff(rp) == 16)
    rows = np.repeat(np.arange(5000), 16)
    assert not np.any(col == rows)
    assert np.all(np.diff(col.reshape(5000, 16), axis=1) > 0)  # sorted, no duplicates
    fwd = set(zip(rows.tolist(), col.tolist()))
    assert all((b, a) in fwd for a, b in list(fwd)[:20000])


def test_initial_states_equal_library():
    from jaxabm_gb300 import sir
    for n, f, s in [(1 << 20, 0.001, 0), (500, 0.001, 3), (7000, 0.3, 9)]:
        assert np.array_equal(ow.sir_initial_states(n, f, s), sir.initial_states(n, f, s))


def test_ensemble_spec_equals_package():
    from jaxabm_gb300 import ensemble
    a, b = ow.sir_ensemble_spec(4096), ensemble.ensemble_spec(4096)
    assert sorted(a) == sorted(b)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert int(a["n"].argmax()) == int(b["n"].argmax())


def test_balanced_slices_cover_every_member_once():
    spec = ow.sir_ensemble_spec(4096)
    for parts in (1, 7, 20):
        sl = ow.balanced_slices(spec["n"], parts)
        assert len(sl) == parts
        assert np.array_equal(np.concatenate(sl), np.arange(4096))
        tot = np.array([spec["n"][s].sum() for s in sl])
        assert tot.max() < 1.05 * spec["n"].sum() / parts + spec["n"].max()
