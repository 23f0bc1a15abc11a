"""Device CSR construction (abm_csr_from_edges) against a stable host sort by source."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _host_csr(edges, n):
    order = np.argsort(edges[:, 0], kind="stable")
    counts = np.bincount(edges[:, 0], minlength=n)
    rp = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=rp[1:])
    return rp.astype(np.int32), edges[order, 1].astype(np.int32)


@pytest.mark.parametrize("n,E,seed", [
    (1, 5, 0),            # one node, self loops
    (200, 3000, 1),       # one radix pass (keys below 256)
    (70_000, 400_000, 2),  # three passes, many empty rows
    (5, 0, 3),            # no edges
    (300_000, 9_000, 4),  # mostly empty rows
])
def test_csr_matches_stable_host_sort(cuda, n, E, seed):
    from jaxabm_gb300.agentpy import csr_from_edges
    rs = np.random.RandomState(seed)
    edges = rs.randint(0, n, size=(E, 2)).astype(np.int32)
    if E > 10:
        edges[: E // 10, 0] = 0  # a hub row with many edges in insertion order
    rp, col = csr_from_edges(edges, n)
    ref_rp, ref_col = _host_csr(edges, n)
    assert np.array_equal(rp.cpu().numpy(), ref_rp)
    assert np.array_equal(col.cpu().numpy(), ref_col)


def test_csr_rejects_out_of_range(cuda):
    from jaxabm_gb300.agentpy import csr_from_edges
    with pytest.raises(ValueError):
        csr_from_edges(np.array([[0, 1], [1, 7]], np.int32), 3)
    with pytest.raises(ValueError):
        csr_from_edges(np.array([[4, 1]], np.int32), 3)


def test_ba_network_from_edges_equals_generator(cuda):
    """A Barabasi-Albert graph given as an edge list whose rows come in shuffled order (each
    row's own edges in order) gives back the generator's CSR."""
    from jaxabm_gb300 import sir
    from jaxabm_gb300.agentpy import csr_from_edges
    rp, col = sir.barabasi_albert(20_000, 4, 7)
    n = len(rp) - 1
    rows = np.random.RandomState(0).permutation(n)
    src = np.concatenate([np.full(rp[r + 1] - rp[r], r) for r in rows]).astype(np.int32)
    dst = np.concatenate([col[rp[r]:rp[r + 1]] for r in rows]).astype(np.int32)
    drp, dcol = csr_from_edges(np.stack([src, dst], axis=1), n)
    assert np.array_equal(drp.cpu().numpy(), rp)
    assert np.array_equal(dcol.cpu().numpy(), col)


def test_network_add_edges_csr(cuda):
    """Network.add_edges (undirected: reverse edges appended) -> csr() on the device."""
    import jaxabm_gb300 as jx
    model = jx.Model({"steps": 1}, seed=0)
    net = jx.Network(model)
    net.add_edges(np.array([[0, 1], [2, 0], [1, 2], [3, 0]], np.int32))
    rp, col = net.csr()
    assert rp.cpu().tolist() == [0, 3, 5, 7, 8]
    # row 0: edges in insertion order (0,1), then reverse edges (0,2), (0,3)
    assert col.cpu().tolist() == [1, 2, 3, 2, 0, 0, 1, 0]
