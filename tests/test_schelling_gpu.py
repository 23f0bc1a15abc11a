"""Schelling parity: positions and per-step (unhappy, moved) bit-exact vs the C oracle."""

import numpy as np
import pytest
import torch

from oracle import coracle, models

pytestmark = pytest.mark.gpu


def _keys(seed, steps):
    from jaxabm_gb300 import _dev
    import jaxabm_gb300.random as jr
    rng, _ = models.model_keys(seed, 1)
    ck = jr.keychain(_dev.keys_from_numpy(rng), steps, 1).reshape(steps, 2).contiguous()
    ref, _ = models.keychain(rng, steps, 1)
    return ck, ref.reshape(steps, 2)


def _run_abi(pos, types, W, H, ck, threshold=(3, 8)):
    from jaxabm_gb300 import _dev, _lib
    n = len(pos)
    p = torch.from_numpy(pos.astype(np.int32)).cuda()
    t = torch.from_numpy(types.astype(np.int8)).cuda()
    grid = torch.empty(W * H, dtype=torch.int8, device="cuda")
    ca = torch.empty(W * H, dtype=torch.int32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.call("abm_schelling_place", _dev.ptr(p), _dev.ptr(t), n, W, H, _dev.ptr(grid),
              _dev.ptr(ca), _dev.ptr(status), None)
    assert int(status.item()) == 0
    steps = ck.shape[0]
    stats = torch.empty((steps, 2), dtype=torch.int32, device="cuda")
    wsb = _lib.load().abm_schelling_workspace_bytes(n, W, H)
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    _lib.call("abm_schelling_run", _dev.ptr(p), _dev.ptr(t), n, W, H, _dev.ptr(grid), _dev.ptr(ca),
              _dev.ptr(ck), steps, threshold[0], threshold[1], _dev.ptr(stats), _dev.ptr(ws),
              wsb, None)
    torch.cuda.synchronize()
    return p.cpu().numpy(), stats.cpu().numpy(), grid.cpu().numpy(), ca.cpu().numpy()


@pytest.mark.parametrize("W,H,density,steps,seed", [
    (8, 8, 0.5, 10, 0), (16, 16, 0.9, 30, 3), (3, 5, 0.6, 12, 2), (64, 32, 0.75, 40, 5),
    (300, 17, 0.9, 15, 7), (256, 256, 0.97, 10, 4),
    (600, 500, 0.9, 6, 8),  # above 2^18 cells: four launches per step instead of one cluster
])
def test_schelling_small_bit_exact(cuda, W, H, density, steps, seed):
    from jaxabm_gb300.schelling import initial_layout
    pos, types = initial_layout(W, H, density, 0.5, seed)
    ck, ckref = _keys(seed, steps)
    p, stats, grid, ca = _run_abi(pos, types, W, H, ck)
    rp, rstats = coracle.schelling_run(pos, types, W, H, ckref)
    assert np.array_equal(stats, rstats)
    assert np.array_equal(p, rp)
    # grid / occupancy consistency
    g = np.full(W * H, -1, np.int8)
    g[rp] = types
    assert np.array_equal(grid, g)
    assert np.array_equal(ca[rp], np.arange(len(pos)))
    assert (ca >= 0).sum() == len(pos)


@pytest.mark.parametrize("W,H,threshold", [(40, 40, (1, 2)), (64, 32, (2, 3)), (50, 50, (0, 1)),
                                           (600, 500, (5, 8)), (30, 30, (1, 1))])
def test_schelling_other_thresholds(cuda, W, H, threshold):
    """Thresholds other than 3/8 (1/2 as in the reference example's default, 2/3, 0: nobody
    unhappy, 5/8 on the four-launch path, 1: everyone with an unlike neighbour unhappy)
    equal the oracle's run with the same (num, den)."""
    from jaxabm_gb300.schelling import initial_layout
    pos, types = initial_layout(W, H, 0.8, 0.5, 11)
    ck, ckref = _keys(11, 20)
    p, stats, _, _ = _run_abi(pos, types, W, H, ck, threshold)
    rp, rstats = coracle.schelling_run(pos, types, W, H, ckref, threshold)
    assert np.array_equal(stats, rstats)
    assert np.array_equal(p, rp)
    if threshold[0] == 0:
        assert stats[:, 0].sum() == 0


def test_schelling_full_config(cuda):
    """256x256 torus, density 0.9, 50/50 types, 37.5% threshold, 200 steps, seed 1."""
    from jaxabm_gb300.schelling import initial_layout
    pos, types = initial_layout(256, 256, 0.9, 0.5, 1)
    assert len(pos) == 58982 and (types == 0).sum() == 29491
    ck, ckref = _keys(1, 200)
    p, stats, _, _ = _run_abi(pos, types, 256, 256, ck)
    rp, rstats = coracle.schelling_run(pos, types, 256, 256, ckref)
    assert np.array_equal(stats, rstats)
    assert np.array_equal(p, rp)
    assert len(np.unique(p)) == len(p)
    assert stats[-1, 0] < stats[0, 0]  # segregation reduces unhappiness


def test_schelling_model_api(cuda):
    import jaxabm_gb300 as jx
    from jaxabm_gb300.schelling import initial_layout
    m = jx.SchellingModel({"width": 40, "height": 40, "steps": 25, "seed": 9})
    res = m.run()
    pos, types = initial_layout(40, 40, 0.9, 0.5, 9)
    _, ckref = _keys(9, 25)
    rp, rstats = coracle.schelling_run(pos, types, 40, 40, ckref)
    assert np.array_equal(np.array([res["unhappy"], res["moved"]]).T, rstats)
    assert np.array_equal(res["agents.agents.position"], rp)
    assert np.array_equal(res["agents.agents.type"], types)


def test_schelling_model_threshold_param(cuda):
    """SchellingModel(threshold=...) reaches the kernel as an exact fraction."""
    import jaxabm_gb300 as jx
    from jaxabm_gb300.schelling import initial_layout
    res = jx.SchellingModel({"width": 40, "height": 40, "steps": 15, "seed": 2,
                             "threshold": 0.5}).run()
    pos, types = initial_layout(40, 40, 0.9, 0.5, 2)
    _, ckref = _keys(2, 15)
    rp, rstats = coracle.schelling_run(pos, types, 40, 40, ckref, (1, 2))
    assert np.array_equal(np.array([res["unhappy"], res["moved"]]).T, rstats)
    assert np.array_equal(res["agents.agents.position"], rp)


def test_schelling_rejects_collisions(cuda):
    from jaxabm_gb300 import _dev, _lib
    p = torch.tensor([0, 5, 5], dtype=torch.int32, device="cuda")
    t = torch.tensor([0, 1, 0], dtype=torch.int8, device="cuda")
    grid = torch.empty(16, dtype=torch.int8, device="cuda")
    ca = torch.empty(16, dtype=torch.int32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.call("abm_schelling_place", _dev.ptr(p), _dev.ptr(t), 3, 4, 4, _dev.ptr(grid),
              _dev.ptr(ca), _dev.ptr(status), None)
    assert int(status.item()) == 1
