"""Random-walk parity: CUDA path (C ABI and the jx.Model API) vs the C oracle.

FP32 states match within 1e-5 (circular distance on the unit torus, where ``% 1.0`` can
send a value to either 0 or 1); per-step means within 1e-5 relative.  The error of the
FP32 run against the FP64 oracle is checked and printed."""

import numpy as np
import pytest
import torch

from oracle import coracle, models

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _circ(a, b):
    d = np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64))
    return np.minimum(d, 1.0 - d)


def _run_abi(seed, n, steps, sigma=0.01):
    from jaxabm_gb300 import _dev, _lib
    import jaxabm_gb300.random as jr
    jr.set_partitionable(True)
    rng, (ik,) = models.model_keys(seed, 1)
    x = torch.empty(n, dtype=torch.float32, device="cuda")
    y = torch.empty(n, dtype=torch.float32, device="cuda")
    ikd = _dev.keys_from_numpy(ik)
    _lib.call("abm_randomwalk_init", _dev.ptr(x), _dev.ptr(y), n, _dev.ptr(ikd), None)
    init = (x.cpu().numpy().copy(), y.cpu().numpy().copy())
    rngd = _dev.keys_from_numpy(rng)
    ck = jr.keychain(rngd, steps, 1).reshape(steps, 2).contiguous()
    means = torch.empty((steps, 2), dtype=torch.float32, device="cuda")
    wsb = _lib.load().abm_randomwalk_workspace_bytes(n, steps)
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    _lib.call("abm_randomwalk_run", _dev.ptr(x), _dev.ptr(y), n, _dev.ptr(ck), steps, sigma,
              _dev.ptr(means), _dev.ptr(ws), wsb, None)
    torch.cuda.synchronize()
    return init, x.cpu().numpy(), y.cpu().numpy(), means.cpu().numpy()


@pytest.mark.parametrize("n,steps", [(1, 3), (31, 5), (1000, 20), (10_000, 100), (4099, 130),
                                     (140_000, 7)])  # the last: one agent per thread
def test_randomwalk_abi_vs_oracle(cuda, n, steps):
    init, x, y, means = _run_abi(0, n, steps)
    rng, (ik,) = models.model_keys(0, 1)
    x0, y0 = coracle.randomwalk_init(ik, n)
    assert np.array_equal(init[0], x0) and np.array_equal(init[1], y0)  # bit-exact init
    ref = coracle.randomwalk_run(0, n, steps, f64=True)
    assert _circ(x, ref["x"]).max() < TOL
    assert _circ(y, ref["y"]).max() < TOL
    np.testing.assert_allclose(means, ref["means"], rtol=TOL)
    err64 = max(_circ(x, ref["x64"]).max(), _circ(y, ref["y64"]).max())
    print(f"randomwalk n={n} steps={steps}: max |x - x_fp64| = {err64:.2e}")
    assert err64 < TOL
    np.testing.assert_allclose(means, ref["means64"], rtol=TOL)


def test_randomwalk_model_api(cuda):
    import jaxabm_gb300 as jx
    model = jx.RandomWalkModel({"n": 10_000, "steps": 100, "seed": 0})
    results = model.run()
    ref = coracle.randomwalk_run(0, 10_000, 100)
    assert list(results["step"]) == list(range(1, 101))
    np.testing.assert_allclose(np.array([results["mean_x"], results["mean_y"]]).T, ref["means"],
                               rtol=TOL)
    assert _circ(results["agents.walkers.x"], ref["x"]).max() < TOL


def test_randomwalk_jaxmodel_per_step_equals_fused(cuda):
    import jaxabm_gb300 as jx
    def make(metrics_fn=None):
        m = jx.JaxModel(config=jx.ModelConfig(seed=3, steps=12), metrics_fn=metrics_fn)
        m.add_agent_collection("w", jx.AgentCollection(jx.agentpy.AgentWrapper(jx.RandomWalker), 777))
        return m
    a = make()
    ra = a.run()
    b = make(metrics_fn=lambda env, states, p: {"sx": states["w"]["x"].sum()})
    rb = b.run()
    assert np.array_equal(a.agent_collections["w"].states["x"].cpu().numpy(),
                          b.agent_collections["w"].states["x"].cpu().numpy())
    np.testing.assert_allclose(ra["mean_x"], rb["mean_x"], rtol=0, atol=0)
    assert len(rb["sx"]) == 12


def test_randomwalk_workspace_too_small(cuda):
    from jaxabm_gb300 import _dev, _lib
    x = torch.zeros(100, device="cuda")
    y = torch.zeros(100, device="cuda")
    ck = torch.zeros((4, 2), dtype=torch.int32, device="cuda")
    means = torch.zeros((4, 2), device="cuda")
    ws = torch.zeros(8, dtype=torch.uint8, device="cuda")
    st = _lib.load().abm_randomwalk_run(_dev.ptr(x), _dev.ptr(y), 100, _dev.ptr(ck), 4, 0.01,
                                        _dev.ptr(means), _dev.ptr(ws), 8, None)
    assert st == _lib.ABM_ERR_WORKSPACE
