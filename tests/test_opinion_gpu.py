"""Opinion model on the GPU.

The float32 forward is one fixed sequence of IEEE-754 float32 operations (table-driven
exponential, correctly rounded reciprocal and division, no fused multiply-adds), so it is
compared BIT FOR BIT with the C oracle's float32 statement of the same sequence, up to the
full configuration (2^18 agents, 16-regular graph, 64 instances, 200 steps).  The float32
dynamics amplify rounding (a steep sigmoid, tau ~ 0.02), so float32 states of some instances
lie more than 1e-5 from the float64 oracle whatever the float32 implementation; that
distance is printed per instance, and the raw moments (what calibration uses) are held to
1e-6 relative of float64.  The adjoint gradient is checked against the float64 adjoint
oracle and float64 central differences; checkpoint invariance, torch.autograd, the model
API and the gradient calibrator complete the file."""

import numpy as np
import pytest
import torch

from oracle import coracle

pytestmark = pytest.mark.gpu


def _graph(n, seed=1):
    from oracle import workloads
    return workloads.random_regular(n, 16, seed)


def _params(B, seed=0):
    from jaxabm_gb300.opinion import calibration_params
    p = calibration_params(B, seed=seed)
    return p[:, 0], p[:, 1], p[:, 2]


def _f64(*a):
    return [np.asarray(x, dtype=np.float64) for x in a]


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def _report_f64(got, o0, rp, col, mu, eps, tau, T, cols, label):
    """Per-instance distance of the float32 states from the float64 oracle (printed) and
    the raw moments' relative error (returned)."""
    ref64 = coracle.opinion_run_f64(o0[:, cols].astype(np.float64), rp, col,
                                    *_f64(mu[cols], eps[cols], tau[cols]), T)
    err = np.abs(got[:, cols].astype(np.float64) - ref64).max(axis=0)
    m32 = coracle.opinion_moments_f64(got[:, cols].astype(np.float64))
    m64 = coracle.opinion_moments_f64(ref64)
    em = (np.abs(m32 - m64) / np.abs(m64)).max(axis=1)
    print(f"{label}: float32 vs float64 per instance: max |state err| " +
          " ".join(f"{c}:{e:.1e}" for c, e in zip(cols, err)) +
          f"; {int((err > 1e-5).sum())}/{len(cols)} instances above 1e-5; "
          f"max moment rel err {em.max():.2e}")
    return em


def test_sigmoid_bit_exact(cuda):
    """The forward's sigmoid equals the oracle's bit for bit on 4M points of [-120, 120],
    random values, and the special values (0, -0, +-inf, nan, the clamp edges, tiny and
    denormal inputs)."""
    from jaxabm_gb300 import _dev, _lib
    rs = np.random.RandomState(0)
    z = np.concatenate([
        np.linspace(-120, 120, 1 << 22, dtype=np.float32),
        (rs.standard_normal(1 << 20) * 20).astype(np.float32),
        np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 87.0, -87.0, 88.0, -88.0, 86.99,
                  -88.01, 1e-30, -1e-30, 1e-40, -1e-40, 3.4e38, -3.4e38], np.float32)])
    dz = torch.from_numpy(z).cuda()
    ds = torch.empty_like(dz)
    _lib.call("abm_opinion_sigmoid", _dev.ptr(dz), _dev.ptr(ds), z.size, None)
    got = ds.cpu().numpy()
    ref = coracle.sigmoid32(z)
    assert np.array_equal(_bits(got), _bits(ref))
    ok = np.abs(z) <= 86
    s64 = 1.0 / (1.0 + np.exp(-z[ok].astype(np.float64)))
    assert (np.abs(got[ok] - s64) / s64).max() < 4e-7  # about 3 ulp of the true sigmoid


@pytest.mark.parametrize("n,B,T", [(64, 4, 10), (4096, 4, 200), (4096, 64, 50), (2000, 8, 30),
                                   (1000, 128, 20)])
def test_forward_bit_exact(cuda, n, B, T):
    from jaxabm_gb300.opinion import OpinionBatch
    rp, col = _graph(n)
    o0 = np.random.RandomState(n).rand(n, B).astype(np.float32)
    mu, eps, tau = _params(B)
    b = OpinionBatch(rp, col, torch.from_numpy(o0), mu, eps, tau)
    got = b.forward(T)[:, :B].cpu().numpy()
    ref32 = coracle.opinion_run_f32(o0, rp, col, mu, eps, tau, T)
    assert np.array_equal(_bits(got), _bits(ref32))
    em = _report_f64(got, o0, rp, col, mu, eps, tau, T, list(range(B)), f"n={n} B={B} T={T}")
    assert np.all(em < 1e-6)
    m = b.moments().cpu().numpy()
    np.testing.assert_allclose(m, coracle.opinion_moments_f64(got.astype(np.float64)), rtol=1e-9)


def test_forward_full_config_bit_exact(cuda):
    """N = 2^18, random 16-regular graph, 64 instances (calibration parameter sets), 200
    steps: all 64 instances equal the float32 oracle bit for bit.  16 of them are compared
    with float64: over 200 steps a few agents of some instances end in another opinion
    cluster than in float64 (distance printed per instance), and the raw moments stay within
    1e-5 relative of float64 (3.4e-6 measured on a GB300)."""
    from jaxabm_gb300.opinion import OpinionBatch, initial_opinions
    n, B, T = 1 << 18, 64, 200
    rp, col = _graph(n, 0)
    o0 = initial_opinions(n, 0)
    mu, eps, tau = _params(B)
    b = OpinionBatch(rp, col, o0, mu, eps, tau)
    got = b.forward(T).cpu().numpy()
    o0h = np.repeat(o0.cpu().numpy()[:, None], B, axis=1)
    ref32 = coracle.opinion_run_f32(o0h, rp, col, mu, eps, tau, T)
    same = np.array([np.array_equal(_bits(got[:, c]), _bits(ref32[:, c])) for c in range(B)])
    assert same.all(), np.flatnonzero(~same)
    em = _report_f64(got, o0h, rp, col, mu, eps, tau, T, list(range(0, B, 4)),
                     "n=2^18 B=64 T=200")
    assert np.all(em < 1e-5)


def test_full_size_properties(cuda):
    """N = 2^18, 16-regular, 64 instances, 200 steps: mean opinion conserved to 1e-6 (the
    update is antisymmetric over each edge), opinions stay in the initial range, and column
    b equals the same instance run in a batch of 4."""
    from jaxabm_gb300.opinion import OpinionBatch, initial_opinions
    n = 1 << 18
    rp, col = _graph(n, 0)
    o0 = initial_opinions(n, 0)
    mu, eps, tau = _params(64)
    b = OpinionBatch(rp, col, o0, mu, eps, tau)
    oT = b.forward(200).clone()
    m = b.moments()
    m0 = float(o0.double().mean())
    assert torch.all(torch.abs(m[:, 0] - m0) < 1e-6)
    assert float(oT.min()) >= float(o0.min()) - 1e-6 and float(oT.max()) <= float(o0.max()) + 1e-6
    small = OpinionBatch(rp, col, o0, mu[5:9], eps[5:9], tau[5:9])
    assert torch.equal(small.forward(200), oT[:, 5:9])


@pytest.mark.parametrize("B,T,k", [(4, 60, 20), (8, 45, 7), (64, 40, 20)])
def test_adjoint_vs_f64_oracle(cuda, B, T, k):
    from jaxabm_gb300.opinion import OpinionBatch
    n = 2048
    rp, col = _graph(n, 3)
    o0 = np.random.RandomState(7).rand(n, B).astype(np.float32)
    mu, eps, tau = _params(B, seed=1)
    target = coracle.opinion_moments_f64(coracle.opinion_run_f64(
        o0[:, :1].astype(np.float64), rp, col, [0.25], [0.15], [0.025], T))[0]
    b = OpinionBatch(rp, col, torch.from_numpy(o0), mu, eps, tau)
    b.forward(T, k)
    g = b.backward(target).cpu().numpy()
    loss_ref, g_ref = coracle.opinion_grad_f64(o0.astype(np.float64), rp, col,
                                               mu.astype(np.float64), eps.astype(np.float64),
                                               tau.astype(np.float64), T, target)
    rel = np.abs(g - g_ref).max(axis=1) / np.maximum(np.abs(g_ref).max(axis=1), 1e-12)
    print(f"adjoint B={B} T={T} k={k}: max normwise rel err vs FP64 = {rel.max():.2e}")
    # float32 states and adjoints (float64 parameter-gradient accumulation) against the
    # float64 reverse sweep: a few 1e-3 at most, where the gradient is small
    assert rel.max() < 5e-3 and np.median(rel) < 5e-4
    loss = b.loss_of(b.moments(), target).cpu().numpy()
    np.testing.assert_allclose(loss, loss_ref, rtol=1e-4, atol=1e-12)


def _loss_f64(o0, rp, col, mu, eps, tau, T, target):
    x = coracle.opinion_run_f64(o0, rp, col, mu, eps, tau, T)
    m = coracle.opinion_moments_f64(x)
    return 0.25 * ((m - np.asarray(target)[None]) ** 2).sum(axis=1)


def _central_differences(o0, rp, col, mu, eps, tau, T, target, h):
    """float64 central differences of the loss in (mu, eps, tau) -> [B, 3]."""
    p = _f64(mu, eps, tau)
    out = np.zeros((len(p[0]), 3))
    for k in range(3):
        up = [v.copy() for v in p]
        dn = [v.copy() for v in p]
        up[k] += h
        dn[k] -= h
        out[:, k] = (_loss_f64(o0, rp, col, *up, T, target)
                     - _loss_f64(o0, rp, col, *dn, T, target)) / (2 * h)
    return out


def _hidden_target(o0col, rp, col, T):
    from jaxabm_gb300.opinion import HIDDEN_PARAMS
    x = coracle.opinion_run_f64(o0col.astype(np.float64), rp, col, *_f64(
        [HIDDEN_PARAMS[0]], [HIDDEN_PARAMS[1]], [HIDDEN_PARAMS[2]]), T)
    return coracle.opinion_moments_f64(x)[0]


def test_adjoint_full_config_vs_f64_adjoint(cuda):
    """N = 2^18, 16-regular, 64 instances, T = 200, a checkpoint every 20 steps: the GPU
    gradients of instances 0 and 1 against the float64 reverse sweep along the same float32
    trajectory (normwise 1e-2), which is the function a float32 run differentiates.  The
    float64 adjoint along the float64 trajectory is printed beside it: over 200 chaotic
    steps the two trajectories differentiate differently (instance 0's tau component by
    ~25 %), although their states differ by 2e-6 at most."""
    from jaxabm_gb300.opinion import OpinionBatch, initial_opinions
    n, B, T, k = 1 << 18, 64, 200, 20
    rp, col = _graph(n, 0)
    o0 = initial_opinions(n, 0)
    mu, eps, tau = _params(B)
    o0h = o0.cpu().numpy()[:, None]
    target = _hidden_target(o0h, rp, col, T)
    b = OpinionBatch(rp, col, o0, mu, eps, tau)
    b.forward(T, k)
    g = b.backward(target).cpu().numpy()
    cols = [0, 1]
    o0c = np.repeat(o0h, len(cols), axis=1)
    _, g32 = coracle.opinion_grad_f64_along_f32(o0c, rp, col, mu[cols], eps[cols], tau[cols], T,
                                                target)
    _, g64 = coracle.opinion_grad_f64(o0c.astype(np.float64), rp, col,
                                      *_f64(mu[cols], eps[cols], tau[cols]), T, target)
    rel = np.abs(g[cols] - g32).max(axis=1) / np.abs(g32).max(axis=1)
    rel64 = np.abs(g[cols] - g64).max(axis=1) / np.abs(g64).max(axis=1)
    print(f"adjoint n=2^18 B=64 T=200 k=20: GPU {g[cols].tolist()}\n  float64 sweep along the "
          f"float32 trajectory {g32.tolist()} (normwise rel err {rel})\n  float64 sweep along "
          f"the float64 trajectory {g64.tolist()} (normwise rel err {rel64})")
    assert np.all(rel < 1e-2)


def test_adjoint_full_size_vs_central_differences_short_horizon(cuda):
    """N = 2^18, 64 instances, T = 20 (one checkpoint segment): the GPU gradient of
    instances 0..3 against float64 central differences with h = 1e-3, every parameter."""
    from jaxabm_gb300.opinion import OpinionBatch, initial_opinions
    n, B, T, k = 1 << 18, 64, 20, 20
    rp, col = _graph(n, 0)
    o0 = initial_opinions(n, 0)
    mu, eps, tau = _params(B)
    o0h = o0.cpu().numpy()[:, None]
    target = _hidden_target(o0h, rp, col, T)
    b = OpinionBatch(rp, col, o0, mu, eps, tau)
    b.forward(T, k)
    g = b.backward(target).cpu().numpy()
    cols = [0, 1, 2, 3]
    fd = _central_differences(np.repeat(o0h, len(cols), axis=1).astype(np.float64), rp, col,
                              mu[cols], eps[cols], tau[cols], T, target, 1e-3)
    rel = np.abs(g[cols] - fd) / np.abs(fd)
    print(f"n=2^18 T=20: GPU adjoint vs float64 central differences (h=1e-3), rel err\n{rel}")
    assert np.all(rel < 1e-2)


def test_adjoint_vs_central_differences_chaotic_horizon(cuda):
    """T = 200 (k = 20) on 2^14 agents: over 200 steps the bounded-confidence map becomes
    chaotic, and the loss varies on scales far below 1e-3 in eps and tau.  Central
    differences converge to the GPU adjoint as h shrinks (h = 1e-6, float64: every parameter
    within 1e-2), while h = 1e-3 measures a secant that differs from the derivative
    (printed; only mu, along which the loss stays smooth, is held to 5e-2 there)."""
    from jaxabm_gb300.opinion import OpinionBatch, initial_opinions
    n, B, T, k = 1 << 14, 4, 200, 20
    rp, col = _graph(n, 0)
    o0 = initial_opinions(n, 0)
    mu, eps, tau = _params(B)
    o0h = o0.cpu().numpy()[:, None]
    target = _hidden_target(o0h, rp, col, T)
    b = OpinionBatch(rp, col, o0, mu, eps, tau)
    b.forward(T, k)
    g = b.backward(target).cpu().numpy()
    o0b = np.repeat(o0h, B, axis=1).astype(np.float64)
    fd6 = _central_differences(o0b, rp, col, mu, eps, tau, T, target, 1e-6)
    fd3 = _central_differences(o0b, rp, col, mu, eps, tau, T, target, 1e-3)
    rel6 = np.abs(g - fd6).max(axis=1) / np.abs(fd6).max(axis=1)
    rel3 = np.abs(g - fd3) / np.abs(g)
    print(f"n=2^14 T=200: GPU vs central differences h=1e-6 (normwise) {rel6};\n"
          f"h=1e-3 (per parameter) {rel3}")
    assert np.all(rel6 < 1e-2)
    assert np.all(rel3[:, 0] < 5e-2)


def test_checkpoint_interval_invariance(cuda):
    from jaxabm_gb300.opinion import OpinionBatch
    n, B, T = 1024, 4, 33
    rp, col = _graph(n, 2)
    o0 = np.random.RandomState(1).rand(n, B).astype(np.float32)
    mu, eps, tau = _params(B, seed=2)
    target = np.array([0.5, 0.3, 0.2, 0.15])
    grads = []
    for k in (1, 5, 20, 33):
        b = OpinionBatch(rp, col, torch.from_numpy(o0), mu, eps, tau)
        b.forward(T, k)
        grads.append(b.backward(target).cpu().numpy())
    for g in grads[1:]:
        assert np.array_equal(g, grads[0])


def test_autograd_function(cuda):
    from jaxabm_gb300.opinion import OpinionBatch, OpinionLoss
    n, B, T = 1024, 4, 30
    rp, col = _graph(n, 4)
    o0 = np.random.RandomState(2).rand(n).astype(np.float32)
    mu0, eps0, tau0 = _params(B, seed=3)
    target = np.array([0.5, 0.3, 0.2, 0.15])
    b = OpinionBatch(rp, col, torch.from_numpy(o0), mu0, eps0, tau0)
    mu = torch.tensor(mu0, device="cuda", requires_grad=True)
    eps = torch.tensor(eps0, device="cuda", requires_grad=True)
    tau = torch.tensor(tau0, device="cuda", requires_grad=True)
    loss = OpinionLoss.apply(mu, eps, tau, b, target, T, 10)
    w = torch.tensor([1.0, 2.0, 0.5, 3.0], device="cuda")
    (loss * w).sum().backward()
    b2 = OpinionBatch(rp, col, torch.from_numpy(o0), mu0, eps0, tau0)
    b2.forward(T, 10)
    g = b2.backward(target, w.double()).cpu().numpy()
    np.testing.assert_allclose(mu.grad.cpu().numpy(), g[:, 0], rtol=1e-6)
    np.testing.assert_allclose(eps.grad.cpu().numpy(), g[:, 1], rtol=1e-6)
    np.testing.assert_allclose(tau.grad.cpu().numpy(), g[:, 2], rtol=1e-6)


def test_opinion_model_api(cuda):
    """jx.OpinionModel through Model.run: final opinions bit-identical to the float32
    oracle, metrics m1..m4 the raw moments after every step."""
    import jaxabm_gb300 as jx
    from jaxabm_gb300.opinion import initial_opinions
    m = jx.OpinionModel({"n": 4096, "steps": 40, "seed": 5})
    res = m.run()
    x = res["agents.people.opinion"]
    rp, col = _graph(4096, 5)
    o0 = initial_opinions(4096, 5).cpu().numpy()
    ref = coracle.opinion_run_f32(o0[:, None], rp, col, [0.3], [0.2], [0.02], 40)[:, 0]
    assert np.array_equal(_bits(x), _bits(ref))
    assert res["step"] == list(range(1, 41))
    last = coracle.opinion_moments_f64(ref[:, None].astype(np.float64))[0]
    np.testing.assert_allclose([res[f"m{k}"][-1] for k in range(1, 5)], last, rtol=1e-12)
    mid = coracle.opinion_run_f32(o0[:, None], rp, col, [0.3], [0.2], [0.02], 7)
    np.testing.assert_allclose([res[f"m{k}"][6] for k in range(1, 5)],
                               coracle.opinion_moments_f64(mid.astype(np.float64))[0],
                               rtol=1e-12)


def test_model_vjp_matches_f64_adjoint(cuda):
    """OpinionModel.final_metrics_vjp (what ModelCalibrator's adam/sgd use): the final
    moments equal the float32 forward's, and the vector-Jacobian product for weights w on
    the moments equals the float64 adjoint oracle's gradient of sum_k w_k m_k."""
    import jaxabm_gb300 as jx
    from jaxabm_gb300.opinion import initial_opinions
    n, T = 4096, 60
    model = jx.OpinionModel({"n": n, "steps": T, "mu": 0.28, "eps": 0.21, "tau": 0.022}, seed=3)
    metrics, vjp = model.final_metrics_vjp(["mu", "eps", "tau"], steps=T)
    rp, col = _graph(n, 3)
    o0 = initial_opinions(n, 3).cpu().numpy()[:, None]
    ref = coracle.opinion_run_f32(o0, rp, col, [0.28], [0.21], [0.022], T)
    np.testing.assert_allclose([metrics[f"m{k}"] for k in range(1, 5)],
                               coracle.opinion_moments_f64(ref.astype(np.float64))[0],
                               rtol=1e-12)
    w = np.array([0.7, -1.3, 0.4, 2.0])
    g = vjp({f"m{k + 1}": w[k] for k in range(4)})
    # the oracle's loss is 0.25 sum (m - t)^2; with t = m - 2 w its gradient is sum w_k dm_k
    m64 = coracle.opinion_moments_f64(coracle.opinion_run_f64(
        o0.astype(np.float64), rp, col, [0.28], [0.21], [0.022], T))[0]
    _, g64 = coracle.opinion_grad_f64(o0.astype(np.float64), rp, col, [0.28], [0.21], [0.022],
                                      T, m64 - 2 * w)
    got = np.array([g["mu"], g["eps"], g["tau"]])
    rel = np.abs(got - g64[0]).max() / np.abs(g64[0]).max()
    print(f"model vjp vs float64 adjoint: rel err {rel:.2e}")
    assert rel < 5e-3


def test_gradient_calibration_reduces_loss(cuda):
    """ModelCalibrator(method="adam") on OpinionModel: recovers moments produced with hidden
    parameters from a start 20 % away; the loss of the robust evaluation falls."""
    import jaxabm_gb300 as jx
    from jaxabm_gb300.analysis import ModelCalibrator
    n, T = 4096, 40
    hidden = {"mu": 0.25, "eps": 0.15, "tau": 0.025}
    truth = jx.OpinionModel(dict(n=n, steps=T, graph_seed=1, **hidden), seed=42).run()
    targets = {f"m{k}": float(truth[f"m{k}"][-1]) for k in range(1, 5)}

    def factory(params=None, config=None):
        return jx.OpinionModel(dict(n=n, steps=T, graph_seed=1, **params), seed=config.seed)

    cal = ModelCalibrator(factory, {"mu": 0.3, "eps": 0.18, "tau": 0.03}, targets,
                          param_bounds={"mu": (0.05, 0.6), "eps": (0.05, 0.5),
                                        "tau": (0.005, 0.1)},
                          learning_rate=0.005, max_iterations=8, method="adam",
                          evaluation_steps=T, num_evaluation_runs=1, tolerance=-1.0,
                          patience=100, loss_type="relative")
    loss0, g0 = cal.loss_and_grad(np.array([0.3, 0.18, 0.03]))
    assert np.all(np.isfinite(g0)) and np.any(g0 != 0)
    cal.calibrate(verbose=False)
    assert len(cal.loss_history) == 8
    assert cal.best_loss < cal.loss_history[0]
