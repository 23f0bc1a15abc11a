"""The FP64 opinion-model adjoint oracle against central finite differences (CPU only)."""

import numpy as np
import pytest

from oracle import coracle
from jaxabm_gb300 import sir


@pytest.fixture(scope="module")
def case(lib):
    rp, col = sir.random_regular(512, 16, 1)
    o0 = np.random.RandomState(0).rand(512, 4)
    mu = np.array([0.3, 0.25, 0.35, 0.3])
    eps = np.array([0.2, 0.15, 0.25, 0.2])
    tau = np.array([0.02, 0.03, 0.025, 0.05])
    T = 50
    target = coracle.opinion_moments_f64(
        coracle.opinion_run_f64(o0[:, :1], rp, col, [0.28], [0.18], [0.022], T))[0]
    return rp, col, o0, mu, eps, tau, T, target


def _fd(case, h):
    rp, col, o0, mu, eps, tau, T, target = case
    def loss(m_, e_, t_):
        mom = coracle.opinion_moments_f64(coracle.opinion_run_f64(o0, rp, col, m_, e_, t_, T))
        return 0.25 * ((mom - target) ** 2).sum(1)
    fd = np.zeros((4, 3))
    for p in range(3):
        plus = [mu.copy(), eps.copy(), tau.copy()]
        minus = [mu.copy(), eps.copy(), tau.copy()]
        plus[p] += h
        minus[p] -= h
        fd[:, p] = (loss(*plus) - loss(*minus)) / (2 * h)
    return fd


def test_adjoint_vs_central_differences_tight(case):
    rp, col, o0, mu, eps, tau, T, target = case
    _, g = coracle.opinion_grad_f64(o0, rp, col, mu, eps, tau, T, target)
    fd = _fd(case, 1e-6)
    np.testing.assert_allclose(g, fd, rtol=1e-5, atol=1e-10)


def test_adjoint_vs_central_differences_h1e3(case):
    """h = 1e-3: truncation error of the difference quotient dominates for tau ~ 0.02
    (the third derivative in tau is large); the adjoint agrees to a few tens of percent
    there and closely for the smooth mu direction."""
    rp, col, o0, mu, eps, tau, T, target = case
    _, g = coracle.opinion_grad_f64(o0, rp, col, mu, eps, tau, T, target)
    fd = _fd(case, 1e-3)
    np.testing.assert_allclose(g[:, 0], fd[:, 0], rtol=2e-2, atol=1e-8)
    assert np.all(np.sign(g) == np.sign(fd)) or np.max(np.abs(g - fd)) < 5e-3


def test_f32_forward_close_to_f64(case):
    rp, col, o0, mu, eps, tau, T, _ = case
    a = coracle.opinion_run_f32(o0.astype(np.float32), rp, col, mu, eps, tau, T)
    b = coracle.opinion_run_f64(o0, rp, col, mu, eps, tau, T)
    assert np.abs(a - b).max() < 1e-5


def test_mean_conserved_on_regular_graph(case):
    rp, col, o0, mu, eps, tau, T, _ = case
    b = coracle.opinion_run_f64(o0, rp, col, mu, eps, tau, T)
    np.testing.assert_allclose(b.mean(0), o0.mean(0), atol=1e-12)


def test_c_forward_equals_numpy_statement(case):
    """The C float64 forward (checker of the GPU forward and of the adjoint's recompute)
    against the direct NumPy statement of the step, within float64 rounding."""
    from oracle import models
    rp, col, o0, mu, eps, tau, T, _ = case
    ref = models.opinion_run_f64(o0, rp, col, mu, eps, tau, 20)
    got = coracle.opinion_run_f64(o0, rp, col, mu, eps, tau, 20)
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-13)
    assert np.abs(ref - o0).max() > 1e-3  # opinions moved


def test_exp_table_is_correctly_rounded():
    """The 32 entries of the table-driven exponential are 2^(j/32) rounded to the nearest
    float32 (checked with 50-digit decimal arithmetic)."""
    from decimal import Decimal, getcontext
    from fractions import Fraction
    getcontext().prec = 50
    ln2 = Decimal(2).ln()
    table = coracle.exp2_table()
    for j in range(32):
        exact = Fraction((ln2 * j / 32).exp())
        t = Fraction(float(table[j]))
        half_ulp = Fraction(float(np.spacing(np.float32(table[j])))) / 2
        assert abs(t - exact) <= half_ulp, j


def test_exp_and_sigmoid_accuracy():
    """The float32 exponential is within 1.05 ulp of exp on [-87, 88]; the sigmoid within
    2e-7 relative for |z| <= 86; out-of-range and special inputs are clamped
    (exp(x) for x < -87 is exp(-87), for x > 88 exp(88); NaN reads as -87)."""
    x = np.linspace(-87, 88, 2_000_001).astype(np.float32)
    y = coracle.expf_tang(x).astype(np.float64)
    ref = np.exp(x.astype(np.float64))
    assert (np.abs(y - ref) / np.spacing(ref.astype(np.float32))).max() < 1.05
    z = np.linspace(-86, 86, 2_000_001).astype(np.float32)
    s = coracle.sigmoid32(z).astype(np.float64)
    sr = 1.0 / (1.0 + np.exp(-z.astype(np.float64)))
    assert (np.abs(s - sr) / sr).max() < 2e-7
    edge = coracle.expf_tang(np.array([-1000, -87, 88, 1000, np.nan, -np.inf, np.inf],
                                      np.float32))
    assert edge[0] == edge[1] == edge[4] == edge[5] and edge[2] == edge[3] == edge[6]
    assert np.isfinite(edge).all()
