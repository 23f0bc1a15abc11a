"""ctypes wrappers of the C oracle (oracle/abm_oracle.c).  TEST INFRASTRUCTURE ONLY."""

import ctypes

import numpy as np

from . import build as _build
from . import models as _models


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def lib():
    L = _build.load()
    return L


def set_threads(n):
    lib().orc_set_threads(ctypes.c_int(int(n)))


def num_threads():
    L = lib()
    L.orc_num_threads.restype = ctypes.c_int
    return L.orc_num_threads()


def threefry(key, c0, c1):
    key = np.ascontiguousarray(key, dtype=np.uint32)
    c0 = np.ascontiguousarray(c0, dtype=np.uint32)
    c1 = np.ascontiguousarray(c1, dtype=np.uint32)
    y0 = np.empty_like(c0)
    y1 = np.empty_like(c1)
    lib().orc_threefry(_p(key), _p(c0), _p(c1), ctypes.c_int64(c0.size), _p(y0), _p(y1))
    return y0, y1


def keychain(rng, steps, ncoll=1):
    rng = np.array(rng, dtype=np.uint32, copy=True)
    out = np.zeros((steps, ncoll, 2), dtype=np.uint32)
    lib().orc_keychain(_p(rng), ctypes.c_int32(ncoll), ctypes.c_int32(steps), _p(out))
    return out, rng


def randomwalk_init(init_key, n):
    x = np.empty(n, np.float32)
    y = np.empty(n, np.float32)
    k = np.ascontiguousarray(init_key, dtype=np.uint32)
    lib().orc_randomwalk_init(_p(x), _p(y), ctypes.c_int64(n), _p(k))
    return x, y


def randomwalk_run(seed, n, steps, sigma=0.01, f64=False):
    """Full run from a seed.  Returns dict with x, y (float32), means (float64[steps,2]
    of the float32 states) and, with f64=True, x64/y64/means64 from float64 arithmetic."""
    rng, (ik,) = _models.model_keys(seed, 1)
    x, y = randomwalk_init(ik, n)
    ck, rng = keychain(rng, steps, 1)
    ck = np.ascontiguousarray(ck.reshape(steps, 2))
    means = np.zeros((steps, 2))
    xd = x.astype(np.float64) if f64 else None
    yd = y.astype(np.float64) if f64 else None
    means64 = np.zeros((steps, 2)) if f64 else None
    lib().orc_randomwalk_run(_p(x), _p(y), _p(xd), _p(yd), ctypes.c_int64(n), _p(ck),
                             ctypes.c_int32(steps), ctypes.c_float(sigma), _p(means),
                             _p(means64))
    out = {"x": x, "y": y, "means": means, "rng": rng}
    if f64:
        out.update(x64=xd, y64=yd, means64=means64)
    return out


def sir_run(row_ptr, col, state, rng, steps, beta, gamma):
    """SIR run from the given compartments and rng.  Returns (final state, counts
    int32[steps, 3], advanced rng)."""
    rp = np.ascontiguousarray(row_ptr, dtype=np.int32)
    cl = np.ascontiguousarray(col, dtype=np.int32)
    st = np.array(state, dtype=np.int8, copy=True)
    r = np.array(rng, dtype=np.uint32, copy=True)
    counts = np.zeros((steps, 3), dtype=np.int32)
    lib().orc_sir_run(_p(rp), _p(cl), ctypes.c_int64(st.size), _p(st), _p(r),
                      ctypes.c_int32(steps), ctypes.c_float(beta), ctypes.c_float(gamma),
                      _p(counts))
    return st, counts, r


def sir_run_many(graphs, states, rngs, steps, betas, gammas):
    """Many SIR runs at once (``graphs`` [(row_ptr, col)], ``states`` int8 arrays, ``rngs``
    uint32[k, 2]), the host threads taking whole instances.  Returns (final states, counts
    int32[k, steps, 3], advanced rngs), each equal to ``sir_run`` of that instance."""
    k = len(graphs)
    rps = [np.ascontiguousarray(g[0], dtype=np.int32) for g in graphs]
    cols = [np.ascontiguousarray(g[1], dtype=np.int32) for g in graphs]
    sts = [np.array(s, dtype=np.int8, copy=True) for s in states]
    r = np.array(rngs, dtype=np.uint32, copy=True).reshape(k, 2)
    counts = np.zeros((k, steps, 3), dtype=np.int32)
    ns = np.array([s.size for s in sts], dtype=np.int64)
    vp = ctypes.c_void_p * max(k, 1)
    lib().orc_sir_run_many(ctypes.c_int64(k), vp(*[a.ctypes.data for a in rps]),
                           vp(*[a.ctypes.data for a in cols]), _p(ns),
                           vp(*[a.ctypes.data for a in sts]), _p(r), ctypes.c_int32(steps),
                           _p(np.ascontiguousarray(betas, dtype=np.float32)),
                           _p(np.ascontiguousarray(gammas, dtype=np.float32)),
                           vp(*[counts[i].ctypes.data for i in range(k)]))
    return sts, counts, r


def schelling_run(pos, types, W, H, coll_keys, threshold=(3, 8)):
    """Schelling steps with the given per-step collection keys uint32[steps, 2]; an agent is
    unhappy iff den * same < num * occupied for ``threshold`` = (num, den).
    Returns (final positions, stats int32[steps, 2] = (unhappy, moved))."""
    p = np.array(pos, dtype=np.int32, copy=True)
    ty = np.ascontiguousarray(types, dtype=np.int8)
    ck = np.ascontiguousarray(coll_keys, dtype=np.uint32).reshape(-1, 2)
    steps = ck.shape[0]
    stats = np.zeros((steps, 2), dtype=np.int32)
    lib().orc_schelling_run(_p(p), _p(ty), ctypes.c_int64(p.size), ctypes.c_int32(W),
                            ctypes.c_int32(H), _p(ck), ctypes.c_int32(steps),
                            ctypes.c_int32(int(threshold[0])), ctypes.c_int32(int(threshold[1])),
                            _p(stats))
    return p, stats


def _params(dtype, *arrs):
    return [np.ascontiguousarray(a, dtype=dtype) for a in arrs]


def expf_tang(x):
    """float32 exp by the oracle's table-driven method (the forward's exponential)."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty_like(x)
    lib().orc_expf_tang_array(_p(x), _p(y), ctypes.c_int64(x.size))
    return y


def sigmoid32(z):
    """float32 sigmoid 1 / (1 + exp(-z)) exactly as the float32 forward evaluates it."""
    z = np.ascontiguousarray(z, dtype=np.float32)
    s = np.empty_like(z)
    lib().orc_sigmoid32_array(_p(z), _p(s), ctypes.c_int64(z.size))
    return s


def exp2_table():
    out = np.empty(32, np.float32)
    lib().orc_exp2_table(_p(out))
    return out


def opinion_run_f32(o, row_ptr, col, mu, eps, tau, steps):
    """Float32 forward (the model's fixed operation sequence); o float32[n, B]."""
    x = np.array(o, dtype=np.float32, copy=True, order="C")
    n, B = x.shape
    rp, cl = _params(np.int32, row_ptr, col)
    m, e, t = _params(np.float32, mu, eps, tau)
    lib().orc_opinion_run_f32(_p(x), _p(rp), _p(cl), ctypes.c_int64(n), ctypes.c_int32(B),
                              _p(m), _p(e), _p(t), ctypes.c_int32(steps))
    return x


def opinion_run_f64(o, row_ptr, col, mu, eps, tau, steps):
    x = np.array(o, dtype=np.float64, copy=True, order="C")
    n, B = x.shape
    rp, cl = _params(np.int32, row_ptr, col)
    m, e, t = _params(np.float64, mu, eps, tau)
    lib().orc_opinion_run_f64(_p(x), _p(rp), _p(cl), ctypes.c_int64(n), ctypes.c_int32(B),
                              _p(m), _p(e), _p(t), ctypes.c_int32(steps))
    return x


def opinion_moments_f64(o):
    x = np.ascontiguousarray(o, dtype=np.float64)
    n, B = x.shape
    m = np.zeros((B, 4))
    lib().orc_opinion_moments_f64(_p(x), ctypes.c_int64(n), ctypes.c_int32(B), _p(m))
    return m


def opinion_grad_f64(o0, row_ptr, col, mu, eps, tau, steps, target):
    """(loss float64[B], grads float64[B, 3]) by the float64 reverse sweep."""
    x = np.ascontiguousarray(o0, dtype=np.float64)
    n, B = x.shape
    rp, cl = _params(np.int32, row_ptr, col)
    m, e, t = _params(np.float64, mu, eps, tau)
    tg = np.ascontiguousarray(target, dtype=np.float64)
    loss = np.zeros(B)
    grads = np.zeros((B, 3))
    lib().orc_opinion_grad_f64(_p(x), _p(rp), _p(cl), ctypes.c_int64(n), ctypes.c_int32(B),
                               _p(m), _p(e), _p(t), ctypes.c_int32(steps), _p(tg), _p(loss),
                               _p(grads))
    return loss, grads


def opinion_grad_f64_along_f32(o0, row_ptr, col, mu, eps, tau, steps, target):
    """(loss float64[B], grads float64[B, 3]) by the float64 reverse sweep along the float32
    trajectory (the states the float32 forward visits, widened to float64)."""
    x = np.ascontiguousarray(o0, dtype=np.float32)
    n, B = x.shape
    rp, cl = _params(np.int32, row_ptr, col)
    m, e, t = _params(np.float32, mu, eps, tau)
    tg = np.ascontiguousarray(target, dtype=np.float64)
    loss = np.zeros(B)
    grads = np.zeros((B, 3))
    lib().orc_opinion_grad_f64_along_f32(_p(x), _p(rp), _p(cl), ctypes.c_int64(n),
                                         ctypes.c_int32(B), _p(m), _p(e), _p(t),
                                         ctypes.c_int32(steps), _p(tg), _p(loss), _p(grads))
    return loss, grads
