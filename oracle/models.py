"""NumPy restatement of the reference's step semantics for the workload models.

TEST INFRASTRUCTURE ONLY (the checker; never imported by the shipped package).

Parity status: model trajectories are UNPINNED against the reference (JAX absent, no
reference golden trajectories exist); the key chain and samplers come from
``oracle/threefry.py``, which is pinned against published known-answer values.

The reference semantics restated here:

* ``Model.initialize`` (jaxabm/model.py:118-144): ``keys = split(PRNGKey(seed), C + 1)``,
  ``rng = keys[0]``, collection ``i`` initialises from ``keys[i + 1]``.
* ``AgentCollection.init`` (jaxabm/agent.py:113-128): per-agent keys ``split(key, N)``.
* ``Model.step`` (jaxabm/model.py:155-168): ``rng, step_key = split(rng)``; per collection
  ``step_key, coll_key = split(step_key)``; ``AgentCollection.update`` gives agent ``i``
  the key ``split(coll_key, N)[i]`` (jaxabm/agent.py:156) and updates all agents from the
  pre-step states (synchronous ``vmap``, jaxabm/agent.py:168-177).
"""

import numpy as np

from . import threefry as tfy


def model_keys(seed, ncoll=1):
    """(rng after initialize, [collection init keys])."""
    keys = tfy.split(tfy.PRNGKey(seed), ncoll + 1)
    return keys[0].copy(), [keys[i + 1].copy() for i in range(ncoll)]


def keychain(rng, steps, ncoll=1):
    """Collection keys uint32[steps, ncoll, 2] of ``steps`` Model.step calls, and the
    advanced rng."""
    rng = np.asarray(rng, dtype=np.uint32).copy()
    out = np.zeros((steps, ncoll, 2), dtype=np.uint32)
    for t in range(steps):
        k = tfy.split(rng, 2)
        rng, step_key = k[0], k[1]
        for c in range(ncoll):
            k = tfy.split(step_key, 2)
            step_key, out[t, c] = k[0], k[1]
    return out, rng


def agent_keys(coll_key, n):
    return tfy.split(coll_key, n)


# ---- random walk ------------------------------------------------------------------------
# Agent (jx.Agent form):
#   setup(key):  kx, ky = split(key); {'x': uniform(kx), 'y': uniform(ky)}
#   step(model_state, key): kx, ky = split(key)
#       x = (x + sigma * normal(kx)) % 1.0 ; y likewise


def randomwalk_init(init_key, n):
    ak = agent_keys(init_key, n)
    sub = tfy.split_batched(ak, 2)                 # [n, 2, 2]
    x = tfy.bits_to_unit_float(tfy.bits_batched(sub[:, 0], 1)[:, 0])
    y = tfy.bits_to_unit_float(tfy.bits_batched(sub[:, 1], 1)[:, 0])
    return x, y


def _mod1_f32(v):
    r = np.fmod(v, np.float32(1.0)).astype(np.float32)
    neg = (r != 0) & (r < 0)
    r[neg] = (r[neg] + np.float32(1.0)).astype(np.float32)
    return r


def randomwalk_step(x, y, coll_key, sigma=0.01):
    n = x.shape[0]
    ak = agent_keys(coll_key, n)
    sub = tfy.split_batched(ak, 2)
    nx = tfy.normal_from_bits(tfy.bits_batched(sub[:, 0], 1)[:, 0])
    ny = tfy.normal_from_bits(tfy.bits_batched(sub[:, 1], 1)[:, 0])
    s = np.float32(sigma)
    x = _mod1_f32((x + (s * nx).astype(np.float32)).astype(np.float32))
    y = _mod1_f32((y + (s * ny).astype(np.float32)).astype(np.float32))
    return x, y


def randomwalk_run(seed, n, steps, sigma=0.01):
    """Full run from a seed: returns (x, y, means float64[steps, 2])."""
    rng, (ik,) = model_keys(seed, 1)
    x, y = randomwalk_init(ik, n)
    ck, rng = keychain(rng, steps, 1)
    means = np.zeros((steps, 2))
    for t in range(steps):
        x, y = randomwalk_step(x, y, ck[t, 0], sigma)
        means[t] = (x.astype(np.float64).mean(), y.astype(np.float64).mean())
    return x, y, means


# ---- SIR on a network --------------------------------------------------------------------
# Agent (jx.Agent form), agent_key = split(coll_key, N)[i]:
#   k_inf, k_rec = split(agent_key)
#   S: becomes I if, for some CSR slot k of its row whose neighbour is I,
#      uniform(k_inf, (deg,))[k] < beta
#   I: becomes R if uniform(k_rec) < gamma
#   R: stays R
# Every agent reads the pre-step compartments (jaxabm/agent.py:168-177); the S, I, R counts
# after each step are the metrics.  This is the direct (dense) statement of the rule: every
# agent evaluates its own draws, whatever its neighbours are.  The C oracle uses the same
# rule; the GPU kernels evaluate it only where it can change a compartment.


def sir_step(state, row_ptr, col, coll_key, beta, gamma):
    """One synchronous SIR step (small cases: a Python loop over agents)."""
    st = np.asarray(state, dtype=np.int8)
    n = st.size
    beta32, gamma32 = np.float32(beta), np.float32(gamma)
    akeys = agent_keys(np.asarray(coll_key, dtype=np.uint32), n)
    new = st.copy()
    for i in range(n):
        if st[i] == 2:
            continue
        k_inf, k_rec = tfy.split(akeys[i], 2)
        if st[i] == 1:
            if tfy.uniform(k_rec, ()) < gamma32:
                new[i] = 2
            continue
        r0, r1 = int(row_ptr[i]), int(row_ptr[i + 1])
        if r1 == r0:
            continue
        infected_nb = st[np.asarray(col[r0:r1], dtype=np.int64)] == 1
        if infected_nb.any():
            u = tfy.uniform(k_inf, (r1 - r0,))
            if np.any(infected_nb & (u < beta32)):
                new[i] = 1
    return new


def sir_run(row_ptr, col, state, rng, steps, beta, gamma):
    """``steps`` SIR steps from compartments ``state`` and the model rng (after
    ``Model.initialize``).  Returns (final compartments, counts int32[steps, 3], rng)."""
    ck, rng_out = keychain(rng, steps, 1)
    st = np.array(state, dtype=np.int8, copy=True)
    counts = np.zeros((steps, 3), dtype=np.int32)
    for t in range(steps):
        st = sir_step(st, row_ptr, col, ck[t, 0], beta, gamma)
        counts[t] = [(st == 0).sum(), (st == 1).sum(), (st == 2).sum()]
    return st, counts, rng_out


# ---- Schelling segregation on a torus grid ----------------------------------------------
# Cell (x, y) of a W x H torus has index x*H + y.  Each step, from the pre-step layout:
#   an agent is unhappy iff den * (same-type Moore neighbours) < num * (occupied neighbours)
#   for the threshold num/den (the workload: 3/8);
#   an unhappy agent i draws idx = min(floor(f32(uniform(agent_key) * e)), e - 1) into the
#   ascending list of the e empty cells (agent_key = split(coll_key, N)[i]; one correctly
#   rounded float32 multiply) and claims that cell; the lowest claiming id wins and moves,
#   the others stay.  Metrics: (unhappy agents, moved agents).


def schelling_step(pos, types, W, H, coll_key, threshold=(3, 8)):
    """One Schelling step (small cases).  Returns (new positions, (unhappy, moved))."""
    num, den = threshold
    pos = np.asarray(pos, dtype=np.int64)
    types = np.asarray(types, dtype=np.int64)
    n = pos.size
    grid = np.full(W * H, -1, dtype=np.int64)
    grid[pos] = types
    empty = np.nonzero(grid < 0)[0]
    e = empty.size
    akeys = agent_keys(np.asarray(coll_key, dtype=np.uint32), n)
    claims = {}
    unhappy = 0
    for i in range(n):
        x, y = divmod(int(pos[i]), H)
        same = occ = 0
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                if dx == 0 and dy == 0:
                    continue
                c = grid[((x + dx) % W) * H + (y + dy) % H]
                if c >= 0:
                    occ += 1
                    same += int(c == types[i])
        if den * same < num * occ:
            unhappy += 1
            if e == 0:
                continue
            u = np.float32(tfy.uniform(akeys[i], ()))
            idx = min(int(np.floor(np.float32(u * np.float32(e)))), e - 1)
            cell = int(empty[idx])
            if cell not in claims or i < claims[cell]:
                claims[cell] = i
    new = pos.copy()
    for cell, i in claims.items():
        new[i] = cell
    return new.astype(np.int32), (unhappy, len(claims))


def schelling_run(pos, types, W, H, coll_keys, threshold=(3, 8)):
    """Schelling steps with per-step collection keys uint32[steps, 2].  Returns (final
    positions, stats int32[steps, 2] = (unhappy, moved))."""
    ck = np.asarray(coll_keys, dtype=np.uint32).reshape(-1, 2)
    p = np.asarray(pos, dtype=np.int32).copy()
    stats = np.zeros((ck.shape[0], 2), dtype=np.int32)
    for t in range(ck.shape[0]):
        p, stats[t] = schelling_step(p, types, W, H, ck[t], threshold)
    return p, stats


# ---- bounded-confidence opinion dynamics --------------------------------------------------
# Per step, from the pre-step opinions o (every instance b its own mu, eps, tau):
#   o_i += mu * (sum over neighbours j of s_ij * d_ij) / deg_i,
#   d_ij = o_j - o_i,  s_ij = sigmoid((eps - |d_ij|) / tau)


def opinion_step_f64(o, row_ptr, col, mu, eps, tau):
    """One synchronous step in float64; o float64[n, B]; mu, eps, tau float64[B]."""
    o = np.asarray(o, dtype=np.float64)
    n = o.shape[0]
    deg = np.diff(np.asarray(row_ptr, dtype=np.int64))
    src = np.repeat(np.arange(n), deg)
    d = o[np.asarray(col, dtype=np.int64)] - o[src]
    s = 1.0 / (1.0 + np.exp(-(np.asarray(eps) - np.abs(d)) / np.asarray(tau)))
    acc = np.zeros_like(o)
    np.add.at(acc, src, s * d)
    return o + np.asarray(mu) * acc / np.maximum(deg, 1)[:, None]


def opinion_run_f64(o, row_ptr, col, mu, eps, tau, steps):
    x = np.array(o, dtype=np.float64, copy=True)
    for _ in range(steps):
        x = opinion_step_f64(x, row_ptr, col, mu, eps, tau)
    return x
