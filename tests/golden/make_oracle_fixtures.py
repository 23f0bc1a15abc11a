"""Writes tests/golden/oracle_small_cases.npz: small SIR, Schelling and random-walk runs
computed by the direct NumPy statements of the rules (oracle/models.py).

The reference runs on JAX, which is not installed, so these vectors are not reference
outputs: they freeze the oracle's own statement of the rules (a regression fixture for the
oracle, also checked against the C oracle that the GPU tests use).  Regenerate from the
repository root with ``python tests/golden/make_oracle_fixtures.py``.
"""

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import models  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_small_cases.npz")


def small_graph(n=60, m=3, seed=11):
    """Seeded symmetric CSR: node i >= m links to m distinct earlier nodes."""
    rs = np.random.RandomState(seed)
    rows = [set() for _ in range(n)]
    for i in range(m, n):
        for j in rs.choice(i, size=m, replace=False):
            rows[i].add(int(j))
            rows[int(j)].add(i)
    rp = np.zeros(n + 1, dtype=np.int32)
    rp[1:] = np.cumsum([len(r) for r in rows])
    col = np.array([c for r in rows for c in sorted(r)], dtype=np.int32)
    return rp, col


def cases():
    out = {}
    # SIR: 60 agents, 3 infected, beta 0.15, gamma 0.1, 15 steps, seed 5
    rp, col = small_graph()
    st0 = np.zeros(60, dtype=np.int8)
    st0[[3, 17, 42]] = 1
    rng, _ = models.model_keys(5, 1)
    st, counts, rng_out = models.sir_run(rp, col, st0, rng, 15, 0.15, 0.1)
    out.update(sir_row_ptr=rp, sir_col=col, sir_state0=st0, sir_seed=np.int64(5),
               sir_beta=np.float32(0.15), sir_gamma=np.float32(0.1), sir_steps=np.int64(15),
               sir_state=st, sir_counts=counts, sir_rng=rng_out)
    # Schelling: 10 x 10 torus, 80 agents (first half type 0), 6 steps, seed 3
    rs = np.random.RandomState(3)
    pos0 = rs.permutation(100)[:80].astype(np.int32)
    types = (np.arange(80) >= 40).astype(np.int8)
    rng, _ = models.model_keys(3, 1)
    ck, _ = models.keychain(rng, 6, 1)
    pos, stats = models.schelling_run(pos0, types, 10, 10, ck.reshape(6, 2))
    out.update(sch_pos0=pos0, sch_types=types, sch_W=np.int64(10), sch_H=np.int64(10),
               sch_coll_keys=ck.reshape(6, 2), sch_pos=pos, sch_stats=stats)
    # random walk: 100 agents, 5 steps, sigma 0.01, seed 0
    x, y, means = models.randomwalk_run(0, 100, 5)
    out.update(rw_x=x, rw_y=y, rw_means=means)
    return out


if __name__ == "__main__":
    np.savez_compressed(OUT, **cases())
    print("wrote", OUT)
