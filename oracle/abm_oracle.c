/*
 * CPU oracle of the agent-step path, plain C + OpenMP.
 *
 * TEST INFRASTRUCTURE ONLY: linked by tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py as the checker, never by the shipped library.
 *
 * Parity status: the threefry2x32 / jax.random layer is pinned against published
 * known-answer values (see oracle/threefry.py and tests/test_oracle_threefry.py);
 * model trajectories are UNPINNED against the reference, because the reference runs on
 * the third-party package `jax` (absent here) and ships no golden trajectories.  The
 * models follow the reference call sites cited at each function.
 *
 * Build: oracle/build.py (gcc -O2 -fopenmp -ffp-contract=off).  -ffp-contract=off keeps
 * every float32 multiply and add separately rounded, like the JAX expressions restated.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "abm_oracle_common.h"

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* ---- jax.random primitives ---------------------------------------------------------- */
void orc_threefry(const uint32_t* k, const uint32_t* c0, const uint32_t* c1, int64_t n,
                  uint32_t* y0, uint32_t* y1) {
  for (int64_t i = 0; i < n; ++i) tf(k[0], k[1], c0[i], c1[i], &y0[i], &y1[i]);
}

/* Model.step key chain (jaxabm/model.py:155-168), partitionable mode. */
void orc_keychain(uint32_t* rng, int32_t ncoll, int32_t steps, uint32_t* coll_keys) {
  key_t2 r = {rng[0], rng[1]};
  for (int32_t t = 0; t < steps; ++t) {
    key_t2 step_key = split_at(r, 1);
    r = split_at(r, 0);
    for (int32_t c = 0; c < ncoll; ++c) {
      key_t2 ck = split_at(step_key, 1);
      step_key = split_at(step_key, 0);
      coll_keys[2 * ((int64_t)t * ncoll + c)] = ck.a;
      coll_keys[2 * ((int64_t)t * ncoll + c) + 1] = ck.b;
    }
  }
  rng[0] = r.a;
  rng[1] = r.b;
}

/* ---- random walk -------------------------------------------------------------------- */
/* AgentCollection.init (jaxabm/agent.py:113-128) of the random-walk agent. */
void orc_randomwalk_init(float* x, float* y, int64_t n, const uint32_t* init_key) {
  const key_t2 k = {init_key[0], init_key[1]};
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    const key_t2 ak = split_at(k, (uint64_t)i);
    x[i] = unit_float(bits_at(split_at(ak, 0), 0));
    y[i] = unit_float(bits_at(split_at(ak, 1), 0));
  }
}

/* JaxModel.run loop (jaxabm/model.py:240-241) over AgentCollection.update
 * (jaxabm/agent.py:156-177) of the random-walk agent, float32 state, plus the float64
 * means of the float32 states after every step.  xd/yd (optional) carry the same walk in
 * float64 arithmetic with float64 normals from the same bits. */
void orc_randomwalk_run(float* x, float* y, double* xd, double* yd, int64_t n,
                        const uint32_t* coll_keys, int32_t steps, float sigma, double* means,
                        double* means_f64) {
  for (int32_t t = 0; t < steps; ++t) {
    const key_t2 ck = {coll_keys[2 * t], coll_keys[2 * t + 1]};
    double sx = 0.0, sy = 0.0, sxd = 0.0, syd = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : sx, sy, sxd, syd)
    for (int64_t i = 0; i < n; ++i) {
      const key_t2 ak = split_at(ck, (uint64_t)i);
      const uint32_t bx = bits_at(split_at(ak, 0), 0);
      const uint32_t by = bits_at(split_at(ak, 1), 0);
      float dx = sigma * normal_from_bits(bx);
      float dy = sigma * normal_from_bits(by);
      x[i] = mod1f(x[i] + dx);
      y[i] = mod1f(y[i] + dy);
      sx += x[i];
      sy += y[i];
      if (xd) {
        xd[i] = mod1d(xd[i] + (double)sigma * normal_from_bits_f64(bx));
        yd[i] = mod1d(yd[i] + (double)sigma * normal_from_bits_f64(by));
        sxd += xd[i];
        syd += yd[i];
      }
    }
    means[2 * t] = sx / (double)n;
    means[2 * t + 1] = sy / (double)n;
    if (means_f64) {
      means_f64[2 * t] = sxd / (double)n;
      means_f64[2 * t + 1] = syd / (double)n;
    }
  }
}

/* ---- SIR on a network ----------------------------------------------------------------
 * One Model.step per iteration (jaxabm/model.py:146-216) with the SIR agent update:
 * coll_key = split(split(rng)[1])[1]; agent_key_i = split(coll_key, n)[i];
 * k_inf, k_rec = split(agent_key_i); S -> I if any I-neighbour slot k has
 * uniform(k_inf, (deg,))[k] < beta; I -> R if uniform(k_rec) < gamma; rng = split(rng)[0].
 * state int8[n] in/out; counts int32[steps][3] (S, I, R after each step). */
void orc_sir_run(const int32_t* rp, const int32_t* col, int64_t n, int8_t* state, uint32_t* rng,
                 int32_t steps, float beta, float gamma, int32_t* counts) {
  int8_t* cur = state;
  int8_t* nxt = (int8_t*)malloc((size_t)n);
  key_t2 r = {rng[0], rng[1]};
  for (int32_t t = 0; t < steps; ++t) {
    const key_t2 coll = split_at(split_at(r, 1), 1);
    int64_t cs = 0, ci = 0, cr = 0;
#pragma omp parallel for schedule(dynamic, 4096) reduction(+ : cs, ci, cr)
    for (int64_t i = 0; i < n; ++i) {
      const int8_t s = cur[i];
      int8_t ns = s;
      if (s == 0) {
        const int32_t row0 = rp[i], deg = rp[i + 1] - rp[i];
        int have = 0;
        key_t2 kinf = {0, 0};
        for (int32_t k = 0; k < deg; ++k) {
          if (cur[col[row0 + k]] == 1) {
            if (!have) {
              kinf = split_at(split_at(coll, (uint64_t)i), 0);
              have = 1;
            }
            if (unit_float(bits_at(kinf, (uint64_t)k)) < beta) {
              ns = 1;
              break;
            }
          }
        }
      } else if (s == 1) {
        const key_t2 krec = split_at(split_at(coll, (uint64_t)i), 1);
        if (unit_float(bits_at(krec, 0)) < gamma) ns = 2;
      }
      nxt[i] = ns;
      cs += ns == 0;
      ci += ns == 1;
      cr += ns == 2;
    }
    counts[3 * t] = (int32_t)cs;
    counts[3 * t + 1] = (int32_t)ci;
    counts[3 * t + 2] = (int32_t)cr;
    int8_t* tmp = cur;
    cur = nxt;
    nxt = tmp;
    r = split_at(r, 0);
  }
  if (cur != state) {
    memcpy(state, cur, (size_t)n);
    free(cur);
  } else {
    free(nxt);
  }
  rng[0] = r.a;
  rng[1] = r.b;
}

/* Many independent SIR models (an ensemble): the host threads take whole instances
 * (largest first, dynamic schedule) and each instance runs orc_sir_run on its thread
 * (the nested parallel loop inside runs with one thread), so small instances keep every
 * core busy.  Arrays of per-instance pointers and parameters; rngs uint32[ninst][2] and
 * states are updated in place as by orc_sir_run. */
void orc_sir_run_many(int64_t ninst, const int32_t* const* rps, const int32_t* const* cols,
                      const int64_t* ns, int8_t* const* states, uint32_t* rngs, int32_t steps,
                      const float* betas, const float* gammas, int32_t* const* counts) {
  int64_t* order = (int64_t*)malloc(sizeof(int64_t) * (size_t)(ninst > 0 ? ninst : 1));
  for (int64_t i = 0; i < ninst; ++i) order[i] = i;
  for (int64_t i = 1; i < ninst; ++i) { /* insertion sort by size, descending */
    const int64_t v = order[i];
    int64_t j = i;
    while (j > 0 && ns[order[j - 1]] < ns[v]) {
      order[j] = order[j - 1];
      --j;
    }
    order[j] = v;
  }
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t k = 0; k < ninst; ++k) {
    const int64_t i = order[k];
    orc_sir_run(rps[i], cols[i], ns[i], states[i], rngs + 2 * i, steps, betas[i], gammas[i],
                counts[i]);
  }
  free(order);
}
