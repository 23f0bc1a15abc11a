/*
 * CPU oracle of the Schelling step (TEST INFRASTRUCTURE ONLY; the checker).
 * Parity status: UNPINNED against the reference -- the reference's Schelling agent is a
 * placeholder (examples/models/schelling_model.py:54-68: `satisfied = jnp.array([True])`,
 * agents never move), so the rule restated here is the workload's definition:
 *   unhappy iff den*same < num*occupied over the Moore-8 torus neighbours (same/occupied
 *   below the threshold num/den, e.g. 3/8 = 37.5%; the example's similarity_threshold,
 *   examples/models/schelling_model.py:36-40, as an exact fraction);
 *   unhappy agent i draws idx = min(floor(f32(uniform(split(coll_key, n)[i]) * e)), e-1)
 *   into the ascending pre-step empty-cell list; lowest claiming id moves.
 * Agents are visited in ascending id order, so "first claim wins" is "lowest id wins".
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "abm_oracle_common.h"

void orc_schelling_run(int32_t* pos, const int8_t* type, int64_t n, int32_t W, int32_t H,
                       const uint32_t* coll_keys, int32_t steps, int32_t thr_num,
                       int32_t thr_den, int32_t* stats) {
  const int64_t C = (int64_t)W * H;
  int8_t* grid = (int8_t*)malloc((size_t)C);
  int32_t* owner = (int32_t*)malloc(sizeof(int32_t) * (size_t)C);
  int32_t* empty = (int32_t*)malloc(sizeof(int32_t) * (size_t)C);
  int32_t* claim = (int32_t*)malloc(sizeof(int32_t) * (size_t)C);
  int32_t* target = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  memset(grid, -1, (size_t)C);
  for (int64_t i = 0; i < n; ++i) grid[pos[i]] = type[i];
  for (int64_t c = 0; c < C; ++c) claim[c] = -1;
  for (int32_t t = 0; t < steps; ++t) {
    const key_t2 ck = {coll_keys[2 * t], coll_keys[2 * t + 1]};
    int64_t e = 0;
    for (int64_t c = 0; c < C; ++c)
      if (grid[c] < 0) empty[e++] = (int32_t)c;
    int32_t unhappy = 0, moved = 0;
#pragma omp parallel for schedule(static) reduction(+ : unhappy)
    for (int64_t i = 0; i < n; ++i) {
      const int32_t x = pos[i] / H, y = pos[i] % H;
      const int8_t g = type[i];
      int occ = 0, same = 0;
      for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy) {
          if (!dx && !dy) continue;
          const int32_t xx = (x + dx + W) % W, yy = (y + dy + H) % H;
          const int8_t v = grid[(int64_t)xx * H + yy];
          occ += v >= 0;
          same += v == g;
        }
      target[i] = -1;
      if ((int64_t)thr_den * same < (int64_t)thr_num * occ) {
        ++unhappy;
        if (e > 0) {
          const float u = unit_float(bits_at(split_at(ck, (uint64_t)i), 0));
          const float prod = u * (float)e;
          int64_t idx = (int64_t)floorf(prod);
          if (idx > e - 1) idx = e - 1;
          target[i] = empty[idx];
        }
      }
    }
    for (int64_t i = 0; i < n; ++i)  /* ascending ids: the first claimant is the lowest */
      if (target[i] >= 0 && claim[target[i]] < 0) claim[target[i]] = (int32_t)i;
    for (int64_t i = 0; i < n; ++i) {
      const int32_t tg = target[i];
      if (tg >= 0 && claim[tg] == i) {
        grid[pos[i]] = -1;
        grid[tg] = type[i];
        pos[i] = tg;
        ++moved;
      }
    }
    for (int64_t i = 0; i < n; ++i)
      if (target[i] >= 0) claim[target[i]] = -1;
    stats[2 * t] = unhappy;
    stats[2 * t + 1] = moved;
  }
  free(grid);
  free(owner);
  free(empty);
  free(claim);
  free(target);
}
