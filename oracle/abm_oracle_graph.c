/*
 * CPU oracle of the network generators (TEST INFRASTRUCTURE ONLY: the checker and the
 * input builder of the CPU baseline; the shipped library has its own generator).
 *
 * The reference builds a Network edge by edge (Network.add_edge, jaxabm/agentpy.py:559-582)
 * and ships no generator; the workloads define their graphs as:
 *   - Barabasi-Albert with attachment m: a star on nodes 0..m with centre 0, then every new
 *     node src = m+1 .. n-1 draws m DISTINCT targets, each uniform over the list of edge
 *     endpoints so far (degree-weighted preferential attachment, Barabasi & Albert 1999),
 *     and its edges are appended to that list as (target, src) in draw order;
 *   - random d-regular (d even): the union of d/2 random Hamiltonian cycles, each drawn as
 *     a Fisher-Yates shuffle of 0..n-1 walked in order; where the next edge of the walk
 *     already exists, the first later node that gives a new edge is swapped in; a cycle
 *     whose walk or closing edge cannot be made new is dropped and redrawn.
 * Random numbers: splitmix64 (Steele, Lea & Flood, OOPSLA 2014); an integer below `bound`
 * is the high 64 bits of next() * bound (Lemire's multiply-shift).  Output is symmetric
 * CSR with every row in ascending order, built here by sorting (node, neighbour) keys.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  uint64_t state;
} orc_sm64;

static uint64_t sm64_next(orc_sm64* g) {
  g->state += 0x9E3779B97F4A7C15ull;
  uint64_t z = g->state;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static uint64_t sm64_below(orc_sm64* g, uint64_t bound) {
  const unsigned __int128 p = (unsigned __int128)sm64_next(g) * bound;
  return (uint64_t)(p >> 64);
}

static int cmp_u64(const void* a, const void* b) {
  const uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
  return (x > y) - (x < y);
}

/* Undirected edges (u[k], v[k]) -> CSR: both directions as (node << 32 | neighbour) keys,
 * sorted, then counted per node.  Returns 0, or -1 on a size problem. */
static int edges_csr(int64_t n, const int32_t* u, const int32_t* v, int64_t m, int32_t* row_ptr,
                     int32_t* col, int64_t cap) {
  if (2 * m > cap) return -1;
  uint64_t* keys = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)(2 * m + 1));
  if (!keys) return -1;
  for (int64_t k = 0; k < m; ++k) {
    keys[2 * k] = ((uint64_t)(uint32_t)u[k] << 32) | (uint32_t)v[k];
    keys[2 * k + 1] = ((uint64_t)(uint32_t)v[k] << 32) | (uint32_t)u[k];
  }
  qsort(keys, (size_t)(2 * m), sizeof(uint64_t), cmp_u64);
  memset(row_ptr, 0, sizeof(int32_t) * (size_t)(n + 1));
  for (int64_t k = 0; k < 2 * m; ++k) {
    row_ptr[(keys[k] >> 32) + 1]++;
    col[k] = (int32_t)(uint32_t)keys[k];
  }
  for (int64_t i = 0; i < n; ++i) row_ptr[i + 1] += row_ptr[i];
  free(keys);
  return 0;
}

int orc_graph_barabasi_albert(int64_t n, int32_t m, uint64_t seed, int32_t* row_ptr,
                              int32_t* col, int64_t cap) {
  if (n <= m || m <= 0) return -1;
  const int64_t nedges = (int64_t)m * (n - m);
  int32_t* u = (int32_t*)malloc(sizeof(int32_t) * (size_t)nedges);
  int32_t* v = (int32_t*)malloc(sizeof(int32_t) * (size_t)nedges);
  int32_t* ends = (int32_t*)malloc(sizeof(int32_t) * (size_t)(2 * nedges));
  int32_t* pick = (int32_t*)malloc(sizeof(int32_t) * (size_t)m);
  if (!u || !v || !ends || !pick) return -1;
  int64_t ne = 0, nend = 0;
  for (int32_t leaf = 1; leaf <= m; ++leaf) {
    u[ne] = 0;
    v[ne++] = leaf;
    ends[nend++] = 0;
    ends[nend++] = leaf;
  }
  orc_sm64 g = {seed};
  for (int64_t src = m + 1; src < n; ++src) {
    int32_t got = 0;
    while (got < m) {
      const int32_t c = ends[sm64_below(&g, (uint64_t)nend)];
      int fresh = 1;
      for (int32_t q = 0; q < got; ++q)
        if (pick[q] == c) fresh = 0;
      if (fresh) pick[got++] = c;
    }
    for (int32_t q = 0; q < m; ++q) {
      u[ne] = (int32_t)src;
      v[ne++] = pick[q];
      ends[nend++] = pick[q];
      ends[nend++] = (int32_t)src;
    }
  }
  const int rc = edges_csr(n, u, v, ne, row_ptr, col, cap);
  free(u);
  free(v);
  free(ends);
  free(pick);
  return rc;
}

/* Adjacency sets as fixed-width rows of d entries (the graph is at most d-regular). */
static int adj_has(const int32_t* adj, const int32_t* len, int32_t d, int32_t a, int32_t b) {
  for (int32_t k = 0; k < len[a]; ++k)
    if (adj[(int64_t)a * d + k] == b) return 1;
  return 0;
}

static void adj_link(int32_t* adj, int32_t* len, int32_t d, int32_t a, int32_t b) {
  adj[(int64_t)a * d + len[a]++] = b;
  adj[(int64_t)b * d + len[b]++] = a;
}

int orc_graph_random_regular(int64_t n, int32_t d, uint64_t seed, int32_t* row_ptr,
                             int32_t* col, int64_t cap) {
  if (d <= 0 || (d & 1) || n <= 2 * (int64_t)d) return -1;
  int32_t* adj = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n * d));
  int32_t* len = (int32_t*)calloc((size_t)n, sizeof(int32_t));
  int32_t* perm = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  int32_t* u = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n * d / 2));
  int32_t* v = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n * d / 2));
  if (!adj || !len || !perm || !u || !v) return -1;
  orc_sm64 g = {seed};
  int64_t ne = 0;
  for (int32_t cyc = 0; cyc < d / 2; ++cyc) {
    int tries = 0;
    for (;;) {
      if (++tries > 65) return -1;
      for (int64_t i = 0; i < n; ++i) perm[i] = (int32_t)i;
      for (int64_t i = n - 1; i > 0; --i) {
        const int64_t j = (int64_t)sm64_below(&g, (uint64_t)(i + 1));
        const int32_t t = perm[i];
        perm[i] = perm[j];
        perm[j] = t;
      }
      int64_t linked = 0;
      int ok = 1;
      for (int64_t i = 0; i + 1 < n && ok; ++i) {
        if (adj_has(adj, len, d, perm[i], perm[i + 1])) {
          int64_t j = i + 2;
          while (j < n && adj_has(adj, len, d, perm[i], perm[j])) ++j;
          if (j == n) {
            ok = 0;
            break;
          }
          const int32_t t = perm[i + 1];
          perm[i + 1] = perm[j];
          perm[j] = t;
        }
        adj_link(adj, len, d, perm[i], perm[i + 1]);
        ++linked;
      }
      if (ok && adj_has(adj, len, d, perm[n - 1], perm[0])) ok = 0;
      if (ok) {
        adj_link(adj, len, d, perm[n - 1], perm[0]);
        for (int64_t i = 0; i < n; ++i) {
          u[ne] = perm[i];
          v[ne++] = perm[(i + 1) % n];
        }
        break;
      }
      for (int64_t i = 0; i < linked; ++i) {  /* drop this walk's edges again */
        len[perm[i]]--;
        len[perm[i + 1]]--;
      }
    }
  }
  const int rc = edges_csr(n, u, v, ne, row_ptr, col, cap);
  free(adj);
  free(len);
  free(perm);
  free(u);
  free(v);
  return rc;
}
