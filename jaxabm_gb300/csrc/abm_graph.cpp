// Host-side network construction for Network environments (native setup code).
//
// The reference builds networks edge by edge with an O(E) concatenation per edge
// (Network.add_edge, jaxabm/agentpy.py:559-582), which is infeasible at millions of edges.
// These generators write CSR adjacency (row_ptr int32[n+1], col int32[E]) directly into
// caller-provided HOST buffers, deterministically from a 64-bit seed on any platform.

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/jaxabm_gb300.h"

namespace {

// splitmix64 (Steele, Lea, Flood, "Fast splittable pseudorandom number generators",
// OOPSLA 2014): a pure-integer stream, identical on every platform.
struct SplitMix64 {
  uint64_t s;
  explicit SplitMix64(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  // uniform integer in [0, bound) by the multiply-shift method (bias < bound / 2^64)
  uint64_t below(uint64_t bound) {
    return (uint64_t)(((unsigned __int128)next() * bound) >> 64);
  }
};

// Undirected edge list (u, v) -> symmetric CSR with each row sorted ascending.
int edges_to_csr(int64_t n, const std::vector<int32_t>& eu, const std::vector<int32_t>& ev,
                 int32_t* row_ptr, int32_t* col, int64_t col_capacity) {
  const int64_t m = (int64_t)eu.size();
  if (2 * m > col_capacity || 2 * m > 0x7FFFFFFFll) return ABM_ERR_BADARG;
  std::vector<int64_t> deg(n + 1, 0);
  for (int64_t e = 0; e < m; ++e) {
    ++deg[eu[e]];
    ++deg[ev[e]];
  }
  row_ptr[0] = 0;
  for (int64_t i = 0; i < n; ++i) row_ptr[i + 1] = (int32_t)(row_ptr[i] + deg[i]);
  std::vector<int64_t> fill(row_ptr, row_ptr + n);
  for (int64_t e = 0; e < m; ++e) {
    col[fill[eu[e]]++] = ev[e];
    col[fill[ev[e]]++] = eu[e];
  }
  for (int64_t i = 0; i < n; ++i) std::sort(col + row_ptr[i], col + row_ptr[i + 1]);
  return ABM_OK;
}

}  // namespace

extern "C" {

int64_t abm_graph_ba_num_edges(int64_t n, int32_t m) {
  if (n <= 0 || m <= 0 || n <= m) return -1;
  return 2 * (int64_t)m * (n - m);
}

int abm_graph_barabasi_albert(int64_t n, int32_t m, uint64_t seed, int32_t* row_ptr,
                              int32_t* col, int64_t col_capacity) {
  if (!row_ptr || !col || n <= 0 || m <= 0 || n <= m || n > 0x7FFFFFFFll) return ABM_ERR_BADARG;
  const int64_t undirected = (int64_t)m * (n - m);
  std::vector<int32_t> eu, ev;
  eu.reserve(undirected);
  ev.reserve(undirected);
  // start: star on nodes 0..m with centre 0
  std::vector<int32_t> repeated;
  repeated.reserve(2 * undirected);
  for (int32_t v = 1; v <= m; ++v) {
    eu.push_back(0);
    ev.push_back(v);
    repeated.push_back(0);
    repeated.push_back(v);
  }
  SplitMix64 rng(seed);
  std::vector<int32_t> targets(m);
  for (int64_t src = m + 1; src < n; ++src) {
    // m distinct targets drawn uniformly from the degree-weighted node list
    int32_t k = 0;
    while (k < m) {
      const int32_t cand = repeated[rng.below(repeated.size())];
      bool dup = false;
      for (int32_t j = 0; j < k; ++j) dup |= targets[j] == cand;
      if (!dup) targets[k++] = cand;
    }
    for (int32_t j = 0; j < m; ++j) {
      eu.push_back((int32_t)src);
      ev.push_back(targets[j]);
      repeated.push_back(targets[j]);
      repeated.push_back((int32_t)src);
    }
  }
  return edges_to_csr(n, eu, ev, row_ptr, col, col_capacity);
}

int abm_graph_random_regular(int64_t n, int32_t d, uint64_t seed, int32_t* row_ptr,
                             int32_t* col, int64_t col_capacity) {
  // Union of d/2 edge-disjoint random Hamiltonian cycles.  Each cycle walks a random node
  // order; when the next edge would repeat an existing one, a later node whose edge is new
  // is swapped into the next position.  A cycle that cannot be closed is rolled back and
  // redrawn.  The result is simple and exactly d-regular (d even, n > 2d).
  if (!row_ptr || !col || n <= 2 * (int64_t)d || d <= 0 || (d & 1) || n > 0x7FFFFFFFll)
    return ABM_ERR_BADARG;
  SplitMix64 rng(seed);
  std::vector<int32_t> eu, ev;
  eu.reserve((int64_t)n * d / 2);
  ev.reserve((int64_t)n * d / 2);
  std::vector<std::vector<int32_t>> adj(n);
  for (auto& a : adj) a.reserve(d);
  auto has_edge = [&](int32_t a, int32_t b) {
    for (int32_t x : adj[a])
      if (x == b) return true;
    return false;
  };
  auto add = [&](int32_t a, int32_t b) {
    adj[a].push_back(b);
    adj[b].push_back(a);
  };
  std::vector<int32_t> order(n);
  for (int32_t c = 0; c < d / 2; ++c) {
    for (int attempt = 0;; ++attempt) {
      if (attempt > 64) return ABM_ERR_BADARG;
      for (int64_t i = 0; i < n; ++i) order[i] = (int32_t)i;
      for (int64_t i = n - 1; i > 0; --i) std::swap(order[i], order[rng.below(i + 1)]);
      int64_t made = 0;
      bool ok = true;
      for (int64_t i = 0; i + 1 < n; ++i) {
        if (has_edge(order[i], order[i + 1])) {
          int64_t j = i + 2;
          while (j < n && has_edge(order[i], order[j])) ++j;
          if (j >= n) {
            ok = false;
            break;
          }
          std::swap(order[i + 1], order[j]);
        }
        add(order[i], order[i + 1]);
        ++made;
      }
      if (ok && has_edge(order[n - 1], order[0])) ok = false;
      if (ok) {
        add(order[n - 1], order[0]);
        for (int64_t i = 0; i < n; ++i) {
          eu.push_back(order[i]);
          ev.push_back(order[(i + 1) % n]);
        }
        break;
      }
      for (int64_t i = 0; i < made; ++i) {  // roll back this cycle's edges
        adj[order[i]].pop_back();
        adj[order[i + 1]].pop_back();
      }
    }
  }
  return edges_to_csr(n, eu, ev, row_ptr, col, col_capacity);
}

}  // extern "C"
