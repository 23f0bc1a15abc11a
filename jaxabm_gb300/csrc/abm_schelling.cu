// Schelling segregation on a W x H torus Grid (K3 Moore-8 gather, K4 relocation).
//
// Cell (x, y) has index c = x * H + y (the (width, height) grid of Grid,
// jaxabm/agentpy.py:465-494); grid[c] = -1 empty, else the occupant's type (0/1);
// cell_agent[c] = occupant id or -1.  Agent semantics per step (partitionable jax.random,
// agent_key = split(coll_key, n)[i], jaxabm/agent.py:156):
//   occ  = occupied Moore-8 neighbours, same = those of the agent's type;
//   unhappy iff den * same < num * occ     (same/occ below the threshold num/den, exact in
//                                           integers; the workload's 37.5% is 3/8)
//   an unhappy agent draws idx = min(floor(uniform(agent_key) * e), e - 1) (one float32
//   multiply) into the pre-step list of the e empty cells in ascending cell order, and
//   claims that cell; of several claimants of one cell the lowest agent id moves, the
//   others stay.  Everyone reads the pre-step grid (synchronous update).
// Metrics per step: number of unhappy agents, number of agents that moved.
//
// Grids of up to 2^18 cells run every step in one thread-block cluster (below); larger
// grids take one step = four launches (no device-side waits anywhere):
//   scan    one CTA per grid row: rows x-1, x, x+1 staged in shared memory (torus halo),
//           unhappiness of every occupant, empty-cell count of the row
//   empties one CTA per row: exclusive prefix over the row counts, ordered warp-ballot
//           compaction of the row's empty cells into the empty list
//   claim   one thread per agent: draw, target, atomicMin claim on the target cell
//   resolve one thread per agent: the claim owner moves; claims are reset for next step

#include <cooperative_groups.h>

#include "abm_common.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int kRowThreads = 256;
constexpr int kAgentThreads = 256;
constexpr int32_t kNoClaim = 0x7F7F7F7F;  // byte-memset pattern 0x7F, above every agent id
constexpr int32_t kPending = -2;

__global__ void __launch_bounds__(kRowThreads)
schelling_scan_kernel(const int8_t* __restrict__ grid, const int32_t* __restrict__ cell_agent,
                      int32_t W, int32_t H, int32_t thr_num, int32_t thr_den,
                      int32_t* __restrict__ target, int32_t* __restrict__ row_empty,
                      int32_t* __restrict__ stats_t) {
  extern __shared__ int8_t rows[];  // 3 x H
  __shared__ int sred[2][kRowThreads / 32];
  const int x = blockIdx.x;
  const int xm = x == 0 ? W - 1 : x - 1, xp = x == W - 1 ? 0 : x + 1;
  for (int y = threadIdx.x; y < H; y += blockDim.x) {
    rows[y] = grid[(size_t)xm * H + y];
    rows[H + y] = grid[(size_t)x * H + y];
    rows[2 * H + y] = grid[(size_t)xp * H + y];
  }
  __syncthreads();
  int empties = 0, unhappy = 0;
  for (int y = threadIdx.x; y < H; y += blockDim.x) {
    const int8_t g = rows[H + y];
    if (g < 0) {
      ++empties;
      continue;
    }
    const int ym = y == 0 ? H - 1 : y - 1, yp = y == H - 1 ? 0 : y + 1;
    const int8_t nb[8] = {rows[ym], rows[y], rows[yp], rows[H + ym], rows[H + yp],
                          rows[2 * H + ym], rows[2 * H + y], rows[2 * H + yp]};
    int occ = 0, same = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      occ += nb[k] >= 0;
      same += nb[k] == g;
    }
    const bool u = thr_den * same < thr_num * occ;
    unhappy += u;
    target[cell_agent[(size_t)x * H + y]] = u ? kPending : -1;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  empties = abm::warp_sum(empties);
  unhappy = abm::warp_sum(unhappy);
  if (lane == 0) {
    sred[0][warp] = empties;
    sred[1][warp] = unhappy;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int e = 0, u = 0;
    for (int w = 0; w < (int)(blockDim.x / 32); ++w) {
      e += sred[0][w];
      u += sred[1][w];
    }
    row_empty[x] = e;
    if (u) atomicAdd(&stats_t[0], u);
  }
}

// Ordered compaction of empty cells: row x's empties go to [prefix(x), prefix(x+1)).
__global__ void __launch_bounds__(kRowThreads)
schelling_empties_kernel(const int8_t* __restrict__ grid, int32_t W, int32_t H,
                         const int32_t* __restrict__ row_empty, int32_t* __restrict__ empty_list,
                         int32_t* __restrict__ e_total) {
  __shared__ int swarp[kRowThreads / 32];
  __shared__ int sbase;
  const int x = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // exclusive prefix of the row counts (each CTA reads the rows before it)
  int part = 0;
  for (int r = threadIdx.x; r < x; r += blockDim.x) part += row_empty[r];
  part = abm::warp_sum(part);
  if (lane == 0) swarp[warp] = part;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < (int)(blockDim.x / 32); ++w) s += swarp[w];
    sbase = s;
    if (x == W - 1) *e_total = s + row_empty[x];
  }
  __syncthreads();
  int base = sbase;
  for (int y0 = 0; y0 < H; y0 += blockDim.x) {
    const int y = y0 + threadIdx.x;
    const bool empty = y < H && grid[(size_t)x * H + y] < 0;
    const unsigned ball = __ballot_sync(0xffffffffu, empty);
    if (lane == 0) swarp[warp] = __popc(ball);
    __syncthreads();
    int before = 0;
    for (int w = 0; w < warp; ++w) before += swarp[w];
    if (empty) empty_list[base + before + __popc(ball & ((1u << lane) - 1u))] = x * H + y;
    int chunk = 0;
    for (int w = 0; w < (int)(blockDim.x / 32); ++w) chunk += swarp[w];
    __syncthreads();
    base += chunk;
  }
}

__global__ void __launch_bounds__(kAgentThreads)
schelling_claim_kernel(int32_t n, const uint32_t* __restrict__ coll_key,
                       const int32_t* __restrict__ empty_list, const int32_t* __restrict__ e_total,
                       int32_t* __restrict__ target, int32_t* __restrict__ claim) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || target[i] != kPending) return;
  const int e = *e_total;
  if (e <= 0) {
    target[i] = -1;
    return;
  }
  const uint2 ak = abm::split_at(abm::load_key(coll_key), (uint64_t)i);
  const float u = abm::unit_float(abm::bits_at(ak, 0));
  int idx = (int)floorf(__fmul_rn(u, (float)e));
  if (idx > e - 1) idx = e - 1;
  const int tgt = empty_list[idx];
  target[i] = tgt;
  atomicMin(&claim[tgt], i);
}

__global__ void __launch_bounds__(kAgentThreads)
schelling_resolve_kernel(int32_t n, int8_t* __restrict__ grid, int32_t* __restrict__ cell_agent,
                         int32_t* __restrict__ pos, const int8_t* __restrict__ type,
                         const int32_t* __restrict__ target, int32_t* __restrict__ claim,
                         int32_t* __restrict__ stats_t) {
  __shared__ int swarp[kAgentThreads / 32];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int moved = 0;
  if (i < n) {
    const int tgt = target[i];
    if (tgt >= 0 && claim[tgt] == i) {
      const int old = pos[i];
      grid[old] = -1;
      cell_agent[old] = -1;
      grid[tgt] = type[i];
      cell_agent[tgt] = i;
      pos[i] = tgt;
      claim[tgt] = kNoClaim;
      moved = 1;
    }
  }
  moved = abm::warp_sum(moved);
  if ((threadIdx.x & 31) == 0) swarp[threadIdx.x >> 5] = moved;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < kAgentThreads / 32; ++w) s += swarp[w];
    if (s) atomicAdd(&stats_t[1], s);
  }
}

// ---- small grids: every step of the run in one thread-block cluster ----------------------
// A grid of up to kClusterMaxCells cells is handled by one cluster of kClusterCtas CTAs of
// 1024 threads for the whole run; the four phases of a step (scan, ordered empty list,
// claim, resolve) are separated by the hardware cluster barrier (release/acquire at cluster
// scope), which makes each phase's global writes visible to the next, so a step costs four
// barriers instead of four launches.  Thread g of the cluster owns the contiguous cells
// [g*chunk, (g+1)*chunk), read from the CTA's rows staged in shared memory with a halo row
// on each side; the empty list stays in ascending cell order (a block scan of the
// per-thread counts plus the lower-ranked CTAs' totals, read through distributed shared
// memory); unhappy agents go to a list (order free: claims are atomicMin), so the claim and
// resolve phases touch only them.  The arithmetic per agent is that of the four-kernel path.
// Cross-CTA data is read with L2-only loads.
constexpr int kClusterCtas = 8;
constexpr int kClusterThreads = 1024;
constexpr int kClusterWarps = kClusterThreads / 32;
constexpr int64_t kClusterMaxCells = int64_t(1) << 18;
constexpr size_t kClusterMaxRowBytes = 96 * 1024;  // staged rows per CTA (wide grids: launches)

__device__ __forceinline__ int block_sum(int v, int* sred) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = abm::warp_sum(v);
  if (lane == 0) sred[warp] = v;
  __syncthreads();
  int total = 0;
  if (warp == 0) {
    total = abm::warp_sum(lane < kClusterWarps ? sred[lane] : 0);
  }
  __syncthreads();
  return total;  // valid in thread 0
}

// One model's arrays for the cluster body.
struct ClusterModel {
  int32_t* pos;
  const int8_t* type;
  int32_t n;
  int8_t* grid;
  int32_t* cell_agent;
  const uint32_t* coll_keys;
  int32_t* stats;
  int32_t* target;
  int32_t* claim;
  int32_t* empty_list;
  int32_t* unhappy_list;
  int32_t* unhappy_count;
  int32_t thr_num, thr_den;
};

// Every step of one model on the calling cluster.  With `init`, the cluster first sets its
// claims to "no claim" and zeroes its statistics and counters (the batched launch, whose
// models have no host-side set-up); otherwise the host did that.
__device__ void schelling_cluster_body(const ClusterModel& Mdl, int32_t W, int32_t H,
                                       int32_t steps, bool init) {
  int32_t* __restrict__ pos = Mdl.pos;
  const int8_t* __restrict__ type = Mdl.type;
  int8_t* grid = Mdl.grid;
  int32_t* cell_agent = Mdl.cell_agent;
  const uint32_t* __restrict__ coll_keys = Mdl.coll_keys;
  int32_t* __restrict__ stats = Mdl.stats;
  int32_t* target = Mdl.target;
  int32_t* claim = Mdl.claim;
  int32_t* empty_list = Mdl.empty_list;
  int32_t* unhappy_list = Mdl.unhappy_list;
  int32_t* unhappy_count = Mdl.unhappy_count;
  const int32_t thr_num = Mdl.thr_num, thr_den = Mdl.thr_den;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ int8_t srows[];  // this CTA's grid rows with one halo row on each side
  __shared__ int swarp[kClusterWarps];
  __shared__ int sred[kClusterWarps];
  __shared__ int s_cta_total;  // empties in this CTA's cells, read by the other CTAs
  const unsigned rank = cluster.block_rank();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nthreads = kClusterCtas * kClusterThreads;
  const int g = (int)rank * kClusterThreads + tid;
  const int C = W * H;
  const int chunk = (C + nthreads - 1) / nthreads;
  const int c0 = min(g * chunk, C), c1 = min(c0 + chunk, C);
  // rows staged by this CTA: x_lo - 1 .. x_hi + 1 (torus), x_lo/x_hi the rows of its cells
  const int cta_c0 = min((int)rank * kClusterThreads * chunk, C);
  const int cta_c1 = min(cta_c0 + kClusterThreads * chunk, C);
  const int x_lo = cta_c0 / H;
  const int x_hi = cta_c1 > cta_c0 ? (cta_c1 - 1) / H : x_lo;
  const int nrows = x_hi - x_lo + 3;
  if (init) {
    for (int c = g; c < C; c += nthreads) claim[c] = kNoClaim;
    for (int k = g; k < 2 * steps; k += nthreads) stats[k] = 0;
    if (g < 2) unhappy_count[g] = 0;
    cluster.sync();
  }
  for (int t = 0; t < steps; ++t) {
    const int32_t* ucount = unhappy_count + (t & 1);
    if (g == 0) unhappy_count[(t + 1) & 1] = 0;  // the counter of the next step
    for (int k = tid; k < nrows * H; k += kClusterThreads) {
      const int r = k / H, y = k - r * H;
      int x = x_lo - 1 + r;
      x = x < 0 ? x + W : (x >= W ? x - W : x);
      srows[k] = __ldcg(grid + x * H + y);
    }
    __syncthreads();
    // scan: unhappiness of the occupants of my cells (neighbours from the staged rows),
    // unhappy agents to the cluster's list, and my empty cells
    int empties = 0, unhappy = 0;
    for (int c = c0; c < c1; ++c) {
      const int x = c / H, y = c - x * H;
      const int r = x - x_lo + 1;
      const int8_t gv = srows[r * H + y];
      if (gv < 0) {
        ++empties;
        continue;
      }
      const int ym = y == 0 ? H - 1 : y - 1, yp = y == H - 1 ? 0 : y + 1;
      const int8_t* up = srows + (r - 1) * H;
      const int8_t* mid = srows + r * H;
      const int8_t* dn = srows + (r + 1) * H;
      const int8_t nb[8] = {up[ym], up[y], up[yp], mid[ym], mid[yp], dn[ym], dn[y], dn[yp]};
      int occ = 0, same = 0;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        occ += nb[k] >= 0;
        same += nb[k] == gv;
      }
      if (thr_den * same < thr_num * occ) {
        ++unhappy;
        const int i = __ldcg(cell_agent + c);
        unhappy_list[atomicAdd(const_cast<int32_t*>(ucount), 1)] = i;
      }
    }
    // ordered position of my empties: block scan, then the lower-ranked CTAs' totals
    int incl = empties;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += u;
    }
    if (lane == 31) swarp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      int w = swarp[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += u;
      }
      swarp[lane] = w;
    }
    __syncthreads();
    const int excl = (warp > 0 ? swarp[warp - 1] : 0) + incl - empties;
    if (tid == kClusterThreads - 1) s_cta_total = excl + empties;
    const int u_cta = block_sum(unhappy, sred);
    if (tid == 0 && u_cta) atomicAdd(&stats[2 * t], u_cta);
    cluster.sync();  // (1) every CTA's total and every unhappy agent are in
    int base = 0, e_total = 0;
#pragma unroll
    for (int r = 0; r < kClusterCtas; ++r) {
      const int v = *cluster.map_shared_rank(&s_cta_total, r);
      base += r < (int)rank ? v : 0;
      e_total += v;
    }
    int pe = base + excl;
    for (int c = c0; c < c1; ++c) {
      const int x = c / H;
      if (srows[(x - x_lo + 1) * H + (c - x * H)] < 0) empty_list[pe++] = c;
    }
    cluster.sync();  // (2) the empty list is complete
    // claim: an unhappy agent draws an empty cell; the lowest id wins it
    const int nu = __ldcg(ucount);
    const uint2 ck = abm::load_key(coll_keys + 2 * (size_t)t);
    if (e_total > 0) {
      for (int k = g; k < nu; k += nthreads) {
        const int i = __ldcg(unhappy_list + k);
        const uint2 ak = abm::split_at(ck, (uint64_t)i);
        const float u = abm::unit_float(abm::bits_at(ak, 0));
        int idx = (int)floorf(__fmul_rn(u, (float)e_total));
        if (idx > e_total - 1) idx = e_total - 1;
        const int tgt = __ldcg(empty_list + idx);
        target[i] = tgt;
        atomicMin(&claim[tgt], i);
      }
    }
    cluster.sync();  // (3) every claim is in
    // resolve: the claim owner moves
    int moved = 0;
    if (e_total > 0) {
      for (int k = g; k < nu; k += nthreads) {
        const int i = __ldcg(unhappy_list + k);
        const int tgt = __ldcg(target + i);
        if (__ldcg(claim + tgt) == i) {
          const int old = pos[i];
          grid[old] = -1;
          cell_agent[old] = -1;
          grid[tgt] = type[i];
          cell_agent[tgt] = i;
          pos[i] = tgt;
          claim[tgt] = kNoClaim;
          ++moved;
        }
      }
    }
    const int m_cta = block_sum(moved, sred);
    if (tid == 0 && m_cta) atomicAdd(&stats[2 * t + 1], m_cta);
    cluster.sync();  // (4) the grid of the next step is complete; totals may be rewritten
  }
}

__global__ void __cluster_dims__(kClusterCtas, 1, 1) __launch_bounds__(kClusterThreads)
schelling_cluster_kernel(ClusterModel Mdl, int32_t W, int32_t H, int32_t steps) {
  schelling_cluster_body(Mdl, W, H, steps, false);
}

// Workspace layout of one model (abm_schelling_workspace_bytes), usable on both sides.
struct Workspace {
  int32_t* claim;
  int32_t* target;
  int32_t* row_empty;
  int32_t* empty_list;
  int32_t* unhappy_list;
  int32_t* e_total;
  int32_t* bad;
  int32_t* unhappy_count;  // two counters, one per step parity
};

__host__ __device__ inline size_t round256(size_t v) { return (v + 255) / 256 * 256; }

__host__ __device__ inline Workspace carve(void* ws, int64_t n, int32_t W, int32_t H) {
  char* p = static_cast<char*>(ws);
  const size_t C = (size_t)W * H;
  Workspace w;
  w.claim = reinterpret_cast<int32_t*>(p);
  p += round256(C * 4);
  w.target = reinterpret_cast<int32_t*>(p);
  p += round256((size_t)n * 4);
  w.row_empty = reinterpret_cast<int32_t*>(p);
  p += round256((size_t)W * 4);
  w.empty_list = reinterpret_cast<int32_t*>(p);
  p += round256(C * 4);
  w.unhappy_list = reinterpret_cast<int32_t*>(p);
  p += round256((size_t)n * 4);
  w.e_total = reinterpret_cast<int32_t*>(p);
  w.bad = w.e_total + 1;
  w.unhappy_count = w.e_total + 2;
  return w;
}

// Many models of one grid shape: cluster m runs member m (abm_schelling_member) entirely.
__global__ void __cluster_dims__(kClusterCtas, 1, 1) __launch_bounds__(kClusterThreads)
schelling_cluster_batch_kernel(const abm_schelling_member* __restrict__ members, int32_t W,
                               int32_t H, int32_t steps) {
  const abm_schelling_member& m = members[blockIdx.x / kClusterCtas];
  const Workspace w = carve(m.workspace, m.n, W, H);
  const ClusterModel Mdl{m.pos, m.type, (int32_t)m.n, m.grid, m.cell_agent, m.coll_keys,
                         m.stats, w.target, w.claim, w.empty_list, w.unhappy_list,
                         w.unhappy_count, m.thr_num, m.thr_den};
  schelling_cluster_body(Mdl, W, H, steps, true);
}

// Bytes of the staged rows of one CTA of schelling_cluster_kernel.
size_t cluster_smem_bytes(int32_t W, int32_t H) {
  const int64_t C = (int64_t)W * H;
  const int64_t chunk = (C + kClusterCtas * kClusterThreads - 1) / (kClusterCtas * kClusterThreads);
  const int64_t cells = chunk * kClusterThreads;          // cells per CTA
  return (size_t)((cells + H - 1) / H + 3) * (size_t)H;   // rows spanned + halo rows
}

// Grid and occupancy map from the agents' positions and types: clear, then place.
__global__ void schelling_clear_kernel(int32_t C, int8_t* __restrict__ grid,
                                       int32_t* __restrict__ cell_agent) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < C) {
    grid[g] = -1;
    cell_agent[g] = -1;
  }
}

__global__ void schelling_place_agents_kernel(int32_t n, int32_t C, const int32_t* __restrict__ pos,
                                              const int8_t* __restrict__ type,
                                              int8_t* __restrict__ grid,
                                              int32_t* __restrict__ cell_agent,
                                              int32_t* __restrict__ bad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = pos[i];
  if (c < 0 || c >= C || type[i] < 0) {
    atomicExch(bad, 1);
    return;
  }
  grid[c] = type[i];
  if (atomicExch(&cell_agent[c], i) != -1) atomicExch(bad, 1);  // two agents on one cell
}

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

}  // namespace

extern "C" {

size_t abm_schelling_workspace_bytes(int64_t n, int32_t W, int32_t H) {
  if (n <= 0 || W <= 0 || H <= 0) return 0;
  const size_t C = (size_t)W * H;
  return align256(C * 4) + align256((size_t)n * 4) + align256((size_t)W * 4) + align256(C * 4) +
         align256((size_t)n * 4) + 256;
}

int abm_schelling_place(const int32_t* pos, const int8_t* type, int64_t n, int32_t W, int32_t H,
                        int8_t* grid, int32_t* cell_agent, int32_t* status, void* stream) {
  if (!pos || !type || !grid || !cell_agent || !status || n <= 0 || W < 3 || H < 3 ||
      (int64_t)W * H > 0x7FFFFFFFll || n > (int64_t)W * H)
    return ABM_ERR_BADARG;
  cudaStream_t s = abm_host::as_stream(stream);
  const int C = W * H;
  int st = abm_host::record_cuda_error(cudaMemsetAsync(status, 0, sizeof(int32_t), s),
                                       "abm_schelling_place/memset");
  if (st) return st;
  schelling_clear_kernel<<<(C + 255) / 256, 256, 0, s>>>(C, grid, cell_agent);
  st = abm_host::check_launch("abm_schelling_place/clear");
  if (st) return st;
  schelling_place_agents_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
      (int32_t)n, C, pos, type, grid, cell_agent, status);
  return abm_host::check_launch("abm_schelling_place/agents");
}

namespace {
bool valid_threshold(int32_t num, int32_t den) {
  return den > 0 && num >= 0 && num <= (1 << 27) && den <= (1 << 27);
}
}  // namespace

int abm_schelling_run(int32_t* pos, const int8_t* type, int64_t n, int32_t W, int32_t H,
                      int8_t* grid, int32_t* cell_agent, const uint32_t* coll_keys, int32_t steps,
                      int32_t thr_num, int32_t thr_den, int32_t* stats, void* workspace,
                      size_t workspace_bytes, void* stream) {
  if (!pos || !type || !grid || !cell_agent || !coll_keys || !stats || n <= 0 || W < 3 ||
      H < 3 || (int64_t)W * H > 0x7FFFFFFFll || n > (int64_t)W * H || steps < 0 || H > 16384 ||
      !valid_threshold(thr_num, thr_den))
    return ABM_ERR_BADARG;
  if (!workspace || workspace_bytes < abm_schelling_workspace_bytes(n, W, H) ||
      !abm_host::aligned(workspace, 256))
    return ABM_ERR_WORKSPACE;
  if (steps == 0) return ABM_OK;
  cudaStream_t s = abm_host::as_stream(stream);
  Workspace w = carve(workspace, n, W, H);
  int st = abm_host::record_cuda_error(
      cudaMemsetAsync(stats, 0, sizeof(int32_t) * 2 * (size_t)steps, s), "abm_schelling_run/memset");
  if (st) return st;
  // every claim slot starts as "no claim" (0x7F7F7F7F exceeds every agent id)
  st = abm_host::record_cuda_error(
      cudaMemsetAsync(w.claim, 0x7F, sizeof(int32_t) * (size_t)W * H, s), "abm_schelling_run/claims");
  if (st) return st;
  if ((int64_t)W * H <= kClusterMaxCells && cluster_smem_bytes(W, H) <= kClusterMaxRowBytes) {
    // one cluster launch for the whole run
    st = abm_host::record_cuda_error(
        cudaMemsetAsync(w.unhappy_count, 0, 2 * sizeof(int32_t), s), "abm_schelling_run/counters");
    if (st) return st;
    const size_t rows_bytes = cluster_smem_bytes(W, H);  // <= kClusterMaxRowBytes
    cudaError_t e = cudaFuncSetAttribute(schelling_cluster_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)rows_bytes);
    if (e != cudaSuccess) return abm_host::record_cuda_error(e, "abm_schelling_run/cluster smem");
    const ClusterModel Mdl{pos, type, (int32_t)n, grid, cell_agent, coll_keys, stats, w.target,
                           w.claim, w.empty_list, w.unhappy_list, w.unhappy_count, thr_num,
                           thr_den};
    schelling_cluster_kernel<<<kClusterCtas, kClusterThreads, rows_bytes, s>>>(Mdl, W, H, steps);
    return abm_host::check_launch("abm_schelling_run/cluster");
  }
  const unsigned agent_blocks = (unsigned)((n + kAgentThreads - 1) / kAgentThreads);
  const size_t smem = 3 * (size_t)H;
  for (int32_t t = 0; t < steps; ++t) {
    int32_t* stats_t = stats + 2 * (size_t)t;
    schelling_scan_kernel<<<W, kRowThreads, smem, s>>>(grid, cell_agent, W, H, thr_num, thr_den,
                                                      w.target, w.row_empty, stats_t);
    if ((st = abm_host::check_launch("abm_schelling_run/scan"))) return st;
    schelling_empties_kernel<<<W, kRowThreads, 0, s>>>(grid, W, H, w.row_empty, w.empty_list,
                                                      w.e_total);
    if ((st = abm_host::check_launch("abm_schelling_run/empties"))) return st;
    schelling_claim_kernel<<<agent_blocks, kAgentThreads, 0, s>>>(
        (int32_t)n, coll_keys + 2 * (size_t)t, w.empty_list, w.e_total, w.target, w.claim);
    if ((st = abm_host::check_launch("abm_schelling_run/claim"))) return st;
    schelling_resolve_kernel<<<agent_blocks, kAgentThreads, 0, s>>>(
        (int32_t)n, grid, cell_agent, pos, type, w.target, w.claim, stats_t);
    if ((st = abm_host::check_launch("abm_schelling_run/resolve"))) return st;
  }
  return ABM_OK;
}

int abm_schelling_run_batch(const abm_schelling_member* members, int32_t count, int32_t W,
                            int32_t H, int32_t steps, void* stream) {
  if (!members || count <= 0 || count > 65535 / kClusterCtas || W < 3 || H < 3 || steps < 0 ||
      !abm_host::aligned(members, 8))
    return ABM_ERR_BADARG;
  if ((int64_t)W * H > kClusterMaxCells || cluster_smem_bytes(W, H) > kClusterMaxRowBytes)
    return ABM_ERR_BADARG;  // larger grids: abm_schelling_run per model
  if (steps == 0) return ABM_OK;
  const size_t rows_bytes = cluster_smem_bytes(W, H);
  cudaError_t e = cudaFuncSetAttribute(schelling_cluster_batch_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)rows_bytes);
  if (e != cudaSuccess) return abm_host::record_cuda_error(e, "abm_schelling_run_batch/smem");
  schelling_cluster_batch_kernel<<<count * kClusterCtas, kClusterThreads, rows_bytes,
                                   abm_host::as_stream(stream)>>>(members, W, H, steps);
  return abm_host::check_launch("abm_schelling_run_batch");
}

}  // extern "C"
