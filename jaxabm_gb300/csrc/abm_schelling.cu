// Schelling segregation on a W x H torus Grid (K3 Moore-8 gather, K4 relocation).
//
// Cell (x, y) has index c = x * H + y (the (width, height) grid of Grid,
// jaxabm/agentpy.py:465-494); grid[c] = -1 empty, else the occupant's type (0/1);
// cell_agent[c] = occupant id or -1.  Agent semantics per step (partitionable jax.random,
// agent_key = split(coll_key, n)[i], jaxabm/agent.py:156):
//   occ  = occupied Moore-8 neighbours, same = those of the agent's type;
//   unhappy iff 8 * same < 3 * occ         (same/occ < 37.5%, exact in integers)
//   an unhappy agent draws idx = min(floor(uniform(agent_key) * e), e - 1) (one float32
//   multiply) into the pre-step list of the e empty cells in ascending cell order, and
//   claims that cell; of several claimants of one cell the lowest agent id moves, the
//   others stay.  Everyone reads the pre-step grid (synchronous update).
// Metrics per step: number of unhappy agents, number of agents that moved.
//
// One step = four launches (no device-side waits anywhere):
//   scan    one CTA per grid row: rows x-1, x, x+1 staged in shared memory (torus halo),
//           unhappiness of every occupant, empty-cell count of the row
//   empties one CTA per row: exclusive prefix over the row counts, ordered warp-ballot
//           compaction of the row's empty cells into the empty list
//   claim   one thread per agent: draw, target, atomicMin claim on the target cell
//   resolve one thread per agent: the claim owner moves; claims are reset for next step

#include "abm_common.cuh"

namespace {

constexpr int kRowThreads = 256;
constexpr int kAgentThreads = 256;
constexpr int32_t kNoClaim = 0x7F7F7F7F;  // byte-memset pattern 0x7F, above every agent id
constexpr int32_t kPending = -2;

__global__ void __launch_bounds__(kRowThreads)
schelling_scan_kernel(const int8_t* __restrict__ grid, const int32_t* __restrict__ cell_agent,
                      int32_t W, int32_t H, int32_t* __restrict__ target,
                      int32_t* __restrict__ row_empty, int32_t* __restrict__ stats_t) {
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
    const bool u = 8 * same < 3 * occ;
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

struct Workspace {
  int32_t* claim;
  int32_t* target;
  int32_t* row_empty;
  int32_t* empty_list;
  int32_t* e_total;
  int32_t* bad;
};

Workspace carve(void* ws, int64_t n, int32_t W, int32_t H) {
  char* p = static_cast<char*>(ws);
  const size_t C = (size_t)W * H;
  Workspace w;
  w.claim = reinterpret_cast<int32_t*>(p);
  p += align256(C * 4);
  w.target = reinterpret_cast<int32_t*>(p);
  p += align256((size_t)n * 4);
  w.row_empty = reinterpret_cast<int32_t*>(p);
  p += align256((size_t)W * 4);
  w.empty_list = reinterpret_cast<int32_t*>(p);
  p += align256(C * 4);
  w.e_total = reinterpret_cast<int32_t*>(p);
  w.bad = w.e_total + 1;
  return w;
}

}  // namespace

extern "C" {

size_t abm_schelling_workspace_bytes(int64_t n, int32_t W, int32_t H) {
  if (n <= 0 || W <= 0 || H <= 0) return 0;
  const size_t C = (size_t)W * H;
  return align256(C * 4) + align256((size_t)n * 4) + align256((size_t)W * 4) + align256(C * 4) +
         256;
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

int abm_schelling_run(int32_t* pos, const int8_t* type, int64_t n, int32_t W, int32_t H,
                      int8_t* grid, int32_t* cell_agent, const uint32_t* coll_keys, int32_t steps,
                      int32_t* stats, void* workspace, size_t workspace_bytes, void* stream) {
  if (!pos || !type || !grid || !cell_agent || !coll_keys || !stats || n <= 0 || W < 3 ||
      H < 3 || (int64_t)W * H > 0x7FFFFFFFll || n > (int64_t)W * H || steps < 0 || H > 16384)
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
  const unsigned agent_blocks = (unsigned)((n + kAgentThreads - 1) / kAgentThreads);
  const size_t smem = 3 * (size_t)H;
  for (int32_t t = 0; t < steps; ++t) {
    int32_t* stats_t = stats + 2 * (size_t)t;
    schelling_scan_kernel<<<W, kRowThreads, smem, s>>>(grid, cell_agent, W, H, w.target,
                                                      w.row_empty, stats_t);
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

}  // extern "C"
