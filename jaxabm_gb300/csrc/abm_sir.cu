// SIR contagion on a Network (CSR), batched over any number of model instances.
//
// Agent semantics (partitionable jax.random; agent i of an instance holds
// agent_key = split(coll_key, n)[i], jaxabm/agent.py:156; k_inf, k_rec = split(agent_key)):
//   S: infected if any neighbour slot k (CSR position row_ptr[i] + k) whose neighbour is I
//      has uniform(k_inf, (deg,))[k] < beta           (bernoulli(beta) per I-edge)
//   I: recovers if uniform(k_rec) < gamma
//   R: stays R
// All agents read the pre-step states (synchronous update, jaxabm/agent.py:168-177); the
// S/I/R counts after each step are the metrics (jaxabm/model.py:193-200).
//
// Layout: each instance has a descriptor (abm_sir_instance) with its CSR, a 2*n int8 state
// double buffer (buffer t&1 is current), its rng (Model.step key chain state) and step
// counter.  Work items are (instance, agent range) tiles of <= 256 agents; one CTA runs one
// tile at a time over a persistent grid.  Per step: the step kernel over all work items,
// then a one-thread-per-instance kernel that advances rng and t.  Kernels never wait on
// anything, so a step can neither hang nor deadlock.
//
// Load balance on heavy-tailed (Barabasi-Albert) degrees: a thread scans its own row when
// deg <= 32; longer rows are scanned by the whole warp, 32 slots per pass, with a warp vote
// ending the scan at the first firing draw ("any" is order-free, so results are exact).

#include "abm_common.cuh"

namespace {

constexpr int kSirThreads = 256;
constexpr int kSirWarps = kSirThreads / 32;
constexpr int kHeavyDeg = 32;
constexpr unsigned kFull = 0xffffffffu;

static_assert(sizeof(abm_sir_instance) == 88, "abm_sir_instance layout");
static_assert(sizeof(abm_work_item) == 16, "abm_work_item layout");

__global__ void __launch_bounds__(kSirThreads)
sir_step_kernel(abm_sir_instance* __restrict__ insts, const int4* __restrict__ work, int nwork) {
  __shared__ int scount[4][kSirWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
    const int4 item = work[w];
    abm_sir_instance* I = insts + item.x;
    const int t = I->t;
    if (t >= I->steps) continue;  // uniform over the CTA
    const int n = I->n;
    const int8_t* __restrict__ cur = I->state + (size_t)(t & 1) * n;
    int8_t* __restrict__ nxt = I->state + (size_t)((t + 1) & 1) * n;
    const int32_t* __restrict__ rp = I->row_ptr;
    const int32_t* __restrict__ col = I->col;
    const float beta = I->beta, gamma = I->gamma;
    // coll_key of step t: given per step, or from the instance's own key chain
    // (step_key = split(rng)[1]; coll_key = split(step_key)[1], jaxabm/model.py:156,164)
    const uint2 coll = I->coll_keys != nullptr
                           ? abm::load_key(I->coll_keys + 2 * (size_t)t)
                           : abm::split_at(abm::split_at(make_uint2(I->rng[0], I->rng[1]), 1), 1);

    const int i = item.y + threadIdx.x;
    const bool valid = i < item.z;
    const int8_t s = valid ? cur[i] : (int8_t)2;
    int8_t ns = s;
    bool heavy = false;
    int row0 = 0, deg = 0, scanned = 0;
    if (s == 0) {
      row0 = rp[i];
      deg = rp[i + 1] - row0;
      if (deg > kHeavyDeg) {
        heavy = true;
      } else {
        bool have = false;
        uint2 kinf = make_uint2(0, 0);
        int k = 0;
        for (; k < deg; ++k) {
          const int j = col[row0 + k];
          if (cur[j] == 1) {
            if (!have) {
              kinf = abm::split_at(abm::split_at(coll, (uint64_t)i), 0);
              have = true;
            }
            if (abm::unit_float(abm::bits_at(kinf, (uint64_t)k)) < beta) {
              ns = 1;
              ++k;
              break;
            }
          }
        }
        scanned = k;
      }
    } else if (s == 1) {
      const uint2 krec = abm::split_at(abm::split_at(coll, (uint64_t)i), 1);
      if (abm::unit_float(abm::bits_at(krec, 0)) < gamma) ns = 2;
    }

    unsigned hmask = __ballot_sync(kFull, heavy);
    while (hmask) {
      const int src = __ffs(hmask) - 1;
      hmask &= hmask - 1;
      const int hi = __shfl_sync(kFull, i, src);
      const int hrow = __shfl_sync(kFull, row0, src);
      const int hdeg = __shfl_sync(kFull, deg, src);
      const uint2 kinf = abm::split_at(abm::split_at(coll, (uint64_t)hi), 0);
      bool fired = false;
      int c = 0;
      for (; c < hdeg && !fired; c += 32) {
        const int k = c + lane;
        bool f = false;
        if (k < hdeg) {
          const int j = col[hrow + k];
          if (cur[j] == 1) f = abm::unit_float(abm::bits_at(kinf, (uint64_t)k)) < beta;
        }
        fired = __any_sync(kFull, f);
      }
      if (lane == src) {
        if (fired) ns = 1;
        scanned = min(c, hdeg);
      }
    }

    if (valid) nxt[i] = ns;
    const int cs = abm::warp_sum((int)(valid && ns == 0));
    const int ci = abm::warp_sum((int)(valid && ns == 1));
    const int cr = abm::warp_sum((int)(valid && ns == 2));
    const int ce = abm::warp_sum(scanned);
    if (lane == 0) {
      scount[0][warp] = cs;
      scount[1][warp] = ci;
      scount[2][warp] = cr;
      scount[3][warp] = ce;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
      int sum = 0;
#pragma unroll
      for (int q = 0; q < kSirWarps; ++q) sum += scount[threadIdx.x][q];
      if (sum) {
        if (threadIdx.x < 3)
          atomicAdd(&I->counts[3 * t + threadIdx.x], sum);
        else
          atomicAdd(&I->edges_scanned, (unsigned long long)sum);
      }
    }
    __syncthreads();
  }
}

// Advance every live instance by one step: rng = split(rng)[0]; t += 1; raise the
// (host-mapped) done flag when the last step has been applied.
__global__ void sir_finalize_kernel(abm_sir_instance* __restrict__ insts, int ninst) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ninst) return;
  abm_sir_instance* I = insts + k;
  const int t = I->t;
  if (t >= I->steps) return;
  const uint2 r = abm::split_at(make_uint2(I->rng[0], I->rng[1]), 0);
  I->rng[0] = r.x;
  I->rng[1] = r.y;
  I->t = t + 1;
  if (t + 1 == I->steps && I->done_flag) {
    __threadfence_system();
    *reinterpret_cast<volatile int32_t*>(I->done_flag) = 1;
  }
}

// Single-instance descriptor and tile list written on the device (keeps abm_sir_run
// free of host-to-device copies, so it can be captured in a CUDA graph).
__global__ void sir_setup_single_kernel(abm_sir_instance* d, int4* work, int ntiles,
                                       const int32_t* row_ptr, const int32_t* col, int8_t* state,
                                       int32_t* counts, const uint32_t* coll_keys, int32_t n,
                                       int32_t steps, float beta, float gamma) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g == 0) {
    d->row_ptr = row_ptr;
    d->col = col;
    d->state = state;
    d->counts = counts;
    d->done_flag = nullptr;
    d->coll_keys = coll_keys;
    d->rng[0] = 0;
    d->rng[1] = 0;
    d->n = n;
    d->t = 0;
    d->steps = steps;
    d->beta = beta;
    d->gamma = gamma;
    d->reserved = 0;
    d->edges_scanned = 0;
  }
  for (int b = g; b < ntiles; b += gridDim.x * blockDim.x) {
    const int begin = b * kSirThreads;
    const int end = min(begin + kSirThreads, n);
    work[b] = make_int4(0, begin, end, 0);
  }
}

int default_grid(int nwork) {
  const int cap = abm_host::sm_count() * 8;  // 8 resident 256-thread CTAs per SM
  return nwork < cap ? (nwork > 0 ? nwork : 1) : cap;
}

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

}  // namespace

extern "C" {

size_t abm_sir_instance_size(void) { return sizeof(abm_sir_instance); }

int abm_sir_steps(abm_sir_instance* insts, int32_t ninst, const abm_work_item* work,
                  int32_t nwork, int32_t nsteps, int32_t grid, void* stream) {
  if (!insts || ninst <= 0 || nwork < 0 || nsteps < 0 || (nwork > 0 && !work))
    return ABM_ERR_BADARG;
  if (!abm_host::aligned(insts, 8) || (work && !abm_host::aligned(work, 16)))
    return ABM_ERR_BADARG;
  cudaStream_t s = abm_host::as_stream(stream);
  const int g = grid > 0 ? grid : default_grid(nwork);
  const int fin_blocks = (ninst + 255) / 256;
  for (int32_t k = 0; k < nsteps; ++k) {
    if (nwork > 0) {
      sir_step_kernel<<<g, kSirThreads, 0, s>>>(insts, reinterpret_cast<const int4*>(work), nwork);
      int st = abm_host::check_launch("abm_sir_steps/step");
      if (st) return st;
    }
    sir_finalize_kernel<<<fin_blocks, 256, 0, s>>>(insts, ninst);
    int st = abm_host::check_launch("abm_sir_steps/finalize");
    if (st) return st;
  }
  return ABM_OK;
}

size_t abm_sir_run_workspace_bytes(int64_t n) {
  if (n <= 0) return 0;
  const int64_t tiles = (n + kSirThreads - 1) / kSirThreads;
  return align256(sizeof(abm_sir_instance)) + (size_t)tiles * sizeof(int4);
}

int abm_sir_run(const int32_t* row_ptr, const int32_t* col, int64_t n, int8_t* state,
                const uint32_t* coll_keys, int32_t steps, float beta, float gamma,
                int32_t* counts, void* workspace, size_t workspace_bytes, void* stream) {
  if (!row_ptr || !col || !state || !coll_keys || !counts || n <= 0 || n > 0x7FFFFFFFll ||
      steps < 0)
    return ABM_ERR_BADARG;
  if (!abm_host::aligned(coll_keys, 8)) return ABM_ERR_BADARG;
  const size_t need = abm_sir_run_workspace_bytes(n);
  if (!workspace || workspace_bytes < need || !abm_host::aligned(workspace, 256))
    return ABM_ERR_WORKSPACE;
  if (steps == 0) return ABM_OK;
  cudaStream_t s = abm_host::as_stream(stream);
  abm_sir_instance* d = static_cast<abm_sir_instance*>(workspace);
  int4* work = reinterpret_cast<int4*>(static_cast<char*>(workspace) +
                                       align256(sizeof(abm_sir_instance)));
  const int ntiles = (int)((n + kSirThreads - 1) / kSirThreads);
  int st = abm_host::record_cuda_error(
      cudaMemsetAsync(counts, 0, sizeof(int32_t) * 3 * (size_t)steps, s), "abm_sir_run/memset");
  if (st) return st;
  sir_setup_single_kernel<<<(ntiles + 255) / 256, 256, 0, s>>>(
      d, work, ntiles, row_ptr, col, state, counts, coll_keys, (int32_t)n, steps, beta, gamma);
  st = abm_host::check_launch("abm_sir_run/setup");
  if (st) return st;
  return abm_sir_steps(d, 1, reinterpret_cast<const abm_work_item*>(work), ntiles, steps, 0,
                       stream);
}

}  // extern "C"
