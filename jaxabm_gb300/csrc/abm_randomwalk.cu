// Random-walk model (the quick-start agent with jax.random noise).
//
// Per agent and step (partitionable jax.random):
//   agent_key = split(coll_key, n)[i]; kx, ky = split(agent_key)
//   x = (x + sigma * normal(kx)) % 1.0 ; y likewise with ky
// followed by the metrics reduction mean(x), mean(y).
//
// Replaces JaxModel.run's Python loop (jaxabm/model.py:240-241) over
// AgentCollection.update (jaxabm/agent.py:156-177) and metrics_fn (jaxabm/model.py:193-200).
// The whole run is one launch: agents are independent between steps, so every thread keeps
// its agent's (x, y) in registers for all steps and only the per-step reductions leave it.
// A batch of independent models (members of one size, each with its own key chain and
// sigma) runs in the same launch: blockIdx.y selects the member, whose arrays follow the
// previous member's, and each member's blocks and reduction tree are those of a run alone,
// so every member's states and means equal its solo run bit for bit.

#include "abm_common.cuh"

namespace {

constexpr int kBlock = 128;
constexpr int kWarps = kBlock / 32;
constexpr int kChunk = 64;  // steps whose keys / warp sums are staged in shared memory

__global__ void __launch_bounds__(kBlock) rw_init_kernel(float* __restrict__ x,
                                                         float* __restrict__ y, int64_t n,
                                                         const uint32_t* __restrict__ init_key) {
  x += blockIdx.y * n;
  y += blockIdx.y * n;
  const uint2 key = abm::load_key(init_key + 2 * (size_t)blockIdx.y);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint2 ak = abm::split_at(key, (uint64_t)i);
    const uint2 kx = abm::split_at(ak, 0), ky = abm::split_at(ak, 1);
    x[i] = abm::unit_float(abm::bits_at(kx, 0));
    y[i] = abm::unit_float(abm::bits_at(ky, 0));
  }
}

// Member blockIdx.y's x, y (n each), key chain (steps keys), sigma and partial sums.
struct Member {
  float* x;
  float* y;
  const uint32_t* keys;
  float sigma;
  float2* partial;
};

__device__ __forceinline__ Member member_of(float* x, float* y, int64_t n,
                                            const uint32_t* coll_keys, int32_t steps,
                                            float sigma, const float* sigmas, float2* partial) {
  const int64_t m = blockIdx.y;
  return Member{x + m * n, y + m * n, coll_keys + 2 * (size_t)steps * m,
                sigmas ? sigmas[m] : sigma, partial + (size_t)steps * gridDim.x * m};
}

__global__ void __launch_bounds__(kBlock) rw_run_kernel(float* __restrict__ x_all,
                                                        float* __restrict__ y_all, int64_t n,
                                                        const uint32_t* __restrict__ keys_all,
                                                        int32_t steps, float sigma0,
                                                        const float* __restrict__ sigmas,
                                                        float2* __restrict__ partial_all) {
  const Member M = member_of(x_all, y_all, n, keys_all, steps, sigma0, sigmas, partial_all);
  float* __restrict__ x = M.x;
  float* __restrict__ y = M.y;
  const uint32_t* __restrict__ coll_keys = M.keys;
  const float sigma = M.sigma;
  float2* __restrict__ partial = M.partial;
  __shared__ uint2 skeys[kChunk];
  __shared__ float2 swarp[kChunk][kWarps];
  const int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x;
  const bool active = i < n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float xi = active ? x[i] : 0.f;
  float yi = active ? y[i] : 0.f;
  for (int32_t t0 = 0; t0 < steps; t0 += kChunk) {
    const int nt = min(kChunk, steps - t0);
    __syncthreads();
    for (int k = threadIdx.x; k < nt; k += kBlock) skeys[k] = abm::load_key(coll_keys + 2 * (int64_t)(t0 + k));
    __syncthreads();
#pragma unroll 2
    for (int k = 0; k < nt; ++k) {
      const uint2 ak = abm::split_at(skeys[k], (uint64_t)i);
      const uint2 kx = abm::split_at(ak, 0), ky = abm::split_at(ak, 1);
      const float nx = abm::normal_from_bits(abm::bits_at(kx, 0));
      const float ny = abm::normal_from_bits(abm::bits_at(ky, 0));
      xi = abm::mod1(__fadd_rn(xi, __fmul_rn(sigma, nx)));
      yi = abm::mod1(__fadd_rn(yi, __fmul_rn(sigma, ny)));
      const float sx = abm::warp_sum(active ? xi : 0.f);
      const float sy = abm::warp_sum(active ? yi : 0.f);
      if (lane == 0) swarp[k][warp] = make_float2(sx, sy);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nt; k += kBlock) {
      float sx = 0.f, sy = 0.f;
#pragma unroll
      for (int w = 0; w < kWarps; ++w) {
        sx += swarp[k][w].x;
        sy += swarp[k][w].y;
      }
      partial[(int64_t)(t0 + k) * gridDim.x + blockIdx.x] = make_float2(sx, sy);
    }
  }
  if (active) {
    x[i] = xi;
    y[i] = yi;
  }
}

// Few agents (n below kWideAgents): one agent per thread would leave most of the GPU idle,
// so each CTA takes kWideAgents-per-block = 32 agents and, for each chunk of kChunk steps,
// first computes their noise draws with all 256 threads (the draws do not depend on the
// state), then warp 0 applies the steps to (x, y) in order -- the same arithmetic per agent
// as rw_run_kernel -- and writes the per-step warp sums.
constexpr int kWideThreads = 256;
constexpr int kWideAgents = 32;
constexpr int64_t kWideBelow = 1 << 17;  // agent count below which the wide kernel is used

__global__ void __launch_bounds__(kWideThreads)
rw_run_wide_kernel(float* __restrict__ x_all, float* __restrict__ y_all, int64_t n,
                   const uint32_t* __restrict__ keys_all, int32_t steps, float sigma0,
                   const float* __restrict__ sigmas, float2* __restrict__ partial_all) {
  const Member M = member_of(x_all, y_all, n, keys_all, steps, sigma0, sigmas, partial_all);
  float* __restrict__ x = M.x;
  float* __restrict__ y = M.y;
  const uint32_t* __restrict__ coll_keys = M.keys;
  const float sigma = M.sigma;
  float2* __restrict__ partial = M.partial;
  __shared__ float2 snoise[kChunk][kWideAgents];
  const int64_t a0 = (int64_t)blockIdx.x * kWideAgents;
  const int lane = threadIdx.x & 31;
  const bool owner = threadIdx.x < kWideAgents;  // warp 0 keeps the agents' state
  const int64_t i = a0 + lane;
  const bool active = owner && i < n;
  float xi = active ? x[i] : 0.f;
  float yi = active ? y[i] : 0.f;
  for (int32_t t0 = 0; t0 < steps; t0 += kChunk) {
    const int nt = min(kChunk, steps - t0);
    for (int p = threadIdx.x; p < nt * kWideAgents; p += kWideThreads) {
      const int k = p / kWideAgents, a = p % kWideAgents;
      const uint2 ak = abm::split_at(abm::load_key(coll_keys + 2 * (int64_t)(t0 + k)),
                                     (uint64_t)(a0 + a));
      const uint2 kx = abm::split_at(ak, 0), ky = abm::split_at(ak, 1);
      snoise[k][a] = make_float2(abm::normal_from_bits(abm::bits_at(kx, 0)),
                                 abm::normal_from_bits(abm::bits_at(ky, 0)));
    }
    __syncthreads();
    if (threadIdx.x < 32) {
      for (int k = 0; k < nt; ++k) {
        const float2 nz = snoise[k][lane];
        xi = abm::mod1(__fadd_rn(xi, __fmul_rn(sigma, nz.x)));
        yi = abm::mod1(__fadd_rn(yi, __fmul_rn(sigma, nz.y)));
        const float sx = abm::warp_sum(active ? xi : 0.f);
        const float sy = abm::warp_sum(active ? yi : 0.f);
        if (lane == 0) partial[(int64_t)(t0 + k) * gridDim.x + blockIdx.x] = make_float2(sx, sy);
      }
    }
    __syncthreads();
  }
  if (active) {
    x[i] = xi;
    y[i] = yi;
  }
}

// means[t] = (sum_b partial[t][b]) / n, one block per step (and member, blockIdx.y), fixed
// reduction tree.
__global__ void rw_means_kernel(const float2* __restrict__ partial, int nblocks, int64_t n,
                                float2* __restrict__ means) {
  __shared__ float2 s[kBlock];
  const int t = blockIdx.x;
  partial += (size_t)gridDim.x * nblocks * blockIdx.y;
  means += (size_t)gridDim.x * blockIdx.y;
  float sx = 0.f, sy = 0.f;
  for (int b = threadIdx.x; b < nblocks; b += kBlock) {
    const float2 p = partial[(int64_t)t * nblocks + b];
    sx += p.x;
    sy += p.y;
  }
  s[threadIdx.x] = make_float2(sx, sy);
  __syncthreads();
  for (int o = kBlock / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      s[threadIdx.x].x += s[threadIdx.x + o].x;
      s[threadIdx.x].y += s[threadIdx.x + o].y;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const float fn = (float)n;
    means[t] = make_float2(s[0].x / fn, s[0].y / fn);
  }
}

int64_t rw_blocks(int64_t n) {
  return n < kWideBelow ? (n + kWideAgents - 1) / kWideAgents : (n + kBlock - 1) / kBlock;
}

}  // namespace

extern "C" {

int abm_randomwalk_init_batch(float* x, float* y, int64_t n, int32_t members,
                              const uint32_t* init_keys, void* stream) {
  if (!x || !y || !init_keys || n <= 0 || members <= 0 || members > 65535) return ABM_ERR_BADARG;
  int64_t blocks = rw_blocks(n);
  const int64_t cap = (int64_t)abm_host::sm_count() * 16;
  if (blocks > cap) blocks = cap;
  rw_init_kernel<<<dim3((unsigned)blocks, (unsigned)members), kBlock, 0,
                   abm_host::as_stream(stream)>>>(x, y, n, init_keys);
  return abm_host::check_launch("abm_randomwalk_init");
}

int abm_randomwalk_init(float* x, float* y, int64_t n, const uint32_t* init_key, void* stream) {
  return abm_randomwalk_init_batch(x, y, n, 1, init_key, stream);
}

size_t abm_randomwalk_batch_workspace_bytes(int64_t n, int32_t steps, int32_t members) {
  if (n <= 0 || steps <= 0 || members <= 0) return 0;
  return (size_t)rw_blocks(n) * (size_t)steps * sizeof(float2) * (size_t)members;
}

size_t abm_randomwalk_workspace_bytes(int64_t n, int32_t steps) {
  return abm_randomwalk_batch_workspace_bytes(n, steps, 1);
}

namespace {
int run_members(float* x, float* y, int64_t n, int32_t members, const uint32_t* coll_keys,
                int32_t steps, float sigma, const float* sigmas, float* means, void* workspace,
                size_t workspace_bytes, void* stream) {
  if (!x || !y || !coll_keys || !means || n <= 0 || steps < 0 || members <= 0 ||
      members > 65535)
    return ABM_ERR_BADARG;
  if (!abm_host::aligned(means, 8)) return ABM_ERR_BADARG;
  if (steps == 0) return ABM_OK;
  const int64_t blocks = rw_blocks(n);
  if (blocks > 0x7FFFFFFF) return ABM_ERR_BADARG;
  const size_t need = abm_randomwalk_batch_workspace_bytes(n, steps, members);
  if (!workspace || workspace_bytes < need || !abm_host::aligned(workspace, 8))
    return ABM_ERR_WORKSPACE;
  cudaStream_t s = abm_host::as_stream(stream);
  float2* partial = static_cast<float2*>(workspace);
  const dim3 grid((unsigned)blocks, (unsigned)members);
  if (n < kWideBelow)
    rw_run_wide_kernel<<<grid, kWideThreads, 0, s>>>(x, y, n, coll_keys, steps, sigma, sigmas,
                                                     partial);
  else
    rw_run_kernel<<<grid, kBlock, 0, s>>>(x, y, n, coll_keys, steps, sigma, sigmas, partial);
  int st = abm_host::check_launch("abm_randomwalk_run");
  if (st) return st;
  rw_means_kernel<<<dim3((unsigned)steps, (unsigned)members), kBlock, 0, s>>>(
      partial, (int)blocks, n, reinterpret_cast<float2*>(means));
  return abm_host::check_launch("abm_randomwalk_means");
}
}  // namespace

int abm_randomwalk_run(float* x, float* y, int64_t n, const uint32_t* coll_keys, int32_t steps,
                       float sigma, float* means, void* workspace, size_t workspace_bytes,
                       void* stream) {
  return run_members(x, y, n, 1, coll_keys, steps, sigma, nullptr, means, workspace,
                     workspace_bytes, stream);
}

int abm_randomwalk_run_batch(float* x, float* y, int64_t n, int32_t members,
                             const uint32_t* coll_keys, int32_t steps, const float* sigmas,
                             float* means, void* workspace, size_t workspace_bytes,
                             void* stream) {
  if (!sigmas) return ABM_ERR_BADARG;
  return run_members(x, y, n, members, coll_keys, steps, 0.0f, sigmas, means, workspace,
                     workspace_bytes, stream);
}

}  // extern "C"
