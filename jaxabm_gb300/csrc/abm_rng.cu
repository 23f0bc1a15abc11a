// K1: threefry2x32 / jax.random primitives and the Model.step key chain.
//
// Replaces jax.random.split/bits/uniform/normal/bernoulli as reached from
// jaxabm/model.py:46,129,156,164,183 and jaxabm/agent.py:115,156.

#include <cstdio>
#include <cstring>

#include "abm_common.cuh"

namespace {

thread_local char g_last_cuda_error[256] = "";
thread_local char g_bounds_detail[256] = "";

constexpr int kThreads = 256;

// Element (key k, index i) of a launch over nkeys x count elements.  Keys with many
// elements use a 2-D grid (keys along y, a key's elements along x: no per-element division);
// keys with few elements (count < kThreads, e.g. one draw per agent key) use a flat 1-D
// grid, with a 32-bit division when the element count allows it.
template <typename F>
__device__ __forceinline__ void for_each_element(int64_t nkeys, int64_t count, bool flat, F&& f) {
  if (flat) {
    const int64_t total = nkeys * count;
    const bool small = total <= 0xFFFFFFFFll;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total;
         g += (int64_t)gridDim.x * blockDim.x) {
      int64_t k, i;
      if (count == 1) {
        k = g;
        i = 0;
      } else if (small) {
        k = (uint32_t)g / (uint32_t)count;
        i = g - k * count;
      } else {
        k = g / count;
        i = g - k * count;
      }
      f(k, i);
    }
  } else {
    for (int64_t k = blockIdx.y; k < nkeys; k += gridDim.y)
      for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count;
           i += (int64_t)gridDim.x * blockDim.x)
        f(k, i);
  }
}

__global__ void split_kernel(const uint32_t* __restrict__ keys, int64_t nkeys, int64_t num,
                             uint32_t* __restrict__ out, int mode, bool flat) {
  for_each_element(nkeys, num, flat, [&](int64_t k, int64_t i) {
    const uint2 key = abm::load_key(keys + 2 * k);
    const uint2 r = mode == ABM_RNG_PARTITIONABLE ? abm::split_at(key, (uint64_t)i)
                                                  : abm::legacy_split_at(key, num, i);
    reinterpret_cast<uint2*>(out)[k * num + i] = r;
  });
}

// kind: 0 bits, 1 uniform, 2 normal, 3 bernoulli
template <int kKind>
__global__ void sample_kernel(const uint32_t* __restrict__ keys, int64_t nkeys, int64_t count,
                              float a, float b, void* __restrict__ out, int mode, bool flat) {
  for_each_element(nkeys, count, flat, [&](int64_t k, int64_t i) {
    const uint2 key = abm::load_key(keys + 2 * k);
    const int64_t g = k * count + i;
    const uint32_t w = mode == ABM_RNG_PARTITIONABLE ? abm::bits_at(key, (uint64_t)i)
                                                     : abm::legacy_bits_at(key, count, i);
    if (kKind == 0) {
      static_cast<uint32_t*>(out)[g] = w;
    } else if (kKind == 1) {
      static_cast<float*>(out)[g] = abm::uniform_from_bits(w, a, b);
    } else if (kKind == 2) {
      static_cast<float*>(out)[g] = abm::normal_from_bits(w);
    } else {
      static_cast<uint8_t*>(out)[g] = abm::unit_float(w) < a ? 1 : 0;
    }
  });
}

// jax.random.randint(key, (count,), minval, maxval, int32): k1, k2 = split(key);
// hi = bits(k1), lo = bits(k2); span = maxval - minval (1 if empty);
// mult = (2^16 mod span)^2 mod span; r = ((hi mod span) * mult + (lo mod span)) mod span
// in wrapping uint32 arithmetic; out = minval + r.
__global__ void randint_kernel(const uint32_t* __restrict__ keys, int64_t nkeys, int64_t count,
                               int32_t minval, int32_t maxval, int32_t* __restrict__ out,
                               int mode, bool flat) {
  const uint32_t span = maxval <= minval ? 1u : (uint32_t)((int64_t)maxval - (int64_t)minval);
  uint32_t mult = 65536u % span;
  mult = (mult * mult) % span;
  for_each_element(nkeys, count, flat, [&](int64_t k, int64_t i) {
    const uint2 key = abm::load_key(keys + 2 * k);
    uint2 k1, k2;
    if (mode == ABM_RNG_PARTITIONABLE) {
      k1 = abm::split_at(key, 0);
      k2 = abm::split_at(key, 1);
    } else {
      k1 = abm::legacy_split_at(key, 2, 0);
      k2 = abm::legacy_split_at(key, 2, 1);
    }
    const uint32_t hi = mode == ABM_RNG_PARTITIONABLE ? abm::bits_at(k1, (uint64_t)i)
                                                      : abm::legacy_bits_at(k1, count, i);
    const uint32_t lo = mode == ABM_RNG_PARTITIONABLE ? abm::bits_at(k2, (uint64_t)i)
                                                      : abm::legacy_bits_at(k2, count, i);
    uint32_t r = (hi % span) * mult + (lo % span);
    r %= span;
    out[k * count + i] = (int32_t)((uint32_t)minval + r);
  });
}

// One thread per model instance walks the sequential chain of Model.step
// (jaxabm/model.py:155-190).  The chain rng_{t+1} = split(rng_t)[0] is inherently
// serial; everything else hangs off it.
__global__ void keychain_kernel(uint32_t* __restrict__ rng, int64_t ninst, int32_t ncoll,
                                int32_t steps, uint32_t* __restrict__ coll_keys,
                                uint32_t* __restrict__ update_keys) {
  const int64_t inst = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (inst >= ninst) return;
  uint2 r = abm::load_key(rng + 2 * inst);
  uint2* out = reinterpret_cast<uint2*>(coll_keys) + inst * (int64_t)steps * ncoll;
  for (int32_t t = 0; t < steps; ++t) {
    uint2 step_key = abm::split_at(r, 1);
    r = abm::split_at(r, 0);
    for (int32_t c = 0; c < ncoll; ++c) {
      out[(int64_t)t * ncoll + c] = abm::split_at(step_key, 1);
      step_key = abm::split_at(step_key, 0);
    }
    if (update_keys)
      reinterpret_cast<uint2*>(update_keys)[inst * (int64_t)steps + t] = abm::split_at(step_key, 1);
  }
  rng[2 * inst] = r.x;
  rng[2 * inst + 1] = r.y;
}

bool flat_launch(int64_t count) { return count < kThreads; }

// Grid for nkeys x count elements (at most 16 CTAs per SM): flat for few elements per key,
// else x covers a key's elements and y the keys.
dim3 grid_for(int64_t nkeys, int64_t count) {
  const int64_t cap = (int64_t)abm_host::sm_count() * 16;
  if (flat_launch(count)) {
    int64_t blocks = (nkeys * count + kThreads - 1) / kThreads;
    if (blocks > cap) blocks = cap;
    return dim3((unsigned)(blocks < 1 ? 1 : blocks));
  }
  int64_t x = (count + kThreads - 1) / kThreads;
  if (x > cap) x = cap;
  if (x < 1) x = 1;
  int64_t y = cap / x;
  if (y > nkeys) y = nkeys;
  if (y > 65535) y = 65535;
  if (y < 1) y = 1;
  return dim3((unsigned)x, (unsigned)y);
}

bool bad_mode(int mode) { return mode != ABM_RNG_LEGACY && mode != ABM_RNG_PARTITIONABLE; }

template <int kKind>
int launch_sample(const uint32_t* keys, int64_t nkeys, int64_t count, float a, float b,
                  void* out, int mode, void* stream) {
  if (!keys || !out || nkeys < 0 || count < 0 || bad_mode(mode)) return ABM_ERR_BADARG;
  if (nkeys == 0 || count == 0) return ABM_OK;
  if (mode == ABM_RNG_LEGACY && count > 0xFFFFFFFFll) return ABM_ERR_BADARG;
  sample_kernel<kKind><<<grid_for(nkeys, count), kThreads, 0, abm_host::as_stream(stream)>>>(
      keys, nkeys, count, a, b, out, mode, flat_launch(count));
  return abm_host::check_launch("abm_rng_sample");
}

}  // namespace

namespace abm_host {
int record_cuda_error(cudaError_t e, const char* where) {
  if (e == cudaSuccess) return ABM_OK;
  snprintf(g_last_cuda_error, sizeof(g_last_cuda_error), "%s: %s", where,
           cudaGetErrorString(e));
  return ABM_ERR_CUDA;
}
int check_launch(const char* where) { return record_cuda_error(cudaGetLastError(), where); }
void set_bounds_detail(const char* where, long long index, long long bound, long long line) {
  snprintf(g_bounds_detail, sizeof(g_bounds_detail),
           "%s: index %lld outside [0, %lld) (checked at source line %lld)", where, index,
           bound, line);
}
int sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
  return n > 0 ? n : 1;
}
}  // namespace abm_host

extern "C" {

int abm_version(void) { return 100; }

const char* abm_status_string(int status) {
  switch (status) {
    case ABM_OK: return "ok";
    case ABM_ERR_BADARG: return "bad argument";
    case ABM_ERR_OOM: return "out of device memory";
    case ABM_ERR_TIMEOUT: return "device wait timed out";
    case ABM_ERR_BOUNDS: return "index out of bounds";
    case ABM_ERR_UNREGISTERED: return "no step kernel registered";
    case ABM_ERR_CUDA: return "CUDA error";
    case ABM_ERR_WORKSPACE: return "workspace too small";
    default: return "unknown status";
  }
}

const char* abm_last_cuda_error(void) { return g_last_cuda_error; }

const char* abm_bounds_detail(void) { return g_bounds_detail; }

int abm_checked_build(void) {
#ifdef ABM_CHECKED
  return 1;
#else
  return 0;
#endif
}

int abm_device_info(int* sm_count, int* cc_major, int* cc_minor) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return abm_host::record_cuda_error(e, "cudaGetDevice");
  if (sm_count) {
    e = cudaDeviceGetAttribute(sm_count, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return abm_host::record_cuda_error(e, "sm count");
  }
  if (cc_major) {
    e = cudaDeviceGetAttribute(cc_major, cudaDevAttrComputeCapabilityMajor, dev);
    if (e != cudaSuccess) return abm_host::record_cuda_error(e, "cc major");
  }
  if (cc_minor) {
    e = cudaDeviceGetAttribute(cc_minor, cudaDevAttrComputeCapabilityMinor, dev);
    if (e != cudaSuccess) return abm_host::record_cuda_error(e, "cc minor");
  }
  return ABM_OK;
}

int abm_rng_split(const uint32_t* keys, int64_t nkeys, int64_t num, uint32_t* out, int mode,
                  void* stream) {
  if (!keys || !out || nkeys < 0 || num < 0 || bad_mode(mode)) return ABM_ERR_BADARG;
  if (nkeys == 0 || num == 0) return ABM_OK;
  if (mode == ABM_RNG_LEGACY && 2 * num > 0xFFFFFFFFll) return ABM_ERR_BADARG;
  split_kernel<<<grid_for(nkeys, num), kThreads, 0, abm_host::as_stream(stream)>>>(
      keys, nkeys, num, out, mode, flat_launch(num));
  return abm_host::check_launch("abm_rng_split");
}

int abm_rng_bits(const uint32_t* keys, int64_t nkeys, int64_t count, uint32_t* out, int mode,
                 void* stream) {
  return launch_sample<0>(keys, nkeys, count, 0.f, 0.f, out, mode, stream);
}

int abm_rng_uniform(const uint32_t* keys, int64_t nkeys, int64_t count, float minval,
                    float maxval, float* out, int mode, void* stream) {
  return launch_sample<1>(keys, nkeys, count, minval, maxval, out, mode, stream);
}

int abm_rng_normal(const uint32_t* keys, int64_t nkeys, int64_t count, float* out, int mode,
                   void* stream) {
  return launch_sample<2>(keys, nkeys, count, 0.f, 0.f, out, mode, stream);
}

int abm_rng_bernoulli(const uint32_t* keys, int64_t nkeys, int64_t count, float p,
                      uint8_t* out, int mode, void* stream) {
  return launch_sample<3>(keys, nkeys, count, p, 0.f, out, mode, stream);
}

int abm_rng_randint(const uint32_t* keys, int64_t nkeys, int64_t count, int32_t minval,
                    int32_t maxval, int32_t* out, int mode, void* stream) {
  if (!keys || !out || nkeys < 0 || count < 0 || bad_mode(mode)) return ABM_ERR_BADARG;
  if (nkeys == 0 || count == 0) return ABM_OK;
  if (mode == ABM_RNG_LEGACY && count > 0xFFFFFFFFll) return ABM_ERR_BADARG;
  randint_kernel<<<grid_for(nkeys, count), kThreads, 0, abm_host::as_stream(stream)>>>(
      keys, nkeys, count, minval, maxval, out, mode, flat_launch(count));
  return abm_host::check_launch("abm_rng_randint");
}

int abm_keychain(uint32_t* rng, int64_t ninst, int32_t ncoll, int32_t steps,
                 uint32_t* coll_keys, uint32_t* update_keys, void* stream) {
  if (!rng || ninst < 0 || ncoll < 0 || steps < 0) return ABM_ERR_BADARG;
  if (ncoll > 0 && steps > 0 && !coll_keys) return ABM_ERR_BADARG;
  if (ninst == 0) return ABM_OK;
  const int threads = 64;
  const int64_t blocks = (ninst + threads - 1) / threads;
  keychain_kernel<<<(unsigned)blocks, threads, 0, abm_host::as_stream(stream)>>>(
      rng, ninst, ncoll, steps, coll_keys, update_keys);
  return abm_host::check_launch("abm_keychain");
}

}  // extern "C"
