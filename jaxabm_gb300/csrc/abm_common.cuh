// Shared device helpers: threefry2x32-20, jax.random key derivation and sampling,
// launch/status plumbing.  All kernels of the library include this header.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/jaxabm_gb300.h"

namespace abm {

constexpr uint32_t kThreefryParity = 0x1BD11BDAu;

// The integer adds of threefry are issued as multiply-adds by a 1 read from constant
// memory: the result is the plain 32-bit sum, but the instruction runs on the FMA pipe
// instead of the ALU pipe, which also carries every rotation and xor (on a GB300 the
// sampler's block rate rose from 3.17e11 to 3.75e11 per second, bit-identical).  The 1
// must stay opaque to the compiler, which would turn a literal back into an add.
static __constant__ uint32_t kFmaPipeOne = 1u;
__device__ __forceinline__ uint32_t fma_pipe_add(uint32_t a, uint32_t b) {
  uint32_t d;
  asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(kFmaPipeOne), "r"(b));
  return d;
}

// Threefry-2x32 with 20 rounds (Salmon et al., SC'11 / Random123): rotation schedule
// 13,15,26,6 then 17,29,16,24, key injection after every fourth round.
#define ABM_TF_ROUND(r)                  \
  x0 = fma_pipe_add(x1, x0);             \
  x1 = __funnelshift_l(x1, x1, (r));     \
  x1 ^= x0;
#define ABM_TF_INJECT(a, b, c)           \
  x0 = fma_pipe_add(x0, (a));            \
  x1 = fma_pipe_add(x1, (b) + (c));

__device__ __forceinline__ uint2 threefry(uint2 key, uint32_t c0, uint32_t c1) {
  const uint32_t ks0 = key.x, ks1 = key.y, ks2 = key.x ^ key.y ^ kThreefryParity;
  uint32_t x0 = c0 + ks0, x1 = c1 + ks1;
  ABM_TF_ROUND(13) ABM_TF_ROUND(15) ABM_TF_ROUND(26) ABM_TF_ROUND(6)
  ABM_TF_INJECT(ks1, ks2, 1u)
  ABM_TF_ROUND(17) ABM_TF_ROUND(29) ABM_TF_ROUND(16) ABM_TF_ROUND(24)
  ABM_TF_INJECT(ks2, ks0, 2u)
  ABM_TF_ROUND(13) ABM_TF_ROUND(15) ABM_TF_ROUND(26) ABM_TF_ROUND(6)
  ABM_TF_INJECT(ks0, ks1, 3u)
  ABM_TF_ROUND(17) ABM_TF_ROUND(29) ABM_TF_ROUND(16) ABM_TF_ROUND(24)
  ABM_TF_INJECT(ks1, ks2, 4u)
  ABM_TF_ROUND(13) ABM_TF_ROUND(15) ABM_TF_ROUND(26) ABM_TF_ROUND(6)
  ABM_TF_INJECT(ks2, ks0, 5u)
  return make_uint2(x0, x1);
}
#undef ABM_TF_INJECT
#undef ABM_TF_ROUND

// ---- partitionable-mode jax.random (JAX >= 0.5 default) ---------------------------
// split(key, n)[i] = threefry(key, (hi(i), lo(i)))
__device__ __forceinline__ uint2 split_at(uint2 key, uint64_t i) {
  return threefry(key, (uint32_t)(i >> 32), (uint32_t)i);
}
// bits(key, shape)[i] = y0 ^ y1 of threefry(key, (hi(i), lo(i)))
__device__ __forceinline__ uint32_t bits_at(uint2 key, uint64_t i) {
  uint2 y = threefry(key, (uint32_t)(i >> 32), (uint32_t)i);
  return y.x ^ y.y;
}

// ---- legacy-mode jax.random --------------------------------------------------------
// threefry_2x32(key, iota(m)) with the counter array zero-padded to even length and its
// first half paired with its second half; element j of the concatenated output.
__device__ __forceinline__ uint32_t legacy_word(uint2 key, uint64_t m, uint64_t j) {
  const uint64_t padded = m + (m & 1u);
  const uint64_t h = padded >> 1;
  const bool second = j >= h;
  const uint64_t p = second ? j - h : j;       // pair index
  const uint32_t c0 = (uint32_t)p;              // counters are iota values (pad = 0)
  const uint64_t hi_idx = p + h;
  const uint32_t c1 = hi_idx < m ? (uint32_t)hi_idx : 0u;
  uint2 y = threefry(key, c0, c1);
  return second ? y.y : y.x;
}
__device__ __forceinline__ uint2 legacy_split_at(uint2 key, uint64_t num, uint64_t i) {
  const uint64_t m = 2 * num;
  return make_uint2(legacy_word(key, m, 2 * i), legacy_word(key, m, 2 * i + 1));
}
__device__ __forceinline__ uint32_t legacy_bits_at(uint2 key, uint64_t count, uint64_t i) {
  return legacy_word(key, count, i);
}

// ---- float conversions (exactly jax.random._uniform) -------------------------------
// top 23 bits as the mantissa of a float in [1, 2), minus one: exactly k * 2^-23.
__device__ __forceinline__ float unit_float(uint32_t b) {
  return __uint_as_float((b >> 9) | 0x3F800000u) - 1.0f;
}
// unit_float(b) is m * 2^-23 with m = b >> 9, so for a float p the comparison
// unit_float(b) < p equals the integer comparison (b >> 9) < unit_threshold(p): the
// scaling by 2^23 and the ceiling are exact, p >= 1 admits every m, and p <= 0 or NaN
// admits none.
__host__ __device__ __forceinline__ uint32_t unit_threshold(float p) {
  if (!(p > 0.0f)) return 0u;
  if (p >= 1.0f) return 1u << 23;
  return static_cast<uint32_t>(ceilf(p * 8388608.0f));
}
__device__ __forceinline__ bool unit_below(uint32_t b, uint32_t threshold) {
  return (b >> 9) < threshold;
}
__device__ __forceinline__ float uniform_from_bits(uint32_t b, float lo, float hi) {
  const float span = __fsub_rn(hi, lo);
  const float v = __fadd_rn(__fmul_rn(unit_float(b), span), lo);
  return fmaxf(lo, v);
}

// Inverse error function: Giles, "Approximating the erfinv function" (GPU Computing
// Gems Jade, 2011), single-precision variant with w = -log1p(-x^2).
__device__ __forceinline__ float erfinv_giles(float x) {
  float w = -log1pf(-__fmul_rn(x, x));
  float p;
  if (w < 5.0f) {
    w = w - 2.5f;
    p = 2.81022636e-08f;
    p = fmaf(p, w, 3.43273939e-07f);
    p = fmaf(p, w, -3.5233877e-06f);
    p = fmaf(p, w, -4.39150654e-06f);
    p = fmaf(p, w, 0.00021858087f);
    p = fmaf(p, w, -0.00125372503f);
    p = fmaf(p, w, -0.00417768164f);
    p = fmaf(p, w, 0.246640727f);
    p = fmaf(p, w, 1.50140941f);
  } else {
    w = sqrtf(w) - 3.0f;
    p = -0.000200214257f;
    p = fmaf(p, w, 0.000100950558f);
    p = fmaf(p, w, 0.00134934322f);
    p = fmaf(p, w, -0.00367342844f);
    p = fmaf(p, w, 0.00573950773f);
    p = fmaf(p, w, -0.0076224613f);
    p = fmaf(p, w, 0.00943887047f);
    p = fmaf(p, w, 1.00167406f);
    p = fmaf(p, w, 2.83297682f);
  }
  return p * x;
}

// nextafter(-1.0f, 0.0f)
constexpr float kNormalLo = -0.99999994039535522461f;
constexpr float kSqrt2 = 1.41421353816986083984f;  // float32(sqrt(2))

__device__ __forceinline__ float normal_from_bits(uint32_t b) {
  const float u = uniform_from_bits(b, kNormalLo, 1.0f);
  return __fmul_rn(kSqrt2, erfinv_giles(u));
}

__device__ __forceinline__ uint2 load_key(const uint32_t* p) {
  return make_uint2(p[0], p[1]);
}

// jnp.remainder(x, 1.0) for float32: truncated fmod, shifted into [0, 1) when negative
// (the +1 can round to exactly 1.0 for tiny negative remainders, as in JAX).
__device__ __forceinline__ float mod1(float v) {
  float r = fmodf(v, 1.0f);
  if (r != 0.0f && r < 0.0f) r = __fadd_rn(r, 1.0f);
  return r;
}

// ---- warp / block reductions (fixed order => deterministic) ------------------------
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ int warp_sum(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---- range-checked build (-DABM_CHECKED) --------------------------------------------
// Gathers whose index comes from caller data (CSR columns and row offsets, row indices)
// go through ABM_IDX(i, n).  In the checked build an index outside [0, n) is replaced by 0,
// so the access stays inside the array (n > 0 at every use), and the first such index of
// the translation unit is recorded with its bound and source line; the entry point then
// waits for its stream and returns ABM_ERR_BOUNDS (abm_host::finish).  In the normal build
// ABM_IDX(i, n) is i and nothing is recorded.
#ifdef ABM_CHECKED
static __device__ unsigned long long g_bounds_hit[4];  // set, index, bound, line
__device__ __forceinline__ long long checked_index(long long i, long long n, int line) {
  if (i >= 0 && i < n) return i;
  if (atomicCAS(&g_bounds_hit[0], 0ull, 1ull) == 0ull) {
    g_bounds_hit[1] = static_cast<unsigned long long>(i);
    g_bounds_hit[2] = static_cast<unsigned long long>(n);
    g_bounds_hit[3] = static_cast<unsigned long long>(line);
  }
  return 0;
}
#define ABM_IDX(i, n) (abm::checked_index((i), (n), __LINE__))
#else
#define ABM_IDX(i, n) (i)
#endif

}  // namespace abm

// ---- host-side helpers --------------------------------------------------------------
namespace abm_host {
// Records the last CUDA error for abm_last_cuda_error(); returns ABM_ERR_CUDA or ABM_OK.
int check_launch(const char* where);
int record_cuda_error(cudaError_t e, const char* where);
inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }
int sm_count();
inline bool aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }
// Text of the last out-of-range index found by a checked build (abm_bounds_detail()).
void set_bounds_detail(const char* where, long long index, long long bound, long long line);

// Launch status of an entry point; in the checked build also the range checks of its
// kernels: the stream is waited for (unless it is being captured into a graph, when the
// check is skipped) and a recorded index becomes ABM_ERR_BOUNDS.
static inline int finish(void* stream, const char* where) {
  const int st = check_launch(where);
#ifdef ABM_CHECKED
  if (st != ABM_OK) return st;
  cudaStream_t s = as_stream(stream);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone)
    return ABM_OK;
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return record_cuda_error(e, where);
  unsigned long long hit[4] = {0, 0, 0, 0};
  e = cudaMemcpyFromSymbol(hit, abm::g_bounds_hit, sizeof(hit));
  if (e != cudaSuccess) return record_cuda_error(e, where);
  if (hit[0] == 0) return ABM_OK;
  const unsigned long long zero[4] = {0, 0, 0, 0};
  e = cudaMemcpyToSymbol(abm::g_bounds_hit, zero, sizeof(zero));
  if (e != cudaSuccess) return record_cuda_error(e, where);
  set_bounds_detail(where, static_cast<long long>(hit[1]), static_cast<long long>(hit[2]),
                    static_cast<long long>(hit[3]));
  return ABM_ERR_BOUNDS;
#else
  (void)stream;
  return st;
#endif
}
}  // namespace abm_host
