// K6: stable stream compaction of a boolean mask (AgentCollection.filter / AgentList.select)
// and K7-style single-pass reductions for AgentCollection.aggregate.
//
// Replaces `int(jnp.sum(mask))` + `{k: v[mask]}` at jaxabm/agent.py:227-242 and
// jaxabm/agentpy.py:330-343, and `jnp.mean(states[var])` at jaxabm/agent.py:198-211.
//
// Compaction is three launches over tiles of 4096 mask bytes (one 128-bit load per thread
// per 16 bytes): (1) per-tile counts, (2) one-block exclusive scan of the tile counts,
// (3) per-tile rank = tile offset + warp offset + lane prefix (warp shuffles) + position
// inside the thread's 16 bytes, so output order is ascending index order.

#include "abm_common.cuh"

namespace {

constexpr int kSelThreads = 256;
constexpr int kSelPerThread = 16;
constexpr int kTile = kSelThreads * kSelPerThread;  // 4096 mask bytes per block

// 16 mask bytes of thread `tid` in tile `tile` (bytes past n read as 0).
__device__ __forceinline__ uint32_t load_flags(const uint8_t* __restrict__ mask, int64_t n,
                                               int64_t base, bool vec_ok) {
  uint32_t bits = 0;
  if (vec_ok && base + kSelPerThread <= n) {
    const uint4 v = *reinterpret_cast<const uint4*>(mask + base);
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int b = 0; b < 4; ++b)
        if ((w[q] >> (8 * b)) & 0xFFu) bits |= 1u << (4 * q + b);
  } else {
#pragma unroll
    for (int j = 0; j < kSelPerThread; ++j)
      if (base + j < n && mask[base + j]) bits |= 1u << j;
  }
  return bits;
}

__global__ void __launch_bounds__(kSelThreads)
select_count_kernel(const uint8_t* __restrict__ mask, int64_t n, bool vec_ok,
                    int32_t* __restrict__ tile_counts) {
  __shared__ int swarp[kSelThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kSelPerThread;
  const int c = __popc(load_flags(mask, n, base, vec_ok));
  const int wsum = abm::warp_sum(c);
  if ((threadIdx.x & 31) == 0) swarp[threadIdx.x >> 5] = wsum;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < kSelThreads / 32; ++w) s += swarp[w];
    tile_counts[blockIdx.x] = s;
  }
}

// Single block: exclusive scan of tile_counts into tile_offsets (int64), total -> *count.
// Warp w owns the contiguous chunk [w*per, (w+1)*per) (per a multiple of 128) and reads it
// 128 counts at a time, four per lane (coalesced): pass 1 sums the chunk, the block scans
// the 32 chunk sums, pass 2 writes the chunk's offsets from warp scans.
__global__ void __launch_bounds__(1024)
select_scan_kernel(const int32_t* __restrict__ tile_counts, int64_t ntiles,
                   int64_t* __restrict__ tile_offsets, int64_t* __restrict__ count) {
  __shared__ int64_t swarp[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t per = ((ntiles + 31) / 32 + 127) / 128 * 128;
  const int64_t c0 = (int64_t)warp * per;
  const int64_t c1 = c0 + per < ntiles ? c0 + per : ntiles;
  // the four counts of lane `lane` in the group starting at b
  auto load4 = [&](int64_t b, int (&v)[4]) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int64_t t = b + 4 * lane + q;
      v[q] = t < c1 ? tile_counts[t] : 0;
    }
  };
  int64_t sum = 0;
  for (int64_t b = c0; b < c1; b += 128) {
    int v[4];
    load4(b, v);
    sum += v[0] + v[1] + v[2] + v[3];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if (lane == 0) swarp[warp] = sum;
  __syncthreads();
  if (warp == 0) {
    int64_t w = swarp[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t u = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += u;
    }
    swarp[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  int64_t run = warp > 0 ? swarp[warp - 1] : 0;
  for (int64_t b = c0; b < c1; b += 128) {
    int v[4];
    load4(b, v);
    const int mine = v[0] + v[1] + v[2] + v[3];
    int incl = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += u;
    }
    int64_t off = run + (incl - mine);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int64_t t = b + 4 * lane + q;
      if (t < c1) tile_offsets[t] = off;
      off += v[q];
    }
    run += __shfl_sync(0xffffffffu, incl, 31);
  }
  if (threadIdx.x == 0) *count = swarp[31];
}

// Each tile's selected indices, in ascending order, are staged in shared memory at their
// rank within the tile and then written out by the whole block with coalesced stores.
__global__ void __launch_bounds__(kSelThreads)
select_scatter_kernel(const uint8_t* __restrict__ mask, int64_t n, bool vec_ok,
                      const int64_t* __restrict__ tile_offsets, int32_t* __restrict__ out_idx) {
  __shared__ int swarp[kSelThreads / 32];
  __shared__ int32_t sidx[kTile];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t tile0 = (int64_t)blockIdx.x * kTile;
  const int64_t base = tile0 + (int64_t)threadIdx.x * kSelPerThread;
  const uint32_t bits = load_flags(mask, n, base, vec_ok);
  const int c = __popc(bits);
  int incl = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += u;
  }
  if (lane == 31) swarp[warp] = incl;
  __syncthreads();
  int warp_excl = 0, total = 0;
#pragma unroll
  for (int w = 0; w < kSelThreads / 32; ++w) {
    warp_excl += w < warp ? swarp[w] : 0;
    total += swarp[w];
  }
  int pos = warp_excl + (incl - c);
  for (uint32_t rest = bits; rest; rest &= rest - 1)
    sidx[pos++] = (int32_t)(base + __ffs(rest) - 1);
  __syncthreads();
  int32_t* __restrict__ dst = out_idx + tile_offsets[blockIdx.x];
  for (int k = threadIdx.x; k < total; k += kSelThreads) dst[k] = sidx[k];
}

// out[r] = src[idx[r]] for rows of `row_bytes` bytes, copied in 4-byte words when possible.
__global__ void gather_rows_words(const uint32_t* __restrict__ src, const int32_t* __restrict__ idx,
                                  int64_t count, int64_t row_words, uint32_t* __restrict__ dst,
                                  int64_t nrows_src) {
  const int64_t total = count * row_words;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = g / row_words, w = g - r * row_words;
    dst[g] = src[(int64_t)ABM_IDX(idx[r], nrows_src) * row_words + w];
  }
}
__global__ void gather_rows_bytes(const uint8_t* __restrict__ src, const int32_t* __restrict__ idx,
                                  int64_t count, int64_t row_bytes, uint8_t* __restrict__ dst,
                                  int64_t nrows_src) {
  const int64_t total = count * row_bytes;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = g / row_bytes, b = g - r * row_bytes;
    dst[g] = src[(int64_t)ABM_IDX(idx[r], nrows_src) * row_bytes + b];
  }
}

// ---- compaction by a predicate program (AgentList.select with a simple condition) --------
// The condition is a postfix program over at most kPredAttrs attribute arrays: comparisons
// of one attribute with a constant push a flag, AND / OR pop two and push one, NOT flips
// the top.  The count and scatter passes evaluate it for their 16 elements per thread, so
// the boolean mask is never written; the tile scan is the mask path's.
constexpr int kPredAttrs = 4;
constexpr int kPredOps = 16;

struct Predicate {
  const void* attr[kPredAttrs];
  int32_t dtype[kPredAttrs];
  int32_t nops;
  int32_t code[kPredOps];
  int32_t arg[kPredOps];
  float value_f32[kPredOps];
  double value_f64[kPredOps];
};

template <typename T>
__device__ __forceinline__ bool compare(T v, T c, int code) {
  switch (code) {
    case ABM_SELECT_LT: return v < c;
    case ABM_SELECT_LE: return v <= c;
    case ABM_SELECT_GT: return v > c;
    case ABM_SELECT_GE: return v >= c;
    case ABM_SELECT_EQ: return v == c;
    default: return v != c;
  }
}

// The program's result for element i (a stack of flags held as bits).
__device__ __forceinline__ bool eval_predicate(const Predicate& P, int64_t i) {
  uint32_t stack = 0;
  int sp = 0;
  for (int k = 0; k < P.nops; ++k) {
    const int code = P.code[k];
    if (code <= ABM_SELECT_NE) {
      const int a = P.arg[k];
      bool r;
      switch (P.dtype[a]) {
        case ABM_SELECT_F32:
          r = compare(static_cast<const float*>(P.attr[a])[i], P.value_f32[k], code);
          break;
        case ABM_SELECT_I32:
          r = compare(static_cast<double>(static_cast<const int32_t*>(P.attr[a])[i]),
                      P.value_f64[k], code);
          break;
        case ABM_SELECT_I8:
          r = compare(static_cast<double>(static_cast<const int8_t*>(P.attr[a])[i]),
                      P.value_f64[k], code);
          break;
        default:
          r = compare(static_cast<double>(static_cast<const uint8_t*>(P.attr[a])[i]),
                      P.value_f64[k], code);
          break;
      }
      stack = (stack & ~(1u << sp)) | (static_cast<uint32_t>(r) << sp);
      ++sp;
    } else if (code == ABM_SELECT_NOT) {
      stack ^= 1u << (sp - 1);
    } else {
      const uint32_t b = (stack >> (sp - 1)) & 1u, a = (stack >> (sp - 2)) & 1u;
      const uint32_t r = code == ABM_SELECT_AND ? (a & b) : (a | b);
      sp -= 1;
      stack = (stack & ~(1u << (sp - 1))) | (r << (sp - 1));
    }
  }
  return (stack & 1u) != 0;
}

__device__ __forceinline__ uint32_t predicate_flags(const Predicate& P, int64_t n, int64_t base) {
  uint32_t bits = 0;
#pragma unroll 4
  for (int j = 0; j < kSelPerThread; ++j)
    if (base + j < n && eval_predicate(P, base + j)) bits |= 1u << j;
  return bits;
}

__global__ void __launch_bounds__(kSelThreads)
select_pred_count_kernel(const Predicate P, int64_t n, int32_t* __restrict__ tile_counts) {
  __shared__ int swarp[kSelThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kSelPerThread;
  const int c = __popc(predicate_flags(P, n, base));
  const int wsum = abm::warp_sum(c);
  if ((threadIdx.x & 31) == 0) swarp[threadIdx.x >> 5] = wsum;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < kSelThreads / 32; ++w) s += swarp[w];
    tile_counts[blockIdx.x] = s;
  }
}

__global__ void __launch_bounds__(kSelThreads)
select_pred_scatter_kernel(const Predicate P, int64_t n, const int64_t* __restrict__ tile_offsets,
                           int32_t* __restrict__ out_idx) {
  __shared__ int swarp[kSelThreads / 32];
  __shared__ int32_t sidx[kTile];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kSelPerThread;
  const uint32_t bits = predicate_flags(P, n, base);
  const int c = __popc(bits);
  int incl = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += u;
  }
  if (lane == 31) swarp[warp] = incl;
  __syncthreads();
  int warp_excl = 0, total = 0;
#pragma unroll
  for (int w = 0; w < kSelThreads / 32; ++w) {
    warp_excl += w < warp ? swarp[w] : 0;
    total += swarp[w];
  }
  int pos = warp_excl + (incl - c);
  for (uint32_t rest = bits; rest; rest &= rest - 1)
    sidx[pos++] = (int32_t)(base + __ffs(rest) - 1);
  __syncthreads();
  int32_t* __restrict__ dst = out_idx + tile_offsets[blockIdx.x];
  for (int k = threadIdx.x; k < total; k += kSelThreads) dst[k] = sidx[k];
}

// ---- reductions -------------------------------------------------------------------------
constexpr int kRedThreads = 256;

// min and max that return NaN when either operand is NaN (as jnp.min / jnp.max do; fmin
// and fmax would drop it).
__device__ __forceinline__ double nan_min(double a, double b) {
  return (a != a || b != b) ? a + b : fmin(a, b);
}
__device__ __forceinline__ double nan_max(double a, double b) {
  return (a != a || b != b) ? a + b : fmax(a, b);
}

__device__ __forceinline__ double combine(int op, double a, double b) {
  return op == 2 ? nan_min(a, b) : (op == 3 ? nan_max(a, b) : a + b);
}

// op: 0 sum, 1 mean, 2 min, 3 max.  Sums accumulate in double in a fixed tree; a NaN
// anywhere makes every result NaN.
__global__ void __launch_bounds__(kRedThreads)
reduce_partial_kernel(const float* __restrict__ x, int64_t n, int op, double* __restrict__ part) {
  __shared__ double s[kRedThreads];
  double acc = (op == 2) ? INFINITY : (op == 3 ? -INFINITY : 0.0);
  for (int64_t i = blockIdx.x * (int64_t)kRedThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kRedThreads)
    acc = combine(op, acc, static_cast<double>(x[i]));
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = kRedThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] = combine(op, s[threadIdx.x], s[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

__global__ void reduce_final_kernel(const double* __restrict__ part, int nparts, int64_t n, int op,
                                    float* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double acc = (op == 2) ? INFINITY : (op == 3 ? -INFINITY : 0.0);
  for (int b = 0; b < nparts; ++b) acc = combine(op, acc, part[b]);
  if (op == 1) acc /= (double)n;
  *out = (float)acc;
}

int reduce_blocks(int64_t n) {
  int64_t b = (n + kRedThreads - 1) / kRedThreads;
  const int64_t cap = (int64_t)abm_host::sm_count() * 4;
  if (b > cap) b = cap;
  return (int)(b < 1 ? 1 : b);
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace

extern "C" {

size_t abm_select_workspace_bytes(int64_t n) {
  if (n <= 0) return 0;
  const int64_t tiles = (n + kTile - 1) / kTile;
  return align_up((size_t)tiles * sizeof(int32_t), 256) + (size_t)tiles * sizeof(int64_t);
}

int abm_select_indices(const uint8_t* mask, int64_t n, int32_t* out_idx, int64_t* count,
                       void* workspace, size_t workspace_bytes, void* stream) {
  if (!mask || !out_idx || !count || n < 0 || n > 0x7FFFFFFFll) return ABM_ERR_BADARG;
  cudaStream_t s = abm_host::as_stream(stream);
  if (n == 0) {
    return abm_host::record_cuda_error(cudaMemsetAsync(count, 0, sizeof(int64_t), s),
                                       "abm_select_indices");
  }
  const size_t need = abm_select_workspace_bytes(n);
  if (!workspace || workspace_bytes < need || !abm_host::aligned(workspace, 256))
    return ABM_ERR_WORKSPACE;
  const int64_t tiles = (n + kTile - 1) / kTile;
  int32_t* tile_counts = static_cast<int32_t*>(workspace);
  int64_t* tile_offsets = reinterpret_cast<int64_t*>(
      static_cast<char*>(workspace) + align_up((size_t)tiles * sizeof(int32_t), 256));
  const bool vec_ok = abm_host::aligned(mask, 16);
  select_count_kernel<<<(unsigned)tiles, kSelThreads, 0, s>>>(mask, n, vec_ok, tile_counts);
  int st = abm_host::check_launch("abm_select_indices/count");
  if (st) return st;
  select_scan_kernel<<<1, 1024, 0, s>>>(tile_counts, tiles, tile_offsets, count);
  st = abm_host::check_launch("abm_select_indices/scan");
  if (st) return st;
  select_scatter_kernel<<<(unsigned)tiles, kSelThreads, 0, s>>>(mask, n, vec_ok, tile_offsets,
                                                                out_idx);
  return abm_host::check_launch("abm_select_indices/scatter");
}

int abm_select_where(const abm_select_attr* attrs, int32_t nattrs, const abm_select_op* program,
                     int32_t nops, int64_t n, int32_t* out_idx, int64_t* count, void* workspace,
                     size_t workspace_bytes, void* stream) {
  if (!attrs || !program || !out_idx || !count || nattrs <= 0 || nattrs > kPredAttrs ||
      nops <= 0 || nops > kPredOps || n < 0 || n > 0x7FFFFFFFll)
    return ABM_ERR_BADARG;
  Predicate P{};
  for (int a = 0; a < nattrs; ++a) {
    if (!attrs[a].data || attrs[a].dtype < ABM_SELECT_F32 || attrs[a].dtype > ABM_SELECT_U8)
      return ABM_ERR_BADARG;
    P.attr[a] = attrs[a].data;
    P.dtype[a] = attrs[a].dtype;
  }
  // the program must leave exactly one flag and never pop an empty stack
  int depth = 0;
  for (int k = 0; k < nops; ++k) {
    const int code = program[k].code;
    if (code >= ABM_SELECT_LT && code <= ABM_SELECT_NE) {
      if (program[k].attr < 0 || program[k].attr >= nattrs) return ABM_ERR_BADARG;
      ++depth;
    } else if (code == ABM_SELECT_NOT) {
      if (depth < 1) return ABM_ERR_BADARG;
    } else if (code == ABM_SELECT_AND || code == ABM_SELECT_OR) {
      if (depth < 2) return ABM_ERR_BADARG;
      --depth;
    } else {
      return ABM_ERR_BADARG;
    }
    P.code[k] = code;
    P.arg[k] = program[k].attr;
    P.value_f32[k] = static_cast<float>(program[k].value);
    P.value_f64[k] = program[k].value;
  }
  if (depth != 1) return ABM_ERR_BADARG;
  P.nops = nops;
  cudaStream_t s = abm_host::as_stream(stream);
  if (n == 0) {
    return abm_host::record_cuda_error(cudaMemsetAsync(count, 0, sizeof(int64_t), s),
                                       "abm_select_where");
  }
  const size_t need = abm_select_workspace_bytes(n);
  if (!workspace || workspace_bytes < need || !abm_host::aligned(workspace, 256))
    return ABM_ERR_WORKSPACE;
  const int64_t tiles = (n + kTile - 1) / kTile;
  int32_t* tile_counts = static_cast<int32_t*>(workspace);
  int64_t* tile_offsets = reinterpret_cast<int64_t*>(
      static_cast<char*>(workspace) + align_up((size_t)tiles * sizeof(int32_t), 256));
  select_pred_count_kernel<<<(unsigned)tiles, kSelThreads, 0, s>>>(P, n, tile_counts);
  int st = abm_host::check_launch("abm_select_where/count");
  if (st) return st;
  select_scan_kernel<<<1, 1024, 0, s>>>(tile_counts, tiles, tile_offsets, count);
  st = abm_host::check_launch("abm_select_where/scan");
  if (st) return st;
  select_pred_scatter_kernel<<<(unsigned)tiles, kSelThreads, 0, s>>>(P, n, tile_offsets, out_idx);
  return abm_host::check_launch("abm_select_where/scatter");
}

int abm_gather_rows(const void* src, int64_t nrows_src, int64_t row_bytes, const int32_t* idx,
                    int64_t count, void* dst, void* stream) {
  if (!src || !dst || row_bytes <= 0 || count < 0 || nrows_src < 0) return ABM_ERR_BADARG;
  if (count == 0) return ABM_OK;
  if (!idx || nrows_src == 0) return ABM_ERR_BADARG;  // no row to gather from
  cudaStream_t s = abm_host::as_stream(stream);
  const int threads = 256;
  const bool words = row_bytes % 4 == 0 && abm_host::aligned(src, 4) && abm_host::aligned(dst, 4);
  const int64_t total = words ? count * (row_bytes / 4) : count * row_bytes;
  int64_t blocks = (total + threads - 1) / threads;
  const int64_t cap = (int64_t)abm_host::sm_count() * 16;
  if (blocks > cap) blocks = cap;
  if (words)
    gather_rows_words<<<(unsigned)blocks, threads, 0, s>>>(
        static_cast<const uint32_t*>(src), idx, count, row_bytes / 4, static_cast<uint32_t*>(dst),
        nrows_src);
  else
    gather_rows_bytes<<<(unsigned)blocks, threads, 0, s>>>(
        static_cast<const uint8_t*>(src), idx, count, row_bytes, static_cast<uint8_t*>(dst),
        nrows_src);
  return abm_host::finish(stream, "abm_gather_rows");
}

size_t abm_reduce_workspace_bytes(int64_t n) {
  if (n <= 0) return 0;
  return (size_t)reduce_blocks(n) * sizeof(double);
}

int abm_reduce_f32(const float* x, int64_t n, int op, float* out, void* workspace,
                   size_t workspace_bytes, void* stream) {
  if (!x || !out || n <= 0 || op < 0 || op > 3) return ABM_ERR_BADARG;
  const size_t need = abm_reduce_workspace_bytes(n);
  if (!workspace || workspace_bytes < need || !abm_host::aligned(workspace, 8))
    return ABM_ERR_WORKSPACE;
  cudaStream_t s = abm_host::as_stream(stream);
  const int blocks = reduce_blocks(n);
  double* part = static_cast<double*>(workspace);
  reduce_partial_kernel<<<blocks, kRedThreads, 0, s>>>(x, n, op, part);
  int st = abm_host::check_launch("abm_reduce_f32/partial");
  if (st) return st;
  reduce_final_kernel<<<1, 32, 0, s>>>(part, blocks, n, op, out);
  return abm_host::check_launch("abm_reduce_f32/final");
}

}  // extern "C"

// ---- compaction without any allocation ---------------------------------------------------
// abm_select_indices needs a workspace, which most callers take from their allocator.  Some
// callers cannot allocate device memory at the moment they need a selection: a host
// application that hands the engine a fixed device-memory budget and forbids growth, or a
// latency-critical loop that must not pay the implicit device synchronisation that
// cudaMalloc/cudaFree can cause.  For them the per-tile scratch lives in a fixed array in
// the library's own device image instead.  Every GPU that loads the library holds this
// array (192 KiB) until the process exits.
#include <mutex>

namespace {

constexpr int64_t kNoAllocMaxN = int64_t(1) << 26;              // 67,108,864 mask entries
constexpr int64_t kNoAllocMaxTiles = kNoAllocMaxN / kTile;       // 16,384 tiles
constexpr size_t kNoAllocCountsBytes = (size_t)kNoAllocMaxTiles * sizeof(int32_t);
constexpr size_t kNoAllocScratchBytes =
    kNoAllocCountsBytes + (size_t)kNoAllocMaxTiles * sizeof(int64_t);

// tile counts (int32[kNoAllocMaxTiles]) followed by tile offsets (int64[kNoAllocMaxTiles])
static __device__ __align__(256) unsigned char g_select_scratch[kNoAllocScratchBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_addr[kNoAllocMaxDevices] = {};
unsigned long long g_noalloc_ctx[kNoAllocMaxDevices] = {};  // context id of each address

// Unique id of the calling thread's current CUDA context (the driver's cuCtxGetCurrent and
// cuCtxGetId, reached through the runtime's entry-point query, so the library links only
// the runtime).  Ids are never reused, so a context torn down and created again (for example
// after cudaDeviceReset) has a new id.  0 when the driver cannot say.
unsigned long long current_context_id() {
  using GetCurrent = int (*)(void**);
  using GetId = int (*)(void*, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {  // under g_noalloc_mu
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
    cudaGetLastError();
    looked_up = true;
  }
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&ctx) == 0 && ctx && get_id(ctx, &id) == 0) return id;
  return 0;
}

// Device address of g_select_scratch in the current device's context.  In host code the
// symbol names a host-side stand-in, so the address must come from the runtime: looked up
// with that device current, and cached with the id of the context it belongs to.  A call
// in another context of the device (the primary context was reset and created again) looks
// the address up again, so no call writes through an address of a destroyed context.
int noalloc_scratch(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return abm_host::record_cuda_error(e, "abm_select_indices_noalloc/device");
  if (dev < 0 || dev >= kNoAllocMaxDevices) return ABM_ERR_BADARG;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  const unsigned long long ctx = current_context_id();  // 0 before the context is current
  if (g_noalloc_addr[dev] == nullptr || ctx == 0 || ctx != g_noalloc_ctx[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_select_scratch);  // makes the primary context current
    if (e != cudaSuccess || p == nullptr)
      return abm_host::record_cuda_error(e != cudaSuccess ? e : cudaErrorInvalidSymbol,
                                         "abm_select_indices_noalloc/cudaGetSymbolAddress");
    g_noalloc_addr[dev] = p;
    g_noalloc_ctx[dev] = current_context_id();
  }
  *out = g_noalloc_addr[dev];
  return ABM_OK;
}

}  // namespace

extern "C" {

int abm_select_indices_noalloc(const uint8_t* mask, int64_t n, int32_t* out_idx, int64_t* count,
                               void* stream) {
  if ((!mask && n > 0) || !out_idx || !count || n < 0) return ABM_ERR_BADARG;
  if (n > kNoAllocMaxN) return ABM_ERR_BADARG;  // beyond the fixed scratch: use abm_select_indices
  cudaStream_t s = abm_host::as_stream(stream);
  if (n == 0) {
    return abm_host::record_cuda_error(cudaMemsetAsync(count, 0, sizeof(int64_t), s),
                                       "abm_select_indices_noalloc");
  }
  void* scratch = nullptr;
  int st = noalloc_scratch(&scratch);
  if (st) return st;
  // Nothing in the scratch has to start at zero: each call writes every tile count and
  // offset it later reads.
  const int64_t tiles = (n + kTile - 1) / kTile;
  int32_t* tile_counts = static_cast<int32_t*>(scratch);
  int64_t* tile_offsets =
      reinterpret_cast<int64_t*>(static_cast<char*>(scratch) + kNoAllocCountsBytes);
  const bool vec_ok = abm_host::aligned(mask, 16);
  select_count_kernel<<<(unsigned)tiles, kSelThreads, 0, s>>>(mask, n, vec_ok, tile_counts);
  st = abm_host::check_launch("abm_select_indices_noalloc/count");
  if (st) return st;
  select_scan_kernel<<<1, 1024, 0, s>>>(tile_counts, tiles, tile_offsets, count);
  st = abm_host::check_launch("abm_select_indices_noalloc/scan");
  if (st) return st;
  select_scatter_kernel<<<(unsigned)tiles, kSelThreads, 0, s>>>(mask, n, vec_ok, tile_offsets,
                                                                out_idx);
  return abm_host::check_launch("abm_select_indices_noalloc/scatter");
}

}  // extern "C"
