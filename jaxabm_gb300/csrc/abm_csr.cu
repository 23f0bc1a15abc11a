// Network CSR construction on the device: a directed edge list (src[e], dst[e]) becomes
// row_ptr int32[n+1] / col int32[E] with row i holding dst[e] of the edges whose source is i,
// in ascending e -- the order of Network.add_edges (jaxabm/agentpy.py:559-582 appends edges;
// the host path sorts them stably by source).
//
// A least-significant-digit radix sort of (source, destination) pairs, 8 bits per pass, is
// stable, so equal sources keep their edge order.  Each pass is three launches over tiles of
// 4096 edges: per-tile digit histograms (digit-major, so one exclusive scan gives every
// (digit, tile) its output offset), the scan, and a stable scatter that ranks each edge among
// the equal digits of its tile (warp match + per-warp counts in shared memory).  Row offsets
// come from the sorted sources.  Edges whose source is outside 0..n-1 sort after every row
// (they are not in any row) and set *status; a destination outside 0..n-1 sets it too.

#include "abm_common.cuh"

namespace {

constexpr int kCsrThreads = 256;
constexpr int kCsrItems = 16;                          // edges per thread and tile
constexpr int kCsrTile = kCsrThreads * kCsrItems;      // 4096
constexpr int kRadix = 256;
constexpr int kCsrWarps = kCsrThreads / 32;

__device__ __forceinline__ int32_t key_of(const int32_t* __restrict__ keys,
                                          const int32_t* __restrict__ src, int64_t e, int32_t n,
                                          int32_t* __restrict__ status) {
  if (keys) return keys[e];
  const int32_t s = src[e];
  if (s < 0 || s >= n) {
    atomicExch(status, 1);
    return n;
  }
  return s;
}

// hist[d * ntiles + tile] = number of edges of the tile whose digit is d.
__global__ void __launch_bounds__(kCsrThreads)
csr_hist_kernel(const int32_t* __restrict__ keys, const int32_t* __restrict__ src, int64_t E,
                int32_t n, int shift, int64_t ntiles, int32_t* __restrict__ hist,
                int32_t* __restrict__ status) {
  __shared__ int32_t h[kRadix];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t t0 = (int64_t)blockIdx.x * kCsrTile;
#pragma unroll 4
  for (int r = 0; r < kCsrItems; ++r) {
    const int64_t e = t0 + (int64_t)r * kCsrThreads + threadIdx.x;
    if (e < E) atomicAdd(&h[(key_of(keys, src, e, n, status) >> shift) & (kRadix - 1)], 1);
  }
  __syncthreads();
  hist[(int64_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Single block: in-place exclusive scan of v[0..m) (int32 totals below 2^31).  Warp w owns a
// contiguous chunk read 128 values at a time, four per lane.
__global__ void __launch_bounds__(1024) csr_scan_kernel(int32_t* __restrict__ v, int64_t m) {
  __shared__ int32_t swarp[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t per = ((m + 31) / 32 + 127) / 128 * 128;
  const int64_t c0 = (int64_t)warp * per;
  const int64_t c1 = c0 + per < m ? c0 + per : m;
  int32_t sum = 0;
  for (int64_t b = c0; b < c1; b += 128)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int64_t t = b + 4 * lane + q;
      sum += t < c1 ? v[t] : 0;
    }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if (lane == 0) swarp[warp] = sum;
  __syncthreads();
  if (warp == 0) {
    int32_t w = swarp[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t u = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += u;
    }
    swarp[lane] = w;
  }
  __syncthreads();
  int32_t run = warp > 0 ? swarp[warp - 1] : 0;
  for (int64_t b = c0; b < c1; b += 128) {
    int32_t x[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int64_t t = b + 4 * lane + q;
      x[q] = t < c1 ? v[t] : 0;
    }
    const int32_t mine = x[0] + x[1] + x[2] + x[3];
    int32_t incl = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t u = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += u;
    }
    int32_t off = run + (incl - mine);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int64_t t = b + 4 * lane + q;
      if (t < c1) v[t] = off;
      off += x[q];
    }
    run += __shfl_sync(0xffffffffu, incl, 31);
  }
}

// Stable scatter of one pass.  Sub-round r of a tile covers its edges r*256 .. r*256+255
// (one per thread, in edge order); an edge's output position is the scanned offset of
// (digit, tile) + the edges of the tile with that digit in earlier sub-rounds + those in
// earlier warps of this sub-round + its rank among equal digits in its warp.
__global__ void __launch_bounds__(kCsrThreads)
csr_scatter_kernel(const int32_t* __restrict__ keys, const int32_t* __restrict__ src,
                   const int32_t* __restrict__ vals, int64_t E, int32_t n, int shift,
                   int64_t ntiles, const int32_t* __restrict__ offsets,
                   int32_t* __restrict__ keys_out, int32_t* __restrict__ vals_out,
                   int32_t* __restrict__ status) {
  __shared__ int32_t base[kRadix];             // offset of (digit, this tile) + earlier rounds
  __shared__ int32_t wcount[kCsrWarps][kRadix];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  base[threadIdx.x] = offsets[(int64_t)threadIdx.x * ntiles + blockIdx.x];
  const int64_t t0 = (int64_t)blockIdx.x * kCsrTile;
  const unsigned lt = (1u << lane) - 1u;
  for (int r = 0; r < kCsrItems; ++r) {
#pragma unroll
    for (int w = 0; w < kCsrWarps; ++w) wcount[w][threadIdx.x] = 0;
    __syncthreads();
    const int64_t e = t0 + (int64_t)r * kCsrThreads + threadIdx.x;
    const bool valid = e < E;
    int32_t k = 0, v = 0;
    if (valid) {
      k = key_of(keys, src, e, n, status);
      v = vals[e];
    }
    const int d = valid ? (k >> shift) & (kRadix - 1) : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int rank = __popc(peers & lt);
    if (valid && rank == 0) wcount[warp][d] = __popc(peers);
    __syncthreads();
    // per digit: exclusive prefix over the warps, and the round's total into base
    {
      const int dd = threadIdx.x;
      int32_t acc = 0;
#pragma unroll
      for (int w = 0; w < kCsrWarps; ++w) {
        const int32_t c = wcount[w][dd];
        wcount[w][dd] = acc;
        acc += c;
      }
      // base[dd] is read below by this sub-round's edges before it advances
      __syncthreads();
      if (valid) {
        const int32_t pos = base[d] + wcount[warp][d] + rank;
        keys_out[pos] = k;
        vals_out[pos] = v;
      }
      __syncthreads();
      base[dd] += acc;
    }
  }
}

// row_ptr[i] = first sorted position whose source is >= i (sources past n-1 sort last).
__global__ void csr_rows_kernel(const int32_t* __restrict__ keys, int64_t E, int32_t n,
                                int32_t* __restrict__ row_ptr) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e <= E;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int32_t prev = e > 0 ? keys[e - 1] : -1;
    const int32_t cur = e < E ? keys[e] : n;
    for (int32_t i = prev + 1; i <= cur && i <= n; ++i) row_ptr[i] = (int32_t)e;
  }
}

// *status = 1 when a destination lies outside 0..n-1.
__global__ void csr_check_dst_kernel(const int32_t* __restrict__ dst, int64_t E, int32_t n,
                                     int32_t* __restrict__ status) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E;
       e += (int64_t)gridDim.x * blockDim.x)
    if (dst[e] < 0 || dst[e] >= n) atomicExch(status, 1);
}

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

int passes_for(int64_t n) {
  int bits = 1;
  while (bits < 31 && (int64_t(1) << bits) <= n) ++bits;  // keys take values 0..n
  return (bits + 7) / 8;
}

}  // namespace

extern "C" {

size_t abm_csr_workspace_bytes(int64_t num_edges, int64_t n) {
  if (num_edges < 0 || n <= 0) return 0;
  const int64_t ntiles = (num_edges + kCsrTile - 1) / kCsrTile;
  return 4 * align256((size_t)num_edges * sizeof(int32_t)) +
         align256((size_t)kRadix * (size_t)(ntiles > 0 ? ntiles : 1) * sizeof(int32_t));
}

int abm_csr_from_edges(const int32_t* src, const int32_t* dst, int64_t num_edges, int64_t n,
                       int32_t* row_ptr, int32_t* col, int32_t* status, void* workspace,
                       size_t workspace_bytes, void* stream) {
  if (!row_ptr || !status || n <= 0 || n >= 0x7FFFFFFFll || num_edges < 0 ||
      num_edges >= 0x7FFFFFFFll || (num_edges > 0 && (!src || !dst || !col)))
    return ABM_ERR_BADARG;
  const size_t need = abm_csr_workspace_bytes(num_edges, n);
  if (!workspace || workspace_bytes < need || !abm_host::aligned(workspace, 256))
    return ABM_ERR_WORKSPACE;
  cudaStream_t s = abm_host::as_stream(stream);
  int st = abm_host::record_cuda_error(cudaMemsetAsync(status, 0, sizeof(int32_t), s),
                                       "abm_csr_from_edges/status");
  if (st) return st;
  if (num_edges == 0) {
    return abm_host::record_cuda_error(
        cudaMemsetAsync(row_ptr, 0, (size_t)(n + 1) * sizeof(int32_t), s), "abm_csr_from_edges/rows");
  }
  const int64_t E = num_edges;
  const int64_t ntiles = (E + kCsrTile - 1) / kCsrTile;
  char* p = static_cast<char*>(workspace);
  int32_t* kbuf[2];
  int32_t* vbuf[2];
  kbuf[0] = reinterpret_cast<int32_t*>(p);
  p += align256((size_t)E * sizeof(int32_t));
  vbuf[0] = reinterpret_cast<int32_t*>(p);
  p += align256((size_t)E * sizeof(int32_t));
  kbuf[1] = reinterpret_cast<int32_t*>(p);
  p += align256((size_t)E * sizeof(int32_t));
  vbuf[1] = reinterpret_cast<int32_t*>(p);
  p += align256((size_t)E * sizeof(int32_t));
  int32_t* hist = reinterpret_cast<int32_t*>(p);

  const int passes = passes_for(n);
  const int32_t* kin = nullptr;  // the first pass reads (and checks) the sources
  const int32_t* vin = dst;
  for (int q = 0; q < passes; ++q) {
    const int shift = 8 * q;
    int32_t* kout = kbuf[q & 1];
    int32_t* vout = q == passes - 1 ? col : vbuf[q & 1];
    csr_hist_kernel<<<(unsigned)ntiles, kCsrThreads, 0, s>>>(kin, src, E, (int32_t)n, shift, ntiles,
                                                             hist, status);
    if ((st = abm_host::check_launch("abm_csr_from_edges/hist"))) return st;
    csr_scan_kernel<<<1, 1024, 0, s>>>(hist, (int64_t)kRadix * ntiles);
    if ((st = abm_host::check_launch("abm_csr_from_edges/scan"))) return st;
    csr_scatter_kernel<<<(unsigned)ntiles, kCsrThreads, 0, s>>>(kin, src, vin, E, (int32_t)n, shift,
                                                                ntiles, hist, kout, vout, status);
    if ((st = abm_host::check_launch("abm_csr_from_edges/scatter"))) return st;
    kin = kout;
    vin = vout;
  }
  const int64_t cap = (int64_t)abm_host::sm_count() * 8;
  int64_t blocks = (E + 1 + 255) / 256;
  if (blocks > cap) blocks = cap;
  csr_rows_kernel<<<(unsigned)blocks, 256, 0, s>>>(kin, E, (int32_t)n, row_ptr);
  if ((st = abm_host::check_launch("abm_csr_from_edges/rows"))) return st;
  csr_check_dst_kernel<<<(unsigned)blocks, 256, 0, s>>>(dst, E, (int32_t)n, status);
  return abm_host::check_launch("abm_csr_from_edges/check");
}

}  // extern "C"
