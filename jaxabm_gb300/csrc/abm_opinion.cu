// Differentiable bounded-confidence opinion model on a symmetric network (K8).
//
// B calibration instances share one CSR graph; their opinions are interleaved o[N][B]
// (float32), so a neighbour's B values are one contiguous 4*B-byte row: a group of B/4
// lanes reads it with 128-bit loads.  Per step, for node i and instance b:
//   d_j = o_j - o_i;  s_j = sigmoid((eps_b - |d_j|) * (1/tau_b))
//   acc = sum_j s_j * d_j  (in CSR order);  o_i' = o_i + mu_b * (acc / deg_i)
// which is the model o_i += mu * mean_j sigmoid((eps - |o_j - o_i|)/tau) (o_j - o_i).
// The forward is exact float32 arithmetic in a fixed order: every operation is one IEEE-754
// operation rounded to nearest -- add, multiply, fused multiply-add (one rounding, written
// out where it is used, never left to the compiler), correctly rounded reciprocal and
// division -- and the sigmoid is 1 / (1 + exp(-z)) with the table-driven exponential below,
// so the C oracle's float32 restatement of the same sequence gives the same bits.
//
// Adjoint (reverse mode, the gradient jax.grad of the reference's run loop would give,
// jaxabm/analysis.py:494-522): with g(d) = s d and g'(d) = s - |d| s (1 - s) / tau,
//   lambda_i^t = lambda_i + mu * sum_{j in N(i)} g'(d_ij) (lambda_j / deg_j - lambda_i / deg_i)
// (valid because the graph is symmetric and g' is even), and the parameter gradients
// accumulate lambda_i^{t+1} dF_i/dtheta at o^t:
//   dF_i/dmu  = (1/deg_i) sum_j g(d_ij)
//   dF_i/deps = (mu/deg_i) sum_j s(1-s) d_ij / tau
//   dF_i/dtau = (mu/deg_i) sum_j s(1-s) (-z_ij / tau) d_ij,   z = (eps - |d|) / tau
// The per-CTA partial sums of the parameter gradients are kept per CTA across all steps
// and reduced in a fixed order, so gradients are deterministic.

#include "abm_common.cuh"

namespace {

constexpr int kOpThreads = 256;

// 16-byte load of the four floats of lane group `sub` of a row into registers.
__device__ __forceinline__ void ld4(const float* __restrict__ row, int sub, float (&a)[4]) {
  const float4 v = reinterpret_cast<const float4*>(row)[sub];
  a[0] = v.x;
  a[1] = v.y;
  a[2] = v.z;
  a[3] = v.w;
}

// 2^(j/32) for j = 0..31, each the float32 nearest to the exact value.
__device__ const float kExp2Table[32] = {
    0x1.000000p+0f, 0x1.059b0ep+0f, 0x1.0b5586p+0f, 0x1.11301ep+0f, 0x1.172b84p+0f,
    0x1.1d4874p+0f, 0x1.2387a6p+0f, 0x1.29e9e0p+0f, 0x1.306fe0p+0f, 0x1.371a74p+0f,
    0x1.3dea64p+0f, 0x1.44e086p+0f, 0x1.4bfdaep+0f, 0x1.5342b6p+0f, 0x1.5ab07ep+0f,
    0x1.6247ecp+0f, 0x1.6a09e6p+0f, 0x1.71f75ep+0f, 0x1.7a1148p+0f, 0x1.82589ap+0f,
    0x1.8ace54p+0f, 0x1.93737cp+0f, 0x1.9c4918p+0f, 0x1.a5503cp+0f, 0x1.ae89fap+0f,
    0x1.b7f770p+0f, 0x1.c199bep+0f, 0x1.cb720ep+0f, 0x1.d5818ep+0f, 0x1.dfc974p+0f,
    0x1.ea4afap+0f, 0x1.f50766p+0f};
constexpr float kExpK = 0x1.715476p+5f;   // 32 / ln 2
constexpr float kExpL1 = 0x1.62c000p-6f;  // ln 2 / 32, leading 11 bits
constexpr float kExpL2 = 0x1.217f7ep-17f; // ln 2 / 32 - kExpL1
constexpr float kExpC3 = 0x1.555556p-3f;  // 1 / 6
constexpr float kExpRound = 0x1.8p+23f;   // 1.5 * 2^23

// exp(x) in float32 by Tang's table-driven method (P. T. P. Tang, "Table-driven
// implementation of the exponential function in IEEE floating-point arithmetic", ACM TOMS
// 15(2), 1989): N = rint(x * 32 / ln 2); r = fma(-N, L2, fma(-N, L1, x)) with
// L1 + L2 = ln 2 / 32 (L1 has 11 significant bits, so x - N L1 is exact); exp(r) - 1 by its
// Taylor polynomial p = fma(r^2, fma(r, 1/6, 1/2), r) (|r| <= ln 2 / 64: truncation error
// below 6e-10); exp(x) = 2^(N >> 5) fma(T[N & 31], p, T[N & 31]).  N is computed without
// a rounding or conversion instruction (below), with the same value as rint.  x is clamped to
// [-87, 88], so every intermediate is normal and the scaling is an exact add to the
// exponent field.  About 1 ulp from exp over the clamped range.  T is kExp2Table staged in
// shared memory.
__device__ __forceinline__ float exp_table(float x, const float* T) {
  x = fminf(fmaxf(x, -87.0f), 88.0f);
  // rint(x * 32 / ln 2) without a rounding or conversion instruction: adding 1.5 * 2^23 to
  // a float of magnitude below 2^22 leaves its nearest integer (ties to even, as rint) in
  // the low mantissa bits; subtracting it back is exact, and the bit patterns' difference
  // is that integer (|x * 32 / ln 2| <= 4064 here)
  const float shifted = __fadd_rn(__fmul_rn(x, kExpK), kExpRound);
  const float nf = __fsub_rn(shifted, kExpRound);
  const int N = __float_as_int(shifted) - __float_as_int(kExpRound);
  const float r = __fmaf_rn(-nf, kExpL2, __fmaf_rn(-nf, kExpL1, x));
  const float p = __fmaf_rn(__fmul_rn(r, r), __fmaf_rn(r, kExpC3, 0.5f), r);
  const float t = T[N & 31];
  const float e = __fmaf_rn(t, p, t);
  return __uint_as_float(__float_as_uint(e) + (static_cast<uint32_t>(N >> 5) << 23));
}

// sigmoid(z) = 1 / (1 + exp(-z)), reciprocal correctly rounded.
__device__ __forceinline__ float sigmoid_exact(float z, const float* T) {
  return __frcp_rn(__fadd_rn(1.0f, exp_table(-z, T)));
}

// The adjoint's sigmoid: the hardware exponential and reciprocal (__expf, __fdividef, about
// 2^-21 relative error for |z| <= 10); the adjoint is checked against the float64 gradient
// and central differences, not bit for bit, and reads states the exact forward produced.
__device__ __forceinline__ float sigmoid_z(float z) { return __fdividef(1.0f, 1.0f + __expf(-z)); }

template <int LPN>
__global__ void __launch_bounds__(kOpThreads)
opinion_step_kernel(const float* __restrict__ o, float* __restrict__ out,
                    const int32_t* __restrict__ rp, const int32_t* __restrict__ col, int n, int B,
                    const float* __restrict__ mu, const float* __restrict__ eps,
                    const float* __restrict__ tau) {
  __shared__ float T[32];
  if (threadIdx.x < 32) T[threadIdx.x] = kExp2Table[threadIdx.x];
  __syncthreads();
  const long long g = (long long)blockIdx.x * kOpThreads + threadIdx.x;
  const int node = (int)(g / LPN);
  const int sub = (int)(g % LPN);
  if (node >= n) return;
  float m[4], ep[4], it[4], oi[4], acc[4] = {0.f, 0.f, 0.f, 0.f};
  ld4(mu, sub, m);
  ld4(eps, sub, ep);
  ld4(tau, sub, it);
#pragma unroll
  for (int c = 0; c < 4; ++c) it[c] = __frcp_rn(it[c]);
  ld4(o + (size_t)node * B, sub, oi);
  const int r0 = rp[node], r1 = rp[node + 1];
#ifdef ABM_CHECKED
  const int nslots = rp[n];
#endif
  // acc += s(d) * d for one neighbour row (instances of this lane)
  auto edge = [&](const float (&oj)[4]) {
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const float d = __fsub_rn(oj[c], oi[c]);
      const float s = sigmoid_exact(__fmul_rn(__fsub_rn(ep[c], fabsf(d)), it[c]), T);
      acc[c] = __fmaf_rn(s, d, acc[c]);
    }
  };
  int e = r0;
  // two neighbour rows in flight per iteration; accumulation stays in CSR order
  for (; e + 1 < r1; e += 2) {
    float oa[4], ob[4];
    ld4(o + (size_t)ABM_IDX(col[ABM_IDX(e, nslots)], n) * B, sub, oa);
    ld4(o + (size_t)ABM_IDX(col[ABM_IDX(e + 1, nslots)], n) * B, sub, ob);
    edge(oa);
    edge(ob);
  }
  if (e < r1) {
    float oa[4];
    ld4(o + (size_t)ABM_IDX(col[ABM_IDX(e, nslots)], n) * B, sub, oa);
    edge(oa);
  }
  float res[4] = {oi[0], oi[1], oi[2], oi[3]};
  const int deg = r1 - r0;
  if (deg > 0) {
    const float fdeg = (float)deg;
#pragma unroll
    for (int c = 0; c < 4; ++c) res[c] = __fmaf_rn(m[c], __fdiv_rn(acc[c], fdeg), oi[c]);
  }
  reinterpret_cast<float4*>(out + (size_t)node * B)[sub] = make_float4(res[0], res[1], res[2], res[3]);
}

// The forward's sigmoid over an array (s[k] = sigmoid(z[k]) exactly as the step computes
// it), for bit-level checks against the oracle.
__global__ void opinion_sigmoid_kernel(const float* __restrict__ z, float* __restrict__ s,
                                       long long n) {
  __shared__ float T[32];
  if (threadIdx.x < 32) T[threadIdx.x] = kExp2Table[threadIdx.x];
  __syncthreads();
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x)
    s[k] = sigmoid_exact(z[k], T);
}

// One adjoint step over instance columns [c0, c0 + 4 LPN): lam_out from lam_in
// (= lambda^{t+1}) at the forward state o (= o^t); gpart[cta][b][3] += this CTA's lambda *
// dF/d(mu, eps, tau).  A launch covers at most kAdjCols columns, so the opinion and adjoint
// rows it gathers (kAdjCols floats per node each) stay in L2 across the step.
template <int LPN>
__global__ void __launch_bounds__(kOpThreads, 4)
opinion_adjoint_kernel(const float* __restrict__ o, const float* __restrict__ lam_in,
                       float* __restrict__ lam_out, const int32_t* __restrict__ rp,
                       const int32_t* __restrict__ col, const float* __restrict__ inv_deg, int n,
                       int B, int c0, const float* __restrict__ mu, const float* __restrict__ eps,
                       const float* __restrict__ tau, double* __restrict__ gpart) {
  extern __shared__ float sg[];  // [kOpThreads][12]: this thread's 4 instances x 3 params
  const long long g = (long long)blockIdx.x * kOpThreads + threadIdx.x;
  const int node = (int)(g / LPN);
  const int sub = (int)(g % LPN);
  // this launch's columns: rows are read from column c0 on
  o += c0;
  lam_in += c0;
  lam_out += c0;
  mu += c0;
  eps += c0;
  tau += c0;
  float gm[4] = {0.f, 0.f, 0.f, 0.f}, ge[4] = {0.f, 0.f, 0.f, 0.f}, gt[4] = {0.f, 0.f, 0.f, 0.f};
  if (node < n) {
    float m[4], ep[4], it[4], oi[4], li[4], li_d[4];
    ld4(mu, sub, m);
    ld4(eps, sub, ep);
    ld4(tau, sub, it);
#pragma unroll
    for (int c = 0; c < 4; ++c) it[c] = 1.0f / it[c];
    ld4(o + (size_t)node * B, sub, oi);
    ld4(lam_in + (size_t)node * B, sub, li);
    const int r0 = rp[node], r1 = rp[node + 1];
#ifdef ABM_CHECKED
    const int nslots = rp[n];
#endif
    const float inv_deg_i = inv_deg[node];
#pragma unroll
    for (int c = 0; c < 4; ++c) li_d[c] = r1 > r0 ? li[c] * inv_deg_i : li[c];
    float sl[4] = {0.f, 0.f, 0.f, 0.f};  // sum_j g'(d) (lam_j/deg_j - lam_i/deg_i)
    float sgd[4] = {0.f, 0.f, 0.f, 0.f}, sse[4] = {0.f, 0.f, 0.f, 0.f}, sst[4] = {0.f, 0.f, 0.f, 0.f};
    // one neighbour's contribution, accumulated in CSR order
    auto edge = [&](const float (&oj)[4], const float (&lj)[4], float inv_deg_j) {
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const float d = oj[c] - oi[c];
        const float a = fabsf(d);
        const float z = (ep[c] - a) * it[c];
        const float s = sigmoid_z(z);
        const float sp = s * (1.0f - s);
        const float gprime = s - a * sp * it[c];
        sl[c] = fmaf(gprime, fmaf(lj[c], inv_deg_j, -li_d[c]), sl[c]);
        sgd[c] = fmaf(s, d, sgd[c]);
        sse[c] = fmaf(sp * it[c], d, sse[c]);
        sst[c] = fmaf(-sp * z * it[c], d, sst[c]);
      }
    };
    int e = r0;
    // two neighbours' opinion and adjoint rows in flight per iteration
    for (; e + 1 < r1; e += 2) {
      const int ja = static_cast<int>(ABM_IDX(col[ABM_IDX(e, nslots)], n));
      const int jb = static_cast<int>(ABM_IDX(col[ABM_IDX(e + 1, nslots)], n));
      float oa[4], la[4], ob[4], lb[4];
      ld4(o + (size_t)ja * B, sub, oa);
      ld4(lam_in + (size_t)ja * B, sub, la);
      ld4(o + (size_t)jb * B, sub, ob);
      ld4(lam_in + (size_t)jb * B, sub, lb);
      const float da = inv_deg[ja], db = inv_deg[jb];
      edge(oa, la, da);
      edge(ob, lb, db);
    }
    if (e < r1) {
      const int j = static_cast<int>(ABM_IDX(col[ABM_IDX(e, nslots)], n));
      float oj[4], lj[4];
      ld4(o + (size_t)j * B, sub, oj);
      ld4(lam_in + (size_t)j * B, sub, lj);
      edge(oj, lj, inv_deg[j]);
    }
    float lo[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      lo[c] = fmaf(m[c], sl[c], li[c]);
      if (r1 > r0) {
        gm[c] = li[c] * (sgd[c] * inv_deg_i);
        ge[c] = li[c] * m[c] * (sse[c] * inv_deg_i);
        gt[c] = li[c] * m[c] * (sst[c] * inv_deg_i);
      }
    }
    reinterpret_cast<float4*>(lam_out + (size_t)node * B)[sub] = make_float4(lo[0], lo[1], lo[2], lo[3]);
  }
  // per-CTA reduction of the parameter gradients per instance column (fixed order; float
  // over the CTA's kNodes nodes, double across CTAs and steps)
  constexpr int kNodes = kOpThreads / LPN;
  float* mine = sg + (size_t)threadIdx.x * 12;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    mine[c] = gm[c];
    mine[4 + c] = ge[c];
    mine[8 + c] = gt[c];
  }
  __syncthreads();
  for (int q = threadIdx.x; q < LPN * 12; q += kOpThreads) {
    const int s_ = q / 12, v = q % 12;
    float acc = 0.0f;
    for (int k = 0; k < kNodes; ++k) acc += sg[(size_t)(k * LPN + s_) * 12 + v];
    // v: param*4 + component; instance b = c0 + 4*s_ + component
    const int param = v / 4, c = v % 4;
    const int b = c0 + 4 * s_ + c;
    gpart[((size_t)blockIdx.x * B + b) * 3 + param] += (double)acc;
  }
}

// lambda^T_i = sum_k dL/dm_k * k * o_i^(k-1) / N for the raw moments m_k, k = 1..4.
__global__ void opinion_adjoint_init_kernel(const float* __restrict__ o, int n, int B,
                                            const double* __restrict__ dldm,
                                            float* __restrict__ lam) {
  const long long total = (long long)n * B;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(g % B);
    const double x = o[g];
    const double* w = dldm + 4 * b;
    lam[g] = (float)((w[0] + 2.0 * w[1] * x + 3.0 * w[2] * x * x + 4.0 * w[3] * x * x * x) / n);
  }
}

// Raw moments: thread b of CTA c sums instance column b over rows [kMomRows c,
// kMomRows (c + 1)) in row order (float64), then the partials are summed over CTAs in
// CTA order.  The order of every sum depends only on n, not on the batch width B, so a
// column's moments are the same in a batch of any width.
constexpr int kMomRows = 64;

__global__ void opinion_moments_partial_kernel(const float* __restrict__ o, int n, int B,
                                               double* __restrict__ part) {
  const int b = threadIdx.x;
  if (b >= B) return;
  double a1 = 0, a2 = 0, a3 = 0, a4 = 0;
  const int r0 = blockIdx.x * kMomRows;
  const int r1 = min(n, r0 + kMomRows);
  for (int i = r0; i < r1; ++i) {
    const double x = o[(size_t)i * B + b];
    const double x2 = x * x;
    a1 += x;
    a2 += x2;
    a3 += x2 * x;
    a4 += x2 * x2;
  }
  double* out = part + ((size_t)blockIdx.x * B + b) * 4;
  out[0] = a1;
  out[1] = a2;
  out[2] = a3;
  out[3] = a4;
}

__global__ void sum_partials_kernel(const double* __restrict__ part, int nparts, int width,
                                    double scale, double* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= width) return;
  double s = 0.0;
  for (int p = 0; p < nparts; ++p) s += part[(size_t)p * width + k];
  out[k] = s * scale;
}

__global__ void inv_degree_kernel(const int32_t* __restrict__ rp, int n, float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const int d = rp[i + 1] - rp[i];
    out[i] = d > 0 ? 1.0f / (float)d : 0.0f;
  }
}

bool valid_batch(int B) { return B >= 4 && B <= 128 && (B & (B - 1)) == 0; }

// Instance columns per adjoint launch (a step of a wider batch is several launches).
constexpr int kAdjCols = 32;

int adjoint_cols(int B) { return B < kAdjCols ? B : kAdjCols; }

int step_blocks(int64_t n, int B) {
  const long long threads = n * (long long)(B / 4);
  return (int)((threads + kOpThreads - 1) / kOpThreads);
}

}  // namespace

#define ABM_OP_DISPATCH(KERNEL, LPN_, GRID, SMEM, STREAM, ...)                         \
  switch (LPN_) {                                                                     \
    case 1: KERNEL<1><<<GRID, kOpThreads, SMEM, STREAM>>>(__VA_ARGS__); break;          \
    case 2: KERNEL<2><<<GRID, kOpThreads, SMEM, STREAM>>>(__VA_ARGS__); break;          \
    case 4: KERNEL<4><<<GRID, kOpThreads, SMEM, STREAM>>>(__VA_ARGS__); break;          \
    case 8: KERNEL<8><<<GRID, kOpThreads, SMEM, STREAM>>>(__VA_ARGS__); break;          \
    case 16: KERNEL<16><<<GRID, kOpThreads, SMEM, STREAM>>>(__VA_ARGS__); break;        \
    default: KERNEL<32><<<GRID, kOpThreads, SMEM, STREAM>>>(__VA_ARGS__); break;        \
  }

extern "C" {

int abm_opinion_run(float* o, float* o_tmp, const int32_t* row_ptr, const int32_t* col, int64_t n,
                    int32_t B, const float* mu, const float* eps, const float* tau,
                    int32_t steps, int32_t ckpt_every, float* checkpoints, void* stream) {
  if (!o || !o_tmp || !row_ptr || !col || !mu || !eps || !tau || n <= 0 || n > 0x7FFFFFFFll ||
      steps < 0 || !valid_batch(B) || (checkpoints && ckpt_every <= 0))
    return ABM_ERR_BADARG;
  if (!abm_host::aligned(o, 16) || !abm_host::aligned(o_tmp, 16) || !abm_host::aligned(mu, 16) ||
      !abm_host::aligned(eps, 16) || !abm_host::aligned(tau, 16) ||
      (checkpoints && !abm_host::aligned(checkpoints, 16)))
    return ABM_ERR_BADARG;
  cudaStream_t s = abm_host::as_stream(stream);
  const size_t bytes = (size_t)n * B * sizeof(float);
  const int lpn = B / 4;
  const int blocks = step_blocks(n, B);
  float* cur = o;
  float* nxt = o_tmp;
  for (int32_t t = 0; t < steps; ++t) {
    if (checkpoints && t % ckpt_every == 0) {
      int st = abm_host::record_cuda_error(
          cudaMemcpyAsync(checkpoints + (size_t)(t / ckpt_every) * n * B, cur, bytes,
                          cudaMemcpyDeviceToDevice, s),
          "abm_opinion_run/checkpoint");
      if (st) return st;
    }
    ABM_OP_DISPATCH(opinion_step_kernel, lpn, blocks, 0, s, cur, nxt, row_ptr, col, (int)n, B, mu,
                    eps, tau);
    int st = abm_host::finish(stream, "abm_opinion_run/step");
    if (st) return st;
    float* tmp = cur;
    cur = nxt;
    nxt = tmp;
  }
  if (cur != o) {
    return abm_host::record_cuda_error(
        cudaMemcpyAsync(o, cur, bytes, cudaMemcpyDeviceToDevice, s), "abm_opinion_run/final");
  }
  return ABM_OK;
}

int abm_opinion_step(const float* o_in, float* o_out, const int32_t* row_ptr, const int32_t* col,
                     int64_t n, int32_t B, const float* mu, const float* eps, const float* tau,
                     void* stream) {
  if (!o_in || !o_out || o_in == o_out || !row_ptr || !col || !mu || !eps || !tau || n <= 0 ||
      n > 0x7FFFFFFFll || !valid_batch(B))
    return ABM_ERR_BADARG;
  if (!abm_host::aligned(o_in, 16) || !abm_host::aligned(o_out, 16) || !abm_host::aligned(mu, 16) ||
      !abm_host::aligned(eps, 16) || !abm_host::aligned(tau, 16))
    return ABM_ERR_BADARG;
  cudaStream_t s = abm_host::as_stream(stream);
  ABM_OP_DISPATCH(opinion_step_kernel, B / 4, step_blocks(n, B), 0, s, o_in, o_out, row_ptr, col,
                  (int)n, B, mu, eps, tau);
  return abm_host::finish(stream, "abm_opinion_step");
}

int abm_opinion_sigmoid(const float* z, float* s, int64_t n, void* stream) {
  if (!z || !s || n <= 0) return ABM_ERR_BADARG;
  long long blocks = (n + 255) / 256;
  const long long cap = (long long)abm_host::sm_count() * 16;
  if (blocks > cap) blocks = cap;
  opinion_sigmoid_kernel<<<(unsigned)blocks, 256, 0, abm_host::as_stream(stream)>>>(z, s, n);
  return abm_host::check_launch("abm_opinion_sigmoid");
}

int abm_opinion_inv_degree(const int32_t* row_ptr, int64_t n, float* inv_deg, void* stream) {
  if (!row_ptr || !inv_deg || n <= 0 || n > 0x7FFFFFFFll) return ABM_ERR_BADARG;
  inv_degree_kernel<<<(unsigned)((n + 255) / 256), 256, 0, abm_host::as_stream(stream)>>>(
      row_ptr, (int)n, inv_deg);
  return abm_host::check_launch("abm_opinion_inv_degree");
}

size_t abm_opinion_moments_workspace_bytes(int64_t n, int32_t B) {
  if (n <= 0 || !valid_batch(B)) return 0;
  const int64_t parts = (n + kMomRows - 1) / kMomRows;
  return (size_t)parts * B * 4 * sizeof(double);
}

int abm_opinion_moments(const float* o, int64_t n, int32_t B, double* moments, void* workspace,
                        size_t workspace_bytes, void* stream) {
  if (!o || !moments || n <= 0 || n > 0x7FFFFFFFll || !valid_batch(B)) return ABM_ERR_BADARG;
  if (!workspace || workspace_bytes < abm_opinion_moments_workspace_bytes(n, B) ||
      !abm_host::aligned(workspace, 8))
    return ABM_ERR_WORKSPACE;
  cudaStream_t s = abm_host::as_stream(stream);
  const int parts = (int)((n + kMomRows - 1) / kMomRows);
  double* part = static_cast<double*>(workspace);
  opinion_moments_partial_kernel<<<parts, (B + 31) / 32 * 32, 0, s>>>(o, (int)n, B, part);
  int st = abm_host::check_launch("abm_opinion_moments/partial");
  if (st) return st;
  sum_partials_kernel<<<(B * 4 + 127) / 128, 128, 0, s>>>(part, parts, B * 4, 1.0 / (double)n,
                                                          moments);
  return abm_host::check_launch("abm_opinion_moments/sum");
}

int abm_opinion_adjoint_init(const float* o, int64_t n, int32_t B, const double* dloss_dmoments,
                             float* lam, void* stream) {
  if (!o || !dloss_dmoments || !lam || n <= 0 || n > 0x7FFFFFFFll || !valid_batch(B))
    return ABM_ERR_BADARG;
  cudaStream_t s = abm_host::as_stream(stream);
  const long long total = n * (long long)B;
  long long blocks = (total + 255) / 256;
  const long long cap = (long long)abm_host::sm_count() * 16;
  if (blocks > cap) blocks = cap;
  opinion_adjoint_init_kernel<<<(unsigned)blocks, 256, 0, s>>>(o, (int)n, B, dloss_dmoments, lam);
  return abm_host::check_launch("abm_opinion_adjoint_init");
}

size_t abm_opinion_grad_workspace_bytes(int64_t n, int32_t B) {
  if (n <= 0 || !valid_batch(B)) return 0;
  return (size_t)step_blocks(n, adjoint_cols(B)) * B * 3 * sizeof(double);
}

int abm_opinion_adjoint_step(const float* o, const float* lam_in, float* lam_out,
                             const int32_t* row_ptr, const int32_t* col, const float* inv_deg,
                             int64_t n, int32_t B, const float* mu, const float* eps,
                             const float* tau, double* grad_partials, size_t grad_partials_bytes,
                             void* stream) {
  if (!o || !lam_in || !lam_out || !row_ptr || !col || !inv_deg || !mu || !eps || !tau || n <= 0 ||
      n > 0x7FFFFFFFll || !valid_batch(B) || lam_in == lam_out)
    return ABM_ERR_BADARG;
  if (!abm_host::aligned(o, 16) || !abm_host::aligned(lam_in, 16) ||
      !abm_host::aligned(lam_out, 16) || !abm_host::aligned(mu, 16) ||
      !abm_host::aligned(eps, 16) || !abm_host::aligned(tau, 16))
    return ABM_ERR_BADARG;
  if (!grad_partials || grad_partials_bytes < abm_opinion_grad_workspace_bytes(n, B) ||
      !abm_host::aligned(grad_partials, 8))
    return ABM_ERR_WORKSPACE;
  cudaStream_t s = abm_host::as_stream(stream);
  const int cols = adjoint_cols(B);
  const int lpn = cols / 4;
  const int blocks = step_blocks(n, cols);
  const size_t smem = (size_t)kOpThreads * 12 * sizeof(float);
  for (int c0 = 0; c0 < B; c0 += cols) {
    ABM_OP_DISPATCH(opinion_adjoint_kernel, lpn, blocks, smem, s, o, lam_in, lam_out, row_ptr,
                    col, inv_deg, (int)n, B, c0, mu, eps, tau, grad_partials);
    const int st = abm_host::finish(stream, "abm_opinion_adjoint_step");
    if (st) return st;
  }
  return ABM_OK;
}

int abm_opinion_grad_reduce(const double* grad_partials, int64_t n, int32_t B, double* grads,
                            void* stream) {
  if (!grad_partials || !grads || n <= 0 || !valid_batch(B)) return ABM_ERR_BADARG;
  cudaStream_t s = abm_host::as_stream(stream);
  const int parts = step_blocks(n, adjoint_cols(B));
  sum_partials_kernel<<<(B * 3 + 127) / 128, 128, 0, s>>>(grad_partials, parts, B * 3, 1.0, grads);
  return abm_host::check_launch("abm_opinion_grad_reduce");
}

}  // extern "C"
