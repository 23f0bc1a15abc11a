/*
 * CPU oracle of the bounded-confidence opinion model and its gradient
 * (TEST INFRASTRUCTURE ONLY; the checker).
 *
 * Parity status: UNPINNED against the reference -- the reference has no opinion model and
 * no golden trajectories; it would compute this gradient with jax.grad through its run
 * loop (jaxabm/analysis.py:494-522).  The FP64 adjoint below is that gradient in exact
 * (float64) arithmetic; the tests also check it against central finite differences.
 *
 * Model, per step, for node i and instance b (o[N][B] interleaved):
 *   o_i += mu * (sum_j sigmoid((eps - |o_j - o_i|) / tau) (o_j - o_i)) / deg_i
 * Loss per instance: 0.25 * sum_{k=1..4} (m_k - target_k)^2, m_k = mean_i o_i^k.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int orc_opinion_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* float32 exponential by Tang's table-driven method (P. T. P. Tang, ACM TOMS 15(2), 1989),
 * every operation a single float32 operation rounded to nearest (built with
 * -ffp-contract=off, so only the fmaf calls written out are fused):
 *   x clamped to [-87, 88]; N = rint(x * 32/ln2); r = fma(-N, L2, fma(-N, L1, x)) with
 *   L1 + L2 = ln2/32 (L1 of 11 significant bits: x - N L1 is exact);
 *   p = fma(r^2, fma(r, 1/6, 1/2), r)  (Taylor; |r| <= ln2/64);
 *   exp(x) = 2^(N >> 5) fma(T[N & 31], p, T[N & 31]),  T[j] = 2^(j/32) rounded to float32;
 * the scaling by 2^(N >> 5) adds to the exponent field (exact: the result stays normal). */
static const float orc_exp2_tab[32] = {
    0x1.000000p+0f, 0x1.059b0ep+0f, 0x1.0b5586p+0f, 0x1.11301ep+0f, 0x1.172b84p+0f,
    0x1.1d4874p+0f, 0x1.2387a6p+0f, 0x1.29e9e0p+0f, 0x1.306fe0p+0f, 0x1.371a74p+0f,
    0x1.3dea64p+0f, 0x1.44e086p+0f, 0x1.4bfdaep+0f, 0x1.5342b6p+0f, 0x1.5ab07ep+0f,
    0x1.6247ecp+0f, 0x1.6a09e6p+0f, 0x1.71f75ep+0f, 0x1.7a1148p+0f, 0x1.82589ap+0f,
    0x1.8ace54p+0f, 0x1.93737cp+0f, 0x1.9c4918p+0f, 0x1.a5503cp+0f, 0x1.ae89fap+0f,
    0x1.b7f770p+0f, 0x1.c199bep+0f, 0x1.cb720ep+0f, 0x1.d5818ep+0f, 0x1.dfc974p+0f,
    0x1.ea4afap+0f, 0x1.f50766p+0f};

static float orc_expf_tang(float x) {
  x = fminf(fmaxf(x, -87.0f), 88.0f);
  const float nf = rintf(x * 0x1.715476p+5f);
  const int32_t N = (int32_t)nf;
  const float r = fmaf(-nf, 0x1.217f7ep-17f, fmaf(-nf, 0x1.62c000p-6f, x));
  const float p = fmaf(r * r, fmaf(r, 0x1.555556p-3f, 0.5f), r);
  const float t = orc_exp2_tab[N & 31];
  const float e = fmaf(t, p, t);
  uint32_t bits;
  memcpy(&bits, &e, 4);
  bits += (uint32_t)(N >> 5) << 23;
  float out;
  memcpy(&out, &bits, 4);
  return out;
}

static float orc_sigmoid32(float z) { return 1.0f / (1.0f + orc_expf_tang(-z)); }

/* The exponential and the sigmoid over arrays, and the table (CPU checks). */
void orc_expf_tang_array(const float* x, float* y, int64_t n) {
  for (int64_t i = 0; i < n; ++i) y[i] = orc_expf_tang(x[i]);
}

void orc_sigmoid32_array(const float* z, float* s, int64_t n) {
  for (int64_t i = 0; i < n; ++i) s[i] = orc_sigmoid32(z[i]);
}

void orc_exp2_table(float* out) { memcpy(out, orc_exp2_tab, sizeof(orc_exp2_tab)); }

/* float32 forward: the fixed operation sequence of the model (see orc_expf_tang), per step
 * and node i, instance b: d = o_j - o_i; z = (eps - |d|) * (1/tau); s = 1 / (1 + exp(-z));
 * acc = fma(s, d, acc) over the CSR row in order; o_i' = fma(mu, acc / deg_i, o_i). */
void orc_opinion_run_f32(float* o, const int32_t* rp, const int32_t* col, int64_t n, int32_t B,
                         const float* mu, const float* eps, const float* tau, int32_t steps) {
  float* nxt = (float*)malloc(sizeof(float) * (size_t)n * B);
  float* itau = (float*)malloc(sizeof(float) * (size_t)B);
  for (int b = 0; b < B; ++b) itau[b] = 1.0f / tau[b];
  float* cur = o;
  for (int32_t t = 0; t < steps; ++t) {
#pragma omp parallel
    {
      float* acc = (float*)malloc(sizeof(float) * (size_t)B);
#pragma omp for schedule(static)
      for (int64_t i = 0; i < n; ++i) {
        const int32_t r0 = rp[i], r1 = rp[i + 1];
        const float* oi = cur + i * B;
        for (int b = 0; b < B; ++b) acc[b] = 0.0f;
        /* every instance accumulates its own sum in CSR order */
        for (int32_t e = r0; e < r1; ++e) {
          const float* oj = cur + (int64_t)col[e] * B;
          for (int b = 0; b < B; ++b) {
            const float d = oj[b] - oi[b];
            acc[b] = fmaf(orc_sigmoid32((eps[b] - fabsf(d)) * itau[b]), d, acc[b]);
          }
        }
        for (int b = 0; b < B; ++b)
          nxt[i * B + b] = (r1 > r0) ? fmaf(mu[b], acc[b] / (float)(r1 - r0), oi[b]) : oi[b];
      }
      free(acc);
    }
    float* tmp = cur;
    cur = nxt;
    nxt = tmp;
  }
  if (cur != o) {
    memcpy(o, cur, sizeof(float) * (size_t)n * B);
    free(cur);
  } else {
    free(nxt);
  }
  free(itau);
}

static void step_f64(const double* cur, double* nxt, const int32_t* rp, const int32_t* col,
                     int64_t n, int32_t B, const double* mu, const double* eps,
                     const double* tau) {
#pragma omp parallel
  {
    double* acc = (double*)malloc(sizeof(double) * (size_t)B);
#pragma omp for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
      const int32_t r0 = rp[i], r1 = rp[i + 1];
      const double* oi = cur + i * B;
      for (int b = 0; b < B; ++b) acc[b] = 0.0;
      for (int32_t e = r0; e < r1; ++e) {
        const double* oj = cur + (int64_t)col[e] * B;
        for (int b = 0; b < B; ++b) {
          const double d = oj[b] - oi[b];
          acc[b] += d / (1.0 + exp(-(eps[b] - fabs(d)) / tau[b]));
        }
      }
      for (int b = 0; b < B; ++b)
        nxt[i * B + b] = (r1 > r0) ? oi[b] + mu[b] * acc[b] / (double)(r1 - r0) : oi[b];
    }
    free(acc);
  }
}

void orc_opinion_run_f64(double* o, const int32_t* rp, const int32_t* col, int64_t n, int32_t B,
                         const double* mu, const double* eps, const double* tau, int32_t steps) {
  double* nxt = (double*)malloc(sizeof(double) * (size_t)n * B);
  double* cur = o;
  for (int32_t t = 0; t < steps; ++t) {
    step_f64(cur, nxt, rp, col, n, B, mu, eps, tau);
    double* tmp = cur;
    cur = nxt;
    nxt = tmp;
  }
  if (cur != o) {
    memcpy(o, cur, sizeof(double) * (size_t)n * B);
    free(cur);
  } else {
    free(nxt);
  }
}

void orc_opinion_moments_f64(const double* o, int64_t n, int32_t B, double* m) {
  for (int b = 0; b < B; ++b) {
    double a1 = 0, a2 = 0, a3 = 0, a4 = 0;
    for (int64_t i = 0; i < n; ++i) {
      const double x = o[i * B + b];
      a1 += x;
      a2 += x * x;
      a3 += x * x * x;
      a4 += x * x * x * x;
    }
    m[4 * b] = a1 / n;
    m[4 * b + 1] = a2 / n;
    m[4 * b + 2] = a3 / n;
    m[4 * b + 3] = a4 / n;
  }
}

/* Loss and its gradient w.r.t. (mu, eps, tau) per instance by the float64 reverse sweep
 * over a stored trajectory traj[(steps+1)][n][B] (float64; owned and freed here). */
static void reverse_sweep_f64(double* traj, const int32_t* rp, const int32_t* col, int64_t n,
                              int32_t B, const double* mu, const double* eps, const double* tau,
                              int32_t steps, const double* target, double* loss, double* grads) {
  const size_t sz = (size_t)n * B;
  const double* oT = traj + (size_t)steps * sz;
  double* m = (double*)malloc(sizeof(double) * 4 * (size_t)B);
  orc_opinion_moments_f64(oT, n, B, m);
  double* lam = (double*)malloc(sizeof(double) * sz);
  double* lam2 = (double*)malloc(sizeof(double) * sz);
  for (int b = 0; b < B; ++b) {
    double L = 0;
    for (int k = 0; k < 4; ++k) L += 0.25 * (m[4 * b + k] - target[k]) * (m[4 * b + k] - target[k]);
    loss[b] = L;
    grads[3 * b] = grads[3 * b + 1] = grads[3 * b + 2] = 0.0;
  }
  for (int64_t i = 0; i < n; ++i)
    for (int b = 0; b < B; ++b) {
      const double x = oT[i * B + b];
      double w[4];
      for (int k = 0; k < 4; ++k) w[k] = 0.5 * (m[4 * b + k] - target[k]);
      lam[i * B + b] = (w[0] + 2 * w[1] * x + 3 * w[2] * x * x + 4 * w[3] * x * x * x) / n;
    }
  /* per-thread partial parameter gradients, summed in thread order after the sweep */
  const int nthreads = orc_opinion_threads();
  double* part = (double*)calloc((size_t)nthreads * 3 * B, sizeof(double));
  for (int32_t t = steps - 1; t >= 0; --t) {
    const double* o = traj + (size_t)t * sz;
#pragma omp parallel num_threads(nthreads)
    {
#ifdef _OPENMP
      double* gp_part = part + (size_t)omp_get_thread_num() * 3 * B;
#else
      double* gp_part = part;
#endif
#pragma omp for schedule(static)
      for (int64_t i = 0; i < n; ++i) {
        const int32_t r0 = rp[i], r1 = rp[i + 1];
        const double di = (double)(r1 - r0);
        for (int b = 0; b < B; ++b) {
          const double oi = o[i * B + b], li = lam[i * B + b];
          double sl = 0, sg = 0, se = 0, st = 0;
          for (int32_t e = r0; e < r1; ++e) {
            const int32_t j = col[e];
            const double d = o[(int64_t)j * B + b] - oi, a = fabs(d);
            const double z = (eps[b] - a) / tau[b];
            const double s = 1.0 / (1.0 + exp(-z)), sp = s * (1 - s);
            const double gp = s - a * sp / tau[b];
            const double dj = (double)(rp[j + 1] - rp[j]);
            sl += gp * (lam[(int64_t)j * B + b] / dj - li / di);
            sg += s * d;
            se += sp / tau[b] * d;
            st += -sp * z / tau[b] * d;
          }
          lam2[i * B + b] = li + mu[b] * sl;
          if (r1 > r0) {
            gp_part[3 * b] += li * sg / di;
            gp_part[3 * b + 1] += li * mu[b] * se / di;
            gp_part[3 * b + 2] += li * mu[b] * st / di;
          }
        }
      }
    }
    double* tmp = lam;
    lam = lam2;
    lam2 = tmp;
  }
  for (int th = 0; th < nthreads; ++th)
    for (int q = 0; q < 3 * B; ++q) grads[q] += part[(size_t)th * 3 * B + q];
  free(part);
  free(traj);
  free(m);
  free(lam);
  free(lam2);
}

/* Loss and gradient along the float64 trajectory from o0.  target: float64[4] (shared);
 * loss float64[B]; grads [B][3]. */
void orc_opinion_grad_f64(const double* o0, const int32_t* rp, const int32_t* col, int64_t n,
                          int32_t B, const double* mu, const double* eps, const double* tau,
                          int32_t steps, const double* target, double* loss, double* grads) {
  const size_t sz = (size_t)n * B;
  double* traj = (double*)malloc(sizeof(double) * sz * (size_t)(steps + 1));
  memcpy(traj, o0, sizeof(double) * sz);
  for (int32_t t = 0; t < steps; ++t)
    step_f64(traj + (size_t)t * sz, traj + (size_t)(t + 1) * sz, rp, col, n, B, mu, eps, tau);
  reverse_sweep_f64(traj, rp, col, n, B, mu, eps, tau, steps, target, loss, grads);
}

/* The same float64 reverse sweep along the float32 trajectory from o0 (the states the
 * float32 forward visits, which is what a float32 adjoint differentiates): the float32
 * states are computed by the float32 forward, widened to float64, and the sweep runs in
 * float64 over them. */
void orc_opinion_grad_f64_along_f32(const float* o0, const int32_t* rp, const int32_t* col,
                                    int64_t n, int32_t B, const float* mu, const float* eps,
                                    const float* tau, int32_t steps, const double* target,
                                    double* loss, double* grads) {
  const size_t sz = (size_t)n * B;
  double* traj = (double*)malloc(sizeof(double) * sz * (size_t)(steps + 1));
  float* cur = (float*)malloc(sizeof(float) * sz);
  memcpy(cur, o0, sizeof(float) * sz);
  double* mu64 = (double*)malloc(sizeof(double) * 3 * (size_t)B);
  double* eps64 = mu64 + B;
  double* tau64 = eps64 + B;
  for (int b = 0; b < B; ++b) {
    mu64[b] = mu[b];
    eps64[b] = eps[b];
    tau64[b] = tau[b];
  }
  for (int32_t t = 0; t <= steps; ++t) {
    for (size_t q = 0; q < sz; ++q) traj[(size_t)t * sz + q] = cur[q];
    if (t < steps) orc_opinion_run_f32(cur, rp, col, n, B, mu, eps, tau, 1);
  }
  free(cur);
  reverse_sweep_f64(traj, rp, col, n, B, mu64, eps64, tau64, steps, target, loss, grads);
  free(mu64);
}
