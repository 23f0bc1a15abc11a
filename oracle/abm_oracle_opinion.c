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

/* float32 forward with the GPU kernel's operation order (fmaf accumulation, multiply by
 * float32(1/tau)); differs from the GPU only by the last bits of expf. */
void orc_opinion_run_f32(float* o, const int32_t* rp, const int32_t* col, int64_t n, int32_t B,
                         const float* mu, const float* eps, const float* tau, int32_t steps) {
  float* nxt = (float*)malloc(sizeof(float) * (size_t)n * B);
  float* itau = (float*)malloc(sizeof(float) * (size_t)B);
  for (int b = 0; b < B; ++b) itau[b] = 1.0f / tau[b];
  float* cur = o;
  for (int32_t t = 0; t < steps; ++t) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
      const int32_t r0 = rp[i], r1 = rp[i + 1];
      for (int b = 0; b < B; ++b) {
        const float oi = cur[i * B + b];
        float acc = 0.0f;
        for (int32_t e = r0; e < r1; ++e) {
          const float d = cur[(int64_t)col[e] * B + b] - oi;
          const float z = (eps[b] - fabsf(d)) * itau[b];
          const float s = 1.0f / (1.0f + expf(-z));
          acc = fmaf(s, d, acc);
        }
        nxt[i * B + b] = (r1 > r0) ? fmaf(mu[b], acc / (float)(r1 - r0), oi) : oi;
      }
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
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    const int32_t r0 = rp[i], r1 = rp[i + 1];
    for (int b = 0; b < B; ++b) {
      const double oi = cur[i * B + b];
      double acc = 0.0;
      for (int32_t e = r0; e < r1; ++e) {
        const double d = cur[(int64_t)col[e] * B + b] - oi;
        const double s = 1.0 / (1.0 + exp(-(eps[b] - fabs(d)) / tau[b]));
        acc += s * d;
      }
      nxt[i * B + b] = (r1 > r0) ? oi + mu[b] * acc / (double)(r1 - r0) : oi;
    }
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

/* Loss and its gradient w.r.t. (mu, eps, tau) per instance by the reverse sweep over the
 * stored float64 trajectory.  target: float64[4] (shared) ; loss float64[B]; grads [B][3]. */
void orc_opinion_grad_f64(const double* o0, const int32_t* rp, const int32_t* col, int64_t n,
                          int32_t B, const double* mu, const double* eps, const double* tau,
                          int32_t steps, const double* target, double* loss, double* grads) {
  const size_t sz = (size_t)n * B;
  double* traj = (double*)malloc(sizeof(double) * sz * (size_t)(steps + 1));
  memcpy(traj, o0, sizeof(double) * sz);
  for (int32_t t = 0; t < steps; ++t)
    step_f64(traj + (size_t)t * sz, traj + (size_t)(t + 1) * sz, rp, col, n, B, mu, eps, tau);
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
  for (int32_t t = steps - 1; t >= 0; --t) {
    const double* o = traj + (size_t)t * sz;
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
          grads[3 * b] += li * sg / di;
          grads[3 * b + 1] += li * mu[b] * se / di;
          grads[3 * b + 2] += li * mu[b] * st / di;
        }
      }
    }
    double* tmp = lam;
    lam = lam2;
    lam2 = tmp;
  }
  free(traj);
  free(m);
  free(lam);
  free(lam2);
}
