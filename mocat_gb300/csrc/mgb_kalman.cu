// Kalman filter and Rauch-Tung-Striebel smoother for the time-homogeneous
// linear-Gaussian model, B independent observation sequences per launch (one
// CTA per sequence, the small matrices in shared memory, float32 as the
// reference computes).
//
// Reference: run_kalman_filter_for_marginals, run_kalman_smoother_for_marginals
// (mocat/src/ssm/linear_gaussian/kalman.py:16-57, 60-104):
//   t = 0   K = C0 H' (H C0 H' + R)^-1, mu = m0 + K (y_0 - H m0), P = C0 - K H C0, where C0 is the
//           initial covariance *square root*, which the reference uses as the covariance (:20)
//   t > 0   mu_p = F mu, P_p = F P F' + Q; the same update with P_p
//   smoother, t = T-2 .. 0: A = F P_t F' + Q, G = P_t F' A^-1,
//           mu_t^s = mu_t + G (mu_{t+1}^s - F mu_t), P_t^s = P_t + G (P_{t+1}^s - A) G'
//           and, optionally, the lag-one terms of run_kalman_smoother_for_marginals_and_lag_ones
//           (:60-94) as the reference forms them (1-D `@` products are dot products)
// Q = Lq Lq', R = LR LR' (transition / likelihood covariances).  Inverses by
// Gauss-Jordan elimination with partial pivoting.  Also (new) the
// prediction-error log-likelihood sum_t log N(y_t; H mu_p, S_t), S_t = H P_p H' + R.
// Matrix products are fma chains in ascending inner index.
#include "mgb_internal.cuh"

namespace mgb {

constexpr int KF_TPB = 128;

// The kernels take the dimensions as KFP::d / KFP::dy: for a compiled pair they are the
// template arguments (compile-time constants, loops fully known), for the run-time
// instance KFP<KF_DMAX, KF_DMAX, true> the values stored in the parameter block; array
// extents are the template arguments either way, and every product is the same
// sequence of operations.
constexpr int KF_DMAX = 32;
template <int D, int DY, bool RT = false>
struct KFP {
  float F[D * D], Q[D * D], H[DY * D], R[DY * DY], m0[D], C0[D * D];
  int rd, rdy;  // run-time dimensions (RT)
  __device__ __forceinline__ int d() const { return RT ? rd : D; }
  __device__ __forceinline__ int dy() const { return RT ? rdy : DY; }
};

// C[r][c] = sum_k A[r][k] B[k][c] (+ Add[r][c]); A (m x k), B (k x n) with row strides
__device__ __forceinline__ void mm(int M, int K, int N, const float *A, const float *B, const float *Add, float *C,
                                   bool transB = false) {
  for (int idx = threadIdx.x; idx < M * N; idx += KF_TPB) {
    const int r = idx / N, c = idx % N;
    float v = __fmul_rn(A[r * K], transB ? B[c * K] : B[c]);
    for (int k = 1; k < K; ++k) v = __fmaf_rn(A[r * K + k], transB ? B[c * K + k] : B[k * N + c], v);
    C[idx] = Add ? __fadd_rn(v, Add[idx]) : v;
  }
}

// inverse of the N x N matrix S into Si by Gauss-Jordan elimination with
// partial pivoting on the augmented [S | I] in W (N x 2N); log|det S| into *logdet
__device__ void gj_inverse(int N, const float *S, float *W, float *Si, float *col, int *piv_row, double *logdet) {
  for (int idx = threadIdx.x; idx < N * 2 * N; idx += KF_TPB) {
    const int r = idx / (2 * N), c = idx % (2 * N);
    W[idx] = c < N ? S[r * N + c] : (c - N == r ? 1.0f : 0.0f);
  }
  if (threadIdx.x == 0) *logdet = 0.0;
  __syncthreads();
  for (int c = 0; c < N; ++c) {
    if (threadIdx.x == 0) {
      int p = c;
      float best = fabsf(W[c * 2 * N + c]);
      for (int r = c + 1; r < N; ++r)
        if (fabsf(W[r * 2 * N + c]) > best) {
          best = fabsf(W[r * 2 * N + c]);
          p = r;
        }
      *piv_row = p;
    }
    __syncthreads();
    const int p = *piv_row;
    if (p != c)
      for (int j = threadIdx.x; j < 2 * N; j += KF_TPB) {
        const float a = W[c * 2 * N + j];
        W[c * 2 * N + j] = W[p * 2 * N + j];
        W[p * 2 * N + j] = a;
      }
    __syncthreads();
    const float pv = W[c * 2 * N + c];
    if (threadIdx.x == 0) *logdet += log(fabs((double)pv));
    for (int r = threadIdx.x; r < N; r += KF_TPB) col[r] = W[r * 2 * N + c];
    __syncthreads();
    for (int j = threadIdx.x; j < 2 * N; j += KF_TPB) W[c * 2 * N + j] = __fdiv_rn(W[c * 2 * N + j], pv);
    __syncthreads();
    for (int idx = threadIdx.x; idx < N * 2 * N; idx += KF_TPB) {
      const int r = idx / (2 * N), j = idx % (2 * N);
      if (r != c) W[idx] = __fsub_rn(W[idx], __fmul_rn(col[r], W[c * 2 * N + j]));
    }
    __syncthreads();
  }
  for (int idx = threadIdx.x; idx < N * N; idx += KF_TPB) Si[idx] = W[(idx / N) * 2 * N + N + idx % N];
  __syncthreads();
}

template <int CD, int CDY, bool RT>
__global__ void __launch_bounds__(KF_TPB) k_kalman_filter(const __grid_constant__ KFP<CD, CDY, RT> p, int64_t T,
                                                           const float *__restrict__ y, float *__restrict__ means,
                                                           float *__restrict__ covs, double *__restrict__ loglik) {
  constexpr int M = CD > CDY ? CD : CDY;
  __shared__ float mu[CD], mup[CD], P[CD * CD], Pp[CD * CD], T1[M * M], T2[M * M], S[CDY * CDY], Si[CDY * CDY],
      W[CDY * 2 * CDY], K[CD * CDY], e[CDY], col[CDY];
  const int D = p.d(), DY = p.dy();
  __shared__ int piv;
  __shared__ double logdet;
  const int64_t b = blockIdx.x;
  const float *yb = y + (size_t)b * T * DY;
  double ll = 0.0;
  for (int64_t t = 0; t < T; ++t) {
    // predicted moments: (m0, C0) at t = 0, else (F mu, F P F' + Q)
    if (t == 0) {
      for (int i = threadIdx.x; i < D; i += KF_TPB) mup[i] = p.m0[i];
      for (int i = threadIdx.x; i < D * D; i += KF_TPB) Pp[i] = p.C0[i];
    } else {
      mm(D, D, 1, p.F, mu, nullptr, mup);
      mm(D, D, D, p.F, P, nullptr, T1);
      __syncthreads();
      mm(D, D, D, T1, p.F, p.Q, Pp, true);  // (F P) F' + Q
    }
    __syncthreads();
    // S = H Pp H' + R, innovation e = y - H mup
    mm(DY, D, D, p.H, Pp, nullptr, T1);
    for (int r = threadIdx.x; r < DY; r += KF_TPB) {
      float hm = __fmul_rn(p.H[r * D], mup[0]);
      for (int k = 1; k < D; ++k) hm = __fmaf_rn(p.H[r * D + k], mup[k], hm);
      e[r] = __fsub_rn(yb[t * DY + r], hm);
    }
    __syncthreads();
    mm(DY, D, DY, T1, p.H, p.R, S, true);
    __syncthreads();
    gj_inverse(DY, S, W, Si, col, &piv, &logdet);
    // K = Pp H' S^-1
    mm(D, D, DY, Pp, p.H, nullptr, T2, true);
    __syncthreads();
    mm(D, DY, DY, T2, Si, nullptr, K);
    __syncthreads();
    // mu = mup + K e; P = Pp - K (H Pp)
    for (int r = threadIdx.x; r < D; r += KF_TPB) {
      float ke = __fmul_rn(K[r * DY], e[0]);
      for (int k = 1; k < DY; ++k) ke = __fmaf_rn(K[r * DY + k], e[k], ke);
      mu[r] = __fadd_rn(mup[r], ke);
    }
    mm(D, DY, D, K, T1, nullptr, T2);  // K (H Pp), T1 = H Pp still
    __syncthreads();
    for (int i = threadIdx.x; i < D * D; i += KF_TPB) P[i] = __fsub_rn(Pp[i], T2[i]);
    if (threadIdx.x == 0 && loglik) {
      double q = 0.0;
      for (int r = 0; r < DY; ++r) {
        double v = 0.0;
        for (int c = 0; c < DY; ++c) v += (double)Si[r * DY + c] * (double)e[c];
        q += (double)e[r] * v;
      }
      ll += -0.5 * (DY * 1.8378770664093453 + logdet + q);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < D; i += KF_TPB) means[((size_t)b * T + t) * D + i] = mu[i];
    for (int i = threadIdx.x; i < D * D; i += KF_TPB) covs[((size_t)b * T + t) * D * D + i] = P[i];
    __syncthreads();
  }
  if (threadIdx.x == 0 && loglik) loglik[b] = ll;
}

template <int CD, int CDY, bool RT>
__global__ void __launch_bounds__(KF_TPB) k_kalman_smoother(const __grid_constant__ KFP<CD, CDY, RT> p, int64_t T,
                                                             const float *__restrict__ fmeans,
                                                             const float *__restrict__ fcovs,
                                                             float *__restrict__ smeans, float *__restrict__ scovs,
                                                             float *__restrict__ lag) {
  __shared__ float mus[CD], Ps[CD * CD], Pf[CD * CD], A[CD * CD], Ai[CD * CD], W[CD * 2 * CD], G[CD * CD],
      T1[CD * CD], T2[CD * CD], L[CD * CD], fm[CD], fmn[CD], dm[CD], col[CD];
  const int D = p.d();
  __shared__ int piv;
  __shared__ double logdet;
  const int64_t b = blockIdx.x;
  const size_t mo = (size_t)b * T * D, co = (size_t)b * T * D * D;
  for (int i = threadIdx.x; i < D; i += KF_TPB) {
    mus[i] = fmeans[mo + (T - 1) * D + i];
    fmn[i] = mus[i];
    smeans[mo + (T - 1) * D + i] = mus[i];
  }
  for (int i = threadIdx.x; i < D * D; i += KF_TPB) {
    Ps[i] = fcovs[co + (T - 1) * D * D + i];
    scovs[co + (T - 1) * D * D + i] = Ps[i];
  }
  __syncthreads();
  for (int64_t t = T - 2; t >= 0; --t) {
    for (int i = threadIdx.x; i < D; i += KF_TPB) fm[i] = fmeans[mo + t * D + i];
    for (int i = threadIdx.x; i < D * D; i += KF_TPB) Pf[i] = fcovs[co + t * D * D + i];
    __syncthreads();
    mm(D, D, D, p.F, Pf, nullptr, T1);  // F Pf
    __syncthreads();
    mm(D, D, D, T1, p.F, p.Q, A, true);  // F Pf F' + Q
    __syncthreads();
    gj_inverse(D, A, W, Ai, col, &piv, &logdet);
    mm(D, D, D, Pf, p.F, nullptr, T1, true);  // Pf F'
    __syncthreads();
    mm(D, D, D, T1, Ai, nullptr, G);  // G = Pf F' A^-1
    // dm = mu_{t+1}^s - F mu_t
    for (int r = threadIdx.x; r < D; r += KF_TPB) {
      float fx = __fmul_rn(p.F[r * D], fm[0]);
      for (int k = 1; k < D; ++k) fx = __fmaf_rn(p.F[r * D + k], fm[k], fx);
      dm[r] = __fsub_rn(mus[r], fx);
    }
    for (int i = threadIdx.x; i < D * D; i += KF_TPB) T2[i] = __fsub_rn(Ps[i], A[i]);  // P_{t+1}^s - A
    // lag-one term (kalman.py:83): the reference's 1-D `@` products are dot products, so
    // E = <mu_t^f, mu_{t+1}^s> + G (P_{t+1}^s + <mu_{t+1}^s - mu_{t+1}^f, mu_{t+1}^s>)
    float dot_a = 0.f, dot_c = 0.f;
    if (lag) {
      dot_a = __fmul_rn(fm[0], mus[0]);
      dot_c = __fmul_rn(__fsub_rn(mus[0], fmn[0]), mus[0]);
      for (int k = 1; k < D; ++k) {
        dot_a = __fmaf_rn(fm[k], mus[k], dot_a);
        dot_c = __fmaf_rn(__fsub_rn(mus[k], fmn[k]), mus[k], dot_c);
      }
    }
    __syncthreads();
    if (lag)
      for (int i = threadIdx.x; i < D * D; i += KF_TPB) L[i] = __fadd_rn(Ps[i], dot_c);
    for (int r = threadIdx.x; r < D; r += KF_TPB) {
      float g = __fmul_rn(G[r * D], dm[0]);
      for (int k = 1; k < D; ++k) g = __fmaf_rn(G[r * D + k], dm[k], g);
      mus[r] = __fadd_rn(fm[r], g);
    }
    mm(D, D, D, G, T2, nullptr, T1);  // G (P^s - A)
    __syncthreads();
    mm(D, D, D, T1, G, Pf, Ps, true);  // ... G' + Pf
    if (lag) {
      float *lo = lag + ((size_t)b * (T - 1) + t) * D * D;
      for (int i = threadIdx.x; i < D * D; i += KF_TPB) {
        const int r = i / D, c = i % D;
        float v = __fmul_rn(G[r * D], L[c]);
        for (int k = 1; k < D; ++k) v = __fmaf_rn(G[r * D + k], L[k * D + c], v);
        lo[i] = __fadd_rn(v, dot_a);
      }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < D; i += KF_TPB) {
      smeans[mo + t * D + i] = mus[i];
      fmn[i] = fm[i];
    }
    for (int i = threadIdx.x; i < D * D; i += KF_TPB) scovs[co + t * D * D + i] = Ps[i];
    __syncthreads();
  }
}

// matrices packed with row strides d (run-time instance: the first d * d entries)
template <int D, int DY, bool RT>
static KFP<D, DY, RT> pack_kf(const mgb_kalman_model *m) {
  KFP<D, DY, RT> p;
  const int d = RT ? m->d : D, dy = RT ? m->dy : DY;
  for (int i = 0; i < d * d; ++i) {
    p.F[i] = m->F[i];
    p.Q[i] = m->Q[i];
    p.C0[i] = m->C0[i];
  }
  for (int i = 0; i < dy * d; ++i) p.H[i] = m->H[i];
  for (int i = 0; i < dy * dy; ++i) p.R[i] = m->R[i];
  for (int i = 0; i < d; ++i) p.m0[i] = m->m0[i];
  p.rd = d;
  p.rdy = dy;
  return p;
}

template <int D, int DY, bool RT = false>
static int kf_run(const mgb_kalman_model *m, int64_t B, int64_t T, const float *y, float *means, float *covs,
                  double *loglik, cudaStream_t s) {
  k_kalman_filter<D, DY, RT><<<(unsigned)B, KF_TPB, 0, s>>>(pack_kf<D, DY, RT>(m), T, y, means, covs, loglik);
  return launch_status();
}

template <int D, int DY, bool RT = false>
static int ks_run(const mgb_kalman_model *m, int64_t B, int64_t T, const float *fm, const float *fc, float *sm,
                  float *sc, float *lag, cudaStream_t s) {
  k_kalman_smoother<D, DY, RT><<<(unsigned)B, KF_TPB, 0, s>>>(pack_kf<D, DY, RT>(m), T, fm, fc, sm, sc,
                                                               T > 1 ? lag : nullptr);
  return launch_status();
}

#define MGB_KF_DISPATCH(FN, ...)                               \
  do {                                                         \
    const int d_ = m->d, dy_ = m->dy;                          \
    if (dy_ == 1) {                                            \
      switch (d_) {                                            \
        case 1: return FN<1, 1>(__VA_ARGS__);                  \
        case 2: return FN<2, 1>(__VA_ARGS__);                  \
        case 3: return FN<3, 1>(__VA_ARGS__);                  \
        case 4: return FN<4, 1>(__VA_ARGS__);                  \
        case 5: return FN<5, 1>(__VA_ARGS__);                  \
        case 8: return FN<8, 1>(__VA_ARGS__);                  \
        case 10: return FN<10, 1>(__VA_ARGS__);                \
        default: break;                                        \
      }                                                        \
    } else if (dy_ == d_) {                                    \
      switch (d_) {                                            \
        case 2: return FN<2, 2>(__VA_ARGS__);                  \
        case 3: return FN<3, 3>(__VA_ARGS__);                  \
        case 4: return FN<4, 4>(__VA_ARGS__);                  \
        case 5: return FN<5, 5>(__VA_ARGS__);                  \
        case 8: return FN<8, 8>(__VA_ARGS__);                  \
        case 10: return FN<10, 10>(__VA_ARGS__);               \
        default: break;                                        \
      }                                                        \
    }                                                          \
    /* no compiled pair: the run-time instance, d, dy <= KF_DMAX */  \
    if (d_ <= KF_DMAX && dy_ <= KF_DMAX) return FN<KF_DMAX, KF_DMAX, true>(__VA_ARGS__); \
    return ERR_UNSUPPORTED;                                    \
  } while (0)

static bool kf_ok(const mgb_kalman_model *m, int64_t B, int64_t T) {
  return m && m->F && m->Q && m->H && m->R && m->m0 && m->C0 && B >= 1 && B <= 0x7FFFFFFF && T >= 1;
}

}  // namespace mgb

using namespace mgb;

extern "C" {

int mgb_kalman_filter(const mgb_kalman_model *m, int64_t B, int64_t T, const float *y, float *means, float *covs,
                      double *loglik, void *stream) {
  if (!kf_ok(m, B, T) || !y || !means || !covs) return ERR_BAD_ARG;
  MGB_KF_DISPATCH(kf_run, m, B, T, y, means, covs, loglik, (cudaStream_t)stream);
}

int mgb_kalman_smoother(const mgb_kalman_model *m, int64_t B, int64_t T, const float *filter_means,
                        const float *filter_covs, float *means, float *covs, float *lag_ones, void *stream) {
  if (!kf_ok(m, B, T) || !filter_means || !filter_covs || !means || !covs) return ERR_BAD_ARG;
  MGB_KF_DISPATCH(ks_run, m, B, T, filter_means, filter_covs, means, covs, lag_ones, (cudaStream_t)stream);
}

}  // extern "C"
