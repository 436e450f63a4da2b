// Linear-Gaussian model pieces shared by the particle-filter kernels:
// the parameter block passed by value to kernels, the potential and
// transition (fma chains in a fixed order so that every value equals the
// oracle's), and the per-particle propagate + weight step.
#pragma once
#include "mgb_internal.cuh"
#include "mgb_resample.cuh"

namespace mgb {

template <int D, int DY>
struct LGP {
  float F[D * D], Lq[D * D], H[DY * D], P[DY * DY], C0[D * D], m0[D];
  float c;
  // structure of the matrices (detected on the host).  Skipping an exactly-zero
  // term of an fma chain leaves the rounded result unchanged (up to the sign of
  // a zero), so the specialised paths give the dense paths' values.
  int lq_diag, h_eye, p_diag;
  uint32_t one;  // == 1: multiplier of the cipher's multiply-adds (see threefry2x32_m)
};

template <int D, int DY>
__device__ __forceinline__ float lg_potential(const LGP<D, DY> &p, const float (&x)[D], const float *y) {
  float diff[DY];
  if (DY == D && p.h_eye) {
#pragma unroll
    for (int j = 0; j < DY; ++j) diff[j] = __fsub_rn(y[j], x[j < D ? j : 0]);
  } else {
#pragma unroll
    for (int j = 0; j < DY; ++j) {
      float hx = __fmul_rn(p.H[j * D], x[0]);
#pragma unroll
      for (int k = 1; k < D; ++k) hx = __fmaf_rn(p.H[j * D + k], x[k], hx);
      diff[j] = __fsub_rn(y[j], hx);
    }
  }
  float quad = 0.0f;
#pragma unroll
  for (int k = 0; k < DY; ++k) {
    float v;
    if (p.p_diag) {
      v = __fmul_rn(diff[k], p.P[k * DY + k]);
    } else {
      v = __fmul_rn(diff[0], p.P[k]);
#pragma unroll
      for (int j = 1; j < DY; ++j) v = __fmaf_rn(diff[j], p.P[j * DY + k], v);
    }
    quad = k == 0 ? __fmul_rn(v, v) : __fmaf_rn(v, v, quad);
  }
  return __fadd_rn(__fmul_rn(0.5f, quad), p.c);
}

// x_new = F x + Lq eps (fma chains in ascending column order)
// row r of the transition mean F x and of the noise Lq e
template <int D, int DY>
__device__ __forceinline__ float lg_mean_row(const LGP<D, DY> &p, const float (&xs)[D], int r) {
  float fx = __fmul_rn(p.F[r * D], xs[0]);
#pragma unroll
  for (int k = 1; k < D; ++k) fx = __fmaf_rn(p.F[r * D + k], xs[k], fx);
  return fx;
}
template <int D, int DY>
__device__ __forceinline__ float lg_noise_row(const LGP<D, DY> &p, const float (&e)[D], int r) {
  if (p.lq_diag) return __fmul_rn(p.Lq[r * D + r], e[r]);
  float le = __fmul_rn(p.Lq[r * D], e[0]);
#pragma unroll
  for (int k = 1; k < D; ++k) le = __fmaf_rn(p.Lq[r * D + k], e[k], le);
  return le;
}
template <int D, int DY>
__device__ __forceinline__ void lg_transition(const LGP<D, DY> &p, const float (&xs)[D], const float (&e)[D],
                                              float (&xn)[D]) {
#pragma unroll
  for (int r = 0; r < D; ++r) xn[r] = __fadd_rn(lg_mean_row<D, DY>(p, xs, r), lg_noise_row<D, DY>(p, e, r));
}

template <int D>
__device__ __forceinline__ void particle_normals(uint32_t k0, uint32_t k1, int64_t n, int64_t i, float (&e)[D]) {
  uint32_t a0, a1;
  split_at(k0, k1, (uint64_t)n, (uint64_t)i, a0, a1);
  uint32_t b[D];
  bits_vec<D>(a0, a1, b);
#pragma unroll
  for (int j = 0; j < D; ++j) e[j] = bits_to_normal(b[j]);
}

// load through L2 only (data written by other blocks of the same kernel) or
// through the read-only path (data fixed for the kernel's lifetime)
template <bool CG, class T>
__device__ __forceinline__ T ld(const T *p) {
  if (CG) return __ldcg(p);
  return __ldg(p);
}

// the arithmetic of lg_particle for a particle whose source state xs and
// log-weight lres are already in registers (callers that prefetch them)
template <int D, int DY>
__device__ __forceinline__ float lg_particle_regs(const LGP<D, DY> &p, int64_t n, uint32_t ka, uint32_t kb, int64_t i,
                                                  const float (&xs)[D], float lres, const float *y,
                                                  float *__restrict__ x_new, float *__restrict__ lw_new) {
  uint32_t b[D];
  bits_vec<D>(ka, kb, b, p.one);
  float e[D], xn[D];
#pragma unroll
  for (int j = 0; j < D; ++j) e[j] = bits_to_normal(b[j]);
  lg_transition<D, DY>(p, xs, e, xn);
#pragma unroll
  for (int r = 0; r < D; ++r) x_new[r * n + i] = xn[r];
  const float l = __fsub_rn(lres, lg_potential<D, DY>(p, xn, y));
  lw_new[i] = l;
  return l;
}

// MUS > 0: also writes the particle's proposal row for the score's backward
// kernel, mu[i * MUS ..] = (F x_src (the transition mean, the same float
// operations as the propagate), the carried log-weight, zero padding)
template <int D, int DY, bool CG = false, int MUS = 0>
__device__ __forceinline__ float lg_particle_e(const LGP<D, DY> &p, int64_t n, const float (&e)[D], int64_t i,
                                               bool res, const float *__restrict__ x_prev, const int32_t *anc,
                                               const float *lws, const float *y, float *__restrict__ x_new,
                                               float *__restrict__ lw_new, float *__restrict__ mu = nullptr) {
  float xs[D], xn[D];
  const int64_t src = res ? (int64_t)ld<CG>(&anc[i]) : i;
#pragma unroll
  for (int j = 0; j < D; ++j) xs[j] = ld<CG>(&x_prev[j * n + src]);
  const float lres = lws ? ld<CG>(&lws[i]) : 0.0f;
  if (MUS > 0) {
    static_assert(MUS == 0 || (MUS % 4 == 0 && MUS > D), "16-byte rows holding D means and the log-weight");
    float row[MUS > 0 ? MUS : 4];
#pragma unroll
    for (int r = 0; r < D; ++r) row[r] = lg_mean_row<D, DY>(p, xs, r);
    row[D] = lres;
#pragma unroll
    for (int r = D + 1; r < MUS; ++r) row[r] = 0.0f;
    float4 *o = reinterpret_cast<float4 *>(mu + i * MUS);
#pragma unroll
    for (int j = 0; j < MUS / 4; ++j) o[j] = make_float4(row[4 * j], row[4 * j + 1], row[4 * j + 2], row[4 * j + 3]);
#pragma unroll
    for (int r = 0; r < D; ++r) xn[r] = __fadd_rn(row[r], lg_noise_row<D, DY>(p, e, r));
  } else {
    lg_transition<D, DY>(p, xs, e, xn);
  }
#pragma unroll
  for (int r = 0; r < D; ++r) x_new[r * n + i] = xn[r];
  const float l = __fsub_rn(lres, lg_potential<D, DY>(p, xn, y));
  lw_new[i] = l;
  return l;
}
template <int D, int DY, bool CG = false, int MUS = 0>
__device__ __forceinline__ float lg_particle(const LGP<D, DY> &p, int64_t n, uint32_t ka, uint32_t kb, int64_t i,
                                             bool res, const float *__restrict__ x_prev, const int32_t *anc,
                                             const float *lws, const float *y, float *__restrict__ x_new,
                                             float *__restrict__ lw_new, float *__restrict__ mu = nullptr) {
  uint32_t b[D];
  bits_vec<D>(ka, kb, b, p.one);
  float e[D];
#pragma unroll
  for (int j = 0; j < D; ++j) e[j] = bits_to_normal(b[j]);
  return lg_particle_e<D, DY, CG, MUS>(p, n, e, i, res, x_prev, anc, lws, y, x_new, lw_new, mu);
}

// initial draw of one particle: x = C0 eps + m0, lw = -potential(x, y0)
template <int D, int DY>
__device__ __forceinline__ float lg_init_particle(const LGP<D, DY> &p, int64_t n, uint32_t ka, uint32_t kb, int64_t i,
                                                  const float *y, float *__restrict__ x, float *__restrict__ lw) {
  uint32_t b[D];
  bits_vec<D>(ka, kb, b, p.one);
  float e[D], xv[D];
#pragma unroll
  for (int j = 0; j < D; ++j) e[j] = bits_to_normal(b[j]);
#pragma unroll
  for (int r = 0; r < D; ++r) {
    float v = __fmul_rn(p.C0[r * D], e[0]);
#pragma unroll
    for (int k = 1; k < D; ++k) v = __fmaf_rn(p.C0[r * D + k], e[k], v);
    xv[r] = __fadd_rn(v, p.m0[r]);
    x[r * n + i] = xv[r];
  }
  const float l = -lg_potential<D, DY>(p, xv, y);
  lw[i] = l;
  return l;
}

template <int D, int DY>
inline LGP<D, DY> pack_lg(const mgb_lg_model *m) {
  LGP<D, DY> p;
  for (int i = 0; i < D * D; ++i) {
    p.F[i] = m->F[i];
    p.Lq[i] = m->Lq[i];
    p.C0[i] = m->C0[i];
  }
  for (int i = 0; i < DY * D; ++i) p.H[i] = m->H[i];
  for (int i = 0; i < DY * DY; ++i) p.P[i] = m->P[i];
  for (int i = 0; i < D; ++i) p.m0[i] = m->m0[i];
  p.c = m->c;
  auto diag = [](const float *a, int k) {
    for (int r = 0; r < k; ++r)
      for (int c = 0; c < k; ++c)
        if (r != c && a[r * k + c] != 0.0f) return 0;
    return 1;
  };
  p.one = 1u;
  p.lq_diag = diag(p.Lq, D);
  p.p_diag = diag(p.P, DY);
  p.h_eye = 0;
  if (DY == D) {
    int eye = 1;
    for (int r = 0; r < D; ++r)
      for (int c = 0; c < D; ++c) eye &= p.H[r * D + c] == (r == c ? 1.0f : 0.0f);
    p.h_eye = eye;
  }
  return p;
}

}  // namespace mgb
