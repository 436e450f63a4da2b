// Many independent stochastic-volatility particle filters of uneven length
// and size in one persistent launch.
//
// Reference path: run_particle_filter_for_marginals
// (mocat/src/ssm/filtering.py:255-324) with BootstrapFilter on
// StochasticVolatility (mocat/src/ssm/scenarios/stochastic_volatility.py:71-108),
// d = 1; mocat runs one series per call.
//
// Work unit: a bundle = up to 16 filters whose particle counts round up to the
// same power-of-two slot size s, with similar T.  A CTA of TPB threads takes
// bundles from a queue (longest first); filter g of the bundle runs on its own
// group of G = max(32, s / ppt) threads, synchronised by named barrier g + 1
// (or __syncwarp when G = 32), for all of its steps.  Per filter, in shared
// memory:
//   C  u64[s]      exact fixed-point weight prefixes; after the ancestor
//                  search, the gathered particles (float)
//   S  u64[s + 2]  multinomial: prefix sums of the n + 1 quantised exponential
//                  spacings (sorted-uniform numerators)
//   X  f32[s]      particles
//   L  f32[s]      log-weights; the ancestors (int32) during a resample
// Per step: propagate pairs (i, i + n/2), which share their key-split cipher
// calls; weight; group logsumexp / ESS with per-warp partials combined by
// every thread (one barrier per non-resampling step); log Z in float64 by the
// group's first thread.  When ESS < threshold n the group resamples before
// propagating: quantise + warp-chunked scan -> C, exponentials + scan -> S,
// merge path of C against S (or the systematic thresholds), gather.
// HBM traffic is the observations (4 bytes per filter-step) and one float64
// per filter.
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <tuple>
#include <vector>

#include "mgb_internal.cuh"
#include "mgb_resample.cuh"
#include "mgb_group.cuh"
#include "mgb_sv.cuh"

namespace mgb {

constexpr int SVB_MAX_GROUPS = 16;
constexpr int SVB_MIN_SLOT = 64;
constexpr size_t SVB_MAX_SMEM = 227 * 1024;

struct SVBatch {
  const int32_t *n, *T;
  const int64_t *y_off;
  const float *y;
  const uint32_t *keys;
  const int32_t *order;
  const int4 *bundles;
  int32_t nbundles, ppt, t_cap;
  float thr;
  double *logz;
  int32_t *nres;
  int *counter;
};

__host__ __device__ inline size_t sv_slot_bytes(int s) { return (size_t)s * 24 + 16; }

// One filter on one thread group (tg = thread in group, wg = warp in group,
// wcta = warp in CTA, bar = named barrier id, gi = group index).
template <int SCHEME>
__device__ __forceinline__ void sv_filter(const SVParams &p, const SVBatch &a, int b, unsigned char *region, int G,
                                          int W, int tg, int wg, int lane, int wcta, int bar, int gi,
                                          float (*red)[4][32], uint32_t (*key_s)[2][2],
                                          unsigned long long *wtot) {
  const int n = a.n[b];
  const int Tfull = a.T[b];
  const int T = a.t_cap > 0 ? min(Tfull, a.t_cap) : Tfull;
  const int s = n + (n & 1);  // array stride
  uint64_t *C = (uint64_t *)region;
  uint64_t *S = C + s;
  float *X = (float *)(S + s + 2);
  float *L = X + s;
  int32_t *A = (int32_t *)L;
  float *XR = (float *)C;
  const float *y = a.y + a.y_off[b];

  // split(key, 2): [0] drives the steps, [1] the initial draw (filtering.py:267-278)
  uint32_t rk0, rk1, sk0, sk1;
  {
    const uint32_t fk0 = a.keys[2 * b], fk1 = a.keys[2 * b + 1];
    split_at(fk0, fk1, 2, 0, rk0, rk1);
    split_at(fk0, fk1, 2, 1, sk0, sk1);
  }
  const float thr_n = __fmul_rn(a.thr, (float)n);
  const float wscale = __int_as_float((weight_shift(n) + 127) << 23);
  const float escale = __int_as_float((exp_shift(n) + 127) << 23);
  const uint64_t magic = SCHEME == MGB_RESAMPLE_SYSTEMATIC ? ~0ull / (uint64_t)n : 0ull;
  const int h = n >> 1;
  const bool paired = (n & 1) == 0;
  double logn = 0.0;
  if (tg == 0) logn = log((double)n);

  double logz = 0.0, lse_prev = 0.0;
  int nres = 0, res = 0;
  float M = 0.0f;
  float yv = __ldg(&y[0]);
  for (int t = 0; t < T; ++t) {
    // next step's key split(rk, Tfull - 1)[t]; read after this step's barrier
    if (tg == G - 1 && t + 1 < T) {
      uint32_t q0, q1;
      split_at(rk0, rk1, (uint64_t)(Tfull - 1), (uint64_t)t, q0, q1);
      key_s[gi][(t + 1) & 1][0] = q0;
      key_s[gi][(t + 1) & 1][1] = q1;
    }
    const uint32_t k0 = t == 0 ? sk0 : key_s[gi][t & 1][0];
    const uint32_t k1 = t == 0 ? sk1 : key_s[gi][t & 1][1];
    const float y_next = t + 1 < T ? __ldg(&y[t + 1]) : 0.0f;

    // ---- resample (only ever with finite weights: NaN / inf give a NaN ESS)
    if (res) {
      ++nres;
      const uint64_t Q = group_scan(C, n, W, wg, lane, wcta, wtot, bar, G,
                                    [&](int j) { return quantise_weight(L[j], M, wscale); });
      if (SCHEME == MGB_RESAMPLE_MULTINOMIAL) {
        // S_j = trunc(E_j 2^SE), E = exponential(k_t, (n + 1,)) in jax's counter layout
        const int N1 = n + 1, hN = (N1 + 1) >> 1;
        for (int q = tg; q < hN; q += G) {
          uint32_t r0, r1;
          threefry2x32_m(k0, k1, (uint32_t)q, q + hN < N1 ? (uint32_t)(q + hN) : 0u, p.one, r0, r1);
          S[q] = __float2ull_rz(__fmul_rn(bits_to_exponential(r0), escale));
          if (q + hN < N1) S[q + hN] = __float2ull_rz(__fmul_rn(bits_to_exponential(r1), escale));
        }
        gbar(bar, G);
        const uint64_t den = group_scan(S, N1, W, wg, lane, wcta, wtot, bar, G, [&](int j) { return S[j]; });
        // merge path: C_i precedes S_k iff C_i den <= S_k Q; A_k = #{i : C_i precedes S_k}
        const int total = 2 * n, per = (total + G - 1) / G, d0 = tg * per;
        if (d0 < total) {
          int lo = d0 > n ? d0 - n : 0, hi = d0 < n ? d0 : n;
          while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (mul_le(C[mid], den, S[d0 - 1 - mid], Q)) lo = mid + 1;
            else hi = mid;
          }
          int i = lo, kk = d0 - lo;
          const int d1 = min(d0 + per, total);
          uint64_t ci = i < n ? C[i] : 0ull, sk = kk < n ? S[kk] : 0ull;
          for (int d = d0; d < d1; ++d) {
            if (i < n && (kk >= n || mul_le(ci, den, sk, Q))) {
              ++i;
              ci = i < n ? C[i] : 0ull;
            } else {
              A[kk] = i < n ? i : n - 1;
              ++kk;
              sk = kk < n ? S[kk] : 0ull;
            }
          }
        }
      } else {
        // systematic: T_k = floor((k 2^23 + m) Q / (n 2^23)), m = bits(k_t) >> 9
        uint32_t r0, r1;
        threefry2x32_m(k0, k1, 0u, 0u, p.one, r0, r1);
        group_systematic_fill(C, n, Q, r0 >> 9, magic, A, tg, G);
      }
      gbar(bar, G);
      for (int k = tg; k < n; k += G) XR[k] = X[A[k]];
      gbar(bar, G);
    }

    // ---- propagate + weight.  t = 0: x = m0 + c0 eps, written fma(m0, 1, c0 eps).
    const bool t0 = t == 0;
    const float pa = t0 ? 1.0f : p.phi, pb = t0 ? p.c0 : p.bsig;
    const float *src = res ? XR : X;
    float m = -INFINITY, s1 = 0.0f, s2 = 0.0f;
    int nanf = 0;
    auto emit = [&](int ii, float e) {
      const float xs = t0 ? p.m0 : src[ii];
      const float lp = (t0 || res) ? 0.0f : L[ii];
      const float xn = __fmaf_rn(xs, pa, __fmul_rn(e, pb));
      const float l = __fsub_rn(lp, sv_potential(p, xn, yv));
      X[ii] = xn;
      L[ii] = l;
      online_acc(l, m, s1, s2, nanf);
    };
    if (paired) {
      // particles i and i + n/2: split(k, n) words come from the same two cipher calls
      for (int i = tg; i < h; i += G) {
        uint32_t r0, r1, q0, q1, a0, a1, b0, b1;
        threefry2x32_m(k0, k1, 2 * i, 2 * i + n, p.one, r0, r1);
        threefry2x32_m(k0, k1, 2 * i + 1, 2 * i + 1 + n, p.one, q0, q1);
        threefry2x32_m(r0, q0, 0u, 0u, p.one, a0, a1);
        threefry2x32_m(r1, q1, 0u, 0u, p.one, b0, b1);
        emit(i, bits_to_normal(a0));
        emit(i + h, bits_to_normal(b0));
      }
    } else {
      for (int i = tg; i < n; i += G) {
        uint32_t e0, e1, a0, a1;
        split_at(k0, k1, (uint64_t)n, (uint64_t)i, e0, e1);
        threefry2x32_m(e0, e1, 0u, 0u, p.one, a0, a1);
        emit(i, bits_to_normal(a0));
      }
    }

    // ---- group logsumexp / ESS: per-warp partials, combined by every thread
    const float mw = warp_max(m);
    const float f = (m > -INFINITY && mw < INFINITY) ? expf(m - mw) : 0.0f;
    const float w1 = warp_sum(s1 * f), w2 = warp_sum(s2 * (f * f));
    const int wn = warp_or(nanf);
    float(*r)[32] = red[t & 1];
    if (lane == 0) {
      r[0][wcta] = mw;
      r[1][wcta] = w1;
      r[2][wcta] = w2;
      r[3][wcta] = wn ? 1.0f : 0.0f;
    }
    gbar(bar, G);
    const int w0 = wcta - wg;
    float Mg = r[0][w0];
    for (int w = 1; w < W; ++w) Mg = fmaxf(Mg, r[0][w0 + w]);
    float g1 = 0.0f, g2 = 0.0f, gn = 0.0f;
    for (int w = 0; w < W; ++w) {
      const float mv = r[0][w0 + w];
      const float fw = (mv > -INFINITY && Mg < INFINITY) ? expf(mv - Mg) : 0.0f;
      g1 += r[1][w0 + w] * fw;
      g2 += r[2][w0 + w] * (fw * fw);
      gn += r[3][w0 + w];
    }
    const bool finite = gn == 0.0f && Mg > -INFINITY && Mg < INFINITY;
    if (tg == 0) {
      double lse;
      if (gn != 0.0f) lse = __longlong_as_double(0x7ff8000000000000ll);
      else if (!finite) lse = Mg == INFINITY ? __longlong_as_double(0x7ff0000000000000ll)
                                             : -__longlong_as_double(0x7ff0000000000000ll);
      else lse = (double)Mg + (double)logf(g1);
      logz = t0 ? lse - logn : logz + lse - (res ? logn : lse_prev);
      lse_prev = lse;
    }
    // the next step resamples when ess = s1^2 / s2 < thr n (a NaN ess never does)
    res = finite && __fdiv_rn(__fmul_rn(g1, g1), g2) < thr_n;
    M = Mg;
    yv = y_next;
  }
  if (tg == 0) {
    a.logz[b] = logz;
    if (a.nres) a.nres[b] = nres;
  }
}

template <int TPB, int SCHEME>
__global__ void __launch_bounds__(TPB, 1) k_sv_batch(const __grid_constant__ SVParams p,
                                                     const __grid_constant__ SVBatch a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ float red[2][4][32];
  __shared__ uint32_t key_s[SVB_MAX_GROUPS][2][2];
  __shared__ unsigned long long wtot[32];
  __shared__ int bundle_s;
  const int lane = threadIdx.x & 31, wcta = threadIdx.x >> 5;
  for (;;) {
    if (threadIdx.x == 0) bundle_s = atomicAdd(a.counter, 1);
    __syncthreads();
    const int bi = bundle_s;
    if (bi >= a.nbundles) break;
    const int4 bd = a.bundles[bi];  // first, count, slot
    const int G = max(32, bd.z / a.ppt), W = G >> 5;
    const int gi = wcta / W;
    if (gi < bd.y)
      sv_filter<SCHEME>(p, a, a.order[bd.x + gi], smem + (size_t)gi * sv_slot_bytes(bd.z), G, W,
                        (int)threadIdx.x - gi * G, wcta - gi * W, lane, wcta, gi + 1, gi, red, key_s, wtot);
    __syncthreads();
  }
}

// ------------------------------------------------------------ host side
namespace {

int next_pow2(int v) {
  int s = 1;
  while (s < v) s <<= 1;
  return s;
}

// filters of slot size `slot` that one CTA runs at once
int groups_per_bundle(int slot, int threads, int ppt) {
  const int G = std::max(32, slot / ppt);
  int g = std::min(threads / G, (threads * ppt) / slot);
  g = std::min(g, G > 32 ? SVB_MAX_GROUPS - 1 : SVB_MAX_GROUPS);  // named barriers 1..15
  return g;
}

bool launch_shape_ok(const mgb_sv_launch &l) {
  if (l.threads != 256 && l.threads != 512 && l.threads != 1024) return false;
  if (l.ppt < 2 || l.ppt > 64 || (l.ppt & (l.ppt - 1))) return false;
  return l.ctas_per_sm >= 0;
}

template <int TPB, int SCHEME>
int launch_sv(const SVParams &p, const SVBatch &a, const mgb_sv_launch &l, cudaStream_t s) {
  auto kern = k_sv_batch<TPB, SCHEME>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)l.smem_bytes) != cudaSuccess)
    return ERR_UNSUPPORTED;
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return ERR_CUDA;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TPB, (size_t)l.smem_bytes) != cudaSuccess ||
      per_sm < 1)
    return ERR_UNSUPPORTED;
  if (l.ctas_per_sm > 0 && l.ctas_per_sm < per_sm) per_sm = l.ctas_per_sm;
  int grid = sms * per_sm;
  if (grid > a.nbundles) grid = a.nbundles;
  kern<<<grid, TPB, (size_t)l.smem_bytes, s>>>(p, a);
  return launch_status();
}

template <int SCHEME>
int launch_sv_tpb(const SVParams &p, const SVBatch &a, const mgb_sv_launch &l, cudaStream_t s) {
  switch (l.threads) {
    case 256: return launch_sv<256, SCHEME>(p, a, l, s);
    case 512: return launch_sv<512, SCHEME>(p, a, l, s);
    case 1024: return launch_sv<1024, SCHEME>(p, a, l, s);
    default: return ERR_BAD_ARG;
  }
}

int run_sv(const mgb_sv_model *m, const int32_t *n, const int32_t *T, const int64_t *y_off, const float *y,
           const uint32_t *keys, const mgb_sv_launch &l, const int32_t *order, const int32_t *bundles, float thr,
           int scheme, int32_t t_cap, int32_t *counter, double *logz, int32_t *nres, cudaStream_t s) {
  SVParams p{m->phi, m->bsig, m->r2, m->cB, m->c0, m->m0, 1u};
  SVBatch a{n, T, y_off, y, keys, order, (const int4 *)bundles, l.nbundles, l.ppt, t_cap, thr, logz, nres,
            (int *)counter};
  if (cudaMemsetAsync(counter, 0, sizeof(int32_t), s) != cudaSuccess) return ERR_CUDA;
  if (scheme == MGB_RESAMPLE_MULTINOMIAL) return launch_sv_tpb<MGB_RESAMPLE_MULTINOMIAL>(p, a, l, s);
  return launch_sv_tpb<MGB_RESAMPLE_SYSTEMATIC>(p, a, l, s);
}

// autotune cache: (device, scheme, threshold bits, probe steps, batch signature) -> (shape, ms)
std::mutex g_tune_mu;
std::map<std::tuple<int, int, uint32_t, int32_t, uint64_t>, std::pair<mgb_sv_launch, float>> g_tune_cache;

uint64_t batch_signature(int64_t B, const int32_t *n, const int32_t *T) {
  uint64_t h = 1469598103934665603ull ^ (uint64_t)B;
  for (int64_t b = 0; b < B; ++b) {
    h = (h ^ (uint32_t)n[b]) * 1099511628211ull;
    h = (h ^ (uint32_t)T[b]) * 1099511628211ull;
  }
  return h;
}

}  // namespace
}  // namespace mgb

using namespace mgb;

extern "C" {

int mgb_pf_sv_batch_plan(int64_t B, const int32_t *n_host, const int32_t *T_host, mgb_sv_launch *launch,
                         int32_t *order_host, int32_t *bundles_host) {
  if (!launch || B < 1 || B > 0x7FFFFFFFll || !launch_shape_ok(*launch)) return ERR_BAD_ARG;
  if (!n_host || !T_host || !order_host || !bundles_host) return ERR_BAD_ARG;
  const int cap = launch->threads * launch->ppt;
  std::vector<int> slot((size_t)B);
  for (int64_t b = 0; b < B; ++b) {
    if (n_host[b] < 2 || n_host[b] > MGB_SV_BATCH_MAX_N || T_host[b] < 1) return ERR_BAD_ARG;
    slot[b] = std::max(SVB_MIN_SLOT, next_pow2(n_host[b] + (n_host[b] & 1)));
    if (slot[b] > cap || sv_slot_bytes(slot[b]) > SVB_MAX_SMEM) return ERR_UNSUPPORTED;
  }
  // filters ordered by (slot descending, T descending, index)
  std::vector<int32_t> idx((size_t)B);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int32_t x, int32_t y) {
    if (slot[x] != slot[y]) return slot[x] > slot[y];
    return T_host[x] > T_host[y];
  });
  struct Bundle {
    int first, count, slot;
    double cost;
  };
  std::vector<Bundle> bl;
  size_t smem = 16;
  for (int64_t i = 0; i < B;) {
    const int s = slot[idx[i]];
    const int g = groups_per_bundle(s, launch->threads, launch->ppt);
    if (g < 1) return ERR_UNSUPPORTED;
    int64_t j = i;
    while (j < B && j - i < g && slot[idx[j]] == s) ++j;
    // a bundle's time ~ particles per thread x its longest T
    const double ppt_eff = (double)s / std::max(32, s / launch->ppt);
    bl.push_back({(int)i, (int)(j - i), s, ppt_eff * (double)T_host[idx[i]]});
    smem = std::max(smem, (size_t)(j - i) * sv_slot_bytes(s));
    i = j;
  }
  if (smem > SVB_MAX_SMEM) return ERR_UNSUPPORTED;
  std::stable_sort(bl.begin(), bl.end(), [](const Bundle &x, const Bundle &y) { return x.cost > y.cost; });
  for (int64_t i = 0; i < B; ++i) order_host[i] = idx[i];
  for (size_t k = 0; k < bl.size(); ++k) {
    bundles_host[4 * k] = bl[k].first;
    bundles_host[4 * k + 1] = bl[k].count;
    bundles_host[4 * k + 2] = bl[k].slot;
    bundles_host[4 * k + 3] = 0;
  }
  launch->nbundles = (int32_t)bl.size();
  launch->smem_bytes = (int64_t)smem;
  return OK;
}

int mgb_pf_sv_batch_run(const mgb_sv_model *m, int64_t B, const int32_t *n_dev, const int32_t *T_dev,
                        const int64_t *y_off_dev, const float *y_dev, const uint32_t *keys_dev,
                        const mgb_sv_launch *launch, const int32_t *order_dev, const int32_t *bundles_dev,
                        float ess_threshold, int scheme, int32_t *counter_dev, double *logz_dev, int32_t *nres_dev,
                        int32_t *err_dev, void *stream) {
  (void)err_dev;  // no device-side failure mode: every wait is a CTA / group barrier
  if (!m || !launch || B < 1 || !launch_shape_ok(*launch) || launch->nbundles < 1 || launch->nbundles > B ||
      launch->smem_bytes < 16 || (size_t)launch->smem_bytes > SVB_MAX_SMEM)
    return ERR_BAD_ARG;
  if (!n_dev || !T_dev || !y_off_dev || !y_dev || !keys_dev || !order_dev || !bundles_dev || !counter_dev ||
      !logz_dev)
    return ERR_BAD_ARG;
  if (scheme != MGB_RESAMPLE_MULTINOMIAL && scheme != MGB_RESAMPLE_SYSTEMATIC) return ERR_UNSUPPORTED;
  return run_sv(m, n_dev, T_dev, y_off_dev, y_dev, keys_dev, *launch, order_dev, bundles_dev, ess_threshold, scheme,
                0, counter_dev, logz_dev, nres_dev, (cudaStream_t)stream);
}

size_t mgb_pf_sv_batch_autotune_workspace(int64_t B) {
  if (B < 1) return 0;
  Carver c(nullptr);
  c.take<int32_t>((size_t)B);      // order
  c.take<int32_t>((size_t)B * 4);  // bundles
  c.take<int32_t>(1);              // counter
  c.take<double>((size_t)B);       // log Z
  return c.bytes();
}

int mgb_pf_sv_batch_autotune(const mgb_sv_model *m, int64_t B, const int32_t *n_host, const int32_t *T_host,
                             const int32_t *n_dev, const int32_t *T_dev, const int64_t *y_off_dev, const float *y_dev,
                             const uint32_t *keys_dev, float ess_threshold, int scheme, int32_t probe_steps,
                             void *ws, size_t ws_bytes, mgb_sv_launch *best, float *best_ms, void *stream) {
  if (!m || !best || B < 1 || !n_host || !T_host || !n_dev || !T_dev || !y_off_dev || !y_dev || !keys_dev || !ws)
    return ERR_BAD_ARG;
  if (scheme != MGB_RESAMPLE_MULTINOMIAL && scheme != MGB_RESAMPLE_SYSTEMATIC) return ERR_UNSUPPORTED;
  if (ws_bytes < mgb_pf_sv_batch_autotune_workspace(B)) return ERR_WORKSPACE;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return ERR_CUDA;
  uint32_t thr_bits;
  std::memcpy(&thr_bits, &ess_threshold, 4);
  const auto key = std::make_tuple(dev, scheme, thr_bits, probe_steps, batch_signature(B, n_host, T_host));
  {
    std::lock_guard<std::mutex> g(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      *best = it->second.first;
      if (best_ms) *best_ms = it->second.second;
      return OK;
    }
  }
  Carver c(ws);
  int32_t *order = c.take<int32_t>((size_t)B);
  int32_t *bundles = c.take<int32_t>((size_t)B * 4);
  int32_t *counter = c.take<int32_t>(1);
  double *logz = c.take<double>((size_t)B);
  cudaStream_t s = (cudaStream_t)stream;
  // candidate shapes {threads, particles per thread}
  static const int32_t cand[][2] = {{256, 32}, {512, 16}, {1024, 8}, {256, 16}, {512, 8}, {256, 8}, {256, 4}};
  std::vector<int32_t> ho((size_t)B), hb((size_t)B * 4);
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return ERR_CUDA;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return ERR_CUDA;
  }
  int rc = OK;
  bool found = false;
  mgb_sv_launch win{};
  float win_ms = 0.0f;
  for (const auto &cd : cand) {
    mgb_sv_launch l{cd[0], cd[1], 0, 0, 0};
    if (mgb_pf_sv_batch_plan(B, n_host, T_host, &l, ho.data(), hb.data()) != OK) continue;
    if (cudaMemcpyAsync(order, ho.data(), sizeof(int32_t) * (size_t)B, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(bundles, hb.data(), sizeof(int32_t) * 4 * (size_t)l.nbundles, cudaMemcpyHostToDevice, s) !=
            cudaSuccess) {
      rc = ERR_CUDA;
      break;
    }
    float ms = 0.0f;
    bool ok = true;
    for (int rep = 0; rep < 2 && ok; ++rep) {  // the second repetition is timed
      if (cudaEventRecord(e0, s) != cudaSuccess) rc = ERR_CUDA;
      ok = run_sv(m, n_dev, T_dev, y_off_dev, y_dev, keys_dev, l, order, bundles, ess_threshold, scheme,
                  probe_steps, counter, logz, nullptr, s) == OK;
      if (cudaEventRecord(e1, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) rc = ERR_CUDA;
      if (rc != OK) break;
      if (cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) rc = ERR_CUDA;
    }
    if (rc != OK) break;
    if (!ok) continue;
    if (!found || ms < win_ms) {
      win = l;
      win_ms = ms;
      found = true;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != OK) return rc;
  if (!found) return ERR_UNSUPPORTED;
  {
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tune_cache[key] = {win, win_ms};
  }
  *best = win;
  if (best_ms) *best_ms = win_ms;
  return OK;
}

}  // extern "C"
