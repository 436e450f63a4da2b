/*
 * ORACLE -- test infrastructure only.  Nothing in the product (mocat_gb300/)
 * may include, link or call this file; only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg use it, and only as the checker.
 *
 * CPU restatement of the random-number layer mocat draws from
 * (`jax.random`, unpinned in setup.py:15-16 of the reference; era
 * jax ~0.2.25-0.4.x with `jax_threefry_partitionable` off):
 *   - threefry2x32-20 block cipher (Salmon et al., "Parallel random numbers:
 *     as easy as 1, 2, 3", SC'11 -- the published Random123 algorithm);
 *   - jax.random's non-partitionable counter layout for `split`,
 *     `random_bits`, `uniform`, `normal`, `exponential`, `gumbel`;
 *   - the float maths those draws need, written from textbook methods so that
 *     the device code (written separately) can reproduce them bit for bit:
 *       logf: range reduction to [sqrt(1/2), sqrt(2)) + 2*atanh series;
 *       expf: Cody-Waite reduction by ln2 + degree-7 Taylor polynomial;
 *       erfinvf: M. Giles, "Approximating the erfinv function" (GPU Computing
 *                Gems Jade, 2011), single-precision branch.
 * Call sites in the reference: mocat/src/ssm/filtering.py:181,199,267,278,294;
 * mocat/src/transport/smc.py:65,82,140; linear_gaussian.py:51,94,139;
 * stochastic_volatility.py:76,93,108; nonlinear_gaussian.py:209,249,275.
 *
 * Compile with -ffp-contract=off: every fused multiply-add below is explicit.
 */
#ifndef MOCAT_ORACLE_RNG_H
#define MOCAT_ORACLE_RNG_H

#include <stdint.h>
#include <string.h>
#include <math.h>

static inline uint32_t o_rotl32(uint32_t v, int r) { return (v << r) | (v >> (32 - r)); }

static inline float o_asf(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static inline uint32_t o_asu(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

/* threefry2x32 with 20 rounds: five groups of four rounds, key injection after
 * each group (Random123; the rotation table is the published one). */
static inline void o_threefry2x32(uint32_t k0, uint32_t k1, uint32_t c0, uint32_t c1,
                                  uint32_t *r0, uint32_t *r1)
{
    static const int rot[2][4] = {{13, 15, 26, 6}, {17, 29, 16, 24}};
    uint32_t ks[3] = {k0, k1, k0 ^ k1 ^ 0x1BD11BDAu};
    uint32_t x0 = c0 + ks[0], x1 = c1 + ks[1];
    for (int g = 0; g < 5; ++g) {
        const int *rr = rot[g & 1];
        for (int i = 0; i < 4; ++i) {
            x0 += x1;
            x1 = o_rotl32(x1, rr[i]);
            x1 ^= x0;
        }
        x0 += ks[(g + 1) % 3];
        x1 += ks[(g + 2) % 3] + (uint32_t)(g + 1);
    }
    *r0 = x0;
    *r1 = x1;
}

/* Element p of jax's threefry_2x32(key, iota(n)): the count vector is padded to
 * even length with a zero, split in halves (x0 = first half, x1 = second
 * half), and the outputs are concatenated [out0, out1] and trimmed to n. */
static inline uint32_t o_bits_at(uint32_t k0, uint32_t k1, uint64_t n, uint64_t p)
{
    uint64_t h = (n + 1) / 2;
    uint32_t r0, r1;
    if (p < h) {
        uint64_t c1 = p + h;
        o_threefry2x32(k0, k1, (uint32_t)p, c1 < n ? (uint32_t)c1 : 0u, &r0, &r1);
        return r0;
    }
    o_threefry2x32(k0, k1, (uint32_t)(p - h), (uint32_t)p, &r0, &r1);
    return r1;
}

/* split(key, num)[i] = (bits[2i], bits[2i+1]) of threefry_2x32(key, iota(2 num)). */
static inline void o_split_at(uint32_t k0, uint32_t k1, uint64_t num, uint64_t i,
                              uint32_t *o0, uint32_t *o1)
{
    *o0 = o_bits_at(k0, k1, 2 * num, 2 * i);
    *o1 = o_bits_at(k0, k1, 2 * num, 2 * i + 1);
}

/* uniform [0,1) mantissa fill: (bits >> 9) | 0x3f800000, minus 1. */
static inline float o_bits_to_unit(uint32_t b) { return o_asf((b >> 9) | 0x3f800000u) - 1.0f; }

/* ---------------- float maths (textbook methods, explicit fma) ---------------- */

/* natural log of a positive normal float */
static inline float o_logf(float x)
{
    uint32_t ix = o_asu(x);
    int e = (int)((ix >> 23) & 0xffu) - 127;
    uint32_t mb = (ix & 0x007fffffu) | 0x3f800000u;
    if (mb > 0x3fb504f3u) { mb -= 0x00800000u; e += 1; }   /* m > sqrt(2): halve */
    float m = o_asf(mb);
    /* log(1 + f) = f - f^2/2 + f^3 q(f), f = m - 1 (exact) in [sqrt(1/2) - 1, sqrt(2) - 1];
     * q: degree-7 weighted least-squares fit (relative error of the sum < 6e-9) */
    float f = m - 1.0f;
    float f2 = f * f;
    float q = fmaf(f, -0x1.38b582p-4f, 0x1.055b72p-3f);
    q = fmaf(f, q, -0x1.0d8544p-3f);
    q = fmaf(f, q, 0x1.22da1cp-3f);
    q = fmaf(f, q, -0x1.547244p-3f);
    q = fmaf(f, q, 0x1.99a008p-3f);
    q = fmaf(f, q, -0x1.000226p-2f);
    q = fmaf(f, q, 0x1.555554p-2f);
    float lm = f + fmaf(f2 * f, q, -0.5f * f2);
    float ef = (float)e;
    return fmaf(ef, 0x1.63p-1f, fmaf(ef, -0x1.bd0106p-13f, lm));   /* e*ln2 split hi/lo */
}

/* exp; returns 0 below -104 (and for -inf), +inf above 88.5, NaN for NaN */
static inline float o_expf(float x)
{
    if (x != x) return x;
    if (x < -104.0f) return 0.0f;
    if (x > 88.5f) return INFINITY;
    float kf = rintf(x * 0x1.715476p+0f);
    float r = fmaf(-kf, 0x1.63p-1f, x);
    r = fmaf(-kf, -0x1.bd0106p-13f, r);
    float p = fmaf(r, 0x1.a01a02p-13f, 0x1.6c16c2p-10f);   /* 1/7!, 1/6! */
    p = fmaf(r, p, 0x1.111112p-7f);                        /* 1/5! */
    p = fmaf(r, p, 0x1.555556p-5f);                        /* 1/4! */
    p = fmaf(r, p, 0x1.555556p-3f);                        /* 1/3! */
    p = fmaf(r, p, 0.5f);
    p = fmaf(r, p, 1.0f);
    p = fmaf(r, p, 1.0f);
    int k = (int)kf;
    if (k < -126) return (p * o_asf((uint32_t)(k + 64 + 127) << 23)) * 0x1p-64f;
    if (k > 127) return (p * 2.0f) * o_asf((uint32_t)(k - 1 + 127) << 23);
    return p * o_asf((uint32_t)(k + 127) << 23);
}

/* Giles (2011) single-precision erfinv; w = -log(1 - x^2) with one rounding */
static inline float o_erfinvf(float x)
{
    float w = -o_logf(fmaf(-x, x, 1.0f));
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

/* jax.random.normal element from raw bits: u = max(lo, f*(1 - lo) + lo) with
 * lo = nextafter(-1, 0) and (1 - lo) == 2.0f in float32; sqrt(2)*erfinv(u). */
static inline float o_bits_to_normal(uint32_t b)
{
    const float lo = -0x1.fffffep-1f;
    float f = o_bits_to_unit(b);
    float u = f * 2.0f + lo;
    if (u < lo) u = lo;
    return 0x1.6a09e6p+0f * o_erfinvf(u);
}

/* jax.random.exponential element: -log1p(-u), evaluated as -log(1 - u) (1-u exact) */
static inline float o_bits_to_exponential(uint32_t b)
{
    float u = o_bits_to_unit(b);
    return -o_logf(1.0f - u);
}

/* jax.random.gumbel element: -log(-log(max(tiny, f + tiny))) */
static inline float o_bits_to_gumbel(uint32_t b)
{
    const float tiny = 0x1p-126f;
    float f = o_bits_to_unit(b);
    float u = f * 1.0f + tiny;
    if (u < tiny) u = tiny;
    return -o_logf(-o_logf(u));
}

#endif
