/*
 * to_math.h - deterministic scalar math shared by the CUDA kernels and the
 * CPU oracle.
 *
 * Every function here is written out operation by operation (explicit fmaf,
 * no library transcendental), so that gcc (built with -ffp-contract=off) and
 * nvcc (built with --fmad=false) produce the same bits.  That is what lets a
 * GPU Monte Carlo path and its CPU restatement consume *identical* random
 * streams without materialising them: a stream value is a pure function of
 * (seed, stream id, path, year, patch).
 *
 * Contents
 *   - Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
 *     easy as 1, 2, 3", SC'11): counter-based generator, checked against the
 *     paper's known-answer vectors in the tests.
 *   - to_logf: frexp split + the atanh series log(m) = 2(s + s^3/3 + ...),
 *     s = (m-1)/(m+1), m in [sqrt(1/2), sqrt(2)).
 *   - to_expf: Cody & Waite (1980) additive range reduction x = k ln2 + r with
 *     a two-part ln2, then the degree-7 Taylor polynomial of e^r on |r|<=ln2/2.
 *   - to_sincospif: quadrant reduction y = q/2 + r (exact), then the Taylor
 *     series of sin(pi r), cos(pi r) on |r| <= 1/4.
 *   - Box-Muller normals and open/half-open uniforms from Philox words, with
 *     a table-assisted log (a 128-entry table of reciprocals and their logs
 *     reduces the mantissa to within 1/200 of 1, then a degree-4 series of
 *     log1p) and sine/cosine (a 128-entry table of sin/cos of 2 pi j/128,
 *     then the angle-addition formulas with degree-5 / degree-4 series for
 *     the remainder, below 2 pi/128); the tables (to_math_tables.h) are
 *     written by make_math_tables.py.
 *
 * The reference draws its streams from cuRAND XORWOW seeded with
 * srand(time(NULL)) (include/gpuCode/SimulateGPU.cu:3186-3214, 3732-3751,
 * 4167-4254), so it is not reproducible; this file is what replaces it.
 */
#ifndef TO_MATH_H
#define TO_MATH_H

#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define TO_HD __host__ __device__ __forceinline__
/* full unrolling of a loop whose trip count is known where it is inlined */
#define TO_UNROLL _Pragma("unroll")
#else
#define TO_HD static inline
#define TO_UNROLL
#endif

#include "to_math_tables.h"

typedef struct { float a, b; } to_f2;
/* the tables, once in device memory and once on the host, from the same
   literals */
#if defined(__CUDACC__)
static __device__ const to_f2 to_log_tab_d[128] = TO_LOG_TABLE_INIT;
static __device__ const to_f2 to_sc_tab_d[128] = TO_SINCOS_TABLE_INIT;
#endif
static const to_f2 to_log_tab_h[128] = TO_LOG_TABLE_INIT;
static const to_f2 to_sc_tab_h[128] = TO_SINCOS_TABLE_INIT;

/* ------------------------------------------------------------------------ */
/* bit casts                                                                 */
/* ------------------------------------------------------------------------ */
TO_HD uint32_t to_f2u(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    union { float f; uint32_t u; } v; v.f = f; return v.u;
#endif
}
TO_HD float to_u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    union { float f; uint32_t u; } v; v.u = u; return v.f;
#endif
}

/* ------------------------------------------------------------------------ */
/* Philox4x32-10                                                             */
/* ------------------------------------------------------------------------ */
#define TO_PHILOX_M0 0xD2511F53u
#define TO_PHILOX_M1 0xCD9E8D57u
#define TO_PHILOX_W0 0x9E3779B9u
#define TO_PHILOX_W1 0xBB67AE85u

typedef struct { uint32_t v[4]; } to_u32x4;

TO_HD void to_mulhilo(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo) {
#if defined(__CUDA_ARCH__)
    *hi = __umulhi(a, b);
    *lo = a * b;
#else
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    *lo = (uint32_t)p;
#endif
}

TO_HD to_u32x4 to_philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2,
                                uint32_t c3, uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        if (r > 0) { k0 += TO_PHILOX_W0; k1 += TO_PHILOX_W1; }
        uint32_t hi0, lo0, hi1, lo1;
        to_mulhilo(TO_PHILOX_M0, c0, &hi0, &lo0);
        to_mulhilo(TO_PHILOX_M1, c2, &hi1, &lo1);
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    }
    to_u32x4 o;
    o.v[0] = c0; o.v[1] = c1; o.v[2] = c2; o.v[3] = c3;
    return o;
}

/* uniform in (0,1): 24 random bits, centred in their cell (never 0 or 1) */
TO_HD float to_u01_open(uint32_t x) {
    return ((float)(x >> 8) + 0.5f) * 0x1p-24f;
}
/* uniform in [0,1) */
TO_HD float to_u01(uint32_t x) {
    return (float)(x >> 8) * 0x1p-24f;
}

/* ------------------------------------------------------------------------ */
/* natural log, x > 0 and normal                                             */
/* ------------------------------------------------------------------------ */
TO_HD float to_logf(float x) {
    uint32_t b = to_f2u(x);
    int e = (int)(b >> 23) - 127;
    float m = to_u2f((b & 0x007FFFFFu) | 0x3F800000u);   /* [1,2) */
    if (m > 1.41421356f) { m = m * 0.5f; e = e + 1; }     /* [0.707,1.414] */
    float s = (m - 1.0f) / (m + 1.0f);
    float s2 = s * s;
    float p = fmaf(s2, 0x1.c71c72p-4f /* 1/9 */, 0x1.24924ap-3f /* 1/7 */);
    p = fmaf(s2, p, 0x1.99999ap-3f /* 1/5 */);
    p = fmaf(s2, p, 0x1.555556p-2f /* 1/3 */);
    p = fmaf(s2, p, 1.0f);
    float lm = (2.0f * s) * p;
    float fe = (float)e;
    /* ln2 = hi + lo, hi has 24 bits */
    return fmaf(fe, 0x1.62e430p-1f, fmaf(fe, -0x1.05c610p-29f, lm));
}

/* ------------------------------------------------------------------------ */
/* exp                                                                       */
/* ------------------------------------------------------------------------ */
TO_HD float to_pow2i(int k) {           /* 2^k for k in [-126, 127] */
    return to_u2f((uint32_t)(k + 127) << 23);
}

TO_HD float to_expf(float x) {
    if (!(x == x)) return x;                       /* NaN propagates */
    if (x > 88.72283f) return to_u2f(0x7F800000u); /* +inf */
    if (x < -103.97208f) return 0.0f;
    float k = rintf(x * 0x1.715476p+0f);           /* x / ln2 */
    float r = fmaf(-k, 0x1.62e430p-1f, x);
    r = fmaf(-k, -0x1.05c610p-29f, r);
    float p = fmaf(r, 0x1.a01a02p-13f /* 1/5040 */, 0x1.6c16c2p-10f /* 1/720 */);
    p = fmaf(r, p, 0x1.111112p-7f /* 1/120 */);
    p = fmaf(r, p, 0x1.555556p-5f /* 1/24 */);
    p = fmaf(r, p, 0x1.555556p-3f /* 1/6 */);
    p = fmaf(r, p, 0.5f);
    p = fmaf(r, p, 1.0f);
    p = fmaf(r, p, 1.0f);
    int ki = (int)k;
    int k1 = ki / 2;
    int k2 = ki - k1;
    return (p * to_pow2i(k1)) * to_pow2i(k2);
}

/* ------------------------------------------------------------------------ */
/* sin(pi y), cos(pi y) for finite y >= 0 (used with y = 2u, u in [0,1))     */
/* ------------------------------------------------------------------------ */
TO_HD void to_sincospif(float y, float* sp, float* cp) {
    float q = rintf(y * 2.0f);          /* nearest quarter turn */
    float r = y - q * 0.5f;             /* exact, |r| <= 1/4 */
    float r2 = r * r;
    /* sin(pi r) = r * S(r^2) */
    float s = fmaf(r2, -0x1.e30750p-8f, 0x1.507834p-4f);
    s = fmaf(r2, s, -0x1.32d2ccp-1f);
    s = fmaf(r2, s, 0x1.466bc6p+1f);
    s = fmaf(r2, s, -0x1.4abbcep+2f);
    s = fmaf(r2, s, 0x1.921fb6p+1f);
    s = s * r;
    /* cos(pi r) = C(r^2) */
    float c = fmaf(r2, 0x1.f9d38ap-10f, -0x1.a6d1f2p-6f);
    c = fmaf(r2, c, 0x1.e1f506p-3f);
    c = fmaf(r2, c, -0x1.55d3c8p+0f);
    c = fmaf(r2, c, 0x1.03c1f0p+2f);
    c = fmaf(r2, c, -0x1.3bd3ccp+2f);
    c = fmaf(r2, c, 1.0f);
    int qi = ((int)q) & 3;
    float so, co;
    if (qi == 0)      { so = s;  co = c;  }
    else if (qi == 1) { so = c;  co = -s; }
    else if (qi == 2) { so = -s; co = -c; }
    else              { so = -c; co = s;  }
    *sp = so; *cp = co;
}

/* ------------------------------------------------------------------------ */
/* log of the open uniform to_u01_open(x), table-assisted: with u = 2^e m,    */
/* m in [1, 2), entry i = the top 7 bits of m's fraction gives R ~ 1/m and    */
/* G = -log R (entries whose interval lies above sqrt 2 read m as m/2 with    */
/* e + 1: their G carries -log 2), t = m R - 1 (|t| < 1/200, one rounding),   */
/* log u = e log 2 + G + log1p t, log1p t = t - t^2/2 + t^3/3 - t^4/4.         */
/* ------------------------------------------------------------------------ */
TO_HD to_f2 to_log_entry(int i) {
#if defined(__CUDA_ARCH__)
    return to_log_tab_d[i];
#else
    return to_log_tab_h[i];
#endif
}

TO_HD to_f2 to_sincos_entry(int j) {
#if defined(__CUDA_ARCH__)
    return to_sc_tab_d[j];
#else
    return to_sc_tab_h[j];
#endif
}

TO_HD float to_log_u01(uint32_t x) {
    const uint32_t b = to_f2u(to_u01_open(x));
    const int i = (int)((b >> 16) & 127u);
    const to_f2 rg = to_log_entry(i);
    const int e = (int)(b >> 23) - 127 + (i >= TO_LOG_SPLIT ? 1 : 0);
    const float m = to_u2f((b & 0x007FFFFFu) | 0x3F800000u);
    const float t = fmaf(m, rg.a, -1.0f);
    float q = fmaf(t, -0.25f, 0x1.555556p-2f /* 1/3 */);
    q = fmaf(t, q, -0.5f);
    q = q * t;
    const float lg = rg.b + fmaf(q, t, t);
    const float fe = (float)e;
    /* ln2 = hi + lo, hi has 24 bits */
    return fmaf(fe, 0x1.62e430p-1f, fmaf(fe, -0x1.05c610p-29f, lg));
}

/* sin and cos of 2 pi to_u01(x): the angle's top 7 bits pick the table entry
   (sin a, cos a), a = 2 pi j / 128; the remaining 17 bits give the remainder
   r < 2 pi / 128, whose sine r - r^3/6 + r^5/120 and cosine 1 - r^2/2 + r^4/24
   combine with the entry by the angle-addition formulas */
TO_HD void to_sincos2pi_u01(uint32_t x, float* sp, float* cp) {
    const int j = (int)(x >> 25);
    const float r = (float)((x >> 8) & 0x1FFFFu) * 0x1.921fb6p-22f;   /* 2 pi 2^-24 */
    const float r2 = r * r;
    float s = fmaf(r2, 0x1.111112p-7f /* 1/120 */, -0x1.555556p-3f /* -1/6 */);
    s = fmaf(r2 * r, s, r);
    float c = fmaf(r2, 0x1.555556p-5f /* 1/24 */, -0.5f);
    c = fmaf(r2, c, 1.0f);
    const to_f2 sc = to_sincos_entry(j);
    *sp = fmaf(sc.a, c, sc.b * s);
    *cp = fmaf(sc.b, c, -(sc.a * s));
}

/* Box-Muller: two Philox words -> two standard normals, radius from the
   open uniform of the first, angle from the half-open uniform of the second */
TO_HD void to_box_muller(uint32_t a, uint32_t b, float* z0, float* z1) {
    float rad = sqrtf(-2.0f * to_log_u01(a));
    float sn, cs;
    to_sincos2pi_u01(b, &sn, &cs);
    *z0 = rad * cs;
    *z1 = rad * sn;
}

/* ------------------------------------------------------------------------ */
/* a / b rounded to nearest, from rb = 1 / b rounded to nearest (computed    */
/* once per divisor): q = RN(a rb); the remainder a - b q is exact in one    */
/* FMA; RN(q + (a - b q) rb) is the correctly rounded quotient whenever no   */
/* step over- or underflows (P. Markstein, "Computation of elementary        */
/* functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1), */
/* 1990).  The same value as the division a / b, bit for bit.                */
/* ------------------------------------------------------------------------ */
TO_HD float to_div_rcp(float a, float b, float rb) {
    const float q = a * rb;
    const float r = fmaf(-q, b, a);
    return fmaf(r, rb, q);
}

/* ------------------------------------------------------------------------ */
/* Stream layout.  A stream value is addressed by (stream, path, year,        */
/* lane-group, lane).  One Philox call yields 4 words -> 4 uniforms or 4      */
/* normals (two Box-Muller pairs).                                            */
/* ------------------------------------------------------------------------ */
enum to_stream_id {
    TO_STREAM_GROWTH      = 1,  /* per (path, year, species*patch) N(0,1)  */
    TO_STREAM_SP_BROWNIAN = 2,  /* per (path, year, species) N(0,1)        */
    TO_STREAM_SP_JUMPSIZE = 3,  /* per (path, year, species) N(0,1)        */
    TO_STREAM_SP_JUMP     = 4,  /* per (path, year, species) U[0,1)        */
    TO_STREAM_CONTROL     = 5,  /* per (path, year) U[0,1)                 */
    TO_STREAM_EX_BROWNIAN = 6,  /* per (path, year, process) N(0,1)        */
    TO_STREAM_EX_JUMPSIZE = 7,  /* per (path, year, process) N(0,1)        */
    TO_STREAM_EX_JUMP     = 8,  /* per (path, year, process) U[0,1)        */
    TO_STREAM_ORE         = 9,  /* per (path, year, commodity) N(0,1)      */
    TO_STREAM_PV_BROWNIAN = 10, /* expected-PV paths                       */
    TO_STREAM_PV_JUMPSIZE = 11,
    TO_STREAM_PV_JUMP     = 12
};

/* key = seed; counter = (group, year, path, stream | road << 8) */
TO_HD to_u32x4 to_stream_block(uint64_t seed, uint32_t stream, uint32_t road,
                               uint32_t path, uint32_t year, uint32_t group) {
    return to_philox4x32_10(group, year, path, stream | (road << 8),
                            (uint32_t)seed, (uint32_t)(seed >> 32));
}

/* four normals for lanes 4*group .. 4*group+3 */
TO_HD void to_normal4(uint64_t seed, uint32_t stream, uint32_t road,
                      uint32_t path, uint32_t year, uint32_t group,
                      float out[4]) {
    to_u32x4 w = to_stream_block(seed, stream, road, path, year, group);
    to_box_muller(w.v[0], w.v[1], &out[0], &out[1]);
    to_box_muller(w.v[2], w.v[3], &out[2], &out[3]);
}

/* normal number (lane & 3) of the group's four: only its Box-Muller pair is
   evaluated, with the same operations as in to_normal4 */
TO_HD float to_normal1(uint64_t seed, uint32_t stream, uint32_t road,
                       uint32_t path, uint32_t year, uint32_t lane) {
    to_u32x4 w = to_stream_block(seed, stream, road, path, year, lane >> 2);
    const int hi = (lane & 2) != 0;
    float z0, z1;
    to_box_muller(hi ? w.v[2] : w.v[0], hi ? w.v[3] : w.v[1], &z0, &z1);
    return (lane & 1) ? z1 : z0;
}

TO_HD float to_uniform1(uint64_t seed, uint32_t stream, uint32_t road,
                        uint32_t path, uint32_t year, uint32_t lane) {
    to_u32x4 w = to_stream_block(seed, stream, road, path, year, lane >> 2);
    return to_u01(w.v[lane & 3]);
}

#endif /* TO_MATH_H */
