/*
 * to_lsm_math.h - per-query and per-path arithmetic of the regression Monte
 * Carlo backward induction, shared by the CUDA kernels and the CPU oracle so
 * that both make the same discontinuous decisions (kNN boundaries, control
 * argmin) on the same inputs.  Written operation by operation; built with
 * --fmad=false / -ffp-contract=off.
 *
 * Reference (include/gpuCode/SimulateGPU.cu):
 *   query grid axis           createQueryPoints      :1177-1190
 *   host normalisation        simulateROVCUDA        :4591-4607 (scaling 2)
 *   Gaussian kernel weights,  multiLocLinReg         :2982-3033
 *   normal equations
 *   solve                     solveLinearSystem      :129-190 (FP32 Gaussian
 *                             elimination; here FP64 square-root-free
 *                             Cholesky, with near-singular directions
 *                             dropped)
 *   interpolation of the      backwardInduction      :2564-2703
 *   regression grid
 */
#ifndef TO_LSM_MATH_H
#define TO_LSM_MATH_H

#include <float.h>
#include <math.h>
#include "to_math.h"

#define TO_LSM_MAXD 5                 /* regression dimensions (species + 1) */
#define TO_LSM_ACC (TO_LSM_MAXD + 1 + (TO_LSM_MAXD + 1) * (TO_LSM_MAXD + 1))

TO_HD float to_lsm_query_axis(int di, float lo, float hi, int R) {
    return ((float)di * (hi - lo)) / (float)(R - 1) + lo;
}

TO_HD float to_lsm_unit_axis(int di, int R) {
    return ((float)di * (1.0f - 0.0f)) / (float)(R - 1) + 0.0f;
}

TO_HD float to_lsm_normalise(float x, float lo, float hi, int is_profit, float scaling) {
    return is_profit ? (x - lo) / (scaling * (hi - lo)) : (x - lo) / (hi - lo);
}

/* Gaussian kernel weight exp(-(d/h)^2/2)/sqrt(2 pi).  The reference
 * divides by sqrt(2 pi) in double (SimulateGPU.cu:2995); the constant
 * cancels in the normal equations, so it is applied here as one float
 * multiply (results differ from the double form by at most one rounding). */
TO_HD float to_lsm_weight(float d, float h) {
    float t = d / h;
    float w = ((-t) * t) / 2.0f;
    return to_expf(w) * 0.3989422804f;
}

/* to_lsm_weight(d, h) for a neighbour within the bandwidth, 0 <= d <= h,
 * with rh = 1 / h computed once per query: the same bits.  t = d / h by
 * to_div_rcp (correctly rounded: t <= 1, and the remainder d - h q is a
 * multiple of about 2^-46 d, far above the float underflow for any float
 * distance d > 0).  w = -t^2 / 2 then lies in [-1/2, 0], where to_expf's
 * range checks never fire and its k = rint(w / ln 2) is 0 or -1: its
 * scaling (p 2^(k/2)) 2^(k - k/2) is p 2^k. */
TO_HD float to_lsm_weight_within(float d, float h, float rh) {
    const float t = to_div_rcp(d, h, rh);
    const float w = ((-t) * t) / 2.0f;
    const float k = rintf(w * 0x1.715476p+0f);
    float r = fmaf(-k, 0x1.62e430p-1f, w);
    r = fmaf(-k, -0x1.05c610p-29f, r);
    float p = fmaf(r, 0x1.a01a02p-13f, 0x1.6c16c2p-10f);
    p = fmaf(r, p, 0x1.111112p-7f);
    p = fmaf(r, p, 0x1.555556p-5f);
    p = fmaf(r, p, 0x1.555556p-3f);
    p = fmaf(r, p, 0.5f);
    p = fmaf(r, p, 1.0f);
    p = fmaf(r, p, 1.0f);
    return (p * to_pow2i((int)k)) * 0.3989422804f;
}

/* acc = [B (m) | A (m x m row-major)], m = dim + 1; only i <= j of A */
TO_HD void to_lsm_acc_init(int dim, float* acc) {
    int m = dim + 1;
    for (int i = 0; i < m + m * m; ++i) acc[i] = 0.0f;
}

TO_HD void to_lsm_acc_add(int dim, float* acc, float z, float y, const float* xv,
                          const float* xq) {
    int m = dim + 1;
    float* B = acc;
    float* A = acc + m;
    float dx[TO_LSM_MAXD];
    for (int j = 0; j < dim; ++j) dx[j] = xv[j] - xq[j];
    B[0] = fmaf(y, z, B[0]);
    for (int j = 0; j < dim; ++j) B[j + 1] = fmaf(y * dx[j], z, B[j + 1]);
    A[0] = A[0] + z;
    for (int j = 0; j < dim; ++j) A[j + 1] = fmaf(dx[j], z, A[j + 1]);
    for (int i = 0; i < dim; ++i)
        for (int j = i; j < dim; ++j)
            A[(i + 1) * m + (j + 1)] = fmaf(dx[j] * dx[i], z, A[(i + 1) * m + (j + 1)]);
}

/* 1 / x for x > 0 in double: the float reciprocal of x refined by two
 * Newton-Raphson steps y <- y + y (1 - x y), each with the residual in one
 * FMA (relative error about 2^-23, then 2^-46, then within an ulp).  x out
 * of float range takes the division. */
TO_HD double to_rcp64(double x) {
    const float xf = (float)x;
    if (!(xf > 1e-37f && xf < 1e37f)) return 1.0 / x;
    double y = (double)(1.0f / xf);
    y = fma(y, fma(-x, y, 1.0), y);
    y = fma(y, fma(-x, y, 1.0), y);
    return y;
}

/* FP64 square-root-free Cholesky (L D L^T) of the (symmetric) normal
 * equations, with the unknowns ordered slopes first and the intercept
 * last: with L unit lower triangular, L y = b and the intercept is
 * y[m-1] / d[m-1], with no back substitution.  Each pivot's reciprocal
 * (to_rcp64) scales its column.  A direction whose pivot falls below 1e-6
 * of its diagonal is dropped (its coefficient set to zero).  Returns the
 * intercept (the regression value at the query), 0 when its own direction
 * is dropped.  Every update s - l u is one fused multiply-add (half the
 * FP64 operations of a multiply and a subtraction; the FP64 pipe bounds
 * the solve).  sums: the right-hand sides B (m values), then the upper
 * triangle i <= j of the matrix A in row order. */
TO_HD float to_lsm_solve_compact(int dim, const double* sums) {
    int m = dim + 1;
    double A[(TO_LSM_MAXD + 1) * (TO_LSM_MAXD + 1)];
    double L[(TO_LSM_MAXD + 1) * (TO_LSM_MAXD + 1)];   /* L[i][j], i > j */
    double U[(TO_LSM_MAXD + 1) * (TO_LSM_MAXD + 1)];   /* L[i][j] d[j] */
    double b[TO_LSM_MAXD + 1], y[TO_LSM_MAXD + 1], inv[TO_LSM_MAXD + 1];
    int keep[TO_LSM_MAXD + 1];
    /* unknown p of the solve is term (p + 1) % m of the accumulated sums
     * (term 0 is the intercept) */
    TO_UNROLL
    for (int i = 0; i < m; ++i) {
        const int oi = (i + 1) % m;
        b[i] = sums[oi];
        TO_UNROLL
        for (int j = 0; j <= i; ++j) {
            const int oj = (j + 1) % m;
            const int a = oi <= oj ? oi : oj, c = oi <= oj ? oj : oi;
            A[i * m + j] = sums[m + a * m - a * (a - 1) / 2 + (c - a)];
        }
    }
    TO_UNROLL
    for (int j = 0; j < m; ++j) {
        double s = A[j * m + j];
        TO_UNROLL
        for (int k = 0; k < j; ++k)
            if (keep[k]) s = fma(-L[j * m + k], U[j * m + k], s);
        if (!(s > 1e-6 * A[j * m + j]) || !(s > 0.0)) { keep[j] = 0; continue; }
        keep[j] = 1;
        inv[j] = to_rcp64(s);
        TO_UNROLL
        for (int i = j + 1; i < m; ++i) {
            double v = A[i * m + j];
            TO_UNROLL
            for (int k = 0; k < j; ++k)
                if (keep[k]) v = fma(-L[i * m + k], U[j * m + k], v);
            U[i * m + j] = v;
            L[i * m + j] = v * inv[j];
        }
    }
    TO_UNROLL
    for (int i = 0; i < m; ++i) {
        if (!keep[i]) { y[i] = 0.0; continue; }
        double v = b[i];
        TO_UNROLL
        for (int k = 0; k < i; ++k)
            if (keep[k]) v = fma(-L[i * m + k], y[k], v);
        y[i] = v;
    }
    return keep[m - 1] ? (float)(y[m - 1] * inv[m - 1]) : 0.0f;
}

/* The same from the accumulator layout acc = [B (m) | A (m x m)]: its
 * sums in the compact order (B, then the upper triangle of A in row
 * order), exactly as doubles. */
TO_HD float to_lsm_solve_intercept(int dim, const float* acc) {
    const int m = dim + 1;
    double sums[(TO_LSM_MAXD + 1) + (TO_LSM_MAXD + 1) * (TO_LSM_MAXD + 2) / 2];
    int e = 0;
    TO_UNROLL
    for (int i = 0; i < m; ++i) sums[e++] = (double)acc[i];
    TO_UNROLL
    for (int i = 0; i < m; ++i)
        TO_UNROLL
        for (int j = i; j < m; ++j) sums[e++] = (double)acc[m + i * m + j];
    return to_lsm_solve_compact(dim, sums);
}

/* float -> int the way the reference's assignment truncates, with the GPU's
 * saturating behaviour for non-finite values */
TO_HD int to_lsm_trunc(float v) {
    if (!(v == v)) return 0;
    if (v >= 2147483520.0f) return 2147483647;
    if (v <= -2147483648.0f) return (-2147483647 - 1);
    return (int)v;
}

TO_HD int to_lsm_lower_index(float s, float lo, float hi, int R) {
    int li = to_lsm_trunc(((float)(R - 1) * (s - lo)) / (hi - lo));
    if (li < 0) li = 0;
    else if (li >= R - 1) li = R - 2;
    return li;
}

/* backwardInduction's interpolation of one control's regression block
 * exactly as the reference evaluates it (SimulateGPU.cu:2575-2697): lower
 * indices from the highest-flow state, the first weight taken from species
 * 0 but applied along the profit axis, the last fold with zero stride. */
TO_HD float to_lsm_interp_ref(const float* rb, int R, int S, int C,
                              const float* state) {
    int d = S + 1;
    int li[TO_LSM_MAXD];
    for (int j = 0; j < S; ++j)
        li[j] = to_lsm_lower_index(state[(C - 1) * S + j], rb[j * R], rb[(j + 1) * R - 1], R);
    li[S] = to_lsm_lower_index(state[S * C], rb[S * R], rb[(S + 1) * R - 1], R);
    float x0 = rb[li[0]], x1 = rb[li[0] + 1];
    float xd = (fabsf(x1 - x0) < FLT_EPSILON || x0 == x1) ? 0.0f
             : (state[(C - 1) * S] - x0) / (x1 - x0);
    float coeffs[1 << (TO_LSM_MAXD - 1)];
    int powR[TO_LSM_MAXD + 1];
    powR[0] = 1;
    for (int e = 1; e <= d; ++e) powR[e] = powR[e - 1] * R;
    for (int jj = 0; jj < (1 << S); ++jj) {
        int idx = R * d;
        int div = jj;
        for (int kk = 0; kk < S; ++kk) {
            int rem = div - 2 * (div / 2);
            div = div / 2;
            idx += (li[S - 1 - kk] + rem) * powR[kk + 1];
        }
        idx += li[S];
        coeffs[jj] = fmaf(rb[idx + 1], xd, rb[idx] * (1.0f - xd));
    }
    for (int jj = 1; jj <= S; ++jj) {
        x0 = rb[jj * R + li[jj]];
        x1 = rb[jj * R + li[jj] + 1];
        xd = (fabsf(x1 - x0) < FLT_EPSILON || x0 == x1) ? 0.0f
           : (state[(C - 1) * S + jj] - x0) / (x1 - x0);
        int e = S - jj - 1;
        int jump = (e >= 0) ? (1 << e) : 0;
        for (int kk = 0; kk < (1 << jj); ++kk)
            coeffs[kk] = fmaf(coeffs[kk + jump], xd, coeffs[kk] * (1.0f - xd));
    }
    return coeffs[0];
}

/* multilinear interpolation of one control's regression block at that
 * control's own state (species states s[0..S-1], profit) */
TO_HD float to_lsm_interp(const float* rb, int R, int S, const float* s, float profit) {
    int d = S + 1;
    int li[TO_LSM_MAXD];
    float w[TO_LSM_MAXD];
    for (int j = 0; j < d; ++j) {
        float v = (j < S) ? s[j] : profit;
        float lo = rb[j * R], hi = rb[j * R + R - 1];
        li[j] = to_lsm_lower_index(v, lo, hi, R);
        float x0 = rb[j * R + li[j]], x1 = rb[j * R + li[j] + 1];
        float t = (x1 - x0 > 0.0f) ? (v - x0) / (x1 - x0) : 0.0f;
        w[j] = t < 0.0f ? 0.0f : (t > 1.0f ? 1.0f : t);
    }
    float acc = 0.0f;
    for (int corner = 0; corner < (1 << d); ++corner) {
        float wt = 1.0f;
        int idx = 0;
        for (int j = 0; j < d; ++j) {
            int bit = (corner >> (d - 1 - j)) & 1;
            wt = wt * (bit ? w[j] : 1.0f - w[j]);
            idx = idx * R + li[j] + bit;
        }
        acc = fmaf(wt, rb[R * d + idx], acc);
    }
    return acc;
}

#endif /* TO_LSM_MATH_H */
