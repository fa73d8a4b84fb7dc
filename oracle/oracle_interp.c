/*
 * oracle_interp.c - CPU restatement of the surrogate evaluations
 * (test infrastructure for transportoptimiser_gb300/csrc/interp.cu).
 *   mode 0: SimulateGPU::interpolateSurrogateMulti's kernel interpolateMulti
 *           (SimulateGPU.cu:3077-3155), float, quirks Q26/Q27 kept;
 *   mode 1: multilinear interpolation in double;
 *   mode 2: Utility::interpolateSurrogate (Utility.cpp:253-363) in double.
 * Layout: [R*d axis values | R^d values], dimension 0 most significant.
 */
#include "oracle_interp.h"

#include <math.h>
#include <stddef.h>

#define MAXD 6

static float ref_kernel(int idx, int d, int R, const float* S, const float* P) {
    int lowerInd[MAXD], rpow[MAXD + 1];
    float coeffs[1 << (MAXD - 1)];
    for (int jj = 0; jj < d; ++jj) {
        float lower = S[jj * R], upper = S[(jj + 1) * R - 1];
        int li = (int)(((float)(R - 1) * (P[d * idx + jj] - lower)) / (upper - lower));
        if (li >= R - 1) li = R - 2;
        else if (li < 0) li = 0;
        lowerInd[jj] = li;
    }
    rpow[0] = 1;
    for (int q = 1; q <= d; ++q) rpow[q] = rpow[q - 1] * R;
    float x0 = S[lowerInd[0]], x1 = S[lowerInd[0] + 1];
    float xd = (P[d * idx] - x0) / (x1 - x0);
    for (int jj = 0; jj < (1 << (d - 1)); ++jj) {
        int idxL = R * d;
        for (int kk = 1; kk < d; ++kk) {
            int q = jj / (1 << (d - kk - 1));
            int rem = (q + 1) - 2 * ((q + 1) / 2);
            idxL += (rem > 0 ? lowerInd[kk] : lowerInd[kk] + 1) * rpow[d - kk - 1];
        }
        int idxU = idxL + (lowerInd[0] + 1) * rpow[d - 1];
        idxL += lowerInd[0] * rpow[d - 1];
        coeffs[jj] = S[idxL] * (1 - xd) + S[idxU] * xd;
    }
    for (int jj = 1; jj < d; ++jj) {
        x0 = S[jj * R + lowerInd[jj]];
        x1 = S[jj * R + lowerInd[jj] + 1];
        xd = (P[jj] - x0) / (x1 - x0);                  /* point 0's predictor (Q26) */
        int jump = (d - jj - 2 >= 0) ? (1 << (d - jj - 2)) : 0;   /* (int)pow(2, -1) = 0 (Q27) */
        for (int kk = 0; kk < (1 << jj); ++kk)
            coeffs[kk] = coeffs[kk] * (1 - xd) + coeffs[kk + jump] * xd;
    }
    return coeffs[0];
}

static double multilinear(const double* S, const double* p, int d, int R) {
    int lo[MAXD];
    double w[MAXD];
    for (int j = 0; j < d; ++j) {
        const double* ax = S + (size_t)j * R;
        double a0 = ax[0], a1 = ax[R - 1];
        (void)a0; (void)a1;
        int i = 0, hi = R - 2;                 /* last i with ax[i] <= p (clamped) */
        while (i < hi) {
            const int mid = (i + hi + 1) >> 1;
            if (ax[mid] <= p[j]) i = mid; else hi = mid - 1;
        }
        double x0 = ax[i], x1 = ax[i + 1];
        w[j] = (x1 != x0) ? (p[j] - x0) / (x1 - x0) : 0.0;
        lo[j] = i;
    }
    double acc = 0.0;
    for (int corner = 0; corner < (1 << d); ++corner) {
        double wt = 1.0;
        size_t off = (size_t)R * d, stride = 1;
        for (int j = d - 1; j >= 0; --j) {
            int b = (corner >> j) & 1;
            wt *= b ? w[j] : 1.0 - w[j];
            off += (size_t)(lo[j] + b) * stride;
            stride *= R;
        }
        acc += wt * S[off];
    }
    return acc;
}

static double utility(const double* S, const double* p, int d, int R) {
    int lowerIdx[MAXD], rpow[MAXD + 1];
    double coeffs[1 << (MAXD - 1)];
    const double eps = 2.220446049250313e-16;
    for (int ii = 0; ii < d; ++ii) {
        double lv = S[ii * R], uv = S[(ii + 1) * R - 1];
        int li = (int)((R - 1) * (p[ii] - lv) / (uv - lv));
        if (li < 0) li = 0;
        else if (li >= R - 1) li = R - 2;
        lowerIdx[ii] = li;
    }
    rpow[0] = 1;
    for (int q = 1; q <= d; ++q) rpow[q] = rpow[q - 1] * R;
    double x0 = S[lowerIdx[0]], x1 = S[lowerIdx[0] + 1];
    double xd = (fabs(x1 - x0) < eps || x0 == x1) ? 0.0 : (p[0] - x0) / (x1 - x0);
    for (int ii = 0; ii < (1 << (d - 1)); ++ii) {
        int idxL = d * R, div = ii;
        for (int jj = 0; jj < d - 1; ++jj) {
            int rem = div - 2 * (div / 2);
            div = div / 2;
            idxL += (rem == 0 ? lowerIdx[d - 2 - jj] : lowerIdx[d - 2 - jj] + 1) * rpow[jj + 1];
        }
        idxL += lowerIdx[d - 1];
        coeffs[ii] = S[idxL] * (1 - xd) + S[idxL + 1] * xd;
    }
    for (int ii = 1; ii < d; ++ii) {
        x0 = S[lowerIdx[ii] + R * ii];
        x1 = S[lowerIdx[ii] + 1 + R * ii];
        xd = (fabs(x1 - x0) < eps || x0 == x1) ? 0.0 : (p[d - ii] - x0) / (x1 - x0);
        for (int jj = 0; jj < (1 << (d - 1 - ii)); ++jj)
            coeffs[jj] = coeffs[jj * 2] * (1 - xd) + coeffs[jj * 2 + 1] * xd;
    }
    return coeffs[0];
}

void or_interpolate_surrogate(int n, int d, int R, const double* S, const double* P, double* out,
                              int mode, float* fS, float* fP) {
    if (mode == 0) {
        size_t ns = (size_t)R * d + (size_t)pow((double)R, d), np = (size_t)n * d;
        for (size_t i = 0; i < ns; ++i) fS[i] = (float)S[i];
        for (size_t i = 0; i < np; ++i) fP[i] = (float)P[i];
        for (int i = 0; i < n; ++i) out[i] = (double)ref_kernel(i, d, R, fS, fP);
    } else {
        for (int i = 0; i < n; ++i)
            out[i] = mode == 1 ? multilinear(S, P + (size_t)i * d, d, R)
                               : utility(S, P + (size_t)i * d, d, R);
    }
}
