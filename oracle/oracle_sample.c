/*
 * oracle_sample.c - CPU restatement of RoadGA::generateSample
 * (include/main/RoadGA.cpp:3288-3462) with its distance matrices
 * (knn_cuda_with_indexes.cu:188-325: projected distance = smallest
 * coordinate difference starting from 100; Euclidean distance), recomputed
 * from scratch every step as the reference does (test infrastructure for
 * transportoptimiser_gb300/csrc/sample.cu).  Euclidean distances as
 * sqrtf(sum t*t) where the reference calls pow.
 */
#include "oracle_sample.h"

#include <math.h>
#include <stdlib.h>

static void dist2(const float* a, const float* b, int d, float* dp, float* d2) {
    float mn = 100.0f, ss = 0.0f;
    for (int k = 0; k < d; ++k) {
        float t = fabsf(a[k] - b[k]);
        mn = fminf(mn, t);
        ss = ss + t * t;
    }
    *dp = mn;
    *d2 = sqrtf(ss);
}

void or_select_samples(int n_cur, const double* cur, int nc, const double* cand, int d, int n,
                       int* sample) {
    float* cf = (float*)malloc(sizeof(float) * (size_t)nc * d);
    float* sf = (float*)malloc(sizeof(float) * (size_t)(n_cur + n + 2) * d);
    for (int k = 0; k < d; ++k) {
        double lo = INFINITY, hi = -INFINITY;
        for (int i = 0; i < n_cur; ++i) { lo = fmin(lo, cur[i * d + k]); hi = fmax(hi, cur[i * d + k]); }
        for (int j = 0; j < nc; ++j) { lo = fmin(lo, cand[j * d + k]); hi = fmax(hi, cand[j * d + k]); }
        for (int j = 0; j < nc; ++j) cf[(size_t)j * d + k] = (float)((cand[j * d + k] - lo) / (hi - lo));
        for (int i = 0; i < n_cur; ++i) sf[(size_t)i * d + k] = (float)((cur[i * d + k] - lo) / (hi - lo));
    }
    int ns = n_cur, step0 = 0;
    if (n_cur == 0) {
        float maxd = 0.0f;
        int p1 = 0, p2 = 0;
        for (int ii = 0; ii < nc; ++ii)
            for (int jj = 0; jj < nc; ++jj) {
                float dp, d2;
                dist2(cf + (size_t)ii * d, cf + (size_t)jj * d, d, &dp, &d2);
                if (dp > maxd) { p1 = ii; p2 = jj; maxd = dp; }
            }
        sample[0] = p1;
        sample[1] = p2;
        for (int k = 0; k < d; ++k) { sf[k] = cf[(size_t)p1 * d + k]; sf[d + k] = cf[(size_t)p2 * d + k]; }
        ns = 2;
        step0 = 2;
    }
    float* mi = (float*)malloc(sizeof(float) * nc);
    float* m2 = (float*)malloc(sizeof(float) * nc);
    for (int step = step0; step < n; ++step) {
        for (int j = 0; j < nc; ++j) {
            float a = INFINITY, b = INFINITY;
            for (int i = 0; i < ns; ++i) {
                float dp, dd;
                dist2(cf + (size_t)j * d, sf + (size_t)i * d, d, &dp, &dd);
                a = fminf(a, dp);
                b = fminf(b, dd);
            }
            mi[j] = a;
            m2[j] = b;
        }
        float dmin = 2.0f * 0.5f / (float)ns;
        float best = 0.0f;
        int pick = 0;
        for (int j = 0; j < nc; ++j)
            if (mi[j] >= dmin && m2[j] > best) { pick = j; best = m2[j]; }
        const double cd = (d == 1) ? ((double)(ns + 1) - 1.0) / 2.0 : 0.0;
        const int ch = (ns + 1) / 2;
        for (int j = 0; j < nc; ++j) {
            float val = (float)(cd * (double)m2[j] + (double)((float)ch * mi[j]));
            if (val > best) { pick = j; best = val; }
        }
        sample[step] = pick;
        for (int k = 0; k < d; ++k) sf[(size_t)ns * d + k] = cf[(size_t)pick * d + k];
        ++ns;
    }
    free(cf); free(sf); free(mi); free(m2);
}
