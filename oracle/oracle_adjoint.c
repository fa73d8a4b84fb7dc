/*
 * oracle_adjoint.c - FP64 restatement of the frozen-policy controlled road
 * valuation whose pathwise sensitivities transportoptimiser_gb300/csrc/
 * adjoint.cu computes (test infrastructure).  Same model, same Philox
 * streams (to_math.h), every value after the random draws in double, so its
 * central finite differences are the FP64 reference gradient.
 *
 *   U_{t+1} = U_t + theta (mu - U_t) dt + U_t sigma z + (e^j - 1) U_t J
 *             (forwardPathKernel, SimulateGPU.cu:930-952)
 *   pi_t = (unit_cost + sum_f fuel_f U_f - revenue sum_c ore_c U_{nF+c}) U_demand
 *   PV = sum_t (1 + rrr dt / 100)^-t flows[c_t] pi_t
 *   g: growth-rate mean recursion (mteKernel, SimulateGPU.cu:691-701)
 *   x_{t+1}[k] = max(m (1 + gr (cap - m) / cap), 0), m = M_{c_t}(h) x_t,
 *   gr = g (1 + v z); E_s = sum_k x_Y[k]
 */
#include "oracle_adjoint.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "../transportoptimiser_gb300/csrc/to_math.h"

typedef struct {
    const or_adj_problem* pr;
    const double* theta;
    int p0, p1;
    double sum[16];
    /* per species, per control: COO of the matrix at theta's hazards */
    int** ck; int** cl; double** cv; int* cn;
} job_t;

static double path_pv(const or_adj_problem* a, const double* th, int p) {
    double U[8];
    for (int u = 0; u < a->U; ++u) U[u] = a->uncert[6 * u];
    double pv = 0.0, disc = 1.0;
    const double dfac = 1.0 / (1.0 + (double)a->rrr * a->dt / 100.0);
    for (int t = 0; t < a->Y; ++t) {
        double uf = 0.0, ore = 0.0;
        for (int f = 0; f < a->nF; ++f) uf += (double)a->fuel_costs[f] * U[a->fuel_idx[f]];
        for (int c = 0; c < a->Cm; ++c) {
            const long fi = (long)c * a->Y * a->P + (long)p * a->Y + t;
            const float z = to_normal1(a->seed, TO_STREAM_ORE, (uint32_t)a->road, (uint32_t)(fi >> 2), 0,
                                       (uint32_t)(fi & 3));
            ore += ((double)a->ore_content[c] + (double)a->ore_sd[c] * z) * U[a->nF + c];
        }
        double pi = ((double)a->unit_cost + uf) - (double)a->unit_revenue * ore;
        if (a->demand_idx >= 0) pi *= U[a->demand_idx];
        pv += disc * (double)a->flows[a->controls[(size_t)t * a->P + p]] * pi;
        for (int u = 0; u < a->U; ++u) {
            const float* up = a->uncert + 6 * u;
            const float uj = to_uniform1(a->seed, TO_STREAM_EX_JUMP, (uint32_t)a->road, p, t, u);
            const float zb = to_normal1(a->seed, TO_STREAM_EX_BROWNIAN, (uint32_t)a->road, p, t, u);
            const float zj = to_normal1(a->seed, TO_STREAM_EX_JUMPSIZE, (uint32_t)a->road, p, t, u);
            const double jump = (uj < up[5]) ? 1.0 : 0.0;
            const double s4 = (double)up[4] * up[4];
            const double jf = (exp((double)zj * up[4] - s4 / 2.0) - 1.0) * jump;
            const double cur = U[u];
            U[u] = cur + th[u] * ((double)up[1] - cur) * a->dt + cur * ((double)zb * th[a->U + u]) + jf * cur;
        }
        disc *= dfac;
    }
    return pv;
}

static double path_end(const job_t* j, int s, int p, double* x, double* m) {
    const or_adj_problem* a = j->pr;
    const double* th = j->theta;
    const int N = a->n_patches[s], NP = a->NP;
    const float* sp = a->params + 8 * s;
    const double mu = th[2 * a->U + s], v = th[2 * a->U + a->S + s];
    const int N4 = (N + 3) & ~3;
    for (int k = 0; k < N; ++k) x[k] = a->init_pops[(size_t)s * NP + k];
    double g = sp[0];
    for (int t = 0; t < a->Y; ++t) {
        const float uj = to_uniform1(a->seed, TO_STREAM_SP_JUMP, (uint32_t)a->road, p, t, s);
        const float zb = to_normal1(a->seed, TO_STREAM_SP_BROWNIAN, (uint32_t)a->road, p, t, s);
        const float zj = to_normal1(a->seed, TO_STREAM_SP_JUMPSIZE, (uint32_t)a->road, p, t, s);
        const double jump = (uj < sp[6]) ? 1.0 : 0.0;
        const double s5 = (double)sp[5] * sp[5];
        const double jf = (exp((double)zj * sp[5] - s5 / 2.0) - 1.0) * jump;
        g = g + sp[4] * (mu - g) * a->dt + g * ((double)zb * sp[2]) + jf * g;
        const int c = a->controls[(size_t)t * a->P + p];
        const int mi = s * a->C + c;
        for (int k = 0; k < N; ++k) m[k] = 0.0;
        for (int e = 0; e < j->cn[mi]; ++e) m[j->ck[mi][e]] += j->cv[mi][e] * x[j->cl[mi][e]];
        for (int k = 0; k < N; ++k) {
            float z4[4];
            to_normal4(a->seed, TO_STREAM_GROWTH, (uint32_t)a->road, (uint32_t)p, t,
                       (uint32_t)((s * N4) >> 2) + (uint32_t)(k >> 2), z4);
            const double gr = g * (1.0 + v * z4[k & 3]);
            const double cap = a->caps[(size_t)s * NP + k];
            const double f = m[k] * (1.0 + gr * (cap - m[k]) / cap);
            x[k] = f > 0.0 ? f : 0.0;
        }
    }
    double e = 0.0;
    for (int k = 0; k < N; ++k) e += x[k];
    return e;
}

static void* run(void* arg) {
    job_t* j = (job_t*)arg;
    const or_adj_problem* a = j->pr;
    double* x = (double*)malloc(sizeof(double) * a->NP);
    double* m = (double*)malloc(sizeof(double) * a->NP);
    for (int i = 0; i < 1 + a->S; ++i) j->sum[i] = 0.0;
    for (int p = j->p0; p < j->p1; ++p) {
        j->sum[0] += path_pv(a, j->theta, p);
        for (int s = 0; s < a->S; ++s) j->sum[1 + s] += path_end(j, s, p, x, m);
    }
    free(x);
    free(m);
    return NULL;
}

void or_adjoint_forward(const or_adj_problem* a, const double* theta, double* outputs,
                        int threads) {
    const int NM = a->S * a->C;
    int** ck = (int**)calloc(NM, sizeof(int*));
    int** cl = (int**)calloc(NM, sizeof(int*));
    double** cv = (double**)calloc(NM, sizeof(double*));
    int* cn = (int*)calloc(NM, sizeof(int));
    for (int s = 0; s < a->S; ++s) {
        const int N = a->n_patches[s], NP = a->NP;
        for (int c = 0; c < a->C; ++c) {
            const int mi = s * a->C + c;
            const float* M = a->mmm + ((size_t)s * a->C + c) * NP * NP;
            int n = 0;
            for (int k = 0; k < N; ++k)
                for (int l = 0; l < N; ++l) n += (M[(size_t)k * NP + l] != 0.0f);
            ck[mi] = (int*)malloc(sizeof(int) * (n + 1));
            cl[mi] = (int*)malloc(sizeof(int) * (n + 1));
            cv[mi] = (double*)malloc(sizeof(double) * (n + 1));
            const double dh = theta[2 * a->U + 2 * a->S + c] - a->base_h[c];
            n = 0;
            for (int k = 0; k < N; ++k)
                for (int l = 0; l < N; ++l) {
                    const float v = M[(size_t)k * NP + l];
                    if (v == 0.0f) continue;
                    const int xc = a->cross[((size_t)s * NP + l) * NP + k];
                    ck[mi][n] = k;
                    cl[mi][n] = l;
                    cv[mi][n] = (double)v * exp(-(double)xc * dh);
                    ++n;
                }
            cn[mi] = n;
        }
    }
    if (threads < 1) threads = 1;
    job_t* jobs = (job_t*)calloc(threads, sizeof(job_t));
    pthread_t* tid = (pthread_t*)calloc(threads, sizeof(pthread_t));
    for (int i = 0; i < threads; ++i) {
        jobs[i].pr = a; jobs[i].theta = theta;
        jobs[i].p0 = (int)((long)a->P * i / threads);
        jobs[i].p1 = (int)((long)a->P * (i + 1) / threads);
        jobs[i].ck = ck; jobs[i].cl = cl; jobs[i].cv = cv; jobs[i].cn = cn;
        pthread_create(&tid[i], NULL, run, &jobs[i]);
    }
    for (int i = 0; i < 1 + a->S; ++i) outputs[i] = 0.0;
    for (int i = 0; i < threads; ++i) {
        pthread_join(tid[i], NULL);
        for (int q = 0; q < 1 + a->S; ++q) outputs[q] += jobs[i].sum[q];
    }
    for (int q = 0; q < 1 + a->S; ++q) outputs[q] /= (double)a->P;
    for (int mi = 0; mi < NM; ++mi) { free(ck[mi]); free(cl[mi]); free(cv[mi]); }
    free(ck); free(cl); free(cv); free(cn); free(jobs); free(tid);
}
