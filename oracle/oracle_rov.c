/*
 * oracle_rov.c - CPU restatement of the reference's controlled-traffic
 * real-options valuation (ALGO4: forward paths under random controls, then
 * regression Monte Carlo backward induction with multiple local linear
 * regression on k nearest neighbours), and of the surrogate builders.
 * TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Reference (TransportOptimiser, include/gpuCode/):
 *   SimulateGPU::simulateROVCUDA        SimulateGPU.cu:3870-5003 (ALGO4)
 *   randControls                        SimulateGPU.cu:720-730
 *   forwardPathKernel                   SimulateGPU.cu:789-956
 *   computePathStates                   SimulateGPU.cu:959-1008
 *   allocateXYRegressionData            SimulateGPU.cu:1012-1069
 *   computeStateMinMax                  SimulateGPU.cu:1073-1148
 *   createQueryPoints                   SimulateGPU.cu:1152-1195
 *   firstPeriodInduction                SimulateGPU.cu:2210-2330
 *   backwardInduction                   SimulateGPU.cu:2333-2784
 *   multiLocLinReg, solveLinearSystem   SimulateGPU.cu:2934-3053, 129-190
 *   knn_cuda_with_indexes::knn          knn_cuda_with_indexes.cu:475-618
 *   buildSurrogateMTECUDA / ROVCUDA     SimulateGPU.cu:5533-5917
 *
 * The normal equations are accumulated in FP32 as in the reference and
 * solved by FP64 square-root-free Cholesky (the reference: FP32 Gaussian
 * elimination); the kNN selection is "k smallest by (squared distance,
 * index)", which is what the reference's stable insertion sort returns.
 * The ROV regressions sum the k nearest in ascending point index over 32
 * lane partials added in lane order (the device's order; the reference
 * sums them one by one in distance order).
 */
#include "oracle_rov.h"
#include "oracle.h"
#include "../transportoptimiser_gb300/csrc/to_math.h"
#include "../transportoptimiser_gb300/csrc/to_lsm_math.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* kNN: k smallest squared distances by (value, index); dist = sqrt, ind is  */
/* 1-based; layout [kk*Q + q] as the reference returns it.                   */
/* ------------------------------------------------------------------------ */
typedef struct { float key; int idx; } knn_item;

static void knn_one(const float* ref, int n, const float* q, int dim, int k,
                    knn_item* best) {
    int m = 0;
    for (int i = 0; i < n; ++i) {
        float s = 0.0f;
        for (int j = 0; j < dim; ++j) {
            float t = ref[(size_t)j * n + i] - q[j];
            s = fmaf(t, t, s);
        }
        if (m < k) {
            int pos = m;
            while (pos > 0 && (best[pos - 1].key > s)) { best[pos] = best[pos - 1]; --pos; }
            best[pos].key = s; best[pos].idx = i;
            ++m;
        } else if (s < best[k - 1].key) {
            int pos = k - 1;
            while (pos > 0 && best[pos - 1].key > s) { best[pos] = best[pos - 1]; --pos; }
            best[pos].key = s; best[pos].idx = i;
        }
    }
}

void or_knn(const float* ref, int n, const float* query, int Q, int dim, int k,
            float* dist, int* ind) {
    knn_item* best = (knn_item*)malloc(sizeof(knn_item) * (size_t)(k > 0 ? k : 1));
    float q[8];
    for (int qi = 0; qi < Q; ++qi) {
        for (int j = 0; j < dim; ++j) q[j] = query[(size_t)j * Q + qi];
        knn_one(ref, n, q, dim, k, best);
        for (int kk = 0; kk < k; ++kk) {
            dist[(size_t)kk * Q + qi] = sqrtf(best[kk].key);
            ind[(size_t)kk * Q + qi] = best[kk].idx + 1;
        }
    }
    free(best);
}

/* ------------------------------------------------------------------------ */
/* multiLocLinReg at one query (SimulateGPU.cu:2942-3052).                   */
/* xraw(i, j): x of neighbour i in dimension j as the kernel reads it.       */
/* lanes = 1: neighbours summed in distance order (surrogate builders).     */
/* lanes = 32: the k nearest in ascending point index, neighbour m of that  */
/* order to partial sum m % 32, and the 32 partial sums added in lane      */
/* order, ((s0 + s1) + s2) + ... + s31, as the device gathers and reduces  */
/* them.                                                                   */
/* ------------------------------------------------------------------------ */
static float local_linear(int dim, int k, int Q, int qi, const float* dist,
                          const int* ind, const float* y, const float* xbuf,
                          int n, int pointmajor, const float* xq, int lanes) {
    enum { ACC = TO_LSM_MAXD + 1 + (TO_LSM_MAXD + 1) * (TO_LSM_MAXD + 1) };
    float acc[32][ACC];
    const int na = (dim + 1) + (dim + 1) * (dim + 1);
    for (int l = 0; l < lanes; ++l) to_lsm_acc_init(dim, acc[l]);
    float h = dist[(size_t)(k - 1) * Q + qi];
    /* the order of the sum: lanes = 1 by distance, lanes = 32 by ascending
     * point index */
    int* ord = (int*)malloc(sizeof(int) * (size_t)k);
    for (int m = 0; m < k; ++m) {
        int v = m, j = m;
        const int key = ind[(size_t)m * Q + qi];
        if (lanes > 1)
            for (; j > 0 && ind[(size_t)ord[j - 1] * Q + qi] > key; --j) ord[j] = ord[j - 1];
        ord[j] = v;
    }
    for (int m = 0; m < k; ++m) {
        const int kk = ord[m];
        float d = dist[(size_t)kk * Q + qi];
        int i = ind[(size_t)kk * Q + qi] - 1;
        float xv[TO_LSM_MAXD];
        for (int j = 0; j < dim; ++j)
            xv[j] = pointmajor ? xbuf[(size_t)i * dim + j] : xbuf[(size_t)j * n + i];
        to_lsm_acc_add(dim, acc[m % lanes], to_lsm_weight(d, h), y[i], xv, xq);
    }
    free(ord);
    for (int e = 0; e < na; ++e) {
        float s = acc[0][e];
        for (int l = 1; l < lanes; ++l) s = s + acc[l][e];
        acc[0][e] = s;
    }
    return to_lsm_solve_intercept(dim, acc[0]);
}

/* The regressions of one (year, control) at the grid queries q0 .. q1-1:
 * the query's k nearest points (as or_knn), then its local linear fit.
 * Queries are independent, so any split of them over threads gives the same
 * values (the reference runs its kNN one thread per query). */
typedef struct {
    int q0, q1, d, k, Q, n, sem;
    const float *xn, *xr, *qn, *xqg, *y;
    float* dist;
    int* ind;
    float* yout;
} reg_job;

static void reg_queries(const reg_job* j) {
    knn_item* best = (knn_item*)malloc(sizeof(knn_item) * (size_t)(j->k > 0 ? j->k : 1));
    float q[8], xq[TO_LSM_MAXD];
    for (int qi = j->q0; qi < j->q1; ++qi) {
        for (int jj = 0; jj < j->d; ++jj) q[jj] = j->qn[(size_t)jj * j->Q + qi];
        knn_one(j->xn, j->n, q, j->d, j->k, best);
        for (int kk = 0; kk < j->k; ++kk) {
            j->dist[(size_t)kk * j->Q + qi] = sqrtf(best[kk].key);
            j->ind[(size_t)kk * j->Q + qi] = best[kk].idx + 1;
        }
        for (int jj = 0; jj < j->d; ++jj) xq[jj] = j->xqg[(size_t)jj * j->Q + qi];
        j->yout[qi] = (j->sem == 0)
            ? local_linear(j->d, j->k, j->Q, qi, j->dist, j->ind, j->y, j->xr, j->n, 1, xq, 32)
            : local_linear(j->d, j->k, j->Q, qi, j->dist, j->ind, j->y, j->xn, j->n, 0, xq, 32);
    }
    free(best);
}

static void* reg_thread(void* a) { reg_queries((const reg_job*)a); return NULL; }

static void reg_all_queries(reg_job base, int threads) {
    if (threads < 1) threads = 1;
    if (threads > 128) threads = 128;
    reg_job jobs[128];
    pthread_t th[128];
    const int per = (base.Q + threads - 1) / threads;
    int used = 0;
    for (int i = 0; i < threads; ++i) {
        reg_job jj = base;
        jj.q0 = i * per;
        jj.q1 = jj.q0 + per > base.Q ? base.Q : jj.q0 + per;
        if (jj.q0 >= jj.q1) break;
        jobs[used++] = jj;
    }
    for (int i = 1; i < used; ++i) pthread_create(&th[i], NULL, reg_thread, &jobs[i]);
    if (used > 0) reg_queries(&jobs[0]);
    for (int i = 1; i < used; ++i) pthread_join(th[i], NULL);
}

/* k rule of the ALGO4 loop (SimulateGPU.cu:4542-4545); 0 when n <= 3, and
 * never more than n (the reference reads past the data then). */
int or_k_rov_mult(int n, int mult) {
    if (n <= 3) return 0;
    int k = (int)((double)mult * (log((double)n) + 1.0));
    return k < n ? k : n;
}

/* k nearest neighbours of the ALGO4 regressions (SimulateGPU.cu:4517);
 * ALGO6 uses 3 (ln n + 1) (its host loop, SimulateGPU.cu:5110) */
int or_k_rov(int n) { return or_k_rov_mult(n, 10); }

/* ------------------------------------------------------------------------ */
/* ROV                                                                        */
/* ------------------------------------------------------------------------ */
/* compressed columns of one (species, control) migration matrix
 * (dense2Sparse, SimulateGPU.cu:5973-5996): forwardPathKernel walks these
 * lists (SimulateGPU.cu:871-922); skipped entries are exact zeros, so the
 * fmaf chain over a list has the bits of the chain over the dense row */
typedef struct {
    int* ptr;
    int* idx;
    float* val;
} rov_csc;

static void csc_migrate(const rov_csc* m, int N, const float* x, float* out) {
    for (int k = 0; k < N; ++k) {
        float a = 0.0f;
        for (int e = m->ptr[k]; e < m->ptr[k + 1]; ++e) a = fmaf(x[m->idx[e]], m->val[e], a);
        out[k] = a;
    }
}

typedef struct {
    const or_rov_problem* pr;
    const rov_csc* csc; /* [S*C] */
    int p0, p1;
    float* totalPops;   /* [P][Y+1][S] */
    float* aars;        /* [P][Y+1][S][C] */
    float* uRes;        /* [P][Y+1][U] (reference stride) */
    int* controls;      /* [P][Y] */
    float* popY;        /* ALGO6: [P][Y][S][maxN] patch populations, start of year */
    float* gmY;         /* ALGO6: [P][Y][S] mean growth rate of the year */
    int maxN;
} rov_fwd_job;

static void rov_forward_paths(rov_fwd_job* j) {
    const or_rov_problem* pr = j->pr;
    const int P = pr->n_paths, Y = pr->n_years, S = pr->n_species, C = pr->n_controls,
              U = pr->n_uncertainties;
    int maxN = 0;
    for (int s = 0; s < S; ++s) if (pr->n_patches[s] > maxN) maxN = pr->n_patches[s];
    float* pop = (float*)malloc(sizeof(float) * (size_t)S * maxN);
    float* npop = (float*)malloc(sizeof(float) * (size_t)maxN);
    float* mig = (float*)malloc(sizeof(float) * (size_t)maxN);
    float gm[8];
    (void)P;
    for (int p = j->p0; p < j->p1; ++p) {
        for (int s = 0; s < S; ++s) {
            int N = pr->n_patches[s];
            for (int k = 0; k < N; ++k) pop[(size_t)s * maxN + k] = pr->init_pops[s][k];
            j->totalPops[((size_t)p * (Y + 1) + 0) * S + s] = or_grouped_sum(pr->init_pops[s], N);
            gm[s] = pr->params[s][0];
        }
        for (int u = 0; u < U; ++u)
            j->uRes[((size_t)p * (Y + 1) + 0) * U + u] = pr->uncert[6 * u + 0];
        for (int t = 0; t < Y; ++t) {
            float uc = to_uniform1(pr->seed, TO_STREAM_CONTROL, pr->road, p, t, 0);
            int control = (int)(uc * (float)C);
            if (control == C) control--;
            j->controls[(size_t)p * Y + t] = control;
            for (int s = 0; s < S; ++s) {
                const float* sp = pr->params[s];
                int N = pr->n_patches[s];
                int N4 = (N + 3) & ~3;
                float* ps = pop + (size_t)s * maxN;
                float uj = to_uniform1(pr->seed, TO_STREAM_SP_JUMP, pr->road, p, t, s);
                float zb = to_normal1(pr->seed, TO_STREAM_SP_BROWNIAN, pr->road, p, t, s);
                float zj = to_normal1(pr->seed, TO_STREAM_SP_JUMPSIZE, pr->road, p, t, s);
                float jp = (pr->sem == 0) ? sp[5] : sp[6];
                float jump = (uj < jp) ? 1.0f : 0.0f;
                float brown = zb * sp[2];
                float s5 = sp[5] * sp[5];
                float jsz = (pr->sem == 0) ? (zj * s5 - s5 / 2.0f) : (zj * sp[5] - s5 / 2.0f);
                gm[s] = gm[s] + sp[4] * (sp[1] - gm[s]) * pr->dt + gm[s] * brown
                        + (to_expf(jsz) - 1.0f) * gm[s] * jump;
                if (j->popY) {
                    memcpy(j->popY + (((size_t)p * Y + t) * S + s) * j->maxN, ps,
                           sizeof(float) * (size_t)N);
                    j->gmY[((size_t)p * Y + t) * S + s] = gm[s];
                }
                float initial = or_grouped_sum(ps, N);
                for (int c = 0; c < C; ++c) {
                    csc_migrate(&j->csc[s * C + c], N, ps, mig);
                    float totc = or_grouped_sum(mig, N);
                    if (c == control) {
                        for (int k0 = 0; k0 < N; k0 += 4) {
                            float z4[4];
                            to_normal4(pr->seed, TO_STREAM_GROWTH, pr->road, p, t,
                                       (uint32_t)((s * N4 + k0) >> 2), z4);
                            for (int q = 0; q < 4 && k0 + q < N; ++q) {
                                const int k = k0 + q;
                                const float z = z4[q];
                                /* Q25: the reference adds the local variability
                                 * (gr = gm + z p7); sem 1 scales it by the mean
                                 * as the MTE kernel does and keeps pops >= 0 */
                                float gr = (pr->sem == 0) ? gm[s] + z * sp[7]
                                                          : fmaf(sp[7] * z, gm[s], gm[s]);
                                float m = mig[k], cp = pr->caps[s][k];
                                float v = (pr->sem == 0)
                                    ? m * (1.0f + gr * (cp - m) / cp / 100.0f)
                                    : fmaxf(m * (1.0f + gr * (cp - m) / cp), 0.0f);
                                npop[k] = v;
                            }
                        }
                    }
                    j->aars[(((size_t)p * (Y + 1) + t) * S + s) * C + c] = totc / initial;
                }
                memcpy(ps, npop, sizeof(float) * (size_t)N);
                j->totalPops[((size_t)p * (Y + 1) + t + 1) * S + s] = or_grouped_sum(ps, N);
            }
            for (int u = 0; u < U; ++u) {
                const float* up = pr->uncert + 6 * u;
                float uj = to_uniform1(pr->seed, TO_STREAM_EX_JUMP, pr->road, p, t, u);
                float zb = to_normal1(pr->seed, TO_STREAM_EX_BROWNIAN, pr->road, p, t, u);
                float zj = to_normal1(pr->seed, TO_STREAM_EX_JUMPSIZE, pr->road, p, t, u);
                float jump = (uj < up[5]) ? 1.0f : 0.0f;
                float curr = j->uRes[((size_t)p * (Y + 1) + t) * U + u];
                float brown = zb * up[2];
                float s4 = up[4] * up[4];
                float jsz = (pr->sem == 0) ? (zj * s4 - s4 / 2.0f) : (zj * up[4] - s4 / 2.0f);
                j->uRes[((size_t)p * (Y + 1) + t + 1) * U + u] =
                    curr + up[3] * (up[1] - curr) * pr->dt + curr * brown
                    + (to_expf(jsz) - 1.0f) * curr * jump;
            }
        }
    }
    free(pop); free(npop); free(mig);
}

static void* rov_fwd_thread(void* a) { rov_forward_paths((rov_fwd_job*)a); return NULL; }

/* ore composition as the reference reads it (SimulateGPU.cu:4246-4251 fills
 * commodity-major, the kernels read path-major) */
static float ore_at(const or_rov_problem* pr, int p, int t, int c) {
    int P = pr->n_paths, Y = pr->n_years, Cm = pr->n_commodities;
    long f, gen;
    if (pr->sem == 0) {
        f = ((long)p * Y + t) * Cm + c;
        gen = f / ((long)Y * P);
    } else {
        gen = c;
        f = (long)c * Y * P + (long)p * Y + t;
    }
    float z = to_normal1(pr->seed, TO_STREAM_ORE, pr->road, (uint32_t)(f >> 2), 0,
                         (uint32_t)(f & 3));
    return pr->ore_content[gen] + pr->ore_sd[gen] * z;
}

/* unit profit at (path, year): unitCost + fuel - revenue * ore price, with
 * the reference's two uResults strides (Q5: `stride_y` is Y+1 or Y) */
static float unit_profit(const or_rov_problem* pr, const float* uRes, int p, int t,
                         int fuel_stride_y, int ore_stride_y) {
    int U = pr->n_uncertainties, nF = pr->n_fuels;
    float uf = 0.0f, ore = 0.0f;
    for (int f = 0; f < nF; ++f)
        uf = fmaf(pr->fuel_costs[f], uRes[((size_t)p * fuel_stride_y + t) * U + pr->fuel_idx[f]], uf);
    for (int c = 0; c < pr->n_commodities; ++c)
        ore = fmaf(ore_at(pr, p, t, c), uRes[((size_t)p * ore_stride_y + t) * U + nF + c], ore);
    float prof = (pr->unit_cost + uf) - pr->unit_revenue * ore;
    if (pr->demand_idx >= 0)
        prof = prof * uRes[((size_t)p * (pr->n_years + 1) + t) * U + pr->demand_idx];
    return prof;
}


/* ALGO6 decisions, the same rules as the backward induction below
 * (SimulateGPU.cu:2375-2463 terminal, :2464-2776 interior); state holds the
 * adjusted populations [C][S] and the unit profit at [S*C] */
static void rov_decide(const or_rov_problem* pr, const float* reg, long blk, int t,
                       int terminal, const float* state, float* best_out, int* bc_out) {
    const int S = pr->n_species, C = pr->n_controls, R = pr->dim_res;
    const float disc = 1.0f + pr->rrr * pr->dt / 100.0f;
    float pay[TO_MAX_C_ORACLE];
    int valid[TO_MAX_C_ORACLE];
    for (int c = 0; c < C; ++c) {
        valid[c] = 1;
        for (int s = 0; s < S; ++s) {
            float thr = (pr->sem == 0) ? pr->params_flat[S * s + 3] : pr->params[s][3];
            if (state[c * S + s] < thr && c > 0) { valid[c] = 0; break; }
        }
        if (!valid[c]) { pay[c] = 0.0f; continue; }
        if (terminal) {
            float v = pr->flows[c] * state[S * C];
            pay[c] = v > 0.0f ? 0.0f : v;
        } else {
            float cur = pr->flows[c] * state[S * C];
            const float* rb = reg + (size_t)t * C * blk + (size_t)c * blk;
            float v = (pr->sem == 0) ? to_lsm_interp_ref(rb, R, S, C, state)
                                     : to_lsm_interp(rb, R, S, state + c * S, state[S * C]);
            double ce = (double)(v / disc);
            if (ce > 0.0) ce = 0.0;
            pay[c] = (float)((double)cur + ce);
        }
    }
    float best = pay[0];
    int bc = 0;
    for (int c = 1; c < C; ++c) {
        if (!valid[c]) continue;
        int better = terminal ? (pay[c] < best)
                   : (pr->sem == 0 ? ((double)pay[c] < 0.975 * (double)best) : (pay[c] < best));
        if (better) { best = pay[c]; bc = c; }
    }
    *best_out = best;
    *bc_out = bc;
}

typedef struct {
    const or_rov_problem* pr;
    const rov_csc* csc; /* [S*C] */
    int p0, p1, t0, maxN;
    const float* popY;
    const float* gmY;
    const float* uRes;
    const float* reg;
    float* condExp;
    int* opt_cont;
} rov_resim_job;

/* ALGO6 (optimalForwardPaths, SimulateGPU.cu:1199-2206, as its comments
 * describe it): each path restarts from its forward-pass patch populations
 * at year t0, takes the decided control every year (regression of the year,
 * terminal rule in the last), migrates and grows with the forward pass's
 * noise and growth mean; the value is the realised payoff flows[c] * profit
 * discounted by (1 + r dt / 100) per year. */
static void rov_resim_paths(rov_resim_job* j) {
    const or_rov_problem* pr = j->pr;
    const int P = pr->n_paths, Y = pr->n_years, S = pr->n_species, C = pr->n_controls,
              R = pr->dim_res, d = S + 1, Y1 = Y + 1, maxN = j->maxN, t0 = j->t0;
    long Q = 1;
    for (int i = 0; i < d; ++i) Q *= R;
    const long blk = (long)R * d + 2L * Q;
    const float disc = 1.0f + pr->rrr * pr->dt / 100.0f;
    float* x = (float*)malloc(sizeof(float) * (size_t)S * maxN);
    float* mig = (float*)malloc(sizeof(float) * (size_t)S * C * maxN);
    float tot[TO_LSM_MAXD];
    for (int p = j->p0; p < j->p1; ++p) {
        for (int s = 0; s < S; ++s) {
            const int N = pr->n_patches[s];
            memcpy(x + (size_t)s * maxN, j->popY + (((size_t)p * Y + t0) * S + s) * maxN,
                   sizeof(float) * (size_t)N);
            tot[s] = or_grouped_sum(x + (size_t)s * maxN, N);
        }
        float val = 0.0f, df = 1.0f;
        int c0 = 0;
        for (int u = t0; u < Y; ++u) {
            float state[TO_MAX_C_ORACLE * TO_LSM_MAXD + 1];
            for (int s = 0; s < S; ++s) {
                const int N = pr->n_patches[s];
                const float* xs = x + (size_t)s * maxN;
                for (int c = 0; c < C; ++c) {
                    float* mg = mig + ((size_t)s * C + c) * maxN;
                    csc_migrate(&j->csc[s * C + c], N, xs, mg);
                    float tt = or_grouped_sum(mg, N);
                    state[c * S + s] = tot[s] * (tt / tot[s]);
                }
            }
            const float prof = unit_profit(pr, j->uRes, p, u, Y1, Y1);
            state[S * C] = prof;
            float best;
            int bc;
            rov_decide(pr, j->reg, blk, u, u == Y - 1, state, &best, &bc);
            val = val + (pr->flows[bc] * prof) * df;
            df = df / disc;
            if (u == t0) c0 = bc;
            if (u == Y - 1) break;
            for (int s = 0; s < S; ++s) {
                const int N = pr->n_patches[s], N4 = (N + 3) & ~3;
                const float* sp = pr->params[s];
                const float g = j->gmY[((size_t)p * Y + u) * S + s];
                const float* mg = mig + ((size_t)s * C + bc) * maxN;
                float* xs = x + (size_t)s * maxN;
                for (int k0 = 0; k0 < N; k0 += 4) {
                    float z4[4];
                    to_normal4(pr->seed, TO_STREAM_GROWTH, pr->road, p, u,
                               (uint32_t)((s * N4 + k0) >> 2), z4);
                    for (int q = 0; q < 4 && k0 + q < N; ++q) {
                        const int k = k0 + q;
                        const float z = z4[q];
                        float gr = (pr->sem == 0) ? g + z * sp[7] : fmaf(sp[7] * z, g, g);
                        float m = mg[k], cp = pr->caps[s][k];
                        xs[k] = (pr->sem == 0) ? m * (1.0f + gr * (cp - m) / cp / 100.0f)
                                               : fmaxf(m * (1.0f + gr * (cp - m) / cp), 0.0f);
                    }
                }
                tot[s] = or_grouped_sum(xs, N);
            }
        }
        j->condExp[(size_t)t0 * P + p] = val;
        j->opt_cont[(size_t)t0 * P + p] = c0;
    }
    free(x);
    free(mig);
}

static void* rov_resim_thread(void* a) { rov_resim_paths((rov_resim_job*)a); return NULL; }

int or_simulate_rov(const or_rov_problem* pr, or_rov_result* res) {
    const int P = pr->n_paths, Y = pr->n_years, S = pr->n_species, C = pr->n_controls,
              U = pr->n_uncertainties, R = pr->dim_res, d = S + 1;
    if (S < 1 || S > TO_LSM_MAXD - 1 || C < 1 || Y < 2 || P < 1 || R < 2) return -1;
    const int algo = pr->algo == 0 ? 4 : pr->algo;
    if ((algo != 4 && algo != 6) || (algo == 6 && pr->sem != 1)) return -1;
    const int kmult = algo == 6 ? 3 : 10;
    int maxN = 0;
    for (int s = 0; s < S; ++s) if (pr->n_patches[s] > maxN) maxN = pr->n_patches[s];
    float* popY = algo == 6 ? (float*)calloc((size_t)P * Y * S * maxN, sizeof(float)) : NULL;
    float* gmY = algo == 6 ? (float*)calloc((size_t)P * Y * S, sizeof(float)) : NULL;
    long Qn = 1;
    for (int i = 0; i < d; ++i) Qn *= R;
    const int Q = (int)Qn;
    const long blk = (long)R * d + 2L * Q;
    float* totalPops = (float*)calloc((size_t)P * (Y + 1) * S, sizeof(float));
    float* aars = (float*)calloc((size_t)P * (Y + 1) * S * C, sizeof(float));
    float* uRes = (float*)calloc((size_t)P * (Y + 1) * U, sizeof(float));
    int* controls = (int*)calloc((size_t)P * Y, sizeof(int));
    float* condExp = (float*)calloc((size_t)P * Y, sizeof(float));
    float* reg = (float*)calloc((size_t)Y * C * blk, sizeof(float));
    rov_csc* csc = (rov_csc*)calloc((size_t)S * C, sizeof(rov_csc));
    for (int s = 0; s < S; ++s)
        for (int c = 0; c < C; ++c) {
            const int N = pr->n_patches[s];
            const float* M = pr->mmm[s] + (size_t)c * N * N;
            rov_csc* m = &csc[s * C + c];
            m->ptr = (int*)malloc(sizeof(int) * (size_t)(N + 1));
            const int nz = or_pack_csc(N, M, m->ptr, NULL, NULL);
            m->idx = (int*)malloc(sizeof(int) * (size_t)(nz > 0 ? nz : 1));
            m->val = (float*)malloc(sizeof(float) * (size_t)(nz > 0 ? nz : 1));
            or_pack_csc(N, M, m->ptr, m->idx, m->val);
        }

    /* forward paths, parallel over paths */
    int nt = pr->n_threads < 1 ? 1 : (pr->n_threads > 128 ? 128 : pr->n_threads);
    rov_fwd_job jobs[128];
    pthread_t th[128];
    int per = (P + nt - 1) / nt, used = 0;
    for (int i = 0; i < nt; ++i) {
        int a = i * per, b = a + per > P ? P : a + per;
        if (a >= b) break;
        rov_fwd_job jj = {pr, csc, a, b, totalPops, aars, uRes, controls, popY, gmY, maxN};
        jobs[used++] = jj;
    }
    for (int i = 1; i < used; ++i) pthread_create(&th[i], NULL, rov_fwd_thread, &jobs[i]);
    if (used > 0) rov_forward_paths(&jobs[0]);
    for (int i = 1; i < used; ++i) pthread_join(th[i], NULL);

    const int Y1 = Y + 1;
    const int sY_ore = (pr->sem == 0) ? Y : Y1;          /* Q5 */
    const float disc = 1.0f + pr->rrr * pr->dt / 100.0f;

    /* terminal year (SimulateGPU.cu:2375-2463) */
    {
        int t = Y - 1;
        for (int p = 0; p < P; ++p) {
            float prof = unit_profit(pr, uRes, p, t, Y1, sY_ore);
            float pay[TO_MAX_C_ORACLE];
            int valid[TO_MAX_C_ORACLE];
            for (int c = 0; c < C; ++c) {
                valid[c] = 1;
                for (int s = 0; s < S; ++s) {
                    float adj = totalPops[((size_t)p * Y1 + t) * S + s] *
                                aars[(((size_t)p * Y1 + t) * S + s) * C + c];
                    float thr = (pr->sem == 0) ? pr->params_flat[S * s + 3] : pr->params[s][3];
                    if (adj < thr && c > 0) { valid[c] = 0; break; }
                }
                if (valid[c]) {
                    float v = pr->flows[c] * prof;
                    pay[c] = v > 0.0f ? 0.0f : v;
                } else pay[c] = 0.0f;
            }
            float best = pay[0];
            int bc = 0;
            for (int c = 1; c < C; ++c)
                if (valid[c] && pay[c] < best) { best = pay[c]; bc = c; }
            condExp[(size_t)t * P + p] = best;
            res->opt_cont[(size_t)t * P + p] = bc;
            res->unit_profits[(size_t)t * P + p] = prof;
            for (int s = 0; s < S; ++s)
                res->adj_pops[((size_t)t * S + s) * P + p] =
                    totalPops[((size_t)p * Y1 + t) * S + s] *
                    aars[(((size_t)p * Y1 + t) * S + s) * C + (C - 1)];
        }
    }

    /* backward induction (SimulateGPU.cu:4437-4981) */
    float* xin = (float*)malloc(sizeof(float) * (size_t)P * d);
    float* xraw = (float*)malloc(sizeof(float) * (size_t)C * d * P);
    float* xnorm = (float*)malloc(sizeof(float) * (size_t)C * d * P);
    float* yv = (float*)malloc(sizeof(float) * (size_t)C * P);
    float* qn = (float*)malloc(sizeof(float) * (size_t)d * Q);
    float* xqg = (float*)malloc(sizeof(float) * (size_t)d * Q);
    int kmax = or_k_rov(P);
    float* dist = (float*)malloc(sizeof(float) * (size_t)(kmax > 0 ? kmax : 1) * Q);
    int* ind = (int*)malloc(sizeof(int) * (size_t)(kmax > 0 ? kmax : 1) * Q);
    int npts[TO_MAX_C_ORACLE];
    for (int t = Y - 2; t > 0; --t) {
        /* computePathStates + allocateXYRegressionData */
        for (int c = 0; c < C; ++c) npts[c] = 0;
        for (int p = 0; p < P; ++p) {
            for (int s = 0; s < S; ++s)
                xin[(size_t)p * d + s] = totalPops[((size_t)p * Y1 + t) * S + s] *
                                         aars[(((size_t)p * Y1 + t) * S + s) * C + (C - 1)];
            xin[(size_t)p * d + S] = unit_profit(pr, uRes, p, t, Y1, Y1);
            int ctl = controls[(size_t)p * Y + t];
            int valid = 1;
            for (int s = 0; s < S; ++s)
                if (xin[(size_t)p * d + s] < pr->params[s][3]) { valid = 0; break; }
            if (valid || ctl == 0) {
                int m = npts[ctl]++;
                yv[(size_t)ctl * P + m] = condExp[(size_t)(t + 1) * P + p];
                for (int j = 0; j < d; ++j)
                    xraw[((size_t)ctl * d + j) * P + m] = xin[(size_t)p * d + j];
            }
        }
        /* computeStateMinMax */
        float xmin[TO_MAX_C_ORACLE + 1][TO_LSM_MAXD], xmax[TO_MAX_C_ORACLE + 1][TO_LSM_MAXD];
        for (int c = 0; c < C; ++c) {
            if (c == 0 || npts[c] > d + 1) {
                for (int j = 0; j < d; ++j) {
                    const float* xs = xraw + ((size_t)c * d + j) * P;
                    float lo = npts[c] > 0 ? xs[0] : 0.0f, hi = lo;
                    for (int m = 0; m < npts[c]; ++m) {
                        if (lo > xs[m]) lo = xs[m];
                        else if (hi < xs[m]) hi = xs[m];
                    }
                    xmin[c][j] = lo; xmax[c][j] = hi;
                }
            } else {
                for (int j = 0; j < d; ++j) { xmin[c][j] = xmin[0][j]; xmax[c][j] = xmax[0][j]; }
            }
        }
        for (int j = 0; j < d; ++j) {
            xmin[C][j] = xmin[0][j]; xmax[C][j] = xmax[0][j];
            for (int c = 1; c < C; ++c) {
                if (xmin[C][j] > xmin[c][j]) xmin[C][j] = xmin[c][j];
                if (xmax[C][j] < xmax[c][j]) xmax[C][j] = xmax[c][j];
            }
        }
        /* createQueryPoints + host normalisation (SimulateGPU.cu:4549-4607) */
        for (int q = 0; q < Q; ++q) {
            int rem = q;
            for (int j = 0; j < d; ++j) {
                int div = 1;
                for (int e = 0; e < d - j - 1; ++e) div *= R;
                int di = rem / div;
                rem -= di * div;
                float raw = to_lsm_query_axis(di, xmin[C][j], xmax[C][j], R);
                float nv = to_lsm_normalise(raw, xmin[C][j], xmax[C][j], j == S, pr->scaling);
                qn[(size_t)j * Q + q] = nv;
                xqg[(size_t)j * Q + q] = (pr->sem == 0) ? to_lsm_unit_axis(di, R) : nv;
                for (int c = 0; c < C; ++c)
                    reg[(size_t)t * C * blk + (size_t)c * blk + (size_t)j * R + di] = raw;
            }
        }
        for (int c = 0; c < C; ++c) {
            int n = npts[c];
            float* yout = reg + (size_t)t * C * blk + (size_t)c * blk + (size_t)R * d;
            int k = or_k_rov_mult(n, kmult);
            if (n < 3 || k == 0) {
                for (int q = 0; q < Q; ++q) yout[q] = 0.0f;
                continue;
            }
            float* xn = xnorm + (size_t)c * d * P;
            for (int j = 0; j < d; ++j)
                for (int m = 0; m < n; ++m)
                    xn[(size_t)j * n + m] = to_lsm_normalise(xraw[((size_t)c * d + j) * P + m],
                                                             xmin[C][j], xmax[C][j], j == S,
                                                             pr->scaling);
            /* sem 0 reads the raw (un-normalised) dim-major buffer point-major
             * (Q7); sem 1 uses the normalised points */
            float* xr = (float*)malloc(sizeof(float) * (size_t)d * n);
            for (int j = 0; j < d; ++j)
                for (int m = 0; m < n; ++m) xr[(size_t)j * n + m] = xraw[((size_t)c * d + j) * P + m];
            reg_job rj = {0, Q, d, k, Q, n, pr->sem, xn, xr, qn, xqg, yv + (size_t)c * P, dist, ind,
                          yout};
            reg_all_queries(rj, nt);
            free(xr);
        }
        /* backwardInduction (SimulateGPU.cu:2464-2776) */
        for (int p = 0; p < P; ++p) {
            float state[TO_MAX_C_ORACLE * TO_LSM_MAXD + 1];
            for (int c = 0; c < C; ++c)
                for (int s = 0; s < S; ++s)
                    state[c * S + s] = totalPops[((size_t)p * Y1 + t) * S + s] *
                                       aars[(((size_t)p * Y1 + t) * S + s) * C + c];
            for (int s = 0; s < S; ++s)
                res->adj_pops[((size_t)t * S + s) * P + p] = state[(C - 1) * S + s];
            int sY = (pr->sem == 0) ? Y : Y1;                   /* Q5 */
            float prof = unit_profit(pr, uRes, p, t, sY, sY);
            state[S * C] = prof;
            res->unit_profits[(size_t)t * P + p] = prof;
            float pay[TO_MAX_C_ORACLE];
            int valid[TO_MAX_C_ORACLE];
            for (int c = 0; c < C; ++c) {
                valid[c] = 1;
                for (int s = 0; s < S; ++s) {
                    float thr = (pr->sem == 0) ? pr->params_flat[S * s + 3] : pr->params[s][3];
                    if (state[c * S + s] < thr && c > 0) { valid[c] = 0; break; }
                }
                if (valid[c]) {
                    float cur = pr->flows[c] * state[S * C];
                    const float* rb = reg + (size_t)t * C * blk + (size_t)c * blk;
                    float v = (pr->sem == 0) ? to_lsm_interp_ref(rb, R, S, C, state)
                                             : to_lsm_interp(rb, R, S, state + c * S, state[S * C]);
                    double ce = (double)(v / disc);
                    if (ce > 0.0) ce = 0.0;
                    pay[c] = (float)((double)cur + ce);
                } else pay[c] = 0.0f;
            }
            float best = pay[0];
            int bc = 0;
            for (int c = 1; c < C; ++c) {
                if (!valid[c]) continue;
                if (pr->sem == 0 ? ((double)pay[c] < 0.975 * (double)best) : (pay[c] < best)) {
                    best = pay[c]; bc = c;
                }
            }
            condExp[(size_t)t * P + p] = best;
            res->opt_cont[(size_t)t * P + p] = bc;
        }
        if (algo == 6) {
            /* the year's value and control come from the re-simulated paths */
            rov_resim_job rj[128];
            pthread_t rth[128];
            int rused = 0, rper = (P + nt - 1) / nt;
            for (int i = 0; i < nt; ++i) {
                int a0 = i * rper, b0 = a0 + rper > P ? P : a0 + rper;
                if (a0 >= b0) break;
                rov_resim_job jr = {pr, csc, a0, b0, t, maxN, popY, gmY, uRes, reg, condExp,
                                    res->opt_cont};
                rj[rused++] = jr;
            }
            for (int i = 1; i < rused; ++i) pthread_create(&rth[i], NULL, rov_resim_thread, &rj[i]);
            if (rused > 0) rov_resim_paths(&rj[0]);
            for (int i = 1; i < rused; ++i) pthread_join(rth[i], NULL);
        }
    }

    /* firstPeriodInduction (SimulateGPU.cu:2210-2330), FP64 sums */
    {
        float prof0 = 0.0f;
        {
            float uf = 0.0f, ore = 0.0f;
            for (int f = 0; f < pr->n_fuels; ++f) uf = fmaf(pr->fuel_costs[f], uRes[pr->fuel_idx[f]], uf);
            for (int c = 0; c < pr->n_commodities; ++c)
                ore = fmaf(ore_at(pr, 0, 0, c), uRes[pr->n_fuels + c], ore);
            prof0 = (pr->unit_cost + uf) - pr->unit_revenue * ore;
            if (pr->demand_idx >= 0) prof0 = prof0 * uRes[pr->demand_idx];
        }
        double sum[TO_MAX_C_ORACLE], cnt[TO_MAX_C_ORACLE], pay[TO_MAX_C_ORACLE];
        int valid[TO_MAX_C_ORACLE];
        for (int c = 0; c < C; ++c) { sum[c] = 0.0; cnt[c] = 0.0; }
        for (int p = 0; p < P; ++p) {
            int c = controls[(size_t)p * Y];
            sum[c] += (double)condExp[(size_t)P + p];
            cnt[c] += 1.0;
        }
        const double discd = (double)disc;
        int stop = C;
        for (int c = 0; c < C; ++c) {
            if (cnt[c] > 0.0) pay[c] = sum[c] / (cnt[c] * discd);
            else { stop = c; break; }
            valid[c] = 1;
            for (int s = 0; s < S; ++s) {
                float thr = (pr->sem == 0) ? pr->params_flat[S * s + 3] : pr->params[s][3];
                float adj = totalPops[s] * aars[(size_t)s * C + c];
                if (adj < thr && c > 0) { valid[c] = 0; break; }
            }
            if (valid[c]) {
                pay[c] += (double)(pr->flows[c] * prof0);
                if (pay[c] > 0.0) pay[c] = 0.0;
            } else pay[c] = NAN;
        }
        for (int c = stop; c < C; ++c) { pay[c] = (c == 0) ? 0.0 : NAN; valid[c] = 0; }
        double best = pay[0];
        int bc = 0;
        for (int c = 1; c < C; ++c)
            if (isfinite(pay[c]) && pay[c] < best) { best = pay[c]; bc = c; }
        double ss = 0.0, m1 = 0.0, n1 = 0.0;
        for (int p = 0; p < P; ++p)
            if (controls[(size_t)p * Y] == bc) {
                double dv = (double)condExp[(size_t)P + p] - best;
                ss += dv * dv;
                m1 += (double)condExp[(size_t)P + p];
                n1 += 1.0;
            }
        for (int p = 0; p < P; ++p) { condExp[p] = (float)best; res->opt_cont[p] = bc; }
        double sdfac = (pr->sem == 0) ? (1.0 + (double)pr->rrr / (100.0 * (double)pr->dt)) : discd;
        res->stats[0] = (double)(float)best;
        res->stats[1] = (double)bc;
        res->stats[2] = (n1 > 0.0) ? sqrt(ss / (n1 * sdfac)) : 0.0;
        /* Monte Carlo standard error of the value (new): sample SD of the
         * discounted year-1 values of the chosen control's paths / sqrt(n) */
        if (n1 > 1.0) {
            double mean = m1 / n1, v = 0.0;
            for (int p = 0; p < P; ++p)
                if (controls[(size_t)p * Y] == bc) {
                    double dv = (double)condExp[(size_t)P + p] - mean;
                    v += dv * dv;
                }
            res->value_se = sqrt(v / (n1 - 1.0)) / sqrt(n1) / discd;
        } else res->value_se = 0.0;
        res->n_best = (int)n1;
    }
    for (size_t i = 0; i < (size_t)P * Y; ++i) res->cond_exp[i] = condExp[i];
    if (res->regression)
        for (size_t i = 0; i < (size_t)Y * C * blk; ++i) res->regression[i] = reg[i];
    if (res->controls)
        for (size_t i = 0; i < (size_t)P * Y; ++i) res->controls[i] = controls[i];
    if (res->total_pops)
        memcpy(res->total_pops, totalPops, sizeof(float) * (size_t)P * (Y + 1) * S);
    if (res->aars)
        memcpy(res->aars, aars, sizeof(float) * (size_t)P * (Y + 1) * S * C);
    if (res->u_results)
        memcpy(res->u_results, uRes, sizeof(float) * (size_t)P * (Y + 1) * U);
    free(xin); free(xraw); free(xnorm); free(yv); free(qn); free(xqg); free(dist); free(ind);
    free(totalPops); free(aars); free(uRes); free(controls); free(condExp); free(reg);
    for (int q = 0; q < S * C; ++q) { free(csc[q].ptr); free(csc[q].idx); free(csc[q].val); }
    free(csc);
    free(popY); free(gmY);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Surrogates (SimulateGPU.cu:5533-5917)                                     */
/* ------------------------------------------------------------------------ */
int or_k_surrogate_mte(int n) {
    int k;
    if (n < 50) k = 5;
    else if (n < 100) k = 7;
    else if (n < 500) k = (int)ceil(0.02 * (n - 100) + 7);
    else k = (int)ceil(log((double)n) + 8);
    return k < n ? k : n;
}

int or_k_surrogate_rov(int n) {
    int k;
    if (n < 50) k = 5;
    else if (n < 100) k = (int)(5 + 5 * ceil((double)((n - 50) / 50)));
    else if (n < 500) k = (int)ceil(10 + 15 * ceil((double)((n - 100) / 400)));
    else k = (int)(25 + ceil((n - 500) * 0.02));
    return k < n ? k : n;
}

/* buildSurrogateMTECUDA: 1-D local-linear surrogate of y on x over R grid
 * points; out = [R x values | R y values] */
void or_build_surrogate_1d(int n, const float* x, const float* y, int R, float* out) {
    float lo = x[0], hi = x[0];
    for (int i = 1; i < n; ++i) { if (x[i] < lo) lo = x[i]; if (x[i] > hi) hi = x[i]; }
    int k = or_k_surrogate_mte(n);
    float* q = (float*)malloc(sizeof(float) * (size_t)R);
    for (int i = 0; i < R; ++i) { q[i] = to_lsm_query_axis(i, lo, hi, R); out[i] = q[i]; }
    float* dist = (float*)malloc(sizeof(float) * (size_t)(k > 0 ? k : 1) * R);
    int* ind = (int*)malloc(sizeof(int) * (size_t)(k > 0 ? k : 1) * R);
    if (n < 3 || k <= 0) {
        for (int i = 0; i < R; ++i) out[R + i] = 0.0f;
    } else {
        or_knn(x, n, q, R, 1, k, dist, ind);
        for (int i = 0; i < R; ++i) {
            float xq[1] = {q[i]};
            out[R + i] = local_linear(1, k, R, i, dist, ind, y, x, n, 1, xq, 1);
        }
    }
    free(q); free(dist); free(ind);
}

/* buildSurrogateROVCUDA: d-D local-linear surrogate; predictors dim-major
 * [d][n]; out = [R*d axis values | R^d values].  sem 0 reads the raw
 * predictors point-major in the regression (Q7) and clips the mean surface
 * at zero (rovCorrection, SimulateGPU.cu:3055-3073) when clip != 0. */
void or_build_surrogate_nd(int n, int d, const float* pred, const float* y, int R,
                           int sem, int clip, float* out) {
    int Q = 1;
    for (int j = 0; j < d; ++j) Q *= R;
    float xmin[TO_LSM_MAXD], xmax[TO_LSM_MAXD];
    for (int j = 0; j < d; ++j) {
        const float* xs = pred + (size_t)j * n;
        float lo = xs[0], hi = xs[0];
        for (int m = 0; m < n; ++m) { if (lo > xs[m]) lo = xs[m]; else if (hi < xs[m]) hi = xs[m]; }
        xmin[j] = lo; xmax[j] = hi;
    }
    int k = or_k_surrogate_rov(n);
    float* qn = (float*)malloc(sizeof(float) * (size_t)d * Q);
    float* xq_all = (float*)malloc(sizeof(float) * (size_t)d * Q);
    for (int q = 0; q < Q; ++q) {
        int rem = q;
        for (int j = 0; j < d; ++j) {
            int div = 1;
            for (int e = 0; e < d - j - 1; ++e) div *= R;
            int di = rem / div;
            rem -= di * div;
            float raw = to_lsm_query_axis(di, xmin[j], xmax[j], R);
            out[(size_t)j * R + di] = raw;
            float nv = to_lsm_normalise(raw, xmin[j], xmax[j], 0, 1.0f);
            qn[(size_t)j * Q + q] = nv;
            xq_all[(size_t)j * Q + q] = (sem == 0) ? to_lsm_unit_axis(di, R) : nv;
        }
    }
    float* pn = (float*)malloc(sizeof(float) * (size_t)d * n);
    for (int j = 0; j < d; ++j)
        for (int m = 0; m < n; ++m)
            pn[(size_t)j * n + m] = to_lsm_normalise(pred[(size_t)j * n + m], xmin[j], xmax[j], 0, 1.0f);
    float* yout = out + (size_t)R * d;
    if (n < 3 || k <= 0) {
        for (int q = 0; q < Q; ++q) yout[q] = 0.0f;
    } else {
        float* dist = (float*)malloc(sizeof(float) * (size_t)k * Q);
        int* ind = (int*)malloc(sizeof(int) * (size_t)k * Q);
        or_knn(pn, n, qn, Q, d, k, dist, ind);
        float xq[TO_LSM_MAXD];
        for (int q = 0; q < Q; ++q) {
            for (int j = 0; j < d; ++j) xq[j] = xq_all[(size_t)j * Q + q];
            float v = (sem == 0) ? local_linear(d, k, Q, q, dist, ind, y, pred, n, 1, xq, 1)
                                 : local_linear(d, k, Q, q, dist, ind, y, pn, n, 0, xq, 1);
            if (clip && v > 0.0f) v = 0.0f;
            yout[q] = v;
        }
        free(dist); free(ind);
    }
    free(qn); free(xq_all); free(pn);
}
