/*
 * oracle.c - CPU restatement of the reference's habitat-patch, road-crossing,
 * species-model, MTE and expected-PV code.  TEST INFRASTRUCTURE ONLY (see
 * oracle.h).  Each function cites the reference file:line it follows; paths
 * are relative to the TransportOptimiser tree.
 */
#include "oracle.h"
#include "../transportoptimiser_gb300/csrc/to_math.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

float or_normal(uint64_t seed, int stream, int road, int path, int year,
                int lane) {
    return to_normal1(seed, (uint32_t)stream, (uint32_t)road, (uint32_t)path,
                      (uint32_t)year, (uint32_t)lane);
}

float or_uniform(uint64_t seed, int stream, int road, int path, int year,
                 int lane) {
    return to_uniform1(seed, (uint32_t)stream, (uint32_t)road, (uint32_t)path,
                       (uint32_t)year, (uint32_t)lane);
}

/* ------------------------------------------------------------------------ */
/* LabelImage, include/utilities/labelmethod.cpp:34-56.  Components are       */
/* numbered 1.. in raster order (index x + W*y) of their first pixel; the     */
/* reference walks 4-neighbours with an explicit stack, which yields the      */
/* same numbering as any traversal that labels a whole component when its    */
/* first pixel is met.                                                        */
/* ------------------------------------------------------------------------ */
int or_label_image(int W, int H, const int* input, int* output) {
    int n = W * H;
    int* stack = (int*)malloc(sizeof(int) * (size_t)(n + 1));
    memset(output, 0, sizeof(int) * (size_t)n);
    int label = 0;
    for (int idx = 0; idx < n; ++idx) {
        if (input[idx] == 0 || output[idx] != 0) continue;
        ++label;
        int sp = 0;
        stack[sp++] = idx;
        output[idx] = label;
        while (sp > 0) {
            int c = stack[--sp];
            int x = c % W, y = c / W;
            int nb[4] = {x > 0 ? c - 1 : -1, x < W - 1 ? c + 1 : -1,
                         y > 0 ? c - W : -1, y < H - 1 ? c + W : -1};
            for (int q = 0; q < 4; ++q) {
                int m = nb[q];
                if (m >= 0 && input[m] != 0 && output[m] == 0) {
                    output[m] = label;
                    stack[sp++] = m;
                }
            }
        }
    }
    free(stack);
    return label;
}

/* ------------------------------------------------------------------------ */
/* patchComputation (SimulateGPU.cu:498-573) and the host compaction of       */
/* SimulateGPU::buildPatches (SimulateGPU.cu:3620-3636).  Candidate index     */
/* idx = (by*xres + bx)*R + (region-1); x offsets are bounded by H and y      */
/* offsets by W exactly as in the reference (square grids only, Q20).        */
/* ------------------------------------------------------------------------ */
int or_build_patches(int W, int H, int skpx, int skpy, int xres, int yres,
                     int n_regions, double xspacing, double yspacing,
                     double sub_patch_area, double max_pop, const int* labels,
                     const double* pops, double* area_o, double* cap_o,
                     double* pop_o, double* cx_o, double* cy_o,
                     int* n_patches) {
    int n_cand = xres * yres * n_regions;
    float fxs = (float)xspacing, fys = (float)yspacing;
    float fspa = (float)sub_patch_area, fcap = (float)max_pop;
    int added = 0;
    for (int idx = 0; idx < n_cand; ++idx) {
        int by = idx / (xres * n_regions);
        int rem = idx - by * (xres * n_regions);
        int bx = rem / n_regions;
        rem = rem - bx * n_regions;
        int region = rem + 1;
        int bsx = ((bx + 1) * skpx <= H) ? skpx : H - bx * skpx;
        int bsy = ((by + 1) * skpy <= W) ? skpy : W - by * skpy;
        float area = 0.0f, cap = 0.0f, pop = 0.0f, cx = 0.0f, cy = 0.0f;
        for (int ii = 0; ii < bsx; ++ii)
            for (int jj = 0; jj < bsy; ++jj) {
                int xc = bx * skpx + ii, yc = by * skpy + jj;
                area += (float)(labels[xc + yc * W] == region);
            }
        if (area > 0.0f) {
            for (int ii = 0; ii < bsx; ++ii)
                for (int jj = 0; jj < bsy; ++jj) {
                    int xc = bx * skpx + ii, yc = by * skpy + jj;
                    if (labels[xc + yc * W] == region) {
                        pop += (float)pops[xc + yc * W];
                        cx += (float)ii;
                        cy += (float)jj;
                    }
                }
            cx = fxs * (cx / area + (float)(bx * skpx));
            cy = fys * (cy / area + (float)(by * skpy));
            area = area * fspa;
            cap = area * fcap;
            int o = *n_patches;
            area_o[o] = (double)area;
            cap_o[o] = (double)cap;
            pop_o[o] = (double)pop;
            cx_o[o] = (double)cx;
            cy_o[o] = (double)cy;
            *n_patches = o + 1;
            ++added;
        }
    }
    return added;
}

/* ------------------------------------------------------------------------ */
/* lineSegmentIntersect (SimulateGPU.cu:3478-3568, kernels 454-493): the      */
/* direction vectors are differenced in double and rounded to float; the      */
/* predicate is evaluated in float without contraction.                       */
/* ------------------------------------------------------------------------ */
void or_line_segment_intersect(int T, const double* xy1, int G,
                               const double* xy2, int* crossings) {
    for (int t = 0; t < T; ++t) {
        float x1 = (float)xy1[t], y1 = (float)xy1[t + T];
        float x21 = (float)(xy1[t + 2 * T] - xy1[t]);
        float y21 = (float)(xy1[t + 3 * T] - xy1[t + T]);
        int c = 0;
        for (int g = 0; g < G; ++g) {
            float x3 = (float)xy2[g], y3 = (float)xy2[g + G];
            float x43 = (float)(xy2[g + 2 * G] - xy2[g]);
            float y43 = (float)(xy2[g + 3 * G] - xy2[g + G]);
            float y13 = y1 - y3;
            float x13 = x1 - x3;
            float numa = x43 * y13 - y43 * x13;
            float numb = x21 * y13 - y21 * x13;
            float deno = y43 * x21 - x43 * y21;
            float ua = numa / deno;
            float ub = numb / deno;
            c += (ua >= 0.0f) && (ua <= 1.0f) && (ub >= 0.0f) && (ub <= 1.0f);
        }
        crossings[t] = c;
    }
}

/* ------------------------------------------------------------------------ */
/* SpeciesRoadPatches::createSpeciesModel (SpeciesRoadPatches.cpp:12-59):     */
/*   generateHabitatPatchesGrid  :62-264 (GPU branch, :160-170)              */
/*   habitatPatchDistances       :270-294                                    */
/*   roadCrossings               :296-381                                    */
/*   computeTransitionProbabilities :383-426                                 */
/*   computeSurvivalProbabilities   :428-451                                 */
/* followed by the mmm = trans o surv_c float cast and the dense2Sparse      */
/* threshold (SimulateGPU.cu:3783-3796, 4102-4117, 5973-5996).               */
/* ------------------------------------------------------------------------ */
int or_species_model(const or_species_in* in, or_species_out* out) {
    int W = in->W, H = in->H, res = in->res;
    int xres = (W % res == 0) ? res : res + 1;
    int yres = (H % res == 0) ? res : res + 1;
    int skpx = (int)floor((double)(W - 1) / (double)res);
    int skpy = (int)floor((double)(H - 1) / (double)res);
    double spa = in->xspacing * in->yspacing;
    int* inp = (int*)malloc(sizeof(int) * (size_t)W * H);
    int* lab = (int*)malloc(sizeof(int) * (size_t)W * H);
    int N = 0;
    for (int h = 0; h < in->n_hab; ++h) {
        int typ = in->habs[h].type;
        if (typ == 3 || typ == 4) continue;   /* CLEAR, ROAD */
        for (int i = 0; i < W * H; ++i) inp[i] = in->hab_map[i] == typ;
        int regions = or_label_image(W, H, inp, lab);
        if (regions <= 0) continue;
        int before = N;
        int n_cand = xres * yres * regions;
        if (N + n_cand > out->max_patches) {
            /* worst case would not fit: count first */
            double *a = (double*)malloc(sizeof(double) * 5 * (size_t)n_cand);
            int nn = 0;
            or_build_patches(W, H, skpx, skpy, xres, yres, regions,
                             in->xspacing, in->yspacing, spa,
                             in->habs[h].max_pop, lab, in->pop_map, a,
                             a + n_cand, a + 2 * n_cand, a + 3 * n_cand,
                             a + 4 * n_cand, &nn);
            if (N + nn > out->max_patches) { free(a); free(inp); free(lab); return -1; }
            for (int i = 0; i < nn; ++i) {
                out->area[N + i] = a[i];
                out->cap[N + i] = a[n_cand + i];
                out->pop[N + i] = a[2 * n_cand + i];
                out->cx[N + i] = a[3 * n_cand + i];
                out->cy[N + i] = a[4 * n_cand + i];
            }
            N += nn;
            free(a);
        } else {
            or_build_patches(W, H, skpx, skpy, xres, yres, regions,
                             in->xspacing, in->yspacing, spa,
                             in->habs[h].max_pop, lab, in->pop_map, out->area,
                             out->cap, out->pop, out->cx, out->cy, &N);
        }
        for (int i = before; i < N; ++i) out->type[i] = h;
    }
    free(inp);
    free(lab);
    out->n_patches = N;

    /* distances (SpeciesRoadPatches.cpp:270-294) */
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) {
            double dx = out->cx[i] - out->cx[j];
            double dy = out->cy[i] - out->cy[j];
            out->dists[i * N + j] = sqrt(dx * dx + dy * dy);
        }

    /* crossings (SpeciesRoadPatches.cpp:296-381).  The reference counts the
     * valid pairs from -1 and then keeps only that many rows, so the last
     * valid pair is never tested and keeps 0 crossings (sem 0). */
    double lam = in->lambda_mean + in->lambda_sd * in->lambda_mult;
    double max_dist_x = log(0.05) / (-lam);
    int T = 0;
    for (int i = 0; i < N; ++i)
        for (int j = i + 1; j < N; ++j)
            if (out->dists[i * N + j] <= max_dist_x) ++T;
    int Tt = (in->sem == 0) ? (T > 0 ? T - 1 : 0) : T;
    out->n_transitions = Tt;
    double* lines = (double*)malloc(sizeof(double) * 4 * (size_t)(Tt > 0 ? Tt : 1));
    int* orgs = (int*)malloc(sizeof(int) * (size_t)(Tt > 0 ? Tt : 1));
    int* dsts = (int*)malloc(sizeof(int) * (size_t)(Tt > 0 ? Tt : 1));
    int* cr = (int*)malloc(sizeof(int) * (size_t)(Tt > 0 ? Tt : 1));
    int t = 0;
    for (int i = 0; i < N && t < Tt; ++i)
        for (int j = i + 1; j < N && t < Tt; ++j)
            if (out->dists[i * N + j] <= max_dist_x) {
                orgs[t] = i; dsts[t] = j;
                lines[t] = out->cx[i];
                lines[t + Tt] = out->cy[i];
                lines[t + 2 * Tt] = out->cx[j];
                lines[t + 3 * Tt] = out->cy[j];
                ++t;
            }
    memset(out->crossings, 0, sizeof(int) * (size_t)N * N);
    if (Tt > 0 && in->G > 0) {
        or_line_segment_intersect(Tt, lines, in->G, in->road, cr);
        for (int q = 0; q < Tt; ++q) {
            out->crossings[orgs[q] * N + dsts[q]] = cr[q];
            out->crossings[dsts[q] * N + orgs[q]] = cr[q];
        }
    }
    free(lines); free(orgs); free(dsts); free(cr);

    /* transition probabilities (SpeciesRoadPatches.cpp:383-426).  sem 0
     * divides by exp(-lambda d) and double-counts lambda_mean in the cut-off
     * distance (as the reference does); sem 1 multiplies by exp(-lambda d)
     * within ln(20)/lambda. */
    double lda = in->lambda_mult * in->lambda_sd + in->lambda_mean;
    double hp = in->hab_pref_mult;
    double max_dist_t = (in->sem == 0)
        ? log(0.05) / (-(in->lambda_mean + in->lambda_sd * lda))
        : log(0.05) / (-lda);
    for (int i = 0; i < N; ++i) {
        double summ = 0.0;
        for (int j = 0; j < N; ++j) {
            double v = 0.0;
            double d = out->dists[i * N + j];
            if (d <= max_dist_t) {
                const or_habitat* hb = &in->habs[out->type[j]];
                double w = out->area[j] * lda * exp(hb->pref_mean + hb->pref_sd * hp);
                if (i == j) v = w;
                else if (in->sem == 0) v = w / exp(-lda * d);
                else v = w * exp(-lda * d);
                summ += v;
            }
            out->trans[i * N + j] = v;
        }
        for (int j = 0; j < N; ++j) out->trans[i * N + j] = out->trans[i * N + j] / summ;
    }

    /* survival (SpeciesRoadPatches.cpp:428-451) and migration matrices */
    for (int c = 0; c < in->n_controls; ++c) {
        double hz = in->hazard[c];
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) {
                double s = exp(-(double)out->crossings[i * N + j] * hz);
                out->surv[((size_t)c * N + i) * N + j] = s;
                float m = (float)(out->trans[i * N + j] * s);
                /* dense2Sparse keeps entries > 1e-5; here they stay dense
                 * with the dropped entries set to zero */
                out->mmm[((size_t)c * N + j) * N + i] = ((double)m > 0.00001) ? m : 0.0f;
            }
    }

    /* initial animals at risk (SpeciesRoadPatches::computeAAR /
     * computeInitialAAR, SpeciesRoadPatches.cpp:453-490): per control
     * 1 - sum_j [(trans o surv_c)^T pops]_j / sum pops, accumulated row by
     * row (ascending destinations, then ascending origins) */
    if (out->iar)
        for (int c = 0; c < in->n_controls; ++c) {
            double tot = 0.0, init = 0.0;
            for (int i = 0; i < N; ++i) {
                double acc = 0.0;
                for (int j = 0; j < N; ++j)
                    if (out->trans[i * N + j] != 0.0)
                        acc += out->trans[i * N + j] * out->surv[((size_t)c * N + i) * N + j];
                tot += out->pop[i] * acc;
                init += out->pop[i];
            }
            out->iar[c] = 1.0 - tot / init;
        }
    return N;
}

/* ------------------------------------------------------------------------ */
/* mteKernel (SimulateGPU.cu:595-717) as driven by simulateMTECUDA            */
/* (SimulateGPU.cu:3680-3843).  Streams: growth N(0,1) per (path, year,       */
/* species*patch), brownian / jump size N(0,1) and jump U[0,1) per            */
/* (path, year, species).                                                     */
/*   Q1 (sem 0): the end population sums the post-migration, pre-growth      */
/*       buffer of the last year.                                             */
/*   Q2: no /100 in the logistic step (the ROV kernel has it).                */
/*   Q3 (sem 0): jump size = z*s^2 - s^2/2; sem 1: z*s - s^2/2.               */
/* ------------------------------------------------------------------------ */
/* Patch totals are summed in groups of four consecutive patches,
 * ((v0 + v1) + v2) + v3, the groups then in ascending order - the order the
 * CUDA kernels use (one warp lane owns a group of four patches). */
float or_grouped_sum(const float* v, int N) {
    float tot = 0.0f;
    for (int g = 0; g < N; g += 4) {
        float s = v[g];
        for (int j = 1; j < 4; ++j) s = s + (g + j < N ? v[g + j] : 0.0f);
        tot = tot + s;
    }
    return tot;
}

typedef struct {
    int p0, p1, n_years, N, species, road, sem;
    float dt;
    const float *params, *init, *caps;
    /* compressed columns of the destination-major matrix: destination k's
     * non-zeros are origins idx[ptr[k] .. ptr[k+1]) ascending, with values */
    const int* ptr;
    const int* idx;
    const float* val;
    uint64_t seed;
    float* out;
} mte_job;

/* One path at a time, as mteKernel does (one thread per path,
 * SimulateGPU.cu:595-717): the migration walks destination k's compressed
 * column (mteKernel :628-635 reads the dense2Sparse CSC lists) in ascending
 * origin order with fused multiply-adds; the growth normals come four per
 * Philox call (the patch group's block), which are the same bits as one
 * to_normal1 per patch. */
static void mte_paths(const mte_job* j) {
    int N = j->N;
    int N4 = (N + 3) & ~3;
    float* pop = (float*)malloc(sizeof(float) * (size_t)N4);
    float* mig = (float*)malloc(sizeof(float) * (size_t)N4);
    const float* sp = j->params;
    float sj2 = sp[5] * sp[5];
    const uint32_t grp0 = (uint32_t)((j->species * N4) >> 2);
    for (int p = j->p0; p < j->p1; ++p) {
        for (int k = 0; k < N; ++k) pop[k] = j->init[k];
        float gm = sp[0];
        for (int t = 0; t < j->n_years; ++t) {
            for (int k = 0; k < N; ++k) {
                float acc = 0.0f;
                for (int e = j->ptr[k]; e < j->ptr[k + 1]; ++e)
                    acc = fmaf(pop[j->idx[e]], j->val[e], acc);
                mig[k] = acc;
            }
            float uj = to_uniform1(j->seed, TO_STREAM_SP_JUMP, j->road, p, t, j->species);
            float zb = to_normal1(j->seed, TO_STREAM_SP_BROWNIAN, j->road, p, t, j->species);
            float zj = to_normal1(j->seed, TO_STREAM_SP_JUMPSIZE, j->road, p, t, j->species);
            float jump = (uj < sp[6]) ? 1.0f : 0.0f;
            float brown = zb * sp[2];
            float jsz = (j->sem == 0) ? (zj * sj2 - sj2 / 2.0f)
                                      : (zj * sp[5] - sj2 / 2.0f);
            gm = gm + sp[4] * (sp[1] - gm) * j->dt + gm * brown
                 + (to_expf(jsz) - 1.0f) * gm * jump;
            for (int k0 = 0; k0 < N; k0 += 4) {
                float z[4];
                to_normal4(j->seed, TO_STREAM_GROWTH, j->road, p, t, grp0 + (k0 >> 2), z);
                for (int q = 0; q < 4 && k0 + q < N; ++q) {
                    const int k = k0 + q;
                    float gr = fmaf(sp[7] * z[q], gm, gm);
                    float m = mig[k];
                    float c = j->caps[k];
                    pop[k] = m * (1.0f + gr * (c - m) / c);
                }
            }
        }
        float e = (j->n_years == 0) ? or_grouped_sum(j->init, N)
                : (j->sem == 0 ? or_grouped_sum(mig, N) : or_grouped_sum(pop, N));
        j->out[p] = e;
    }
    free(pop);
    free(mig);
}

static void* mte_thread(void* a) { mte_paths((const mte_job*)a); return NULL; }

/* dense2Sparse (SimulateGPU.cu:5973-5996) of a destination-major N x N
 * matrix: entries > 0 of row k (destination k) in ascending origin order.
 * The skipped entries are exact zeros, so fmaf over the list gives the bits
 * of fmaf over the whole dense row.  Returns the non-zero count. */
int or_pack_csc(int N, const float* mmm, int* ptr, int* idx, float* val) {
    int n = 0;
    for (int k = 0; k < N; ++k) {
        ptr[k] = n;
        const float* row = mmm + (size_t)k * N;
        for (int l = 0; l < N; ++l)
            if (row[l] > 0.0f) {
                if (idx) { idx[n] = l; val[n] = row[l]; }
                ++n;
            }
    }
    ptr[N] = n;
    return n;
}

void or_simulate_mte(int n_paths, int n_years, int N, float dt,
                     const float* params8, const float* init_pops,
                     const float* caps, const float* mmm, uint64_t seed,
                     int road, int species, int sem, int n_threads,
                     float* end_pops) {
    if (n_threads < 1) n_threads = 1;
    if (n_threads > 256) n_threads = 256;
    int* ptr = (int*)malloc(sizeof(int) * (size_t)(N + 1));
    int nnz = or_pack_csc(N, mmm, ptr, NULL, NULL);
    int* idx = (int*)malloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
    float* val = (float*)malloc(sizeof(float) * (size_t)(nnz > 0 ? nnz : 1));
    or_pack_csc(N, mmm, ptr, idx, val);
    mte_job jobs[256];
    pthread_t th[256];
    int per = (n_paths + n_threads - 1) / n_threads;
    int used = 0;
    for (int i = 0; i < n_threads; ++i) {
        int p0 = i * per, p1 = p0 + per;
        if (p1 > n_paths) p1 = n_paths;
        if (p0 >= p1) break;
        mte_job j = {p0, p1, n_years, N, species, road, sem, dt, params8,
                     init_pops, caps, ptr, idx, val, seed, end_pops};
        jobs[used++] = j;
    }
    if (used == 1) {
        mte_paths(&jobs[0]);
    } else {
        for (int i = 0; i < used; ++i) pthread_create(&th[i], NULL, mte_thread, &jobs[i]);
        for (int i = 0; i < used; ++i) pthread_join(th[i], NULL);
    }
    free(ptr);
    free(idx);
    free(val);
}

/* ------------------------------------------------------------------------ */
/* expPVPath (SimulateGPU.cu:256-279) and SimulateGPU::expPV (3163-3259).     */
/* params = {gr, meanP, timeStep, rrr, current, reversion, jumpProb,          */
/*           noiseSD (already x timeStep x multiplier), poissonJump}.         */
/*   Q11 (sem 0): path idx reads the flat streams at idx+year (overlapping    */
/*        windows) and the returned "SD" is sqrt(sum of squared deviations);  */
/*        sem 1 reads idx*Y+year and returns the sample SD.                   */
/*   Q3: jump sizes are N(-s^2/2, s^2) with s = poissonJump.                  */
/* The growth and discount powers are accumulated by repeated products.       */
/* ------------------------------------------------------------------------ */
static float pv_stream(uint64_t seed, int stream, int road, long flat, int normal) {
    uint32_t path = (uint32_t)(flat >> 2);
    uint32_t lane = (uint32_t)(flat & 3);
    return normal ? to_normal1(seed, (uint32_t)stream, (uint32_t)road, path, 0, lane)
                  : to_uniform1(seed, (uint32_t)stream, (uint32_t)road, path, 0, lane);
}

void or_exp_pv(int n_paths, int n_years, const float* prm, uint64_t seed,
               int road, int sem, float* values, double* mean, double* sd) {
    float gr = prm[0], meanP = prm[1], ts = prm[2], rrr = prm[3];
    float cur0 = prm[4], rev = prm[5], jp = prm[6], nsd = prm[7], pj = prm[8];
    float pj2 = pj * pj;
    for (int p = 0; p < n_paths; ++p) {
        float value = 0.0f, curr = cur0;
        float g = 1.0f, r = 1.0f;
        for (int t = 0; t < n_years; ++t) {
            long flat = (sem == 0) ? (long)p + t : (long)p * n_years + t;
            float zb = pv_stream(seed, TO_STREAM_PV_BROWNIAN, road, flat, 1);
            float zj = pv_stream(seed, TO_STREAM_PV_JUMPSIZE, road, flat, 1);
            float uj = pv_stream(seed, TO_STREAM_PV_JUMP, road, flat, 0);
            float brown = zb * nsd;
            float jsz = zj * pj2 + (-pj2 / 2.0f);
            float jumped = (uj < jp) ? 1.0f : 0.0f;
            curr = curr + (rev * (meanP - curr) * ts + curr * brown
                           + (to_expf(jsz) - 1.0f) * curr * jumped);
            value = value + g * curr / r;
            g = g * (1.0f + gr);
            r = r * (1.0f + rrr);
        }
        values[p] = value;
    }
    double tot = 0.0;
    for (int p = 0; p < n_paths; ++p) tot += (double)values[p];
    double m = tot / (double)n_paths;
    double ss = 0.0;
    for (int p = 0; p < n_paths; ++p) {
        double d = (double)values[p] - m;
        ss += d * d;
    }
    *mean = m;
    *sd = (sem == 0) ? sqrt(ss) : sqrt(ss / (double)(n_paths > 1 ? n_paths - 1 : 1));
}

/* Materialise a fused stream in a reference-style array:
 * out[(p*Y + t)*L + l] = stream value at lane (lane_offset + l). */
void or_fill_stream(uint64_t seed, int stream, int road, int normal,
                    int n_paths, int n_years, int L, int lane_offset,
                    float* out) {
    for (int p = 0; p < n_paths; ++p)
        for (int t = 0; t < n_years; ++t)
            for (int l = 0; l < L; ++l) {
                size_t o = ((size_t)p * n_years + t) * L + l;
                out[o] = normal
                    ? to_normal1(seed, (uint32_t)stream, (uint32_t)road, (uint32_t)p,
                                 (uint32_t)t, (uint32_t)(lane_offset + l))
                    : to_uniform1(seed, (uint32_t)stream, (uint32_t)road, (uint32_t)p,
                                  (uint32_t)t, (uint32_t)(lane_offset + l));
            }
}

/* Flat expected-PV streams (index j -> lane j&3 of block j>>2). */
void or_fill_pv_stream(uint64_t seed, int stream, int road, int normal,
                       long n, float* out) {
    for (long j = 0; j < n; ++j) out[j] = pv_stream(seed, stream, road, j, normal);
}

/* ------------------------------------------------------------------------ */
/* RoadCells::computeRoadCells (include/road/RoadCells.cpp:10-272) for a      */
/* polyline x[0..n), y[0..n) on a grid with spacing (xs, ys) and origin 0:    */
/* every span is reparametrised at its crossings of the grid lines            */
/* (x = k xs, y = k ys), the points of a span sorted by (x, y) ascending when  */
/* the span runs towards larger x, else descending; consecutive equal points  */
/* are dropped (unique_rows); each piece between consecutive points lies in   */
/* the cell (ceil(mid_x / xs), ceil(mid_y / ys)) of its midpoint, index       */
/* row + col W (sub2ind on the W x H vegetation matrix).  The cells inside    */
/* the grid are returned sorted and unique.                                   */
/*   Q38 (sem 0): the x of a vertical-grid-line crossing is computed from the  */
/*        y of row q of the span's crossing list (RoadCells.cpp:189-194 reads  */
/*        pairs.block(0,1,...)), which for a span that also crosses vertical  */
/*        lines is a horizontal crossing's y; sem 1 uses its own y.           */
/* ------------------------------------------------------------------------ */
typedef struct { double x, y; } or_pt;

static int pt_less(or_pt a, or_pt b) { return a.x < b.x || (a.x == b.x && a.y < b.y); }

static int span_points(double x0, double y0, double x1, double y1, double xs, double ys,
                       int sem, or_pt* pts) {
    const int h = (int)(x1 / xs) - (int)(x0 / xs);
    const int v = (int)(y1 / ys) - (int)(y0 / ys);
    const int ah = h < 0 ? -h : h, av = v < 0 ? -v : v;
    const double m = (y1 - y0) / (x1 - x0), b = y0 - x0 * m;
    const double m2 = (x1 - x0) / (y1 - y0), b2 = x0 - y0 * m2;
    for (int q = 0; q < ah; ++q) {
        double px;
        if (h > 0) px = xs * (floor(x0 / xs) + (double)(q + 1));
        else if (fmod(x0, xs) == 0.0) px = xs * (ceil(x0 / xs) - (double)q);
        else px = xs * (ceil(x0 / xs) - (double)(q + 1));
        pts[q].x = px;
        pts[q].y = isfinite(m) ? m * px + b : y0;
    }
    for (int q = 0; q < av; ++q) {
        double py;
        if (v > 0) py = ys * (floor(y0 / ys) + (double)(q + 1));
        else if (fmod(y0, ys) == 0.0) py = ys * (ceil(y0 / ys) - (double)q);
        else py = ys * (ceil(y0 / ys) - (double)(q + 1));
        pts[ah + q].y = py;
    }
    for (int q = 0; q < av; ++q) {
        const double src = (sem == 0) ? pts[q].y : pts[ah + q].y;
        double px;
        if (isfinite(m)) px = (src - b) / m;
        else if (isfinite(m2)) px = b2 + m2 * src;
        else px = x0;
        pts[ah + q].x = px;
    }
    const int n = ah + av;
    /* insertion sort (ascending, or descending when the span runs to smaller x) */
    const int asc = x1 >= x0;
    for (int i = 1; i < n; ++i) {
        or_pt t = pts[i];
        int j = i - 1;
        while (j >= 0 && (asc ? pt_less(t, pts[j]) : pt_less(pts[j], t))) { pts[j + 1] = pts[j]; --j; }
        pts[j + 1] = t;
    }
    return n;
}

static int cmp_int(const void* a, const void* b) {
    int x = *(const int*)a, y = *(const int*)b;
    return (x > y) - (x < y);
}

int or_road_cells(int n, const double* x, const double* y, int W, int H, double xs, double ys,
                  int sem, int* cells, int cap) {
    if (n < 2) return 0;
    int maxp = 2;
    for (int i = 0; i + 1 < n; ++i) {
        int h = (int)(x[i + 1] / xs) - (int)(x[i] / xs), v = (int)(y[i + 1] / ys) - (int)(y[i] / ys);
        int k = (h < 0 ? -h : h) + (v < 0 ? -v : v);
        if (k > maxp) maxp = k;
    }
    or_pt* pts = (or_pt*)malloc(sizeof(or_pt) * (size_t)(maxp + 2));
    int* tmp = (int*)malloc(sizeof(int) * (size_t)(n * (maxp + 2)));
    int nc = 0;
    for (int i = 0; i + 1 < n; ++i) {
        const int k = span_points(x[i], y[i], x[i + 1], y[i + 1], xs, ys, sem, pts + 1);
        pts[0].x = x[i]; pts[0].y = y[i];
        pts[k + 1].x = x[i + 1]; pts[k + 1].y = y[i + 1];
        for (int q = 0; q <= k; ++q) {
            const or_pt a = pts[q], bq = pts[q + 1];
            if (a.x == bq.x && a.y == bq.y) continue;
            const int r = (int)ceil((0.5 * (a.x + bq.x) - 0.0) / xs);
            const int c = (int)ceil((0.5 * (a.y + bq.y) - 0.0) / ys);
            if (r >= 0 && r < W && c >= 0 && c < H) tmp[nc++] = r + c * W;
        }
    }
    qsort(tmp, (size_t)nc, sizeof(int), cmp_int);
    int m = 0;
    for (int i = 0; i < nc; ++i)
        if (i == 0 || tmp[i] != tmp[i - 1]) {
            if (m < cap) cells[m] = tmp[i];
            ++m;
        }
    free(pts);
    free(tmp);
    return m;
}
