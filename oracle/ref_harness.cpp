/*
 * ref_harness.cpp - host-side drivers for the reference kernels compiled by
 * oracle/build_ref.sh.  Each driver restates the reference's host wrapper
 * (allocation and copies dropped; launches replaced by loops over the grid)
 * and takes the random streams as arrays in the reference's own layout, so
 * that the reference arithmetic runs on exactly the inputs the oracle sees.
 * TEST INFRASTRUCTURE ONLY; built into oracle/_ref/ and never shipped.
 */
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

struct to_dim3 { unsigned int x, y, z; };
thread_local to_dim3 blockIdx, threadIdx, blockDim, gridDim;
struct to_ref_texture { const float* data; int width; };
thread_local to_ref_texture texA;

/* ---- reference kernels (include/gpuCode/SimulateGPU.cu) ---------------- */
void patchComputation(int noCandidates, int W, int H, int skpx, int skpy,
        int xres, int yres, float subPatchArea, float xspacing,
        float yspacing, float capacity, int uniqueRegions,
        const int* labelledImage, const float* pops, float* results);
void pathAdjacencyKernel(int noTransitions, int noSegments, float* XY1,
        float* XY2, float* X4_X3, float* Y4_Y3, float* X2_X1, float* Y2_Y1,
        int* adjacency);
void roadCrossingsKernel(int rows, int segs, int* adjacency, int* cross);
void mteKernel(int noPaths, int nYears, int noPatches, float timeStep,
        float* rgr, float* brownians, float* jumpSizes, float* jumps,
        float* speciesParams, float* initPops, float* caps, float* mmm,
        int* rowIdx, int* elemsPerCol, float* pathPops, float* eps);
void expPVPath(const int noPaths, const float gr, const int nYears,
        const float meanP, const float timeStep, const float rrr,
        float current, float reversion, float jumpProb, const float* brownian,
        const float* jumpSize, const float* jump, float* result);
void randControls(int noPaths, int nYears, int noControls, float* randCont,
        int* control);
void forwardPathKernel(int noPaths, int nYears, int noSpecies, int noPatches,
        int noControls, int noUncertainties, float timeStep, float* initPops,
        float* pops, float* mmm, int* rowIdx, int* elemsPerCol, int maxElems,
        float* speciesParams, float* caps, float* aars, float* uncertParams,
        int* controls, float* uJumps, float* uBrownian, float* uJumpSizes,
        float* uJumpsSpecies, float* uBrownianSpecies, float* uJumpSizesSpecies,
        float* rgr, float* uResults, float* totalPops);
void computePathStates(int noPaths, int noDims, int nYears, int noControls,
        int year, float unitCost, float unitRevenue, int* controls, int noFuels,
        float* fuelCosts, float* uResults, float* uComposition,
        int noUncertainties, int* fuelIdx, int noCommodities, float* aars,
        float* totalPops, float* xin, int* currControls);
void allocateXYRegressionData(int noPaths, int noControls, int noDims,
        int nYears, float* speciesParams, int year, int* controls, float* xin,
        float* condExp, int* dataPoints, float* xvals, float* yvals);
void computeStateMinMax(int noControls, int noDims, int noPaths,
        int* dataPoints, float* xvals, float* xmins, float* xmaxes);
void interpolateMulti(int points, int noDims, int dimRes, float* surrogate,
        float* predictors, float* results);
void createQueryPoints(int noPoints, int noDims, int dimRes, int control,
        int noControls, int year, float* xmins, float* xmaxes,
        float* regression, float* queryPts);
void firstPeriodInduction(int noPaths, int nYears, int noSpecies,
        int noControls, float timeStep, float unitCost, float unitRevenue,
        float rrr, int noFuels, int noCommodities, float* Q, float* fuelCosts,
        float* totalPops, float* speciesParams, int* controls, float* aars,
        float* uComposition, float* uResults, int* fuelIdx, float* condExp,
        int* optCont, float* stats);
void backwardInduction(int start, int noPaths, int nYears, int noSpecies,
        int noControls, int noUncertainties, float timeStep, float unitCost,
        float unitRevenue, float rrr, int noFuels, int noCommodities,
        int dimRes, float* Q, float* fuelCosts, float* totalPops,
        float* speciesParams, int* controls, float* aars, float* regression,
        float* uComposition, float* uResults, int* fuelIdx, float* condExp,
        int* optCont, float* adjPops, float* unitProfits, float* regCoeffs);
void multiLocLinReg(int noPoints, int noDims, int dimRes, int nYears,
        int noControls, int year, int control, int k, int* dataPoints,
        float* xvals, float* yvals, float* regression, float* xmins,
        float* xmaxes, float* dist, int* ind);
void rovCorrection(int noPoints, int noDims, int dimRes, int nYears,
        int noControls, int year, int control, float* regression);
void cuComputeDistanceTexture(int wA, float* B, int wB, int pB, int dim,
        float* AB);
void cuInsertionSort(float* dist, int dist_pitch, int* ind, int ind_pitch,
        int width, int height, int k);
void cuParallelSqrt(float* dist, int width, int pitch, int k);
namespace SimulateGPU {
void dense2Sparse(float* denseIn, int rows, int cols, float* sparseOut,
                  int* elemsPerCol, int* rowIdx, int& totalElements);
}
/* ---- include/utilities/labelmethod.cpp -------------------------------- */
int LabelImage(unsigned short width, unsigned short height, int* input,
               int* output);

static inline void set_thread(unsigned bx, unsigned by) {
    blockDim.x = blockDim.y = blockDim.z = 1;
    threadIdx.x = threadIdx.y = threadIdx.z = 0;
    blockIdx.x = bx; blockIdx.y = by; blockIdx.z = 0;
}

extern "C" {

int ref_label_image(int W, int H, const int* input, int* output) {
    std::vector<int> in(input, input + (size_t)W * H);
    std::memset(output, 0, sizeof(int) * (size_t)W * H);
    return LabelImage((unsigned short)W, (unsigned short)H, in.data(), output);
}

/* SimulateGPU::buildPatches, SimulateGPU.cu:3573-3645 */
int ref_build_patches(int W, int H, int skpx, int skpy, int xres, int yres,
                      int n_regions, double xspacing, double yspacing,
                      double sub_patch_area, double max_pop, const int* labels,
                      const double* pops, double* area, double* cap,
                      double* pop, double* cx, double* cy, int* n_patches) {
    int n = xres * yres * n_regions;
    std::vector<float> res((size_t)5 * n);
    std::vector<float> popsf((size_t)W * H);
    for (size_t i = 0; i < popsf.size(); ++i) popsf[i] = (float)pops[i];
    gridDim.x = n; gridDim.y = 1;
    for (int i = 0; i < n; ++i) {
        set_thread((unsigned)i, 0);
        patchComputation(n, W, H, skpx, skpy, xres, yres,
                         (float)sub_patch_area, (float)xspacing,
                         (float)yspacing, (float)max_pop, n_regions, labels,
                         popsf.data(), res.data());
    }
    int added = 0;
    for (int i = 0; i < n; ++i) {
        if (res[5 * i] > 0) {
            int o = (*n_patches)++;
            area[o] = (double)res[5 * i];
            cx[o] = (double)res[5 * i + 3];
            cy[o] = (double)res[5 * i + 4];
            pop[o] = (double)res[5 * i + 2];
            cap[o] = (double)res[5 * i + 1];
            ++added;
        }
    }
    return added;
}

/* SimulateGPU::lineSegmentIntersect, SimulateGPU.cu:3478-3568 */
void ref_line_segment_intersect(int T, const double* xy1, int G,
                                const double* xy2, int* crossings) {
    std::vector<float> x43(G), y43(G), x21(T), y21(T), a(4 * (size_t)T),
        b(4 * (size_t)G);
    for (int g = 0; g < G; ++g) {
        x43[g] = (float)(xy2[g + 2 * G] - xy2[g]);
        y43[g] = (float)(xy2[g + 3 * G] - xy2[g + G]);
    }
    for (int t = 0; t < T; ++t) {
        x21[t] = (float)(xy1[t + 2 * T] - xy1[t]);
        y21[t] = (float)(xy1[t + 3 * T] - xy1[t + T]);
    }
    for (size_t i = 0; i < a.size(); ++i) a[i] = (float)xy1[i];
    for (size_t i = 0; i < b.size(); ++i) b[i] = (float)xy2[i];
    std::vector<int> adj((size_t)T * G);
    gridDim.x = T * G; gridDim.y = 1;
    for (int i = 0; i < T * G; ++i) {
        set_thread((unsigned)i, 0);
        pathAdjacencyKernel(T, G, a.data(), b.data(), x43.data(), y43.data(),
                            x21.data(), y21.data(), adj.data());
    }
    for (int t = 0; t < T; ++t) {
        set_thread((unsigned)t, 0);
        roadCrossingsKernel(T, G, adj.data(), crossings);
    }
}

/* dense2Sparse, SimulateGPU.cu:5973-5996 */
int ref_dense2sparse(int N, const float* dense_colmajor, float* vals,
                     int* elems_per_col, int* row_idx) {
    std::vector<float> d(dense_colmajor, dense_colmajor + (size_t)N * N);
    int total = 0;
    SimulateGPU::dense2Sparse(d.data(), N, N, vals, elems_per_col, row_idx,
                              total);
    return total;
}

/* simulateMTECUDA for one species, SimulateGPU.cu:3680-3843, with the
 * cuRAND arrays replaced by the given streams (reference layouts:
 * rgr[p*(Y*N) + t*N + k], others [p*Y + t]).  mmm is destination-major
 * (Eigen column-major) N x N. */
void ref_simulate_mte(int n_paths, int n_years, int N, float dt,
                      const float* params8, const float* init_pops,
                      const float* caps, const float* mmm, const float* rgr,
                      const float* brownians, const float* jump_sizes,
                      const float* jumps, float* end_pops) {
    std::vector<float> vals((size_t)N * N);
    std::vector<int> epc(N), rows((size_t)N * N);
    int total = ref_dense2sparse(N, mmm, vals.data(), epc.data(), rows.data());
    (void)total;
    std::vector<float> sp(params8, params8 + 8), ip(init_pops, init_pops + N),
        cp(caps, caps + N);
    std::vector<float> g(rgr, rgr + (size_t)n_paths * n_years * N);
    std::vector<float> br(brownians, brownians + (size_t)n_paths * n_years);
    std::vector<float> js(jump_sizes, jump_sizes + (size_t)n_paths * n_years);
    std::vector<float> jp(jumps, jumps + (size_t)n_paths * n_years);
    std::vector<float> path_pops((size_t)n_paths * 2 * N);
    gridDim.x = n_paths; gridDim.y = 1;
    for (int p = 0; p < n_paths; ++p) {
        set_thread((unsigned)p, 0);
        mteKernel(n_paths, n_years, N, dt, g.data(), br.data(), js.data(),
                  jp.data(), sp.data(), ip.data(), cp.data(), vals.data(),
                  rows.data(), epc.data(), path_pops.data(), end_pops);
    }
}

/* SimulateGPU::expPV, SimulateGPU.cu:3163-3259; streams are the flat
 * arrays the reference fills with cuRAND.  params as or_exp_pv. */
void ref_exp_pv(int n_paths, int n_years, const float* prm,
                const float* brownian, const float* jump_size,
                const float* jump, float* values, double* mean, double* sd) {
    gridDim.x = n_paths; gridDim.y = 1;
    for (int p = 0; p < n_paths; ++p) {
        set_thread((unsigned)p, 0);
        expPVPath(n_paths, prm[0], n_years, prm[1], prm[2], prm[3], prm[4],
                  prm[5], prm[6], brownian, jump_size, jump, values);
    }
    double total = 0.0;
    for (int p = 0; p < n_paths; ++p) total += values[p];
    double m = total / (double)n_paths;
    total = 0.0;
    for (int p = 0; p < n_paths; ++p) total += std::pow(values[p] - m, 2);
    *mean = m;
    *sd = std::sqrt(total);
}

/* knn_cuda_with_indexes::knn (knn_cuda_with_indexes.cu:475-618), texture
 * form: ref and query dim-major; dist/ind [kk*Q + q], ind 1-based */
void ref_knn(const float* ref_pts, int n, const float* query, int Q, int dim,
             int k, float* dist_out, int* ind_out) {
    std::vector<float> ab((size_t)n * Q);
    std::vector<int> ind((size_t)n * Q);
    std::vector<float> qv(query, query + (size_t)Q * dim);
    texA.data = ref_pts;
    texA.width = n;
    for (int y = 0; y < n; ++y)
        for (int x = 0; x < Q; ++x) {
            set_thread((unsigned)x, (unsigned)y);
            cuComputeDistanceTexture(n, qv.data(), Q, Q, dim, ab.data());
        }
    for (int x = 0; x < Q; ++x) {
        set_thread((unsigned)x, 0);
        cuInsertionSort(ab.data(), Q, ind.data(), Q, Q, n, k);
    }
    for (int y = 0; y < k; ++y)
        for (int x = 0; x < Q; ++x) {
            set_thread((unsigned)x, (unsigned)y);
            cuParallelSqrt(ab.data(), Q, Q, k);
        }
    for (size_t i = 0; i < (size_t)k * Q; ++i) { dist_out[i] = ab[i]; ind_out[i] = ind[i]; }
}

/* SimulateGPU::simulateROVCUDA, ALGO4 branch (SimulateGPU.cu:3870-5003) for
 * one species, with every cuRAND array passed in its reference layout:
 *   rand_cont[P*Y], rgr[P*Y*N], sp_br/sp_js/sp_jp[P*Y], ex_br/ex_js/ex_jp
 *   [P*Y*U], ucomp[P*Y*Cm] (commodity-major as generated).
 * Outputs: cond_exp/opt_cont/unit_profits [Y*P], adj_pops [Y*P],
 * regression [Y*C*(R*d + 2R^d)], stats[3]. */
void ref_simulate_rov(int P, int Y, int N, int C, int U, int R, float dt,
                      const float* params8, const float* init_pops,
                      const float* caps, const float* mmm_cnn, const float* flows,
                      const float* uncert, int n_fuels, const float* fuel_costs,
                      const int* fuel_idx, int n_comm, float unit_cost,
                      float unit_revenue, float rrr, const float* rand_cont,
                      const float* rgr, const float* sp_br, const float* sp_js,
                      const float* sp_jp, const float* ex_br, const float* ex_js,
                      const float* ex_jp, const float* ucomp, float* cond_exp,
                      int* opt_cont, float* unit_profits, float* adj_pops,
                      float* regression, float* stats) {
    const int S = 1, d = 2;
    const float scaling = 2.0f;
    int maxElements = 0;
    std::vector<float> sparseAll((size_t)C * N * N);
    std::vector<int> rowAll((size_t)C * N * N), epcAll((size_t)C * N);
    for (int c = 0; c < C; ++c) {
        int tot = ref_dense2sparse(N, mmm_cnn + (size_t)c * N * N,
                                   sparseAll.data() + (size_t)c * N * N,
                                   epcAll.data() + (size_t)c * N,
                                   rowAll.data() + (size_t)c * N * N);
        if (tot > maxElements) maxElements = tot;
    }
    int me = maxElements > 0 ? maxElements : 1;
    std::vector<float> d_sparse((size_t)C * me);
    std::vector<int> d_row((size_t)C * me);
    for (int c = 0; c < C; ++c) {
        for (int i = 0; i < me; ++i) {
            d_sparse[(size_t)c * me + i] = sparseAll[(size_t)c * N * N + i];
            d_row[(size_t)c * me + i] = rowAll[(size_t)c * N * N + i];
        }
    }
    std::vector<float> sp(params8, params8 + 8), ip(init_pops, init_pops + N),
        cp(caps, caps + N), up(uncert, uncert + 6 * U), fc(fuel_costs, fuel_costs + n_fuels),
        Qv(flows, flows + C);
    std::vector<int> fi(fuel_idx, fuel_idx + n_fuels);
    std::vector<float> rc(rand_cont, rand_cont + (size_t)P * Y);
    std::vector<int> controls((size_t)P * Y);
    gridDim.x = P * Y; gridDim.y = 1;
    for (int i = 0; i < P * Y; ++i) {
        set_thread((unsigned)i, 0);
        randControls(P, Y, C, rc.data(), controls.data());
    }
    std::vector<float> g(rgr, rgr + (size_t)P * Y * N);
    std::vector<float> a1(sp_br, sp_br + (size_t)P * Y), a2(sp_js, sp_js + (size_t)P * Y),
        a3(sp_jp, sp_jp + (size_t)P * Y);
    std::vector<float> b1(ex_br, ex_br + (size_t)P * Y * U), b2(ex_js, ex_js + (size_t)P * Y * U),
        b3(ex_jp, ex_jp + (size_t)P * Y * U);
    std::vector<float> uc(ucomp, ucomp + (size_t)P * Y * (n_comm > 0 ? n_comm : 1));
    std::vector<float> pops((size_t)P * (Y + 1) * N), totalPops((size_t)P * (Y + 1)),
        aars((size_t)P * (Y + 1) * C), uRes((size_t)P * (Y + 1) * U);
    for (int p = 0; p < P; ++p) {
        set_thread((unsigned)p, 0);
        forwardPathKernel(P, Y, S, N, C, U, dt, ip.data(), pops.data(), d_sparse.data(),
                          d_row.data(), epcAll.data(), me, sp.data(), cp.data(),
                          aars.data(), up.data(), controls.data(), b3.data(), b1.data(),
                          b2.data(), a3.data(), a1.data(), a2.data(), g.data(),
                          uRes.data(), totalPops.data());
    }
    const int Qn = (int)std::pow((double)R, d);
    const size_t blk = (size_t)R * d + 2 * (size_t)Qn;
    std::vector<float> condExp((size_t)P * Y), unitProfits((size_t)P * Y), adj((size_t)S * P),
        reg((size_t)Y * C * blk), regCoeffs((size_t)C * P), st(3);
    std::vector<int> optCont((size_t)P * Y);
    for (int p = 0; p < P; ++p) {
        set_thread((unsigned)p, 0);
        backwardInduction(Y - 1, P, Y, S, C, U, dt, unit_cost, unit_revenue, rrr, n_fuels,
                          n_comm, R, Qv.data(), fc.data(), totalPops.data(), sp.data(),
                          controls.data(), aars.data(), reg.data(), uc.data(), uRes.data(),
                          fi.data(), condExp.data(), optCont.data(), adj.data(),
                          unitProfits.data(), regCoeffs.data());
    }
    for (int p = 0; p < P; ++p) adj_pops[(size_t)(Y - 1) * P + p] = adj[p];
    std::vector<float> xmins((size_t)(C + 1) * d), xmaxes((size_t)(C + 1) * d);
    for (int t = Y - 2; t > 0; --t) {
        std::vector<float> xin((size_t)d * P), xvals((size_t)C * d * P), yvals((size_t)C * P);
        std::vector<int> dataPoints(C), ctemp(P);
        for (int p = 0; p < P; ++p) {
            set_thread((unsigned)p, 0);
            computePathStates(P, d, Y, C, t, unit_cost, unit_revenue, controls.data(),
                              n_fuels, fc.data(), uRes.data(), uc.data(), U, fi.data(),
                              n_comm, aars.data(), totalPops.data(), xin.data(), ctemp.data());
        }
        set_thread(0, 0);
        allocateXYRegressionData(P, C, d, Y, sp.data(), t, ctemp.data(), xin.data(),
                                 condExp.data(), dataPoints.data(), xvals.data(), yvals.data());
        computeStateMinMax(C, d, P, dataPoints.data(), xvals.data(), xmins.data(), xmaxes.data());
        for (int jj = 0; jj < C; ++jj) {
            int n = dataPoints[jj];
            int k = 0;
            if (n > 3) k = 10 * (std::log(n) + 1);
            std::vector<float> query((size_t)Qn * d), refX((size_t)n * d);
            for (int q = 0; q < Qn; ++q) {
                set_thread((unsigned)q, 0);
                createQueryPoints(Qn, d, R, jj, C, t, xmins.data(), xmaxes.data(), reg.data(),
                                  query.data());
            }
            for (int kk = 0; kk < d; ++kk)
                for (int i = 0; i < n; ++i)
                    refX[(size_t)kk * n + i] = xvals[(size_t)jj * P * d + (size_t)kk * P + i];
            std::vector<float> d_refX = refX;
            float xmn[8], xmx[8];
            for (int kk = 0; kk < d; ++kk) { xmn[kk] = xmins[C * d + kk]; xmx[kk] = xmaxes[C * d + kk]; }
            for (int kk = 0; kk < d - 1; ++kk) {
                for (int i = 0; i < n; ++i)
                    refX[(size_t)kk * n + i] = (refX[(size_t)kk * n + i] - xmn[kk]) / (xmx[kk] - xmn[kk]);
                for (int q = 0; q < Qn; ++q)
                    query[(size_t)kk * Qn + q] = (query[(size_t)kk * Qn + q] - xmn[kk]) / (xmx[kk] - xmn[kk]);
            }
            {
                int kk = d - 1;
                float den = scaling * (xmx[kk] - xmn[kk]);
                for (int i = 0; i < n; ++i)
                    refX[(size_t)kk * n + i] = (refX[(size_t)kk * n + i] - xmn[kk]) / den;
                for (int q = 0; q < Qn; ++q)
                    query[(size_t)kk * Qn + q] = (query[(size_t)kk * Qn + q] - xmn[kk]) / den;
            }
            std::vector<float> dist((size_t)(k > 0 ? k : 1) * Qn);
            std::vector<int> ind((size_t)(k > 0 ? k : 1) * Qn);
            if (k > 0) ref_knn(refX.data(), n, query.data(), Qn, d, k, dist.data(), ind.data());
            float zmin[8] = {0, 0, 0, 0, 0, 0, 0, 0}, zmax[8] = {1, 1, 1, 1, 1, 1, 1, 1};
            for (int q = 0; q < Qn; ++q) {
                set_thread((unsigned)q, 0);
                if (k > 0 || n < 3)
                    multiLocLinReg(Qn, d, R, Y, C, t, jj, k, dataPoints.data(), d_refX.data(),
                                   yvals.data() + (size_t)jj * P, reg.data(), zmin, zmax,
                                   dist.data(), ind.data());
            }
        }
        for (int p = 0; p < P; ++p) {
            set_thread((unsigned)p, 0);
            backwardInduction(t, P, Y, S, C, U, dt, unit_cost, unit_revenue, rrr, n_fuels,
                              n_comm, R, Qv.data(), fc.data(), totalPops.data(), sp.data(),
                              controls.data(), aars.data(), reg.data(), uc.data(), uRes.data(),
                              fi.data(), condExp.data(), optCont.data(), adj.data(),
                              unitProfits.data(), regCoeffs.data());
        }
        for (int p = 0; p < P; ++p) adj_pops[(size_t)t * P + p] = adj[p];
    }
    set_thread(0, 0);
    firstPeriodInduction(P, Y, S, C, dt, unit_cost, unit_revenue, rrr, n_fuels, n_comm,
                         Qv.data(), fc.data(), totalPops.data(), sp.data(), controls.data(),
                         aars.data(), uc.data(), uRes.data(), fi.data(), condExp.data(),
                         optCont.data(), st.data());
    for (size_t i = 0; i < (size_t)P * Y; ++i) {
        cond_exp[i] = condExp[i];
        opt_cont[i] = optCont[i];
        unit_profits[i] = unitProfits[i];
    }
    for (size_t i = 0; i < reg.size(); ++i) regression[i] = reg[i];
    for (int i = 0; i < 3; ++i) stats[i] = st[i];
}

/* SimulateGPU::buildSurrogateROVCUDA (SimulateGPU.cu:5694-5917), mean
 * surface (with rovCorrection) or SD surface; predictors dim-major [d][n] */
void ref_build_surrogate_rov(int n, int d, const float* pred, const float* y, int R,
                             int correct, float* out) {
    int k;
    if (n < 50) k = 5;
    else if (n < 100) k = (int)(5 + 5 * std::ceil((n - 50) / 50));
    else if (n < 500) k = (int)std::ceil(10 + 15 * std::ceil((n - 100) / 400));
    else k = (int)(25 + std::ceil((n - 500) * 0.02));
    k = std::min(n, k);
    int Qn = (int)std::pow((double)R, d);
    std::vector<float> xv(pred, pred + (size_t)d * n), yv(y, y + n);
    std::vector<float> xmins((size_t)2 * d), xmaxes((size_t)2 * d);
    int samples = n;
    set_thread(0, 0);
    computeStateMinMax(1, d, n, &samples, xv.data(), xmins.data(), xmaxes.data());
    std::vector<float> sur((size_t)R * d + Qn), query((size_t)Qn * d);
    for (int q = 0; q < Qn; ++q) {
        set_thread((unsigned)q, 0);
        createQueryPoints(Qn, d, R, 0, 1, 0, xmins.data(), xmaxes.data(), sur.data(), query.data());
    }
    std::vector<float> pn = xv;
    for (int j = 0; j < d; ++j) {
        float lo = pn[(size_t)j * n], hi = lo;
        for (int m = 0; m < n; ++m) { lo = std::min(lo, pn[(size_t)j * n + m]); hi = std::max(hi, pn[(size_t)j * n + m]); }
        for (int m = 0; m < n; ++m) pn[(size_t)j * n + m] = (pn[(size_t)j * n + m] - lo) / (hi - lo);
        for (int q = 0; q < Qn; ++q) query[(size_t)j * Qn + q] = (query[(size_t)j * Qn + q] - lo) / (hi - lo);
    }
    std::vector<float> dist((size_t)k * Qn);
    std::vector<int> ind((size_t)k * Qn);
    ref_knn(pn.data(), n, query.data(), Qn, d, k, dist.data(), ind.data());
    float zmin[8] = {0, 0, 0, 0, 0, 0, 0, 0}, zmax[8] = {1, 1, 1, 1, 1, 1, 1, 1};
    for (int q = 0; q < Qn; ++q) {
        set_thread((unsigned)q, 0);
        multiLocLinReg(Qn, d, R, 1, 1, 0, 0, k, &samples, xv.data(), yv.data(), sur.data(),
                       zmin, zmax, dist.data(), ind.data());
    }
    if (correct)
        for (int q = 0; q < Qn; ++q) {
            set_thread((unsigned)q, 0);
            rovCorrection(Qn, d, R, 1, 1, 0, 0, sur.data());
        }
    for (size_t i = 0; i < sur.size(); ++i) out[i] = sur[i];
}

/* SimulateGPU::interpolateSurrogateMulti's kernel (SimulateGPU.cu:3077-3155)
 * over n points (float, as the wrapper casts its inputs) */
void ref_interpolate_multi(int n, int d, int R, const float* sur, const float* pred,
                           float* out) {
    std::vector<float> s(sur, sur + (size_t)R * d + (size_t)std::pow((double)R, d));
    std::vector<float> p(pred, pred + (size_t)n * d);
    for (int i = 0; i < n; ++i) {
        set_thread((unsigned)i, 0);
        interpolateMulti(n, d, R, s.data(), p.data(), out);
    }
}

}  /* extern "C" */
