/*
 * ref_harness.cpp - host-side drivers for the reference kernels compiled by
 * oracle/build_ref.sh.  Each driver restates the reference's host wrapper
 * (allocation and copies dropped; launches replaced by loops over the grid)
 * and takes the random streams as arrays in the reference's own layout, so
 * that the reference arithmetic runs on exactly the inputs the oracle sees.
 * TEST INFRASTRUCTURE ONLY; built into oracle/_ref/ and never shipped.
 */
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

}  /* extern "C" */
