// to_rov.cuh - argument block of the ROV kernels and the kNN / regression
// launchers shared with the surrogate builders.
#pragma once
#include "to_internal.cuh"
#include "to_lsm_math.h"

#define TO_ROV_MAXC 8
#define TO_KNN_KMAX 256
#define TO_KNN_GCELLS 4096

// uniform cell grid over one control's normalised regression points:
// cell_j(x) = clamp(floor((x - lo_j) * inv_j), 0, G_j - 1), dimension 0
// fastest; ok = 0 when a coordinate is not finite (full scan instead)
struct to_knn_grid {
    float lo[TO_LSM_MAXD], hi[TO_LSM_MAXD], inv[TO_LSM_MAXD], w[TO_LSM_MAXD];
    int G[TO_LSM_MAXD];
    int ok;
    float T0;                 // first squared-distance threshold of a query
};

// A batch of nr roads with the same dimensions: path arrays are road-major
// ([..][PT], road r's paths at r*P .. r*P+P-1) and the regressions are
// grouped by (road, control), group g = r*C + c.
struct to_rov_args {
    int P, Y, S, C, U, R, Q;          // paths per road, years, species, controls, processes, dimRes, R^d
    int nr, PT, G;                    // roads, paths of all roads (nr*P), groups (nr*C)
    const int* road_ids;              // [nr] road id of each road (random streams)
    int nF, Cm, demand_idx, sem, road;
    float dt, rrr, unit_cost, unit_revenue, scaling;
    uint64_t seed;
    int np, ne;                       // stride / effective width of patch arrays
    int tile_paths, l_chunk;          // forward tile (launcher)
    // inputs (device)
    const int* n_patches;             // [nr][S]
    const float* params;              // [S*8]
    const float* init_pops;           // [nr][S][np]
    const float* caps;                // [nr][S][np] (padding 1)
    const float* mmm;                 // [nr][S][C][np][np] destination-major
    const float* flows;               // [C]
    const float* uncert;              // [U*6]
    const float* fuel_costs;          // [nF]
    const int* fuel_idx;              // [nF]
    const float* ore_content;         // [Cm]
    const float* ore_sd;              // [Cm]
    // path state (device)
    int* controls;                    // [Y][PT]
    float* uRes;                      // [U][Y+1][PT]
    float* totalPops;                 // [S][Y+1][PT]
    float* aars;                      // [S][C][Y][PT]
    // regression scratch (device), per group g = r*C + c
    float* xraw;                      // [G][d][P] compacted raw states
    float* xn;                        // [G][d][P] normalised
    float* yv;                        // [G][P]
    int* npts;                        // [G]
    int* kc;                          // [G]
    float* gmin;                      // [nr][d]
    float* gmax;                      // [nr][d]
    float* qax;                       // [nr][d][R] normalised grid axes of the year (may be null)
    float* gsx;                       // [G][d][P] points in cell order
    int* gsi;                         // [G][P] their original indices
    int* gcell;                       // [G][TO_KNN_GCELLS + 1] cell starts
    to_knn_grid* ggrid;               // [G]
    float* kth;                       // [G][Q] k-th squared distance, year before
    int* lcnt;                        // [G][lblocks] points per group and path chunk
    unsigned* lkey;                   // [G][d][2] min / max keys of the states
    int lblocks;                      // path chunks of the compaction
    int k_mult;                       // k = k_mult (ln n + 1): 10 ALGO4, 3 ALGO6
    int algo;                         // 4 or 6
    float* popsY;                     // ALGO6: [Y][S][ne][P] patch populations, start of year
    float* gmY;                       // ALGO6: [Y][S][P] mean growth rate of the year
    int* knn_next;                    // work counter of the kNN kernel
    double* knn_acc;                  // [G*Q][(d+1)(d+4)/2] normal-equation sums per listed query
    int kmax;
    // touched-query mode (corrected semantics, ALGO4, surfaces not
    // returned): a year's regressions are fitted only at the grid queries
    // some path's interpolation reads; the others are never read
    int touched;
    unsigned char* qmark;             // [G][Q] marks of the current year (kept zero between years)
    int* qlist;                       // [G*Q] flat items g*Q + q of the marked queries
    int* qcount;                      // number of entries in qlist
    unsigned* qroad;                  // [nr] queries fitted per road over the years (may be null)
    // 1: reg holds only the current year's blocks (the regressions of year
    // t are written and read within year t; nothing returns them)
    int reg_one_year;
    int* flags;                       // device error word (plan checks), may be null
    // outputs (device)
    float* reg;                       // [Y][G][R*d + 2Q]
    float* condExp;                   // [Y][PT]
    int* optCont;                     // [Y][PT]
    float* unitProfits;               // [Y][PT]
    float* adjPops;                   // [Y][S][PT]
    double* stats;                    // [nr][5]: value, control, SD, SE, n
};

// regression block of (year t, group g): axis values [R*d], then the Q
// grid values, then Q standard deviations
__host__ __device__ __forceinline__ float* to_rov_reg_block(const to_rov_args& a, int t, size_t g) {
    const size_t blk = (size_t)a.R * (a.S + 1) + 2 * (size_t)a.Q;
    return a.reg + ((size_t)(a.reg_one_year ? 0 : t) * a.G + g) * blk;
}

// grid query q of the current year: normalised coordinates (for kNN) and
// the coordinates the regression centres on (createQueryPoints + host
// normalisation; sem 0 centres on the unit grid, SimulateGPU.cu:2964-2966)
template <int D>
__device__ __forceinline__ void to_rov_query(const to_rov_args& a, int road, int q, float* qn,
                                             float* xq) {
    const int R = a.R;
    const float* lo = a.gmin + (size_t)road * D;
    const float* hi = a.gmax + (size_t)road * D;
    const float* ax = a.qax ? a.qax + (size_t)road * D * R : nullptr;
    const bool pow2 = (R & (R - 1)) == 0;
    const int lr = pow2 ? __ffs(R) - 1 : 0;           // log2 R
    int rem = q;
    int div = a.Q / R;
#pragma unroll
    for (int j = 0; j < D; ++j) {
        int di;
        if (pow2) {
            // q's base-R digit of dimension j (dimension 0 most significant)
            di = (q >> (lr * (D - 1 - j))) & (R - 1);
        } else {
            di = rem / div;
            rem -= di * div;
            div /= R;
        }
        // the year's normalised axis values, computed once per road
        // (k_lsm_stats) with the same operations
        const float nv = ax ? ax[j * R + di]
                            : to_lsm_normalise(to_lsm_query_axis(di, lo[j], hi[j], R), lo[j],
                                               hi[j], j == a.S, a.scaling);
        qn[j] = nv;
        xq[j] = (a.sem == 0) ? to_lsm_unit_axis(di, R) : nv;
    }
}

struct to_csc;
namespace to_k {
// csc: the packed migration matrices for the sparse forward pass, or null
to_status rov_run(to_ctx ctx, to_rov_args a, const to_csc* csc);
// kNN + local linear regressions of year t (cell grid, then fused kernel)
to_status knn_rov(to_ctx ctx, const to_rov_args& a, int t);
// generic kNN: ref dim-major [dim][n], query dim-major [dim][Q]
to_status knn(to_ctx ctx, const float* ref, int n, const float* query, int Q,
              int dim, int k, float* dist, int* ind);
}
