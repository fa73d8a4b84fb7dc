/*
 * oracle.h - CPU restatement of the reference's Monte Carlo road-evaluation
 * path (TransportOptimiser, include/gpuCode/SimulateGPU.cu and the host code
 * that feeds it).  TEST INFRASTRUCTURE ONLY: the tests, the smoke check and
 * bench.py's CPU-baseline leg load it as the checker.  The product
 * (libtransopt.so) never links or calls it.
 *
 * Parity pin: the reference ships no golden outputs for this path.  The
 * oracle is pinned against the reference's own kernels, compiled for the
 * host CPU from their source lines by oracle/build_ref.sh (outputs in
 * oracle/_ref/, only where the reference tree is mounted), through the
 * committed fixtures in tests/golden/.
 *
 * Arithmetic: the oracle is compiled with -ffp-contract=off and writes every
 * fused multiply-add explicitly, matching the CUDA kernels (built with
 * --fmad=false and the same explicit fmaf calls), so that the SIMT GPU path
 * and this file agree bit for bit on identical inputs.
 *
 * Semantics: sem = 0 reproduces the reference's arithmetic quirks exactly
 * (the "Q" notes next to each function); sem = 1 is the corrected model.
 */
#ifndef TO_ORACLE_H
#define TO_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* labelmethod.cpp:34-56 */
int or_label_image(int W, int H, const int* input, int* output);

/* SimulateGPU.cu:498-573 (patchComputation) + 3573-3645 (buildPatches).
 * Appends patches starting at *n_patches; returns the number appended. */
int or_build_patches(int W, int H, int skpx, int skpy, int xres, int yres,
                     int n_regions, double xspacing, double yspacing,
                     double sub_patch_area, double max_pop, const int* labels,
                     const double* pops, double* area, double* cap,
                     double* pop, double* cx, double* cy, int* n_patches);

/* SimulateGPU.cu:454-493 + 3478-3568; xy1 is T x 4, xy2 is G x 4, both
 * column-major (x1 | y1 | x2 | y2) as the reference's Eigen matrices. */
void or_line_segment_intersect(int T, const double* xy1, int G,
                               const double* xy2, int* crossings);

typedef struct {
    int type;              /* habitat type code (0..2 habitable here)      */
    double max_pop;        /* capacity per unit area                        */
    double pref_mean;      /* habitat preference mean                       */
    double pref_sd;        /* habitat preference sd                         */
} or_habitat;

typedef struct {
    int W, H, res;                 /* grid cells and coarse resolution    */
    double xspacing, yspacing;
    double x0, y0;                 /* unused by the GPU patch path        */
    int n_hab;                     /* habitat types of the species        */
    const or_habitat* habs;
    const int* hab_map;            /* W*H type codes, col-major x + y*W   */
    const double* pop_map;         /* W*H initial animals                 */
    int G;                         /* visible road segments               */
    const double* road;            /* G x 4 col-major                     */
    double lambda_mean, lambda_sd, lambda_mult, hab_pref_mult;
    int n_controls;
    const double* hazard;          /* per control: Q_c (w + len)/(spd 3600) */
    int sem;
} or_species_in;

typedef struct {
    int max_patches;               /* capacity of the arrays below         */
    int n_patches;
    double *area, *cap, *pop, *cx, *cy;
    int* type;
    double* dists;                 /* N*N row-major                        */
    int* crossings;                /* N*N row-major                        */
    double* trans;                 /* N*N row-major origin x destination   */
    double* surv;                  /* C*N*N                                */
    float* mmm;                    /* C*N*N, destination-major: [c][k][l]  */
    int n_transitions;             /* pairs tested for crossings           */
    double* iar;                   /* [C] initial animals at risk (may be NULL) */
} or_species_out;

/* SpeciesRoadPatches.cpp:12-451 + SimulateGPU.cu:5973-5996 (dense2Sparse
 * threshold kept as explicit zeros) */
int or_species_model(const or_species_in* in, or_species_out* out);

/* SimulateGPU.cu:595-717 + 3650-3864.  mmm: N*N destination-major for the
 * highest-flow control.  end_pops: n_paths floats. */
/* RoadCells::computeRoadCells (RoadCells.cpp:10-272): sorted unique cells
 * x + y W of a polyline of n points; returns the count (cells holds at most
 * cap of them) */
int or_road_cells(int n, const double* x, const double* y, int W, int H, double xs, double ys,
                  int sem, int* cells, int cap);
/* compressed columns of a destination-major N x N matrix (entries > 0,
 * ascending origin order); idx / val may be NULL to count only */
int or_pack_csc(int N, const float* mmm, int* ptr, int* idx, float* val);
void or_simulate_mte(int n_paths, int n_years, int N, float dt,
                     const float* params8, const float* init_pops,
                     const float* caps, const float* mmm, uint64_t seed,
                     int road, int species, int sem, int n_threads,
                     float* end_pops);

/* SimulateGPU.cu:256-279 + 3163-3259.  params: {gr, meanP, timeStep, rrr,
 * current, reversion, jumpProb, noiseSD, poissonJump}; returns the per-path
 * values and the reference's (mean, "SD") pair. */
void or_exp_pv(int n_paths, int n_years, const float* params, uint64_t seed,
               int road, int sem, float* values, double* mean, double* sd);

/* patch totals: groups of four, ((v0 + v1) + v2) + v3, groups ascending */
float or_grouped_sum(const float* v, int N);

/* stream helpers for tests (materialise the fused streams) */
void or_fill_stream(uint64_t seed, int stream, int road, int normal,
                    int n_paths, int n_years, int L, int lane_offset,
                    float* out);
void or_fill_pv_stream(uint64_t seed, int stream, int road, int normal,
                       long n, float* out);
float or_normal(uint64_t seed, int stream, int road, int path, int year,
                int lane);
float or_uniform(uint64_t seed, int stream, int road, int path, int year,
                 int lane);

#ifdef __cplusplus
}
#endif
#endif
