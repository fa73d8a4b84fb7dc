/*
 * transopt.h - C ABI of the GB300 (sm_103a) Monte Carlo road-evaluation
 * engine.  It replaces the GPU entry points of TransportOptimiser's
 * `namespace SimulateGPU` (include/gpuCode/SimulateGPU.h:34-482) and the
 * vendored kNN (include/gpuCode/knn_cuda_with_indexes.h:4-47).
 *
 * Conventions
 *   - Every entry point returns a to_status; nothing throws across the ABI
 *     (the reference threw `const char*`, SimulateGPU.cu:14-26).
 *   - Functions without a `_d` suffix take HOST pointers and do their own
 *     host<->device copies, like the reference wrappers (which allocated,
 *     copied, launched and synchronised inside every call).  `_d` variants
 *     take DEVICE pointers and enqueue on the context's stream.
 *   - Scratch memory comes from a per-context arena that grows on demand and
 *     is reused between calls.
 *   - Matrices keep the reference's layouts where a caller passes them in:
 *     segment lists are G x 4 column-major (x1 | y1 | x2 | y2), grids are
 *     column-major W x H (cell x + y*W), migration matrices are
 *     destination-major (Eigen column-major of mmm(origin, destination)).
 *   - `sem` selects TO_SEM_REFERENCE (reproduce the reference's arithmetic,
 *     quirks included) or TO_SEM_CORRECTED.
 *   - Random numbers are Philox4x32-10 streams addressed by (seed, road,
 *     stream, path, year, lane); runs are reproducible for a given seed.
 */
#ifndef TRANSOPT_H
#define TRANSOPT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    TO_OK = 0,
    TO_ERR_INVALID = 1,      /* bad argument or size                        */
    TO_ERR_CUDA = 2,         /* CUDA runtime error (message via to_last_error) */
    TO_ERR_ALLOC = 3,        /* device or host allocation failed            */
    TO_ERR_NONFINITE = 4,    /* NaN/Inf found in an input                    */
    TO_ERR_TIMEOUT = 5,      /* a bounded device wait gave up                */
    TO_ERR_UNSUPPORTED = 6,  /* size or mode outside what is built          */
    TO_ERR_NO_DEVICE = 7
} to_status;

typedef enum { TO_SEM_REFERENCE = 0, TO_SEM_CORRECTED = 1 } to_sem;

typedef enum {
    TO_MIG_AUTO = 0,         /* sparse when the matrices fit, else dense     */
    TO_MIG_SIMT_FP32 = 1,    /* dense CUDA-core FP32                         */
    TO_MIG_TC_3XTF32 = 2,    /* dense tcgen05 kind::tf32, 3 MMAs (hi/lo)     */
    TO_MIG_SPARSE_FP32 = 3   /* compressed columns in shared memory          */
} to_migration;
/* Every FP32 form sums each destination's terms in ascending origin order
 * with fused multiply-adds, so the sparse and dense CUDA-core forms are
 * bit-identical to each other and to the CPU oracle. */

typedef struct to_ctx_s* to_ctx;

/* ---- context ----------------------------------------------------------- */
/* SimulateGPU::deviceCount, SimulateGPU.h:44 */
to_status to_device_count(int* count);
to_status to_ctx_create(int device, to_ctx* ctx);
to_status to_ctx_destroy(to_ctx ctx);
/* enqueue `_d` work on a caller stream (cudaStream_t passed as void*) */
to_status to_ctx_set_stream(to_ctx ctx, void* stream);
/* wait for the context's stream; then report (and clear) what enqueued `_d`
 * work flagged on the device: TO_ERR_UNSUPPORTED (a generation outgrew its
 * captured plan, capacities exceeded) or TO_ERR_TIMEOUT (a bounded wait) */
to_status to_ctx_synchronize(to_ctx ctx);
const char* to_status_string(to_status s);
const char* to_last_error(to_ctx ctx);
/* number of kernels this context has launched (for accounting) */
uint64_t to_ctx_launch_count(to_ctx ctx);
/* Fault injection for tests of the failure paths, all on the host side or
 * in a bounded device wait (no reference counterpart).  One-shot: the armed
 * fault fires once, in the next call that reaches it.
 *   TO_FAULT_ALLOC: the next scratch reservation is refused as a failed
 *     device allocation would be (TO_ERR_ALLOC); the context stays usable.
 *   TO_FAULT_WAIT: the next tensor-core migration kernel waits on a barrier
 *     that nothing completes, before it issues any copy or MMA, with no time
 *     allowed; it takes its abort path (error word, TMEM freed) and the call
 *     returns TO_ERR_TIMEOUT; with nothing in flight the context stays
 *     usable.  (A wait that runs out while copies or MMAs are in flight is a
 *     different case: the context should then be destroyed.) */
#define TO_FAULT_NONE 0
#define TO_FAULT_ALLOC 1
#define TO_FAULT_WAIT 2
to_status to_ctx_inject_fault(to_ctx ctx, int fault);
/* per-kernel CUDA-event timing: enable (clears the record), then read the
 * summed milliseconds and launch count of one kernel by name */
to_status to_ctx_profile(to_ctx ctx, int enable);
to_status to_ctx_kernel_time(to_ctx ctx, const char* name, double* ms,
                             int* launches);

/* ---- habitat patches --------------------------------------------------- */
/* LabelImage, include/utilities/labelmethod.cpp:34.  4-connected labels of
 * input != 0 numbered 1.. in raster order of the first pixel (x + y*W).
 * One CTA per image, union-find in shared memory (W*H <= 56000). */
to_status to_label_image(to_ctx ctx, int W, int H, const int* input,
                         int* output, int* n_regions);

/* SimulateGPU::buildPatches, SimulateGPU.h:134-140 / SimulateGPU.cu:3573.
 * For one habitat type with `labels` from to_label_image, appends the
 * non-empty (coarse block x region) patches at index *n_patches in the
 * reference order (by*xres + bx)*regions + region-1.  Outputs are host
 * arrays of capacity max_patches; *init_pop accumulates the patch pops. */
to_status to_build_patches(to_ctx ctx, int W, int H, int skpx, int skpy,
                           int xres, int yres, int n_regions, double xspacing,
                           double yspacing, double sub_patch_area,
                           double max_pop, const int* labels,
                           const double* pops, int max_patches, double* area,
                           double* cap, double* pop, double* cx, double* cy,
                           double* init_pop, int* n_patches);

/* ---- road crossings ---------------------------------------------------- */
/* SimulateGPU::lineSegmentIntersect, SimulateGPU.h:107-108 /
 * SimulateGPU.cu:3478.  crossings[t] = number of segments of xy2 (G x 4)
 * that line t of xy1 (T x 4) intersects; float predicate, exact. */
to_status to_line_segment_intersect(to_ctx ctx, int T, const double* xy1,
                                    int G, const double* xy2, int* crossings);

/* ---- species-road model ------------------------------------------------ */
typedef struct {
    int type;                /* habitat code in hab_map                       */
    double max_pop;          /* capacity per unit area                        */
    double pref_mean;        /* habitat preference                            */
    double pref_sd;
} to_habitat;

typedef struct {
    int W, H, res;           /* grid cells; coarse patch resolution           */
    double xspacing, yspacing;
    int n_hab;
    const to_habitat* habs;  /* host array                                    */
    const int* hab_map;      /* W*H habitat codes, road cells already ROAD(4) */
    const double* pop_map;   /* W*H animals                                   */
    int G;                   /* visible road segments                         */
    const double* road;      /* G x 4 column-major                            */
    double lambda_mean, lambda_sd, lambda_mult, hab_pref_mult;
    int n_controls;
    const double* hazard;    /* per control Q_c (vehicle width + length)/(speed 3600) */
    int sem;
} to_species_in;

typedef struct {
    int max_patches;         /* capacity of every array below                 */
    int n_patches;           /* out                                           */
    int n_transitions;       /* out: patch pairs tested against the road      */
    double *area, *cap, *pop, *cx, *cy;  /* [max_patches]                   */
    int* type;               /* index into habs                               */
    int* crossings;          /* N*N row-major (optional, may be NULL)         */
    double* trans;           /* N*N row-major origin x destination (optional) */
    double* surv;            /* C*N*N (optional)                              */
    float* mmm;              /* C*N*N destination-major [c][k][l] (optional)  */
    double* iar;             /* [C] initial animals at risk per control,
                                SpeciesRoadPatches::computeInitialAAR,
                                SpeciesRoadPatches.cpp:453-490 (optional)     */
} to_species_out;

/* SpeciesRoadPatches::createSpeciesModel, SpeciesRoadPatches.cpp:12-451, on
 * the device: labels, patches, distances, crossings, transition and
 * survival probabilities, and the migration matrices mmm_c = trans o surv_c
 * (float, entries <= 1e-5 set to zero as dense2Sparse drops them,
 * SimulateGPU.cu:5973). */
to_status to_species_model(to_ctx ctx, const to_species_in* in,
                           to_species_out* out);

/* ---- MTE --------------------------------------------------------------- */
typedef struct {
    int n_patches;           /* N                                              */
    const float* params;     /* [8]: growth current, mean, sd, threshold,
                                reversion, jump size, jump prob, local var.
                                (SimulateGPU.cu:3694-3714)                    */
    const float* init_pops;  /* [N]                                           */
    const float* caps;       /* [N]                                           */
    const float* mmm;        /* [N*N] destination-major, highest-flow control */
} to_mte_species;

typedef struct {
    int n_species, n_paths, n_years;
    float dt;
    uint64_t seed;
    int road;                /* stream id of the road                         */
    int sem;
    int migration;           /* to_migration                                  */
    const to_mte_species* species;  /* host array [n_species]                */
} to_mte_problem;

typedef struct {
    double mean, sd;         /* end population (Simulator.cpp:184-191 SD)     */
    double se;               /* Monte Carlo standard error of the mean        */
    double p_below;          /* P(end < 0.2 x initial population)             */
    double init_total;
} to_mte_stats;

/* SimulateGPU::simulateMTECUDA, SimulateGPU.h:152-156 / SimulateGPU.cu:3650.
 * end_pops (optional) is n_paths x n_species column-major (species-major),
 * like the reference's endPops; stats (optional) is [n_species]. */
to_status to_simulate_mte(to_ctx ctx, const to_mte_problem* prob,
                          double* end_pops, to_mte_stats* stats);


/* ---- MTE without device allocation ---------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory - a host program that has handed the whole device to its own pool
 * allocator, or one that must not add allocations (and the synchronisation
 * they imply) to a GA loop - this entry point takes every input and output
 * as caller-owned device memory and allocates nothing: the per-path end
 * populations it needs go to a fixed array compiled into the library
 * (species x paths <= 2,097,152 floats, 8 MiB held by every GPU that loads
 * the library until exit; larger problems return TO_ERR_UNSUPPORTED).
 * The first call on a device looks up that array's device address, so make
 * it before any stream capture.  All calls share the array: calls that
 * overlap on the GPU race on it.  Work is enqueued on `stream`
 * (cudaStream_t, may be 0); d_stats receives [n_species][5] doubles: mean,
 * SD, standard error, P(end < 0.2 x initial), initial population.
 * n_patches lives in device memory, so the host cannot check it: a species
 * whose n_patches[s] is negative or above npad gets NaN in all five of its
 * statistics (nothing is read past its rows) while the call still returns
 * TO_OK; NaN statistics therefore mean a patch count outside [0, npad].
 * n_species is at most 65535 (TO_ERR_UNSUPPORTED above).  A CUDA error
 * already pending on the calling thread is reported as TO_ERR_CUDA before
 * anything is enqueued, and left pending for its owner. */
typedef struct {
    int n_species, n_paths, n_years;
    int npad;                /* row stride of the arrays below, multiple of 4 */
    float dt;
    uint64_t seed;
    int road, sem;
    const int* n_patches;    /* device [n_species]                            */
    const float* params;     /* device [n_species][8]                         */
    const float* init_pops;  /* device [n_species][npad], zero padded         */
    const float* caps;       /* device [n_species][npad], padding 1.0         */
    const float* mmm;        /* device [n_species][npad][npad] destination-major,
                                zero padded                                   */
} to_mte_device_problem;

to_status to_simulate_mte_noalloc_d(void* stream,
                                    const to_mte_device_problem* prob,
                                    double* d_stats);

/* ---- expected present value of an uncertain price ---------------------- */
typedef struct {
    float gr;                /* traffic growth x time step                     */
    float mean;              /* long-run mean (x scenario multiplier)          */
    float time_step;
    float rrr;               /* discount rate                                  */
    float current;
    float reversion;         /* mean-reversion strength (x multiplier)         */
    float jump_prob;
    float noise_sd;          /* brownian sd (x time step x multiplier)         */
    float jump_sd;           /* Poisson jump size (x multiplier)               */
} to_exp_pv_params;

/* SimulateGPU::expPV, SimulateGPU.h:53 / SimulateGPU.cu:3163.  values
 * (optional) receives the per-path PV; mean and sd as the reference sets
 * expPV / expPVSD (sem 0: sd = sqrt(sum of squared deviations)). */
to_status to_exp_pv(to_ctx ctx, const to_exp_pv_params* prm, int n_paths,
                     int n_years, uint64_t seed, int road, int sem,
                     float* values, double* mean, double* sd);



/* ---- ROV (controlled traffic) --------------------------------------------- */
typedef struct {
    int n_patches;           /* N                                              */
    const float* params;     /* [8] (SimulateGPU.cu:3993-4015 layout)          */
    const float* init_pops;  /* [N]                                           */
    const float* caps;       /* [N]                                           */
    const float* mmm;        /* [C][N][N] destination-major, one per control  */
} to_rov_species;

typedef struct {
    int n_species, n_paths, n_years, n_controls, dim_res;
    const to_rov_species* species;   /* host [n_species]                      */
    const float* flows;      /* [C] traffic flow of each control (Q)           */
    int n_uncertainties;
    const float* uncert;     /* [U*6] current, mean, sd, reversion, jump size,
                                jump prob; fuels first (SimulateGPU.cu:4020-4070) */
    int n_fuels;
    const float* fuel_costs; /* [n_fuels]                                     */
    const int* fuel_idx;     /* [n_fuels] process index of each fuel term     */
    int n_commodities;
    const float* ore_content;/* [Cm]                                          */
    const float* ore_sd;     /* [Cm] (x multiplier)                           */
    float unit_cost, unit_revenue, dt, rrr;
    int demand_idx;          /* process multiplying the unit profit, -1: none */
    uint64_t seed;
    int road, sem, migration;
    int algo;                /* 4 (or 0): ALGO4, regression values; 6: ALGO6,
                                each year's value is the realised discounted
                                payoff of the path re-simulated from that year
                                under the regression-optimal controls
                                (optimalForwardPaths, SimulateGPU.cu:1199-2206,
                                5011-5436); sem 1 and sparse migration only */
} to_rov_problem;

typedef struct {
    double* cond_exp;        /* [Y][P] optional (reference condExp, P x Y)    */
    int* opt_cont;           /* [Y][P] optional                               */
    double* unit_profits;    /* [Y][P] optional                               */
    double* adj_pops;        /* [Y][S][P] optional                            */
    double* regression;      /* [Y*C*(R*d + 2 R^d)] optional, d = S + 1       */
    double value;            /* stats: road value (condExp(0))                */
    double control;          /* optimal first-period control                  */
    double sd;               /* the reference's SD statistic                  */
    double se;               /* Monte Carlo standard error of the value       */
    int n_best;              /* paths behind the value                        */
} to_rov_result;

/* SimulateGPU::simulateROVCUDA with ALGO4, SimulateGPU.h:187-191 /
 * SimulateGPU.cu:3870-5003.  Reference semantics (sem 0) need one species
 * (the reference indexes multi-species patch vectors as if shared). */
to_status to_simulate_rov(to_ctx ctx, const to_rov_problem* prob,
                          to_rov_result* res);

/* A batch of roads valued together (the batched form of simulateROVCUDA for
 * a GA generation; no reference counterpart): n_roads problems with the same
 * dimensions, processes, costs, seed and species parameters, each with its
 * own species models (patches, capacities, migration matrices) and road id.
 * One launch per stage serves every road; the regressions are per (road,
 * control).  Each road's result equals to_simulate_rov on that road alone.
 * Corrected semantics (sem 1), ALGO4, sparse migration, >= 128 paths per
 * road when n_roads > 1. */
to_status to_simulate_rov_batch(to_ctx ctx, int n_roads, const to_rov_problem* probs,
                                to_rov_result* results);

/* knn_cuda_with_indexes::knn, knn_cuda_with_indexes.h:4-47: ref (dim x n)
 * and query (dim x Q) dim-major, host pointers; dist / ind are k x Q
 * (dist[kk*Q + q], ind 1-based) in ascending (distance, index) order. */
to_status to_knn(to_ctx ctx, const float* ref, int n, const float* query,
                 int Q, int dim, int k, float* dist, int* ind);


/* ---- surrogates ------------------------------------------------------------
 * SimulateGPU::buildSurrogateMTECUDA, SimulateGPU.h:235 / SimulateGPU.cu:5533:
 * 1-D local-linear surrogate of the end population (mean, then SD) against
 * the initial animals-at-risk over dim_res grid points.  out_mean / out_sd
 * (optional) hold [dim_res x values | dim_res y values]. */
to_status to_build_surrogate_mte(to_ctx ctx, int samples, const double* iars,
                                 const double* pops_mean, const double* pops_sd,
                                 int dim_res, double* out_mean, double* out_sd);

/* SimulateGPU::buildSurrogateROVCUDA, SimulateGPU.h:244 / SimulateGPU.cu:5694:
 * predictors dim-major [n_dims][samples] (IAR per species, then unit use);
 * outputs [dim_res*n_dims axis values | dim_res^n_dims values]; the mean
 * surface is clipped at zero (rovCorrection).  sem 0 regresses on the raw
 * predictors as the reference reads them (see TO_SEM_REFERENCE). */
to_status to_build_surrogate_rov(to_ctx ctx, int samples, int n_dims,
                                 const double* predictors, const double* values,
                                 const double* values_sd, int dim_res, int sem,
                                 double* out_mean, double* out_sd);

/* ---- batched GA generation ------------------------------------------------
 * A scene (habitat map, species, initial-population maps) is uploaded once
 * and stays resident in HBM; each GA generation then streams in only the
 * road geometry (road cells and visible segments per road) and values every
 * road in a few launches: one CTA per (road, species) builds the species
 * model, one launch runs every road's Monte Carlo paths, one reduces them.
 * This batches what RoadGA::evaluateGeneration / computeSurrogate
 * (include/main/RoadGA.cpp:2040-2099, 1553-1748) do one road per call.
 */
typedef struct {
    int n_hab;
    const to_habitat* habs;  /* host [n_hab]                                  */
    const double* pop_map;   /* host W*H animals                              */
    const double* hazard;    /* host [n_controls]                             */
    const float* params;     /* host [8] (SimulateGPU.cu:3694-3714 layout)    */
    double lambda_mean, lambda_sd, lambda_mult, hab_pref_mult;
} to_species_desc;

typedef struct {
    int W, H, res;
    double xspacing, yspacing;
    const int* base_map;     /* host W*H habitat codes without roads          */
    int n_species;
    const to_species_desc* species;
    int n_controls;
    int max_patches;         /* per (road, species) capacity                  */
    int max_roads;           /* capacity of the per-generation buffers        */
    int max_cells;           /* total road cells per generation               */
    int max_segments;        /* total road segments per generation            */
} to_scene;

typedef struct to_gen_s* to_gen;

typedef struct {
    int mte_paths;           /* Monte Carlo paths per road                     */
    int n_years;
    float dt;
    uint64_t seed;
    int road0;               /* stream id of the first road                    */
    int sem;
    int migration;           /* to_migration; TO_MIG_AUTO = autotuned          */
    int graph;               /* 1: capture the generation as a CUDA graph and
                                replay it while the calls match (same roads
                                pointers and options, shapes within the plan) */
} to_eval_opts;

/* ---- pathwise sensitivities (adjoint) ------------------------------------
 * The controlled road valuation with the exercise policy frozen: per path
 * the controls c[t][p] are given (e.g. to_rov_result.opt_cont).  Outputs
 * (1 + S): E[PV] with PV = sum_t (1 + rrr dt/100)^-t flows[c_t] unit_profit_t, and
 * E[end population] per species (corrected growth, sem 1).  Parameters
 * theta (2U + 2S + C): OU reversion theta_u, OU volatility sigma_u, growth-
 * rate mean mu_s (species params[1]), growth variability v_s (params[7]),
 * crossing hazard h_c (the matrices of rov->species are taken as built
 * with `hazard`; h_c rescales entry (k, l) of control c by
 * exp(-crossings[s][l][k] (h_c - hazard[c]))).  No reference counterpart. */
typedef struct {
    const to_rov_problem* rov;
    const int* controls;          /* [n_years][n_paths] frozen policy            */
    const int* const* crossings;  /* per species [N][N] road crossings (i -> j)  */
    const double* hazard;         /* [C] hazards the matrices were built with     */
} to_adjoint_problem;

typedef struct to_tape_s* to_tape;

/* forward: outputs[1 + S]; keeps the population checkpoints (every 10
 * years) in a tape for the backward call (tape may be NULL) */
to_status to_adjoint_forward(to_ctx ctx, const to_adjoint_problem* prob,
                             const double* theta, double* outputs, to_tape* tape);
/* backward: grad_theta = sum_i grad_outputs[i] d outputs[i] / d theta */
to_status to_adjoint_backward(to_ctx ctx, to_tape tape, const double* grad_outputs,
                              double* grad_theta);
to_status to_tape_destroy(to_tape tape);

/* 16 features per road for the learned surrogate (road cells rasterised on
 * the device): 0 length / W, 1 segments / 64, 2 road cells / W, 3 / 4
 * road crossings per animal of species 0 moving 5 / 12 cells, 5..7 share
 * of the road's cells on habitat codes 2, 3, 5, 8 share of species 0's
 * initial animals on road cells, 9 / 10 / 11 / 14 share of them within
 * 3 / 6 / 12 / 24 cells (Chebyshev) of the road, 12 / 13 bounding-box
 * width and height / W, 15 sinuosity / 10.  No reference counterpart.
 * Host arrays; features [n_roads][16]. */
to_status to_road_features(to_ctx ctx, to_gen gen, int n_roads, const int* seg_off,
                           const double* segs, float* features);
/* device arrays (cell_off / cells may be NULL: rasterised here) */
to_status to_road_features_d(to_ctx ctx, to_gen gen, int n_roads, const int* seg_off,
                             const double* segs, const int* cell_off, const int* cells,
                             float* features);

/* Local-linear grid surrogate at n_points points (predictors [n][n_dims]),
 * surrogate [R*d axis values | R^d values] as the builders return it.
 * mode 0: SimulateGPU::interpolateSurrogateMulti (SimulateGPU.h:257 /
 * SimulateGPU.cu:5919-5968 and its kernel :3077-3155) as it computes, in
 * float; mode 1: multilinear interpolation in double; mode 2:
 * Utility::interpolateSurrogate (Utility.cpp:253-363), the per-road host
 * evaluation, in double, batched.  Host arrays. */
to_status to_interpolate_surrogate(to_ctx ctx, int n_points, int n_dims, int dim_res,
                                   const double* surrogate, const double* predictors,
                                   double* results, int mode);

/* RoadGA::generateSample (RoadGA.cpp:3288-3462): choose n designs to
 * simulate from candidates [n_candidates][n_dims] (host, row-major) given
 * the current samples [n_current][n_dims] (may be 0: then the first two are
 * the most distant pair), by the reference's max-min rule on its projected
 * and Euclidean distances after joint normalisation.  sample[n] receives
 * candidate indices. */
to_status to_select_samples(to_ctx ctx, int n_current, const double* current, int n_candidates,
                            const double* candidates, int n_dims, int n, int* sample);

/* The autotuner's record: one line per tuned shape, "kind ne paths rs ->
 * choice (sparse ms, simt ms, tc ms)", -1 where a kernel was not feasible.
 * Writes at most len bytes (NUL-terminated); returns the number of lines. */
int to_ctx_tuning(to_ctx ctx, char* buf, int len);

/* result block per (road, species), TO_RESULT_STRIDE doubles:
 *   0 n_patches, 1 n_transitions, 2 mte mean, 3 mte sd, 4 mte se,
 *   5 P(end < 0.2 init), 6 initial population, 7 non-zeros of the
 *   highest-flow migration matrix (-1 when the dense form ran),
 *   8 this species' MTE penalty, 9 the road's MTE penalty (sum over its
 *   species; both 0 until to_scene_set_penalty),
 *   10..14 the road's ROV valuation when the scene has one
 *   (to_scene_set_rov; else NaN): value, optimal first-period control, the
 *   reference's SD statistic, Monte Carlo standard error, paths behind the
 *   value,
 *   15 the share of the ROV's regression grid its backward pass read, and so
 *   fitted, over its years and controls (0 without a ROV),
 *   16..23 initial animals at risk of control c = 0..7
 *   (SpeciesRoadPatches::computeInitialAAR, SpeciesRoadPatches.cpp:453-490;
 *   NaN past n_controls) */
#define TO_RESULT_STRIDE 24

to_status to_scene_create(to_ctx ctx, const to_scene* scene, to_gen* gen);
to_status to_scene_destroy(to_gen gen);

/* The MTE penalty of Simulator::simulateMTE (Simulator.cpp:196-214): per
 * species, (threshold > lb) * (threshold - lb) * init_population *
 * cost_per_animal with lb = z * SD + mean of the end population and
 * z = NormalCDFInverse(1 - confidence) (Abramowitz & Stegun 26.2.23, as
 * Utility.cpp:165-193).  threshold is the species threshold times the
 * scenario's population level.  Host arrays [n_species]. */
typedef struct {
    double confidence;
    const double* threshold;
    const double* init_population;
    const double* cost_per_animal;
} to_penalty;
to_status to_scene_set_penalty(to_ctx ctx, to_gen gen, const to_penalty* penalty);

/* Adds the ROV valuation (simulateROVCUDA, ALGO4, SimulateGPU.cu:3870-5003)
 * of every road to to_evaluate_roads, in the same launch sequence (and the
 * same captured graph) as the species models and the MTE: the road-
 * independent fields of `rov` (paths per road, years, controls, dim_res,
 * processes, fuels, commodities, costs, dt, rrr, demand_idx, seed) apply to
 * every road, and so do its species' params when `species` is not NULL
 * (else the scene's); the species' patch fields and the road and migration
 * fields are ignored - each road uses the species models the generation
 * builds (all controls' packed matrices) with road id road0 + r.  n_species and n_controls must
 * be the scene's, sem 1, algo 4 (or 0), >= 128 paths.  Road r's result
 * equals to_simulate_rov_batch on the same models.  Scratch for max_roads
 * roads is allocated here; rov == NULL switches the ROV off. */
to_status to_scene_set_rov(to_ctx ctx, to_gen gen, const to_rov_problem* rov);

/* Roads as CSR lists: road r owns cells [cell_off[r], cell_off[r+1]) of
 * `cells` (index x + y*W, set to ROAD) and segments [seg_off[r], seg_off[r+1])
 * of `segs` (4 doubles x1, y1, x2, y2 per segment).  Host pointers;
 * results (host) is [n_roads][n_species][TO_RESULT_STRIDE]. */
to_status to_evaluate_roads(to_ctx ctx, to_gen gen, int n_roads,
                            const int* cell_off, const int* cells,
                            const int* seg_off, const double* segs,
                            const to_eval_opts* opts, double* results);
/* cell_off and cells may both be NULL: the road cells are then computed
 * from the segments on the device (a segment of length L sampled at
 * max(2, ceil(4L)) + 1 evenly spaced points, each in the cell of its
 * coordinates rounded half to even, inside the grid).
 * Same with every array (inputs and results) in device memory; enqueued on
 * the context stream without synchronising. */
to_status to_evaluate_roads_d(to_ctx ctx, to_gen gen, int n_roads,
                              const int* cell_off, const int* cells,
                              const int* seg_off, const double* segs,
                              const to_eval_opts* opts, double* results);

/* Inspection of the last evaluation of a scene (no reference counterpart;
 * for tests and tools that check a generation road by road).  Both wait for
 * the context stream.  to_gen_end_pops: the n_paths per-path end
 * populations of (road, species) (n_paths must be the last call's
 * mte_paths).  to_gen_species_model: that road's species model as the
 * migration kernel read it - patch count, initial populations and
 * capacities [N], and the migration matrices expanded to dense
 * destination-major [C][N][N] floats (from the packed columns when the
 * sparse kernel ran, else from the dense form); nnz[C] (optional) gets the
 * packed non-zero counts, -1 where none were packed.  Arrays may be NULL;
 * N > max_patches is TO_ERR_INVALID with *n_patches set. */
to_status to_gen_end_pops(to_ctx ctx, to_gen gen, int road, int species, int n_paths,
                          float* end_pops);
to_status to_gen_species_model(to_ctx ctx, to_gen gen, int road, int species, int max_patches,
                               int* n_patches, float* init_pops, float* caps, float* mmm,
                               int* nnz);

/* ------------------------------------------------------------------------
 * Learned surrogate (no counterpart in the reference, whose GA fitness uses
 * the local-linear grid surrogates): an MLP 16 -> 128 -> 128 -> 3 with ReLU,
 * BF16 tensor-core GEMMs with FP32 accumulation, trained by Adam on FP32
 * master parameters.  Parameter vector (FP32, TO_MLP_NPARAM):
 *   W1[128][16], b1[128], W2[128][128], b2[128], W3[3][128], b3[3].
 * Rows of x are TO_MLP_IN floats, rows of y / t are TO_MLP_OUT floats.
 * ---------------------------------------------------------------------- */
#define TO_MLP_IN 16
#define TO_MLP_HID 128
#define TO_MLP_OUT 3
#define TO_MLP_NPARAM (16 * 128 + 128 + 128 * 128 + 128 + 3 * 128 + 3)

/* y = f(x) for n rows (host buffers) */
to_status to_mlp_predict(to_ctx ctx, const float* params, int n, const float* x, float* y);
/* the same on device buffers, on the context's stream */
to_status to_mlp_predict_d(to_ctx ctx, const float* d_params, int n, const float* d_x, float* d_y);
/* gradient of mean((y - t)^2) over all n rows and outputs; *loss = that mean */
to_status to_mlp_grad(to_ctx ctx, const float* params, int n, const float* x, const float* t,
                      float* grad, double* loss);
/* Adam (lr, 0.9, 0.999, 1e-8) over `epochs` seeded shuffles in mini-batches;
 * params updated in place; loss_curve[epochs] = mean squared error seen in
 * each epoch (may be NULL) */
to_status to_mlp_train(to_ctx ctx, float* params, int n, const float* x, const float* t,
                       int epochs, int batch, float lr, uint64_t seed, double* loss_curve);

#ifdef __cplusplus
}
#endif
#endif /* TRANSOPT_H */
