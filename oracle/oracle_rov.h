/*
 * oracle_rov.h - CPU restatement of the reference's ROV valuation (ALGO4),
 * kNN and surrogate builders.  TEST INFRASTRUCTURE ONLY (see oracle.h).
 */
#ifndef TO_ORACLE_ROV_H
#define TO_ORACLE_ROV_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TO_MAX_C_ORACLE 8

typedef struct {
    int n_paths, n_years, n_species, n_controls, n_uncertainties, dim_res;
    const int* n_patches;               /* [S]                                 */
    const float* const* params;         /* [S] -> [8]                          */
    const float* params_flat;           /* [S*8], the reference's flat layout  */
    const float* const* init_pops;      /* [S] -> [N_s]                        */
    const float* const* caps;           /* [S] -> [N_s]                        */
    const float* const* mmm;            /* [S] -> [C][N][N] destination-major  */
    const float* flows;                 /* [C]                                 */
    const float* uncert;                /* [U*6] current, mean, sd, reversion,
                                           jump size, jump prob; fuels first   */
    int n_fuels;
    const float* fuel_costs;            /* [n_fuels]                           */
    const int* fuel_idx;                /* [n_fuels]                           */
    int n_commodities;
    const float* ore_content;           /* [Cm]                                */
    const float* ore_sd;                /* [Cm]                                */
    float unit_cost, unit_revenue, dt, rrr, scaling;
    int demand_idx;                     /* process multiplying the profit, -1  */
    uint64_t seed;
    int road, sem, n_threads;
    int algo;                           /* 4 (or 0): ALGO4; 6: ALGO6 path
                                           re-simulation (sem 1 only)        */
} or_rov_problem;

typedef struct {
    float* cond_exp;                    /* [Y][P]                              */
    int* opt_cont;                      /* [Y][P]                              */
    float* unit_profits;                /* [Y][P]                              */
    float* adj_pops;                    /* [Y][S][P]                           */
    float* regression;                  /* [Y][C][R*d + 2 R^d] (optional)      */
    int* controls;                      /* [P][Y] (optional)                   */
    float* total_pops;                  /* [P][Y+1][S] (optional)              */
    float* aars;                        /* [P][Y+1][S][C] (optional)           */
    float* u_results;                   /* [P][Y+1][U] (optional)              */
    double stats[3];                    /* value, control, "SD"                */
    double value_se;                    /* Monte Carlo standard error of value */
    int n_best;
} or_rov_result;

int or_simulate_rov(const or_rov_problem* pr, or_rov_result* res);
void or_knn(const float* ref, int n, const float* query, int Q, int dim, int k,
            float* dist, int* ind);
int or_k_rov(int n);
int or_k_rov_mult(int n, int mult);
int or_k_surrogate_mte(int n);
int or_k_surrogate_rov(int n);
void or_build_surrogate_1d(int n, const float* x, const float* y, int R, float* out);
void or_build_surrogate_nd(int n, int d, const float* pred, const float* y, int R,
                           int sem, int clip, float* out);

#ifdef __cplusplus
}
#endif
#endif
