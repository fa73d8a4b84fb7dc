/* oracle_adjoint.h - FP64 restatement of the frozen-policy road valuation
 * (test infrastructure for the adjoint kernels). */
#ifndef ORACLE_ADJOINT_H
#define ORACLE_ADJOINT_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct {
    int P, Y, S, C, U, NP;
    float dt, rrr;
    uint64_t seed;
    int road;
    const float* uncert;        /* [U][6] */
    const float* flows;         /* [C] */
    int nF;
    const float* fuel_costs;    /* [nF] */
    const int* fuel_idx;        /* [nF] */
    int Cm;
    const float* ore_content;   /* [Cm] */
    const float* ore_sd;        /* [Cm] */
    float unit_cost, unit_revenue;
    int demand_idx;
    const int* controls;        /* [Y][P] */
    const int* n_patches;       /* [S] */
    const float* params;        /* [S][8] */
    const float* init_pops;     /* [S][NP] */
    const float* caps;          /* [S][NP] */
    const float* mmm;           /* [S][C][NP][NP] destination-major */
    const int* cross;           /* [S][NP][NP] crossings of pair (l, k) at [l][k] */
    const double* base_h;       /* [C] */
} or_adj_problem;

/* outputs[1 + S] = E[PV], E[end population_s] at theta (2U + 2S + C) */
void or_adjoint_forward(const or_adj_problem* pr, const double* theta, double* outputs,
                        int threads);
#ifdef __cplusplus
}
#endif
#endif
