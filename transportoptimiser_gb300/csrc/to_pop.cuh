// to_pop.cuh - argument blocks of the population Monte Carlo kernels.
#pragma once
#include "to_internal.cuh"

struct to_mte_args {
    int n_paths, n_years, S, C, c_use;
    float dt;
    uint64_t seed;
    int sem;
    int road0;                   // stream id of road 0 of the batch
    int rs0;                     // first (road, species) of the launch
    int npad;                    // NP: stride of the per-road arrays
    int npe;                     // effective width (multiple of 4, >= every N)
    int tile_paths, l_chunk;     // filled by the launcher
    const int* n_patches;        // [RS]
    const float* mmm;            // [RS][C][NP][NP] destination-major
    const float* init_pops;      // [RS][NP]
    const float* caps;           // [RS][NP]
    const float* params;         // [S][8]
    float* end_pops;             // [RS][P]
    int* flags;                  // device error word (plan checks), may be null
    const int* order;            // [n_rs] launch order of the (road, species), or null
    int* order_buf;              // scratch for it ([n_rs] ints), or null: the
                                 // sparse launcher then orders widest first
    int fault_wait;              // test hook (to_ctx_inject_fault): the tensor-core
                                 // kernel's first wait, on a barrier nothing arrives
                                 // at, runs out at once
};

namespace to_k {
to_status mte_simt(to_ctx ctx, to_mte_args a, int n_rs);
to_status mte_tc(to_ctx ctx, to_mte_args a, int n_rs);
to_status mte_stats(to_ctx ctx, const to_mte_args& a, int n_rs, double* d_stats);
to_status exp_pv(to_ctx ctx, const float* d_prm, int P, int Y, uint64_t seed,
                 int road, int sem, float* d_values, double* d_stats);
}
