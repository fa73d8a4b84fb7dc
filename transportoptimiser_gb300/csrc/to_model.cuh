// to_model.cuh - device-side argument blocks of the species-road model and
// the population kernels (plain calls use a batch of one road).
#pragma once
#include "to_internal.cuh"

#define TO_MAX_HAB 8
#define TO_MAX_CONTROLS 8

struct to_model_species {
    int n_hab;
    int hab_type[TO_MAX_HAB];
    double hab_max_pop[TO_MAX_HAB];
    double hab_pref_mean[TO_MAX_HAB];
    double hab_pref_sd[TO_MAX_HAB];
    double hazard[TO_MAX_CONTROLS];   // Q_c (w + len)/(speed 3600)
    double lambda_mean, lambda_sd, lambda_mult, hab_pref_mult;
};

struct to_model_args {
    int W, H, S, C;
    int skpx, skpy, xres, yres;
    float xs, ys, spa;
    const int* hab_map;          // [W*H] habitat codes
    const int* cell_off;         // [R+1] road cells CSR (may be null)
    const int* cells;            // cell indices set to ROAD
    const float* pop_map;        // [S][W*H]
    const to_model_species* species;   // device [S]
    const int* seg_off;          // [R+1] road segments CSR
    const double* segs;          // 4 doubles (x1, y1, x2, y2) per segment
    int sem;
    int rs0;                     // first (road, species) of the launch (rs = road*S + species)
    int max_patches;             // NM: stride of per-(road,species) arrays
    int npad;                    // NP: padded patch count of the matrices
    // outputs, all indexed by rs = road*S + species
    int* n_patches;              // [RS]
    int* n_transitions;          // [RS]
    double *area, *cap, *pop, *cx, *cy;   // [RS][NM]
    int* type;                   // [RS][NM]
    int* crossings_scratch;      // [RS][NM*NM] (N*N packed)
    int* crossings_out;          // optional [RS][NM][NM]
    double* trans_scratch;       // [RS][NM][NM]
    uint16_t* trans_dest;        // [RS][NM][NM] in-range destinations per origin row
    double* trans;               // optional [RS][NM][NM]
    double* surv;                // optional [RS][C][NM][NM]
    float* mmm;                  // [RS][C][NP][NP] destination-major
    // csc_ptr non-null: the migration matrices go straight into the packed
    // form (what k_pack_csc makes of the dense ones) and the dense [C][NP][NP]
    // block of each (road, species) is only scratch, never zeroed
    int* csc_ptr;                // [RS*C][NP+1]
    uint16_t* csc_idx;           // [RS*C][csc_cap]
    float* csc_val;              // [RS*C][csc_cap]
    int* csc_nnz;                // [RS*C], -1 above csc_cap
    int csc_cap;
    // labels shared by the species of a road: one labelling per (road,
    // habitable type) into global memory, read by every species' patch
    // pass (n_label_types 0: each CTA labels in its own shared memory)
    int n_label_types;           // T
    const int* label_types;      // [T] habitat codes
    int* labels;                 // [R][T][W*H] LabelImage numbers, 0 background
    double* iar;                 // optional [RS][C] initial animals at risk per control
    float* init_pops;            // [RS][NP]
    float* caps;                 // [RS][NP] (padding 1.0)
    int* d_flags;
};

namespace to_k {
to_status species_model(to_ctx ctx, const to_model_args& a, int n_rs);
}
