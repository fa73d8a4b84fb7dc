// to_sparse.cuh - compressed-column migration matrices and the sparse
// population kernels (sparse_pop.cu).
#pragma once
#include "to_internal.cuh"

struct to_csc {
    int* ptr;          // [matrices][NP + 1] column starts
    uint16_t* idx;     // [matrices][cap] origin patch of each non-zero
    float* val;        // [matrices][cap]
    int* nnz;          // [matrices] non-zeros, -1 when above cap
    int cap;           // capacity per matrix in global memory
    int cap_smem;      // largest nnz of the launch (shared-memory lists)
    // optional union form of the C <= 3 matrices of each (road, species):
    // destination k's entries are the origins where any control has a
    // non-zero, ascending, each as {origin, value of control 0, 1, 2} with
    // 0 where a control has none (an exact zero term, so every control's
    // sums keep their bits)
    int4* uent;        // [road-species][ucap]
    int* uptr;         // [road-species][NP + 1]
    int* unnz;         // [road-species], -1 when above ucap
    int ucap;          // capacity per road-species in global memory
    int ucap_smem;     // largest union of the launch
};

struct to_mte_args;
struct to_rov_args;

namespace to_k {
to_status pack_csc(to_ctx ctx, const float* mmm, int NP, int C, const int* n_patches,
                   int n_rs, to_csc& csc, int rs0 = 0);
size_t mte_sparse_smem(int NE, int cap_smem);
size_t rov_sparse_smem(int NE, int C, int cap_smem);
// the union form of every (road, species)'s C <= 3 packed matrices
to_status union_csc(to_ctx ctx, int NP, int C, const int* n_patches, int n_rs, to_csc& csc);
size_t rov_union_smem(int NE, int C, int ucap_smem);
to_status mte_sparse(to_ctx ctx, to_mte_args a, int n_rs, to_csc csc);
to_status rov_forward_sparse(to_ctx ctx, const to_rov_args& a, to_csc csc);
// ALGO6: paths re-simulated from year t0 under the optimal policy
size_t rov_resim_smem(int NE, int S, int C, int cap_smem);
to_status rov_resim_sparse(to_ctx ctx, const to_rov_args& a, to_csc csc, int t0);
}
