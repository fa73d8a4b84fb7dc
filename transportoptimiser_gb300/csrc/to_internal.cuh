// to_internal.cuh - context, scratch arena and launch helpers shared by the
// CUDA translation units of libtransopt.so.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/transopt.h"
#include "to_math.h"

#define TO_SM_TARGET 152

struct to_ctx_s {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // device scratch arena: one buffer, bump-allocated per call
    char* arena = nullptr;
    size_t arena_cap = 0;
    size_t arena_off = 0;
    // pinned host staging
    char* pinned = nullptr;
    size_t pinned_cap = 0;
    // persistent device scratch of the tensor-core migration (packed
    // hi/lo matrix blocks), grown on demand
    char* tc_buf = nullptr;
    size_t tc_cap = 0;
    // device error word for bounded waits / in-kernel checks
    int* d_flags = nullptr;
    uint64_t launches = 0;
    // optional per-kernel event timing (to_ctx_profile)
    bool profile = false;
    static constexpr int kMaxProf = 4096;
    int n_prof = 0;
    const char* prof_name[kMaxProf];
    cudaEvent_t prof_ev[kMaxProf][2];
    int prof_ev_alloc = 0;
    int sm_count = 0;
    size_t smem_optin = 0;
    // autotuner: measured migration-kernel choice per problem shape
    struct tune_entry {
        uint64_t key;
        int kind;               // 0 batched generation, 1 single-road MTE
        int ne, paths, n_rs, choice;
        float ms[3];            // sparse, dense SIMT, tensor core (-1: not feasible)
    };
    std::vector<tune_entry> tune;
    char err[512] = {0};
    int fault = 0;              // to_ctx_inject_fault: armed one-shot fault
};

// device-side error codes written to ctx->d_flags[0]
enum { TO_DEVERR_NONE = 0, TO_DEVERR_REGIONS = 1, TO_DEVERR_UNION = 2,
       TO_DEVERR_PATCHES = 3, TO_DEVERR_SPIN = 4, TO_DEVERR_PLAN = 5,
       TO_DEVERR_CELL = 6 };

to_status to_set_error(to_ctx ctx, to_status s, const char* fmt, ...);
to_status to_check_cuda(to_ctx ctx, cudaError_t e, const char* what);

#define TO_TRY(expr)                                                       \
    do {                                                                   \
        to_status _s = (expr);                                             \
        if (_s != TO_OK) return _s;                                        \
    } while (0)

#define TO_CUDA(ctx, expr) TO_TRY(to_check_cuda((ctx), (expr), #expr))

#define TO_LAUNCHED(ctx)                                                   \
    do {                                                                   \
        (ctx)->launches++;                                                 \
        TO_CUDA((ctx), cudaGetLastError());                                \
    } while (0)

// Reserve `bytes` of arena for the current call; resets the bump pointer.
to_status to_arena_reserve(to_ctx ctx, size_t bytes);
// Bump-allocate 256-byte aligned scratch (after to_arena_reserve).
template <class T>
static inline T* to_arena_take(to_ctx ctx, size_t count) {
    size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
    if (ctx->arena_off + bytes > ctx->arena_cap) return nullptr;
    T* p = reinterpret_cast<T*>(ctx->arena + ctx->arena_off);
    ctx->arena_off += bytes;
    return p;
}
static inline size_t to_align256(size_t b) { return (b + 255) & ~size_t(255); }

to_status to_read_device_flags(to_ctx ctx, int* flag);
// reads and clears the device error word; TO_ERR_TIMEOUT for a bounded wait
// that ran out, TO_ERR_UNSUPPORTED for the other device checks
to_status to_check_device_flags(to_ctx ctx);

// Bracket a launch with events when profiling is on.
void to_prof_begin(to_ctx ctx, const char* name);
void to_prof_end(to_ctx ctx);

// Kernel launch entry points implemented in the .cu files.
namespace to_k {
// patches.cu
to_status label_image(to_ctx ctx, int W, int H, const int* d_in, int* d_out,
                      int* d_nreg);
to_status build_patches(to_ctx ctx, int W, int H, int skpx, int skpy, int xres,
                        int yres, int nreg, float xs, float ys, float spa,
                        float maxpop, const int* d_labels, const float* d_pops,
                        int max_patches, double* d_out5, int* d_count);
to_status line_segment_intersect(to_ctx ctx, int T, const double* d_xy1, int G,
                                 const double* d_xy2, int* d_cross);
// raster.cu
// RoadCells::computeRoadCells for every road (grid spacing xs, ys; sem 0
// keeps the reference's vertical-crossing quirk)
to_status rasterise_roads(to_ctx ctx, int R, const int* seg_off, const double* segs, int W,
                          int H, double xs, double ys, int sem, int* cell_off, int* cells,
                          int max_cells, int* counts_scratch);
to_status road_features(to_ctx ctx, int R, int W, int H, const int* base, const float* popmap,
                        const int* seg_off, const double* segs, const int* cell_off,
                        const int* cells, float* feat);
}  // namespace to_k
