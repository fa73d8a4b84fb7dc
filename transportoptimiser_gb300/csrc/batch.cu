// batch.cu - a whole GA generation of roads valued in a handful of launches.
//
// RoadGA::evaluateGeneration (include/main/RoadGA.cpp:2040-2099) and the
// surrogate sampling loop (RoadGA.cpp:1687-1748) call the species model and
// SimulateGPU::simulateMTECUDA once per road from a host thread pool, with a
// device allocation, copy and synchronisation inside every call.  Here the
// scene is resident in HBM (to_scene_create) and a generation is:
//   1. one launch, one CTA per (road, species): labels, patches, crossings,
//      transition / survival probabilities, migration matrices;
//   2. one read of the largest patch count (the only host round trip);
//   3. one launch over (path tile, road*species): every road's Monte Carlo;
//   4. one launch: FP64 statistics per (road, species).
// The migration kernel (sparse, dense SIMT or tensor-core 3xTF32) is chosen
// by an autotuner that times the feasible ones on the first generation of
// a shape and keeps the fastest (to_ctx_tuning reports the choices).  With
// opts.graph the whole generation is captured once as a CUDA graph, with
// the shapes planned from the previous generation plus a margin, and
// replayed without any host round trip; kernels that meet a road outside
// the plan write NaN and raise a flag, and the host entry point then
// re-plans and re-runs.
#include <cmath>
#include <cstring>
#include <vector>

#include "to_grid.h"
#include "to_internal.cuh"
#include "to_model.cuh"
#include "to_pop.cuh"
#include "to_rov.cuh"
#include "to_sparse.cuh"

struct to_gen_s {
    to_ctx ctx = nullptr;
    int W = 0, H = 0, S = 0, C = 0, NM = 0, NP = 0;
    int max_roads = 0, max_cells = 0, max_segs = 0;
    int skpx = 0, skpy = 0, xres = 0, yres = 0;
    float xs = 1, ys = 1, spa = 1;
    // resident scene
    int* d_base = nullptr;
    float* d_popmap = nullptr;           // [S][W*H]
    to_model_species* d_species = nullptr;
    float* d_params = nullptr;           // [S][8]
    int n_label_types = 0;               // habitable types of any species
    int* d_label_types = nullptr;        // [T]
    int* d_labels = nullptr;             // [max_roads][T][W*H]
    // per-generation buffers
    char* buf = nullptr;
    size_t buf_bytes = 0;
    int *d_cell_off, *d_cells, *d_seg_off;
    double* d_segs;
    int *d_np, *d_nt;
    double *d_area, *d_cap, *d_pop, *d_cx, *d_cy;
    int* d_type;
    int* d_cross;
    double* d_tv;
    uint16_t* d_tdest;
    float *d_mmm, *d_ip, *d_cp;
    float* d_end = nullptr;              // grown on demand [RS][P]
    int* d_mte_order = nullptr;          // [RS] the MTE's launch order (k_mte_order)
    size_t end_cap = 0;
    double* d_stats;                     // [RS][5]
    double* d_results;                   // [RS][8]
    to_csc csc;                          // [RS*C] packed migration matrices
    int* d_counts = nullptr;             // [max_roads] road cell counts (device rasterisation)
    float* d_feat = nullptr;             // [max_roads][16] surrogate features
    // captured generation (opts.graph)
    cudaGraphExec_t exec = nullptr;
    uint64_t graph_key = 0;
    int plan_ne = 0, plan_cap = 0, plan_choice = -1;
    uint64_t graph_launches = 0;         // kernels in the captured generation
    // what the last evaluation left readable (to_gen_species_model /
    // to_gen_end_pops): its shape and which migration-matrix forms it wrote
    int last_R = 0, last_paths = 0;
    bool last_dense = false, last_csc = false;
    bool graph_dense = false, graph_csc = false;
    double* d_iar = nullptr;             // [RS][C] initial animals at risk
    // MTE penalty (to_scene_set_penalty): z = inverse normal CDF of
    // (1 - confidence); per species threshold, initial population, cost
    double pen_z = 0.0;
    double* d_pen = nullptr;             // [S][3]
    // ROV of every road (to_scene_set_rov)
    bool rov_on = false;
    to_rov_args rov{};                   // road-independent fields + scratch
    char* rov_buf = nullptr;
    size_t rov_bytes = 0;
    int* d_road_ids = nullptr;           // [max_roads]
    double* d_rov_stats = nullptr;       // [max_roads][5]
    float* d_rov_params = nullptr;       // [S][8] species parameters of the ROV
};

namespace {

inline uint32_t __float_as_uint_host(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}

// MTE penalty of one species (Simulator::simulateMTE, Simulator.cpp:196-214):
// the shortfall of the lower confidence bound z*SD + mean below the
// threshold, times the initial population and the cost per animal
__device__ __forceinline__ double mte_penalty(double mean, double sd, double z,
                                              const double* pen) {
    const double lb = z * sd + mean;
    return (double)(pen[0] > lb) * (pen[0] - lb) * pen[1] * pen[2];
}

__global__ void k_pack_results(int n_rs, int S, const int* __restrict__ np,
                               const int* __restrict__ nt,
                               const double* __restrict__ stats,
                               const int* __restrict__ nnz, int C,
                               const double* __restrict__ iar, double pen_z,
                               const double* __restrict__ pen,
                               const double* __restrict__ rov_stats,
                               const unsigned* __restrict__ qroad, double q_all,
                               double* __restrict__ out) {
    int rs = blockIdx.x * blockDim.x + threadIdx.x;
    if (rs >= n_rs) return;
    const int road = rs / S, sp = rs - road * S;
    double* o = out + (size_t)rs * TO_RESULT_STRIDE;
    o[0] = np[rs];
    o[1] = nt[rs];
    for (int q = 0; q < 5; ++q) o[2 + q] = stats[5 * (size_t)rs + q];
    // non-zeros of the highest-flow migration matrix (-1: dense path used)
    o[7] = nnz ? (double)nnz[(size_t)rs * C + C - 1] : -1.0;
    // penalty: this species' share, then the road's sum over its species
    double mine = 0.0, road_pen = 0.0;
    for (int s = 0; s < S; ++s) {
        const double* st = stats + 5 * ((size_t)road * S + s);
        const double v = mte_penalty(st[0], st[1], pen_z, pen + 3 * s);
        if (s == sp) mine = v;
        road_pen += v;
    }
    o[8] = mine;
    o[9] = road_pen;
    for (int q = 0; q < 5; ++q) o[10 + q] = rov_stats ? rov_stats[5 * (size_t)road + q] : NAN;
    // share of the regression grid the road's backward pass read (and so
    // fitted), over its years and controls
    o[15] = (rov_stats && qroad && q_all > 0.0) ? (double)qroad[road] / q_all : 0.0;
    for (int c = 0; c < 8; ++c) o[16 + c] = c < C ? iar[(size_t)rs * C + c] : NAN;
}

__global__ void k_road_ids(int R, int road0, int* __restrict__ ids) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < R) ids[r] = road0 + r;
}

__global__ void k_max_int(int n, const int* __restrict__ v, int* out) {
    int m = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) m = max(m, v[i]);
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ int s[32];
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        int r = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r = max(r, s[i]);
        *out = r;
    }
}

// out[0] = min, out[1] = max of v[0..n)
__global__ void k_min_max_int(int n, const int* __restrict__ v, int* out) {
    int lo = 0x7fffffff, hi = -0x7fffffff;
    for (int i = threadIdx.x; i < n; i += blockDim.x) { lo = min(lo, v[i]); hi = max(hi, v[i]); }
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    __shared__ int s_lo[32], s_hi[32];
    if ((threadIdx.x & 31) == 0) { s_lo[threadIdx.x >> 5] = lo; s_hi[threadIdx.x >> 5] = hi; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < (int)(blockDim.x >> 5); ++i) { lo = min(lo, s_lo[i]); hi = max(hi, s_hi[i]); }
        lo = min(lo, s_lo[0]); hi = max(hi, s_hi[0]);
        out[0] = lo;
        out[1] = hi;
    }
}

template <class T>
T* carve(char*& p, size_t n) {
    T* r = reinterpret_cast<T*>(p);
    p += to_align256(n * sizeof(T));
    return r;
}

enum { CH_SPARSE = 0, CH_SIMT = 1, CH_TC = 2 };

uint64_t mix(uint64_t h, uint64_t v) {
    h ^= v + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
    return h;
}

void model_args(to_gen g, int R, const int* cell_off, const int* cells, const int* seg_off,
                const double* segs, const to_eval_opts* o, to_ctx ctx, to_model_args& a) {
    memset(&a, 0, sizeof(a));
    a.W = g->W; a.H = g->H; a.S = g->S; a.C = g->C;
    a.skpx = g->skpx; a.skpy = g->skpy; a.xres = g->xres; a.yres = g->yres;
    a.xs = g->xs; a.ys = g->ys; a.spa = g->spa;
    a.hab_map = g->d_base; a.cell_off = cell_off; a.cells = cells;
    a.pop_map = g->d_popmap; a.species = g->d_species;
    a.seg_off = seg_off; a.segs = segs;
    a.sem = o->sem; a.max_patches = g->NM; a.npad = g->NP;
    a.n_patches = g->d_np; a.n_transitions = g->d_nt;
    a.area = g->d_area; a.cap = g->d_cap; a.pop = g->d_pop;
    a.cx = g->d_cx; a.cy = g->d_cy; a.type = g->d_type;
    a.crossings_scratch = g->d_cross; a.trans_scratch = g->d_tv; a.trans_dest = g->d_tdest;
    a.mmm = g->d_mmm; a.init_pops = g->d_ip; a.caps = g->d_cp;
    a.d_flags = ctx->d_flags;
    a.n_label_types = g->n_label_types; a.label_types = g->d_label_types; a.labels = g->d_labels;
    a.iar = g->d_iar;
}

// the model kernel writes the packed migration matrices (no dense ones)
void csc_direct(to_gen g, to_model_args& a) {
    a.csc_ptr = g->csc.ptr; a.csc_idx = g->csc.idx; a.csc_val = g->csc.val;
    a.csc_nnz = g->csc.nnz; a.csc_cap = g->csc.cap;
}

to_status grow_end(to_ctx ctx, to_gen g, size_t n) {
    if (n > g->end_cap) {
        if (g->d_end) TO_CUDA(ctx, cudaFree(g->d_end));
        g->d_end = nullptr;
        TO_CUDA(ctx, cudaMalloc(&g->d_end, n * sizeof(float)));
        g->end_cap = n;
    }
    return TO_OK;
}

to_mte_args mte_args(to_ctx ctx, to_gen g, const to_eval_opts* o, int NE) {
    to_mte_args m;
    memset(&m, 0, sizeof(m));
    m.n_paths = o->mte_paths; m.n_years = o->n_years; m.S = g->S; m.C = g->C;
    m.c_use = g->C - 1;
    m.dt = o->dt; m.seed = o->seed; m.sem = o->sem; m.road0 = o->road0;
    m.npad = g->NP; m.npe = NE; m.n_patches = g->d_np; m.mmm = g->d_mmm;
    m.init_pops = g->d_ip; m.caps = g->d_cp; m.params = g->d_params;
    m.end_pops = g->d_end; m.flags = ctx->d_flags;
    m.order_buf = g->d_mte_order;
    return m;
}

to_status run_choice(to_ctx ctx, to_gen g, const to_mte_args& m, int RS, int choice) {
    if (choice == CH_SPARSE) return to_k::mte_sparse(ctx, m, RS, g->csc);
    if (choice == CH_TC) return to_k::mte_tc(ctx, m, RS);
    return to_k::mte_simt(ctx, m, RS);
}

// The ROV valuation of every road (simulateROVCUDA's ALGO4 per road, as
// to_simulate_rov_batch runs it) on the species models this generation
// built: the packed migration matrices of every control, the roads' patch
// counts, initial populations and capacities, all already in HBM.
to_status rov_stage(to_ctx ctx, to_gen g, int R, int NE, int road0) {
    to_rov_args a = g->rov;
    a.nr = R; a.PT = R * a.P; a.G = R * a.C;
    a.lblocks = (a.PT + 1023) / 1024;
    a.np = g->NP; a.ne = NE;
    a.n_patches = g->d_np; a.params = g->d_rov_params; a.init_pops = g->d_ip;
    a.caps = g->d_cp; a.mmm = g->d_mmm; a.road_ids = g->d_road_ids;
    a.stats = g->d_rov_stats;
    k_road_ids<<<(R + 127) / 128, 128, 0, ctx->stream>>>(R, road0, g->d_road_ids);
    TO_LAUNCHED(ctx);
    // the kNN's per-query search radius starts from last year's; clear it
    // so that every generation starts the same way
    TO_CUDA(ctx, cudaMemsetAsync(a.kth, 0, (size_t)a.G * a.Q * sizeof(float), ctx->stream));
    to_csc csc = g->csc;
    if (csc.uent) {
        // every control's packed columns in one list per destination; at most
        // as many entries as the widest packed matrix (nested patterns)
        csc.ucap_smem = csc.cap_smem;
        if (to_k::rov_union_smem(NE, g->C, csc.ucap_smem) > ctx->smem_optin) csc.uent = nullptr;
        else TO_TRY(to_k::union_csc(ctx, g->NP, g->C, g->d_np, R * g->S, csc));
    }
    return to_k::rov_run(ctx, a, &csc);
}

// The launches after the model: migration Monte Carlo, statistics, the ROV
// of every road when the scene has one, results.
to_status tail(to_ctx ctx, to_gen g, const to_mte_args& m, int RS, int choice,
               double* d_results_out) {
    TO_TRY(run_choice(ctx, g, m, RS, choice));
    TO_TRY(to_k::mte_stats(ctx, m, RS, g->d_stats));
    const int R = RS / g->S;
    if (g->rov_on) TO_TRY(rov_stage(ctx, g, R, m.npe, m.road0));
    k_pack_results<<<(RS + 127) / 128, 128, 0, ctx->stream>>>(
        RS, g->S, g->d_np, g->d_nt, g->d_stats, choice == CH_SPARSE ? g->csc.nnz : nullptr, g->C,
        g->d_iar, g->pen_z, g->d_pen, g->rov_on ? g->d_rov_stats : nullptr,
        g->rov_on ? g->rov.qroad : nullptr,
        g->rov_on ? (double)(g->rov.Y - 2) * g->rov.C * g->rov.Q : 0.0, d_results_out);
    TO_LAUNCHED(ctx);
    return TO_OK;
}

// Autotuner: time each feasible migration kernel once on this generation
// (CUDA events on the context stream) and keep the fastest for the shape.
to_status tuned_choice(to_ctx ctx, to_gen g, const to_mte_args& m, int RS, int NE,
                       bool sparse_ok, bool tc_ok, int* choice) {
    const uint64_t key = mix(mix(mix(mix(0, 0), (uint64_t)NE), (uint64_t)m.n_paths),
                             mix((uint64_t)RS, (uint64_t)m.n_years * 2 + (sparse_ok ? 1 : 0)));
    for (const auto& e : ctx->tune)
        if (e.key == key && e.kind == 0) { *choice = e.choice; return TO_OK; }
    to_ctx_s::tune_entry te;
    te.key = key; te.kind = 0; te.ne = NE; te.paths = m.n_paths; te.n_rs = RS;
    te.ms[0] = te.ms[1] = te.ms[2] = -1.0f;
    cudaEvent_t e0, e1;
    TO_CUDA(ctx, cudaEventCreate(&e0));
    TO_CUDA(ctx, cudaEventCreate(&e1));
    int best = -1;
    const bool feas[3] = {sparse_ok, true, tc_ok};
    for (int c = 0; c < 3; ++c) {
        if (!feas[c]) continue;
        TO_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
        to_status st = run_choice(ctx, g, m, RS, c);
        TO_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
        TO_CUDA(ctx, cudaEventSynchronize(e1));
        if (st != TO_OK) continue;
        float ms = 0.0f;
        TO_CUDA(ctx, cudaEventElapsedTime(&ms, e0, e1));
        te.ms[c] = ms;
        if (best < 0 || ms < te.ms[best]) best = c;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best < 0) return to_set_error(ctx, TO_ERR_UNSUPPORTED, "no feasible migration kernel");
    te.choice = best;
    ctx->tune.push_back(te);
    *choice = best;
    return TO_OK;
}

// Direct (planning) evaluation: model, one read of the shapes, chosen
// migration kernel.  Fills the plan when asked.
to_status evaluate_direct(to_ctx ctx, to_gen g, int R, const int* cell_off,
                          const int* cells, const int* seg_off, const double* segs,
                          const to_eval_opts* o, double* d_results_out, int* plan) {
    const int S = g->S, RS = R * S, NP = g->NP;
    if (!cell_off) {
        // road cells from the segments, on the device
        TO_TRY(to_k::rasterise_roads(ctx, R, seg_off, segs, g->W, g->H, g->xs, g->ys, o->sem,
                                     g->d_cell_off, g->d_cells, g->max_cells, g->d_counts));
        cell_off = g->d_cell_off;
        cells = g->d_cells;
    }
    to_model_args a;
    model_args(g, R, cell_off, cells, seg_off, segs, o, ctx, a);
    // sparse migration asked for: the model kernel writes the packed
    // matrices itself (the tuner's dense candidates need the dense form)
    // (the ROV stage reads the packed matrices of every control, so a scene
    // with a ROV always takes them from the model and runs the sparse kernel)
    const bool packed = (o->migration == TO_MIG_SPARSE_FP32) || g->rov_on;
    if (packed) csc_direct(g, a);
    TO_TRY(to_k::species_model(ctx, a, RS));
    // the widest species model decides the tile shape of the path kernel
    int* d_max = reinterpret_cast<int*>(g->d_results + (size_t)g->max_roads * S * TO_RESULT_STRIDE);
    k_max_int<<<1, 1024, 0, ctx->stream>>>(RS, g->d_np, d_max);
    TO_LAUNCHED(ctx);
    const bool try_sparse = (o->migration == TO_MIG_AUTO || o->migration == TO_MIG_SPARSE_FP32 ||
                             g->rov_on);
    if (try_sparse) {
        if (!packed) TO_TRY(to_k::pack_csc(ctx, g->d_mmm, NP, g->C, g->d_np, RS, g->csc));
        k_min_max_int<<<1, 1024, 0, ctx->stream>>>(RS * g->C, g->csc.nnz, d_max + 1);
        TO_LAUNCHED(ctx);
    }
    int mm[3] = {0, 0, 0};
    TO_CUDA(ctx, cudaMemcpyAsync(mm, d_max, 3 * sizeof(int), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    int maxN = mm[0];
    if (maxN <= 0) maxN = 4;
    const int NE = (maxN + 3) & ~3;
    g->csc.cap_smem = (mm[2] + 7) & ~7;
    const bool sparse_ok = try_sparse && mm[1] >= 0 &&
                           to_k::mte_sparse_smem(NE, g->csc.cap_smem) <= ctx->smem_optin;
    if (try_sparse && !sparse_ok && (o->migration == TO_MIG_SPARSE_FP32 || g->rov_on))
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "matrices too dense for the sparse form");
    if (g->rov_on && (mm[1] < 0 ||
                      to_k::rov_sparse_smem(NE, g->C, g->csc.cap_smem) > ctx->smem_optin))
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "the ROV forward pass does not fit %d patches",
                            NE);
    TO_TRY(grow_end(ctx, g, (size_t)RS * o->mte_paths));
    to_mte_args m = mte_args(ctx, g, o, NE);
    int choice;
    if (o->migration == TO_MIG_SPARSE_FP32 || g->rov_on) choice = CH_SPARSE;
    else if (o->migration == TO_MIG_TC_3XTF32) choice = CH_TC;
    else if (o->migration == TO_MIG_SIMT_FP32) choice = CH_SIMT;
    else TO_TRY(tuned_choice(ctx, g, m, RS, NE, sparse_ok, NE <= 512, &choice));
    TO_TRY(tail(ctx, g, m, RS, choice, d_results_out));
    if (plan) { plan[0] = NE; plan[1] = g->csc.cap_smem; plan[2] = choice; }
    g->last_R = R; g->last_paths = o->mte_paths;
    g->last_dense = !packed; g->last_csc = try_sparse;
    return TO_OK;
}

// road-independent key of the scene's valuation settings (a captured
// generation is replayed only while they are unchanged)
uint64_t settings_key(to_gen g) {
    uint64_t h = mix(0, g->rov_on ? (uint64_t)g->rov.P * 131 + (uint64_t)g->rov.R : 0);
    h = mix(h, (uint64_t)(uintptr_t)g->rov_buf);
    uint64_t zb;
    memcpy(&zb, &g->pen_z, 8);
    return mix(h, zb);
}

// opts.graph: replay the captured generation when the call matches it,
// else plan directly and capture.
to_status evaluate(to_ctx ctx, to_gen g, int R, const int* cell_off,
                   const int* cells, const int* seg_off, const double* segs,
                   const to_eval_opts* o, double* d_results_out) {
    if (!o->graph) return evaluate_direct(ctx, g, R, cell_off, cells, seg_off, segs, o,
                                          d_results_out, nullptr);
    uint64_t key = 0;
    const uint64_t fields[] = {(uint64_t)R, (uint64_t)(uintptr_t)cell_off,
                               (uint64_t)(uintptr_t)cells, (uint64_t)(uintptr_t)seg_off,
                               (uint64_t)(uintptr_t)segs, (uint64_t)(uintptr_t)d_results_out,
                               (uint64_t)o->mte_paths, (uint64_t)o->n_years,
                               (uint64_t)__float_as_uint_host(o->dt), o->seed,
                               (uint64_t)o->road0, (uint64_t)o->sem, (uint64_t)o->migration,
                               (uint64_t)(uintptr_t)ctx->stream, settings_key(g)};
    for (uint64_t f : fields) key = mix(key, f);
    if (g->exec && g->graph_key == key) {
        TO_CUDA(ctx, cudaGraphLaunch(g->exec, ctx->stream));
        ctx->launches += g->graph_launches;
        g->last_R = R; g->last_paths = o->mte_paths;
        g->last_dense = g->graph_dense; g->last_csc = g->graph_csc;
        return TO_OK;
    }
    if (g->exec) { cudaGraphExecDestroy(g->exec); g->exec = nullptr; }
    int plan[3];
    TO_TRY(evaluate_direct(ctx, g, R, cell_off, cells, seg_off, segs, o, d_results_out, plan));
    // plan with a margin so that the next generations of a GA still fit
    const int S = g->S, RS = R * S;
    int ne = (plan[0] + 16 + 3) & ~3;
    if (ne > g->NP) ne = g->NP;
    int cap = ((plan[1] + plan[1] / 4 + 64) + 7) & ~7;
    if (cap > g->csc.cap) cap = g->csc.cap;
    if ((plan[2] == CH_SPARSE && to_k::mte_sparse_smem(ne, cap) > ctx->smem_optin) ||
        (g->rov_on && to_k::rov_sparse_smem(ne, g->C, cap) > ctx->smem_optin) ||
        plan[2] == CH_TC) {
        // no margin where it does not fit (or would resize the tensor-core
        // scratch, which cannot be allocated inside a capture)
        ne = plan[0];
        cap = plan[1];
    }
    const int choice = plan[2];
    g->csc.cap_smem = cap;
    to_model_args a;
    model_args(g, R, cell_off, cells, seg_off, segs, o, ctx, a);
    to_mte_args m = mte_args(ctx, g, o, ne);
    const bool prof = ctx->profile;
    ctx->profile = false;                      // no event records inside the capture
    const uint64_t l0 = ctx->launches;
    TO_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    to_status st = TO_OK;
    if (!cell_off) {
        st = to_k::rasterise_roads(ctx, R, seg_off, segs, g->W, g->H, g->xs, g->ys, o->sem,
                                   g->d_cell_off, g->d_cells, g->max_cells, g->d_counts);
        a.cell_off = g->d_cell_off;
        a.cells = g->d_cells;
    }
    if (choice == CH_SPARSE) csc_direct(g, a);  // packed matrices straight from the model
    if (st == TO_OK) st = to_k::species_model(ctx, a, RS);
    if (st == TO_OK) st = tail(ctx, g, m, RS, choice, d_results_out);
    cudaGraph_t graph = nullptr;
    cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
    ctx->profile = prof;
    if (st != TO_OK) { if (graph) cudaGraphDestroy(graph); return st; }
    TO_CUDA(ctx, ce);
    ce = cudaGraphInstantiate(&g->exec, graph, 0);
    cudaGraphDestroy(graph);
    TO_CUDA(ctx, ce);
    g->graph_key = key;
    g->plan_ne = ne; g->plan_cap = cap; g->plan_choice = choice;
    g->graph_launches = ctx->launches - l0;
    // the capture ran nothing: the planning pass above left the buffers; a
    // replay leaves the forms the captured kernels write
    g->graph_dense = (choice != CH_SPARSE);
    g->graph_csc = (choice == CH_SPARSE);
    return TO_OK;
}

}  // namespace

extern "C" {

to_status to_scene_create(to_ctx ctx, const to_scene* sc, to_gen* out) {
    if (!ctx || !sc || !out || sc->W <= 0 || sc->H <= 0 || sc->res <= 0 ||
        !sc->base_map || sc->n_species <= 0 || !sc->species ||
        sc->n_controls <= 0 || sc->n_controls > TO_MAX_CONTROLS ||
        sc->max_patches <= 0 || sc->max_roads <= 0 || sc->max_cells < 0 ||
        sc->max_segments <= 0)
        return TO_ERR_INVALID;
    {
        const int r = sc->res;
        const int xr = (sc->W % r == 0) ? r : r + 1, yr = (sc->H % r == 0) ? r : r + 1;
        const int sx = (int)std::floor((double)(sc->W - 1) / (double)r);
        const int sy = (int)std::floor((double)(sc->H - 1) / (double)r);
        if (!to_blocks_inside(sc->W, sc->H, sx, sy, xr, yr))
            return to_set_error(ctx, TO_ERR_UNSUPPORTED,
                                "coarse blocks of a %d x %d grid at resolution %d run past it",
                                sc->W, sc->H, r);
    }
    cudaSetDevice(ctx->device);
    to_gen g = new to_gen_s();
    g->ctx = ctx;
    g->W = sc->W; g->H = sc->H; g->S = sc->n_species; g->C = sc->n_controls;
    g->NM = sc->max_patches; g->NP = (sc->max_patches + 3) & ~3;
    g->max_roads = sc->max_roads; g->max_cells = sc->max_cells;
    g->max_segs = sc->max_segments;
    int res = sc->res;
    g->xres = (g->W % res == 0) ? res : res + 1;
    g->yres = (g->H % res == 0) ? res : res + 1;
    g->skpx = (int)std::floor((double)(g->W - 1) / (double)res);
    g->skpy = (int)std::floor((double)(g->H - 1) / (double)res);
    g->xs = (float)sc->xspacing; g->ys = (float)sc->yspacing;
    g->spa = (float)(sc->xspacing * sc->yspacing);
    const size_t n = (size_t)g->W * g->H;
    const int S = g->S, C = g->C, NM = g->NM, NP = g->NP;
    std::vector<to_model_species> hs(S);
    std::vector<float> pm((size_t)S * n), prm((size_t)S * 8);
    std::vector<int> ltypes;           // habitable types of any species, first appearance
    for (int s = 0; s < S; ++s)
        for (int h = 0; h < sc->species[s].n_hab && sc->species[s].habs; ++h) {
            const int t = sc->species[s].habs[h].type;
            if (t == 3 || t == 4) continue;
            bool seen = false;
            for (int v : ltypes) seen |= (v == t);
            if (!seen) ltypes.push_back(t);
        }
    g->n_label_types = (int)ltypes.size();
    for (int s = 0; s < S; ++s) {
        const to_species_desc& d = sc->species[s];
        if (d.n_hab <= 0 || d.n_hab > TO_MAX_HAB || !d.habs || !d.pop_map || !d.hazard ||
            !d.params) { delete g; return TO_ERR_INVALID; }
        memset(&hs[s], 0, sizeof(to_model_species));
        hs[s].n_hab = d.n_hab;
        for (int h = 0; h < d.n_hab; ++h) {
            hs[s].hab_type[h] = d.habs[h].type;
            hs[s].hab_max_pop[h] = d.habs[h].max_pop;
            hs[s].hab_pref_mean[h] = d.habs[h].pref_mean;
            hs[s].hab_pref_sd[h] = d.habs[h].pref_sd;
        }
        for (int c = 0; c < C; ++c) hs[s].hazard[c] = d.hazard[c];
        hs[s].lambda_mean = d.lambda_mean; hs[s].lambda_sd = d.lambda_sd;
        hs[s].lambda_mult = d.lambda_mult; hs[s].hab_pref_mult = d.hab_pref_mult;
        for (size_t i = 0; i < n; ++i) pm[(size_t)s * n + i] = (float)d.pop_map[i];
        for (int q = 0; q < 8; ++q) prm[(size_t)s * 8 + q] = d.params[q];
    }
    auto fail = [&](cudaError_t e) {
        to_check_cuda(ctx, e, "to_scene_create");
        to_scene_destroy(g);
        return e == cudaErrorMemoryAllocation ? TO_ERR_ALLOC : TO_ERR_CUDA;
    };
    cudaError_t e;
    if ((e = cudaMalloc(&g->d_base, n * sizeof(int))) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&g->d_popmap, pm.size() * sizeof(float))) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&g->d_species, S * sizeof(to_model_species))) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&g->d_params, prm.size() * sizeof(float))) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&g->d_label_types, (ltypes.size() + 1) * sizeof(int))) != cudaSuccess)
        return fail(e);
    if (!ltypes.empty())
        cudaMemcpy(g->d_label_types, ltypes.data(), ltypes.size() * sizeof(int),
                   cudaMemcpyHostToDevice);
    cudaMemcpy(g->d_base, sc->base_map, n * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(g->d_popmap, pm.data(), pm.size() * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(g->d_species, hs.data(), S * sizeof(to_model_species), cudaMemcpyHostToDevice);
    cudaMemcpy(g->d_params, prm.data(), prm.size() * sizeof(float), cudaMemcpyHostToDevice);

    const size_t R = g->max_roads, RS = R * S;
    size_t bytes = 0;
    auto acc = [&](size_t b) { bytes += to_align256(b); };
    acc((R + 1) * 4); acc((size_t)(g->max_cells > 0 ? g->max_cells : 1) * 4);
    acc((R + 1) * 4); acc((size_t)g->max_segs * 32);
    acc(RS * 4); acc(RS * 4);
    for (int q = 0; q < 5; ++q) acc(RS * NM * 8);
    acc(RS * NM * 4);
    acc(RS * NM * NM * 4);
    acc(RS * NM * NM * 8);
    acc(RS * NM * NM * 2);
    acc(RS * C * NP * NP * 4);
    acc(RS * NP * 4); acc(RS * NP * 4);
    acc(RS * 5 * 8);
    acc((RS * TO_RESULT_STRIDE + 64) * 8);
    acc((R + 1) * 4);
    acc(R * 16 * 4);
    acc(R * g->n_label_types * n * 4);
    const size_t cap = (size_t)NP * 32;
    acc(RS * C * (NP + 1) * 4); acc(RS * C * cap * 2); acc(RS * C * cap * 4); acc(RS * C * 4);
    acc(RS * C * 8);
    acc(RS * 4);                               // the MTE's launch order
    // union form of each road-species' C <= 3 matrices (the ROV forward
    // pass's form): the species models' patterns are nested - control c's
    // entries are a subset of the lowest-hazard control's - so a union
    // holds no more entries than that control's packed matrix
    const size_t ucap = C <= 3 ? cap : 0;
    if (C <= 3) { acc(RS * ucap * 16); acc(RS * (NP + 1) * 4); acc(RS * 4); }
    if ((e = cudaMalloc(&g->buf, bytes)) != cudaSuccess) return fail(e);
    g->buf_bytes = bytes;
    char* p = g->buf;
    g->d_cell_off = carve<int>(p, R + 1);
    g->d_cells = carve<int>(p, g->max_cells > 0 ? g->max_cells : 1);
    g->d_seg_off = carve<int>(p, R + 1);
    g->d_segs = carve<double>(p, (size_t)g->max_segs * 4);
    g->d_np = carve<int>(p, RS);
    g->d_nt = carve<int>(p, RS);
    g->d_area = carve<double>(p, RS * NM);
    g->d_cap = carve<double>(p, RS * NM);
    g->d_pop = carve<double>(p, RS * NM);
    g->d_cx = carve<double>(p, RS * NM);
    g->d_cy = carve<double>(p, RS * NM);
    g->d_type = carve<int>(p, RS * NM);
    g->d_cross = carve<int>(p, RS * NM * NM);
    g->d_tv = carve<double>(p, RS * NM * NM);
    g->d_tdest = carve<uint16_t>(p, RS * NM * NM);
    g->d_mmm = carve<float>(p, RS * C * NP * NP);
    g->d_ip = carve<float>(p, RS * NP);
    g->d_cp = carve<float>(p, RS * NP);
    g->d_stats = carve<double>(p, RS * 5);
    g->d_results = carve<double>(p, RS * TO_RESULT_STRIDE + 64);
    g->d_counts = carve<int>(p, R + 1);
    g->d_feat = carve<float>(p, R * 16);
    g->d_labels = carve<int>(p, R * g->n_label_types * n);
    g->csc.ptr = carve<int>(p, RS * C * (NP + 1));
    g->csc.idx = carve<uint16_t>(p, RS * C * cap);
    g->csc.val = carve<float>(p, RS * C * cap);
    g->csc.nnz = carve<int>(p, RS * C);
    g->csc.cap = (int)cap;
    g->csc.cap_smem = 0;
    g->d_iar = carve<double>(p, RS * C);
    g->d_mte_order = carve<int>(p, RS);
    g->csc.uent = nullptr; g->csc.uptr = nullptr; g->csc.unnz = nullptr;
    g->csc.ucap = 0; g->csc.ucap_smem = 0;
    if (C <= 3) {
        g->csc.uent = carve<int4>(p, RS * ucap);
        g->csc.uptr = carve<int>(p, RS * (NP + 1));
        g->csc.unnz = carve<int>(p, RS);
        g->csc.ucap = (int)ucap;
    }
    if ((e = cudaMalloc(&g->d_pen, (size_t)S * 3 * sizeof(double))) != cudaSuccess) return fail(e);
    if ((e = cudaMemset(g->d_pen, 0, (size_t)S * 3 * sizeof(double))) != cudaSuccess) return fail(e);
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return fail(e);
    *out = g;
    return TO_OK;
}

to_status to_scene_destroy(to_gen g) {
    if (!g) return TO_OK;
    if (g->ctx) cudaSetDevice(g->ctx->device);
    cudaDeviceSynchronize();
    if (g->exec) cudaGraphExecDestroy(g->exec);
    cudaFree(g->d_base);
    cudaFree(g->d_popmap);
    cudaFree(g->d_species);
    cudaFree(g->d_params);
    cudaFree(g->d_label_types);
    cudaFree(g->buf);
    cudaFree(g->d_end);
    cudaFree(g->d_pen);
    cudaFree(g->rov_buf);
    delete g;
    return TO_OK;
}

// Abramowitz & Stegun 26.2.23 rational approximation of the upper normal
// quantile, as Utility::NormalCDFInverse / RationalApproximation use it
// (include/utilities/Utility.cpp:165-193); |error| < 4.5e-4
static double normal_cdf_inverse(double p) {
    auto ra = [](double t) {
        return t - ((0.010328 * t + 0.802853) * t + 2.515517) /
                   (((0.001308 * t + 0.189269) * t + 1.432788) * t + 1.0);
    };
    return p < 0.5 ? -ra(std::sqrt(-2.0 * std::log(p))) : ra(std::sqrt(-2.0 * std::log(1.0 - p)));
}

to_status to_scene_set_penalty(to_ctx ctx, to_gen g, const to_penalty* pen) {
    if (!ctx || !g || !pen || !(pen->confidence > 0.0) || !(pen->confidence < 1.0) ||
        !pen->threshold || !pen->init_population || !pen->cost_per_animal)
        return TO_ERR_INVALID;
    cudaSetDevice(ctx->device);
    std::vector<double> h((size_t)g->S * 3);
    for (int s = 0; s < g->S; ++s) {
        h[3 * s] = pen->threshold[s];
        h[3 * s + 1] = pen->init_population[s];
        h[3 * s + 2] = pen->cost_per_animal[s];
        for (int q = 0; q < 3; ++q)
            if (!std::isfinite(h[3 * s + q]))
                return to_set_error(ctx, TO_ERR_NONFINITE, "penalty of species %d", s);
    }
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    TO_CUDA(ctx, cudaMemcpy(g->d_pen, h.data(), h.size() * sizeof(double),
                            cudaMemcpyHostToDevice));
    g->pen_z = normal_cdf_inverse(1.0 - pen->confidence);
    return TO_OK;
}

to_status to_scene_set_rov(to_ctx ctx, to_gen g, const to_rov_problem* t) {
    if (!ctx || !g) return TO_ERR_INVALID;
    cudaSetDevice(ctx->device);
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (g->exec) { cudaGraphExecDestroy(g->exec); g->exec = nullptr; }
    g->rov_on = false;
    if (g->rov_buf) { cudaFree(g->rov_buf); g->rov_buf = nullptr; g->rov_bytes = 0; }
    if (!t) return TO_OK;
    const int S = g->S, C = g->C, P = t->n_paths, Y = t->n_years, U = t->n_uncertainties;
    const int Rr = t->dim_res, d = S + 1, NR = g->max_roads;
    const int algo = t->algo == 0 ? 4 : t->algo;
    if (t->n_species != S || t->n_controls != C || P < 128 || Y < 3 || Rr < 2 || U < 0 ||
        (U > 0 && !t->uncert) || !t->flows || t->n_fuels < 0 || t->n_commodities < 0 ||
        t->n_fuels + t->n_commodities > U || t->n_fuels > 16 || t->n_commodities > 16 ||
        t->demand_idx >= U)
        return TO_ERR_INVALID;
    if (t->sem != 1 || algo != 4 || d > TO_LSM_MAXD)
        return to_set_error(ctx, TO_ERR_UNSUPPORTED,
                            "a generation's ROV is ALGO4 with corrected semantics, <= %d species",
                            TO_LSM_MAXD - 1);
    for (int f = 0; f < t->n_fuels; ++f)
        if (!t->fuel_costs || !t->fuel_idx || t->fuel_idx[f] < 0 || t->fuel_idx[f] >= U)
            return TO_ERR_INVALID;
    if (t->n_commodities > 0 && (!t->ore_content || !t->ore_sd)) return TO_ERR_INVALID;
    for (int i = 0; i < 6 * U; ++i)
        if (!std::isfinite(t->uncert[i])) return to_set_error(ctx, TO_ERR_NONFINITE, "uncert %d", i);
    long Ql = 1;
    for (int j = 0; j < d; ++j) Ql *= Rr;
    if (Ql > (1L << 22) || (long)NR * C * Ql > 0x7fffffffL)
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "grid %ld x %d groups", Ql, NR * C);
    const int Q = (int)Ql;
    if ((long)NR * P > (1L << 30)) return to_set_error(ctx, TO_ERR_UNSUPPORTED, "paths");
    int kmax = (P > 3) ? (int)(10.0 * (std::log((double)P) + 1.0)) : 1;
    if (kmax > P) kmax = P;
    if (kmax > TO_KNN_KMAX) return to_set_error(ctx, TO_ERR_UNSUPPORTED, "k %d", kmax);
    const size_t PT = (size_t)NR * P, G = (size_t)NR * C;
    const size_t blk = (size_t)Rr * d + 2 * (size_t)Q;
    const size_t nacc = (size_t)(d + 1) * (d + 4) / 2;   // sums a query (doubles)
    const int lblocks = (int)((PT + 1023) / 1024);
    const size_t U1 = (size_t)(U > 0 ? U : 1);
    size_t bytes = 0;
    auto acc = [&](size_t b) { bytes += to_align256(b); };
    acc(C * 4); acc(6 * U1 * 4); acc(16 * 4); acc(16 * 4); acc(16 * 4); acc(16 * 4);
    acc(NR * 4); acc((size_t)NR * 5 * 8); acc((size_t)S * 8 * 4);
    acc((size_t)Y * PT * 4); acc(U1 * (Y + 1) * PT * 4); acc((size_t)S * (Y + 1) * PT * 4);
    acc((size_t)S * C * Y * PT * 4);
    acc(G * d * P * 4); acc(G * d * P * 4); acc(G * P * 4); acc(G * 4); acc(G * 4);
    acc((size_t)NR * d * 4); acc((size_t)NR * d * 4); acc(G * d * P * 4); acc(G * P * 4);
    acc((size_t)NR * d * Rr * 4);
    acc(G * (TO_KNN_GCELLS + 1) * 4); acc(G * sizeof(to_knn_grid)); acc(G * Q * 4);
    acc(G * lblocks * 4); acc(G * d * 2 * 4); acc(4); acc(G * Q * nacc * 8);
    acc(G * blk * 4);
    acc((size_t)Y * PT * 4); acc((size_t)Y * PT * 4); acc((size_t)Y * PT * 4);
    acc((size_t)Y * S * PT * 4);
    acc(G * Q); acc(G * Q * 4); acc(4); acc((size_t)NR * 4);
    cudaError_t e = cudaMalloc(&g->rov_buf, bytes);
    if (e != cudaSuccess) {
        g->rov_buf = nullptr;
        cudaGetLastError();
        return to_set_error(ctx, e == cudaErrorMemoryAllocation ? TO_ERR_ALLOC : TO_ERR_CUDA,
                            "%zu bytes of ROV scratch", bytes);
    }
    TO_CUDA(ctx, cudaMemset(g->rov_buf, 0, bytes));
    g->rov_bytes = bytes;
    char* p = g->rov_buf;
    to_rov_args a;
    memset(&a, 0, sizeof(a));
    a.P = P; a.Y = Y; a.S = S; a.C = C; a.U = U; a.R = Rr; a.Q = Q;
    a.nF = t->n_fuels; a.Cm = t->n_commodities; a.demand_idx = t->demand_idx;
    a.sem = 1; a.road = 0; a.dt = t->dt; a.rrr = t->rrr;
    a.unit_cost = t->unit_cost; a.unit_revenue = t->unit_revenue; a.scaling = 2.0f;
    a.seed = t->seed; a.kmax = kmax; a.algo = 4; a.k_mult = 10;
    a.touched = 1; a.reg_one_year = 1; a.flags = ctx->d_flags;
    float* d_flows = carve<float>(p, C);
    float* d_unc = carve<float>(p, 6 * U1);
    float* d_fc = carve<float>(p, 16);
    int* d_fi = carve<int>(p, 16);
    float* d_oc = carve<float>(p, 16);
    float* d_os = carve<float>(p, 16);
    g->d_road_ids = carve<int>(p, NR);
    g->d_rov_stats = carve<double>(p, (size_t)NR * 5);
    g->d_rov_params = carve<float>(p, (size_t)S * 8);
    a.controls = carve<int>(p, (size_t)Y * PT);
    a.uRes = carve<float>(p, U1 * (Y + 1) * PT);
    a.totalPops = carve<float>(p, (size_t)S * (Y + 1) * PT);
    a.aars = carve<float>(p, (size_t)S * C * Y * PT);
    a.xraw = carve<float>(p, G * d * P);
    a.xn = carve<float>(p, G * d * P);
    a.yv = carve<float>(p, G * P);
    a.npts = carve<int>(p, G);
    a.kc = carve<int>(p, G);
    a.gmin = carve<float>(p, (size_t)NR * d);
    a.gmax = carve<float>(p, (size_t)NR * d);
    a.qax = carve<float>(p, (size_t)NR * d * Rr);
    a.gsx = carve<float>(p, G * d * P);
    a.gsi = carve<int>(p, G * P);
    a.gcell = carve<int>(p, G * (TO_KNN_GCELLS + 1));
    a.ggrid = carve<to_knn_grid>(p, G);
    a.kth = carve<float>(p, G * Q);
    a.lcnt = carve<int>(p, G * lblocks);
    a.lkey = carve<unsigned>(p, G * d * 2);
    a.knn_next = carve<int>(p, 1);
    a.knn_acc = carve<double>(p, G * Q * nacc);
    a.reg = carve<float>(p, G * blk);
    a.condExp = carve<float>(p, (size_t)Y * PT);
    a.optCont = carve<int>(p, (size_t)Y * PT);
    a.unitProfits = carve<float>(p, (size_t)Y * PT);
    a.adjPops = carve<float>(p, (size_t)Y * S * PT);
    a.qmark = carve<unsigned char>(p, G * Q);
    a.qlist = carve<int>(p, G * Q);
    a.qcount = carve<int>(p, 1);
    a.qroad = carve<unsigned>(p, NR);
    TO_CUDA(ctx, cudaMemcpy(d_flows, t->flows, C * sizeof(float), cudaMemcpyHostToDevice));
    if (U > 0)
        TO_CUDA(ctx, cudaMemcpy(d_unc, t->uncert, 6 * (size_t)U * sizeof(float),
                                cudaMemcpyHostToDevice));
    if (t->n_fuels > 0) {
        TO_CUDA(ctx, cudaMemcpy(d_fc, t->fuel_costs, t->n_fuels * sizeof(float),
                                cudaMemcpyHostToDevice));
        TO_CUDA(ctx, cudaMemcpy(d_fi, t->fuel_idx, t->n_fuels * sizeof(int),
                                cudaMemcpyHostToDevice));
    }
    if (t->n_commodities > 0) {
        TO_CUDA(ctx, cudaMemcpy(d_oc, t->ore_content, t->n_commodities * sizeof(float),
                                cudaMemcpyHostToDevice));
        TO_CUDA(ctx, cudaMemcpy(d_os, t->ore_sd, t->n_commodities * sizeof(float),
                                cudaMemcpyHostToDevice));
    }
    a.flows = d_flows; a.uncert = d_unc; a.fuel_costs = d_fc; a.fuel_idx = d_fi;
    a.ore_content = d_oc; a.ore_sd = d_os;
    // species parameters of the ROV: the template's where it gives them,
    // else the scene's (the MTE's)
    if (t->species) {
        std::vector<float> prm((size_t)S * 8);
        for (int sp = 0; sp < S; ++sp) {
            if (!t->species[sp].params) return TO_ERR_INVALID;
            for (int q = 0; q < 8; ++q) prm[(size_t)sp * 8 + q] = t->species[sp].params[q];
        }
        TO_CUDA(ctx, cudaMemcpy(g->d_rov_params, prm.data(), prm.size() * sizeof(float),
                                cudaMemcpyHostToDevice));
    } else {
        TO_CUDA(ctx, cudaMemcpy(g->d_rov_params, g->d_params, (size_t)S * 8 * sizeof(float),
                                cudaMemcpyDeviceToDevice));
    }
    g->rov = a;
    g->rov_on = true;
    return TO_OK;
}

static to_status check_eval(to_ctx ctx, to_gen g, int R, const to_eval_opts* o) {
    if (!ctx || !g || !o || R <= 0 || R > g->max_roads || o->mte_paths <= 0 ||
        o->n_years < 0)
        return TO_ERR_INVALID;
    return TO_OK;
}

to_status to_evaluate_roads(to_ctx ctx, to_gen g, int R, const int* cell_off,
                            const int* cells, const int* seg_off,
                            const double* segs, const to_eval_opts* o,
                            double* results) {
    TO_TRY(check_eval(ctx, g, R, o));
    if (!seg_off || !segs || !results || (!cell_off != !cells && cell_off && cell_off[R] > 0))
        return TO_ERR_INVALID;
    cudaSetDevice(ctx->device);
    const bool raster = (cell_off == nullptr);
    const int ncell = raster ? 0 : cell_off[R] - cell_off[0];
    const int nseg = seg_off[R] - seg_off[0];
    if ((!raster && cell_off[0] != 0) || seg_off[0] != 0 || ncell > g->max_cells ||
        nseg > g->max_segs || (ncell > 0 && !cells))
        return TO_ERR_INVALID;
    for (int r = 0; r < R; ++r)
        if ((!raster && cell_off[r + 1] < cell_off[r]) || seg_off[r + 1] < seg_off[r])
            return TO_ERR_INVALID;
    for (int q = 0; q < ncell; ++q)
        if (cells[q] < 0 || cells[q] >= g->W * g->H) return TO_ERR_INVALID;
    for (int q = 0; q < 4 * nseg; ++q)
        if (!std::isfinite(segs[q])) return to_set_error(ctx, TO_ERR_NONFINITE, "segment %d", q / 4);
    if (!raster) {
        TO_CUDA(ctx, cudaMemcpyAsync(g->d_cell_off, cell_off, (R + 1) * sizeof(int),
                                     cudaMemcpyHostToDevice, ctx->stream));
        if (ncell > 0)
            TO_CUDA(ctx, cudaMemcpyAsync(g->d_cells, cells, ncell * sizeof(int),
                                         cudaMemcpyHostToDevice, ctx->stream));
    }
    TO_CUDA(ctx, cudaMemcpyAsync(g->d_seg_off, seg_off, (R + 1) * sizeof(int),
                                 cudaMemcpyHostToDevice, ctx->stream));
    TO_CUDA(ctx, cudaMemcpyAsync(g->d_segs, segs, (size_t)nseg * 4 * sizeof(double),
                                 cudaMemcpyHostToDevice, ctx->stream));
    TO_TRY(evaluate(ctx, g, R, raster ? nullptr : g->d_cell_off, raster ? nullptr : g->d_cells,
                    g->d_seg_off, g->d_segs, o, g->d_results));
    TO_CUDA(ctx, cudaMemcpyAsync(results, g->d_results,
                                 (size_t)R * g->S * TO_RESULT_STRIDE * sizeof(double),
                                 cudaMemcpyDeviceToHost, ctx->stream));
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    int f = 0;
    TO_TRY(to_read_device_flags(ctx, &f));
    if (f == TO_DEVERR_PLAN && o->graph) {
        // a road outside the captured plan: drop the graph, plan and run again
        int z = 0;
        TO_CUDA(ctx, cudaMemcpy(ctx->d_flags, &z, sizeof(int), cudaMemcpyHostToDevice));
        if (g->exec) { cudaGraphExecDestroy(g->exec); g->exec = nullptr; }
        TO_TRY(evaluate(ctx, g, R, raster ? nullptr : g->d_cell_off,
                        raster ? nullptr : g->d_cells, g->d_seg_off, g->d_segs, o, g->d_results));
        TO_CUDA(ctx, cudaMemcpyAsync(results, g->d_results,
                                     (size_t)R * g->S * TO_RESULT_STRIDE * sizeof(double),
                                     cudaMemcpyDeviceToHost, ctx->stream));
        TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        TO_TRY(to_read_device_flags(ctx, &f));
    }
    if (f != 0) {
        cudaMemsetAsync(ctx->d_flags, 0, sizeof(int), ctx->stream);
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "device check %d failed", f);
    }
    return TO_OK;
}

to_status to_evaluate_roads_d(to_ctx ctx, to_gen g, int R, const int* cell_off,
                              const int* cells, const int* seg_off,
                              const double* segs, const to_eval_opts* o,
                              double* results) {
    TO_TRY(check_eval(ctx, g, R, o));
    if (!seg_off || !segs || !results || (!cell_off != !cells)) return TO_ERR_INVALID;
    cudaSetDevice(ctx->device);
    return evaluate(ctx, g, R, cell_off, cells, seg_off, segs, o, results);
}

to_status to_road_features_d(to_ctx ctx, to_gen g, int R, const int* seg_off,
                             const double* segs, const int* cell_off, const int* cells,
                             float* features) {
    if (!ctx || !g || R <= 0 || R > g->max_roads || !seg_off || !segs || !features ||
        (!cell_off != !cells))
        return TO_ERR_INVALID;
    cudaSetDevice(ctx->device);
    if (!cell_off) {
        TO_TRY(to_k::rasterise_roads(ctx, R, seg_off, segs, g->W, g->H, g->xs, g->ys, TO_SEM_CORRECTED,
                                     g->d_cell_off, g->d_cells, g->max_cells, g->d_counts));
        cell_off = g->d_cell_off;
        cells = g->d_cells;
    }
    return to_k::road_features(ctx, R, g->W, g->H, g->d_base, g->d_popmap, seg_off, segs,
                               cell_off, cells, features);
}

to_status to_road_features(to_ctx ctx, to_gen g, int R, const int* seg_off, const double* segs,
                           float* features) {
    if (!ctx || !g || R <= 0 || R > g->max_roads || !seg_off || !segs || !features)
        return TO_ERR_INVALID;
    cudaSetDevice(ctx->device);
    const int nseg = seg_off[R] - seg_off[0];
    if (seg_off[0] != 0 || nseg > g->max_segs) return TO_ERR_INVALID;
    for (int q = 0; q < 4 * nseg; ++q)
        if (!std::isfinite(segs[q])) return to_set_error(ctx, TO_ERR_NONFINITE, "segment %d", q / 4);
    TO_CUDA(ctx, cudaMemcpyAsync(g->d_seg_off, seg_off, (R + 1) * sizeof(int),
                                 cudaMemcpyHostToDevice, ctx->stream));
    TO_CUDA(ctx, cudaMemcpyAsync(g->d_segs, segs, (size_t)nseg * 4 * sizeof(double),
                                 cudaMemcpyHostToDevice, ctx->stream));
    TO_TRY(to_road_features_d(ctx, g, R, g->d_seg_off, g->d_segs, nullptr, nullptr, g->d_feat));
    TO_CUDA(ctx, cudaMemcpyAsync(features, g->d_feat, (size_t)R * 16 * sizeof(float),
                                 cudaMemcpyDeviceToHost, ctx->stream));
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    int f = 0;
    TO_TRY(to_read_device_flags(ctx, &f));
    if (f != 0) {
        cudaMemsetAsync(ctx->d_flags, 0, sizeof(int), ctx->stream);
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "road cells exceed the scene capacity");
    }
    return TO_OK;
}

to_status to_gen_end_pops(to_ctx ctx, to_gen g, int road, int species, int n_paths,
                          float* out) {
    if (!ctx || !g || !out || road < 0 || road >= g->last_R || species < 0 ||
        species >= g->S || n_paths != g->last_paths || !g->d_end)
        return TO_ERR_INVALID;
    cudaSetDevice(ctx->device);
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const size_t rs = (size_t)road * g->S + species;
    TO_CUDA(ctx, cudaMemcpy(out, g->d_end + rs * n_paths, (size_t)n_paths * sizeof(float),
                            cudaMemcpyDeviceToHost));
    return TO_OK;
}

to_status to_gen_species_model(to_ctx ctx, to_gen g, int road, int species, int max_patches,
                               int* n_patches, float* init_pops, float* caps, float* mmm,
                               int* nnz) {
    if (!ctx || !g || !n_patches || road < 0 || road >= g->last_R || species < 0 ||
        species >= g->S || max_patches <= 0)
        return TO_ERR_INVALID;
    cudaSetDevice(ctx->device);
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const size_t rs = (size_t)road * g->S + species;
    const int C = g->C, NP = g->NP;
    int N = 0;
    TO_CUDA(ctx, cudaMemcpy(&N, g->d_np + rs, sizeof(int), cudaMemcpyDeviceToHost));
    *n_patches = N;
    if (N > max_patches || N > NP) return to_set_error(ctx, TO_ERR_INVALID, "%d patches", N);
    if (init_pops)
        TO_CUDA(ctx, cudaMemcpy(init_pops, g->d_ip + rs * NP, (size_t)N * sizeof(float),
                                cudaMemcpyDeviceToHost));
    if (caps)
        TO_CUDA(ctx, cudaMemcpy(caps, g->d_cp + rs * NP, (size_t)N * sizeof(float),
                                cudaMemcpyDeviceToHost));
    std::vector<int> nz(C, -1);
    if (g->last_csc)
        TO_CUDA(ctx, cudaMemcpy(nz.data(), g->csc.nnz + rs * C, C * sizeof(int),
                                cudaMemcpyDeviceToHost));
    if (nnz) for (int c = 0; c < C; ++c) nnz[c] = nz[c];
    if (!mmm) return TO_OK;
    std::vector<float> dense((size_t)NP * NP);
    std::vector<int> ptr(NP + 1);
    std::vector<uint16_t> idx;
    std::vector<float> val;
    for (int c = 0; c < C; ++c) {
        const size_t mtx = rs * C + c;
        float* o = mmm + (size_t)c * N * N;
        if (g->last_csc && nz[c] >= 0) {
            // the packed form the sparse kernel read, expanded
            TO_CUDA(ctx, cudaMemcpy(ptr.data(), g->csc.ptr + mtx * (NP + 1),
                                    (NP + 1) * sizeof(int), cudaMemcpyDeviceToHost));
            idx.resize(nz[c] > 0 ? nz[c] : 1);
            val.resize(nz[c] > 0 ? nz[c] : 1);
            if (nz[c] > 0) {
                TO_CUDA(ctx, cudaMemcpy(idx.data(), g->csc.idx + mtx * g->csc.cap,
                                        nz[c] * sizeof(uint16_t), cudaMemcpyDeviceToHost));
                TO_CUDA(ctx, cudaMemcpy(val.data(), g->csc.val + mtx * g->csc.cap,
                                        nz[c] * sizeof(float), cudaMemcpyDeviceToHost));
            }
            memset(o, 0, (size_t)N * N * sizeof(float));
            for (int k = 0; k < N; ++k)
                for (int e = ptr[k]; e < ptr[k + 1]; ++e) {
                    if (e < 0 || e >= nz[c] || idx[e] >= N)
                        return to_set_error(ctx, TO_ERR_INVALID, "packed matrix %d", c);
                    o[(size_t)k * N + idx[e]] = val[e];
                }
        } else if (g->last_dense) {
            TO_CUDA(ctx, cudaMemcpy(dense.data(), g->d_mmm + mtx * NP * NP,
                                    (size_t)NP * NP * sizeof(float), cudaMemcpyDeviceToHost));
            for (int k = 0; k < N; ++k)
                memcpy(o + (size_t)k * N, dense.data() + (size_t)k * NP, N * sizeof(float));
        } else {
            return to_set_error(ctx, TO_ERR_INVALID, "no matrix form of control %d", c);
        }
    }
    return TO_OK;
}

}  // extern "C"
