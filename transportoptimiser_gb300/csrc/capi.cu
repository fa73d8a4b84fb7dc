// capi.cu - the C ABI (include/transopt.h): contexts, scratch arena and the
// host-pointer entry points that mirror TransportOptimiser's SimulateGPU::
// wrappers.  Each wrapper packs its inputs into the device layout, enqueues
// the kernels on the context stream and copies the results back, the same
// contract as the reference (which did cudaMalloc / H2D / launch /
// cudaDeviceSynchronize / D2H / cudaFree inside every call).
#include <cmath>
#include <cstdarg>
#include <string>
#include <vector>

#include "to_grid.h"
#include "to_internal.cuh"
#include "to_model.cuh"
#include "to_pop.cuh"
#include "to_sparse.cuh"

to_status to_set_error(to_ctx ctx, to_status s, const char* fmt, ...) {
    if (ctx) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(ctx->err, sizeof(ctx->err), fmt, ap);
        va_end(ap);
    }
    return s;
}

to_status to_check_cuda(to_ctx ctx, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return TO_OK;
    to_set_error(ctx, e == cudaErrorMemoryAllocation ? TO_ERR_ALLOC : TO_ERR_CUDA,
                 "%s: %s", what, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? TO_ERR_ALLOC : TO_ERR_CUDA;
}

to_status to_arena_reserve(to_ctx ctx, size_t bytes) {
    ctx->arena_off = 0;
    if (ctx->fault == TO_FAULT_ALLOC) {
        // test hook: this reservation is refused as a failed allocation would be
        ctx->fault = TO_FAULT_NONE;
        return to_set_error(ctx, TO_ERR_ALLOC, "scratch of %zu bytes refused (injected)", bytes);
    }
    if (bytes <= ctx->arena_cap) return TO_OK;
    if (ctx->arena) {
        TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        TO_CUDA(ctx, cudaFree(ctx->arena));
        ctx->arena = nullptr;
        ctx->arena_cap = 0;
    }
    size_t cap = bytes + bytes / 4 + (1 << 20);
    const cudaError_t e = cudaMalloc(&ctx->arena, cap);
    if (e != cudaSuccess) {
        ctx->arena = nullptr;
        cudaGetLastError();
        return to_set_error(ctx, e == cudaErrorMemoryAllocation ? TO_ERR_ALLOC : TO_ERR_CUDA,
                            "scratch of %zu bytes: %s", cap, cudaGetErrorString(e));
    }
    ctx->arena_cap = cap;
    return TO_OK;
}

to_status to_read_device_flags(to_ctx ctx, int* flag) {
    TO_CUDA(ctx, cudaMemcpyAsync(flag, ctx->d_flags, sizeof(int),
                                 cudaMemcpyDeviceToHost, ctx->stream));
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return TO_OK;
}

void to_prof_begin(to_ctx ctx, const char* name) {
    if (!ctx->profile || ctx->n_prof >= to_ctx_s::kMaxProf) return;
    int i = ctx->n_prof;
    if (i >= ctx->prof_ev_alloc) {
        cudaEventCreate(&ctx->prof_ev[i][0]);
        cudaEventCreate(&ctx->prof_ev[i][1]);
        ctx->prof_ev_alloc = i + 1;
    }
    ctx->prof_name[i] = name;
    cudaEventRecord(ctx->prof_ev[i][0], ctx->stream);
}

void to_prof_end(to_ctx ctx) {
    if (!ctx->profile || ctx->n_prof >= to_ctx_s::kMaxProf) return;
    cudaEventRecord(ctx->prof_ev[ctx->n_prof][1], ctx->stream);
    ctx->n_prof++;
}

to_status to_check_device_flags(to_ctx ctx) {
    int f = 0;
    TO_TRY(to_read_device_flags(ctx, &f));
    if (f != TO_DEVERR_NONE) {
        int z = 0;
        TO_CUDA(ctx, cudaMemcpyAsync(ctx->d_flags, &z, sizeof(int),
                                     cudaMemcpyHostToDevice, ctx->stream));
        TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        const char* what = f == TO_DEVERR_REGIONS ? "too many regions in a block"
                         : f == TO_DEVERR_UNION ? "union-find did not converge"
                         : f == TO_DEVERR_PATCHES ? "patch capacity exceeded"
                         : f == TO_DEVERR_SPIN ? "bounded wait expired"
                         : f == TO_DEVERR_CELL ? "road cell outside the grid"
                         : f == TO_DEVERR_PLAN ? "roads outgrew the captured plan"
                         : "device check failed";
        return to_set_error(ctx, f == TO_DEVERR_SPIN ? TO_ERR_TIMEOUT
                                                      : TO_ERR_UNSUPPORTED,
                            "%s", what);
    }
    return TO_OK;
}

template <class T>
static to_status h2d(to_ctx ctx, T* d, const T* h, size_t n) {
    if (n == 0) return TO_OK;
    TO_CUDA(ctx, cudaMemcpyAsync(d, h, n * sizeof(T), cudaMemcpyHostToDevice,
                                 ctx->stream));
    return TO_OK;
}
template <class T>
static to_status d2h(to_ctx ctx, T* h, const T* d, size_t n) {
    if (n == 0) return TO_OK;
    TO_CUDA(ctx, cudaMemcpyAsync(h, d, n * sizeof(T), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    return TO_OK;
}

extern "C" {

const char* to_status_string(to_status s) {
    switch (s) {
        case TO_OK: return "ok";
        case TO_ERR_INVALID: return "invalid argument";
        case TO_ERR_CUDA: return "CUDA error";
        case TO_ERR_ALLOC: return "allocation failed";
        case TO_ERR_NONFINITE: return "non-finite input";
        case TO_ERR_TIMEOUT: return "bounded device wait expired";
        case TO_ERR_UNSUPPORTED: return "unsupported size or mode";
        case TO_ERR_NO_DEVICE: return "no CUDA device";
    }
    return "unknown status";
}

const char* to_last_error(to_ctx ctx) { return ctx ? ctx->err : ""; }

to_status to_ctx_inject_fault(to_ctx ctx, int fault) {
    if (!ctx || fault < TO_FAULT_NONE || fault > TO_FAULT_WAIT) return TO_ERR_INVALID;
    ctx->fault = fault;
    return TO_OK;
}

to_status to_ctx_profile(to_ctx ctx, int enable) {
    if (!ctx) return TO_ERR_INVALID;
    ctx->profile = enable != 0;
    ctx->n_prof = 0;
    return TO_OK;
}

to_status to_ctx_kernel_time(to_ctx ctx, const char* name, double* ms, int* launches) {
    if (!ctx || !name || !ms) return TO_ERR_INVALID;
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double tot = 0.0;
    int cnt = 0;
    for (int i = 0; i < ctx->n_prof; ++i) {
        if (strcmp(ctx->prof_name[i], name) != 0) continue;
        float t = 0.0f;
        TO_CUDA(ctx, cudaEventElapsedTime(&t, ctx->prof_ev[i][0], ctx->prof_ev[i][1]));
        tot += t;
        ++cnt;
    }
    *ms = tot;
    if (launches) *launches = cnt;
    return TO_OK;
}
uint64_t to_ctx_launch_count(to_ctx ctx) { return ctx ? ctx->launches : 0; }

to_status to_device_count(int* count) {
    if (!count) return TO_ERR_INVALID;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) { cudaGetLastError(); *count = 0; return TO_OK; }
    *count = n;
    return TO_OK;
}

to_status to_ctx_create(int device, to_ctx* out) {
    if (!out) return TO_ERR_INVALID;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return TO_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= n) return TO_ERR_INVALID;
    to_ctx ctx = new to_ctx_s();
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess) { delete ctx; return TO_ERR_CUDA; }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) { delete ctx; return TO_ERR_CUDA; }
    ctx->sm_count = prop.multiProcessorCount;
    ctx->smem_optin = prop.sharedMemPerBlockOptin;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return TO_ERR_CUDA;
    }
    ctx->own_stream = true;
    if (cudaMalloc(&ctx->d_flags, 64 * sizeof(int)) != cudaSuccess) {
        cudaStreamDestroy(ctx->stream);
        delete ctx;
        return TO_ERR_ALLOC;
    }
    cudaMemset(ctx->d_flags, 0, 64 * sizeof(int));
    cudaDeviceSynchronize();
    *out = ctx;
    return TO_OK;
}

to_status to_ctx_destroy(to_ctx ctx) {
    if (!ctx) return TO_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->arena) cudaFree(ctx->arena);
    if (ctx->tc_buf) cudaFree(ctx->tc_buf);
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    if (ctx->d_flags) cudaFree(ctx->d_flags);
    for (int i = 0; i < ctx->prof_ev_alloc; ++i) {
        cudaEventDestroy(ctx->prof_ev[i][0]);
        cudaEventDestroy(ctx->prof_ev[i][1]);
    }
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return TO_OK;
}

to_status to_ctx_set_stream(to_ctx ctx, void* stream) {
    if (!ctx) return TO_ERR_INVALID;
    if (ctx->own_stream && ctx->stream) {
        cudaStreamSynchronize(ctx->stream);
        cudaStreamDestroy(ctx->stream);
    }
    ctx->stream = (cudaStream_t)stream;
    ctx->own_stream = false;
    return TO_OK;
}

int to_ctx_tuning(to_ctx ctx, char* buf, int len) {
    if (!ctx) return 0;
    static const char* names[3] = {"sparse", "simt", "tc"};
    std::string out;
    for (const auto& e : ctx->tune) {
        char line[256];
        snprintf(line, sizeof(line), "%s ne=%d paths=%d rs=%d -> %s (sparse %.3f ms, simt %.3f ms, tc %.3f ms)\n",
                 e.kind == 0 ? "generation" : "mte", e.ne, e.paths, e.n_rs,
                 names[e.choice < 0 || e.choice > 2 ? 1 : e.choice], e.ms[0], e.ms[1], e.ms[2]);
        out += line;
    }
    if (buf && len > 0) {
        size_t n = out.size() < (size_t)(len - 1) ? out.size() : (size_t)(len - 1);
        memcpy(buf, out.data(), n);
        buf[n] = 0;
    }
    return (int)ctx->tune.size();
}

to_status to_ctx_synchronize(to_ctx ctx) {
    if (!ctx) return TO_ERR_INVALID;
    cudaSetDevice(ctx->device);
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    // what the enqueued `_d` work reported on the device (a plan outgrown, a
    // bounded wait run out), read and cleared
    return to_check_device_flags(ctx);
}

// ---- LabelImage ------------------------------------------------------------
to_status to_label_image(to_ctx ctx, int W, int H, const int* input,
                         int* output, int* n_regions) {
    if (!ctx || !input || !output || W <= 0 || H <= 0) return TO_ERR_INVALID;
    cudaSetDevice(ctx->device);
    size_t n = (size_t)W * H;
    TO_TRY(to_arena_reserve(ctx, 2 * to_align256(n * 4) + 256));
    int* d_in = to_arena_take<int>(ctx, n);
    int* d_out = to_arena_take<int>(ctx, n);
    int* d_nr = to_arena_take<int>(ctx, 1);
    TO_TRY(h2d(ctx, d_in, input, n));
    TO_TRY(to_k::label_image(ctx, W, H, d_in, d_out, d_nr));
    TO_TRY(d2h(ctx, output, d_out, n));
    int nr = 0;
    TO_TRY(d2h(ctx, &nr, d_nr, 1));
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    TO_TRY(to_check_device_flags(ctx));
    if (n_regions) *n_regions = nr;
    return TO_OK;
}

// ---- buildPatches ----------------------------------------------------------
to_status to_build_patches(to_ctx ctx, int W, int H, int skpx, int skpy,
                           int xres, int yres, int n_regions, double xspacing,
                           double yspacing, double sub_patch_area,
                           double max_pop, const int* labels,
                           const double* pops, int max_patches, double* area,
                           double* cap, double* pop, double* cx, double* cy,
                           double* init_pop, int* n_patches) {
    if (!ctx || !labels || !pops || !n_patches || W <= 0 || H <= 0 ||
        skpx <= 0 || skpy <= 0 || xres <= 0 || yres <= 0 || max_patches < 0)
        return TO_ERR_INVALID;
    if (!to_blocks_inside(W, H, skpx, skpy, xres, yres))
        return to_set_error(ctx, TO_ERR_UNSUPPORTED,
                            "coarse blocks of %d x %d cells run past the %d x %d grid",
                            skpx, skpy, W, H);
    if (n_regions <= 0) return TO_OK;
    cudaSetDevice(ctx->device);
    size_t n = (size_t)W * H;
    int start = *n_patches;
    if (start > max_patches) return TO_ERR_INVALID;
    TO_TRY(to_arena_reserve(ctx, to_align256(n * 4) * 2 +
                                 to_align256((size_t)max_patches * 5 * 8) + 512));
    int* d_lab = to_arena_take<int>(ctx, n);
    float* d_pops = to_arena_take<float>(ctx, n);
    double* d_out = to_arena_take<double>(ctx, (size_t)5 * (max_patches > 0 ? max_patches : 1));
    int* d_cnt = to_arena_take<int>(ctx, 1);
    std::vector<float> pf(n);
    for (size_t i = 0; i < n; ++i) pf[i] = (float)pops[i];
    TO_TRY(h2d(ctx, d_lab, labels, n));
    TO_TRY(h2d(ctx, d_pops, pf.data(), n));
    TO_TRY(h2d(ctx, d_cnt, &start, 1));
    TO_TRY(to_k::build_patches(ctx, W, H, skpx, skpy, xres, yres, n_regions,
                               (float)xspacing, (float)yspacing,
                               (float)sub_patch_area, (float)max_pop, d_lab,
                               d_pops, max_patches, d_out, d_cnt));
    int end = 0;
    TO_TRY(d2h(ctx, &end, d_cnt, 1));
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    TO_TRY(to_check_device_flags(ctx));
    std::vector<double> o((size_t)5 * (end > start ? end - start : 0));
    if (end > start) {
        TO_CUDA(ctx, cudaMemcpy(o.data(), d_out + (size_t)5 * start,
                                o.size() * sizeof(double), cudaMemcpyDeviceToHost));
    }
    for (int i = start; i < end; ++i) {
        const double* v = &o[(size_t)5 * (i - start)];
        if (area) area[i] = v[0];
        if (cap) cap[i] = v[1];
        if (pop) pop[i] = v[2];
        if (cx) cx[i] = v[3];
        if (cy) cy[i] = v[4];
        if (init_pop) *init_pop += v[2];
    }
    *n_patches = end;
    return TO_OK;
}

// ---- lineSegmentIntersect --------------------------------------------------
to_status to_line_segment_intersect(to_ctx ctx, int T, const double* xy1,
                                    int G, const double* xy2, int* crossings) {
    if (!ctx || T < 0 || G < 0 || (T > 0 && (!xy1 || !crossings)) ||
        (G > 0 && !xy2))
        return TO_ERR_INVALID;
    if (T == 0) return TO_OK;
    cudaSetDevice(ctx->device);
    TO_TRY(to_arena_reserve(ctx, to_align256((size_t)T * 32) +
                                 to_align256((size_t)(G > 0 ? G : 1) * 32) +
                                 to_align256((size_t)T * 4)));
    double* d1 = to_arena_take<double>(ctx, (size_t)4 * T);
    double* d2 = to_arena_take<double>(ctx, (size_t)4 * (G > 0 ? G : 1));
    int* dc = to_arena_take<int>(ctx, T);
    TO_TRY(h2d(ctx, d1, xy1, (size_t)4 * T));
    if (G > 0) TO_TRY(h2d(ctx, d2, xy2, (size_t)4 * G));
    TO_TRY(to_k::line_segment_intersect(ctx, T, d1, G, d2, dc));
    TO_TRY(d2h(ctx, crossings, dc, T));
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return TO_OK;
}

// ---- species-road model ----------------------------------------------------
to_status to_species_model(to_ctx ctx, const to_species_in* in,
                           to_species_out* out) {
    if (!ctx || !in || !out || in->W <= 0 || in->H <= 0 || in->res <= 0 ||
        !in->hab_map || !in->pop_map || in->n_hab <= 0 ||
        in->n_hab > TO_MAX_HAB || in->n_controls <= 0 ||
        in->n_controls > TO_MAX_CONTROLS || !in->hazard || in->G < 0 ||
        (in->G > 0 && !in->road) || out->max_patches <= 0 || !out->area ||
        !out->cap || !out->pop || !out->cx || !out->cy || !out->type)
        return TO_ERR_INVALID;
    cudaSetDevice(ctx->device);
    const int W = in->W, H = in->H, res = in->res, C = in->n_controls;
    const int NM = out->max_patches;
    const int NP = (NM + 3) & ~3;
    to_model_args a;
    memset(&a, 0, sizeof(a));
    a.W = W; a.H = H; a.S = 1; a.C = C;
    a.xres = (W % res == 0) ? res : res + 1;
    a.yres = (H % res == 0) ? res : res + 1;
    a.skpx = (int)std::floor((double)(W - 1) / (double)res);
    a.skpy = (int)std::floor((double)(H - 1) / (double)res);
    if (a.skpx <= 0 || a.skpy <= 0) return TO_ERR_INVALID;
    if (!to_blocks_inside(W, H, a.skpx, a.skpy, a.xres, a.yres))
        return to_set_error(ctx, TO_ERR_UNSUPPORTED,
                            "coarse blocks of a %d x %d grid at resolution %d run past it",
                            W, H, res);
    a.xs = (float)in->xspacing; a.ys = (float)in->yspacing;
    a.spa = (float)(in->xspacing * in->yspacing);
    a.sem = in->sem; a.max_patches = NM; a.npad = NP;
    to_model_species hs;
    memset(&hs, 0, sizeof(hs));
    hs.n_hab = in->n_hab;
    for (int h = 0; h < in->n_hab; ++h) {
        hs.hab_type[h] = in->habs[h].type;
        hs.hab_max_pop[h] = in->habs[h].max_pop;
        hs.hab_pref_mean[h] = in->habs[h].pref_mean;
        hs.hab_pref_sd[h] = in->habs[h].pref_sd;
    }
    for (int c = 0; c < C; ++c) hs.hazard[c] = in->hazard[c];
    hs.lambda_mean = in->lambda_mean; hs.lambda_sd = in->lambda_sd;
    hs.lambda_mult = in->lambda_mult; hs.hab_pref_mult = in->hab_pref_mult;
    size_t n = (size_t)W * H;
    size_t bytes = to_align256(n * 4) * 2 + to_align256(sizeof(hs)) +
                   to_align256((size_t)(in->G > 0 ? in->G : 1) * 32) + 256 * 4 +
                   to_align256((size_t)NM * 8) * 5 + to_align256((size_t)NM * 4) +
                   to_align256((size_t)NM * NM * 4) * 2 +
                   to_align256((size_t)NM * NM * 8) * 2 +
                   to_align256((size_t)NM * NM * 2) +
                   to_align256((size_t)C * NM * NM * 8) +
                   to_align256((size_t)C * NP * NP * 4) + to_align256((size_t)NP * 4) * 2 +
                   to_align256((size_t)C * 8) + 4096;
    TO_TRY(to_arena_reserve(ctx, bytes));
    int* d_hab = to_arena_take<int>(ctx, n);
    float* d_pop = to_arena_take<float>(ctx, n);
    to_model_species* d_sp = to_arena_take<to_model_species>(ctx, 1);
    double* d_road = to_arena_take<double>(ctx, (size_t)4 * (in->G > 0 ? in->G : 1));
    int* d_G = to_arena_take<int>(ctx, 2);
    int* d_np = to_arena_take<int>(ctx, 1);
    int* d_nt = to_arena_take<int>(ctx, 1);
    a.area = to_arena_take<double>(ctx, NM);
    a.cap = to_arena_take<double>(ctx, NM);
    a.pop = to_arena_take<double>(ctx, NM);
    a.cx = to_arena_take<double>(ctx, NM);
    a.cy = to_arena_take<double>(ctx, NM);
    a.type = to_arena_take<int>(ctx, NM);
    a.crossings_scratch = to_arena_take<int>(ctx, (size_t)NM * NM);
    a.crossings_out = to_arena_take<int>(ctx, (size_t)NM * NM);
    a.trans_scratch = to_arena_take<double>(ctx, (size_t)NM * NM);
    a.trans_dest = to_arena_take<uint16_t>(ctx, (size_t)NM * NM);
    a.trans = to_arena_take<double>(ctx, (size_t)NM * NM);
    a.surv = to_arena_take<double>(ctx, (size_t)C * NM * NM);
    a.mmm = to_arena_take<float>(ctx, (size_t)C * NP * NP);
    a.init_pops = to_arena_take<float>(ctx, NP);
    a.caps = to_arena_take<float>(ctx, NP);
    a.iar = out->iar ? to_arena_take<double>(ctx, C) : nullptr;
    if (!a.caps || (out->iar && !a.iar)) return to_set_error(ctx, TO_ERR_ALLOC, "arena sizing");
    std::vector<float> pf(n);
    for (size_t i = 0; i < n; ++i) pf[i] = (float)in->pop_map[i];
    int G = in->G;
    std::vector<double> segs((size_t)4 * (G > 0 ? G : 1));
    for (int g = 0; g < G; ++g)
        for (int q = 0; q < 4; ++q) segs[(size_t)4 * g + q] = in->road[g + (size_t)q * G];
    int seg_off[2] = {0, G};
    TO_TRY(h2d(ctx, d_hab, in->hab_map, n));
    TO_TRY(h2d(ctx, d_pop, pf.data(), n));
    TO_TRY(h2d(ctx, d_sp, &hs, 1));
    if (G > 0) TO_TRY(h2d(ctx, d_road, segs.data(), (size_t)4 * G));
    TO_TRY(h2d(ctx, d_G, seg_off, 2));
    a.hab_map = d_hab; a.cell_off = nullptr; a.cells = nullptr; a.pop_map = d_pop;
    a.species = d_sp; a.segs = d_road; a.seg_off = d_G;
    a.n_patches = d_np; a.n_transitions = d_nt; a.d_flags = ctx->d_flags;
    TO_TRY(to_k::species_model(ctx, a, 1));
    int N = 0, nt = 0;
    TO_TRY(d2h(ctx, &N, d_np, 1));
    TO_TRY(d2h(ctx, &nt, d_nt, 1));
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    TO_TRY(to_check_device_flags(ctx));
    out->n_patches = N;
    out->n_transitions = nt;
    TO_TRY(d2h(ctx, out->area, a.area, N));
    TO_TRY(d2h(ctx, out->cap, a.cap, N));
    TO_TRY(d2h(ctx, out->pop, a.pop, N));
    TO_TRY(d2h(ctx, out->cx, a.cx, N));
    TO_TRY(d2h(ctx, out->cy, a.cy, N));
    TO_TRY(d2h(ctx, out->type, a.type, N));
    std::vector<int> cr;
    std::vector<double> tr, sv;
    std::vector<float> mm;
    if (out->crossings) { cr.resize((size_t)NM * NM); TO_TRY(d2h(ctx, cr.data(), a.crossings_out, cr.size())); }
    if (out->trans) { tr.resize((size_t)NM * NM); TO_TRY(d2h(ctx, tr.data(), a.trans, tr.size())); }
    if (out->surv) { sv.resize((size_t)C * NM * NM); TO_TRY(d2h(ctx, sv.data(), a.surv, sv.size())); }
    if (out->mmm) { mm.resize((size_t)C * NP * NP); TO_TRY(d2h(ctx, mm.data(), a.mmm, mm.size())); }
    if (out->iar) TO_TRY(d2h(ctx, out->iar, a.iar, (size_t)C));
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) {
            if (out->crossings) out->crossings[(size_t)i * N + j] = cr[(size_t)i * NM + j];
            if (out->trans) out->trans[(size_t)i * N + j] = tr[(size_t)i * NM + j];
            for (int c = 0; c < C; ++c) {
                if (out->surv) out->surv[((size_t)c * N + i) * N + j] = sv[((size_t)c * NM + i) * NM + j];
                if (out->mmm) out->mmm[((size_t)c * N + i) * N + j] = mm[((size_t)c * NP + i) * NP + j];
            }
        }
    return TO_OK;
}

// ---- MTE -------------------------------------------------------------------
to_status to_simulate_mte(to_ctx ctx, const to_mte_problem* prob,
                          double* end_pops, to_mte_stats* stats) {
    if (!ctx || !prob || prob->n_species <= 0 || prob->n_paths <= 0 ||
        prob->n_years < 0 || !prob->species)
        return TO_ERR_INVALID;
    cudaSetDevice(ctx->device);
    const int S = prob->n_species, P = prob->n_paths;
    int maxN = 0;
    for (int s = 0; s < S; ++s) {
        const to_mte_species& sp = prob->species[s];
        if (sp.n_patches <= 0 || !sp.params || !sp.init_pops || !sp.caps || !sp.mmm)
            return TO_ERR_INVALID;
        if (sp.n_patches > maxN) maxN = sp.n_patches;
        for (int k = 0; k < sp.n_patches; ++k)
            if (!std::isfinite(sp.init_pops[k]) || !std::isfinite(sp.caps[k]) ||
                !(sp.caps[k] > 0.0f))
                return to_set_error(ctx, TO_ERR_NONFINITE,
                                    "species %d patch %d: bad population or capacity", s, k);
        for (int q = 0; q < 8; ++q)
            if (!std::isfinite(sp.params[q]))
                return to_set_error(ctx, TO_ERR_NONFINITE, "species %d param %d", s, q);
    }
    if (maxN > 1020) return to_set_error(ctx, TO_ERR_UNSUPPORTED, "%d patches", maxN);
    const int NP = (maxN + 3) & ~3;
    std::vector<float> mmm((size_t)S * NP * NP, 0.0f), ip((size_t)S * NP, 0.0f),
        cp((size_t)S * NP, 1.0f), prm((size_t)S * 8);
    std::vector<int> np(S);
    for (int s = 0; s < S; ++s) {
        const to_mte_species& sp = prob->species[s];
        int N = sp.n_patches;
        np[s] = N;
        for (int k = 0; k < N; ++k) {
            ip[(size_t)s * NP + k] = sp.init_pops[k];
            cp[(size_t)s * NP + k] = sp.caps[k];
            for (int l = 0; l < N; ++l)
                mmm[((size_t)s * NP + k) * NP + l] = sp.mmm[(size_t)k * N + l];
        }
        for (int q = 0; q < 8; ++q) prm[(size_t)s * 8 + q] = sp.params[q];
    }
    const int cap = NP * 64 < NP * NP ? NP * 64 : NP * NP;
    size_t bytes = to_align256(mmm.size() * 4) + 2 * to_align256(ip.size() * 4) +
                   to_align256(prm.size() * 4) + to_align256((size_t)S * 4) +
                   to_align256((size_t)S * P * 4) + to_align256((size_t)S * 5 * 8) +
                   to_align256((size_t)S * (NP + 1) * 4) + to_align256((size_t)S * cap * 2) +
                   to_align256((size_t)S * cap * 4) + to_align256((size_t)S * 4);
    TO_TRY(to_arena_reserve(ctx, bytes));
    to_mte_args a;
    memset(&a, 0, sizeof(a));
    float* d_mmm = to_arena_take<float>(ctx, mmm.size());
    float* d_ip = to_arena_take<float>(ctx, ip.size());
    float* d_cp = to_arena_take<float>(ctx, cp.size());
    float* d_prm = to_arena_take<float>(ctx, prm.size());
    int* d_np = to_arena_take<int>(ctx, S);
    float* d_end = to_arena_take<float>(ctx, (size_t)S * P);
    double* d_stats = to_arena_take<double>(ctx, (size_t)S * 5);
    to_csc csc;
    csc.ptr = to_arena_take<int>(ctx, (size_t)S * (NP + 1));
    csc.idx = to_arena_take<uint16_t>(ctx, (size_t)S * cap);
    csc.val = to_arena_take<float>(ctx, (size_t)S * cap);
    csc.nnz = to_arena_take<int>(ctx, S);
    csc.cap = cap;
    csc.cap_smem = 0;
    TO_TRY(h2d(ctx, d_mmm, mmm.data(), mmm.size()));
    TO_TRY(h2d(ctx, d_ip, ip.data(), ip.size()));
    TO_TRY(h2d(ctx, d_cp, cp.data(), cp.size()));
    TO_TRY(h2d(ctx, d_prm, prm.data(), prm.size()));
    TO_TRY(h2d(ctx, d_np, np.data(), np.size()));
    a.n_paths = P; a.n_years = prob->n_years; a.S = S; a.C = 1; a.c_use = 0;
    a.dt = prob->dt; a.seed = prob->seed; a.sem = prob->sem; a.road0 = prob->road;
    a.npad = NP; a.npe = NP; a.n_patches = d_np; a.mmm = d_mmm; a.init_pops = d_ip;
    a.caps = d_cp; a.params = d_prm; a.end_pops = d_end;
    bool sparse = false;
    if (prob->migration == TO_MIG_AUTO || prob->migration == TO_MIG_SPARSE_FP32) {
        TO_TRY(to_k::pack_csc(ctx, d_mmm, NP, 1, d_np, S, csc));
        std::vector<int> nz(S);
        TO_CUDA(ctx, cudaMemcpyAsync(nz.data(), csc.nnz, S * sizeof(int), cudaMemcpyDeviceToHost,
                                     ctx->stream));
        TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        int mx = 0;
        bool ok = true;
        for (int v : nz) { if (v < 0) ok = false; mx = v > mx ? v : mx; }
        csc.cap_smem = (mx + 7) & ~7;
        sparse = ok && to_k::mte_sparse_smem(NP, csc.cap_smem) <= ctx->smem_optin;
        if (!sparse && prob->migration == TO_MIG_SPARSE_FP32)
            return to_set_error(ctx, TO_ERR_UNSUPPORTED, "matrices too dense for the sparse form");
    }
    if (sparse) {
        TO_TRY(to_k::mte_sparse(ctx, a, S, csc));
    } else if (prob->migration == TO_MIG_TC_3XTF32) {
        TO_TRY(to_k::mte_tc(ctx, a, S));
    } else {
        TO_TRY(to_k::mte_simt(ctx, a, S));
    }
    TO_TRY(to_k::mte_stats(ctx, a, S, d_stats));
    std::vector<float> ef((size_t)S * P);
    std::vector<double> st((size_t)S * 5);
    TO_TRY(d2h(ctx, ef.data(), d_end, ef.size()));
    TO_TRY(d2h(ctx, st.data(), d_stats, st.size()));
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    // a bounded wait that ran out (tensor-core kernel) or a plan check
    TO_TRY(to_check_device_flags(ctx));
    if (end_pops)
        for (size_t i = 0; i < ef.size(); ++i) end_pops[i] = (double)ef[i];
    if (stats)
        for (int s = 0; s < S; ++s) {
            stats[s].mean = st[5 * s];
            stats[s].sd = st[5 * s + 1];
            stats[s].se = st[5 * s + 2];
            stats[s].p_below = st[5 * s + 3];
            stats[s].init_total = st[5 * s + 4];
        }
    return TO_OK;
}

// ---- expPV -----------------------------------------------------------------
to_status to_exp_pv(to_ctx ctx, const to_exp_pv_params* prm, int n_paths,
                    int n_years, uint64_t seed, int road, int sem,
                    float* values, double* mean, double* sd) {
    if (!ctx || !prm || n_paths <= 0 || n_years < 0) return TO_ERR_INVALID;
    cudaSetDevice(ctx->device);
    float p[9] = {prm->gr, prm->mean, prm->time_step, prm->rrr, prm->current,
                  prm->reversion, prm->jump_prob, prm->noise_sd, prm->jump_sd};
    for (int i = 0; i < 9; ++i)
        if (!std::isfinite(p[i])) return to_set_error(ctx, TO_ERR_NONFINITE, "expPV parameter %d", i);
    TO_TRY(to_arena_reserve(ctx, 256 + to_align256((size_t)n_paths * 4) + 256));
    float* d_p = to_arena_take<float>(ctx, 9);
    float* d_v = to_arena_take<float>(ctx, n_paths);
    double* d_s = to_arena_take<double>(ctx, 2);
    TO_TRY(h2d(ctx, d_p, p, 9));
    TO_TRY(to_k::exp_pv(ctx, d_p, n_paths, n_years, seed, road, sem, d_v, d_s));
    double st[2];
    if (values) TO_TRY(d2h(ctx, values, d_v, n_paths));
    TO_TRY(d2h(ctx, st, d_s, 2));
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (mean) *mean = st[0];
    if (sd) *sd = st[1];
    return TO_OK;
}

}  // extern "C"
