// surrogate.cu - local-linear surrogate builders used by the GA fitness.
//
// Reference: SimulateGPU::buildSurrogateMTECUDA (include/gpuCode/
// SimulateGPU.cu:5533-5692: 1-D surrogate of the end population against the
// initial animals-at-risk) and SimulateGPU::buildSurrogateROVCUDA
// (SimulateGPU.cu:5694-5917: d-D surrogate of the ROV value against the
// IARs and unit use), both built from a k-nearest-neighbour local linear
// regression on a dim_res^d grid (createQueryPoints, knn, multiLocLinReg,
// rovCorrection).  The reference copies the samples and the grid between
// host and device around each step; here one preparation kernel (min / max,
// normalisation, grid) feeds the warp-per-query kNN and a thread-per-grid-
// point regression, all on the device.
#include <cmath>
#include <cstring>
#include <vector>

#include "to_internal.cuh"
#include "to_lsm_math.h"
#include "to_rov.cuh"

namespace {

struct SurrArgs {
    int n, d, R, Q, k, normalize, sem, clip;
    const float* raw;     // [d][n]
    const float* y;       // [n]
    float* pn;            // [d][n] points the kNN sees
    float* qn;            // [d][Q] queries the kNN sees
    float* xq;            // [d][Q] regression centres
    float* dist;          // [k][Q]
    int* ind;             // [k][Q]
    float* out;           // [R*d + Q]
};

__global__ void __launch_bounds__(1024) k_surr_prepare(SurrArgs a) {
    __shared__ float s_lo[TO_LSM_MAXD], s_hi[TO_LSM_MAXD];
    __shared__ float w_lo[32], w_hi[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = 0; j < a.d; ++j) {
        float lo = INFINITY, hi = -INFINITY;
        for (int m = threadIdx.x; m < a.n; m += blockDim.x) {
            float v = a.raw[(size_t)j * a.n + m];
            lo = fminf(lo, v);
            hi = fmaxf(hi, v);
        }
        for (int o = 16; o > 0; o >>= 1) {
            lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        }
        if (lane == 0) { w_lo[warp] = lo; w_hi[warp] = hi; }
        __syncthreads();
        if (threadIdx.x == 0) {
            float l = w_lo[0], h = w_hi[0];
            for (int w = 1; w < nw; ++w) { l = fminf(l, w_lo[w]); h = fmaxf(h, w_hi[w]); }
            s_lo[j] = l;
            s_hi[j] = h;
        }
        __syncthreads();
    }
    for (int q = threadIdx.x; q < a.n * a.d; q += blockDim.x) {
        int j = q / a.n;
        float v = a.raw[q];
        a.pn[q] = a.normalize ? to_lsm_normalise(v, s_lo[j], s_hi[j], 0, 1.0f) : v;
    }
    for (int q = threadIdx.x; q < a.Q; q += blockDim.x) {
        int rem = q;
        int div = a.Q / a.R;
        for (int j = 0; j < a.d; ++j) {
            int di = rem / div;
            rem -= di * div;
            div /= a.R;
            float raw = to_lsm_query_axis(di, s_lo[j], s_hi[j], a.R);
            a.out[(size_t)j * a.R + di] = raw;
            float nv = a.normalize ? to_lsm_normalise(raw, s_lo[j], s_hi[j], 0, 1.0f) : raw;
            a.qn[(size_t)j * a.Q + q] = nv;
            a.xq[(size_t)j * a.Q + q] = a.normalize ? (a.sem == 0 ? to_lsm_unit_axis(di, a.R) : nv)
                                                    : raw;
        }
    }
}

__global__ void k_surr_regress(SurrArgs a) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= a.Q) return;
    float* yout = a.out + (size_t)a.R * a.d;
    if (a.n < 3 || a.k <= 0) { yout[q] = 0.0f; return; }
    float xq[TO_LSM_MAXD];
    for (int j = 0; j < a.d; ++j) xq[j] = a.xq[(size_t)j * a.Q + q];
    float acc[TO_LSM_ACC];
    to_lsm_acc_init(a.d, acc);
    const float h = a.dist[(size_t)(a.k - 1) * a.Q + q];
    for (int kk = 0; kk < a.k; ++kk) {
        float dd = a.dist[(size_t)kk * a.Q + q];
        int i = a.ind[(size_t)kk * a.Q + q] - 1;
        float xv[TO_LSM_MAXD];
        for (int j = 0; j < a.d; ++j)
            xv[j] = (a.sem == 0 || !a.normalize) ? a.raw[(size_t)i * a.d + j]
                                                 : a.pn[(size_t)j * a.n + i];
        to_lsm_acc_add(a.d, acc, to_lsm_weight(dd, h), a.y[i], xv, xq);
    }
    float v = to_lsm_solve_intercept(a.d, acc);
    if (a.clip && v > 0.0f) v = 0.0f;        // rovCorrection (SimulateGPU.cu:3055-3073)
    yout[q] = v;
}

// k rules of the two builders (SimulateGPU.cu:5545-5554, 5711-5722), never
// more than the number of samples
int k_mte(int n) {
    int k;
    if (n < 50) k = 5;
    else if (n < 100) k = 7;
    else if (n < 500) k = (int)std::ceil(0.02 * (n - 100) + 7);
    else k = (int)std::ceil(std::log((double)n) + 8);
    return k < n ? k : n;
}
int k_rov(int n) {
    int k;
    if (n < 50) k = 5;
    else if (n < 100) k = (int)(5 + 5 * std::ceil((double)((n - 50) / 50)));
    else if (n < 500) k = (int)std::ceil(10 + 15 * std::ceil((double)((n - 100) / 400)));
    else k = (int)(25 + std::ceil((n - 500) * 0.02));
    return k < n ? k : n;
}

to_status build(to_ctx ctx, int n, int d, const double* pred, const double* const* ys,
                int n_y, const int* clips, int R, int k, int normalize, int sem,
                double* const* outs) {
    long Ql = 1;
    for (int j = 0; j < d; ++j) Ql *= R;
    if (Ql > (1 << 22) || d > TO_LSM_MAXD)
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "grid %d^%d", R, d);
    const int Q = (int)Ql;
    const int kk = k > 0 ? k : 1;
    std::vector<float> raw((size_t)d * n), yf((size_t)n);
    for (size_t i = 0; i < raw.size(); ++i) {
        if (!std::isfinite(pred[i])) return to_set_error(ctx, TO_ERR_NONFINITE, "predictor %zu", i);
        raw[i] = (float)pred[i];
    }
    size_t bytes = 4 * to_align256((size_t)d * n * 4) + to_align256((size_t)n * 4) +
                   2 * to_align256((size_t)d * Q * 4) + 2 * to_align256((size_t)kk * Q * 4) +
                   to_align256(((size_t)R * d + Q) * 4);
    TO_TRY(to_arena_reserve(ctx, bytes + 4096));
    SurrArgs a;
    memset(&a, 0, sizeof(a));
    a.n = n; a.d = d; a.R = R; a.Q = Q; a.k = k; a.normalize = normalize; a.sem = sem;
    float* d_raw = to_arena_take<float>(ctx, (size_t)d * n);
    float* d_y = to_arena_take<float>(ctx, n);
    a.raw = d_raw; a.y = d_y;
    a.pn = to_arena_take<float>(ctx, (size_t)d * n);
    a.qn = to_arena_take<float>(ctx, (size_t)d * Q);
    a.xq = to_arena_take<float>(ctx, (size_t)d * Q);
    a.dist = to_arena_take<float>(ctx, (size_t)kk * Q);
    a.ind = to_arena_take<int>(ctx, (size_t)kk * Q);
    a.out = to_arena_take<float>(ctx, (size_t)R * d + Q);
    TO_CUDA(ctx, cudaMemcpyAsync(d_raw, raw.data(), raw.size() * 4, cudaMemcpyHostToDevice,
                                 ctx->stream));
    k_surr_prepare<<<1, 1024, 0, ctx->stream>>>(a);
    TO_LAUNCHED(ctx);
    if (n >= 3 && k > 0) TO_TRY(to_k::knn(ctx, a.pn, n, a.qn, Q, d, k, a.dist, a.ind));
    std::vector<float> of((size_t)R * d + Q);
    for (int v = 0; v < n_y; ++v) {
        for (int i = 0; i < n; ++i) {
            if (!std::isfinite(ys[v][i])) return to_set_error(ctx, TO_ERR_NONFINITE, "value %d", i);
            yf[i] = (float)ys[v][i];
        }
        TO_CUDA(ctx, cudaMemcpyAsync(d_y, yf.data(), (size_t)n * 4, cudaMemcpyHostToDevice,
                                     ctx->stream));
        a.clip = clips[v];
        to_prof_begin(ctx, "surrogate_regress");
        k_surr_regress<<<(Q + 127) / 128, 128, 0, ctx->stream>>>(a);
        to_prof_end(ctx);
        TO_LAUNCHED(ctx);
        TO_CUDA(ctx, cudaMemcpyAsync(of.data(), a.out, of.size() * 4, cudaMemcpyDeviceToHost,
                                     ctx->stream));
        TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (outs[v])
            for (size_t i = 0; i < of.size(); ++i) outs[v][i] = (double)of[i];
    }
    return TO_OK;
}

}  // namespace

extern "C" {

to_status to_build_surrogate_mte(to_ctx ctx, int samples, const double* iars,
                                 const double* pops_mean, const double* pops_sd, int dim_res,
                                 double* out_mean, double* out_sd) {
    if (!ctx || samples <= 0 || !iars || !pops_mean || dim_res < 2) return TO_ERR_INVALID;
    cudaSetDevice(ctx->device);
    const double* ys[2] = {pops_mean, pops_sd};
    double* outs[2] = {out_mean, out_sd};
    int clips[2] = {0, 0};
    return build(ctx, samples, 1, iars, ys, pops_sd ? 2 : 1, clips, dim_res, k_mte(samples),
                 0, 0, outs);
}

to_status to_build_surrogate_rov(to_ctx ctx, int samples, int n_dims, const double* predictors,
                                 const double* values, const double* values_sd, int dim_res,
                                 int sem, double* out_mean, double* out_sd) {
    if (!ctx || samples <= 0 || n_dims <= 0 || !predictors || !values || dim_res < 2)
        return TO_ERR_INVALID;
    cudaSetDevice(ctx->device);
    const double* ys[2] = {values, values_sd};
    double* outs[2] = {out_mean, out_sd};
    int clips[2] = {1, 0};
    return build(ctx, samples, n_dims, predictors, ys, values_sd ? 2 : 1, clips, dim_res,
                 k_rov(samples), 1, sem, outs);
}

}  // extern "C"
