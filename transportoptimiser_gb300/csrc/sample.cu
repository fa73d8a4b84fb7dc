// sample.cu - space-filling selection of GA designs to simulate
// (RoadGA::generateSample, include/main/RoadGA.cpp:3288-3462, with the
// distance kernels knn_cuda_with_indexes::computeDistances,
// knn_cuda_with_indexes.cu:188-325, 620-738).
//
// The reference normalises current samples and candidates together per
// dimension, then adds samples one at a time: for every candidate it
// recomputes the distance matrices to all current samples on the GPU (the
// "projected" distance: the smallest coordinate difference, initialised at
// 100; and the Euclidean distance), copies them to the host and scans them.
// Rule per step (n = current sample count, d = dimensions):
//   d_min = 1 / n; best = max of the Euclidean minimum among candidates
//   whose projected minimum >= d_min (first index);
//   val_j = ((pow(n + 1, 1 / d) - 1) / 2) * minD2_j + ((n + 1) / 2) * minDI_j
//   (integer 1 / d and (n + 1) / 2, quirk Q30); a candidate whose val
//   exceeds the running best replaces the choice (the scan runs whether or
//   not the first one succeeded, quirk Q31).
// With no current samples the first two are the pair with the largest
// projected distance (first in row order).
// Here one CTA keeps every candidate's running minima (updated with the one
// new sample per step, not recomputed) and picks each sample with two
// block arg-max reductions; nothing leaves the device until the end.
// Euclidean distances use t*t and sqrtf where the reference calls pow.
#include <cmath>
#include <vector>

#include "to_internal.cuh"

namespace {

constexpr int kThreads = 1024;

struct Best {
    float v;
    int i;
};

__device__ __forceinline__ Best better(Best a, Best b) {
    // larger value; equal values: smaller index (the first in a scan)
    if (b.v > a.v || (b.v == a.v && b.i < a.i && b.i >= 0)) return b;
    return a;
}

__device__ Best block_best(Best x, Best* s) {
    for (int o = 16; o > 0; o >>= 1) {
        Best y;
        y.v = __shfl_xor_sync(0xffffffffu, x.v, o);
        y.i = __shfl_xor_sync(0xffffffffu, x.i, o);
        x = better(x.i < 0 ? y : x, y.i < 0 ? x : y);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) s[warp] = x;
    __syncthreads();
    if (warp == 0) {
        x = (lane < (int)(blockDim.x >> 5)) ? s[lane] : Best{-INFINITY, -1};
        for (int o = 16; o > 0; o >>= 1) {
            Best y;
            y.v = __shfl_xor_sync(0xffffffffu, x.v, o);
            y.i = __shfl_xor_sync(0xffffffffu, x.i, o);
            x = better(x.i < 0 ? y : x, y.i < 0 ? x : y);
        }
        if (lane == 0) s[0] = x;
    }
    __syncthreads();
    return s[0];
}

__device__ __forceinline__ void dists(const float* c, int nc, int j, const float* s, int ns, int i,
                                      int d, float& dproj, float& d2) {
    float mn = 100.0f, ss = 0.0f;
    for (int k = 0; k < d; ++k) {
        const float t = fabsf(s[(size_t)k * ns + i] - c[(size_t)k * nc + j]);
        mn = fminf(mn, t);
        ss = ss + t * t;
    }
    dproj = mn;
    d2 = sqrtf(ss);
}

// c: candidates dim-major [d][nc]; cur: samples dim-major [d][cap] with n0
// filled; out: chosen candidate indices [n]
__global__ void __launch_bounds__(kThreads)
k_select(int nc, int d, int n0, int n, int cap, const float* __restrict__ c, float* __restrict__ cur,
         float* __restrict__ minDI, float* __restrict__ minD2, int* __restrict__ out) {
    __shared__ Best s_b[32];
    __shared__ int s_pick;
    int ns = n0, first_out = 0;
    if (n0 == 0) {
        // the pair with the largest projected distance (row order)
        Best b{-INFINITY, -1};
        for (long q = threadIdx.x; q < (long)nc * nc; q += blockDim.x) {
            const int ii = (int)(q / nc), jj = (int)(q - (long)ii * nc);
            float dp, d2;
            dists(c, nc, ii, c, nc, jj, d, dp, d2);
            if (dp > 0.0f) b = better(b, Best{dp, (int)q});
        }
        b = block_best(b, s_b);
        const int q = b.i >= 0 ? b.i : 0;
        if (threadIdx.x == 0) { out[0] = q / nc; out[1] = q % nc; }
        __syncthreads();
        for (int k = threadIdx.x; k < d; k += blockDim.x) {
            cur[(size_t)k * cap + 0] = c[(size_t)k * nc + out[0]];
            cur[(size_t)k * cap + 1] = c[(size_t)k * nc + out[1]];
        }
        ns = 2;
        first_out = 2;
        __syncthreads();
    }
    // running minima over the current samples
    for (int j = threadIdx.x; j < nc; j += blockDim.x) {
        float mi = INFINITY, m2 = INFINITY;
        for (int i = 0; i < ns; ++i) {
            float dp, d2;
            dists(c, nc, j, cur, cap, i, d, dp, d2);
            mi = fminf(mi, dp);
            m2 = fminf(m2, d2);
        }
        minDI[j] = mi;
        minD2[j] = m2;
    }
    __syncthreads();
    for (int step = first_out; step < n; ++step) {
        const float dmin = 2.0f * 0.5f / (float)ns;
        const double cd = (d == 1) ? ((double)(ns + 1) - 1.0) / 2.0 : 0.0;   // pow(n+1, 1/d)
        const int ch = (ns + 1) / 2;
        Best b1{-INFINITY, -1}, b2{-INFINITY, -1};
        for (int j = threadIdx.x; j < nc; j += blockDim.x) {
            const float mi = minDI[j], m2 = minD2[j];
            if (mi >= dmin && m2 > 0.0f) b1 = better(b1, Best{m2, j});
            const float val = (float)(cd * (double)m2 + (double)((float)ch * mi));
            b2 = better(b2, Best{val, j});
        }
        b1 = block_best(b1, s_b);
        const float best1 = b1.i >= 0 ? b1.v : 0.0f;
        b2 = block_best(b2, s_b);
        if (threadIdx.x == 0) {
            int pick = b1.i >= 0 ? b1.i : -1;
            if (b2.i >= 0 && b2.v > best1) pick = b2.i;
            if (pick < 0) pick = 0;
            s_pick = pick;
            out[step] = pick;
        }
        __syncthreads();
        const int pk = s_pick;
        for (int k = threadIdx.x; k < d; k += blockDim.x)
            cur[(size_t)k * cap + ns] = c[(size_t)k * nc + pk];
        __syncthreads();
        for (int j = threadIdx.x; j < nc; j += blockDim.x) {
            float dp, d2;
            dists(c, nc, j, cur, cap, ns, d, dp, d2);
            minDI[j] = fminf(minDI[j], dp);
            minD2[j] = fminf(minD2[j], d2);
        }
        ++ns;
        __syncthreads();
    }
}

}  // namespace

extern "C" to_status to_select_samples(to_ctx ctx, int n_current, const double* current,
                                       int n_candidates, const double* candidates, int n_dims,
                                       int n, int* sample) {
    if (!ctx || n_current < 0 || n_candidates <= 0 || n_dims <= 0 || n <= 0 || !candidates ||
        !sample || (n_current > 0 && !current) || (n_current == 0 && (n < 2 || n_candidates < 2)))
        return TO_ERR_INVALID;
    const size_t nc = (size_t)n_candidates, d = (size_t)n_dims;
    for (size_t q = 0; q < nc * d; ++q)
        if (!std::isfinite(candidates[q])) return to_set_error(ctx, TO_ERR_NONFINITE, "candidate %zu", q / d);
    for (size_t q = 0; q < (size_t)n_current * d; ++q)
        if (!std::isfinite(current[q])) return to_set_error(ctx, TO_ERR_NONFINITE, "sample %zu", q / d);
    // joint normalisation per dimension (double), then float, dim-major
    std::vector<float> cf(nc * d);
    const int cap = n_current + n + 2;
    std::vector<float> sf((size_t)cap * d, 0.0f);
    for (size_t k = 0; k < d; ++k) {
        double lo = INFINITY, hi = -INFINITY;
        for (int i = 0; i < n_current; ++i) { lo = fmin(lo, current[i * d + k]); hi = fmax(hi, current[i * d + k]); }
        for (size_t j = 0; j < nc; ++j) { lo = fmin(lo, candidates[j * d + k]); hi = fmax(hi, candidates[j * d + k]); }
        for (size_t j = 0; j < nc; ++j) cf[k * nc + j] = (float)((candidates[j * d + k] - lo) / (hi - lo));
        for (int i = 0; i < n_current; ++i)
            sf[k * cap + i] = (float)((current[i * d + k] - lo) / (hi - lo));
    }
    cudaSetDevice(ctx->device);
    const size_t bytes = to_align256(cf.size() * 4) + to_align256(sf.size() * 4) +
                         2 * to_align256(nc * 4) + to_align256((size_t)n * 4);
    TO_TRY(to_arena_reserve(ctx, bytes + 1024));
    float* dC = to_arena_take<float>(ctx, cf.size());
    float* dS = to_arena_take<float>(ctx, sf.size());
    float* dMI = to_arena_take<float>(ctx, nc);
    float* dM2 = to_arena_take<float>(ctx, nc);
    int* dO = to_arena_take<int>(ctx, n);
    TO_CUDA(ctx, cudaMemcpyAsync(dC, cf.data(), cf.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    TO_CUDA(ctx, cudaMemcpyAsync(dS, sf.data(), sf.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    to_prof_begin(ctx, "select_samples");
    k_select<<<1, kThreads, 0, ctx->stream>>>(n_candidates, n_dims, n_current, n, cap, dC, dS,
                                               dMI, dM2, dO);
    to_prof_end(ctx);
    TO_LAUNCHED(ctx);
    TO_CUDA(ctx, cudaMemcpyAsync(sample, dO, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return TO_OK;
}
