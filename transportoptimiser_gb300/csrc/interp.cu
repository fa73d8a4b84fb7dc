// interp.cu - evaluation of the local-linear grid surrogates at many points.
//
// Surrogate layout (buildSurrogate*CUDA): [R*d axis values | R^d values],
// axis j at [j*R, (j+1)*R), value index R*d + sum_j i_j R^(d-1-j) (dimension
// 0 most significant).  Three arithmetics, one thread per point:
//   mode 0  SimulateGPU::interpolateSurrogateMulti's kernel interpolateMulti
//           (SimulateGPU.cu:3077-3155) in float, as it computes: for
//           dimensions > 0 it reads the predictors of point 0 (quirk Q26)
//           and folds the corner coefficients with a stride of
//           (int)pow(2, d - j - 2) (zero in the last dimension, quirk Q27).
//           For d = 1, the case the reference calls (RoadGA.cpp:1257), it
//           is plain linear interpolation.
//   mode 1  multilinear interpolation in double (the corrected form).
//   mode 2  Utility::interpolateSurrogate (Utility.cpp:253-363), the
//           per-road host evaluation, in double, as it computes (for d > 1
//           it pairs dimension 0's weight with the last dimension's
//           neighbours, quirk Q28).
#include <cmath>

#include "to_internal.cuh"

namespace {

constexpr int kMaxDims = 6;

__device__ float interp_ref_kernel(int idx, int d, int R, const float* S, const float* P) {
    int lowerInd[kMaxDims];
    float coeffs[1 << (kMaxDims - 1)];
    for (int jj = 0; jj < d; ++jj) {
        const float lower = S[jj * R], upper = S[(jj + 1) * R - 1];
        int li = (int)(((float)(R - 1) * (P[d * idx + jj] - lower)) / (upper - lower));
        if (li >= R - 1) li = R - 2;
        else if (li < 0) li = 0;
        lowerInd[jj] = li;
    }
    float x0 = S[lowerInd[0]], x1 = S[lowerInd[0] + 1];
    float xd = (P[d * idx] - x0) / (x1 - x0);
    const int nco = 1 << (d - 1);
    int rpow[kMaxDims + 1];
    rpow[0] = 1;
    for (int q = 1; q <= d; ++q) rpow[q] = rpow[q - 1] * R;
    for (int jj = 0; jj < nco; ++jj) {
        int idxL = R * d;
        for (int kk = 1; kk < d; ++kk) {
            const int q = jj / (1 << (d - kk - 1));
            const int rem = (q + 1) - 2 * ((q + 1) / 2);
            idxL += (rem > 0 ? lowerInd[kk] : lowerInd[kk] + 1) * rpow[d - kk - 1];
        }
        const int idxU = idxL + (lowerInd[0] + 1) * rpow[d - 1];
        idxL += lowerInd[0] * rpow[d - 1];
        coeffs[jj] = S[idxL] * (1 - xd) + S[idxU] * xd;
    }
    for (int jj = 1; jj < d; ++jj) {
        x0 = S[jj * R + lowerInd[jj]];
        x1 = S[jj * R + lowerInd[jj] + 1];
        xd = (P[jj] - x0) / (x1 - x0);
        const int jump = (d - jj - 2 >= 0) ? (1 << (d - jj - 2)) : 0;
        for (int kk = 0; kk < (1 << jj); ++kk)
            coeffs[kk] = coeffs[kk] * (1 - xd) + coeffs[kk + jump] * xd;
    }
    return coeffs[0];
}

__device__ double interp_multilinear(const double* S, const double* p, int d, int R) {
    int lo[kMaxDims];
    double w[kMaxDims];
    for (int j = 0; j < d; ++j) {
        const double* ax = S + (size_t)j * R;
        const double a0 = ax[0], a1 = ax[R - 1];
        (void)a0; (void)a1;
        int i = 0, hi = R - 2;                 /* last i with ax[i] <= p (clamped) */
        while (i < hi) {
            const int mid = (i + hi + 1) >> 1;
            if (ax[mid] <= p[j]) i = mid; else hi = mid - 1;
        }
        const double x0 = ax[i], x1 = ax[i + 1];
        double t = (x1 != x0) ? (p[j] - x0) / (x1 - x0) : 0.0;
        lo[j] = i;
        w[j] = t;
    }
    double acc = 0.0;
    for (int corner = 0; corner < (1 << d); ++corner) {
        double wt = 1.0;
        size_t off = (size_t)R * d, stride = 1;
        for (int j = d - 1; j >= 0; --j) {
            const int b = (corner >> j) & 1;
            wt *= b ? w[j] : 1.0 - w[j];
            off += (size_t)(lo[j] + b) * stride;
            stride *= R;
        }
        acc += wt * S[off];
    }
    return acc;
}

__device__ double interp_utility(const double* S, const double* p, int d, int R) {
    int lowerIdx[kMaxDims];
    double coeffs[1 << (kMaxDims - 1)];
    const double eps = 2.220446049250313e-16;
    for (int ii = 0; ii < d; ++ii) {
        const double lv = S[ii * R], uv = S[(ii + 1) * R - 1];
        int li = (int)((R - 1) * (p[ii] - lv) / (uv - lv));
        if (li < 0) li = 0;
        else if (li >= R - 1) li = R - 2;
        lowerIdx[ii] = li;
    }
    double x0 = S[lowerIdx[0]], x1 = S[lowerIdx[0] + 1];
    double xd = (fabs(x1 - x0) < eps || x0 == x1) ? 0.0 : (p[0] - x0) / (x1 - x0);
    int rpow[kMaxDims + 1];
    rpow[0] = 1;
    for (int q = 1; q <= d; ++q) rpow[q] = rpow[q - 1] * R;
    for (int ii = 0; ii < (1 << (d - 1)); ++ii) {
        int idxL = d * R, div = ii;
        for (int jj = 0; jj < d - 1; ++jj) {
            const int rem = div - 2 * (div / 2);
            div = div / 2;
            idxL += (rem == 0 ? lowerIdx[d - 2 - jj] : lowerIdx[d - 2 - jj] + 1) * rpow[jj + 1];
        }
        idxL += lowerIdx[d - 1];
        coeffs[ii] = S[idxL] * (1 - xd) + S[idxL + 1] * xd;
    }
    for (int ii = 1; ii < d; ++ii) {
        x0 = S[lowerIdx[ii] + R * ii];
        x1 = S[lowerIdx[ii] + 1 + R * ii];
        xd = (fabs(x1 - x0) < eps || x0 == x1) ? 0.0 : (p[d - ii] - x0) / (x1 - x0);
        for (int jj = 0; jj < (1 << (d - 1 - ii)); ++jj)
            coeffs[jj] = coeffs[jj * 2] * (1 - xd) + coeffs[jj * 2 + 1] * xd;
    }
    return coeffs[0];
}

__global__ void k_interp(int n, int d, int R, int mode, const double* __restrict__ Sd,
                         const double* __restrict__ Pd, const float* __restrict__ Sf,
                         const float* __restrict__ Pf, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (mode == 0) out[i] = (double)interp_ref_kernel(i, d, R, Sf, Pf);
    else if (mode == 1) out[i] = interp_multilinear(Sd, Pd + (size_t)i * d, d, R);
    else out[i] = interp_utility(Sd, Pd + (size_t)i * d, d, R);
}

__global__ void k_to_float(size_t n, const double* __restrict__ a, float* __restrict__ b) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

}  // namespace

extern "C" to_status to_interpolate_surrogate(to_ctx ctx, int n_points, int n_dims, int dim_res,
                                              const double* surrogate, const double* predictors,
                                              double* results, int mode) {
    if (!ctx || n_points < 0 || n_dims < 1 || n_dims > kMaxDims || dim_res < 2 || !surrogate ||
        (n_points > 0 && (!predictors || !results)) || mode < 0 || mode > 2)
        return TO_ERR_INVALID;
    if (n_points == 0) return TO_OK;
    double rq = std::pow((double)dim_res, n_dims);
    if (rq > 1e8) return to_set_error(ctx, TO_ERR_UNSUPPORTED, "surrogate of %g values", rq);
    const size_t ns = (size_t)dim_res * n_dims + (size_t)rq;
    const size_t np = (size_t)n_points * n_dims;
    for (size_t i = 0; i < ns; ++i)
        if (!std::isfinite(surrogate[i])) return to_set_error(ctx, TO_ERR_NONFINITE, "surrogate %zu", i);
    for (size_t i = 0; i < np; ++i)
        if (!std::isfinite(predictors[i])) return to_set_error(ctx, TO_ERR_NONFINITE, "predictor %zu", i);
    cudaSetDevice(ctx->device);
    const size_t bytes = to_align256(ns * 8) + to_align256(np * 8) + to_align256(ns * 4) +
                         to_align256(np * 4) + to_align256((size_t)n_points * 8);
    TO_TRY(to_arena_reserve(ctx, bytes + 1024));
    double* dS = to_arena_take<double>(ctx, ns);
    double* dP = to_arena_take<double>(ctx, np);
    float* fS = to_arena_take<float>(ctx, ns);
    float* fP = to_arena_take<float>(ctx, np);
    double* dR = to_arena_take<double>(ctx, n_points);
    TO_CUDA(ctx, cudaMemcpyAsync(dS, surrogate, ns * 8, cudaMemcpyHostToDevice, ctx->stream));
    TO_CUDA(ctx, cudaMemcpyAsync(dP, predictors, np * 8, cudaMemcpyHostToDevice, ctx->stream));
    if (mode == 0) {
        // the reference casts its Eigen vectors to float before the kernel
        k_to_float<<<64, 256, 0, ctx->stream>>>(ns, dS, fS);
        k_to_float<<<64, 256, 0, ctx->stream>>>(np, dP, fP);
        ctx->launches += 2;
    }
    k_interp<<<(n_points + 255) / 256, 256, 0, ctx->stream>>>(n_points, n_dims, dim_res, mode, dS,
                                                              dP, fS, fP, dR);
    TO_LAUNCHED(ctx);
    TO_CUDA(ctx, cudaMemcpyAsync(results, dR, (size_t)n_points * 8, cudaMemcpyDeviceToHost,
                                 ctx->stream));
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return TO_OK;
}
