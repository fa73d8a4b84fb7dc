// exppv.cu - expected present value of one unit of usage under a
// mean-reverting price with jumps.
//
// Reference: expPVPath (include/gpuCode/SimulateGPU.cu:256-279) and
// SimulateGPU::expPV (SimulateGPU.cu:3163-3259), called per fuel and
// commodity by Uncertainty::computeExpPV (include/valuation/Uncertainty.cpp:37-75).
// Streams are Philox, addressed by a flat (path, year) index so that the
// reference's overlapping windows (path idx reads idx+year) and the corrected
// idx*Y+year layout read the same stream.
#include "to_internal.cuh"
#include "to_pop.cuh"

namespace {

__device__ __forceinline__ float pv_stream(uint64_t seed, int stream, int road,
                                           long flat, bool normal) {
    uint32_t path = (uint32_t)(flat >> 2), lane = (uint32_t)(flat & 3);
    return normal ? to_normal1(seed, stream, road, path, 0, lane)
                  : to_uniform1(seed, stream, road, path, 0, lane);
}

// prm: gr, meanP, timeStep, rrr, current, reversion, jumpProb, noiseSD, jumpSD
__global__ void k_exp_pv(const float* __restrict__ prm, int P, int Y,
                         uint64_t seed, int road, int sem,
                         float* __restrict__ values) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    float gr = prm[0], meanP = prm[1], ts = prm[2], rrr = prm[3];
    float curr = prm[4], rev = prm[5], jp = prm[6], nsd = prm[7], pj = prm[8];
    float pj2 = pj * pj;
    float value = 0.0f, g = 1.0f, r = 1.0f;
    for (int t = 0; t < Y; ++t) {
        long flat = (sem == 0) ? (long)p + t : (long)p * Y + t;
        float zb = pv_stream(seed, TO_STREAM_PV_BROWNIAN, road, flat, true);
        float zj = pv_stream(seed, TO_STREAM_PV_JUMPSIZE, road, flat, true);
        float uj = pv_stream(seed, TO_STREAM_PV_JUMP, road, flat, false);
        float brown = zb * nsd;
        float jsz = zj * pj2 + (-pj2 / 2.0f);
        float jumped = (uj < jp) ? 1.0f : 0.0f;
        curr = curr + (rev * (meanP - curr) * ts + curr * brown
                       + (to_expf(jsz) - 1.0f) * curr * jumped);
        value = value + g * curr / r;
        g = g * (1.0f + gr);
        r = r * (1.0f + rrr);
    }
    values[p] = value;
}

// mean and the reference's "SD" (sem 0: sqrt of the sum of squared
// deviations; sem 1: sample SD), FP64
__global__ void k_exp_pv_stats(int P, int sem, const float* __restrict__ v,
                               double* __restrict__ out) {
    __shared__ double s[32];
    double sum = 0.0;
    for (int p = threadIdx.x; p < P; p += blockDim.x) sum += (double)v[p];
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if ((threadIdx.x & 31) == 0) s[w] = sum;
    __syncthreads();
    double tot = 0.0;
    for (int i = 0; i < nw; ++i) tot += s[i];
    double mean = tot / (double)P;
    __syncthreads();
    double sq = 0.0;
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        double d = (double)v[p] - mean;
        sq += d * d;
    }
    for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
    if ((threadIdx.x & 31) == 0) s[w] = sq;
    __syncthreads();
    if (threadIdx.x == 0) {
        double q = 0.0;
        for (int i = 0; i < nw; ++i) q += s[i];
        out[0] = mean;
        out[1] = (sem == 0) ? sqrt(q) : sqrt(q / (double)(P > 1 ? P - 1 : 1));
    }
}

}  // namespace

namespace to_k {
to_status exp_pv(to_ctx ctx, const float* d_prm, int P, int Y, uint64_t seed,
                 int road, int sem, float* d_values, double* d_stats) {
    int threads = 128;
    k_exp_pv<<<(P + threads - 1) / threads, threads, 0, ctx->stream>>>(
        d_prm, P, Y, seed, road, sem, d_values);
    TO_LAUNCHED(ctx);
    k_exp_pv_stats<<<1, 1024, 0, ctx->stream>>>(P, sem, d_values, d_stats);
    TO_LAUNCHED(ctx);
    return TO_OK;
}
}  // namespace to_k
