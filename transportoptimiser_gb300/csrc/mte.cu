// mte.cu - fixed-traffic (MTE) animal-population Monte Carlo.
//
// Reference: mteKernel (include/gpuCode/SimulateGPU.cu:595-717) driven by
// SimulateGPU::simulateMTECUDA (SimulateGPU.cu:3650-3864); end-population
// mean / SD as Simulator::simulateMTE (include/main/Simulator.cpp:178-191).
//
// The reference runs one thread per path over a CSC matrix with path-major
// strided population buffers and a pre-generated P*Y*N normal array.  Here a
// CTA owns a tile of paths for all years: populations stay in shared memory,
// the migration step is a (paths x N)(N x N) product (SIMT FP32 here, FMA in
// ascending origin order so the oracle can mirror it exactly; the tcgen05
// 3xTF32 form is in tc_migrate.cu), and the growth normals come from Philox
// in registers, four patches per call, so no random array touches HBM.
#include "to_internal.cuh"
#include "to_pop.cuh"

namespace {

// Thread (pg, kg) owns paths tile*TP + 4pg..4pg+3 and patches 4kg..4kg+3.
__global__ void __launch_bounds__(1024)
k_mte_simt(to_mte_args a) {
    extern __shared__ float smem[];
    const int NP = a.npad, NE = a.npe, KG = NE >> 2;
    const int TP = a.tile_paths;
    const int rs = a.rs0 + blockIdx.y;
    const int road = rs / a.S, sp = rs - road * a.S;
    const int tid = threadIdx.x;
    const int pg = tid / KG, kg = tid - pg * KG;
    const bool active = pg < (TP >> 2);
    const int LC = a.l_chunk;
    float* Mt = smem;                       // [LC][NE]
    float* pop = Mt + (size_t)LC * NE;      // [TP][NE]
    float* mig = pop + (size_t)TP * NE;     // [TP][NE]
    float* gm = mig + (size_t)TP * NE;      // [TP]

    const int N = a.n_patches[rs];
    if (N > NE) {
        if (tid == 0 && a.flags) atomicExch(a.flags, TO_DEVERR_PLAN);
        for (int q = tid; q < TP; q += blockDim.x)
            if (blockIdx.x * TP + q < a.n_paths) a.end_pops[(size_t)rs * a.n_paths + blockIdx.x * TP + q] = NAN;
        return;
    }
    const float* M = a.mmm + ((size_t)rs * a.C + a.c_use) * NP * NP;
    const float* ip = a.init_pops + (size_t)rs * NP;
    const float* cp = a.caps + (size_t)rs * NP;
    const float* sp8 = a.params + 8 * sp;
    const float p0 = sp8[0], p1 = sp8[1], p2 = sp8[2], p4 = sp8[4], p5 = sp8[5],
                p6 = sp8[6], p7 = sp8[7];
    const float sj2 = p5 * p5;
    const int N4 = (N + 3) & ~3;
    const uint32_t road_id = (uint32_t)(a.road0 + road);
    const int path0 = blockIdx.x * TP;

    for (int q = tid; q < TP * NE; q += blockDim.x) {
        int l = q % NE;
        pop[q] = (l < N) ? ip[l] : 0.0f;
    }
    for (int q = tid; q < TP; q += blockDim.x) gm[q] = p0;
    float cap4[4];
    for (int j = 0; j < 4; ++j) cap4[j] = cp[kg * 4 + j];
    const bool resident = (LC == NE);
    if (resident) {
        for (int q = tid; q < NE * NE; q += blockDim.x) {
            int k = q / NE, l = q - k * NE;
            Mt[l * NE + k] = M[(size_t)k * NP + l];
        }
    }
    __syncthreads();

    for (int t = 0; t < a.n_years; ++t) {
        // growth-rate mean (SimulateGPU.cu:691-701), one thread per path
        for (int q = tid; q < TP; q += blockDim.x) {
            uint32_t path = (uint32_t)(path0 + q);
            float uj = to_uniform1(a.seed, TO_STREAM_SP_JUMP, road_id, path, t, sp);
            float zb = to_normal1(a.seed, TO_STREAM_SP_BROWNIAN, road_id, path, t, sp);
            float zj = to_normal1(a.seed, TO_STREAM_SP_JUMPSIZE, road_id, path, t, sp);
            float jump = (uj < p6) ? 1.0f : 0.0f;
            float brown = zb * p2;
            float jsz = (a.sem == 0) ? (zj * sj2 - sj2 / 2.0f) : (zj * p5 - sj2 / 2.0f);
            float g = gm[q];
            g = g + p4 * (p1 - g) * a.dt + g * brown + (to_expf(jsz) - 1.0f) * g * jump;
            gm[q] = g;
        }
        // migration: acc[i][j] = sum_l pop[p_i][l] * M[k_j][l], l ascending
        float acc[4][4];
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) acc[i][j] = 0.0f;
        for (int l0 = 0; l0 < NE; l0 += LC) {
            if (!resident) {
                __syncthreads();
                for (int q = tid; q < LC * NE; q += blockDim.x) {
                    int k = q / LC, l = q - k * LC;
                    Mt[l * NE + k] = M[(size_t)k * NP + l0 + l];
                }
                __syncthreads();
            }
            if (active) {
                const float* pr = pop + (size_t)(pg * 4) * NE + l0;
                for (int l = 0; l < LC; ++l) {
                    float4 m = *reinterpret_cast<const float4*>(Mt + l * NE + kg * 4);
                    float a0 = pr[l], a1 = pr[NE + l], a2 = pr[2 * NE + l],
                          a3 = pr[3 * NE + l];
                    acc[0][0] = fmaf(a0, m.x, acc[0][0]); acc[0][1] = fmaf(a0, m.y, acc[0][1]);
                    acc[0][2] = fmaf(a0, m.z, acc[0][2]); acc[0][3] = fmaf(a0, m.w, acc[0][3]);
                    acc[1][0] = fmaf(a1, m.x, acc[1][0]); acc[1][1] = fmaf(a1, m.y, acc[1][1]);
                    acc[1][2] = fmaf(a1, m.z, acc[1][2]); acc[1][3] = fmaf(a1, m.w, acc[1][3]);
                    acc[2][0] = fmaf(a2, m.x, acc[2][0]); acc[2][1] = fmaf(a2, m.y, acc[2][1]);
                    acc[2][2] = fmaf(a2, m.z, acc[2][2]); acc[2][3] = fmaf(a2, m.w, acc[2][3]);
                    acc[3][0] = fmaf(a3, m.x, acc[3][0]); acc[3][1] = fmaf(a3, m.y, acc[3][1]);
                    acc[3][2] = fmaf(a3, m.z, acc[3][2]); acc[3][3] = fmaf(a3, m.w, acc[3][3]);
                }
            }
        }
        __syncthreads();   // all reads of pop done, gm ready
        if (active) {
            const bool last = (t == a.n_years - 1);
            for (int i = 0; i < 4; ++i) {
                int pl = pg * 4 + i;
                uint32_t path = (uint32_t)(path0 + pl);
                float z[4];
                to_normal4(a.seed, TO_STREAM_GROWTH, road_id, path, t,
                           (uint32_t)((sp * N4) >> 2) + kg, z);
                float g = gm[pl];
                float4 np;
                float* npv = &np.x;
                for (int j = 0; j < 4; ++j) {
                    float m = acc[i][j];
                    float gr = fmaf(p7 * z[j], g, g);
                    float c = cap4[j];
                    npv[j] = m * (1.0f + gr * (c - m) / c);
                }
                *reinterpret_cast<float4*>(pop + (size_t)pl * NE + kg * 4) = np;
                if (last)
                    *reinterpret_cast<float4*>(mig + (size_t)pl * NE + kg * 4) =
                        make_float4(acc[i][0], acc[i][1], acc[i][2], acc[i][3]);
            }
        }
        __syncthreads();
    }
    // end population: the last migration buffer (Q1) or the grown one
    for (int q = tid; q < TP; q += blockDim.x) {
        int path = path0 + q;
        if (path >= a.n_paths) continue;
        const float* src = (a.n_years == 0) ? pop + (size_t)q * NE
                         : (a.sem == 0 ? mig : pop) + (size_t)q * NE;
        float e = 0.0f;     // groups of four, ((v0 + v1) + v2) + v3, ascending
        for (int g = 0; g < NE; g += 4) e = e + (((src[g] + src[g + 1]) + src[g + 2]) + src[g + 3]);
        a.end_pops[(size_t)rs * a.n_paths + path] = e;
    }
}

// Per (road, species) statistics in FP64: mean, population SD
// (Simulator.cpp:184-191), standard error and P(end < 0.2 init).  A patch
// count outside [0, NP] (a caller's device input that the host could not
// check) gives NaN in all five and reads nothing past the species' row.
__global__ void k_mte_stats(int P, const float* __restrict__ end_pops,
                            const float* __restrict__ init_pops, int NP,
                            const int* __restrict__ n_patches,
                            double* __restrict__ stats) {
    const int rs = blockIdx.x;
    const float* e = end_pops + (size_t)rs * P;
    __shared__ double s_sum[32], s_sq[32], s_cnt[32];
    __shared__ double s_init;
    const int N = n_patches[rs];
    if (N < 0 || N > NP) {
        if (threadIdx.x < 5) stats[5 * (size_t)rs + threadIdx.x] = (double)NAN;
        return;
    }
    if (threadIdx.x == 0) {
        double t = 0.0;
        const float* ip = init_pops + (size_t)rs * NP;
        for (int k = 0; k < N; ++k) t += (double)ip[k];
        s_init = t;
    }
    __syncthreads();
    double sum = 0.0;
    for (int p = threadIdx.x; p < P; p += blockDim.x) sum += (double)e[p];
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if ((threadIdx.x & 31) == 0) s_sum[w] = sum;
    __syncthreads();
    double tot = 0.0;
    for (int i = 0; i < nw; ++i) tot += s_sum[i];
    double mean = tot / (double)P;
    double thr = 0.2 * s_init;
    double sq = 0.0, cnt = 0.0;
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        double d = (double)e[p] - mean;
        sq += d * d;
        cnt += ((double)e[p] < thr) ? 1.0 : 0.0;
    }
    for (int o = 16; o > 0; o >>= 1) {
        sq += __shfl_xor_sync(0xffffffffu, sq, o);
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
    if ((threadIdx.x & 31) == 0) { s_sq[w] = sq; s_cnt[w] = cnt; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double q = 0.0, c = 0.0;
        for (int i = 0; i < nw; ++i) { q += s_sq[i]; c += s_cnt[i]; }
        double sd = sqrt(q / (double)P);
        double* o = stats + 5 * (size_t)rs;
        o[0] = mean;
        o[1] = sd;
        o[2] = (P > 1) ? sqrt(q / (double)(P - 1)) / sqrt((double)P) : 0.0;
        o[3] = c / (double)P;
        o[4] = s_init;
    }
}

}  // namespace

namespace to_k {

to_status mte_simt(to_ctx ctx, to_mte_args a, int n_rs) {
    if (a.npe <= 0) a.npe = a.npad;
    if (!a.flags) a.flags = ctx->d_flags;
    const int NP = a.npe;
    if (NP % 4 != 0 || NP <= 0 || a.npe > a.npad)
        return to_set_error(ctx, TO_ERR_INVALID, "npad %d npe %d", a.npad, a.npe);
    const int KG = NP / 4;
    int pgroups = 256 / KG;
    if (pgroups < 1) pgroups = 1;
    if (pgroups > 16) pgroups = 16;
    if (pgroups * KG > 1024) return to_set_error(ctx, TO_ERR_UNSUPPORTED, "patches %d", NP);
    a.tile_paths = 4 * pgroups;
    size_t budget = 200 * 1024;
    size_t fixed = (size_t)(2 * a.tile_paths * NP + a.tile_paths) * sizeof(float);
    size_t full = (size_t)NP * NP * sizeof(float);
    if (fixed + full <= budget) a.l_chunk = NP;
    else {
        int lc = 64;
        while (lc > 4 && (fixed + (size_t)lc * NP * sizeof(float) > budget || NP % lc)) lc >>= 1;
        if (NP % lc) lc = 4;
        a.l_chunk = lc;
    }
    size_t smem = fixed + (size_t)a.l_chunk * NP * sizeof(float);
    TO_CUDA(ctx, cudaFuncSetAttribute(k_mte_simt,
                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((a.n_paths + a.tile_paths - 1) / a.tile_paths, n_rs);
    int threads = ((pgroups * KG + 31) / 32) * 32;
    to_prof_begin(ctx, "mte_simt");
    k_mte_simt<<<grid, threads, smem, ctx->stream>>>(a);
    to_prof_end(ctx);
    TO_LAUNCHED(ctx);
    return TO_OK;
}

to_status mte_stats(to_ctx ctx, const to_mte_args& a, int n_rs, double* d_stats) {
    k_mte_stats<<<n_rs, 256, 0, ctx->stream>>>(a.n_paths, a.end_pops,
        a.init_pops, a.npad, a.n_patches, d_stats);
    TO_LAUNCHED(ctx);
    return TO_OK;
}

}  // namespace to_k

// ---------------------------------------------------------------------------
// to_simulate_mte_noalloc_d: the MTE statistics entry point for callers that
// cannot allocate device memory.  The per-path end populations, the only
// scratch this computation needs, live in a fixed file-scope device array
// that every GPU loading the library holds until the process exits.
// ---------------------------------------------------------------------------
#include <mutex>

#define TO_NOALLOC_MTE_MAX_VALUES (1 << 21)   // species x paths; 8 MiB of floats

static __device__ __align__(256) float g_mte_noalloc_end[TO_NOALLOC_MTE_MAX_VALUES];

namespace {

struct NoallocDevice {
    std::once_flag once;
    cudaError_t status = cudaSuccess;
    float* end = nullptr;   // device address of g_mte_noalloc_end on this device
};
NoallocDevice g_noalloc_dev[64];

}  // namespace

extern "C" to_status to_simulate_mte_noalloc_d(void* stream,
                                               const to_mte_device_problem* pr,
                                               double* d_stats) {
    if (!pr || !d_stats || pr->n_species <= 0 || pr->n_paths <= 0 || pr->n_years < 0 ||
        pr->npad <= 0 || pr->npad % 4 != 0 || pr->npad > 1020 || !pr->n_patches ||
        !pr->params || !pr->init_pops || !pr->caps || !pr->mmm)
        return TO_ERR_INVALID;
    if ((long long)pr->n_species * pr->n_paths > TO_NOALLOC_MTE_MAX_VALUES ||
        pr->n_species > 65535)      // species are the grid's y dimension
        return TO_ERR_UNSUPPORTED;
    // an error left pending by the caller's own work is not this call's:
    // report it without clearing it, and launch nothing
    if (cudaPeekAtLastError() != cudaSuccess) return TO_ERR_CUDA;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return TO_ERR_NO_DEVICE;
    }
    // one-time set-up on this device (the device is current here): the
    // host-side name of the array is not a device address, so fetch the
    // device address once and keep it
    NoallocDevice& nd = g_noalloc_dev[dev];
    std::call_once(nd.once, [&nd]() {
        void* p = nullptr;
        nd.status = cudaGetSymbolAddress(&p, g_mte_noalloc_end);
        nd.end = static_cast<float*>(p);
    });
    if (nd.status != cudaSuccess || !nd.end) return TO_ERR_CUDA;

    to_mte_args a;
    memset(&a, 0, sizeof(a));
    a.n_paths = pr->n_paths; a.n_years = pr->n_years; a.S = pr->n_species;
    a.C = 1; a.c_use = 0; a.dt = pr->dt; a.seed = pr->seed; a.sem = pr->sem;
    a.road0 = pr->road; a.npad = pr->npad; a.npe = pr->npad;
    a.n_patches = pr->n_patches; a.mmm = pr->mmm; a.init_pops = pr->init_pops;
    a.caps = pr->caps; a.params = pr->params; a.end_pops = nd.end;
    // tile shape as the allocating entry point chooses it
    const int NP = a.npe, KG = NP / 4;
    int pgroups = 256 / KG;
    if (pgroups < 1) pgroups = 1;
    if (pgroups > 16) pgroups = 16;
    a.tile_paths = 4 * pgroups;
    const size_t budget = 200 * 1024;
    const size_t fixed = (size_t)(2 * a.tile_paths * NP + a.tile_paths) * sizeof(float);
    if (fixed + (size_t)NP * NP * sizeof(float) <= budget) a.l_chunk = NP;
    else {
        int lc = 64;
        while (lc > 4 && (fixed + (size_t)lc * NP * sizeof(float) > budget || NP % lc)) lc >>= 1;
        if (NP % lc) lc = 4;
        a.l_chunk = lc;
    }
    const size_t smem = fixed + (size_t)a.l_chunk * NP * sizeof(float);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaFuncSetAttribute(k_mte_simt, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess) {
        cudaGetLastError();   // this call's own error (none was pending)
        return TO_ERR_CUDA;
    }
    dim3 grid((a.n_paths + a.tile_paths - 1) / a.tile_paths, a.S);
    int threads = ((pgroups * KG + 31) / 32) * 32;
    k_mte_simt<<<grid, threads, smem, st>>>(a);
    k_mte_stats<<<a.S, 256, 0, st>>>(a.n_paths, a.end_pops, a.init_pops, a.npad,
                                     a.n_patches, d_stats);
    if (cudaGetLastError() != cudaSuccess) return TO_ERR_CUDA;
    return TO_OK;
}
