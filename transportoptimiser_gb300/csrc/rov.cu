// rov.cu - controlled-traffic real-options valuation on the device
// (ALGO4: forward paths under random controls, regression Monte Carlo
// backward induction with multiple local linear regression on k nearest
// neighbours).
//
// Reference (include/gpuCode/SimulateGPU.cu): simulateROVCUDA :3870-5003,
// randControls :720, forwardPathKernel :789, computePathStates :959,
// allocateXYRegressionData :1012, computeStateMinMax :1073,
// createQueryPoints :1152, firstPeriodInduction :2210, backwardInduction
// :2333, multiLocLinReg :2934, knn_cuda_with_indexes::knn (kNN).
//
// What changes on GB300:
//  * the forward pass keeps every path tile's populations in shared memory
//    for all years and evaluates all controls' migrations from one read of
//    the populations; the random streams are regenerated from Philox where
//    they are consumed (nothing of size P*Y*N is stored);
//  * the reference's serial <<<1,1>>> compaction and min/max kernels become
//    per-chunk counts, an ordered scatter and a per-road finish over all SMs;
//  * kNN runs on the device (knn.cu): persistent warps, one query at a time,
//    the same neighbour set and order as the reference's stable insertion
//    sort without its P x Q distance matrix or host round trips;
//  * the local linear systems are accumulated in FP32 and solved in FP64
//    (Cholesky); expectations are reduced in FP64;
//  * several roads can be valued in one batch: paths are road-major and the
//    regressions are grouped by (road, control).
// Every per-query / per-path formula comes from to_lsm_math.h so the SIMT
// path reproduces the oracle bit for bit.
#include <cmath>
#include <cstring>
#include <vector>

#include "to_internal.cuh"
#include "to_lsm_math.h"
#include "to_rov.cuh"
#include "to_rov_dev.cuh"
#include "to_sparse.cuh"

namespace {

using to_rovd::adj_pop;
using to_rovd::ore_at;
using to_rovd::threshold;
using to_rovd::unit_profit;

// ---------------------------------------------------------------------------
// exogenous processes and random controls (forwardPathKernel :930-952,
// randControls :720-730): uRes[u][t][p], controls[t][p]
// ---------------------------------------------------------------------------
__global__ void k_rov_exog(to_rov_args a) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.PT) return;
    const int Y = a.Y, U = a.U, P = a.PT;
    const int r = p / a.P, pl = p - r * a.P;      // road, path within it
    const uint32_t road = (uint32_t)a.road_ids[r];
    for (int u = 0; u < U; ++u) a.uRes[((size_t)u * (Y + 1)) * P + p] = a.uncert[6 * u];
    for (int t = 0; t < Y; ++t) {
        float uc = to_uniform1(a.seed, TO_STREAM_CONTROL, road, pl, t, 0);
        int control = (int)(uc * (float)a.C);
        if (control == a.C) control--;
        a.controls[(size_t)t * P + p] = control;
        for (int u = 0; u < U; ++u) {
            const float* up = a.uncert + 6 * u;
            float uj = to_uniform1(a.seed, TO_STREAM_EX_JUMP, road, pl, t, u);
            float zb = to_normal1(a.seed, TO_STREAM_EX_BROWNIAN, road, pl, t, u);
            float zj = to_normal1(a.seed, TO_STREAM_EX_JUMPSIZE, road, pl, t, u);
            float jump = (uj < up[5]) ? 1.0f : 0.0f;
            float curr = a.uRes[((size_t)u * (Y + 1) + t) * P + p];
            float brown = zb * up[2];
            float s4 = up[4] * up[4];
            float jsz = (a.sem == 0) ? (zj * s4 - s4 / 2.0f) : (zj * up[4] - s4 / 2.0f);
            a.uRes[((size_t)u * (Y + 1) + t + 1) * P + p] =
                curr + up[3] * (up[1] - curr) * a.dt + curr * brown
                + (to_expf(jsz) - 1.0f) * curr * jump;
        }
    }
}

// ---------------------------------------------------------------------------
// forward paths (forwardPathKernel :789-956).  One CTA = a tile of TP paths,
// one species at a time, all years; thread (pg, kg) owns paths 4pg..4pg+3
// and patches 4kg..4kg+3 for every control.
// ---------------------------------------------------------------------------
template <int CMAX>
__global__ void __launch_bounds__(512)
k_rov_forward(to_rov_args a) {
    extern __shared__ float smem[];
    const int NE = a.ne, KG = NE >> 2, TP = a.tile_paths, LC = a.l_chunk;
    const int C = a.C, Y = a.Y, P = a.P;
    const int tid = threadIdx.x, pg = tid / KG, kg = tid - pg * KG;
    const bool active = pg < (TP >> 2);
    const int path0 = blockIdx.x * TP;
    float* Mt = smem;                               // [C][LC][NE]
    float* pop = Mt + (size_t)C * LC * NE;          // [TP][NE]
    float* mig = pop + (size_t)TP * NE;             // [TP][NE]
    float* gm = mig + (size_t)TP * NE;              // [TP]
    float* tot = gm + TP;                           // [TP]
    int* ctl = reinterpret_cast<int*>(tot + TP);    // [TP]
    const uint32_t road = (uint32_t)a.road;
    const bool resident = (LC == NE);

    for (int s = 0; s < a.S; ++s) {
        const int N = a.n_patches[s];
        const int N4 = (N + 3) & ~3;
        const float* sp = a.params + 8 * s;
        const float* M = a.mmm + (size_t)s * C * a.np * a.np;
        const float* ip = a.init_pops + (size_t)s * a.np;
        float cap4[4];
        for (int j = 0; j < 4; ++j) cap4[j] = a.caps[(size_t)s * a.np + kg * 4 + j];
        __syncthreads();
        for (int q = tid; q < TP * NE; q += blockDim.x) {
            int l = q % NE;
            pop[q] = (l < N) ? ip[l] : 0.0f;
        }
        if (resident) {
            for (int q = tid; q < C * NE * NE; q += blockDim.x) {
                int c = q / (NE * NE), r = q - c * NE * NE;
                int k = r / NE, l = r - k * NE;
                Mt[((size_t)c * NE + l) * NE + k] = M[((size_t)c * a.np + k) * a.np + l];
            }
        }
        __syncthreads();
        for (int q = tid; q < TP; q += blockDim.x) {
            gm[q] = sp[0];
            const float* v = pop + (size_t)q * NE;
            float tt = 0.0f;    // groups of four, ((v0 + v1) + v2) + v3, ascending
            for (int g4 = 0; g4 < NE; g4 += 4) tt = tt + (((v[g4] + v[g4 + 1]) + v[g4 + 2]) + v[g4 + 3]);
            tot[q] = tt;
            int path = path0 + q;
            if (path < P) a.totalPops[((size_t)s * (Y + 1) + 0) * P + path] = tt;
        }
        __syncthreads();
        for (int t = 0; t < Y; ++t) {
            for (int q = tid; q < TP; q += blockDim.x) {
                uint32_t path = (uint32_t)(path0 + q);
                float uj = to_uniform1(a.seed, TO_STREAM_SP_JUMP, road, path, t, s);
                float zb = to_normal1(a.seed, TO_STREAM_SP_BROWNIAN, road, path, t, s);
                float zj = to_normal1(a.seed, TO_STREAM_SP_JUMPSIZE, road, path, t, s);
                float jp = (a.sem == 0) ? sp[5] : sp[6];
                float jump = (uj < jp) ? 1.0f : 0.0f;
                float brown = zb * sp[2];
                float s5 = sp[5] * sp[5];
                float jsz = (a.sem == 0) ? (zj * s5 - s5 / 2.0f) : (zj * sp[5] - s5 / 2.0f);
                float g = gm[q];
                gm[q] = g + sp[4] * (sp[1] - g) * a.dt + g * brown
                        + (to_expf(jsz) - 1.0f) * g * jump;
                ctl[q] = (path0 + q < P) ? a.controls[(size_t)t * P + path0 + q] : 0;
            }
            float acc[CMAX][4][4];
#pragma unroll
            for (int c = 0; c < CMAX; ++c)
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[c][i][j] = 0.0f;
            for (int l0 = 0; l0 < NE; l0 += LC) {
                if (!resident) {
                    __syncthreads();
                    for (int q = tid; q < C * LC * NE; q += blockDim.x) {
                        int c = q / (LC * NE), r = q - c * LC * NE;
                        int k = r / LC, l = r - k * LC;
                        Mt[((size_t)c * LC + l) * NE + k] =
                            M[((size_t)c * a.np + k) * a.np + l0 + l];
                    }
                    __syncthreads();
                }
                if (active) {
                    const float* pr = pop + (size_t)(pg * 4) * NE + l0;
                    for (int l = 0; l < LC; ++l) {
                        float a0 = pr[l], a1 = pr[NE + l], a2 = pr[2 * NE + l],
                              a3 = pr[3 * NE + l];
#pragma unroll
                        for (int c = 0; c < CMAX; ++c) {
                            if (c >= C) break;
                            float4 m = *reinterpret_cast<const float4*>(
                                Mt + ((size_t)c * LC + l) * NE + kg * 4);
                            acc[c][0][0] = fmaf(a0, m.x, acc[c][0][0]); acc[c][0][1] = fmaf(a0, m.y, acc[c][0][1]);
                            acc[c][0][2] = fmaf(a0, m.z, acc[c][0][2]); acc[c][0][3] = fmaf(a0, m.w, acc[c][0][3]);
                            acc[c][1][0] = fmaf(a1, m.x, acc[c][1][0]); acc[c][1][1] = fmaf(a1, m.y, acc[c][1][1]);
                            acc[c][1][2] = fmaf(a1, m.z, acc[c][1][2]); acc[c][1][3] = fmaf(a1, m.w, acc[c][1][3]);
                            acc[c][2][0] = fmaf(a2, m.x, acc[c][2][0]); acc[c][2][1] = fmaf(a2, m.y, acc[c][2][1]);
                            acc[c][2][2] = fmaf(a2, m.z, acc[c][2][2]); acc[c][2][3] = fmaf(a2, m.w, acc[c][2][3]);
                            acc[c][3][0] = fmaf(a3, m.x, acc[c][3][0]); acc[c][3][1] = fmaf(a3, m.y, acc[c][3][1]);
                            acc[c][3][2] = fmaf(a3, m.z, acc[c][3][2]); acc[c][3][3] = fmaf(a3, m.w, acc[c][3][3]);
                        }
                    }
                }
            }
            // per-control totals (AAR numerators) summed patch-ascending
            for (int c = 0; c < C; ++c) {
                __syncthreads();
                if (active) {
#pragma unroll
                    for (int cc = 0; cc < CMAX; ++cc) {
                        if (cc != c) continue;
#pragma unroll
                        for (int i = 0; i < 4; ++i)
                            *reinterpret_cast<float4*>(mig + (size_t)(pg * 4 + i) * NE + kg * 4) =
                                make_float4(acc[cc][i][0], acc[cc][i][1], acc[cc][i][2], acc[cc][i][3]);
                    }
                }
                __syncthreads();
                for (int q = tid; q < TP; q += blockDim.x) {
                    const float* v = mig + (size_t)q * NE;
                    float tc = 0.0f;
                    for (int g4 = 0; g4 < NE; g4 += 4)
                        tc = tc + (((v[g4] + v[g4 + 1]) + v[g4 + 2]) + v[g4 + 3]);
                    int path = path0 + q;
                    if (path < P)
                        a.aars[(((size_t)s * C + c) * Y + t) * P + path] = tc / tot[q];
                }
            }
            __syncthreads();
            // growth under the path's random control
            if (active) {
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    int pl = pg * 4 + i;
                    uint32_t path = (uint32_t)(path0 + pl);
                    float z[4];
                    to_normal4(a.seed, TO_STREAM_GROWTH, road, path, t,
                               (uint32_t)((s * N4) >> 2) + kg, z);
                    int c = ctl[pl];
                    float mv[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
                    for (int cc = 0; cc < CMAX; ++cc)
                        if (cc == c)
#pragma unroll
                            for (int j = 0; j < 4; ++j) mv[j] = acc[cc][i][j];
                    float g = gm[pl];
                    float4 np;
                    float* npv = &np.x;
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        float m = mv[j];
                        float gr = (a.sem == 0) ? g + z[j] * sp[7] : fmaf(sp[7] * z[j], g, g);
                        float cp = cap4[j];
                        npv[j] = (a.sem == 0) ? m * (1.0f + gr * (cp - m) / cp / 100.0f)
                                              : fmaxf(m * (1.0f + gr * (cp - m) / cp), 0.0f);
                    }
                    *reinterpret_cast<float4*>(pop + (size_t)pl * NE + kg * 4) = np;
                }
            }
            __syncthreads();
            for (int q = tid; q < TP; q += blockDim.x) {
                const float* v = pop + (size_t)q * NE;
                float tt = 0.0f;
                for (int g4 = 0; g4 < NE; g4 += 4)
                    tt = tt + (((v[g4] + v[g4 + 1]) + v[g4 + 2]) + v[g4 + 3]);
                tot[q] = tt;
                int path = path0 + q;
                if (path < P) a.totalPops[((size_t)s * (Y + 1) + t + 1) * P + path] = tt;
            }
            __syncthreads();
        }
    }
}


// terminal year (backwardInduction :2375-2463)
__global__ void k_rov_terminal(to_rov_args a) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.PT) return;
    const int t = a.Y - 1, C = a.C, S = a.S;
    float state[TO_ROV_MAXC * (TO_LSM_MAXD - 1) + 1];
    for (int c = 0; c < C; ++c)
        for (int s = 0; s < S; ++s) state[c * S + s] = adj_pop(a, p, t, s, c);
    float prof = unit_profit(a, p, t, a.Y + 1, a.sem == 0 ? a.Y : a.Y + 1);
    state[S * C] = prof;
    float best;
    int bc;
    to_rovd::decide_terminal(a, state, best, bc);
    a.condExp[(size_t)t * a.PT + p] = best;
    a.optCont[(size_t)t * a.PT + p] = bc;
    a.unitProfits[(size_t)t * a.PT + p] = prof;
    for (int s = 0; s < S; ++s)
        a.adjPops[((size_t)t * S + s) * a.PT + p] = state[(C - 1) * S + s];
}

// Per year: regression states, stable compaction by the year's random
// control (allocateXYRegressionData :1012-1069), per-control and global
// min/max (computeStateMinMax :1073-1148), k, normalised points and the
// axis values of the regression grid.  Points are grouped by (road,
// control), g = r*C + c.  Launches over chunks of kLsmChunk paths:
// per-chunk counts by group, then the scatter in path order (earlier
// chunks of the road + earlier warps + rank among the warp's lanes of the
// same group) with min/max folded into order-preserving integer keys; then
// one thread per road for its totals, k, min/max rules and grid axes, and
// the normalisation across the grid.

constexpr int kLsmChunk = 1024;
// roads of a batch have at least this many paths, so a chunk touches at
// most kLsmChunk / kLsmMinPaths + 2 roads
constexpr int kLsmMinPaths = 128;
constexpr int kLsmLocal = (kLsmChunk / kLsmMinPaths + 2) * TO_ROV_MAXC;

// the year's regression group of path p: (road, control) when every
// species' adjusted population clears its threshold (or the control is 0),
// else -1
__device__ __forceinline__ int lsm_group(const to_rov_args& a, int p, int t) {
    if (p >= a.PT) return -1;
    const int ctl = a.controls[(size_t)t * a.PT + p];
    const int g = (p / a.P) * a.C + ctl;
    if (ctl == 0) return g;
    for (int s = 0; s < a.S; ++s)
        if (adj_pop(a, p, t, s, a.C - 1) < a.params[8 * s + 3]) return -1;
    return g;
}

// first group of chunk b and how many groups it can hold
__device__ __forceinline__ void lsm_chunk_groups(const to_rov_args& a, int b, int& g0, int& nloc) {
    const int p0 = b * kLsmChunk;
    const int p1 = min(p0 + kLsmChunk, a.PT) - 1;
    const int r0 = p0 / a.P, r1 = p1 / a.P;
    g0 = r0 * a.C;
    nloc = (r1 - r0 + 1) * a.C;
}

// order-preserving unsigned key of a float (min/max through integer atomics)
__device__ __forceinline__ unsigned lsm_key(float v) {
    unsigned k = __float_as_uint(v);
    return (k & 0x80000000u) ? ~k : (k | 0x80000000u);
}
__device__ __forceinline__ float lsm_unkey(unsigned k) {
    k = (k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k;
    return __uint_as_float(k);
}

__global__ void __launch_bounds__(kLsmChunk) k_lsm_count(to_rov_args a, int t) {
    __shared__ int s_cnt[kLsmLocal];
    const int d = a.S + 1, tid = threadIdx.x, lane = tid & 31;
    int g0, nloc;
    lsm_chunk_groups(a, blockIdx.x, g0, nloc);
    for (int q = tid; q < nloc; q += blockDim.x) s_cnt[q] = 0;
    if (blockIdx.x == 0)
        for (int q = tid; q < a.G * d; q += blockDim.x) {
            a.lkey[2 * q] = 0xFFFFFFFFu;
            a.lkey[2 * q + 1] = 0u;
        }
    __syncthreads();
    const int grp = lsm_group(a, blockIdx.x * kLsmChunk + tid, t);
    const unsigned peers = __match_any_sync(0xffffffffu, grp);
    if (grp >= 0 && lane == __ffs(peers) - 1) atomicAdd(&s_cnt[grp - g0], __popc(peers));
    __syncthreads();
    for (int q = tid; q < nloc; q += blockDim.x)
        a.lcnt[(size_t)(g0 + q) * gridDim.x + blockIdx.x] = s_cnt[q];
}

__global__ void __launch_bounds__(kLsmChunk) k_lsm_scatter(to_rov_args a, int t) {
    const int P = a.P, S = a.S, C = a.C, d = S + 1, nb = gridDim.x;
    __shared__ int s_off[kLsmLocal];
    __shared__ int s_scan[kLsmLocal][32];
    __shared__ unsigned s_key[kLsmLocal][TO_LSM_MAXD][2];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
    int g0, nloc;
    lsm_chunk_groups(a, blockIdx.x, g0, nloc);
    // chunk offsets: warp q sums group q's counts in the road's earlier chunks
    for (int q = warp; q < nloc; q += nw) {
        const int g = g0 + q;
        const int bfirst = (int)(((size_t)(g / C) * P) / kLsmChunk);
        int acc = 0;
        for (int b = bfirst + lane; b < (int)blockIdx.x; b += 32) acc += a.lcnt[(size_t)g * nb + b];
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) s_off[q] = acc;
    }
    for (int q = tid; q < nloc * 32; q += blockDim.x) s_scan[q >> 5][q & 31] = 0;
    for (int q = tid; q < nloc * d; q += blockDim.x) {
        s_key[q / d][q % d][0] = 0xFFFFFFFFu;
        s_key[q / d][q % d][1] = 0u;
    }
    __syncthreads();                     // zeroed before any warp adds to them
    const int p = blockIdx.x * kLsmChunk + tid;
    const int grp = lsm_group(a, p, t);
    float xv[TO_LSM_MAXD];
    if (grp >= 0) {
        for (int s = 0; s < S; ++s) xv[s] = adj_pop(a, p, t, s, C - 1);
        xv[S] = unit_profit(a, p, t, a.Y + 1, a.Y + 1);
    }
    // lanes of the same group: rank, count and min / max of the states
    const unsigned peers = __match_any_sync(0xffffffffu, grp);
    const int before = __popc(peers & ((1u << lane) - 1u));
    const bool leader = lane == __ffs(peers) - 1;
    if (grp >= 0) {
        const int lq = grp - g0;
        if (leader) s_scan[lq][warp] = __popc(peers);
        for (int j = 0; j < d; ++j) {
            const unsigned lo = __reduce_min_sync(peers, lsm_key(xv[j]));
            const unsigned hi = __reduce_max_sync(peers, lsm_key(xv[j]));
            if (leader) {
                atomicMin(&s_key[lq][j][0], lo);
                atomicMax(&s_key[lq][j][1], hi);
            }
        }
    }
    __syncthreads();
    if (grp >= 0) {
        const int lq = grp - g0;
        int pos = s_off[lq] + before;
        for (int w = 0; w < warp; ++w) pos += s_scan[lq][w];
        a.yv[(size_t)grp * P + pos] = a.condExp[(size_t)(t + 1) * a.PT + p];
        for (int j = 0; j < d; ++j) a.xraw[((size_t)grp * d + j) * P + pos] = xv[j];
    }
    for (int q = tid; q < nloc * d; q += blockDim.x) {
        const int lq = q / d, j = q % d;
        if (s_key[lq][j][1] != 0u) {     // the chunk holds points of the group
            const size_t gq = (size_t)(g0 + lq) * d + j;
            atomicMin(&a.lkey[2 * gq], s_key[lq][j][0]);
            atomicMax(&a.lkey[2 * gq + 1], s_key[lq][j][1]);
        }
    }
}

// a warp per road, lanes over its (control, dimension, bin) items: group
// totals, the reference's min/max rules, the road's combined range, k and
// the regression grid axes
constexpr int kStatsWarps = 4;

__global__ void __launch_bounds__(kStatsWarps * 32) k_lsm_stats(to_rov_args a, int t, int nb) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int r = blockIdx.x * kStatsWarps + w;
    if (r >= a.nr) return;
    __shared__ int s_cnt[kStatsWarps][TO_ROV_MAXC];
    __shared__ float s_mn[kStatsWarps][TO_ROV_MAXC + 1][TO_LSM_MAXD];
    __shared__ float s_mx[kStatsWarps][TO_ROV_MAXC + 1][TO_LSM_MAXD];
    const int P = a.P, S = a.S, C = a.C, d = S + 1, R = a.R;
    const int bfirst = (int)(((size_t)r * P) / kLsmChunk);
    const int blast = (int)(((size_t)r * P + P - 1) / kLsmChunk);
    int* cnt = s_cnt[w];
    float (*mn)[TO_LSM_MAXD] = s_mn[w];
    float (*mx)[TO_LSM_MAXD] = s_mx[w];
    for (int c = lane; c < C; c += 32) {
        const size_t g = (size_t)r * C + c;
        int n = 0;
        for (int b = bfirst; b <= blast; ++b) n += a.lcnt[g * nb + b];
        cnt[c] = n;
    }
    __syncwarp();
    // each control's own ranges (control 0, and any with more than d + 1
    // points), then the others take control 0's
    for (int q = lane; q < C * d; q += 32) {
        const int c = q / d, j = q - c * d;
        const size_t g = (size_t)r * C + c;
        if (!((c == 0) || (cnt[c] > d + 1))) continue;
        if (cnt[c] > 0) {
            float lo = lsm_unkey(a.lkey[2 * (g * d + j)]);
            float hi = lsm_unkey(a.lkey[2 * (g * d + j) + 1]);
            // the reference scans from the first point with
            // "if (xmin > x) ... else if (xmax < x)": plain min and max,
            // except that a first value of -0/+0 keeps its sign when it is
            // the extreme
            const float first = a.xraw[(g * d + j) * P];
            if (lo == first) lo = first;
            if (hi == first) hi = first;
            mn[c][j] = lo; mx[c][j] = hi;
        } else {
            mn[c][j] = 0.0f; mx[c][j] = 0.0f;
        }
    }
    __syncwarp();
    for (int q = lane; q < C * d; q += 32) {
        const int c = q / d, j = q - c * d;
        if ((c == 0) || (cnt[c] > d + 1)) continue;
        mn[c][j] = mn[0][j]; mx[c][j] = mx[0][j];
    }
    __syncwarp();
    for (int j = lane; j < d; j += 32) {
        float lo = mn[0][j], hi = mx[0][j];
        for (int c = 1; c < C; ++c) {
            if (lo > mn[c][j]) lo = mn[c][j];
            if (hi < mx[c][j]) hi = mx[c][j];
        }
        mn[C][j] = lo; mx[C][j] = hi;
        a.gmin[(size_t)r * d + j] = lo;
        a.gmax[(size_t)r * d + j] = hi;
    }
    __syncwarp();
    if (a.qax)
        for (int q = lane; q < d * R; q += 32) {
            const int j = q / R, di = q - j * R;
            const float lo = mn[C][j], hi = mx[C][j];
            a.qax[((size_t)r * d + j) * R + di] =
                to_lsm_normalise(to_lsm_query_axis(di, lo, hi, R), lo, hi, j == S, a.scaling);
        }
    for (int c = lane; c < C; c += 32) {
        const size_t g = (size_t)r * C + c;
        const int n = cnt[c];
        int k = 0;
        if (n > 3) {
            k = (int)((double)a.k_mult * (log((double)n) + 1.0));
            if (k > n) k = n;
        }
        a.npts[g] = n;
        a.kc[g] = k;
    }
    // axis values of the regression grid (createQueryPoints :1187-1190)
    for (int q = lane; q < C * d * R; q += 32) {
        const int c = q / (d * R), jr = q - c * d * R, j = jr / R, di = jr - j * R;
        float* ax = to_rov_reg_block(a, t, (size_t)r * C + c);
        ax[(size_t)j * R + di] = to_lsm_query_axis(di, mn[C][j], mx[C][j], R);
    }
}

// normalised points (host normalisation, SimulateGPU.cu:4591-4603)
__global__ void __launch_bounds__(256) k_lsm_norm(to_rov_args a) {
    const int P = a.P, S = a.S, C = a.C, d = S + 1;
    const size_t total = (size_t)a.G * d * P;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < total;
         q += (size_t)gridDim.x * blockDim.x) {
        const size_t gj = q / P;
        const int m = (int)(q - gj * P);
        const int g = (int)(gj / d), j = (int)(gj - (size_t)g * d);
        if (m >= a.npts[g]) continue;
        const size_t r = (size_t)(g / C);
        a.xn[q] = to_lsm_normalise(a.xraw[q], a.gmin[r * d + j], a.gmax[r * d + j], j == S,
                                   a.scaling);
    }
}

// Touched-query mode, corrected semantics: k_rov_backward at year t reads
// control c's regression block of the path's road at the 2^d corners of
// the cell holding the path's own state for c (to_lsm_interp), for every
// control valid for the path (decide_interior).  Mark exactly those grid
// queries; k_lsm_list compacts the marks into the year's work list and
// clears them again.  The reads happen after this year's axes are written
// (k_lsm_stats), so the corners are the ones the backward pass will read.
__global__ void __launch_bounds__(256) k_lsm_mark(to_rov_args a, int t) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0) *a.qcount = 0;
    if (p >= a.PT) return;
    const int C = a.C, S = a.S, d = S + 1, R = a.R;
    const int r = p / a.P;
    float state[TO_ROV_MAXC * (TO_LSM_MAXD - 1) + 1];
    for (int c = 0; c < C; ++c)
        for (int s = 0; s < S; ++s) state[c * S + s] = adj_pop(a, p, t, s, c);
    const int sy = a.Y + 1;
    const float prof = unit_profit(a, p, t, sy, sy);
    for (int c = 0; c < C; ++c) {
        bool valid = true;
        for (int s = 0; s < S; ++s)
            if (state[c * S + s] < threshold(a, s) && c > 0) { valid = false; break; }
        if (!valid) continue;
        const size_t g = (size_t)r * C + c;
        const float* rb = to_rov_reg_block(a, t, g);
        int li[TO_LSM_MAXD];
        for (int j = 0; j < d; ++j) {
            const float v = (j < S) ? state[c * S + j] : prof;
            li[j] = to_lsm_lower_index(v, rb[j * R], rb[j * R + R - 1], R);
        }
        unsigned char* mk = a.qmark + g * a.Q;
        for (int corner = 0; corner < (1 << d); ++corner) {
            int idx = 0;
            for (int j = 0; j < d; ++j) idx = idx * R + li[j] + ((corner >> (d - 1 - j)) & 1);
            mk[idx] = 1;
        }
    }
}

// compaction of the year's marks into flat items g*Q + q (any order: each
// item writes only its own outputs), clearing them for the next year
__global__ void __launch_bounds__(1024) k_lsm_list(to_rov_args a) {
    __shared__ int s_w[32];
    __shared__ int s_base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const size_t total = (size_t)a.G * a.Q;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool on = i < total && a.qmark[i] != 0;
    const unsigned b = __ballot_sync(0xffffffffu, on);
    if (lane == 0) s_w[warp] = __popc(b);
    __syncthreads();
    if (threadIdx.x == 0) {
        int tot = 0;
        for (int w = 0; w < nw; ++w) { const int v = s_w[w]; s_w[w] = tot; tot += v; }
        s_base = tot > 0 ? atomicAdd(a.qcount, tot) : 0;
    }
    __syncthreads();
    if (on) {
        a.qlist[s_base + s_w[warp] + __popc(b & ((1u << lane) - 1u))] = (int)i;
        a.qmark[i] = 0;
    }
    if (a.qroad && b) {
        // queries fitted per road (a warp's 32 items mostly share one road)
        const int road = (int)(i / ((size_t)a.Q * a.C));
        const unsigned same = __match_any_sync(0xffffffffu, road);
        if (on && lane == __ffs(same & b) - 1) atomicAdd(&a.qroad[road], (unsigned)__popc(same & b));
    }
}

}  // namespace

namespace {

// backwardInduction for 0 < t < Y-1 (:2464-2776)
__global__ void k_rov_backward(to_rov_args a, int t) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.PT) return;
    const int C = a.C, S = a.S;
    float state[TO_ROV_MAXC * (TO_LSM_MAXD - 1) + 1];
    for (int c = 0; c < C; ++c)
        for (int s = 0; s < S; ++s) state[c * S + s] = adj_pop(a, p, t, s, c);
    for (int s = 0; s < S; ++s)
        a.adjPops[((size_t)t * S + s) * a.PT + p] = state[(C - 1) * S + s];
    int sy = (a.sem == 0) ? a.Y : a.Y + 1;
    float prof = unit_profit(a, p, t, sy, sy);
    state[S * C] = prof;
    a.unitProfits[(size_t)t * a.PT + p] = prof;
    float best;
    int bc;
    to_rovd::decide_interior(a, t, p / a.P, state, best, bc);
    a.condExp[(size_t)t * a.PT + p] = best;
    a.optCont[(size_t)t * a.PT + p] = bc;
}

// firstPeriodInduction (:2210-2330) with FP64 reductions; one CTA.
__global__ void k_rov_first(to_rov_args a) {
    // one CTA per road; its paths are base .. base+P-1 of the batch
    const int P = a.P, C = a.C, S = a.S, Y = a.Y;
    const size_t PT = (size_t)a.PT, base = (size_t)blockIdx.x * P;
    __shared__ double s_sum[TO_ROV_MAXC][32], s_cnt[TO_ROV_MAXC][32];
    __shared__ double s_best;
    __shared__ int s_bc;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    double sum[TO_ROV_MAXC], cnt[TO_ROV_MAXC];
    for (int c = 0; c < C; ++c) { sum[c] = 0.0; cnt[c] = 0.0; }
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        int c = a.controls[base + p];
        sum[c] += (double)a.condExp[PT + base + p];
        cnt[c] += 1.0;
    }
    for (int c = 0; c < C; ++c) {
        for (int o = 16; o > 0; o >>= 1) {
            sum[c] += __shfl_xor_sync(0xffffffffu, sum[c], o);
            cnt[c] += __shfl_xor_sync(0xffffffffu, cnt[c], o);
        }
        if (lane == 0) { s_sum[c][warp] = sum[c]; s_cnt[c][warp] = cnt[c]; }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float uf = 0.0f, ore = 0.0f;
        for (int f = 0; f < a.nF; ++f)
            uf = fmaf(a.fuel_costs[f], a.uRes[((size_t)a.fuel_idx[f] * (Y + 1)) * PT + base], uf);
        for (int c = 0; c < a.Cm; ++c)
            ore = fmaf(ore_at(a, (int)base, 0, c),
                       a.uRes[((size_t)(a.nF + c) * (Y + 1)) * PT + base], ore);
        float prof0 = (a.unit_cost + uf) - a.unit_revenue * ore;
        if (a.demand_idx >= 0)
            prof0 = prof0 * a.uRes[((size_t)a.demand_idx * (Y + 1)) * PT + base];
        const double discd = (double)(1.0f + a.rrr * a.dt / 100.0f);
        double pay[TO_ROV_MAXC];
        int stop = C;
        for (int c = 0; c < C; ++c) {
            double sm = 0.0, cn = 0.0;
            for (int w = 0; w < nw; ++w) { sm += s_sum[c][w]; cn += s_cnt[c][w]; }
            if (cn > 0.0) pay[c] = sm / (cn * discd);
            else { stop = c; break; }
            bool valid = true;
            for (int s = 0; s < S; ++s) {
                float adj = a.totalPops[((size_t)s * (Y + 1)) * PT + base] *
                            a.aars[(((size_t)s * C + c) * Y) * PT + base];
                if (adj < threshold(a, s) && c > 0) { valid = false; break; }
            }
            if (valid) {
                pay[c] += (double)(a.flows[c] * prof0);
                if (pay[c] > 0.0) pay[c] = 0.0;
            } else pay[c] = NAN;
        }
        for (int c = stop; c < C; ++c) pay[c] = (c == 0) ? 0.0 : NAN;
        double best = pay[0];
        int bc = 0;
        for (int c = 1; c < C; ++c)
            if (isfinite(pay[c]) && pay[c] < best) { best = pay[c]; bc = c; }
        s_best = best;
        s_bc = bc;
    }
    __syncthreads();
    const double best = s_best;
    const int bc = s_bc;
    double ss = 0.0, m1 = 0.0, n1 = 0.0;
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        if (a.controls[base + p] == bc) {
            double v = (double)a.condExp[PT + base + p];
            ss += (v - best) * (v - best);
            m1 += v;
            n1 += 1.0;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        ss += __shfl_xor_sync(0xffffffffu, ss, o);
        m1 += __shfl_xor_sync(0xffffffffu, m1, o);
        n1 += __shfl_xor_sync(0xffffffffu, n1, o);
    }
    __syncthreads();
    if (lane == 0) { s_sum[0][warp] = ss; s_sum[1][warp] = m1; s_cnt[0][warp] = n1; }
    __syncthreads();
    double SS = 0.0, M1 = 0.0, N1 = 0.0;
    for (int w = 0; w < nw; ++w) { SS += s_sum[0][w]; M1 += s_sum[1][w]; N1 += s_cnt[0][w]; }
    const double discd = (double)(1.0f + a.rrr * a.dt / 100.0f);
    // sample variance of the chosen control's year-1 values
    double mean = N1 > 0.0 ? M1 / N1 : 0.0;
    double vv = 0.0;
    for (int p = threadIdx.x; p < P; p += blockDim.x)
        if (a.controls[base + p] == bc) {
            double v = (double)a.condExp[PT + base + p] - mean;
            vv += v * v;
        }
    for (int o = 16; o > 0; o >>= 1) vv += __shfl_xor_sync(0xffffffffu, vv, o);
    __syncthreads();
    if (lane == 0) s_sum[2 % TO_ROV_MAXC][warp] = vv;
    __syncthreads();
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        a.condExp[base + p] = (float)best;
        a.optCont[base + p] = bc;
    }
    if (threadIdx.x == 0) {
        double V = 0.0;
        for (int w = 0; w < nw; ++w) V += s_sum[2 % TO_ROV_MAXC][w];
        double sdfac = (a.sem == 0) ? (1.0 + (double)a.rrr / (100.0 * (double)a.dt)) : discd;
        double* st = a.stats + 5 * (size_t)blockIdx.x;
        st[0] = (double)(float)best;
        st[1] = (double)bc;
        st[2] = (N1 > 0.0) ? sqrt(SS / (N1 * sdfac)) : 0.0;
        st[3] = (N1 > 1.0) ? sqrt(V / (N1 - 1.0)) / sqrt(N1) / discd : 0.0;
        st[4] = N1;
    }
}

}  // namespace

namespace to_k {

to_status rov_backward(to_ctx ctx, const to_rov_args& a, int pblocks, int tpb,
                       const to_csc* csc);

to_status rov_run(to_ctx ctx, to_rov_args a, const to_csc* csc) {
    const int P = a.PT;                        // every path of the batch
    const int tpb = 128;
    const int pblocks = (P + tpb - 1) / tpb;
    to_prof_begin(ctx, "rov_exog");
    k_rov_exog<<<pblocks, tpb, 0, ctx->stream>>>(a);
    to_prof_end(ctx);
    TO_LAUNCHED(ctx);
    if (csc) {
        TO_TRY(rov_forward_sparse(ctx, a, *csc));
        return rov_backward(ctx, a, pblocks, tpb, csc);
    }
    if (a.nr != 1)
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "batched roads need the sparse migration form");
    // forward tile shape
    const int NE = a.ne, KG = NE / 4;
    int pgroups = 256 / KG;
    if (pgroups < 1) pgroups = 1;
    if (pgroups > 16) pgroups = 16;
    if (pgroups * KG > 1024) return to_set_error(ctx, TO_ERR_UNSUPPORTED, "patches %d", NE);
    a.tile_paths = 4 * pgroups;
    size_t fixed = (size_t)(2 * a.tile_paths * NE + 3 * a.tile_paths) * sizeof(float);
    size_t budget = 200 * 1024;
    if (fixed + (size_t)a.C * NE * NE * 4 <= budget) a.l_chunk = NE;
    else {
        int lc = 64;
        while (lc > 4 && (fixed + (size_t)a.C * lc * NE * 4 > budget || NE % lc)) lc >>= 1;
        if (NE % lc) lc = 4;
        a.l_chunk = lc;
    }
    size_t smem = fixed + (size_t)a.C * a.l_chunk * NE * sizeof(float);
    dim3 grid((P + a.tile_paths - 1) / a.tile_paths);
    int threads = ((pgroups * KG + 31) / 32) * 32;
    if (a.C > TO_ROV_MAXC) return to_set_error(ctx, TO_ERR_UNSUPPORTED, "controls %d", a.C);
    to_prof_begin(ctx, "rov_forward");
    if (a.C <= 3) {
        TO_CUDA(ctx, cudaFuncSetAttribute(k_rov_forward<3>,
                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_rov_forward<3><<<grid, threads, smem, ctx->stream>>>(a);
    } else {
        TO_CUDA(ctx, cudaFuncSetAttribute(k_rov_forward<TO_ROV_MAXC>,
                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_rov_forward<TO_ROV_MAXC><<<grid, threads, smem, ctx->stream>>>(a);
    }
    to_prof_end(ctx);
    TO_LAUNCHED(ctx);
    return rov_backward(ctx, a, pblocks, tpb, nullptr);
}

to_status rov_backward(to_ctx ctx, const to_rov_args& a, int pblocks, int tpb,
                       const to_csc* csc) {
    if (a.algo == 6 && (!csc || !a.popsY || !a.gmY || a.nr != 1))
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "ALGO6 needs the sparse forward pass, one road");
    if (a.touched && (a.sem != 1 || a.algo != 4 || !a.qmark || !a.qlist || !a.qcount ||
                      (size_t)a.G * a.Q > (size_t)0x7fffffff))
        return to_set_error(ctx, TO_ERR_INVALID, "touched-query mode: sem 1, ALGO4, scratch");
    if (a.touched)
        TO_CUDA(ctx, cudaMemsetAsync(a.qmark, 0, (size_t)a.G * a.Q, ctx->stream));
    if (a.qroad) TO_CUDA(ctx, cudaMemsetAsync(a.qroad, 0, (size_t)a.nr * sizeof(unsigned), ctx->stream));
    k_rov_terminal<<<pblocks, tpb, 0, ctx->stream>>>(a);
    TO_LAUNCHED(ctx);
    if (a.lblocks != (a.PT + kLsmChunk - 1) / kLsmChunk || (a.nr > 1 && a.P < kLsmMinPaths))
        return to_set_error(ctx, TO_ERR_INVALID, "regression chunks %d", a.lblocks);
    int fblocks = (int)(((size_t)a.G * (a.S + 1) * a.P + 255) / 256);
    if (fblocks > 4 * 152) fblocks = 4 * 152;
    for (int t = a.Y - 2; t > 0; --t) {
        to_prof_begin(ctx, "lsm_prepare");
        k_lsm_count<<<a.lblocks, kLsmChunk, 0, ctx->stream>>>(a, t);
        TO_LAUNCHED(ctx);
        k_lsm_scatter<<<a.lblocks, kLsmChunk, 0, ctx->stream>>>(a, t);
        TO_LAUNCHED(ctx);
        k_lsm_stats<<<(a.nr + kStatsWarps - 1) / kStatsWarps, kStatsWarps * 32, 0, ctx->stream>>>(
            a, t, a.lblocks);
        TO_LAUNCHED(ctx);
        k_lsm_norm<<<fblocks, 256, 0, ctx->stream>>>(a);
        TO_LAUNCHED(ctx);
        if (a.touched) {
            k_lsm_mark<<<(a.PT + 255) / 256, 256, 0, ctx->stream>>>(a, t);
            TO_LAUNCHED(ctx);
            k_lsm_list<<<(int)(((size_t)a.G * a.Q + 1023) / 1024), 1024, 0, ctx->stream>>>(a);
            TO_LAUNCHED(ctx);
        }
        to_prof_end(ctx);
        TO_TRY(knn_rov(ctx, a, t));      // kNN and the local linear regressions
        to_prof_begin(ctx, "rov_backward");
        k_rov_backward<<<pblocks, tpb, 0, ctx->stream>>>(a, t);
        to_prof_end(ctx);
        TO_LAUNCHED(ctx);
        // ALGO6: the year's value becomes the realised payoff of each path
        // re-simulated from year t under the regression-optimal controls
        if (a.algo == 6) TO_TRY(rov_resim_sparse(ctx, a, *csc, t));
    }
    k_rov_first<<<a.nr, 1024, 0, ctx->stream>>>(a);
    TO_LAUNCHED(ctx);
    return TO_OK;
}

}  // namespace to_k
