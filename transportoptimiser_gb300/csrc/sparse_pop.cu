// sparse_pop.cu - population Monte Carlo with the migration matrices in
// compressed-column form, resident in shared memory.
//
// The reference multiplies each path's population vector by a CSC matrix
// (dense2Sparse, SimulateGPU.cu:5973-5996; mteKernel :628-635;
// forwardPathKernel :871-922), one thread per path, reading strided global
// memory.  The matrices are very sparse (local migration: 2-5% non-zero,
// ~8 per column on the benchmark grids), so a dense (paths x N)(N x N)
// product would spend >95% of its work on zeros.  Here:
//   * k_pack_csc packs every (road, species, control) matrix once;
//   * a CTA owns 32 paths (lane = path) and keeps their populations
//     ([patch][lane], conflict-free) and the CSC lists in shared memory for
//     all years; its warps split the destination patches in groups of four,
//     so one Philox call gives the four growth normals a lane needs;
//   * each destination sums its non-zeros in ascending origin order with
//     explicit FMAs - the same chain as the dense form (skipped terms are
//     exact zeros), so results stay bit-identical to the oracle;
//   * patch totals use the fixed grouped order ((v0+v1)+v2)+v3, groups
//     ascending.
#include <cstring>

#include "to_internal.cuh"
#include "to_pop.cuh"
#include "to_rov.cuh"
#include "to_sparse.cuh"

namespace {

constexpr int kLanes = 32;

// One CTA per matrix (rs*C + c): row k of the destination-major matrix is
// destination k's column.  Entries > 0 in ascending origin order.
__global__ void k_pack_csc(const float* __restrict__ mmm, int NP, int C,
                           const int* __restrict__ n_patches, int cap,
                           int* __restrict__ ptr, uint16_t* __restrict__ idx,
                           float* __restrict__ val, int* __restrict__ nnz) {
    const int mtx = blockIdx.x;
    const int rs = mtx / C;
    const int N = n_patches[rs];
    const float* M = mmm + (size_t)mtx * NP * NP;
    int* p = ptr + (size_t)mtx * (NP + 1);
    uint16_t* ix = idx + (size_t)mtx * cap;
    float* vv = val + (size_t)mtx * cap;
    __shared__ int s_cnt[1024 + 1];
    __shared__ int s_tot;
    for (int k = threadIdx.x; k <= NP; k += blockDim.x) s_cnt[k] = 0;
    __syncthreads();
    for (int k = threadIdx.x; k < NP; k += blockDim.x) {
        int c = 0;
        if (k < N)
            for (int l = 0; l < N; ++l) c += M[(size_t)k * NP + l] > 0.0f;
        s_cnt[k + 1] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 0; k < NP; ++k) s_cnt[k + 1] += s_cnt[k];
        s_tot = s_cnt[NP];
        nnz[mtx] = (s_tot <= cap) ? s_tot : -1;
    }
    __syncthreads();
    for (int k = threadIdx.x; k <= NP; k += blockDim.x) p[k] = s_cnt[k];
    if (s_tot > cap) return;
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
        int o = s_cnt[k];
        for (int l = 0; l < N; ++l) {
            float m = M[(size_t)k * NP + l];
            if (m > 0.0f) { ix[o] = (uint16_t)l; vv[o] = m; ++o; }
        }
    }
}

__device__ __forceinline__ float grouped4(float a, float b, float c, float d) {
    return ((a + b) + c) + d;
}

// ---------------------------------------------------------------------------
// MTE (mteKernel :595-717) - grid (ceil(P/32), RS).  Warp w owns groups
// w, w+W, ... (at most MAXG); the next year's populations wait in registers
// until every warp has read this year's, so one shared buffer suffices.
// ---------------------------------------------------------------------------
constexpr int kMaxG = 4;

template <int MAXG>
__global__ void __launch_bounds__(1024, 1)
k_mte_sparse(to_mte_args a, to_csc csc) {
    extern __shared__ unsigned char sm_raw[];
    const int NE = a.npe, NG = NE >> 2, NP = a.npad;
    const int rs = blockIdx.y;
    const int road = rs / a.S, sp = rs - road * a.S;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, W = blockDim.x >> 5;
    const int mtx = rs * a.C + a.c_use;
    const int nnz = csc.nnz[mtx];
    if (nnz < 0 || nnz > csc.cap_smem || a.n_patches[rs] > NE) {
        // outside the shape this launch was planned for: flag, no result
        if (threadIdx.x == 0 && a.flags) atomicExch(a.flags, TO_DEVERR_PLAN);
        const int p = blockIdx.x * kLanes + (int)threadIdx.x;
        if (threadIdx.x < kLanes && p < a.n_paths) a.end_pops[(size_t)rs * a.n_paths + p] = NAN;
        return;
    }
    float* cur = reinterpret_cast<float*>(sm_raw);             // [NE][32]
    float* part = cur + (size_t)NE * kLanes;                   // [NG][32]
    float* capv = part + (size_t)NG * kLanes;                  // [NE]
    float* gm = capv + NE;                                     // [32]
    int* cptr = reinterpret_cast<int*>(gm + kLanes);           // [NE+1]
    float* cval = reinterpret_cast<float*>(cptr + NE + 1);     // [cap_smem]
    uint16_t* cidx = reinterpret_cast<uint16_t*>(cval + csc.cap_smem);   // [cap_smem]

    const int N = a.n_patches[rs];
    const int N4 = (N + 3) & ~3;
    const float* ip = a.init_pops + (size_t)rs * NP;
    const float* sp8 = a.params + 8 * sp;
    const float p0 = sp8[0], p1 = sp8[1], p2 = sp8[2], p4 = sp8[4], p5 = sp8[5],
                p6 = sp8[6], p7 = sp8[7];
    const float sj2 = p5 * p5;
    const uint32_t road_id = (uint32_t)(a.road0 + road);
    const int path = blockIdx.x * kLanes + lane;

    for (int q = threadIdx.x; q < NE * kLanes; q += blockDim.x) {
        int k = q / kLanes;
        cur[q] = (k < N) ? ip[k] : 0.0f;
    }
    for (int k = threadIdx.x; k < NE; k += blockDim.x)
        capv[k] = a.caps[(size_t)rs * NP + k];
    for (int k = threadIdx.x; k <= NE; k += blockDim.x)
        cptr[k] = csc.ptr[(size_t)mtx * (NP + 1) + (k <= NP ? k : NP)];
    for (int e = threadIdx.x; e < nnz; e += blockDim.x) {
        cval[e] = csc.val[(size_t)mtx * csc.cap + e];
        cidx[e] = csc.idx[(size_t)mtx * csc.cap + e];
    }
    if (warp == 0) gm[lane] = p0;
    __syncthreads();

    for (int t = 0; t < a.n_years; ++t) {
        if (warp == 0) {
            float uj = to_uniform1(a.seed, TO_STREAM_SP_JUMP, road_id, path, t, sp);
            float zb = to_normal1(a.seed, TO_STREAM_SP_BROWNIAN, road_id, path, t, sp);
            float zj = to_normal1(a.seed, TO_STREAM_SP_JUMPSIZE, road_id, path, t, sp);
            float jump = (uj < p6) ? 1.0f : 0.0f;
            float brown = zb * p2;
            float jsz = (a.sem == 0) ? (zj * sj2 - sj2 / 2.0f) : (zj * p5 - sj2 / 2.0f);
            float g = gm[lane];
            gm[lane] = g + p4 * (p1 - g) * a.dt + g * brown + (to_expf(jsz) - 1.0f) * g * jump;
        }
        __syncthreads();
        const float g = gm[lane];
        const bool last = (t == a.n_years - 1);
        float nv[MAXG][4];
#pragma unroll
        for (int gi = 0; gi < MAXG; ++gi) {
            const int grp = warp + gi * W;
            if (grp < NG) {
            float z[4];
            to_normal4(a.seed, TO_STREAM_GROWTH, road_id, path, t,
                       (uint32_t)((sp * N4) >> 2) + grp, z);
            float m4[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                int k = grp * 4 + j;
                float acc = 0.0f;
                for (int e = cptr[k]; e < cptr[k + 1]; ++e)
                    acc = fmaf(cur[(int)cidx[e] * kLanes + lane], cval[e], acc);
                m4[j] = acc;
                float gr = fmaf(p7 * z[j], g, g);
                float c = capv[k];
                nv[gi][j] = acc * (1.0f + gr * (c - acc) / c);
            }
            if (last) part[grp * kLanes + lane] = grouped4(m4[0], m4[1], m4[2], m4[3]);
            }
        }
        __syncthreads();
#pragma unroll
        for (int gi = 0; gi < MAXG; ++gi) {
            const int grp = warp + gi * W;
            if (grp < NG) {
#pragma unroll
                for (int j = 0; j < 4; ++j) cur[(grp * 4 + j) * kLanes + lane] = nv[gi][j];
            }
        }
    }
    __syncthreads();
    if (warp == 0 && path < a.n_paths) {
        float e = 0.0f;
        if (a.n_years > 0 && a.sem == 0) {
            for (int grp = 0; grp < NG; ++grp) e = e + part[grp * kLanes + lane];
        } else {
            for (int grp = 0; grp < NG; ++grp) {
                const float* v = cur + (size_t)grp * 4 * kLanes + lane;
                e = e + grouped4(v[0], v[kLanes], v[2 * kLanes], v[3 * kLanes]);
            }
        }
        a.end_pops[(size_t)rs * a.n_paths + path] = e;
    }
}

// ---------------------------------------------------------------------------
// ROV forward paths (forwardPathKernel :789-956) - grid ceil(P/32)
// ---------------------------------------------------------------------------
template <int CMAX, int MAXG>
__global__ void __launch_bounds__(1024, 1)
k_rov_forward_sparse(to_rov_args a, to_csc csc) {
    extern __shared__ unsigned char sm_raw[];
    const int NE = a.ne, NG = NE >> 2, NP = a.np, C = a.C, Y = a.Y, P = a.P;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, W = blockDim.x >> 5;
    const int path = blockIdx.x * kLanes + lane;
    float* cur = reinterpret_cast<float*>(sm_raw);                 // [NE][32]
    float* part = cur + (size_t)NE * kLanes;                       // [C+1][NG][32]
    float* capv = part + (size_t)(C + 1) * NG * kLanes;            // [NE]
    float* gm = capv + NE;                                         // [32]
    float* tot = gm + kLanes;                                      // [32]
    float* ntot = tot + kLanes;                                    // [32]
    int* ctl = reinterpret_cast<int*>(ntot + kLanes);              // [32]
    int* cptr = ctl + kLanes;                                      // [C][NE+1]
    float* cval = reinterpret_cast<float*>(cptr + (size_t)C * (NE + 1));  // [C][cap_smem]
    uint16_t* cidx = reinterpret_cast<uint16_t*>(cval + (size_t)C * csc.cap_smem);
    const uint32_t road = (uint32_t)a.road;

    for (int s = 0; s < a.S; ++s) {
        const int N = a.n_patches[s];
        const int N4 = (N + 3) & ~3;
        const float* sp = a.params + 8 * s;
        const float* ip = a.init_pops + (size_t)s * NP;
        __syncthreads();
        for (int q = threadIdx.x; q < NE * kLanes; q += blockDim.x) {
            int k = q / kLanes;
            cur[q] = (k < N) ? ip[k] : 0.0f;
        }
        for (int k = threadIdx.x; k < NE; k += blockDim.x) capv[k] = a.caps[(size_t)s * NP + k];
        for (int c = 0; c < C; ++c) {
            const int mtx = s * C + c;
            const int nnz = csc.nnz[mtx];
            for (int k = threadIdx.x; k <= NE; k += blockDim.x)
                cptr[c * (NE + 1) + k] = csc.ptr[(size_t)mtx * (NP + 1) + (k <= NP ? k : NP)];
            for (int e = threadIdx.x; e < nnz; e += blockDim.x) {
                cval[(size_t)c * csc.cap_smem + e] = csc.val[(size_t)mtx * csc.cap + e];
                cidx[(size_t)c * csc.cap_smem + e] = csc.idx[(size_t)mtx * csc.cap + e];
            }
        }
        __syncthreads();
        if (warp == 0) {
            float tt = 0.0f;
            for (int grp = 0; grp < NG; ++grp) {
                const float* v = cur + (size_t)grp * 4 * kLanes + lane;
                tt = tt + grouped4(v[0], v[kLanes], v[2 * kLanes], v[3 * kLanes]);
            }
            tot[lane] = tt;
            gm[lane] = sp[0];
            if (path < P) a.totalPops[((size_t)s * (Y + 1)) * P + path] = tt;
        }
        __syncthreads();
        for (int t = 0; t < Y; ++t) {
            if (warp == 0) {
                float uj = to_uniform1(a.seed, TO_STREAM_SP_JUMP, road, path, t, s);
                float zb = to_normal1(a.seed, TO_STREAM_SP_BROWNIAN, road, path, t, s);
                float zj = to_normal1(a.seed, TO_STREAM_SP_JUMPSIZE, road, path, t, s);
                float jp = (a.sem == 0) ? sp[5] : sp[6];
                float jump = (uj < jp) ? 1.0f : 0.0f;
                float brown = zb * sp[2];
                float s5 = sp[5] * sp[5];
                float jsz = (a.sem == 0) ? (zj * s5 - s5 / 2.0f) : (zj * sp[5] - s5 / 2.0f);
                float g = gm[lane];
                gm[lane] = g + sp[4] * (sp[1] - g) * a.dt + g * brown
                           + (to_expf(jsz) - 1.0f) * g * jump;
                ctl[lane] = (path < P) ? a.controls[(size_t)t * P + path] : 0;
            }
            __syncthreads();
            const float g = gm[lane];
            const int my_c = ctl[lane];
            float nv[MAXG][4];
#pragma unroll
            for (int gi = 0; gi < MAXG; ++gi) {
                const int grp = warp + gi * W;
                if (grp < NG) {
                float z[4];
                to_normal4(a.seed, TO_STREAM_GROWTH, road, path, t,
                           (uint32_t)((s * N4) >> 2) + grp, z);
                float mc[CMAX][4];
                float np4[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    int k = grp * 4 + j;
                    float mv = 0.0f;
#pragma unroll
                    for (int c = 0; c < CMAX; ++c) {
                        if (c >= C) break;
                        const int* cp = cptr + c * (NE + 1);
                        const float* cv = cval + (size_t)c * csc.cap_smem;
                        const uint16_t* ci = cidx + (size_t)c * csc.cap_smem;
                        float acc = 0.0f;
                        for (int e = cp[k]; e < cp[k + 1]; ++e)
                            acc = fmaf(cur[(int)ci[e] * kLanes + lane], cv[e], acc);
                        mc[c][j] = acc;
                        if (c == my_c) mv = acc;
                    }
                    float gr = (a.sem == 0) ? g + z[j] * sp[7] : fmaf(sp[7] * z[j], g, g);
                    float cpk = capv[k];
                    float v = (a.sem == 0) ? mv * (1.0f + gr * (cpk - mv) / cpk / 100.0f)
                                           : fmaxf(mv * (1.0f + gr * (cpk - mv) / cpk), 0.0f);
                    nv[gi][j] = v;
                    np4[j] = v;
                }
#pragma unroll
                for (int c = 0; c < CMAX; ++c) {
                    if (c >= C) break;
                    part[((size_t)c * NG + grp) * kLanes + lane] =
                        grouped4(mc[c][0], mc[c][1], mc[c][2], mc[c][3]);
                }
                part[((size_t)C * NG + grp) * kLanes + lane] =
                    grouped4(np4[0], np4[1], np4[2], np4[3]);
                }
            }
            __syncthreads();
            // totals: warp c sums control c's AAR numerator, warp C the new
            // populations (groups ascending)
            for (int c = warp; c <= C; c += W) {
                float tt = 0.0f;
                for (int grp = 0; grp < NG; ++grp)
                    tt = tt + part[((size_t)c * NG + grp) * kLanes + lane];
                if (path < P) {
                    if (c < C) a.aars[(((size_t)s * C + c) * Y + t) * P + path] = tt / tot[lane];
                    else a.totalPops[((size_t)s * (Y + 1) + t + 1) * P + path] = tt;
                }
                if (c == C) ntot[lane] = tt;
            }
            if (warp == 0) tot[lane] = 0.0f;   // replaced below, after the barrier
            __syncthreads();
            if (warp == 0) tot[lane] = ntot[lane];
#pragma unroll
            for (int gi = 0; gi < MAXG; ++gi) {
                const int grp = warp + gi * W;
                if (grp < NG) {
#pragma unroll
                    for (int j = 0; j < 4; ++j) cur[(grp * 4 + j) * kLanes + lane] = nv[gi][j];
                }
            }
            __syncthreads();
        }
    }
}

}  // namespace

namespace to_k {

to_status pack_csc(to_ctx ctx, const float* mmm, int NP, int C, const int* n_patches,
                   int n_rs, to_csc& csc) {
    if (NP > 1024) return to_set_error(ctx, TO_ERR_UNSUPPORTED, "patches %d", NP);
    k_pack_csc<<<n_rs * C, 256, 0, ctx->stream>>>(mmm, NP, C, n_patches, csc.cap,
                                                 csc.ptr, csc.idx, csc.val, csc.nnz);
    TO_LAUNCHED(ctx);
    return TO_OK;
}

size_t mte_sparse_smem(int NE, int cap_smem) {
    if (NE > 32 * kMaxG * 4) return ~size_t(0);
    int NG = NE / 4;
    return (size_t)(NE * kLanes + NG * kLanes + NE + kLanes) * 4 + (size_t)(NE + 1) * 4 +
           (size_t)cap_smem * 4 + (size_t)cap_smem * 2 + 16;
}

// warps per CTA: enough that no warp owns more than kMaxG groups of four
// (32 warps at most, so NE <= 512 for the sparse kernels)
static int warps_for(int NE, int min_warps) {
    int NG = NE / 4;
    int w = (NG + kMaxG - 1) / kMaxG;
    if (w < min_warps) w = min_warps;
    if (w > 32) w = 32;
    return w;
}

to_status mte_sparse(to_ctx ctx, to_mte_args a, int n_rs, to_csc csc) {
    if (a.npe <= 0) a.npe = a.npad;
    if (!a.flags) a.flags = ctx->d_flags;
    const int NE = a.npe;
    size_t smem = mte_sparse_smem(NE, csc.cap_smem);
    if (smem > ctx->smem_optin)
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "sparse MTE needs %zu B", smem);
    TO_CUDA(ctx, cudaFuncSetAttribute(k_mte_sparse<kMaxG>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int warps = warps_for(NE, 4);
    if ((NE / 4 + warps - 1) / warps > kMaxG)
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "patches %d", NE);
    dim3 grid((a.n_paths + kLanes - 1) / kLanes, n_rs);
    to_prof_begin(ctx, "mte_sparse");
    k_mte_sparse<kMaxG><<<grid, warps * 32, smem, ctx->stream>>>(a, csc);
    to_prof_end(ctx);
    TO_LAUNCHED(ctx);
    return TO_OK;
}

size_t rov_sparse_smem(int NE, int C, int cap_smem) {
    if (NE > 32 * kMaxG * 4 || C + 1 > 32) return ~size_t(0);
    int NG = NE / 4;
    return (size_t)(NE * kLanes + (C + 1) * NG * kLanes + NE + 4 * kLanes) * 4 +
           (size_t)C * (NE + 1) * 4 + (size_t)C * cap_smem * 6 + 16;
}

to_status rov_forward_sparse(to_ctx ctx, const to_rov_args& a, to_csc csc) {
    size_t smem = rov_sparse_smem(a.ne, a.C, csc.cap_smem);
    if (smem > ctx->smem_optin)
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "sparse ROV needs %zu B", smem);
    int warps = warps_for(a.ne, a.C + 1 > 4 ? a.C + 1 : 4);
    if ((a.ne / 4 + warps - 1) / warps > kMaxG)
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "patches %d", a.ne);
    const int blocks = (a.P + kLanes - 1) / kLanes;
    to_prof_begin(ctx, "rov_forward_sparse");
    if (a.C <= 3) {
        TO_CUDA(ctx, cudaFuncSetAttribute(k_rov_forward_sparse<3, kMaxG>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_rov_forward_sparse<3, kMaxG><<<blocks, warps * 32, smem, ctx->stream>>>(a, csc);
    } else {
        TO_CUDA(ctx, cudaFuncSetAttribute(k_rov_forward_sparse<TO_ROV_MAXC, kMaxG>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_rov_forward_sparse<TO_ROV_MAXC, kMaxG><<<blocks, warps * 32, smem, ctx->stream>>>(a, csc);
    }
    to_prof_end(ctx);
    TO_LAUNCHED(ctx);
    return TO_OK;
}

}  // namespace to_k
