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
#include "to_rov_dev.cuh"
#include "to_sparse.cuh"

namespace {

constexpr int kLanes = 32;

// One CTA per matrix (rs*C + c): row k of the destination-major matrix is
// destination k's column.  Entries > 0 in ascending origin order.  A warp
// per row reads it coalesced: a count pass, a CTA scan of the row counts,
// then a ballot-compaction pass.
__global__ void __launch_bounds__(1024)
k_pack_csc(const float* __restrict__ mmm, int NP, int C, const int* __restrict__ n_patches,
           int cap, int* __restrict__ ptr, uint16_t* __restrict__ idx, float* __restrict__ val,
           int* __restrict__ nnz, int mtx0) {
    const int mtx = mtx0 + blockIdx.x;
    const int rs = mtx / C;
    const int N = n_patches[rs];
    const float* M = mmm + (size_t)mtx * NP * NP;
    int* p = ptr + (size_t)mtx * (NP + 1);
    uint16_t* ix = idx + (size_t)mtx * cap;
    float* vv = val + (size_t)mtx * cap;
    __shared__ int s_cnt[1024 + 1];
    __shared__ int s_w[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    for (int k = warp; k < NP; k += nw) {
        int c = 0;
        if (k < N)
            for (int l0 = 0; l0 < N; l0 += 32) {
                const int l = l0 + lane;
                c += __popc(__ballot_sync(0xffffffffu, l < N && M[(size_t)k * NP + l] > 0.0f));
            }
        if (lane == 0) s_cnt[k] = c;
    }
    __syncthreads();
    // exclusive scan of s_cnt[0..NP) (NP <= 1024: one value per thread)
    const int v = threadIdx.x < NP ? s_cnt[threadIdx.x] : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_w[warp] = x;
    __syncthreads();
    int wb = 0, tot = 0;
    for (int w = 0; w < nw; ++w) { if (w < warp) wb += s_w[w]; tot += s_w[w]; }
    __syncthreads();
    if (threadIdx.x < NP) s_cnt[threadIdx.x] = wb + x - v;
    if (threadIdx.x == 0) { s_cnt[NP] = tot; nnz[mtx] = (tot <= cap) ? tot : -1; }
    __syncthreads();
    for (int k = threadIdx.x; k <= NP; k += blockDim.x) p[k] = s_cnt[k];
    if (tot > cap) return;
    for (int k = warp; k < N; k += nw) {
        int o = s_cnt[k];
        for (int l0 = 0; l0 < N; l0 += 32) {
            const int l = l0 + lane;
            const float m = (l < N) ? M[(size_t)k * NP + l] : 0.0f;
            const unsigned b = __ballot_sync(0xffffffffu, m > 0.0f);
            if (m > 0.0f) {
                const int q = o + __popc(b & lt);
                ix[q] = (uint16_t)l;
                vv[q] = m;
            }
            o += __popc(b);
        }
    }
}

__device__ __forceinline__ float grouped4(float a, float b, float c, float d) {
    return ((a + b) + c) + d;
}

// ---------------------------------------------------------------------------
// MTE (mteKernel :595-717) - grid (ceil(P/PW), RS), the (road, species) of
// grid row y taken from a.order when it is set (widest first, k_mte_order).
// A warp's groups of four destinations are dealt in snake order over the
// groups sorted by entries (warp w takes ranks w, 2W-1-w, 2W+w), at most
// MAXG a warp; the next year's populations wait in registers until every
// warp has read this year's, so one shared buffer suffices.  The growth
// mean's draws are made kGmChunk years at a time by the whole CTA, and
// every warp carries its lanes' growth means itself.  The values do not
// depend on which warp computes a group.
// ---------------------------------------------------------------------------
constexpr int kMaxG = 4;
constexpr int kGmChunk = 16;

template <int MAXG, int PPL>
__global__ void __launch_bounds__(1024, 1)
k_mte_sparse(to_mte_args a, to_csc csc) {
    // PPL paths per lane: lane owns paths lane + 32 i; every non-zero read
    // from shared memory serves all of them
    constexpr int PW = kLanes * PPL;                           // paths per CTA
    extern __shared__ __align__(16) unsigned char sm_raw[];
    const int NE = a.npe, NG = NE >> 2, NP = a.npad;
    const int rs = a.rs0 + (a.order ? a.order[blockIdx.y] : (int)blockIdx.y);
    const int road = rs / a.S, sp = rs - road * a.S;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, W = blockDim.x >> 5;
    const int mtx = rs * a.C + a.c_use;
    const int nnz = csc.nnz[mtx];
    if (nnz < 0 || nnz > csc.cap_smem || a.n_patches[rs] > NE) {
        // outside the shape this launch was planned for: flag, no result
        if (threadIdx.x == 0 && a.flags) atomicExch(a.flags, TO_DEVERR_PLAN);
        const int p = blockIdx.x * PW + (int)threadIdx.x;
        if (threadIdx.x < PW && p < a.n_paths) a.end_pops[(size_t)rs * a.n_paths + p] = NAN;
        return;
    }
    int2* cent = reinterpret_cast<int2*>(sm_raw);              // [cap_smem] (row byte offset, value)
    float* cur = reinterpret_cast<float*>(cent + csc.cap_smem);// [NE][PW]
    float* part = cur + (size_t)NE * PW;                       // [NG][PW]
    float2* capr = reinterpret_cast<float2*>(part + (size_t)NG * PW);  // [NE] capacity, 1/capacity
    float* xs = reinterpret_cast<float*>(capr + NE);           // [kGmChunk][3][PW] draws
    int* cptr = reinterpret_cast<int*>(xs + kGmChunk * 3 * PW);// [NE+1]
    int* order = cptr + NE + 1;                                // [NG] groups, widest first

    const int N = a.n_patches[rs];
    const int N4 = (N + 3) & ~3;
    // groups of this (road, species); the launch is shaped for the widest
    // model, and the groups past N4 would only ever hold zeros (no
    // non-zeros reach them, the growth of 0 is 0) so they are not visited.
    // Their totals are +0, which leaves a sum that started at +0 unchanged.
    const int NGr = N4 >> 2;
    const float* ip = a.init_pops + (size_t)rs * NP;
    const float* sp8 = a.params + 8 * sp;
    const float p0 = sp8[0], p1 = sp8[1], p2 = sp8[2], p4 = sp8[4], p5 = sp8[5],
                p6 = sp8[6], p7 = sp8[7];
    const float sj2 = p5 * p5;
    const uint32_t road_id = (uint32_t)(a.road0 + road);
    const int path0 = blockIdx.x * PW + lane;

    for (int q = threadIdx.x; q < NE * PW; q += blockDim.x) {
        int k = q / PW;
        cur[q] = (k < N) ? ip[k] : 0.0f;
    }
    for (int k = threadIdx.x; k < NE; k += blockDim.x) {
        const float cp = a.caps[(size_t)rs * NP + k];
        capr[k] = make_float2(cp, 1.0f / cp);
    }
    for (int k = threadIdx.x; k <= NE; k += blockDim.x)
        cptr[k] = csc.ptr[(size_t)mtx * (NP + 1) + (k <= NP ? k : NP)];
    for (int e = threadIdx.x; e < nnz; e += blockDim.x) {
        const int l = csc.idx[(size_t)mtx * csc.cap + e];
        cent[e] = make_int2(l * PW * (int)sizeof(float),
                            __float_as_int(csc.val[(size_t)mtx * csc.cap + e]));
    }
    __syncthreads();
    for (int gq = threadIdx.x; gq < NGr; gq += blockDim.x) {
        const int w = cptr[4 * gq + 4] - cptr[4 * gq];
        int rank = 0;
        for (int u = 0; u < NGr; ++u) {
            const int wu = cptr[4 * u + 4] - cptr[4 * u];
            rank += (wu > w) || (wu == w && u < gq);
        }
        order[rank] = gq;
    }
    float g[PPL];
#pragma unroll
    for (int i = 0; i < PPL; ++i) g[i] = p0;

    for (int t = 0; t < a.n_years; ++t) {
        if (t % kGmChunk == 0) {
            // the next years' growth-mean draws, one thread each: jump
            // indicator, Brownian term, jump factor minus one
            const int nc = min(kGmChunk, a.n_years - t);
            for (int q = threadIdx.x; q < nc * 3 * PW; q += blockDim.x) {
                const int yy = q / (3 * PW), r = q - yy * 3 * PW;
                const int which = r / PW, i = r - which * PW;
                const uint32_t path = (uint32_t)(blockIdx.x * PW + i);
                const int ty = t + yy;
                float v;
                if (which == 0) {
                    v = (to_uniform1(a.seed, TO_STREAM_SP_JUMP, road_id, path, ty, sp) < p6) ? 1.0f
                                                                                              : 0.0f;
                } else if (which == 1) {
                    v = to_normal1(a.seed, TO_STREAM_SP_BROWNIAN, road_id, path, ty, sp) * p2;
                } else {
                    const float zj = to_normal1(a.seed, TO_STREAM_SP_JUMPSIZE, road_id, path, ty, sp);
                    const float jsz = (a.sem == 0) ? (zj * sj2 - sj2 / 2.0f) : (zj * p5 - sj2 / 2.0f);
                    v = to_expf(jsz) - 1.0f;
                }
                xs[q] = v;
            }
            __syncthreads();
        }
        const float* xt = xs + (t % kGmChunk) * 3 * PW;
#pragma unroll
        for (int i = 0; i < PPL; ++i) {
            const int pi = lane + kLanes * i;
            const float jump = xt[pi], brown = xt[PW + pi], em1 = xt[2 * PW + pi];
            g[i] = g[i] + p4 * (p1 - g[i]) * a.dt + g[i] * brown + em1 * g[i] * jump;
        }
        const bool last = (t == a.n_years - 1);
        float nv[MAXG][4][PPL];
#pragma unroll
        for (int gi = 0; gi < MAXG; ++gi) {
            const int slot = gi * W + ((gi & 1) ? W - 1 - warp : warp);
            if (slot < NGr) {
                const int grp = order[slot];
                float z[PPL][4];
#pragma unroll
                for (int i = 0; i < PPL; ++i)
                    to_normal4(a.seed, TO_STREAM_GROWTH, road_id, (uint32_t)(path0 + kLanes * i), t,
                               (uint32_t)((sp * N4) >> 2) + grp, z[i]);
                float msum[PPL];            // grouped4 of the migrated values, in order
                // the group's column pointers: one 16-byte load and one word
                const int4 c4 = reinterpret_cast<const int4*>(cptr)[grp];
                const int cb[5] = {c4.x, c4.y, c4.z, c4.w, cptr[grp * 4 + 4]};
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int k = grp * 4 + j;
                    float acc[PPL];
#pragma unroll
                    for (int i = 0; i < PPL; ++i) acc[i] = 0.0f;
                    const int e1 = cb[j + 1];
#pragma unroll 2
                    for (int e = cb[j]; e < e1; ++e) {
                        const int2 ce = cent[e];
                        const float* row = reinterpret_cast<const float*>(
                            reinterpret_cast<const unsigned char*>(cur) + ce.x) + lane;
                        const float v = __int_as_float(ce.y);
#pragma unroll
                        for (int i = 0; i < PPL; ++i) acc[i] = fmaf(row[kLanes * i], v, acc[i]);
                    }
                    const float2 cr = capr[k];
#pragma unroll
                    for (int i = 0; i < PPL; ++i) {
                        msum[i] = (j == 0) ? acc[i] : msum[i] + acc[i];
                        float gr = fmaf(p7 * z[i][j], g[i], g[i]);
                        // the division as to_div_rcp: the same bits
                        nv[gi][j][i] = acc[i] * (1.0f + to_div_rcp(gr * (cr.x - acc[i]), cr.x, cr.y));
                    }
                }
                if (last)
#pragma unroll
                    for (int i = 0; i < PPL; ++i)
                        part[grp * PW + lane + kLanes * i] = msum[i];
            }
        }
        __syncthreads();
#pragma unroll
        for (int gi = 0; gi < MAXG; ++gi) {
            const int slot = gi * W + ((gi & 1) ? W - 1 - warp : warp);
            if (slot < NGr) {
                const int grp = order[slot];
#pragma unroll
                for (int j = 0; j < 4; ++j)
#pragma unroll
                    for (int i = 0; i < PPL; ++i)
                        cur[(grp * 4 + j) * PW + lane + kLanes * i] = nv[gi][j][i];
            }
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < PW; i += blockDim.x) {
        const int path = blockIdx.x * PW + i;
        if (path >= a.n_paths) continue;
        float e = 0.0f;
        if (a.n_years > 0 && a.sem == 0) {
            for (int grp = 0; grp < NGr; ++grp) e = e + part[grp * PW + i];
        } else {
            for (int grp = 0; grp < NGr; ++grp) {
                const float* v = cur + (size_t)grp * 4 * PW + i;
                e = e + grouped4(v[0], v[PW], v[2 * PW], v[3 * PW]);
            }
        }
        a.end_pops[(size_t)rs * a.n_paths + path] = e;
    }
}

// The launch order of the MTE's (road, species): by descending packed
// entries of the used control (ties by index), so the widest models start
// first and the last wave holds the narrow ones.  One CTA.
__global__ void __launch_bounds__(1024) k_mte_order(int n_rs, int rs0, int C, int c_use,
                                                    const int* __restrict__ nnz, int* order) {
    for (int i = threadIdx.x; i < n_rs; i += blockDim.x) {
        const int w = nnz[(size_t)(rs0 + i) * C + c_use];
        int rank = 0;
        for (int j = 0; j < n_rs; ++j) {
            const int wj = nnz[(size_t)(rs0 + j) * C + c_use];
            rank += (wj > w) || (wj == w && j < i);
        }
        order[rank] = i;
    }
}

// ---------------------------------------------------------------------------
// Union of the C <= 3 controls' packed columns of one (road, species): one
// CTA; a thread per destination merges its C ascending origin lists (count,
// CTA scan, write).
// ---------------------------------------------------------------------------
__device__ __forceinline__ int union_step(const int* b, const int* e, const uint16_t* const* ix,
                                          int C, int* pos) {
    int lo = 0x7fffffff;
    for (int c = 0; c < C; ++c)
        if (pos[c] < e[c] && (int)ix[c][pos[c]] < lo) lo = ix[c][pos[c]];
    return lo;
}

__global__ void __launch_bounds__(256)
k_union_csc(int NP, int C, const int* __restrict__ n_patches, to_csc csc) {
    const int rs = blockIdx.x;
    const int N = n_patches[rs];
    __shared__ int s_tmp[32];
    int* up = csc.uptr + (size_t)rs * (NP + 1);
    const uint16_t* ix[3];
    const float* vv[3];
    bool ok = true;
    for (int c = 0; c < C; ++c) {
        const size_t mtx = (size_t)rs * C + c;
        ix[c] = csc.idx + mtx * csc.cap;
        vv[c] = csc.val + mtx * csc.cap;
        ok = ok && csc.nnz[mtx] >= 0;
    }
    if (!ok) {                                    // a control above its capacity
        if (threadIdx.x == 0) csc.unnz[rs] = -1;
        return;
    }
    // pass 1: union size of each column; a thread takes a run of columns
    const int chunk = (NP + (int)blockDim.x - 1) / (int)blockDim.x;
    const int k0 = (int)threadIdx.x * chunk, k1 = min(NP, k0 + chunk);
    int cnt = 0;
    for (int k = k0; k < k1; ++k) {
        int b[3], e[3], pos[3];
        for (int c = 0; c < C; ++c) {
            const int* p = csc.ptr + ((size_t)rs * C + c) * (NP + 1);
            b[c] = pos[c] = k < N ? p[k] : 0;
            e[c] = k < N ? p[k + 1] : 0;
        }
        int n = 0;
        for (;;) {
            const int lo = union_step(b, e, ix, C, pos);
            if (lo == 0x7fffffff) break;
            for (int c = 0; c < C; ++c) if (pos[c] < e[c] && (int)ix[c][pos[c]] == lo) ++pos[c];
            ++n;
        }
        up[k] = n;
        cnt += n;
    }
    // CTA exclusive scan of the per-thread totals
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int x = cnt;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_tmp[warp] = x;
    __syncthreads();
    int base = 0, total = 0;
    for (int w = 0; w < nw; ++w) { if (w < warp) base += s_tmp[w]; total += s_tmp[w]; }
    base += x - cnt;
    for (int k = k0; k < k1; ++k) { const int n = up[k]; up[k] = base; base += n; }
    if (threadIdx.x == 0) {
        up[NP] = total;
        csc.unnz[rs] = total <= csc.ucap ? total : -1;
    }
    if (total > csc.ucap) return;
    // pass 2: the entries
    int4* out = csc.uent + (size_t)rs * csc.ucap;
    for (int k = k0; k < k1; ++k) {
        int b[3], e[3], pos[3];
        for (int c = 0; c < C; ++c) {
            const int* p = csc.ptr + ((size_t)rs * C + c) * (NP + 1);
            b[c] = pos[c] = k < N ? p[k] : 0;
            e[c] = k < N ? p[k + 1] : 0;
        }
        int q = up[k];
        for (;;) {
            const int lo = union_step(b, e, ix, C, pos);
            if (lo == 0x7fffffff) break;
            float v[3] = {0.0f, 0.0f, 0.0f};
            for (int c = 0; c < C; ++c)
                if (pos[c] < e[c] && (int)ix[c][pos[c]] == lo) { v[c] = vv[c][pos[c]]; ++pos[c]; }
            out[q++] = make_int4(lo, __float_as_int(v[0]), __float_as_int(v[1]),
                                 __float_as_int(v[2]));
        }
    }
}

// ---------------------------------------------------------------------------
// ROV forward paths on the union columns (C <= 3 controls) - grid (ceil(P/32),
// roads), up to 32 warps.  As k_rov_forward_sparse, but
//  * each non-zero of destination k is one 16-byte shared load {row byte
//    offset, value of control 0, 1, 2} that serves every control's
//    migration (three FMA chains, each in ascending origin order with exact
//    zero terms where a control has no entry);
//  * a warp takes the year's groups of four destinations from a shared
//    counter, widest group first, and writes the new populations to the
//    second buffer, so that no warp waits at the year's barrier for a fixed
//    share of wide columns;
//  * the growth mean's three draws per path are drawn for kGmChunk years at
//    a time by the whole CTA, and every warp carries the lane's growth mean
//    forward itself (same expression, same bits) - two barriers a year.
// The values equal k_rov_forward_sparse's bit for bit: every group's
// arithmetic and every sum's order is unchanged, only who computes it.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024, 1)
k_rov_forward_union(to_rov_args a, to_csc csc) {
    extern __shared__ __align__(16) unsigned char sm_raw[];
    const int NE = a.ne, NG = NE >> 2, C = a.C, Y = a.Y, P = a.P;
    const size_t PT = (size_t)a.PT;
    const int rd = blockIdx.y;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, W = blockDim.x >> 5;
    const int path = blockIdx.x * kLanes + lane;
    const size_t gp = (size_t)rd * P + path;
    int4* ue = reinterpret_cast<int4*>(sm_raw);                    // [ucap_smem]
    float* bufA = reinterpret_cast<float*>(ue + csc.ucap_smem);    // [NE][32]
    float* bufB = bufA + (size_t)NE * kLanes;                      // [NE][32]
    float* part = bufB + (size_t)NE * kLanes;                      // [C+1][NG][32]
    float2* capr = reinterpret_cast<float2*>(part + (size_t)(C + 1) * NG * kLanes);  // [NE]
    float* xs = reinterpret_cast<float*>(capr + NE);               // [kGmChunk][3][32]
    float* tot = xs + kGmChunk * 3 * kLanes;                       // [32]
    float* ntot = tot + kLanes;                                    // [32]
    int* uptr = reinterpret_cast<int*>(ntot + kLanes);             // [NE+1]
    int* order = uptr + NE + 1;                                    // [NG]
    int* grab = order + NG;                                        // [2]
    const uint32_t road = (uint32_t)a.road_ids[rd];

    for (int s = 0; s < a.S; ++s) {
        const int rs = rd * a.S + s;
        const int N = a.n_patches[rs];
        const int N4 = (N + 3) & ~3;
        const int NGr = N4 >> 2;
        const float* sp = a.params + 8 * s;
        const float* ip = a.init_pops + (size_t)rs * a.np;
        const int nu = csc.unnz[rs];
        if (nu < 0 || nu > csc.ucap_smem || N > NE) {
            // outside the shape this launch was planned for: flag, no result
            if (threadIdx.x == 0 && a.flags) atomicExch(a.flags, TO_DEVERR_PLAN);
            if (warp == 0 && path < P)
                for (int t = 0; t <= Y; ++t)
                    a.totalPops[((size_t)s * (Y + 1) + t) * PT + gp] = NAN;
            continue;
        }
        __syncthreads();
        float* cur = bufA;
        float* nxt = bufB;
        for (int q = threadIdx.x; q < NE * kLanes; q += blockDim.x) {
            const int k = q / kLanes;
            cur[q] = (k < N) ? ip[k] : 0.0f;
            nxt[q] = 0.0f;
        }
        for (int k = threadIdx.x; k < NE; k += blockDim.x) {
            const float cp = a.caps[(size_t)rs * a.np + k];
            capr[k] = make_float2(cp, 1.0f / cp);          // capacity, its reciprocal
        }
        for (int k = threadIdx.x; k <= NE; k += blockDim.x)
            uptr[k] = csc.uptr[(size_t)rs * (a.np + 1) + (k <= a.np ? k : a.np)];
        for (int e = threadIdx.x; e < nu; e += blockDim.x) {
            int4 v = csc.uent[(size_t)rs * csc.ucap + e];
            v.x *= kLanes * (int)sizeof(float);                    // origin -> row byte offset
            ue[e] = v;
        }
        if (threadIdx.x < 2) grab[threadIdx.x] = 0;
        __syncthreads();
        // the groups in descending order of entries (ties: lower group first)
        for (int gq = threadIdx.x; gq < NGr; gq += blockDim.x) {
            const int w = uptr[4 * gq + 4] - uptr[4 * gq];
            int rank = 0;
            for (int u = 0; u < NGr; ++u) {
                const int wu = uptr[4 * u + 4] - uptr[4 * u];
                rank += (wu > w) || (wu == w && u < gq);
            }
            order[rank] = gq;
        }
        if (warp == 0) {
            float tt = 0.0f;
            for (int grp = 0; grp < NGr; ++grp) {
                const float* v = cur + (size_t)grp * 4 * kLanes + lane;
                tt = tt + grouped4(v[0], v[kLanes], v[2 * kLanes], v[3 * kLanes]);
            }
            tot[lane] = tt;
            if (path < P) a.totalPops[((size_t)s * (Y + 1)) * PT + gp] = tt;
        }
        const float jp = (a.sem == 0) ? sp[5] : sp[6];
        const float s5 = sp[5] * sp[5];
        float g = sp[0];                                           // this lane's growth mean
        for (int t = 0; t < Y; ++t) {
            if (t % kGmChunk == 0) {
                // the next years' growth-mean draws, one thread each
                const int nc = min(kGmChunk, Y - t);
                for (int q = threadIdx.x; q < nc * 3 * kLanes; q += blockDim.x) {
                    const int yy = q / (3 * kLanes), r = q - yy * 3 * kLanes;
                    const int which = r >> 5, i = r & 31;
                    const uint32_t pth = (uint32_t)(blockIdx.x * kLanes + i);
                    const int ty = t + yy;
                    float v;
                    if (which == 0) {
                        v = (to_uniform1(a.seed, TO_STREAM_SP_JUMP, road, pth, ty, s) < jp) ? 1.0f
                                                                                             : 0.0f;
                    } else if (which == 1) {
                        v = to_normal1(a.seed, TO_STREAM_SP_BROWNIAN, road, pth, ty, s) * sp[2];
                    } else {
                        const float zj = to_normal1(a.seed, TO_STREAM_SP_JUMPSIZE, road, pth, ty, s);
                        const float jsz = (a.sem == 0) ? (zj * s5 - s5 / 2.0f)
                                                       : (zj * sp[5] - s5 / 2.0f);
                        v = to_expf(jsz) - 1.0f;
                    }
                    xs[q] = v;
                }
                __syncthreads();
            }
            {
                const float* xt = xs + (t % kGmChunk) * 3 * kLanes;
                const float jump = xt[lane], brown = xt[kLanes + lane], em1 = xt[2 * kLanes + lane];
                g = g + sp[4] * (sp[1] - g) * a.dt + g * brown + em1 * g * jump;
            }
            if (warp == 0 && a.gmY && path < P) a.gmY[((size_t)t * a.S + s) * P + path] = g;
            const int my_c = (path < P) ? a.controls[(size_t)t * PT + gp] : 0;
            if (a.popsY) {
                for (int q = threadIdx.x; q < NE * kLanes; q += blockDim.x) {
                    const int pth = blockIdx.x * kLanes + (q & (kLanes - 1));
                    if (pth < P)
                        a.popsY[(((size_t)t * a.S + s) * NE + (q >> 5)) * P + pth] = cur[q];
                }
            }
            const unsigned char* curb = reinterpret_cast<const unsigned char*>(cur) + lane * 4;
            int* gc = grab + (t & 1);
            for (;;) {
                int i = 0;
                if (lane == 0) i = atomicAdd(gc, 1);
                i = __shfl_sync(0xffffffffu, i, 0);
                if (i >= NGr) break;
                const int grp = order[i];
                float z[4];
                to_normal4(a.seed, TO_STREAM_GROWTH, road, path, t,
                           (uint32_t)((s * N4) >> 2) + grp, z);
                float m0[4], m1[4], m2[4], np4[4];
                // the group's column pointers: one 16-byte load and one word
                const int4 u4 = reinterpret_cast<const int4*>(uptr)[grp];
                const int ub[5] = {u4.x, u4.y, u4.z, u4.w, uptr[grp * 4 + 4]};
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int k = grp * 4 + j;
                    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f;
                    const int e1 = ub[j + 1];
#pragma unroll 4
                    for (int e = ub[j]; e < e1; ++e) {
                        const int4 en = ue[e];
                        const float x = *reinterpret_cast<const float*>(curb + en.x);
                        a0 = fmaf(x, __int_as_float(en.y), a0);
                        a1 = fmaf(x, __int_as_float(en.z), a1);
                        a2 = fmaf(x, __int_as_float(en.w), a2);
                    }
                    m0[j] = a0; m1[j] = a1; m2[j] = a2;
                    const float mv = (my_c == 0) ? a0 : ((my_c == 1) ? a1 : a2);
                    const float gr = (a.sem == 0) ? g + z[j] * sp[7] : fmaf(sp[7] * z[j], g, g);
                    const float2 cr = capr[k];
                    // the divisions as to_div_rcp: the same bits
                    const float v = (a.sem == 0)
                        ? mv * (1.0f + to_div_rcp(to_div_rcp(gr * (cr.x - mv), cr.x, cr.y), 100.0f,
                                                  0.01f))
                        : fmaxf(mv * (1.0f + to_div_rcp(gr * (cr.x - mv), cr.x, cr.y)), 0.0f);
                    nxt[k * kLanes + lane] = v;
                    np4[j] = v;
                }
                part[((size_t)0 * NG + grp) * kLanes + lane] = grouped4(m0[0], m0[1], m0[2], m0[3]);
                if (C > 1)
                    part[((size_t)1 * NG + grp) * kLanes + lane] = grouped4(m1[0], m1[1], m1[2], m1[3]);
                if (C > 2)
                    part[((size_t)2 * NG + grp) * kLanes + lane] = grouped4(m2[0], m2[1], m2[2], m2[3]);
                part[((size_t)C * NG + grp) * kLanes + lane] = grouped4(np4[0], np4[1], np4[2], np4[3]);
            }
            // last used in the year before; two barriers before the next year
            if (threadIdx.x == 0) grab[(t + 1) & 1] = 0;
            __syncthreads();
            for (int c = warp; c <= C; c += W) {
                float tt = 0.0f;
#pragma unroll 8
                for (int grp = 0; grp < NGr; ++grp)
                    tt = tt + part[((size_t)c * NG + grp) * kLanes + lane];
                if (path < P) {
                    if (c < C) a.aars[(((size_t)s * C + c) * Y + t) * PT + gp] = tt / tot[lane];
                    else a.totalPops[((size_t)s * (Y + 1) + t + 1) * PT + gp] = tt;
                }
                if (c == C) ntot[lane] = tt;
            }
            __syncthreads();
            if (warp == 0) tot[lane] = ntot[lane];
            float* tmp = cur;
            cur = nxt;
            nxt = tmp;
        }
    }
}

// ---------------------------------------------------------------------------
// ROV forward paths (forwardPathKernel :789-956) - grid ceil(P/32)
// ---------------------------------------------------------------------------
template <int CMAX, int MAXG>
__global__ void __launch_bounds__(1024, 1)
k_rov_forward_sparse(to_rov_args a, to_csc csc) {
    extern __shared__ unsigned char sm_raw[];
    // grid (path tiles of a road, roads): lane = path of road blockIdx.y
    const int NE = a.ne, NG = NE >> 2, NP = a.np, C = a.C, Y = a.Y, P = a.P;
    const size_t PT = (size_t)a.PT;
    const int rd = blockIdx.y;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, W = blockDim.x >> 5;
    const int path = blockIdx.x * kLanes + lane;
    const size_t gp = (size_t)rd * P + path;                    // path of the batch
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
    const uint32_t road = (uint32_t)a.road_ids[rd];

    for (int s = 0; s < a.S; ++s) {
        const int rs = rd * a.S + s;
        const int N = a.n_patches[rs];
        const int N4 = (N + 3) & ~3;
        const int NGr = N4 >> 2;           // this road's groups (see k_mte_sparse)
        const float* sp = a.params + 8 * s;
        const float* ip = a.init_pops + (size_t)rs * NP;
        __syncthreads();
        for (int q = threadIdx.x; q < NE * kLanes; q += blockDim.x) {
            int k = q / kLanes;
            cur[q] = (k < N) ? ip[k] : 0.0f;
        }
        for (int k = threadIdx.x; k < NE; k += blockDim.x) capv[k] = a.caps[(size_t)rs * NP + k];
        for (int c = 0; c < C; ++c) {
            const int mtx = rs * C + c;
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
            for (int grp = 0; grp < NGr; ++grp) {
                const float* v = cur + (size_t)grp * 4 * kLanes + lane;
                tt = tt + grouped4(v[0], v[kLanes], v[2 * kLanes], v[3 * kLanes]);
            }
            tot[lane] = tt;
            gm[lane] = sp[0];
            if (path < P) a.totalPops[((size_t)s * (Y + 1)) * PT + gp] = tt;
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
                ctl[lane] = (path < P) ? a.controls[(size_t)t * PT + gp] : 0;
                if (a.gmY && path < P) a.gmY[((size_t)t * a.S + s) * P + path] = gm[lane];
            }
            __syncthreads();
            if (a.popsY) {
                // ALGO6 restarts paths from here: the year's starting patch
                // populations, 32 consecutive paths per row
                for (int q = threadIdx.x; q < NE * kLanes; q += blockDim.x) {
                    const int pth = blockIdx.x * kLanes + (q & (kLanes - 1));
                    if (pth < P)
                        a.popsY[(((size_t)t * a.S + s) * NE + (q >> 5)) * P + pth] = cur[q];
                }
            }
            const float g = gm[lane];
            const int my_c = ctl[lane];
            float nv[MAXG][4];
#pragma unroll
            for (int gi = 0; gi < MAXG; ++gi) {
                const int grp = warp + gi * W;
                if (grp < NGr) {
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
                for (int grp = 0; grp < NGr; ++grp)
                    tt = tt + part[((size_t)c * NG + grp) * kLanes + lane];
                if (path < P) {
                    if (c < C) a.aars[(((size_t)s * C + c) * Y + t) * PT + gp] = tt / tot[lane];
                    else a.totalPops[((size_t)s * (Y + 1) + t + 1) * PT + gp] = tt;
                }
                if (c == C) ntot[lane] = tt;
            }
            __syncthreads();                   // every warp has read tot
            if (warp == 0) tot[lane] = ntot[lane];
#pragma unroll
            for (int gi = 0; gi < MAXG; ++gi) {
                const int grp = warp + gi * W;
                if (grp < NGr) {
#pragma unroll
                    for (int j = 0; j < 4; ++j) cur[(grp * 4 + j) * kLanes + lane] = nv[gi][j];
                }
            }
            __syncthreads();
        }
    }
}


// ---------------------------------------------------------------------------
// ALGO6 path re-simulation (optimalForwardPaths :1199-2206, as its comments
// describe it).  Grid ceil(P/32): a CTA re-simulates 32 paths (lane = path)
// from year t0 to the horizon with every species together, since each
// year's control depends on all species' states:
//   A. all warps: every (species, control) migration of this year's
//      populations into shared memory (CSC, ascending origins, as forward);
//   B. warps (s, c): the grouped total and the adjusted population
//      tot * (total / tot), the forward pass's arithmetic;
//   C. warp 0: the decision (regression of the year, or the terminal rule
//      in the last year) and the realised payoff flows[c] * profit,
//      discounted by (1 + r dt / 100) per year;
//   D. all warps: growth of the chosen control's migrated populations with
//      the forward pass's noise and growth mean (stored by it);
//   E. warps s: the new totals.
// The year-t0 value replaces condExp[t0] and the year-t0 control optCont[t0].
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024, 1)
k_rov_resim_sparse(to_rov_args a, to_csc csc, int t0) {
    extern __shared__ unsigned char sm_raw[];
    const int NE = a.ne, NG = NE >> 2, NP = a.np, C = a.C, S = a.S, Y = a.Y, P = a.P;
    const int SC = S * C;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, W = blockDim.x >> 5;
    const int path = blockIdx.x * kLanes + lane;
    float* cur = reinterpret_cast<float*>(sm_raw);                  // [S][NE][32]
    float* mig = cur + (size_t)S * NE * kLanes;                     // [S][C][NE][32]
    float* capv = mig + (size_t)SC * NE * kLanes;                   // [S][NE]
    float* tot = capv + (size_t)S * NE;                             // [S][32]
    float* adj = tot + (size_t)S * kLanes;                          // [S][C][32]
    int* ctl = reinterpret_cast<int*>(adj + (size_t)SC * kLanes);   // [32]
    int* cptr = ctl + kLanes;                                       // [S*C][NE+1]
    float* cval = reinterpret_cast<float*>(cptr + (size_t)SC * (NE + 1));  // [S*C][cap_smem]
    uint16_t* cidx = reinterpret_cast<uint16_t*>(cval + (size_t)SC * csc.cap_smem);
    const uint32_t road = (uint32_t)a.road;

    for (int q = threadIdx.x; q < S * NE * kLanes; q += blockDim.x) {
        const int sk = q >> 5, pth = blockIdx.x * kLanes + (q & (kLanes - 1));
        const int s = sk / NE, k = sk - s * NE;
        cur[q] = (pth < P) ? a.popsY[(((size_t)t0 * S + s) * NE + k) * P + pth] : 0.0f;
    }
    for (int q = threadIdx.x; q < S * NE; q += blockDim.x) {
        const int s = q / NE, k = q - s * NE;
        capv[q] = a.caps[(size_t)s * NP + k];
    }
    for (int m = 0; m < SC; ++m) {
        const int nnz = csc.nnz[m];
        for (int k = threadIdx.x; k <= NE; k += blockDim.x)
            cptr[m * (NE + 1) + k] = csc.ptr[(size_t)m * (NP + 1) + (k <= NP ? k : NP)];
        for (int e = threadIdx.x; e < nnz; e += blockDim.x) {
            cval[(size_t)m * csc.cap_smem + e] = csc.val[(size_t)m * csc.cap + e];
            cidx[(size_t)m * csc.cap_smem + e] = csc.idx[(size_t)m * csc.cap + e];
        }
    }
    __syncthreads();
    for (int s = warp; s < S; s += W) {
        float tt = 0.0f;
        for (int grp = 0; grp < NG; ++grp) {
            const float* v = cur + ((size_t)s * NE + grp * 4) * kLanes + lane;
            tt = tt + grouped4(v[0], v[kLanes], v[2 * kLanes], v[3 * kLanes]);
        }
        tot[s * kLanes + lane] = tt;
    }
    const float disc = 1.0f + a.rrr * a.dt / 100.0f;
    float val = 0.0f, df = 1.0f;        // warp 0: realised value, discount factor
    int c0 = 0;
    for (int u = t0; u < Y; ++u) {
        __syncthreads();
        // A. migrations of every (species, control)
        for (int s = 0; s < S; ++s) {
            const float* cs = cur + (size_t)s * NE * kLanes + lane;
            for (int grp = warp; grp < NG; grp += W) {
                for (int c = 0; c < C; ++c) {
                    const int m = s * C + c;
                    const int* cp = cptr + m * (NE + 1);
                    const float* cv = cval + (size_t)m * csc.cap_smem;
                    const uint16_t* ci = cidx + (size_t)m * csc.cap_smem;
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const int k = grp * 4 + j;
                        float acc = 0.0f;
                        for (int e = cp[k]; e < cp[k + 1]; ++e)
                            acc = fmaf(cs[(int)ci[e] * kLanes], cv[e], acc);
                        mig[((size_t)m * NE + k) * kLanes + lane] = acc;
                    }
                }
            }
        }
        __syncthreads();
        // B. adjusted populations tot * (migrated total / tot)
        for (int m = warp; m < SC; m += W) {
            const int s = m / C;
            float tt = 0.0f;
            for (int grp = 0; grp < NG; ++grp) {
                const float* v = mig + ((size_t)m * NE + grp * 4) * kLanes + lane;
                tt = tt + grouped4(v[0], v[kLanes], v[2 * kLanes], v[3 * kLanes]);
            }
            const float ts = tot[s * kLanes + lane];
            adj[m * kLanes + lane] = ts * (tt / ts);
        }
        __syncthreads();
        // C. the decision and the realised payoff
        if (warp == 0) {
            int bc = 0;
            if (path < P) {
                float state[TO_ROV_MAXC * (TO_LSM_MAXD - 1) + 1];
                for (int c = 0; c < C; ++c)
                    for (int s = 0; s < S; ++s) state[c * S + s] = adj[(s * C + c) * kLanes + lane];
                const float prof = to_rovd::unit_profit(a, path, u, Y + 1, Y + 1);
                state[S * C] = prof;
                float best;
                if (u == Y - 1) to_rovd::decide_terminal(a, state, best, bc);
                else to_rovd::decide_interior(a, u, 0, state, best, bc);
                val = val + (a.flows[bc] * prof) * df;
                df = df / disc;
            }
            if (u == t0) c0 = bc;
            ctl[lane] = bc;
        }
        __syncthreads();
        if (u == Y - 1) break;
        // D. growth of the chosen control's migrated populations
        const int cu = ctl[lane];
        for (int s = 0; s < S; ++s) {
            const float* sp = a.params + 8 * s;
            const int N4 = (a.n_patches[s] + 3) & ~3;
            const float g = (path < P) ? a.gmY[((size_t)u * S + s) * P + path] : 0.0f;
            for (int grp = warp; grp < NG; grp += W) {
                float z[4];
                to_normal4(a.seed, TO_STREAM_GROWTH, road, path, u,
                           (uint32_t)((s * N4) >> 2) + grp, z);
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int k = grp * 4 + j;
                    const float mv = mig[(((size_t)s * C + cu) * NE + k) * kLanes + lane];
                    const float gr = (a.sem == 0) ? g + z[j] * sp[7] : fmaf(sp[7] * z[j], g, g);
                    const float cpk = capv[s * NE + k];
                    cur[((size_t)s * NE + k) * kLanes + lane] =
                        (a.sem == 0) ? mv * (1.0f + gr * (cpk - mv) / cpk / 100.0f)
                                     : fmaxf(mv * (1.0f + gr * (cpk - mv) / cpk), 0.0f);
                }
            }
        }
        __syncthreads();
        // E. totals of the new populations
        for (int s = warp; s < S; s += W) {
            float tt = 0.0f;
            for (int grp = 0; grp < NG; ++grp) {
                const float* v = cur + ((size_t)s * NE + grp * 4) * kLanes + lane;
                tt = tt + grouped4(v[0], v[kLanes], v[2 * kLanes], v[3 * kLanes]);
            }
            tot[s * kLanes + lane] = tt;
        }
    }
    if (warp == 0 && path < P) {
        a.condExp[(size_t)t0 * P + path] = val;
        a.optCont[(size_t)t0 * P + path] = c0;
    }
}

}  // namespace

namespace to_k {

to_status pack_csc(to_ctx ctx, const float* mmm, int NP, int C, const int* n_patches,
                   int n_rs, to_csc& csc, int rs0) {
    if (NP > 1024) return to_set_error(ctx, TO_ERR_UNSUPPORTED, "patches %d", NP);
    to_prof_begin(ctx, "pack_csc");
    k_pack_csc<<<n_rs * C, 1024, 0, ctx->stream>>>(mmm, NP, C, n_patches, csc.cap,
                                                 csc.ptr, csc.idx, csc.val, csc.nnz, rs0 * C);
    to_prof_end(ctx);
    TO_LAUNCHED(ctx);
    return TO_OK;
}

// paths per lane of the MTE kernel: two when the tile fits (every non-zero
// read then serves two paths), else one
static int mte_ppl(int NE, int cap_smem, size_t smem_cap);

size_t mte_sparse_smem_ppl(int NE, int cap_smem, int ppl) {
    const int maxg = ppl == 1 ? kMaxG : 3;      // 32 warps of maxg groups of four
    if (NE > 32 * maxg * 4) return ~size_t(0);
    const int NG = NE / 4, PW = kLanes * ppl;
    return (size_t)cap_smem * 8 + (size_t)(NE * PW + NG * PW + 2 * NE + kGmChunk * 3 * PW) * 4 +
           (size_t)(NE + 1 + NG) * 4 + 16;
}

size_t mte_sparse_smem(int NE, int cap_smem) { return mte_sparse_smem_ppl(NE, cap_smem, 1); }

static int mte_ppl(int NE, int cap_smem, size_t smem_cap) {
    return mte_sparse_smem_ppl(NE, cap_smem, 2) <= smem_cap ? 2 : 1;
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
    if (csc.cap_smem & 1)       // the 8-byte entries must leave the column pointers 16-byte aligned
        return to_set_error(ctx, TO_ERR_INVALID, "packed capacity %d is odd", csc.cap_smem);
    const int ppl = (a.n_paths > kLanes) ? mte_ppl(NE, csc.cap_smem, ctx->smem_optin) : 1;
    size_t smem = mte_sparse_smem_ppl(NE, csc.cap_smem, ppl);
    if (smem > ctx->smem_optin)
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "sparse MTE needs %zu B", smem);
    int warps = warps_for(NE, 4);
    if ((NE / 4 + warps - 1) / warps > kMaxG)
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "patches %d", NE);
    const int PW = kLanes * ppl;
    dim3 grid((a.n_paths + PW - 1) / PW, n_rs);
    if (a.order_buf && n_rs > 1) {
        k_mte_order<<<1, 1024, 0, ctx->stream>>>(n_rs, a.rs0, a.C, a.c_use, csc.nnz, a.order_buf);
        TO_LAUNCHED(ctx);
        a.order = a.order_buf;
    }
    to_prof_begin(ctx, "mte_sparse");
    if (ppl == 2) {
        // 32 warps of at most three groups (NE <= 384): a shorter chain of
        // groups per warp between the year's barriers than 24 warps of four,
        // and within 64 registers a thread
        TO_CUDA(ctx, cudaFuncSetAttribute(k_mte_sparse<3, 2>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_mte_sparse<3, 2><<<grid, 1024, smem, ctx->stream>>>(a, csc);
    } else {
        TO_CUDA(ctx, cudaFuncSetAttribute(k_mte_sparse<kMaxG, 1>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_mte_sparse<kMaxG, 1><<<grid, warps * 32, smem, ctx->stream>>>(a, csc);
    }
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

size_t rov_union_smem(int NE, int C, int ucap_smem) {
    if (NE > 32 * kMaxG * 4 || C > 3) return ~size_t(0);
    const int NG = NE / 4;
    return (size_t)ucap_smem * 16 +
           (size_t)(2 * NE * kLanes + (C + 1) * NG * kLanes + 2 * NE + kGmChunk * 3 * kLanes +
                    2 * kLanes) * 4 +
           (size_t)(NE + 1 + NG + 2) * 4 + 16;
}

to_status union_csc(to_ctx ctx, int NP, int C, const int* n_patches, int n_rs, to_csc& csc) {
    if (C > 3 || !csc.uent || !csc.uptr || !csc.unnz)
        return to_set_error(ctx, TO_ERR_INVALID, "union form: %d controls", C);
    k_union_csc<<<n_rs, 256, 0, ctx->stream>>>(NP, C, n_patches, csc);
    TO_LAUNCHED(ctx);
    return TO_OK;
}

to_status rov_forward_sparse(to_ctx ctx, const to_rov_args& a, to_csc csc) {
    if (csc.uent && a.C <= 3) {
        const size_t smem = rov_union_smem(a.ne, a.C, csc.ucap_smem);
        if (smem > ctx->smem_optin)
            return to_set_error(ctx, TO_ERR_UNSUPPORTED, "union ROV needs %zu B", smem);
        const dim3 blocks((a.P + kLanes - 1) / kLanes, a.nr);
        const int NG = a.ne / 4;
        const int warps = NG < 32 ? (NG > 4 ? NG : 4) : 32;
        to_prof_begin(ctx, "rov_forward_sparse");
        TO_CUDA(ctx, cudaFuncSetAttribute(k_rov_forward_union,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_rov_forward_union<<<blocks, warps * 32, smem, ctx->stream>>>(a, csc);
        to_prof_end(ctx);
        TO_LAUNCHED(ctx);
        return TO_OK;
    }
    size_t smem = rov_sparse_smem(a.ne, a.C, csc.cap_smem);
    if (smem > ctx->smem_optin)
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "sparse ROV needs %zu B", smem);
    int warps = warps_for(a.ne, a.C + 1 > 4 ? a.C + 1 : 4);
    if ((a.ne / 4 + warps - 1) / warps > kMaxG)
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "patches %d", a.ne);
    const dim3 blocks((a.P + kLanes - 1) / kLanes, a.nr);
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


size_t rov_resim_smem(int NE, int S, int C, int cap_smem) {
    const size_t SC = (size_t)S * C;
    return ((size_t)S * NE * kLanes + SC * NE * kLanes + (size_t)S * NE + (size_t)S * kLanes +
            SC * kLanes) * 4 + kLanes * 4 + SC * (NE + 1) * 4 + SC * cap_smem * 6 + 16;
}

to_status rov_resim_sparse(to_ctx ctx, const to_rov_args& a, to_csc csc, int t0) {
    const size_t smem = rov_resim_smem(a.ne, a.S, a.C, csc.cap_smem);
    if (smem > ctx->smem_optin)
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "ALGO6 re-simulation needs %zu B", smem);
    const int blocks = (a.P + kLanes - 1) / kLanes;
    to_prof_begin(ctx, "rov_resim");
    TO_CUDA(ctx, cudaFuncSetAttribute(k_rov_resim_sparse,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_rov_resim_sparse<<<blocks, 1024, smem, ctx->stream>>>(a, csc, t0);
    to_prof_end(ctx);
    TO_LAUNCHED(ctx);
    return TO_OK;
}

}  // namespace to_k
