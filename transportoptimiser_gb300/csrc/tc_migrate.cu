// tc_migrate.cu - MTE population Monte Carlo with the migration step on the
// fifth-generation tensor cores (tcgen05, kind::tf32) in 3xTF32.
//
// Reference: mteKernel (include/gpuCode/SimulateGPU.cu:595-717): per path
// and year, growth-rate mean update, migration pop'[k] = sum_l M[k][l]
// pop[l], then logistic growth per patch.  The growth and noise arithmetic
// here is the SIMT kernel's (mte.cu); only the migration sum differs: it is
// D[k][p] = sum_l M[k][l] pop[p][l] on the tensor core with FP32 values split
// x = hi + lo (hi = x rounded to nearest-even TF32, 10 mantissa bits; lo =
// x - hi, exact in FP32) and
//     D = A_hi B_hi + A_hi B_lo + A_lo B_hi        (FP32 accumulation in TMEM)
// which recovers FP32-level accuracy: the dropped A_lo B_lo term is ~2^-22
// relative.  Rounding (not truncating) the split makes lo symmetric about
// zero, so that term and the tensor core's own truncation of lo leave no
// systematic bias to compound over 50 yearly steps (truncation biased the
// expected end population by 2e-5).  Results agree with the SIMT path to
// FP32 rounding, not bit for bit.
//
// Layout.  M-tiles of 128 destinations (TMEM lane = destination), N = a
// tile of TP paths (TMEM column = path), K = source patches in groups of 16.
// The matrix of each (road, species) is packed once per call into
// [tile][group] blocks of 128 x 16 FP32, hi then lo, each in the no-swizzle
// K-major core-matrix layout (k_tc_pack), and streamed every year through a
// shared-memory ring by 1-D bulk copies (cp.async.bulk, mbarrier
// complete_tx).  The populations (B operand, hi and lo) live in shared
// memory for all years; the epilogue reads D from TMEM, applies growth and
// writes the next year's B.  One thread issues copies and MMAs; every wait
// is bounded and reports TO_DEVERR_SPIN.
#include "to_internal.cuh"
#include "to_pop.cuh"
#include "to_tc.cuh"

namespace {

constexpr int KGRP = 16;                      // sources per ring stage (2 MMA k-steps)
constexpr int BLK = 128 * KGRP * 4;           // bytes of one hi or lo block
constexpr int STAGE = 2 * BLK;                // hi + lo
constexpr uint32_t LBO = 128, SBO_A = KGRP * 4 * 8;

// x rounded to the nearest TF32 value (ties to even); finite inputs
__device__ __forceinline__ float tf32_hi(float x) {
    const uint32_t u = __float_as_uint(x);
    return __uint_as_float((u + 0xFFFu + ((u >> 13) & 1u)) & 0xFFFFE000u);
}

__global__ void k_tc_pack(to_mte_args a, int MT, int KGN, float* __restrict__ packed) {
    const int rs = a.rs0 + blockIdx.y, blk = blockIdx.x;
    const int m = blk / KGN, g = blk - m * KGN;
    const int N = a.n_patches[rs], NP = a.npad;
    const float* M = a.mmm + ((size_t)rs * a.C + a.c_use) * NP * NP;
    float* dst = packed + ((size_t)rs * MT * KGN + blk) * (STAGE / 4);
    for (int e = threadIdx.x; e < 128 * KGRP; e += blockDim.x) {
        const int r = e / KGRP, j = e - r * KGRP;
        const int k = m * 128 + r, l = g * KGRP + j;
        const float v = (k < N && l < N) ? M[(size_t)k * NP + l] : 0.0f;
        const float hi = tf32_hi(v);
        const uint32_t off = to_tc::kmaj_off(r, j, KGRP * 4, 4) >> 2;
        dst[off] = hi;
        dst[BLK / 4 + off] = v - hi;
    }
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, void* mbar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 :: "r"(to_tc::smem_u32(mbar)), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(to_tc::smem_u32(dst)), "l"(src), "r"(bytes), "r"(to_tc::smem_u32(mbar))
                 : "memory");
}

struct TcShape {
    int MT, KGN, TP, nstage, tcols;
    size_t kb, smem;
};

// dynamic shared memory map
__host__ __device__ inline size_t off_ring() { return 0; }
__host__ __device__ inline size_t off_bhi(const TcShape& s) { return (size_t)s.nstage * STAGE; }
__host__ __device__ inline size_t off_blo(const TcShape& s) { return off_bhi(s) + (size_t)s.TP * s.kb; }
__host__ __device__ inline size_t off_gm(const TcShape& s) { return off_blo(s) + (size_t)s.TP * s.kb; }
__host__ __device__ inline size_t off_end(const TcShape& s) { return off_gm(s) + (size_t)s.TP * 4; }
__host__ __device__ inline size_t off_z(const TcShape& s) { return off_end(s) + (size_t)s.MT * 4 * s.TP * 4; }
__host__ __device__ inline size_t smem_total(const TcShape& s) { return off_z(s) + 4 * 128 * 4; }

template <int TCOLS>
__global__ void __launch_bounds__(128, 1)
k_mte_tc(to_mte_args a, TcShape sh, const float* __restrict__ packed, int* __restrict__ err) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ __align__(8) uint64_t full[4], empty[4], done;
    __shared__ uint32_t tslot;
    __shared__ int s_abort;
    const int MT = sh.MT, KGN = sh.KGN, TP = sh.TP, NS = sh.nstage;
    const int NCH = MT * KGN;
    const uint32_t KB = (uint32_t)sh.kb, SBO_B = KB * 8;
    unsigned char* ring = sm + off_ring();
    unsigned char* bhi = sm + off_bhi(sh);
    unsigned char* blo = sm + off_blo(sh);
    float* gm = reinterpret_cast<float*>(sm + off_gm(sh));
    float* endp = reinterpret_cast<float*>(sm + off_end(sh));
    float* zs = reinterpret_cast<float*>(sm + off_z(sh));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int rs = a.rs0 + blockIdx.y;
    const int road = rs / a.S, sp = rs - road * a.S;
    const int N = a.n_patches[rs], NP = a.npad;
    if (N > KGN * KGRP || N > MT * 128) {
        if (threadIdx.x == 0 && a.flags) atomicExch(a.flags, TO_DEVERR_PLAN);
        for (int q = threadIdx.x; q < TP; q += 128)
            if (blockIdx.x * TP + q < a.n_paths) a.end_pops[(size_t)rs * a.n_paths + blockIdx.x * TP + q] = NAN;
        return;
    }
    const float* ip = a.init_pops + (size_t)rs * NP;
    const float* cp = a.caps + (size_t)rs * NP;
    const float* sp8 = a.params + 8 * sp;
    const float p0 = sp8[0], p1 = sp8[1], p2 = sp8[2], p4 = sp8[4], p5 = sp8[5],
                p6 = sp8[6], p7 = sp8[7];
    const float sj2 = p5 * p5;
    const int N4 = (N + 3) & ~3;
    const uint32_t road_id = (uint32_t)(a.road0 + road);
    const int path0 = blockIdx.x * TP;
    const float* pk = packed + (size_t)rs * NCH * (STAGE / 4);

    // initial populations (every path the same), hi / lo split
    for (int q = tid; q < TP * KGN * KGRP; q += 128) {
        const int p = q / (KGN * KGRP), l = q - p * (KGN * KGRP);
        const float v = (l < N) ? ip[l] : 0.0f;
        const float hi = tf32_hi(v);
        const uint32_t off = to_tc::kmaj_off(p, l, (int)KB, 4);
        *reinterpret_cast<float*>(bhi + off) = hi;
        *reinterpret_cast<float*>(blo + off) = v - hi;
    }
    for (int q = tid; q < TP; q += 128) gm[q] = p0;
    float cap[4];
    for (int m = 0; m < 4; ++m) {
        const int k = m * 128 + tid;
        cap[m] = (m < MT && k < N) ? cp[k] : 1.0f;
    }
    if (tid == 0) {
        for (int s = 0; s < NS; ++s) { to_tc::mbar_init(&full[s], 1); to_tc::mbar_init(&empty[s], 1); }
        to_tc::mbar_init(&done, 1);
        s_abort = 0;
    }
    if (warp == 0) to_tc::tmem_alloc<TCOLS>(&tslot);
    to_tc::fence_async_smem();
    to_tc::fence_before_sync();
    __syncthreads();
    to_tc::fence_after_sync();
    const uint32_t tmem = tslot;
    const uint32_t id = to_tc::idesc(2, 128, TP);
    bool ok = true;
    uint32_t gi_base = 0;          // chunk counter across years (ring phases)
    if (a.fault_wait) {
        // test hook: a wait that nothing completes, before any copy or MMA
        // is issued, with no time allowed - the abort path below runs
        // (error word, TMEM freed) with nothing in flight
        const bool w = to_tc::mbar_wait_limit(&done, 0u, 0ull);
        if (__syncthreads_or(!w)) ok = false;
    }

    for (int t = 0; t < a.n_years && ok; ++t) {
        // growth-rate mean (SimulateGPU.cu:691-701), one thread per path
        for (int q = tid; q < TP; q += 128) {
            const uint32_t path = (uint32_t)(path0 + q);
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
        // ---- migration: one thread streams the matrix and issues the MMAs
        if (tid == 0 && ok) {
            auto load = [&](int i) -> bool {
                const uint32_t gi = gi_base + (uint32_t)i;
                const int s = (int)(gi % (uint32_t)NS);
                const uint32_t use = gi / (uint32_t)NS;
                if (use > 0 && !to_tc::mbar_wait(&empty[s], (use - 1) & 1u)) return false;
                bulk_load(ring + (size_t)s * STAGE, pk + (size_t)i * (STAGE / 4), STAGE, &full[s]);
                return true;
            };
            for (int i = 0; i < NS - 1 && i < NCH && ok; ++i) ok = load(i);
            for (int i = 0; i < NCH && ok; ++i) {
                if (i + NS - 1 < NCH) ok = load(i + NS - 1);
                if (!ok) break;
                const uint32_t gi = gi_base + (uint32_t)i;
                const int s = (int)(gi % (uint32_t)NS);
                if (!to_tc::mbar_wait(&full[s], (gi / (uint32_t)NS) & 1u)) { ok = false; break; }
                to_tc::fence_after_sync();
                const int m = i / KGN, g = i - m * KGN;
                const uint32_t d = tmem + (uint32_t)(m * TP);
                const uint32_t a_hi = to_tc::smem_u32(ring + (size_t)s * STAGE);
                const uint32_t a_lo = a_hi + BLK;
                const uint32_t b_hi = to_tc::smem_u32(bhi) + (uint32_t)g * (KGRP * 4 / 16) * LBO;
                const uint32_t b_lo = to_tc::smem_u32(blo) + (uint32_t)g * (KGRP * 4 / 16) * LBO;
#pragma unroll
                for (int ks = 0; ks < KGRP / 8; ++ks) {
                    const uint64_t ah = to_tc::sdesc(a_hi + 256 * ks, LBO, SBO_A);
                    const uint64_t al = to_tc::sdesc(a_lo + 256 * ks, LBO, SBO_A);
                    const uint64_t bh = to_tc::sdesc(b_hi + 256 * ks, LBO, SBO_B);
                    const uint64_t bl = to_tc::sdesc(b_lo + 256 * ks, LBO, SBO_B);
                    to_tc::mma_tf32(d, ah, bh, id, (g > 0 || ks > 0) ? 1u : 0u);
                    to_tc::mma_tf32(d, ah, bl, id, 1u);
                    to_tc::mma_tf32(d, al, bh, id, 1u);
                }
                to_tc::commit(&empty[s]);
            }
            to_tc::commit(&done);
            if (!ok) s_abort = 1;
        }
        gi_base += (uint32_t)NCH;
        // every thread: wait for this year's MMAs
        bool w = to_tc::mbar_wait(&done, (uint32_t)t & 1u);
        if (__syncthreads_or(!w) || s_abort) ok = false;
        to_tc::fence_after_sync();
        if (!ok) break;
        // ---- epilogue: growth on D, next year's B (hi / lo)
        const bool last = (t == a.n_years - 1);
        for (int m = 0; m < MT; ++m) {
            const int k = m * 128 + tid;
            const bool valid = k < N;
            const int kg = k >> 2;
            for (int p16 = 0; p16 < TP; p16 += 16) {
                float v[16];
                to_tc::tmem_ld16(to_tc::lane_addr(tmem + (uint32_t)(m * TP), warp, p16), v);
                float es[16];
#pragma unroll
                for (int p4 = 0; p4 < 16; p4 += 4) {
                    // lane i of each quad draws the 4 normals of path p4+i for
                    // the quad's 4 destinations; the quad exchanges them
                    float zz[4];
                    const uint32_t path = (uint32_t)(path0 + p16 + p4 + (lane & 3));
                    to_normal4(a.seed, TO_STREAM_GROWTH, road_id, path, t,
                               (uint32_t)((sp * N4) >> 2) + (uint32_t)kg, zz);
                    float* zw = zs + warp * 128;
#pragma unroll
                    for (int c = 0; c < 4; ++c) zw[lane * 4 + c] = zz[c];
                    __syncwarp();
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const int p = p16 + p4 + i;
                        const float z = zw[((lane & ~3) + i) * 4 + (k & 3)];
                        const float mv = v[p4 + i];
                        const float g = gm[p];
                        const float gr = fmaf(p7 * z, g, g);
                        const float c = cap[m];
                        float np = valid ? mv * (1.0f + gr * (c - mv) / c) : 0.0f;
                        if (k < KGN * KGRP) {       // B holds sources 0..KGN*16-1
                            const float hi = tf32_hi(np);
                            const uint32_t off = to_tc::kmaj_off(p, k, (int)KB, 4);
                            *reinterpret_cast<float*>(bhi + off) = hi;
                            *reinterpret_cast<float*>(blo + off) = np - hi;
                        }
                        es[p4 + i] = valid ? ((a.sem == 0) ? mv : np) : 0.0f;
                    }
                    __syncwarp();
                }
                if (last) {
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        float x = es[j];
                        for (int o = 16; o > 0; o >>= 1) x = x + __shfl_xor_sync(0xffffffffu, x, o);
                        if (lane == 0) endp[(m * 4 + warp) * TP + p16 + j] = x;
                    }
                }
            }
        }
        to_tc::fence_async_smem();
        to_tc::fence_before_sync();
        __syncthreads();
        to_tc::fence_after_sync();
    }
    if (ok) {
        for (int q = tid; q < TP; q += 128) {
            const int path = path0 + q;
            if (path >= a.n_paths) continue;
            float e = 0.0f;
            if (a.n_years == 0) {
                for (int l = 0; l < N; ++l) e = e + ip[l];
            } else {
                for (int i = 0; i < MT * 4; ++i) e = e + endp[i * TP + q];
            }
            a.end_pops[(size_t)rs * a.n_paths + path] = e;
        }
    } else if (tid == 0) {
        atomicExch(err, TO_DEVERR_SPIN);
    }
    to_tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) to_tc::tmem_free<TCOLS>(tmem);
}

bool pick_shape(int N, size_t smem_cap, TcShape& sh) {
    sh.MT = (N + 127) / 128;
    sh.KGN = (N + KGRP - 1) / KGRP;
    sh.kb = (size_t)sh.KGN * KGRP * 4;
    if (sh.MT > 4) return false;
    for (int tp : {128, 64, 32, 16}) {
        if (sh.MT * tp > 512) continue;
        for (int ns : {4, 3, 2}) {
            sh.TP = tp;
            sh.nstage = ns;
            sh.smem = smem_total(sh);
            if (sh.smem + 2048 <= smem_cap) {
                int cols = 32;
                while (cols < sh.MT * tp) cols <<= 1;
                sh.tcols = cols;
                return true;
            }
        }
    }
    return false;
}

template <int TC>
to_status launch_tc(to_ctx ctx, const to_mte_args& a, int n_rs, const TcShape& sh,
                    const float* packed) {
    TO_CUDA(ctx, cudaFuncSetAttribute(k_mte_tc<TC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sh.smem));
    dim3 grid((a.n_paths + sh.TP - 1) / sh.TP, n_rs);
    k_mte_tc<TC><<<grid, 128, sh.smem, ctx->stream>>>(a, sh, packed, ctx->d_flags);
    return TO_OK;
}

}  // namespace

namespace to_k {

to_status mte_tc(to_ctx ctx, to_mte_args a, int n_rs) {
    int maxN = a.npe > 0 ? a.npe : a.npad;
    if (!a.flags) a.flags = ctx->d_flags;
    if (ctx->fault == TO_FAULT_WAIT) { a.fault_wait = 1; ctx->fault = TO_FAULT_NONE; }
    TcShape sh;
    if (!pick_shape(maxN, ctx->smem_optin, sh))
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "tensor-core migration: %d patches", maxN);
    const size_t bytes = (size_t)n_rs * sh.MT * sh.KGN * STAGE;
    if (bytes > ctx->tc_cap) {
        if (ctx->tc_buf) {
            TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            TO_CUDA(ctx, cudaFree(ctx->tc_buf));
            ctx->tc_buf = nullptr;
            ctx->tc_cap = 0;
        }
        TO_CUDA(ctx, cudaMalloc(&ctx->tc_buf, bytes));
        ctx->tc_cap = bytes;
    }
    float* packed = reinterpret_cast<float*>(ctx->tc_buf);
    to_prof_begin(ctx, "tc_pack");
    k_tc_pack<<<dim3(sh.MT * sh.KGN, n_rs), 256, 0, ctx->stream>>>(a, sh.MT, sh.KGN, packed);
    to_prof_end(ctx);
    TO_LAUNCHED(ctx);
    to_prof_begin(ctx, "mte_tc");
    switch (sh.tcols) {
        case 32: TO_TRY(launch_tc<32>(ctx, a, n_rs, sh, packed)); break;
        case 64: TO_TRY(launch_tc<64>(ctx, a, n_rs, sh, packed)); break;
        case 128: TO_TRY(launch_tc<128>(ctx, a, n_rs, sh, packed)); break;
        case 256: TO_TRY(launch_tc<256>(ctx, a, n_rs, sh, packed)); break;
        default: TO_TRY(launch_tc<512>(ctx, a, n_rs, sh, packed)); break;
    }
    to_prof_end(ctx);
    TO_LAUNCHED(ctx);
    return TO_OK;
}

}  // namespace to_k
