// mlp.cu - learned surrogate of the road-evaluation outputs: an MLP
// 16 -> 128 -> 128 -> 3 (ReLU), trained and evaluated with this library's
// own kernels.  The reference has no learned surrogate (its GA fitness uses
// the local-linear grid surrogates, SimulateGPU.cu:5533-5917); this is the
// learned alternative used for GA screening, with the plain Monte Carlo as
// the fallback and the measure of its error.
//
// One CTA owns a tile of 128 rows (TMEM lane = row) and runs the whole
// forward and, for training, the whole backward pass on it:
//   F1  H1 = X W1^T            tcgen05 kind::f16, M=128 N=128 K=16
//   F2  H2 = H1 W2^T           M=128 N=128 K=128
//   L3  Y = H2 W3^T + b3       SIMT (3 outputs)
//   B2  dH1 = dH2 W2           M=128 (rows) N=128 K=128
//   G2  dW2 = dH2^T H1         M=128 (units) N=128 K=128 (rows)
//   G1  dW1 = dH1^T X          M=128 N=16 K=128
// Operands are BF16 in shared memory (K-major core-matrix tiles written by
// the threads, transposed copies where a GEMM contracts over rows),
// accumulators FP32 in TMEM.  Rounding points (every value that feeds an
// MMA is rounded to BF16 once; biases, ReLU, layer 3 and all reductions in
// FP32) are restated by the oracle.  Each tile writes its gradient partial;
// k_mlp_adam sums the partials in tile order (deterministic) and applies
// Adam to the FP32 master parameters.
#include <cuda_bf16.h>

#include <cmath>
#include <vector>

#include "to_internal.cuh"
#include "to_tc.cuh"

namespace {

constexpr int IN = TO_MLP_IN, HID = TO_MLP_HID, OUT = TO_MLP_OUT;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + HID * IN, OFF_W2 = OFF_B1 + HID,
              OFF_B2 = OFF_W2 + HID * HID, OFF_W3 = OFF_B2 + HID, OFF_B3 = OFF_W3 + OUT * HID,
              NPARAM = OFF_B3 + OUT;
static_assert(NPARAM == TO_MLP_NPARAM, "parameter layout");
constexpr int PSTRIDE = (NPARAM + 3) & ~3;           // per-tile partial stride (16-byte rows)

// shared memory map (bytes)
constexpr int KB_IN = IN * 2, KB_HID = HID * 2;      // K bytes per row of the bf16 tiles
constexpr int S_X = 0;                               // X   [128 rows][16]
constexpr int S_W1 = S_X + 128 * KB_IN;              // W1  [128 units][16]
constexpr int S_XT = S_W1 + 128 * KB_IN;             // X^T [16][128 rows]
constexpr int S_A = S_XT + IN * KB_HID;              // H1 [row][unit] -> dH2 [row][unit] -> dH1^T [unit][row]
constexpr int S_B = S_A + 128 * KB_HID;              // W2 [out][in] -> H2 (row-major bf16)
constexpr int S_W2T = S_B + 128 * KB_HID;            // W2^T [in][out]
constexpr int S_H1T = S_W2T + 128 * KB_HID;          // H1^T [unit][row]
constexpr int S_D2T = S_H1T + 128 * KB_HID;          // dH2^T [unit][row]
constexpr int S_F = S_D2T + 128 * KB_HID;            // fp32: W3, b1, b2, b3, dY, loss
constexpr int F_W3 = 0, F_B1 = F_W3 + OUT * HID, F_B2 = F_B1 + HID, F_B3 = F_B2 + HID,
              F_DY = F_B3 + 4, F_L = F_DY + 128 * OUT, F_END = F_L + 128;
constexpr int SMEM_BYTES = S_F + F_END * 4;

constexpr uint32_t SBO_IN = KB_IN * 8, SBO_HID = KB_HID * 8, LBO = 128;

__device__ __forceinline__ float bf(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }
__device__ __forceinline__ unsigned short bfbits(float x) {
    return __bfloat16_as_ushort(__float2bfloat16_rn(x));
}
__device__ __forceinline__ void st_bf16(unsigned char* base, uint32_t off, float x) {
    *reinterpret_cast<unsigned short*>(base + off) = bfbits(x);
}
__device__ __forceinline__ float ld_bf16(const unsigned char* base, uint32_t off) {
    return __bfloat162float(__ushort_as_bfloat16(*reinterpret_cast<const unsigned short*>(base + off)));
}
// 8 consecutive K elements of one row as one 16-byte store
__device__ __forceinline__ void st_bf16x8(unsigned char* base, uint32_t off, const float* v) {
    uint4 q;
    q.x = bfbits(v[0]) | ((uint32_t)bfbits(v[1]) << 16);
    q.y = bfbits(v[2]) | ((uint32_t)bfbits(v[3]) << 16);
    q.z = bfbits(v[4]) | ((uint32_t)bfbits(v[5]) << 16);
    q.w = bfbits(v[6]) | ((uint32_t)bfbits(v[7]) << 16);
    *reinterpret_cast<uint4*>(base + off) = q;
}

// issue a K = 16*steps chain of MMAs into tmem_d (one elected thread)
__device__ __forceinline__ void mma_chain(uint32_t tmem_d, const unsigned char* a, uint32_t sbo_a,
                                          const unsigned char* b, uint32_t sbo_b, uint32_t id,
                                          int steps) {
    for (int s = 0; s < steps; ++s)
        to_tc::mma_bf16(tmem_d, to_tc::sdesc(to_tc::smem_u32(a + 256 * s), LBO, sbo_a),
                        to_tc::sdesc(to_tc::smem_u32(b + 256 * s), LBO, sbo_b), id, s > 0);
}

// CTA-wide wait on the MMA barrier; false (all threads) if any timed out
__device__ __forceinline__ bool wait_mma(uint64_t* mbar, uint32_t& phase) {
    bool ok = to_tc::mbar_wait(mbar, phase);
    phase ^= 1u;
    ok = !__syncthreads_or(!ok);
    to_tc::fence_after_sync();
    return ok;
}

__device__ __forceinline__ void publish_smem() {
    to_tc::fence_async_smem();
    to_tc::fence_before_sync();
    __syncthreads();
    to_tc::fence_after_sync();
}

// rows: optional row index list (training order); t/part/loss only when BWD
template <bool BWD>
__global__ void __launch_bounds__(128, 1)
k_mlp(const float* __restrict__ params, int n, const int* __restrict__ rows,
      const float* __restrict__ x, const float* __restrict__ t, float inv_count,
      float* __restrict__ y_out, float* __restrict__ part, double* __restrict__ loss_part,
      int* __restrict__ err) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tslot;
    float* f = reinterpret_cast<float*>(sm + S_F);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int r0 = blockIdx.x * 128;
    const int gr = r0 + tid;
    const bool valid = gr < n;
    const int src = valid ? (rows ? rows[gr] : gr) : 0;

    // ---- stage parameters (bf16 operand tiles, fp32 for the SIMT parts)
    for (int e = tid; e < HID * IN; e += 128) {
        int o = e / IN, k = e - o * IN;
        st_bf16(sm + S_W1, to_tc::kmaj_off(o, k, KB_IN, 2), params[OFF_W1 + e]);
    }
    for (int e = tid; e < HID * HID; e += 128) {
        int o = e / HID, i = e - o * HID;
        float w = params[OFF_W2 + e];
        st_bf16(sm + S_B, to_tc::kmaj_off(o, i, KB_HID, 2), w);
        if (BWD) st_bf16(sm + S_W2T, to_tc::kmaj_off(i, o, KB_HID, 2), w);
    }
    for (int e = tid; e < OUT * HID; e += 128) f[F_W3 + e] = bf(params[OFF_W3 + e]);
    f[F_B1 + tid] = params[OFF_B1 + tid];
    f[F_B2 + tid] = params[OFF_B2 + tid];
    if (tid < OUT) f[F_B3 + tid] = params[OFF_B3 + tid];
    {
        float xv[IN];
#pragma unroll
        for (int k = 0; k < IN; ++k) xv[k] = valid ? x[(size_t)src * IN + k] : 0.0f;
        st_bf16x8(sm + S_X, to_tc::kmaj_off(tid, 0, KB_IN, 2), xv);
        st_bf16x8(sm + S_X, to_tc::kmaj_off(tid, 8, KB_IN, 2), xv + 8);
        if (BWD)
#pragma unroll
            for (int k = 0; k < IN; ++k) st_bf16(sm + S_XT, to_tc::kmaj_off(k, tid, KB_HID, 2), xv[k]);
    }
    if (tid == 0) to_tc::mbar_init(&mbar, 1);
    if (warp == 0) to_tc::tmem_alloc<256>(&tslot);
    publish_smem();
    const uint32_t tmem = tslot;
    const uint32_t T0 = tmem, T1 = tmem + 128;     // two 128-column accumulators
    uint32_t phase = 0;
    bool ok = true;

    // ---- F1
    if (tid == 0) {
        mma_chain(T0, sm + S_X, SBO_IN, sm + S_W1, SBO_IN, to_tc::idesc(1, 128, HID), 1);
        to_tc::commit(&mbar);
    }
    ok = wait_mma(&mbar, phase);
    uint32_t mask1[4] = {0, 0, 0, 0};
    if (ok) {
        for (int c0 = 0; c0 < HID; c0 += 16) {
            float v[16];
            to_tc::tmem_ld16(to_tc::lane_addr(T0, warp, c0), v);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                float a = v[j] + f[F_B1 + c0 + j];
                if (a > 0.0f) mask1[(c0 + j) >> 5] |= 1u << ((c0 + j) & 31);
                v[j] = a > 0.0f ? a : 0.0f;
            }
            st_bf16x8(sm + S_A, to_tc::kmaj_off(tid, c0, KB_HID, 2), v);
            st_bf16x8(sm + S_A, to_tc::kmaj_off(tid, c0 + 8, KB_HID, 2), v + 8);
            if (BWD)
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    st_bf16(sm + S_H1T, to_tc::kmaj_off(c0 + j, tid, KB_HID, 2), v[j]);
        }
    }
    publish_smem();

    // ---- F2
    if (ok && tid == 0) {
        mma_chain(T1, sm + S_A, SBO_HID, sm + S_B, SBO_HID, to_tc::idesc(1, 128, HID), HID / 16);
        to_tc::commit(&mbar);
    }
    if (ok) ok = wait_mma(&mbar, phase);

    // ---- layer 3 (SIMT) on bf16 H2; H2 kept row-major in S_B for dW3
    float y[OUT] = {0.0f, 0.0f, 0.0f};
    unsigned short* h2s = reinterpret_cast<unsigned short*>(sm + S_B);
    if (ok) {
        for (int c0 = 0; c0 < HID; c0 += 16) {
            float v[16];
            to_tc::tmem_ld16(to_tc::lane_addr(T1, warp, c0), v);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int o = c0 + j;
                float a = v[j] + f[F_B2 + o];
                float h = bf(a > 0.0f ? a : 0.0f);
                if (BWD) h2s[tid * HID + o] = bfbits(h);
#pragma unroll
                for (int q = 0; q < OUT; ++q) y[q] = y[q] + h * f[F_W3 + q * HID + o];
            }
        }
#pragma unroll
        for (int q = 0; q < OUT; ++q) y[q] = y[q] + f[F_B3 + q];
    }
    if (!BWD) {
        if (ok && valid)
            for (int q = 0; q < OUT; ++q) y_out[(size_t)gr * OUT + q] = y[q];
    } else {
        // ---- loss gradient
        float l = 0.0f;
#pragma unroll
        for (int q = 0; q < OUT; ++q) {
            float d = valid ? y[q] - t[(size_t)src * OUT + q] : 0.0f;
            l = l + d * d;
            f[F_DY + tid * OUT + q] = 2.0f * d * inv_count;
        }
        f[F_L + tid] = l;
        to_tc::fence_before_sync();
        __syncthreads();
        to_tc::fence_after_sync();
        if (tid == 0) {
            double s = 0.0;
            for (int i = 0; i < 128; ++i) s += (double)f[F_L + i];
            loss_part[blockIdx.x] = s;
        }
        // ---- dH2 = (dY W3) * relu'(a2)
        const float dy0 = f[F_DY + tid * OUT + 0], dy1 = f[F_DY + tid * OUT + 1],
                    dy2 = f[F_DY + tid * OUT + 2];
        if (ok) {
            for (int c0 = 0; c0 < HID; c0 += 16) {
                float v[16];
                to_tc::tmem_ld16(to_tc::lane_addr(T1, warp, c0), v);
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int o = c0 + j;
                    float a = v[j] + f[F_B2 + o];
                    float g = (dy0 * f[F_W3 + o] + dy1 * f[F_W3 + HID + o]) + dy2 * f[F_W3 + 2 * HID + o];
                    v[j] = a > 0.0f ? g : 0.0f;
                }
                st_bf16x8(sm + S_A, to_tc::kmaj_off(tid, c0, KB_HID, 2), v);
                st_bf16x8(sm + S_A, to_tc::kmaj_off(tid, c0 + 8, KB_HID, 2), v + 8);
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    st_bf16(sm + S_D2T, to_tc::kmaj_off(c0 + j, tid, KB_HID, 2), v[j]);
            }
        }
        publish_smem();
        // ---- B2 (dH1 pre-mask) into T0, G2 (dW2) into T1
        if (ok && tid == 0) {
            mma_chain(T0, sm + S_A, SBO_HID, sm + S_W2T, SBO_HID, to_tc::idesc(1, 128, HID), HID / 16);
            mma_chain(T1, sm + S_D2T, SBO_HID, sm + S_H1T, SBO_HID, to_tc::idesc(1, 128, HID), HID / 16);
            to_tc::commit(&mbar);
        }
        // meanwhile: dW3, db3, db2 (rows summed in order)
        float* gp = part + (size_t)blockIdx.x * PSTRIDE;
        {
            const int o = tid;
            float g0 = 0.0f, g1 = 0.0f, g2 = 0.0f, gb2 = 0.0f;
            for (int r = 0; r < 128; ++r) {
                float h = __bfloat162float(__ushort_as_bfloat16(h2s[r * HID + o]));
                g0 = g0 + f[F_DY + r * OUT + 0] * h;
                g1 = g1 + f[F_DY + r * OUT + 1] * h;
                g2 = g2 + f[F_DY + r * OUT + 2] * h;
                gb2 = gb2 + ld_bf16(sm + S_A, to_tc::kmaj_off(r, o, KB_HID, 2));
            }
            gp[OFF_W3 + o] = g0;
            gp[OFF_W3 + HID + o] = g1;
            gp[OFF_W3 + 2 * HID + o] = g2;
            gp[OFF_B2 + o] = gb2;
            if (tid < OUT) {
                float s = 0.0f;
                for (int r = 0; r < 128; ++r) s = s + f[F_DY + r * OUT + tid];
                gp[OFF_B3 + tid] = s;
            }
        }
        if (ok) ok = wait_mma(&mbar, phase);
        if (ok) {
            // dH1 = B2 * relu'(a1), stored transposed for G1; dW2 rows out
            for (int c0 = 0; c0 < HID; c0 += 16) {
                float v[16];
                to_tc::tmem_ld16(to_tc::lane_addr(T0, warp, c0), v);
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int i = c0 + j;
                    float g = ((mask1[i >> 5] >> (i & 31)) & 1u) ? v[j] : 0.0f;
                    st_bf16(sm + S_A, to_tc::kmaj_off(i, tid, KB_HID, 2), g);
                }
                to_tc::tmem_ld16(to_tc::lane_addr(T1, warp, c0), v);
                float4* dst = reinterpret_cast<float4*>(gp + OFF_W2 + (size_t)tid * HID + c0);
#pragma unroll
                for (int j = 0; j < 4; ++j) dst[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
            }
        }
        publish_smem();
        // ---- G1 (dW1) into T0
        if (ok && tid == 0) {
            mma_chain(T0, sm + S_A, SBO_HID, sm + S_XT, SBO_HID, to_tc::idesc(1, 128, IN), HID / 16);
            to_tc::commit(&mbar);
        }
        {
            float s = 0.0f;
            for (int r = 0; r < 128; ++r) s = s + ld_bf16(sm + S_A, to_tc::kmaj_off(tid, r, KB_HID, 2));
            gp[OFF_B1 + tid] = s;
        }
        if (ok) ok = wait_mma(&mbar, phase);
        if (ok) {
            float v[16];
            to_tc::tmem_ld16(to_tc::lane_addr(T0, warp, 0), v);
            float4* dst = reinterpret_cast<float4*>(gp + OFF_W1 + (size_t)tid * IN);
#pragma unroll
            for (int j = 0; j < 4; ++j) dst[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
        }
    }
    if (!ok && tid == 0) atomicExch(err, TO_DEVERR_SPIN);
    to_tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) to_tc::tmem_free<256>(tmem);
}

// grad = sum of tile partials (tile order); optional Adam update
__global__ void k_mlp_adam(int tiles, const float* __restrict__ part, float* __restrict__ grad,
                           float* __restrict__ params, float* __restrict__ m,
                           float* __restrict__ v, float lr, float b1, float b2, float eps,
                           float c1, float c2) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= NPARAM) return;
    float g = 0.0f;
    for (int i = 0; i < tiles; ++i) g = g + part[(size_t)i * PSTRIDE + p];
    if (grad) grad[p] = g;
    if (params) {
        float mm = b1 * m[p] + (1.0f - b1) * g;
        float vv = b2 * v[p] + (1.0f - b2) * g * g;
        m[p] = mm;
        v[p] = vv;
        params[p] = params[p] - lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    }
}

__global__ void k_sum_loss(int tiles, const double* __restrict__ lp, double* __restrict__ out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double s = 0.0;
        for (int i = 0; i < tiles; ++i) s += lp[i];
        *out += s;
    }
}

template <bool BWD>
to_status launch_mlp(to_ctx ctx, const float* params, int n, const int* rows, const float* x,
                     const float* t, float inv_count, float* y, float* part, double* lp) {
    static bool attr[2] = {false, false};
    if (!attr[BWD]) {
        TO_CUDA(ctx, cudaFuncSetAttribute(k_mlp<BWD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          SMEM_BYTES));
        attr[BWD] = true;
    }
    const int tiles = (n + 127) / 128;
    to_prof_begin(ctx, BWD ? "mlp_fwd_bwd" : "mlp_fwd");
    k_mlp<BWD><<<tiles, 128, SMEM_BYTES, ctx->stream>>>(params, n, rows, x, t, inv_count, y, part,
                                                         lp, ctx->d_flags);
    to_prof_end(ctx);
    TO_LAUNCHED(ctx);
    return TO_OK;
}

}  // namespace

namespace to_k {

to_status mlp_forward(to_ctx ctx, const float* d_params, int n, const float* d_x, float* d_y) {
    if (n <= 0) return TO_OK;
    return launch_mlp<false>(ctx, d_params, n, nullptr, d_x, nullptr, 0.0f, d_y, nullptr, nullptr);
}

size_t mlp_part_floats(int n) { return (size_t)((n + 127) / 128) * PSTRIDE; }

// gradient of mean((y - t)^2) over the n selected rows; d_part: mlp_part_floats(n)
to_status mlp_grad(to_ctx ctx, const float* d_params, int n, const int* d_rows, const float* d_x,
                   const float* d_t, float* d_part, double* d_lp, float* d_grad, float* d_params_upd,
                   float* d_m, float* d_v, float lr, int step) {
    const int tiles = (n + 127) / 128;
    TO_TRY(launch_mlp<true>(ctx, d_params, n, d_rows, d_x, d_t, 1.0f / (3.0f * (float)n), nullptr,
                            d_part, d_lp));
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    k_mlp_adam<<<(NPARAM + 255) / 256, 256, 0, ctx->stream>>>(tiles, d_part, d_grad, d_params_upd,
                                                              d_m, d_v, lr, b1, b2, 1e-8f, c1, c2);
    TO_LAUNCHED(ctx);
    return TO_OK;
}

to_status mlp_sum_loss(to_ctx ctx, int tiles, const double* d_lp, double* d_out) {
    k_sum_loss<<<1, 32, 0, ctx->stream>>>(tiles, d_lp, d_out);
    TO_LAUNCHED(ctx);
    return TO_OK;
}

}  // namespace to_k

// ---- C ABI ------------------------------------------------------------------
namespace {

to_status mlp_check_flags(to_ctx ctx) {
    int f = 0;
    TO_TRY(to_read_device_flags(ctx, &f));
    if (f != TO_DEVERR_NONE) {
        int z = 0;
        TO_CUDA(ctx, cudaMemcpy(ctx->d_flags, &z, sizeof(int), cudaMemcpyHostToDevice));
        return to_set_error(ctx, TO_ERR_TIMEOUT, "tensor-core wait expired in the MLP kernel");
    }
    return TO_OK;
}

// seeded Fisher-Yates shuffle (splitmix64 stream)
void shuffle_rows(int* r, int n, uint64_t& state) {
    for (int i = 0; i < n; ++i) r[i] = i;
    for (int i = n - 1; i > 0; --i) {
        state += 0x9E3779B97F4A7C15ull;
        uint64_t z = state;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        int j = (int)(z % (uint64_t)(i + 1));
        int t = r[i]; r[i] = r[j]; r[j] = t;
    }
}

bool finite_all(const float* v, size_t n) {
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(v[i])) return false;
    return true;
}

}  // namespace

extern "C" {

to_status to_mlp_predict_d(to_ctx ctx, const float* d_params, int n, const float* d_x, float* d_y) {
    if (!ctx || n < 0 || (n > 0 && (!d_params || !d_x || !d_y))) return TO_ERR_INVALID;
    cudaSetDevice(ctx->device);
    return to_k::mlp_forward(ctx, d_params, n, d_x, d_y);
}

to_status to_mlp_predict(to_ctx ctx, const float* params, int n, const float* x, float* y) {
    if (!ctx || !params || n < 0 || (n > 0 && (!x || !y))) return TO_ERR_INVALID;
    if (n == 0) return TO_OK;
    cudaSetDevice(ctx->device);
    const size_t bytes = to_align256((size_t)NPARAM * 4) + to_align256((size_t)n * IN * 4) +
                         to_align256((size_t)n * OUT * 4);
    TO_TRY(to_arena_reserve(ctx, bytes + 1024));
    float* d_p = to_arena_take<float>(ctx, NPARAM);
    float* d_x = to_arena_take<float>(ctx, (size_t)n * IN);
    float* d_y = to_arena_take<float>(ctx, (size_t)n * OUT);
    TO_CUDA(ctx, cudaMemcpyAsync(d_p, params, (size_t)NPARAM * 4, cudaMemcpyHostToDevice, ctx->stream));
    TO_CUDA(ctx, cudaMemcpyAsync(d_x, x, (size_t)n * IN * 4, cudaMemcpyHostToDevice, ctx->stream));
    TO_TRY(to_k::mlp_forward(ctx, d_p, n, d_x, d_y));
    TO_CUDA(ctx, cudaMemcpyAsync(y, d_y, (size_t)n * OUT * 4, cudaMemcpyDeviceToHost, ctx->stream));
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return mlp_check_flags(ctx);
}

to_status to_mlp_grad(to_ctx ctx, const float* params, int n, const float* x, const float* t,
                      float* grad, double* loss) {
    if (!ctx || !params || n <= 0 || !x || !t || !grad) return TO_ERR_INVALID;
    cudaSetDevice(ctx->device);
    const int tiles = (n + 127) / 128;
    const size_t bytes = to_align256((size_t)NPARAM * 4) * 2 + to_align256((size_t)n * IN * 4) +
                         to_align256((size_t)n * OUT * 4) + to_align256(to_k::mlp_part_floats(n) * 4) +
                         to_align256((size_t)tiles * 8) + 256;
    TO_TRY(to_arena_reserve(ctx, bytes + 1024));
    float* d_p = to_arena_take<float>(ctx, NPARAM);
    float* d_g = to_arena_take<float>(ctx, NPARAM);
    float* d_x = to_arena_take<float>(ctx, (size_t)n * IN);
    float* d_t = to_arena_take<float>(ctx, (size_t)n * OUT);
    float* d_part = to_arena_take<float>(ctx, to_k::mlp_part_floats(n));
    double* d_lp = to_arena_take<double>(ctx, tiles);
    double* d_l = to_arena_take<double>(ctx, 1);
    TO_CUDA(ctx, cudaMemcpyAsync(d_p, params, (size_t)NPARAM * 4, cudaMemcpyHostToDevice, ctx->stream));
    TO_CUDA(ctx, cudaMemcpyAsync(d_x, x, (size_t)n * IN * 4, cudaMemcpyHostToDevice, ctx->stream));
    TO_CUDA(ctx, cudaMemcpyAsync(d_t, t, (size_t)n * OUT * 4, cudaMemcpyHostToDevice, ctx->stream));
    TO_CUDA(ctx, cudaMemsetAsync(d_l, 0, 8, ctx->stream));
    TO_TRY(to_k::mlp_grad(ctx, d_p, n, nullptr, d_x, d_t, d_part, d_lp, d_g, nullptr, nullptr,
                          nullptr, 0.0f, 1));
    TO_TRY(to_k::mlp_sum_loss(ctx, tiles, d_lp, d_l));
    double l = 0.0;
    TO_CUDA(ctx, cudaMemcpyAsync(grad, d_g, (size_t)NPARAM * 4, cudaMemcpyDeviceToHost, ctx->stream));
    TO_CUDA(ctx, cudaMemcpyAsync(&l, d_l, 8, cudaMemcpyDeviceToHost, ctx->stream));
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (loss) *loss = l / (3.0 * n);
    return mlp_check_flags(ctx);
}

to_status to_mlp_train(to_ctx ctx, float* params, int n, const float* x, const float* t,
                       int epochs, int batch, float lr, uint64_t seed, double* loss_curve) {
    if (!ctx || !params || n <= 0 || !x || !t || epochs < 0 || batch <= 0 || !(lr > 0.0f))
        return TO_ERR_INVALID;
    if (!finite_all(x, (size_t)n * IN) || !finite_all(t, (size_t)n * OUT) ||
        !finite_all(params, NPARAM))
        return to_set_error(ctx, TO_ERR_NONFINITE, "non-finite MLP training input");
    cudaSetDevice(ctx->device);
    if (batch > n) batch = n;
    const int tiles = (batch + 127) / 128;
    const size_t ep = epochs > 0 ? epochs : 1;
    const size_t bytes = to_align256((size_t)NPARAM * 4) * 3 + to_align256((size_t)n * IN * 4) +
                         to_align256((size_t)n * OUT * 4) + to_align256(ep * n * 4) +
                         to_align256(to_k::mlp_part_floats(batch) * 4) + to_align256((size_t)tiles * 8) +
                         to_align256(ep * 8);
    TO_TRY(to_arena_reserve(ctx, bytes + 2048));
    float* d_p = to_arena_take<float>(ctx, NPARAM);
    float* d_m = to_arena_take<float>(ctx, NPARAM);
    float* d_v = to_arena_take<float>(ctx, NPARAM);
    float* d_x = to_arena_take<float>(ctx, (size_t)n * IN);
    float* d_t = to_arena_take<float>(ctx, (size_t)n * OUT);
    int* d_rows = to_arena_take<int>(ctx, ep * n);
    float* d_part = to_arena_take<float>(ctx, to_k::mlp_part_floats(batch));
    double* d_lp = to_arena_take<double>(ctx, tiles);
    double* d_loss = to_arena_take<double>(ctx, ep);
    std::vector<int> rows(ep * n);
    uint64_t st = seed;
    for (size_t e = 0; e < ep; ++e) shuffle_rows(rows.data() + e * n, n, st);
    TO_CUDA(ctx, cudaMemcpyAsync(d_p, params, (size_t)NPARAM * 4, cudaMemcpyHostToDevice, ctx->stream));
    TO_CUDA(ctx, cudaMemsetAsync(d_m, 0, (size_t)NPARAM * 4, ctx->stream));
    TO_CUDA(ctx, cudaMemsetAsync(d_v, 0, (size_t)NPARAM * 4, ctx->stream));
    TO_CUDA(ctx, cudaMemcpyAsync(d_x, x, (size_t)n * IN * 4, cudaMemcpyHostToDevice, ctx->stream));
    TO_CUDA(ctx, cudaMemcpyAsync(d_t, t, (size_t)n * OUT * 4, cudaMemcpyHostToDevice, ctx->stream));
    TO_CUDA(ctx, cudaMemcpyAsync(d_rows, rows.data(), ep * n * 4, cudaMemcpyHostToDevice, ctx->stream));
    TO_CUDA(ctx, cudaMemsetAsync(d_loss, 0, ep * 8, ctx->stream));
    int step = 0;
    for (int e = 0; e < epochs; ++e) {
        for (int s0 = 0; s0 < n; s0 += batch) {
            const int bs = n - s0 < batch ? n - s0 : batch;
            ++step;
            TO_TRY(to_k::mlp_grad(ctx, d_p, bs, d_rows + (size_t)e * n + s0, d_x, d_t, d_part, d_lp,
                                  nullptr, d_p, d_m, d_v, lr, step));
            TO_TRY(to_k::mlp_sum_loss(ctx, (bs + 127) / 128, d_lp, d_loss + e));
        }
    }
    std::vector<double> lc(ep);
    TO_CUDA(ctx, cudaMemcpyAsync(params, d_p, (size_t)NPARAM * 4, cudaMemcpyDeviceToHost, ctx->stream));
    TO_CUDA(ctx, cudaMemcpyAsync(lc.data(), d_loss, ep * 8, cudaMemcpyDeviceToHost, ctx->stream));
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (loss_curve)
        for (int e = 0; e < epochs; ++e) loss_curve[e] = lc[e] / (3.0 * n);
    return mlp_check_flags(ctx);
}

}  // extern "C"
