// knn.cu - k nearest neighbours and multiple local linear regression.
//
// Reference: knn_cuda_with_indexes::knn (include/gpuCode/
// knn_cuda_with_indexes.cu:475-618: a P x Q distance matrix, a per-query
// insertion sort over it, a sqrt pass, with host copies around each call)
// and multiLocLinReg (SimulateGPU.cu:2934-3053).
//
// Here a warp owns a run of neighbouring grid queries.  The reference points
// of the problem sit in shared memory.  For each query the warp gathers
// every point within a squared-distance threshold in one ballot-compaction
// pass (the threshold adapts until between k and 256 points qualify and is
// carried to the next, neighbouring, query), then bitonic-sorts the
// survivors by (squared distance, index): exactly the set and order the
// reference's stable insertion sort returns.  When exact ties prevent the
// window, a 4 x 8-bit radix select on the same keys takes over.  Nothing of
// size P x Q is written; for the ROV the local linear regression runs in the
// same warp right after the selection.
#include "to_internal.cuh"
#include "to_lsm_math.h"
#include "to_rov.cuh"

namespace {

constexpr int kWarps = 8;

struct WarpScratch {
    unsigned hist[256];
    unsigned long long sel[TO_KNN_KMAX];
    float gy[TO_KNN_KMAX];                    // neighbour responses
    float gx[TO_KNN_KMAX * TO_LSM_MAXD];      // neighbour predictors
};

__device__ __forceinline__ float sqdist(const float* ref, int stride, int i, int dim,
                                        const float* q) {
    float s = 0.0f;
    for (int j = 0; j < dim; ++j) {
        float t = ref[(size_t)j * stride + i] - q[j];
        s = fmaf(t, t, s);
    }
    return s;
}

// k smallest (key, index) of n points for one query; results in ws.sel[0..k)
// sorted ascending.  ref is dim-major with the given stride.
__device__ void warp_select(const float* ref, int stride, int n, int dim,
                            const float* q, int k, WarpScratch& ws) {
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    unsigned prefix = 0, remaining = (unsigned)k;
    for (int shift = 24; shift >= 0; shift -= 8) {
        for (int b = lane; b < 256; b += 32) ws.hist[b] = 0;
        __syncwarp();
        const unsigned hmask = (shift == 24) ? 0u : (0xFFFFFFFFu << (shift + 8));
        for (int base = 0; base < n; base += 32) {
            int i = base + lane;
            bool ok = i < n;
            unsigned key = ok ? __float_as_uint(sqdist(ref, stride, i, dim, q)) : 0u;
            ok = ok && ((key & hmask) == (prefix & hmask));
            unsigned digit = (key >> shift) & 255u;
            unsigned act = __ballot_sync(0xffffffffu, ok);
            if (ok) {
                unsigned peers = __match_any_sync(act, digit);
                int leader = __ffs(peers) - 1;
                if (lane == leader) atomicAdd(&ws.hist[digit], (unsigned)__popc(peers));
            }
        }
        __syncwarp();
        // find the digit holding the remaining-th key
        unsigned h[8];
        unsigned local = 0;
        for (int j = 0; j < 8; ++j) { h[j] = ws.hist[lane * 8 + j]; local += h[j]; }
        unsigned incl = local;
        for (int o = 1; o < 32; o <<= 1) {
            unsigned v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        unsigned excl = incl - local;
        int found = -1;
        unsigned before = 0;
        if (excl < remaining && remaining <= incl) {
            unsigned c = excl;
            for (int j = 0; j < 8; ++j) {
                if (c + h[j] >= remaining) { found = lane * 8 + j; before = c; break; }
                c += h[j];
            }
        }
        unsigned who = __ballot_sync(0xffffffffu, found >= 0);
        int src = who ? __ffs(who) - 1 : 0;
        found = __shfl_sync(0xffffffffu, found, src);
        before = __shfl_sync(0xffffffffu, before, src);
        if (found < 0) found = 255;          // cannot happen for k <= n
        remaining -= before;
        prefix |= (unsigned)found << shift;
        __syncwarp();
    }
    // gather: every key below the threshold, then the first `remaining`
    // keys equal to it in index order
    const unsigned T = prefix;
    const unsigned n_less = (unsigned)k - remaining;
    unsigned c_less = 0, c_eq = 0;
    for (int base = 0; base < n; base += 32) {
        int i = base + lane;
        unsigned key = (i < n) ? __float_as_uint(sqdist(ref, stride, i, dim, q)) : 0xFFFFFFFFu;
        bool lt = (i < n) && key < T;
        bool eq = (i < n) && key == T;
        unsigned ml = __ballot_sync(0xffffffffu, lt);
        unsigned me = __ballot_sync(0xffffffffu, eq);
        if (lt) ws.sel[c_less + __popc(ml & lt_mask)] =
            ((unsigned long long)key << 32) | (unsigned)i;
        if (eq) {
            unsigned r = c_eq + __popc(me & lt_mask);
            if (r < remaining)
                ws.sel[n_less + r] = ((unsigned long long)key << 32) | (unsigned)i;
        }
        c_less += __popc(ml);
        c_eq += __popc(me);
    }
    __syncwarp();
    // bitonic sort of the k survivors (padded to a power of two)
    int kp = 1;
    while (kp < k) kp <<= 1;
    for (int i = k + lane; i < kp; i += 32) ws.sel[i] = ~0ull;
    __syncwarp();
    for (int size = 2; size <= kp; size <<= 1) {
        for (int stride2 = size >> 1; stride2 > 0; stride2 >>= 1) {
            for (int i = lane; i < kp; i += 32) {
                int j = i ^ stride2;
                if (j > i) {
                    unsigned long long a = ws.sel[i], b = ws.sel[j];
                    bool up = ((i & size) == 0);
                    if ((a > b) == up) { ws.sel[i] = b; ws.sel[j] = a; }
                }
            }
            __syncwarp();
        }
    }
}

// Threshold form of the same selection.  All points with squared distance
// <= T are gathered (ballot compaction, one pass); T is adapted until at
// least k and at most TO_KNN_KMAX points qualify, then the survivors are
// bitonic-sorted by (key, index).  Every point closer than the k-th is kept,
// so the result equals warp_select's.  T is carried over from the previous
// (neighbouring) query, so one pass usually suffices.  Returns false when
// exact ties keep the count from entering the window (caller falls back to
// warp_select).
__device__ bool warp_select_threshold(const float* ref, int stride, int n, int dim,
                                      const float* q, int k, float& T, WarpScratch& ws) {
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    float lo = -1.0f, hi = -1.0f;        // bracket: count(lo) < k, count(hi) > cap
    int cnt = 0;
    for (int iter = 0; iter < 64; ++iter) {
        cnt = 0;
        for (int base = 0; base < n; base += 32) {
            int i = base + lane;
            float key = (i < n) ? sqdist(ref, stride, i, dim, q) : INFINITY;
            bool le = (i < n) && key <= T;
            unsigned m = __ballot_sync(0xffffffffu, le);
            int pos = cnt + __popc(m & lt_mask);
            if (le && pos < TO_KNN_KMAX)
                ws.sel[pos] = ((unsigned long long)__float_as_uint(key) << 32) | (unsigned)i;
            cnt += __popc(m);
        }
        if (cnt >= k && cnt <= TO_KNN_KMAX) break;
        if (cnt < k) lo = T; else hi = T;
        float nt;
        if (lo < 0.0f) nt = T * 0.25f;
        else if (hi < 0.0f) nt = (T > 0.0f) ? T * 4.0f : 1e-30f;
        else nt = sqrtf(fmaxf(lo, 1e-38f) * hi);
        if (!(nt > lo) || (hi >= 0.0f && !(nt < hi))) { cnt = -1; break; }
        T = nt;
    }
    __syncwarp();
    if (cnt < k || cnt > TO_KNN_KMAX) return false;
    int kp = 1;
    while (kp < cnt) kp <<= 1;
    for (int i = cnt + lane; i < kp; i += 32) ws.sel[i] = ~0ull;
    __syncwarp();
    for (int size = 2; size <= kp; size <<= 1) {
        for (int stride2 = size >> 1; stride2 > 0; stride2 >>= 1) {
            for (int i = lane; i < kp; i += 32) {
                int j = i ^ stride2;
                if (j > i) {
                    unsigned long long a = ws.sel[i], b = ws.sel[j];
                    bool up = ((i & size) == 0);
                    if ((a > b) == up) { ws.sel[i] = b; ws.sel[j] = a; }
                }
            }
            __syncwarp();
        }
    }
    // next query starts from a threshold a little above this k-th distance
    float kth = __uint_as_float((unsigned)(ws.sel[k - 1] >> 32));
    T = (kth > 0.0f) ? kth * 1.5f : 1e-30f;
    return true;
}

// ROV: kNN + multiLocLinReg fused.  Grid (ceil(Q / (kWarps*kRun)), C); a
// warp handles kRun consecutive grid queries of control c, whose points
// (xn[c][j][P]) sit in shared memory.  After the selection the warp gathers
// the neighbours' responses and predictors, and lane 0 accumulates the
// normal equations in neighbour order and solves them (to_lsm_math.h).
constexpr int kRun = 4;

__global__ void __launch_bounds__(kWarps * 32)
k_knn_rov(to_rov_args a, int t, int smem_points) {
    extern __shared__ unsigned char sm_raw[];
    WarpScratch* wsa = reinterpret_cast<WarpScratch*>(sm_raw);
    float* sref = reinterpret_cast<float*>(sm_raw + sizeof(WarpScratch) * kWarps);
    const int c = blockIdx.y;
    const int d = a.S + 1, R = a.R;
    const int n = a.npts[c], k = a.kc[c];
    const size_t blk = (size_t)R * d + 2 * (size_t)a.Q;
    float* yout = a.reg + (size_t)t * a.C * blk + (size_t)c * blk + (size_t)R * d;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int q0 = (blockIdx.x * kWarps + warp) * kRun;
    if (n < 3 || k <= 0) {
        for (int r = lane; r < kRun; r += 32)
            if (q0 + r < a.Q) yout[q0 + r] = 0.0f;
        return;
    }
    const float* src = a.xn + (size_t)c * d * a.P;
    const float* ref = src;
    int stride = a.P;
    if (n <= smem_points) {
        for (int q = threadIdx.x; q < n * d; q += blockDim.x) {
            int j = q / n, m = q - j * n;
            sref[(size_t)j * n + m] = src[(size_t)j * a.P + m];
        }
        __syncthreads();
        ref = sref;
        stride = n;
    }
    WarpScratch& ws = wsa[warp];
    const float* y = a.yv + (size_t)c * a.P;
    const float* xr = a.xraw + (size_t)c * d * a.P;
    float T = powf((float)k / (float)n, 2.0f / (float)d);
    for (int r = 0; r < kRun; ++r) {
        const int qi = q0 + r;
        if (qi >= a.Q) break;
        float qn[TO_LSM_MAXD], xq[TO_LSM_MAXD];
        to_rov_query(a, qi, qn, xq);
        if (!warp_select_threshold(ref, stride, n, d, qn, k, T, ws)) {
            warp_select(ref, stride, n, d, qn, k, ws);
            T = powf((float)k / (float)n, 2.0f / (float)d);
        }
        // gather the neighbours' responses and predictors
        for (int kk = lane; kk < k; kk += 32) {
            int i = (int)(ws.sel[kk] & 0xFFFFFFFFu);
            ws.gy[kk] = y[i];
            for (int j = 0; j < d; ++j) {
                float xv;
                if (a.sem == 0) {
                    // the reference reads its dim-major buffer (stride n)
                    // point-major (multiLocLinReg, SimulateGPU.cu:3002)
                    int f = i * d + j;
                    int jj = f / n, m = f - jj * n;
                    xv = xr[(size_t)jj * a.P + m];
                } else {
                    xv = ref[(size_t)j * stride + i];
                }
                ws.gx[kk * TO_LSM_MAXD + j] = xv;
            }
        }
        __syncwarp();
        if (lane == 0) {
            float acc[TO_LSM_ACC];
            to_lsm_acc_init(d, acc);
            const float h = sqrtf(__uint_as_float((unsigned)(ws.sel[k - 1] >> 32)));
            for (int kk = 0; kk < k; ++kk) {
                float dd = sqrtf(__uint_as_float((unsigned)(ws.sel[kk] >> 32)));
                to_lsm_acc_add(d, acc, to_lsm_weight(dd, h), ws.gy[kk],
                               &ws.gx[kk * TO_LSM_MAXD], xq);
            }
            yout[qi] = to_lsm_solve_intercept(d, acc);
        }
        __syncwarp();
    }
}

// generic: explicit dim-major queries
__global__ void __launch_bounds__(kWarps * 32)
k_knn_generic(const float* ref_g, int n, const float* query, int Q, int dim, int k,
              float* dist, int* ind, int smem_points) {
    extern __shared__ unsigned char sm_raw[];
    WarpScratch* wsa = reinterpret_cast<WarpScratch*>(sm_raw);
    float* sref = reinterpret_cast<float*>(sm_raw + sizeof(WarpScratch) * kWarps);
    const float* ref = ref_g;
    if (n <= smem_points) {
        for (int q = threadIdx.x; q < n * dim; q += blockDim.x) sref[q] = ref_g[q];
        __syncthreads();
        ref = sref;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int qi = blockIdx.x * kWarps + warp;
    if (qi >= Q) return;
    float q[TO_LSM_MAXD + 3];
    for (int j = 0; j < dim; ++j) q[j] = query[(size_t)j * Q + qi];
    WarpScratch& ws = wsa[warp];
    float T = powf((float)k / (float)n, 2.0f / (float)dim);
    if (!warp_select_threshold(ref, n, n, dim, q, k, T, ws)) warp_select(ref, n, n, dim, q, k, ws);
    for (int kk = lane; kk < k; kk += 32) {
        unsigned long long v = ws.sel[kk];
        dist[(size_t)kk * Q + qi] = sqrtf(__uint_as_float((unsigned)(v >> 32)));
        ind[(size_t)kk * Q + qi] = (int)(v & 0xFFFFFFFFu) + 1;
    }
}

size_t knn_smem(int dim, int points) {
    return sizeof(WarpScratch) * kWarps + (size_t)dim * points * sizeof(float);
}

}  // namespace

namespace to_k {

to_status knn_rov(to_ctx ctx, const to_rov_args& a, int t) {
    const int d = a.S + 1;
    if (a.kmax > TO_KNN_KMAX)
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "k %d exceeds %d", a.kmax, TO_KNN_KMAX);
    size_t cap = ctx->smem_optin > 8192 ? ctx->smem_optin - 8192 : 48 * 1024;
    int pts = a.P;
    while (pts > 0 && knn_smem(d, pts) > cap) pts = pts * 3 / 4;
    size_t smem = knn_smem(d, pts);
    TO_CUDA(ctx, cudaFuncSetAttribute(k_knn_rov, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    dim3 grid((a.Q + kWarps * kRun - 1) / (kWarps * kRun), a.C);
    to_prof_begin(ctx, "knn");
    k_knn_rov<<<grid, kWarps * 32, smem, ctx->stream>>>(a, t, pts);
    to_prof_end(ctx);
    TO_LAUNCHED(ctx);
    return TO_OK;
}

to_status knn(to_ctx ctx, const float* ref, int n, const float* query, int Q, int dim,
              int k, float* dist, int* ind) {
    if (k > TO_KNN_KMAX || k > n || k <= 0 || dim > TO_LSM_MAXD + 3)
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "knn k=%d n=%d dim=%d", k, n, dim);
    size_t cap = ctx->smem_optin > 8192 ? ctx->smem_optin - 8192 : 48 * 1024;
    int pts = n;
    while (pts > 0 && knn_smem(dim, pts) > cap) pts = pts * 3 / 4;
    size_t smem = knn_smem(dim, pts);
    TO_CUDA(ctx, cudaFuncSetAttribute(k_knn_generic,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_knn_generic<<<(Q + kWarps - 1) / kWarps, kWarps * 32, smem, ctx->stream>>>(
        ref, n, query, Q, dim, k, dist, ind, pts);
    TO_LAUNCHED(ctx);
    return TO_OK;
}

}  // namespace to_k
