// knn.cu - k nearest neighbours and multiple local linear regression.
//
// Reference: knn_cuda_with_indexes::knn (include/gpuCode/
// knn_cuda_with_indexes.cu:475-618: a P x Q distance matrix, a per-query
// insertion sort over it, a sqrt pass, with host copies around each call)
// and multiLocLinReg (SimulateGPU.cu:2934-3053).
//
// A warp handles one query at a time.  It gathers every point within a
// squared-distance threshold T by ballot compaction; T adapts until between
// k and the store size qualify, then a threshold with exactly k of them at
// or below it is searched among the stored keys (ties at the k-th place
// broken by index): exactly the set the reference's stable insertion sort
// returns.  The kNN entry point then sorts them by (squared distance,
// index), as the reference returns them; the ROV sorts them by index.
// Groups of at most 320 points keep every key in registers and search the
// exact-k threshold on them, and their compaction already yields index
// order, with no sort.  When the search fails (ties keep the count out of
// the window), a 4 x 8-bit radix select on the same keys takes over.
//
// For the ROV the points of each control are first binned into a uniform
// cell grid (k_knn_grid, a counting sort), so a threshold pass visits only
// the cells a ball of radius sqrt(T) can touch - cell rows of dimension 0
// are contiguous in the sorted order - instead of all n points.  The ranges
// are widened by a small tolerance, so no point with key <= T is missed.
// The local linear regression runs in the same warp right after the
// selection, over the k nearest in ascending point index: lane l
// accumulates neighbours l, l+32, ... of that order, and each normal-
// equation sum adds the 32 lane partials in lane order (the oracle does the
// same).  Nothing of size P x Q is written.
#include "to_internal.cuh"
#include "to_lsm_math.h"
#include "to_rov.cuh"

namespace {

constexpr int kWarps = 8;
constexpr unsigned kFull = 0xffffffffu;

// a threshold pass keeps up to kStore candidates; the k nearest are then
// refined out of them without another pass over the points
constexpr int kStore = 2 * TO_KNN_KMAX;

struct WarpScratch {
    unsigned long long sel[kStore];
    unsigned hist[256];                       // radix select
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

// bitonic sort of up to 128 entries held in registers, four a lane
// (element e = 4 lane + i): strides 1 and 2 pair a lane's own registers,
// larger strides pair lanes through shuffles.  The entries are distinct
// (the point index is in the low word), so any sorting network gives the
// same order.
__device__ __forceinline__ void warp_sort_reg128(WarpScratch& ws, int cnt) {
    const int lane = threadIdx.x & 31;
    unsigned long long v[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int e = lane * 4 + i;
        v[i] = e < cnt ? ws.sel[e] : ~0ull;
    }
#pragma unroll
    for (int size = 2; size <= 128; size <<= 1) {
#pragma unroll
        for (int s2 = size >> 1; s2 > 0; s2 >>= 1) {
            if (s2 >= 4) {
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int e = lane * 4 + i;
                    const unsigned long long w = __shfl_xor_sync(0xffffffffu, v[i], s2 >> 2);
                    const bool take_min = ((e & s2) == 0) == ((e & size) == 0);
                    const bool less = v[i] < w;
                    v[i] = (take_min == less) ? v[i] : w;
                }
            } else {
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int j = i ^ s2;
                    if (j > i) {
                        const bool up = (((lane * 4 + i) & size) == 0);
                        if ((v[i] > v[j]) == up) {
                            const unsigned long long t = v[i];
                            v[i] = v[j];
                            v[j] = t;
                        }
                    }
                }
            }
        }
    }
    __syncwarp();
#pragma unroll
    for (int i = 0; i < 4; ++i) ws.sel[lane * 4 + i] = v[i];
    __syncwarp();
}

// bitonic sort of ws.sel[0..cnt), padded to a power of two; every lane
// owns compare-exchange pairs, so no lane idles
__device__ __noinline__ void warp_sort_sel(WarpScratch& ws, int cnt) {
    if (cnt <= 128) {
        warp_sort_reg128(ws, cnt);
        return;
    }
    const int lane = threadIdx.x & 31;
    int kp = 1;
    while (kp < cnt) kp <<= 1;
    for (int i = cnt + lane; i < kp; i += 32) ws.sel[i] = ~0ull;
    __syncwarp();
    const int half = kp >> 1;
    for (int size = 2; size <= kp; size <<= 1) {
        for (int s2 = size >> 1; s2 > 0; s2 >>= 1) {
            for (int pi = lane; pi < half; pi += 32) {
                const int i = ((pi & ~(s2 - 1)) << 1) | (pi & (s2 - 1));
                const int j = i + s2;
                const unsigned long long a = ws.sel[i], b = ws.sel[j];
                const bool up = ((i & size) == 0);
                if ((a > b) == up) { ws.sel[i] = b; ws.sel[j] = a; }
            }
            __syncwarp();
        }
    }
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
    warp_sort_sel(ws, k);
}

__device__ __forceinline__ unsigned long long pack_sel(float key, int i) {
    return ((unsigned long long)__float_as_uint(key) << 32) | (unsigned)i;
}

// Threshold form of the selection.  pass(T) gathers into ws.sel every point
// whose key is <= T and returns how many qualified.  A pass may lower T on
// its way (the cell-grid pass does when its store fills: it keeps only the
// stored keys under a new threshold, so the store still holds every point
// with key <= the final T); past kStore it stops storing, and it may stop
// counting once far above the window.  T is adapted until at least k and at
// most kStore points qualify.  The threshold is then narrowed among the
// stored keys alone until at most the power of two above k remain, and the
// survivors are sorted by (key, index).  Every point closer than the k-th is
// kept, so the result equals warp_select's.  The threshold update assumes a
// locally uniform density, count ~ T^(dim/2), kept inside the bracket of
// thresholds already seen.  Returns false when exact ties keep the count out
// of the window.
__device__ __forceinline__ bool next_threshold(int cnt, int k, float target, float expo,
                                               float& T, float& lo, float& hi) {
    if (cnt < k) lo = T; else hi = T;
    float nt;
    // the threshold only steers the search (every key <= T is kept and the
    // selection is exact), so the fast quotient and power are enough here
    if (cnt == 0) nt = (T > 0.0f) ? T * 16.0f : 1e-30f;
    else nt = T * __powf(__fdividef(target, (float)cnt), expo);
    if ((lo >= 0.0f && !(nt > lo)) || (hi >= 0.0f && !(nt < hi))) {
        if (lo >= 0.0f && hi >= 0.0f) nt = sqrtf(fmaxf(lo, 1e-38f) * hi);
        else if (hi < 0.0f) nt = (T > 0.0f) ? T * 4.0f : 1e-30f;
        else nt = T * 0.25f;
    }
    if (!(nt > lo) || (hi >= 0.0f && !(nt < hi))) return false;
    T = nt;
    return true;
}

// One step of the exact search for a threshold with exactly k keys at or
// below it: interpolate (count ~ T^(dim/2)); where that leaves the bracket,
// halve the bracket's bit patterns (keys are >= 0, so their bits order as
// the values).  False when the bracket holds no float strictly inside it:
// equal keys then straddle the k-th place.  The step only steers: the keys
// taken are the exact k nearest whatever path T takes, so its quotient and
// power are the fast ones.
__device__ __forceinline__ bool exact_step(int cnt, int k, float expo, float& T, float& lo,
                                           float& hi) {
    if (cnt < k) lo = T; else hi = T;
    float nt = (cnt == 0) ? ((T > 0.0f) ? T * 16.0f : 1e-30f)
                          : T * __powf(__fdividef((float)k, (float)cnt), expo);
    const bool has_lo = lo >= 0.0f, has_hi = hi >= 0.0f;
    if ((has_lo && !(nt > lo)) || (has_hi && !(nt < hi)) || !(nt < INFINITY)) {
        if (has_lo && has_hi) {
            const unsigned ul = __float_as_uint(lo), uh = __float_as_uint(hi);
            if (uh - ul < 2u) return false;
            nt = __uint_as_float(ul + (uh - ul) / 2u);
        } else if (!has_hi) {
            nt = (T > 0.0f) ? T * 4.0f : 1e-30f;
        } else {
            nt = T * 0.25f;
        }
    }
    T = nt;
    return true;
}

__device__ __forceinline__ float sel_key(const WarpScratch& ws, int i) {
    // high word of the packed (key, index) entry
    return __uint_as_float(reinterpret_cast<const unsigned*>(ws.sel)[2 * i + 1]);
}

// Lower T among the cnt stored candidates (all with key <= T) until between
// lo_n and hi_n of them have key <= T, then compact those to the front in
// their stored order (in place: a write never passes the read position).
// Returns false, changing nothing, when ties make the window unreachable.
__device__ __noinline__ bool narrow_stored(WarpScratch& ws, int& cnt, float& T, int lo_n, int hi_n,
                              float expo) {
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    const float target = 0.5f * (float)(lo_n + hi_n);
    float lo = -1.0f, hi = T, T2 = T;
    int c2 = cnt;
    bool ok = false;
    for (int iter = 0; iter < 64; ++iter) {
        if (!next_threshold(c2, lo_n, target, expo, T2, lo, hi)) break;
        unsigned cl = 0;
        for (int i = lane; i < cnt; i += 32) cl += (sel_key(ws, i) <= T2) ? 1u : 0u;
        c2 = (int)__reduce_add_sync(kFull, cl);
        if (c2 >= lo_n && c2 <= hi_n) { ok = true; break; }
    }
    if (!ok) return false;
    int pos0 = 0;
    for (int base = 0; base < cnt; base += 32) {
        const int i = base + lane;
        const unsigned long long v = (i < cnt) ? ws.sel[i] : ~0ull;
        const bool le = (i < cnt) && __uint_as_float((unsigned)(v >> 32)) <= T2;
        const unsigned m = __ballot_sync(kFull, le);
        if (le) ws.sel[pos0 + __popc(m & lt_mask)] = v;
        pos0 += __popc(m);
    }
    __syncwarp();
    cnt = c2;
    T = T2;
    return true;
}

// The k nearest among the cnt stored candidates (all with key <= T): a
// threshold with exactly k stored keys at or below it (exact_step), the
// survivors moved to the front in stored order (in place: a write never
// passes the read position); where equal keys straddle the k-th place,
// every key below the tied value and then the tied ones of lowest index.
// Returns the k-th smallest key, or -1 when the search fails.
__device__ __noinline__ float narrow_exact(WarpScratch& ws, int cnt, float T, int k, float expo) {
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    float lo = -1.0f, hi = -1.0f;
    bool tie = false;
    int c2 = cnt;
    for (int iter = 0; c2 != k; ++iter) {
        if (iter == 200) return -1.0f;
        if (!exact_step(c2, k, expo, T, lo, hi)) { tie = true; break; }
        unsigned cl = 0;
        for (int i = lane; i < cnt; i += 32) cl += (sel_key(ws, i) <= T) ? 1u : 0u;
        c2 = (int)__reduce_add_sync(kFull, cl);
    }
    unsigned thr = 0xFFFFFFFFu;          // the largest index taken at the tied key
    if (tie) {
        unsigned below = 0;
        for (int i = lane; i < cnt; i += 32) below += (sel_key(ws, i) < hi) ? 1u : 0u;
        const int need = k - (int)__reduce_add_sync(kFull, below);
        for (int r = 0; r < need; ++r) {
            unsigned m = 0xFFFFFFFFu;
            for (int i = lane; i < cnt; i += 32) {
                const unsigned long long v = ws.sel[i];
                const unsigned idx = (unsigned)v;
                if (sel_key(ws, i) == hi && (r == 0 || idx > thr)) m = min(m, idx);
            }
            thr = __reduce_min_sync(kFull, m);
        }
    }
    int pos0 = 0;
    unsigned top = 0;
    for (int base = 0; base < cnt; base += 32) {
        const int i = base + lane;
        const unsigned long long v = (i < cnt) ? ws.sel[i] : ~0ull;
        const float kv = __uint_as_float((unsigned)(v >> 32));
        const bool take = (i < cnt) && (tie ? (kv < hi || (kv == hi && (unsigned)v <= thr))
                                             : kv <= T);
        const unsigned m = __ballot_sync(kFull, take);
        if (take) {
            ws.sel[pos0 + __popc(m & lt_mask)] = v;
            top = max(top, __float_as_uint(kv));
        }
        pos0 += __popc(m);
    }
    __syncwarp();
    return __uint_as_float(__reduce_max_sync(kFull, top));
}

// Threshold passes until between k and kStore points qualify, then the
// exact k nearest among them (narrow_exact, stored order).  Returns the
// k-th smallest key, or -1 when the window or the search fails.
template <class Pass>
__device__ float threshold_select(int k, int dim, float& T, WarpScratch& ws, Pass pass) {
    float lo = -1.0f, hi = -1.0f;        // bracket: count(lo) < k, count(hi) > window
    const float expo = 2.0f / (float)dim;
    const float target = sqrtf((float)k * (float)kStore);
    int cnt = -1;
    for (int iter = 0; iter < 64; ++iter) {
        if (!(T < INFINITY) || !(T >= 0.0f)) { cnt = -1; break; }
        cnt = pass(T);
        if (cnt >= k && cnt <= kStore) break;
        if (!next_threshold(cnt, k, target, expo, T, lo, hi)) { cnt = -1; break; }
    }
    __syncwarp();
    if (cnt < k || cnt > kStore) return -1.0f;
    return narrow_exact(ws, cnt, T, k, expo);
}

// full scan over n points in index order (dim-major, given stride)
struct ScanPass {
    const float* ref;
    int stride, n, dim;
    const float* q;
    WarpScratch* ws;
    __device__ int operator()(float& T) const {
        const int lane = threadIdx.x & 31;
        const unsigned lt_mask = (1u << lane) - 1u;
        int cnt = 0;
        for (int base = 0; base < n; base += 32) {
            int i = base + lane;
            float key = (i < n) ? sqdist(ref, stride, i, dim, q) : INFINITY;
            bool le = (i < n) && key <= T;
            unsigned m = __ballot_sync(kFull, le);
            int pos = cnt + __popc(m & lt_mask);
            if (le && pos < kStore) ws->sel[pos] = pack_sel(key, i);
            cnt += __popc(m);
            if (cnt > 4 * kStore) {
                // far above the window: extrapolate over the unscanned part
                float f = (float)(base + 32) / (float)n;
                return (int)fminf((float)cnt / f, 1e9f);
            }
        }
        return cnt;
    }
};

__device__ __forceinline__ int cell_of(float x, float lo, float inv, int G) {
    float f = (x - lo) * inv;
    if (!(f > 0.0f)) return 0;
    if (f >= (float)G) return G - 1;
    int c = (int)f;
    return c < G - 1 ? c : G - 1;
}

// Pass over the cells a ball of radius sqrt(T) around q can touch.  Cell
// rows (runs of dimension-0 cells, contiguous in the sorted order) are set up
// 32 at a time, one per lane: the row's lower-bound distance, its dimension-0
// range and its point range.  The warp then walks the concatenated point
// ranges of the batch in full chunks of 32; a lane finds the row of its point
// in a small per-warp table (its row index only moves forward).
template <int D>
struct GridPass {
    const to_knn_grid* g;
    const float* gs;      // [D][stride] points in cell order
    const int* gi;        // original indices
    const int* gc;        // cell starts
    int stride;
    const float* q;
    WarpScratch* ws;
    int k;
    // T may come back lower: when the store fills, the stored keys are cut
    // to a threshold keeping between k and kStore / 2 of them, and the rest
    // of the pass uses it (its cells were chosen for the larger radius)
    __device__ int operator()(float& T) const {
        const int lane = threadIdx.x & 31;
        const unsigned lt_mask = (1u << lane) - 1u;
        const float r = sqrtf(T);
        const float expo = 2.0f / (float)D;
        bool over = false;                  // ties kept the store from being cut
        int* row_off = reinterpret_cast<int*>(ws->hist);   // [33] batch offsets
        int* row_beg = row_off + 33;                         // [32] first point of a row
        int cl[D], span[D];
        float tol[D];
#pragma unroll
        for (int j = 0; j < D; ++j) {
            tol[j] = r * 1e-4f + 1e-6f * (1.0f + fabsf(q[j]) + fabsf(g->lo[j]) + fabsf(g->hi[j]));
            cl[j] = cell_of(q[j] - (r + tol[j]), g->lo[j], g->inv[j], g->G[j]);
            span[j] = cell_of(q[j] + (r + tol[j]), g->lo[j], g->inv[j], g->G[j]) - cl[j] + 1;
        }
        int nrows = 1;
#pragma unroll
        for (int j = 1; j < D; ++j) nrows *= span[j];
        int cnt = 0;
        for (int rb = 0; rb < nrows; rb += 32) {
            // this lane's row
            const int row = rb + lane;
            int beg = 0, len = 0;
            if (row < nrows) {
                int rem = row, cell = 0, mul = g->G[0];
                float lb2 = 0.0f;
#pragma unroll
                for (int j = 1; j < D; ++j) {
                    const int cj = cl[j] + rem % span[j];
                    rem /= span[j];
                    cell += cj * mul;
                    mul *= g->G[j];
                    if (g->inv[j] > 0.0f) {
                        const float slo = g->lo[j] + (float)cj * g->w[j];
                        const float shi = slo + g->w[j];
                        const float e = fmaxf(slo - q[j], q[j] - shi) - tol[j];
                        if (e > 0.0f) lb2 = lb2 + e * e;
                    }
                }
                const float Tp = T * 1.0002f + 1e-30f;
                if (lb2 <= Tp) {
                    const float r0 = sqrtf(Tp - lb2) + tol[0];
                    const int a0 = cell_of(q[0] - r0, g->lo[0], g->inv[0], g->G[0]);
                    const int b0 = cell_of(q[0] + r0, g->lo[0], g->inv[0], g->G[0]);
                    beg = gc[cell + a0];
                    len = gc[cell + b0 + 1] - beg;
                }
            }
            // exclusive scan of the row lengths
            int incl = len;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(kFull, incl, o);
                if (lane >= o) incl += v;
            }
            const int total = __shfl_sync(kFull, incl, 31);
            __syncwarp();
            row_off[lane] = incl - len;
            row_beg[lane] = beg;
            if (lane == 31) row_off[32] = total;
            __syncwarp();
            int my = 0;                     // row of this lane's point
            auto take = [&](float key, bool in, int gidx) {
                bool le = in && key <= T;
                unsigned m = __ballot_sync(kFull, le);
                if (!over && cnt + __popc(m) > kStore) {
                    if (narrow_stored(*ws, cnt, T, k, kStore / 2, expo)) {
                        le = in && key <= T;
                        m = __ballot_sync(kFull, le);
                    } else {
                        over = true;
                    }
                }
                const int pos = cnt + __popc(m & lt_mask);
                if (le && pos < kStore) ws->sel[pos] = pack_sel(key, gidx);
                cnt += __popc(m);
            };
            // two chunks of 32 points an iteration: every coordinate and
            // index load is issued before the first key is compared
            for (int base = 0; base < total; base += 64) {
                const int fa = base + lane, fb = fa + 32;
                const bool ina = fa < total, inb = fb < total;
                int ia = 0, ib = 0;
                if (ina) {
                    while (fa >= row_off[my + 1]) ++my;
                    ia = row_beg[my] + (fa - row_off[my]);
                }
                if (inb) {
                    while (fb >= row_off[my + 1]) ++my;
                    ib = row_beg[my] + (fb - row_off[my]);
                }
                const int ga = ina ? gi[ia] : 0, gb = inb ? gi[ib] : 0;
                const float ka = ina ? sqdist(gs, stride, ia, D, q) : INFINITY;
                const float kb = inb ? sqdist(gs, stride, ib, D, q) : INFINITY;
                take(ka, ina, ga);
                take(kb, inb, gb);
            }
            if (over && cnt > 4 * kStore) return cnt;   // far above the window
            __syncwarp();
        }
        return cnt;
    }
};

// groups of at most this many points keep every key in registers (10 per
// lane: the generation's groups hold about P/C = 256 points; fewer slots
// send the larger groups to the cell grid, more cost every query the
// empty slots) and search the threshold on them, without the cell grid.
// (Copies of the search for 8 and 9 slots, taken by the smaller groups,
// made the kernel slower: 40.3 -> 43.7 ms a 256-road generation.)
constexpr int kRegKeys = 10;
constexpr int kReg = 32 * kRegKeys;

// Per regression group (road, control): bounding box of the normalised
// points, a cell grid of about 32n/k cells (at most TO_KNN_GCELLS; a few
// points per cell, since rows are set up 32 at a time and cost little), and
// a counting sort of the points into it.  One CTA per group.
__global__ void __launch_bounds__(1024) k_knn_grid(to_rov_args a) {
    const int c = blockIdx.x, d = a.S + 1, P = a.P;
    const int n = a.npts[c], k = a.kc[c];
    __shared__ int s_cnt[TO_KNN_GCELLS];
    __shared__ unsigned s_umin[TO_LSM_MAXD], s_umax[TO_LSM_MAXD];
    __shared__ int s_bad;
    __shared__ int s_wsum[32];
    __shared__ to_knn_grid s_g;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const float* xs = a.xn + (size_t)c * d * P;
    if (tid < d) { s_umin[tid] = 0xFFFFFFFFu; s_umax[tid] = 0u; }
    if (tid == 0) s_bad = 0;
    if (c == 0 && tid == 0) *a.knn_next = 0;     // work counter of k_knn_rov
    __syncthreads();
    for (int j = 0; j < d; ++j) {
        float lo = INFINITY, hi = -INFINITY;
        bool bad = false;
        for (int m = tid; m < n; m += blockDim.x) {
            float x = xs[(size_t)j * P + m];
            bad = bad || !isfinite(x);
            lo = fminf(lo, x);
            hi = fmaxf(hi, x);
        }
        for (int o = 16; o > 0; o >>= 1) {
            lo = fminf(lo, __shfl_xor_sync(kFull, lo, o));
            hi = fmaxf(hi, __shfl_xor_sync(kFull, hi, o));
        }
        unsigned kl = __float_as_uint(lo), kh = __float_as_uint(hi);
        kl = (kl & 0x80000000u) ? ~kl : (kl | 0x80000000u);
        kh = (kh & 0x80000000u) ? ~kh : (kh | 0x80000000u);
        if (__any_sync(kFull, bad) && lane == 0) s_bad = 1;
        if (lane == 0) { atomicMin(&s_umin[j], kl); atomicMax(&s_umax[j], kh); }
    }
    __syncthreads();
    if (tid == 0) {
        to_knn_grid g;
        g.ok = (!s_bad && n >= 3 && k > 0) ? 1 : 0;
        int target = (k > 0) ? (int)(32LL * n / k) : 1;
        if (target < 1) target = 1;
        int gd = (int)floorf(powf((float)target, 1.0f / (float)d));
        if (gd < 1) gd = 1;
        if (gd > 64) gd = 64;
        for (;;) {
            long long cells = 1;
            for (int j = 0; j < d; ++j) cells *= gd;
            if (cells <= TO_KNN_GCELLS || gd == 1) break;
            --gd;
        }
        for (int j = 0; j < TO_LSM_MAXD; ++j) {
            g.lo[j] = 0.0f; g.hi[j] = 0.0f; g.inv[j] = 0.0f; g.w[j] = 0.0f; g.G[j] = 1;
        }
        for (int j = 0; j < d; ++j) {
            unsigned kl = s_umin[j], kh = s_umax[j];
            kl = (kl & 0x80000000u) ? (kl & 0x7FFFFFFFu) : ~kl;
            kh = (kh & 0x80000000u) ? (kh & 0x7FFFFFFFu) : ~kh;
            float lo = __uint_as_float(kl), hi = __uint_as_float(kh);
            float ext = hi - lo;
            g.lo[j] = lo;
            g.hi[j] = hi;
            if (ext > 0.0f && isfinite(ext) && (float)gd / ext < INFINITY) {
                g.G[j] = gd;
                g.inv[j] = (float)gd / ext;
                g.w[j] = ext / (float)gd;
            }
        }
        if (!g.ok) for (int j = 0; j < TO_LSM_MAXD; ++j) { g.lo[j] = g.hi[j] = 0.0f; }
        // a query's first threshold when it has no k-th distance from the
        // year before: the squared width of the widest cell
        float T0 = 0.0f;
        for (int j = 0; j < d; ++j)
            if (g.inv[j] > 0.0f) T0 = fmaxf(T0, 1.0f / (g.inv[j] * g.inv[j]));
        if (!(T0 > 0.0f) && n > 0 && k > 0) T0 = powf((float)k / (float)n, 2.0f / (float)d);
        g.T0 = T0;
        s_g = g;
        a.ggrid[c] = g;
    }
    __syncthreads();
    // groups the register search takes need only the box (T0), not the cells
    if (!s_g.ok || n <= kReg) return;
    int ncell = 1;
    for (int j = 0; j < d; ++j) ncell *= s_g.G[j];
    for (int i = tid; i < ncell; i += blockDim.x) s_cnt[i] = 0;
    __syncthreads();
    auto cell_idx = [&](int m) {
        int cell = 0, mul = 1;
        for (int j = 0; j < d; ++j) {
            cell += cell_of(xs[(size_t)j * P + m], s_g.lo[j], s_g.inv[j], s_g.G[j]) * mul;
            mul *= s_g.G[j];
        }
        return cell;
    };
    for (int m = tid; m < n; m += blockDim.x) atomicAdd(&s_cnt[cell_idx(m)], 1);
    __syncthreads();
    // exclusive scan of the counts: 4 consecutive cells per thread
    int* gc = a.gcell + (size_t)c * (TO_KNN_GCELLS + 1);
    int v[4], loc = 0;
    for (int u = 0; u < 4; ++u) {
        int i = tid * 4 + u;
        v[u] = (i < ncell) ? s_cnt[i] : 0;
        loc += v[u];
    }
    int incl = loc;
    for (int o = 1; o < 32; o <<= 1) {
        int t2 = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += t2;
    }
    if (lane == 31) s_wsum[warp] = incl;
    __syncthreads();
    int wbase = 0;
    for (int w = 0; w < warp; ++w) wbase += s_wsum[w];
    int run = wbase + incl - loc;
    __syncthreads();
    for (int u = 0; u < 4; ++u) {
        int i = tid * 4 + u;
        if (i < ncell) { s_cnt[i] = run; gc[i] = run; }
        run += v[u];
    }
    if (tid == 0) gc[ncell] = n;
    __syncthreads();
    float* gs = a.gsx + (size_t)c * d * P;
    int* gi = a.gsi + (size_t)c * P;
    for (int m = tid; m < n; m += blockDim.x) {
        int pos = atomicAdd(&s_cnt[cell_idx(m)], 1);
        for (int j = 0; j < d; ++j) gs[(size_t)j * P + pos] = xs[(size_t)j * P + m];
        gi[pos] = m;
    }
}

// ROV: kNN + multiLocLinReg fused.  Persistent warps take (control, grid
// query) items from a counter, so no warp waits on another: items differ a
// lot in cost (queries outside the point cloud need wide radii).  A query's
// threshold starts from its k-th distance of the year before, times
// kSeedGrow (kSeedGrowReg where the keys are in registers).  After the
// selection every lane accumulates the normal equations of neighbours lane,
// lane+32, ... of the k nearest in ascending point index; the 32 partials
// of each sum are added in lane order through shared memory, and the
// item's sums are stored as doubles at its list position.  k_knn_solve
// then solves one system per thread (FP64 square-root-free Cholesky,
// to_lsm_math.h).
constexpr float kSeedGrow = 1.4f;
// the register search re-counts cheaply: it starts from last year's k-th
// distance itself (about k keys qualify)
constexpr float kSeedGrowReg = 1.0f;

// The k nearest of keys held in registers (lane l holds points l, l+32,
// ...): the threshold moves until exactly k keys are at or below it; where
// equal keys straddle the k-th place, every key below the tied value is
// taken and then the lowest-index keys at it - the k smallest by (key,
// index).  The k points go to ws.sel in ascending point index (the order
// the regression sums them in).  Returns the k-th smallest key, or -1 when
// the threshold leaves the finite range (the caller falls back).
__device__ float reg_select_exact(const float (&key)[kRegKeys], int k, int dim, float T,
                                  WarpScratch& ws) {
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    const float expo = 2.0f / (float)dim;
    float lo = -1.0f, hi = -1.0f;
    bool tie = false;
    for (int iter = 0;; ++iter) {
        if (iter == 200 || !(T < INFINITY) || !(T >= 0.0f)) return -1.0f;
        unsigned mine = 0;
#pragma unroll
        for (int u = 0; u < kRegKeys; ++u) mine += (key[u] <= T) ? 1u : 0u;
        const int cnt = (int)__reduce_add_sync(kFull, mine);
        if (cnt == k) break;
        if (!exact_step(cnt, k, expo, T, lo, hi)) { tie = true; break; }
    }
    // tie: lo and hi are adjacent floats, fewer than k keys <= lo and more
    // than k <= hi, so the keys in between all equal hi
    int need = 0;
    if (tie) {
        unsigned below = 0;
#pragma unroll
        for (int u = 0; u < kRegKeys; ++u) below += (key[u] < hi) ? 1u : 0u;
        need = k - (int)__reduce_add_sync(kFull, below);
    }
    int pos = 0, eqs = 0;
    unsigned top = 0;
#pragma unroll
    for (int u = 0; u < kRegKeys; ++u) {
        bool take;
        if (!tie) {
            take = key[u] <= T;
        } else {
            const bool eq = key[u] == hi;
            const unsigned me = __ballot_sync(kFull, eq);
            take = key[u] < hi || (eq && eqs + __popc(me & lt_mask) < need);
            eqs += __popc(me);
        }
        const unsigned m = __ballot_sync(kFull, take);
        if (take) {
            ws.sel[pos + __popc(m & lt_mask)] = pack_sel(key[u], lane + 32 * u);
            top = max(top, __float_as_uint(key[u]));
        }
        pos += __popc(m);
    }
    __syncwarp();
    return __uint_as_float(__reduce_max_sync(kFull, top));
}

// ws.sel[0..k) from (key, index) order into ascending index order: the
// words swapped, one sort, swapped back
__device__ __noinline__ void to_index_order(WarpScratch& ws, int k) {
    const int lane = threadIdx.x & 31;
    for (int i = lane; i < k; i += 32) {
        const unsigned long long v = ws.sel[i];
        ws.sel[i] = (v << 32) | (v >> 32);
    }
    __syncwarp();
    warp_sort_sel(ws, k);
    for (int i = lane; i < k; i += 32) {
        const unsigned long long v = ws.sel[i];
        ws.sel[i] = (v << 32) | (v >> 32);
    }
    __syncwarp();
}

template <int D>
__host__ __device__ constexpr int knn_acc_len() { return (D + 1) + (D + 1) * (D + 1); }
// the sums a regression keeps: (D + 1) right-hand sides, then the upper
// triangle i <= j of the (D + 1)^2 matrix in row order
template <int D>
__host__ __device__ constexpr int knn_sums() { return (D + 1) + (D + 1) * (D + 2) / 2; }

size_t knn_rov_smem() { return sizeof(WarpScratch) * kWarps; }

template <int D>
__global__ void __launch_bounds__(kWarps * 32, 4)
k_knn_rov(to_rov_args a, int t) {
    extern __shared__ __align__(16) unsigned char sm_raw[];
    constexpr int M = D + 1, NA = knn_acc_len<D>();
    constexpr int NS = knn_sums<D>();
    const int P = a.P, Q = a.Q;
    const int lane = threadIdx.x & 31;
    WarpScratch& ws = reinterpret_cast<WarpScratch*>(sm_raw)[threadIdx.x >> 5];
    // (group, query) items, group g = road*C + control: every grid query, or
    // the year's list of the queries the backward pass reads
    const int items = a.touched ? *a.qcount : a.G * Q;
    const bool qpow2 = (Q & (Q - 1)) == 0;
    const int qshift = qpow2 ? __ffs(Q) - 1 : 0;
    // two positions of the year's list a request (half the round trips to
    // the counter) where the list holds at least two items a warp; one
    // where it is short (a single road), so that no warp waits idle
    const int take = (items >= 2 * (int)gridDim.x * kWarps) ? 2 : 1;
    for (;;) {
        int l0 = 0;
        if (lane == 0) l0 = atomicAdd(a.knn_next, take);
        l0 = __shfl_sync(kFull, l0, 0);
        if (l0 >= items) break;
        for (int li = l0; li < l0 + take && li < items; ++li) {
            const int item = a.touched ? a.qlist[li] : li;
            const int c = qpow2 ? (item >> qshift) : item / Q;
            const int qi = item - c * Q;
            const int n = a.npts[c], k = a.kc[c];
            if (n < 3 || k <= 0) continue;           // k_knn_solve writes 0
            const float* xs = a.xn + (size_t)c * D * P;
            const float* y = a.yv + (size_t)c * P;
            const float* xr = a.xraw + (size_t)c * D * P;
            const float T0 = a.ggrid[c].T0;
            float* kth_prev = a.kth + (size_t)c * Q;
            const float kp = kth_prev[qi];
            float T = kp > 0.0f ? kp * kSeedGrow : T0;
            float qn[D], xq[D];
            to_rov_query<D>(a, c / a.C, qi, qn, xq);
            // the k nearest into ws.sel in ascending point index; kth = the k-th
            // smallest distance (squared)
            float kth = -1.0f;
            if (n <= kReg) {
                float key[kRegKeys];
#pragma unroll
                for (int u = 0; u < kRegKeys; ++u) {
                    const int i = lane + 32 * u;
                    key[u] = (i < n) ? sqdist(xs, P, i, D, qn) : INFINITY;
                }
                kth = reg_select_exact(key, k, D, kp > 0.0f ? kp * kSeedGrowReg : T0, ws);
            } else {
                if (a.ggrid[c].ok) {
                    // the cell grid, copied only where it is used
                    const to_knn_grid g = a.ggrid[c];
                    GridPass<D> gp{&g, a.gsx + (size_t)c * D * P, a.gsi + (size_t)c * P,
                                   a.gcell + (size_t)c * (TO_KNN_GCELLS + 1), P, qn, &ws, k};
                    kth = threshold_select(k, D, T, ws, gp);
                } else {
                    ScanPass sp{xs, P, n, D, qn, &ws};
                    kth = threshold_select(k, D, T, ws, sp);
                }
                if (kth >= 0.0f) to_index_order(ws, k);
            }
            if (kth < 0.0f) {                         // exact radix selection
                warp_select(xs, P, n, D, qn, k, ws);
                kth = __uint_as_float((unsigned)(ws.sel[k - 1] >> 32));
                to_index_order(ws, k);
            }
            if (lane == 0) kth_prev[qi] = kth;
            // lane-strided local linear regression
            float acc[NA];
            to_lsm_acc_init(D, acc);
            const float h = sqrtf(kth), rh = 1.0f / h;
            for (int kk = lane; kk < k; kk += 32) {
                const unsigned long long v = ws.sel[kk];
                const int i = (int)(v & 0xFFFFFFFFu);
                const float dd = sqrtf(__uint_as_float((unsigned)(v >> 32)));
                float xv[D];
#pragma unroll
                for (int j = 0; j < D; ++j) {
                    if (a.sem == 0) {
                        // the reference reads its dim-major buffer (stride n)
                        // point-major (multiLocLinReg, SimulateGPU.cu:3002)
                        int f = i * D + j;
                        int jj = f / n, m = f - jj * n;
                        xv[j] = xr[(size_t)jj * P + m];
                    } else {
                        xv[j] = xs[(size_t)j * P + i];
                    }
                }
                // dd <= h: every neighbour lies within the k-th distance
                to_lsm_acc_add(D, acc, to_lsm_weight_within(dd, h, rh), y[i], xv, xq);
            }
            // the item's NS sums, at its list position
            double* sa = a.knn_acc + (size_t)li * NS;
            // the normal-equation sums: every lane's partials into shared memory
            // (sum e in row e, lane in column, rows 33 wide), then lane e adds
            // row e's 32 partials in lane order
            static_assert(NS * 33 * sizeof(float) <= sizeof(WarpScratch), "reduction rows");
            float* red = reinterpret_cast<float*>(&ws);
            __syncwarp();
            {
                int e = 0;
#pragma unroll
                for (int i = 0; i < M; ++i) red[(e++) * 33 + lane] = acc[i];
#pragma unroll
                for (int i = 0; i < M; ++i)
#pragma unroll
                    for (int j = i; j < M; ++j) red[(e++) * 33 + lane] = acc[M + i * M + j];
            }
            __syncwarp();
            if (lane < NS) {
                float x = red[lane * 33];
#pragma unroll 8
                for (int l = 1; l < 32; ++l) x = x + red[lane * 33 + l];
                sa[lane] = (double)x;                // exact; spares the solve a conversion
            }
            __syncwarp();
        }
    }
}

// One regression system per thread over the year's list, 128 at a time: a
// chunk's sums (NS doubles a system, consecutive list positions) are copied
// to shared memory word by word with consecutive threads on consecutive
// words (rows padded to an odd stride), then each thread solves its own and
// writes the intercept at grid query qi of group c (0 where the group has
// too few points).
template <int D>
__global__ void __launch_bounds__(128) k_knn_solve(to_rov_args a, int t) {
    constexpr int NS = knn_sums<D>(), NSP = NS | 1;
    __shared__ double s[128 * NSP];
    const int total = a.touched ? *a.qcount : a.G * a.Q;
    for (int base = blockIdx.x * 128; base < total; base += gridDim.x * 128) {
        const int cnt = min(128, total - base);
        __syncthreads();
        const double* src = a.knn_acc + (size_t)base * NS;
        for (int q = threadIdx.x; q < cnt * NS; q += 128) {
            const int i = q / NS;
            s[i * NSP + (q - i * NS)] = src[q];
        }
        __syncthreads();
        if ((int)threadIdx.x >= cnt) continue;
        const int li = base + threadIdx.x;
        const int item = a.touched ? a.qlist[li] : li;
        if (item >= a.G * a.Q) continue;
        const int c = item / a.Q, qi = item - c * a.Q;
        const int n = a.npts[c], k = a.kc[c];
        const float y = (n >= 3 && k > 0) ? to_lsm_solve_compact(D, s + threadIdx.x * NSP) : 0.0f;
        (to_rov_reg_block(a, t, c) + (size_t)a.R * D)[qi] = y;
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
    ScanPass sp{ref, n, n, dim, q, &ws};
    // the k nearest, then sorted by (distance, index) as the reference returns them
    if (threshold_select(k, dim, T, ws, sp) >= 0.0f) warp_sort_sel(ws, k);
    else warp_select(ref, n, n, dim, q, k, ws);
    for (int kk = lane; kk < k; kk += 32) {
        unsigned long long v = ws.sel[kk];
        dist[(size_t)kk * Q + qi] = sqrtf(__uint_as_float((unsigned)(v >> 32)));
        ind[(size_t)kk * Q + qi] = (int)(v & 0xFFFFFFFFu) + 1;
    }
}

template <int D>
to_status launch_knn_rov(to_ctx ctx, const to_rov_args& a, int t) {
    const size_t smem = knn_rov_smem();
    TO_CUDA(ctx, cudaFuncSetAttribute(k_knn_rov<D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    int per_sm = 0;
    TO_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_knn_rov<D>,
                                                               kWarps * 32, smem));
    if (per_sm < 1) per_sm = 1;
    const int items = a.G * a.Q;
    int grid = (ctx->sm_count > 0 ? ctx->sm_count : 152) * per_sm;
    if (grid > (items + kWarps - 1) / kWarps) grid = (items + kWarps - 1) / kWarps;
    to_prof_begin(ctx, "knn");
    k_knn_rov<D><<<grid, kWarps * 32, smem, ctx->stream>>>(a, t);
    to_prof_end(ctx);
    TO_LAUNCHED(ctx);
    to_prof_begin(ctx, "knn_solve");
    const int sblocks = (items + 127) / 128;
    const int smax = (ctx->sm_count > 0 ? ctx->sm_count : 152) * 16;
    k_knn_solve<D><<<sblocks < smax ? sblocks : smax, 128, 0, ctx->stream>>>(a, t);
    to_prof_end(ctx);
    TO_LAUNCHED(ctx);
    return TO_OK;
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
    if (d < 2 || d > TO_LSM_MAXD)
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "regression dimension %d", d);
    to_prof_begin(ctx, "knn_grid");
    k_knn_grid<<<a.G, 1024, 0, ctx->stream>>>(a);
    to_prof_end(ctx);
    TO_LAUNCHED(ctx);
    switch (d) {
        case 2: TO_TRY(launch_knn_rov<2>(ctx, a, t)); break;
        case 3: TO_TRY(launch_knn_rov<3>(ctx, a, t)); break;
        case 4: TO_TRY(launch_knn_rov<4>(ctx, a, t)); break;
        default: TO_TRY(launch_knn_rov<5>(ctx, a, t)); break;
    }
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
