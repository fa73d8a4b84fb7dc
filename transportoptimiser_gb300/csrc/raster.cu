// raster.cu - road cells of a generation of polylines on the device, and the
// per-road features the learned surrogate reads.
//
// The reference builds a road's cells on the host once per road per
// evaluation (RoadCells::computeRoadCells, include/road/RoadCells.cpp:10-272):
// each span between consecutive road points is cut at its crossings of the
// grid lines x = k xs and y = k ys, the span's points are sorted by (x, y)
// (ascending when the span runs towards larger x, else descending), equal
// neighbours are dropped, and each piece between consecutive points lies in
// the cell (ceil(mid_x / xs), ceil(mid_y / ys)) of its midpoint.  Here a CTA
// per road has each warp take one span at a time: the lanes write the
// span's crossings to shared memory, rank them (the same order an
// insertion sort gives: a point's rank counts the points before it, ties
// by position), and mark the midpoint cells of consecutive points in a
// shared-memory bitmap of the grid; the road's cells leave in ascending
// order.  The arithmetic is the reference's, operation for operation, in
// double; `sem` 0 keeps its quirk for the x of a vertical-line crossing
// (computed from row q of the crossing list, RoadCells.cpp:189-194), 1 uses
// the crossing's own y.
#include "to_internal.cuh"
#include "to_model.cuh"

namespace {

constexpr int kRasterWarps = 4;
constexpr int kSpanMax = 1024;         // crossings of one span
struct SpanPt { double x, y; };

__device__ __forceinline__ bool pt_less(SpanPt a, SpanPt b) {
    return a.x < b.x || (a.x == b.x && a.y < b.y);
}

struct RasterArgs {
    const int* seg_off;
    const double* segs;
    int W, H, sem;
    double xs, ys;
    int* flags;
};

// marks the cells of road r in the bitmap (W*H bits); scratch: per warp
// two buffers of kSpanMax points
__device__ void mark_road(int r, const RasterArgs& a, unsigned* bits, SpanPt* scratch) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    SpanPt* raw = scratch + (size_t)warp * 2 * kSpanMax;
    SpanPt* srt = raw + kSpanMax;
    const double xs = a.xs, ys = a.ys;
    const int g0 = a.seg_off[r], g1 = a.seg_off[r + 1];
    for (int g = g0 + warp; g < g1; g += nw) {
        const double x0 = a.segs[4 * (size_t)g], y0 = a.segs[4 * (size_t)g + 1];
        const double x1 = a.segs[4 * (size_t)g + 2], y1 = a.segs[4 * (size_t)g + 3];
        const int h = (int)(x1 / xs) - (int)(x0 / xs);
        const int v = (int)(y1 / ys) - (int)(y0 / ys);
        const int ah = h < 0 ? -h : h, av = v < 0 ? -v : v, n = ah + av;
        if (n > kSpanMax) {                    // longer than any span inside the grid
            if (lane == 0 && a.flags) atomicExch(a.flags, TO_DEVERR_CELL);
            continue;
        }
        const double m = (y1 - y0) / (x1 - x0), b = y0 - x0 * m;
        const double m2 = (x1 - x0) / (y1 - y0), b2 = x0 - y0 * m2;
        const bool mf = isfinite(m), m2f = isfinite(m2);
        for (int q = lane; q < ah; q += 32) {
            double px;
            if (h > 0) px = xs * (floor(x0 / xs) + (double)(q + 1));
            else if (fmod(x0, xs) == 0.0) px = xs * (ceil(x0 / xs) - (double)q);
            else px = xs * (ceil(x0 / xs) - (double)(q + 1));
            raw[q].x = px;
            raw[q].y = mf ? m * px + b : y0;
        }
        for (int q = lane; q < av; q += 32) {
            double py;
            if (v > 0) py = ys * (floor(y0 / ys) + (double)(q + 1));
            else if (fmod(y0, ys) == 0.0) py = ys * (ceil(y0 / ys) - (double)q);
            else py = ys * (ceil(y0 / ys) - (double)(q + 1));
            raw[ah + q].y = py;
        }
        __syncwarp();
        for (int q = lane; q < av; q += 32) {
            const double src = (a.sem == 0) ? raw[q].y : raw[ah + q].y;
            raw[ah + q].x = mf ? (src - b) / m : (m2f ? b2 + m2 * src : x0);
        }
        __syncwarp();
        const bool asc = x1 >= x0;
        for (int i = lane; i < n; i += 32) {
            const SpanPt pi = raw[i];
            int rank = 0;
            for (int j = 0; j < n; ++j) {
                const SpanPt pj = raw[j];
                const bool before = asc ? pt_less(pj, pi) : pt_less(pi, pj);
                const bool tie = !pt_less(pj, pi) && !pt_less(pi, pj);
                rank += (before || (tie && j < i)) ? 1 : 0;
            }
            srt[rank] = pi;
        }
        __syncwarp();
        for (int k = lane; k <= n; k += 32) {
            SpanPt pa, pb;
            if (k == 0) { pa.x = x0; pa.y = y0; } else pa = srt[k - 1];
            if (k == n) { pb.x = x1; pb.y = y1; } else pb = srt[k];
            if (pa.x == pb.x && pa.y == pb.y) continue;
            const double cxd = ceil((0.5 * (pa.x + pb.x) - 0.0) / xs);
            const double cyd = ceil((0.5 * (pa.y + pb.y) - 0.0) / ys);
            if (!(cxd >= 0.0 && cxd < (double)a.W && cyd >= 0.0 && cyd < (double)a.H)) continue;
            const int c = (int)cxd + (int)cyd * a.W;
            atomicOr(&bits[c >> 5], 1u << (c & 31));
        }
        __syncwarp();
    }
}

__device__ __forceinline__ SpanPt* span_scratch(unsigned* bits, int nw) {
    return reinterpret_cast<SpanPt*>(bits + ((nw + 3) & ~3));
}

__global__ void k_raster_count(int R, RasterArgs ra, int* __restrict__ counts) {
    extern __shared__ __align__(16) unsigned bits[];
    __shared__ int s_c;
    const int r = blockIdx.x;
    const int W = ra.W, H = ra.H;
    const int nw = (W * H + 31) >> 5;
    for (int i = threadIdx.x; i < nw; i += blockDim.x) bits[i] = 0u;
    if (threadIdx.x == 0) s_c = 0;
    __syncthreads();
    mark_road(r, ra, bits, span_scratch(bits, nw));
    __syncthreads();
    int c = 0;
    for (int i = threadIdx.x; i < nw; i += blockDim.x) c += __popc(bits[i]);
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&s_c, c);
    __syncthreads();
    if (threadIdx.x == 0) counts[r] = s_c;
}

// exclusive scan of counts[0..R) into off[0..R] (one CTA)
__global__ void k_scan_counts(int R, const int* __restrict__ counts, int* __restrict__ off,
                              int max_cells, int* flags) {
    __shared__ int s_w[32];
    const int nt = blockDim.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int carry = 0;
    for (int b = 0; b < R; b += nt) {
        const int i = b + threadIdx.x;
        const int v = i < R ? counts[i] : 0;
        int x = v;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_w[warp] = x;
        __syncthreads();
        int wb = 0, tot = 0;
        for (int w = 0; w < (nt >> 5); ++w) { if (w < warp) wb += s_w[w]; tot += s_w[w]; }
        if (i < R) off[i] = carry + wb + x - v;
        carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        off[R] = carry;
        if (carry > max_cells && flags) atomicExch(flags, TO_DEVERR_PATCHES);
    }
}

__global__ void k_raster_write(int R, RasterArgs ra, const int* __restrict__ off, int max_cells,
                               int* __restrict__ cells) {
    extern __shared__ __align__(16) unsigned bits[];
    __shared__ int s_w[32];
    const int r = blockIdx.x;
    const int W = ra.W, H = ra.H;
    const int nw = (W * H + 31) >> 5;
    for (int i = threadIdx.x; i < nw; i += blockDim.x) bits[i] = 0u;
    __syncthreads();
    mark_road(r, ra, bits, span_scratch(bits, nw));
    __syncthreads();
    // ascending cell order: each thread takes a contiguous run of words
    const int nt = blockDim.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int chunk = (nw + nt - 1) / nt;
    const int w0 = threadIdx.x * chunk, w1 = min(nw, w0 + chunk);
    int c = 0;
    for (int i = w0; i < w1; ++i) c += __popc(bits[i]);
    int x = c;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_w[warp] = x;
    __syncthreads();
    int wb = 0;
    for (int w = 0; w < warp; ++w) wb += s_w[w];
    int pos = off[r] + wb + x - c;
    for (int i = w0; i < w1; ++i) {
        unsigned b = bits[i];
        while (b) {
            const int j = __ffs(b) - 1;
            b &= b - 1;
            if (pos < max_cells) cells[pos] = i * 32 + j;
            ++pos;
        }
    }
}

__device__ __forceinline__ int bit_at(const unsigned* b, int c) { return (b[c >> 5] >> (c & 31)) & 1; }

// proper intersection of segments p1-p2 and p3-p4 (double)
__device__ __forceinline__ int seg_hit(double x1, double y1, double x2, double y2, double x3,
                                       double y3, double x4, double y4) {
    const double d = (x2 - x1) * (y4 - y3) - (y2 - y1) * (x4 - x3);
    if (d == 0.0) return 0;
    const double ua = ((x3 - x1) * (y4 - y3) - (y3 - y1) * (x4 - x3)) / d;
    const double ub = ((x3 - x1) * (y2 - y1) - (y3 - y1) * (x2 - x1)) / d;
    return (ua >= 0.0 && ua <= 1.0 && ub >= 0.0 && ub <= 1.0) ? 1 : 0;
}

// the same test in FP32 on a segment given as origin + direction
__device__ __forceinline__ int seg_hit_f(float x1, float y1, float dx, float dy, float x3,
                                         float y3, float ex, float ey) {
    const float d = dx * ey - dy * ex;
    if (d == 0.0f) return 0;
    const float ua = ((x3 - x1) * ey - (y3 - y1) * ex) / d;
    const float ub = ((x3 - x1) * dy - (y3 - y1) * dx) / d;
    return (ua >= 0.0f && ua <= 1.0f && ub >= 0.0f && ub <= 1.0f) ? 1 : 0;
}

constexpr int kFeatSegs = 256;           // segments staged in shared memory

// 16 features per road (surrogate inputs):
//  0 length / W, 1 segments / 64, 2 road cells / W, 3 / 4 crossing
//  exposure: road crossings per animal of species 0 moving 5 / 12 cells
//  (probes from a 5-cell lattice in 8 directions, weighted by the animals
//  at both ends), 5..7 share of the road's cells on habitat codes 2, 3, 5,
//  8 share of species 0's initial animals on road cells, 9..11 share of
//  them within 3, 6, 12 cells of the road (Chebyshev distance: the animals
//  at risk), 12 / 13 bounding-box width / height / W, 14 share within 24
//  cells, 15 sinuosity / 10.
// The "within r" sets are the road bitmap dilated by a (2r+1)^2 square,
// row windows then column windows, a thread per row / column.
__global__ void k_road_features(int R, int W, int H, const int* __restrict__ base,
                                const float* __restrict__ popmap, const int* __restrict__ seg_off,
                                const double* __restrict__ segs, const int* __restrict__ cell_off,
                                const int* __restrict__ cells, float* __restrict__ feat) {
    extern __shared__ unsigned fbits[];
    const int r = blockIdx.x;
    const int n = W * H, nw = (n + 31) >> 5;
    unsigned* road = fbits;          // [nw]
    unsigned* rowd = fbits + nw;     // [nw] row-dilated
    __shared__ double s_acc[18];
    __shared__ double s_tot;
    if (threadIdx.x < 18) s_acc[threadIdx.x] = 0.0;
    if (threadIdx.x == 0) s_tot = 0.0;
    for (int i = threadIdx.x; i < nw; i += blockDim.x) road[i] = 0u;
    __syncthreads();
    double tot = 0.0, loss = 0.0, hist[5] = {0, 0, 0, 0, 0};
    for (int i = threadIdx.x; i < n; i += blockDim.x) tot += popmap[i];
    const int c0 = cell_off[r], c1 = cell_off[r + 1];
    for (int q = c0 + threadIdx.x; q < c1; q += blockDim.x) {
        const int c = cells[q];
        const int t = base[c];
        const int b = t < 3 ? t : (t == 3 ? 3 : (t == 5 ? 4 : -1));
        if (b >= 0) hist[b] += 1.0;
        loss += popmap[c];
        atomicOr(&road[c >> 5], 1u << (c & 31));
    }
    atomicAdd(&s_tot, tot);
    atomicAdd(&s_acc[8], loss);
    for (int b = 2; b < 5; ++b) atomicAdd(&s_acc[3 + b], hist[b]);
    const int g0 = seg_off[r], g1 = seg_off[r + 1];
    __shared__ float s_seg[4][kFeatSegs];    // x3, y3, x4 - x3, y4 - y3
    const bool seg_smem = g1 - g0 <= kFeatSegs;
    if (seg_smem)
        for (int g = threadIdx.x; g < g1 - g0; g += blockDim.x) {
            const double* sg = segs + 4 * (size_t)(g0 + g);
            s_seg[0][g] = (float)sg[0];
            s_seg[1][g] = (float)sg[1];
            s_seg[2][g] = (float)(sg[2] - sg[0]);
            s_seg[3][g] = (float)(sg[3] - sg[1]);
        }
    __syncthreads();
    {
        // crossing exposure of animals moving 5 and 12 cells in 8 directions
        // (FP32: surrogate inputs, compared only through the network)
        const float kc = 0.70710678f;
        const float dir_x[8] = {1.0f, kc, 0.0f, -kc, -1.0f, -kc, 0.0f, kc};
        const float dir_y[8] = {0.0f, kc, 1.0f, kc, 0.0f, -kc, -1.0f, -kc};
        const int nx = (W + 4) / 5, ny = (H + 4) / 5;
        const int nprobe = nx * ny * 16;
        double ex[2] = {0.0, 0.0}, ew[2] = {0.0, 0.0};
        for (int q = threadIdx.x; q < nprobe; q += blockDim.x) {
            const int dir = q & 7, di = (q >> 3) & 1, cell = q >> 4;
            const int ix = cell % nx, iy = cell / nx;
            const int x0 = 5 * ix + 2, y0 = 5 * iy + 2;
            if (x0 >= W || y0 >= H) continue;
            const float dist = di ? 12.0f : 5.0f;
            const float dx = dist * dir_x[dir], dy = dist * dir_y[dir];
            const int cx1 = (int)rintf((float)x0 + dx), cy1 = (int)rintf((float)y0 + dy);
            if (cx1 < 0 || cx1 >= W || cy1 < 0 || cy1 >= H) continue;
            const double w = (double)popmap[x0 + y0 * W] * (double)popmap[cx1 + cy1 * W];
            if (!(w > 0.0)) continue;
            int hits = 0;
            if (seg_smem) {
                for (int g = 0; g < g1 - g0; ++g)
                    hits += seg_hit_f((float)x0, (float)y0, dx, dy, s_seg[0][g], s_seg[1][g],
                                      s_seg[2][g], s_seg[3][g]);
            } else {
                for (int g = g0; g < g1; ++g) {
                    const double* sg = segs + 4 * (size_t)g;
                    hits += seg_hit(x0, y0, x0 + dx, y0 + dy, sg[0], sg[1], sg[2], sg[3]);
                }
            }
            ex[di] += w * hits;
            ew[di] += w;
        }
        for (int d = 0; d < 2; ++d) {
            atomicAdd(&s_acc[3 + d], ex[d]);
            atomicAdd(&s_acc[16 + d], ew[d]);
        }
    }
    const int radii[4] = {3, 6, 12, 24};
    const int slot[4] = {9, 10, 11, 14};
    for (int ri = 0; ri < 4; ++ri) {
        const int rad = radii[ri];
        __syncthreads();
        for (int i = threadIdx.x; i < nw; i += blockDim.x) rowd[i] = 0u;
        __syncthreads();
        for (int y = threadIdx.x; y < H; y += blockDim.x) {
            int cnt = 0;
            for (int x = 0; x < rad && x < W; ++x) cnt += bit_at(road, x + y * W);
            for (int x = 0; x < W; ++x) {
                if (x + rad < W) cnt += bit_at(road, x + rad + y * W);
                if (x - rad - 1 >= 0) cnt -= bit_at(road, x - rad - 1 + y * W);
                if (cnt > 0) atomicOr(&rowd[(x + y * W) >> 5], 1u << ((x + y * W) & 31));
            }
        }
        __syncthreads();
        double at = 0.0;
        for (int x = threadIdx.x; x < W; x += blockDim.x) {
            int cnt = 0;
            for (int y = 0; y < rad && y < H; ++y) cnt += bit_at(rowd, x + y * W);
            for (int y = 0; y < H; ++y) {
                if (y + rad < H) cnt += bit_at(rowd, x + (y + rad) * W);
                if (y - rad - 1 >= 0) cnt -= bit_at(rowd, x + (y - rad - 1) * W);
                if (cnt > 0) at += popmap[x + y * W];
            }
        }
        atomicAdd(&s_acc[slot[ri]], at);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double len = 0.0;
        double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300;
        for (int g = g0; g < g1; ++g) {
            const double* sg = segs + 4 * (size_t)g;
            len += hypot(sg[2] - sg[0], sg[3] - sg[1]);
            xmin = fmin(xmin, fmin(sg[0], sg[2])); xmax = fmax(xmax, fmax(sg[0], sg[2]));
            ymin = fmin(ymin, fmin(sg[1], sg[3])); ymax = fmax(ymax, fmax(sg[1], sg[3]));
        }
        const double w = (double)W;
        const int nc = c1 - c0;
        const double T = s_tot > 0.0 ? s_tot : 1.0;
        float* f = feat + (size_t)r * 16;
        f[0] = (float)(len / w);
        f[1] = (float)((g1 - g0) / 64.0);
        f[2] = (float)(nc / w);
        f[3] = s_acc[16] > 0.0 ? (float)(s_acc[3] / s_acc[16]) : 0.0f;
        f[4] = s_acc[17] > 0.0 ? (float)(s_acc[4] / s_acc[17]) : 0.0f;
        for (int b = 2; b < 5; ++b) f[3 + b] = nc > 0 ? (float)(s_acc[3 + b] / nc) : 0.0f;
        f[8] = (float)(s_acc[8] / T);
        f[9] = (float)(s_acc[9] / T);
        f[10] = (float)(s_acc[10] / T);
        f[11] = (float)(s_acc[11] / T);
        f[12] = g1 > g0 ? (float)((xmax - xmin) / w) : 0.0f;
        f[13] = g1 > g0 ? (float)((ymax - ymin) / w) : 0.0f;
        f[14] = (float)(s_acc[14] / T);
        double ex = 0.0;
        if (g1 > g0) {
            const double* a = segs + 4 * (size_t)g0;
            const double* b = segs + 4 * (size_t)(g1 - 1);
            ex = hypot(b[2] - a[0], b[3] - a[1]);
        }
        f[15] = (float)((ex > 1e-9 ? len / ex : 1.0) / 10.0);
    }
}

}  // namespace

namespace to_k {

to_status rasterise_roads(to_ctx ctx, int R, const int* seg_off, const double* segs, int W, int H,
                          double xs, double ys, int sem, int* cell_off, int* cells, int max_cells,
                          int* counts_scratch) {
    const size_t nw = (size_t)((W * H + 31) >> 5);
    const size_t smem = ((nw + 3) & ~size_t(3)) * sizeof(unsigned) +
                        (size_t)kRasterWarps * 2 * kSpanMax * sizeof(SpanPt);
    if (smem > ctx->smem_optin)
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "grid %d x %d too large to rasterise", W, H);
    if (!(xs > 0.0) || !(ys > 0.0)) return to_set_error(ctx, TO_ERR_INVALID, "grid spacing");
    RasterArgs ra{seg_off, segs, W, H, sem, xs, ys, ctx->d_flags};
    TO_CUDA(ctx, cudaFuncSetAttribute(k_raster_count, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    TO_CUDA(ctx, cudaFuncSetAttribute(k_raster_write, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    to_prof_begin(ctx, "rasterise");
    k_raster_count<<<R, kRasterWarps * 32, smem, ctx->stream>>>(R, ra, counts_scratch);
    k_scan_counts<<<1, 1024, 0, ctx->stream>>>(R, counts_scratch, cell_off, max_cells, ctx->d_flags);
    k_raster_write<<<R, kRasterWarps * 32, smem, ctx->stream>>>(R, ra, cell_off, max_cells, cells);
    to_prof_end(ctx);
    ctx->launches += 3;
    TO_CUDA(ctx, cudaGetLastError());
    return TO_OK;
}

to_status road_features(to_ctx ctx, int R, int W, int H, const int* base, const float* popmap,
                        const int* seg_off, const double* segs, const int* cell_off,
                        const int* cells, float* feat) {
    const size_t smem = (size_t)2 * ((W * H + 31) >> 5) * sizeof(unsigned);
    if (smem > ctx->smem_optin)
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "grid %d x %d too large for features", W, H);
    TO_CUDA(ctx, cudaFuncSetAttribute(k_road_features, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    to_prof_begin(ctx, "road_features");
    k_road_features<<<R, 256, smem, ctx->stream>>>(R, W, H, base, popmap, seg_off, segs,
                                                    cell_off, cells, feat);
    to_prof_end(ctx);
    TO_LAUNCHED(ctx);
    return TO_OK;
}

}  // namespace to_k
