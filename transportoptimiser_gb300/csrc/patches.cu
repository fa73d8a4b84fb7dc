// patches.cu - habitat labelling, habitat patches, road crossings and the
// species-road migration model on the device.
//
// Reference path (TransportOptimiser):
//   LabelImage                       include/utilities/labelmethod.cpp:34-56
//   SimulateGPU::buildPatches        include/gpuCode/SimulateGPU.cu:3573-3645
//   patchComputation kernel          include/gpuCode/SimulateGPU.cu:498-573
//   SimulateGPU::lineSegmentIntersect SimulateGPU.cu:3478-3568 (+454-493)
//   SpeciesRoadPatches::createSpeciesModel include/road/SpeciesRoadPatches.cpp:12-451
//   dense2Sparse threshold           include/gpuCode/SimulateGPU.cu:5973-5996
//
// GB300 layout: one CTA per (road, species) keeps the whole label image in
// shared memory (W*H int32 <= 224 KB), labels it with a lock-free
// union-find (atomicMin on shared memory), extracts the patches, and then
// builds crossings, transition and survival probabilities and the
// destination-major float migration matrices for every control.  Nothing
// round-trips to the host between those steps.
#include "to_internal.cuh"
#include "to_model.cuh"

namespace {

#define TO_SURV_TABLE_SEGS 255         // survival table by crossing count up to this

__device__ __forceinline__ int uf_find(volatile int* par, int x) {
    int p = par[x];
    int guard = 0;
    while (p != x && guard < (1 << 20)) { x = p; p = par[x]; ++guard; }
    return x;
}

// Playne & Hawick style lock-free union: roots only ever decrease, so the
// loop makes progress on every failed attempt.
__device__ __forceinline__ bool uf_union(int* par, int a, int b) {
    volatile int* vp = par;
    for (int it = 0; it < (1 << 20); ++it) {
        a = uf_find(vp, a);
        b = uf_find(vp, b);
        if (a == b) return true;
        if (a < b) {
            int old = atomicMin(&par[b], a);
            if (old == b) return true;
            b = old;
        } else {
            int old = atomicMin(&par[a], b);
            if (old == a) return true;
            a = old;
        }
    }
    return false;
}

// Block-wide exclusive scan of one int per thread (blockDim.x <= 1024).
__device__ int cta_exclusive_scan(int v, int* s_tmp, int* total) {
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int nw = (blockDim.x + 31) >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_tmp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = (lane < nw) ? s_tmp[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        s_tmp[lane] = w;   // inclusive over warps
    }
    __syncthreads();
    int warp_base = (warp > 0) ? s_tmp[warp - 1] : 0;
    int tot = s_tmp[nw - 1];
    __syncthreads();
    if (total) *total = tot;
    return warp_base + x - v;
}

// Labels the foreground of a W*H image held as par[] in shared memory
// (par[i] = i for foreground, -1 for background on entry).  On exit par[i]
// holds the LabelImage number (1.. in raster order of first pixel) or 0.
// Returns the number of regions.
//
// Run-based: a thread per image row points every foreground pixel at the
// start of its horizontal run; vertical unions are made only where a run
// pair first touches (the pixel's left neighbour does not already link the
// same two runs), so the lock-free unions touch run starts only.
__device__ int cta_label(int n, int W, int* par, int* s_tmp, int* d_flags) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const int H = n / W;
    for (int y = tid; y < H; y += nt) {
        int start = -1;
        for (int x = 0; x < W; ++x) {
            const int i = x + y * W;
            if (par[i] < 0) { start = -1; continue; }
            if (start < 0) start = i;
            par[i] = start;
        }
    }
    __syncthreads();
    bool ok = true;
    for (int i = W + tid; i < n; i += nt) {
        if (par[i] < 0 || par[i - W] < 0) continue;
        const int x = i % W;
        if (x > 0 && par[i - 1] >= 0 && par[i - 1 - W] >= 0) continue;   // same run pair
        ok &= uf_union(par, par[i], par[i - W]);
    }
    if (!ok && d_flags) atomicExch(d_flags, TO_DEVERR_UNION);
    __syncthreads();
    for (int i = tid; i < n; i += nt)
        if (par[i] >= 0) par[i] = uf_find(par, par[i]);
    __syncthreads();
    // rank the roots (root = smallest raster index of its component)
    int chunk = (n + nt - 1) / nt;
    int lo = tid * chunk, hi = min(n, lo + chunk);
    int cnt = 0;
    for (int i = lo; i < hi; ++i) cnt += (par[i] == i);
    int total = 0;
    int base = cta_exclusive_scan(cnt, s_tmp, &total);
    for (int i = lo; i < hi; ++i)
        if (par[i] == i) par[i] = -(base++ + 2);
    __syncthreads();
    for (int i = tid; i < n; i += nt) {
        int v = par[i];
        if (v >= 0) par[i] = -par[v] - 1;      // non-root: label of its root
    }
    __syncthreads();
    for (int i = tid; i < n; i += nt) {
        int v = par[i];
        if (v <= -2) par[i] = -v - 1;           // root
        else if (v == -1) par[i] = 0;           // background
    }
    __syncthreads();
    return total;
}

// Extent of coarse block (bx, by) as patchComputation has it
// (SimulateGPU.cu:510-520: the x extent is bounded by H and the y extent by W).
__device__ __forceinline__ void block_extent(int bx, int by, int W, int H, int skpx, int skpy,
                                             int& bsx, int& bsy) {
    bsx = ((bx + 1) * skpx <= H) ? skpx : H - bx * skpx;
    bsy = ((by + 1) * skpy <= W) ? skpy : W - by * skpy;
}

// Finishes one patch exactly as patchComputation (SimulateGPU.cu:560-563).
__device__ __forceinline__ void finish_patch(int cnt, float pop, float sx, float sy, int bx,
        int by, int skpx, int skpy, float xs, float ys, float spa, float maxpop, float out[5]) {
    float area = (float)cnt;
    float cx = xs * (sx / area + (float)(bx * skpx));
    float cy = ys * (sy / area + (float)(by * skpy));
    area = area * spa;
    out[0] = area;
    out[1] = area * maxpop;
    out[2] = pop;
    out[3] = cx;
    out[4] = cy;
}

// In-place exclusive scan of v[0..n) by the whole CTA; returns the total.
__device__ int cta_scan_array(int* v, int n, int* s_tmp) {
    const int nt = blockDim.x;
    const int chunk = (n + nt - 1) / nt;
    const int lo = threadIdx.x * chunk, hi = min(n, lo + chunk);
    int sum = 0;
    for (int i = lo; i < hi; ++i) sum += v[i];
    int total = 0;
    int run = cta_exclusive_scan(sum, s_tmp, &total);
    for (int i = lo; i < hi; ++i) { int c = v[i]; v[i] = run; run += c; }
    __syncthreads();
    return total;
}

// Patches of one labelled image: every (coarse block, region) pair in block
// order (b = by * xres + bx), regions ascending within a block - the order
// the reference compacts them in.  A warp per block lists its distinct
// regions (counted first, then written at scanned offsets); then a thread
// per (block, region) accumulates count, population and centroid sums over
// the block's cells in the reference's order (x offset outer, y offset
// inner), so the float sums match it bit for bit.  Appends to the patch
// list at *s_count (shared).  s_list: nblocks + 1 + max_out ints of shared
// memory.  Returns false on overflow.
template <class LabelFn, class PopFn, class Emit>
__device__ bool cta_block_patches(int W, int H, int skpx, int skpy, int xres, int yres,
                                  int max_out, int* s_count, int* s_tmp, int* s_list,
                                  LabelFn lab, PopFn popf, Emit emit) {
    const int nblocks = xres * yres;
    int* s_off = s_list;                  // [nblocks + 1]
    int* s_lab = s_list + nblocks + 1;    // [max_out]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int base = *s_count;
    const int room = max_out - base;
    for (int pass = 0; pass < 2; ++pass) {
        for (int b = warp; b < nblocks; b += nw) {
            const int by = b / xres, bx = b - by * xres;
            int bsx, bsy;
            block_extent(bx, by, W, H, skpx, skpy, bsx, bsy);
            const int ncell = (bsx > 0 && bsy > 0) ? bsx * bsy : 0;
            const int out = pass ? s_off[b] : 0;
            int lastr = 0, cnt = 0;
            for (;;) {
                int mn = 0x7fffffff;
                for (int e = lane; e < ncell; e += 32) {
                    const int ii = e / bsy, jj = e - ii * bsy;
                    const int r = lab((bx * skpx + ii) + (by * skpy + jj) * W);
                    if (r > lastr && r < mn) mn = r;
                }
                mn = __reduce_min_sync(0xffffffffu, mn);
                if (mn == 0x7fffffff) break;
                if (pass && lane == 0 && out + cnt < room) s_lab[out + cnt] = mn;
                ++cnt;
                lastr = mn;
            }
            if (!pass && lane == 0) s_off[b] = cnt;
        }
        __syncthreads();
        if (!pass) {
            const int total = cta_scan_array(s_off, nblocks, s_tmp);
            if (threadIdx.x == 0) s_off[nblocks] = total;
            __syncthreads();
        }
    }
    const int total = s_off[nblocks];
    const int nemit = min(total, room > 0 ? room : 0);
    for (int t = threadIdx.x; t < nemit; t += blockDim.x) {
        int lo = 0, hi = nblocks;                 // block: last b with s_off[b] <= t
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (s_off[mid] <= t) lo = mid; else hi = mid;
        }
        const int b = lo, by = b / xres, bx = b - by * xres;
        int bsx, bsy;
        block_extent(bx, by, W, H, skpx, skpy, bsx, bsy);
        const int r = s_lab[t];
        int cnt = 0;
        float pop = 0.0f, sx = 0.0f, sy = 0.0f;
        for (int ii = 0; ii < bsx; ++ii)
            for (int jj = 0; jj < bsy; ++jj) {
                const int c = (bx * skpx + ii) + (by * skpy + jj) * W;
                if (lab(c) != r) continue;
                cnt += 1;
                pop = pop + popf(c);
                sx = sx + (float)ii;
                sy = sy + (float)jj;
            }
        emit(base + t, cnt, pop, sx, sy, bx, by);
    }
    __syncthreads();
    if (threadIdx.x == 0) *s_count = base + total;
    __syncthreads();
    return base + total <= max_out;
}

// ---- kernels ---------------------------------------------------------------

__global__ void k_label_image(int W, int H, const int* __restrict__ in,
                              int* __restrict__ out, int* n_regions,
                              int* d_flags) {
    extern __shared__ int smem[];
    int n = W * H;
    int* par = smem;
    int* s_tmp = smem + n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) par[i] = in[i] ? i : -1;
    __syncthreads();
    int nr = cta_label(n, W, par, s_tmp, d_flags);
    for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = par[i];
    if (threadIdx.x == 0) *n_regions = nr;
}

// buildPatches on given labels: out5[5*o + {area,cap,pop,cx,cy}] (double)
__global__ void k_build_patches(int W, int H, int skpx, int skpy, int xres,
                                int yres, float xs, float ys, float spa,
                                float maxpop, const int* __restrict__ labels,
                                const float* __restrict__ pops, int max_out,
                                double* __restrict__ out5, int* count,
                                int* d_flags) {
    extern __shared__ int s_list[];
    __shared__ int s_tmp[33];
    __shared__ int s_count;
    if (threadIdx.x == 0) s_count = *count;
    __syncthreads();
    auto lab = [&](int c) { return labels[c]; };
    auto popf = [&](int c) { return pops[c]; };
    auto emit = [&](int o, int cnt, float pop, float sx, float sy, int bx, int by) {
        float v[5];
        finish_patch(cnt, pop, sx, sy, bx, by, skpx, skpy, xs, ys, spa, maxpop, v);
        for (int f = 0; f < 5; ++f) out5[5 * (size_t)o + f] = (double)v[f];
    };
    bool ok = cta_block_patches(W, H, skpx, skpy, xres, yres, max_out, &s_count, s_tmp,
                                s_list, lab, popf, emit);
    if (!ok && d_flags) atomicExch(d_flags, TO_DEVERR_PATCHES);
    if (threadIdx.x == 0) *count = min(s_count, max_out);
}

// Segment-segment predicate in float without contraction
// (pathAdjacencyKernel, SimulateGPU.cu:465-476).
__device__ __forceinline__ int seg_cross(float x1, float y1, float x21,
                                         float y21, float x3, float y3,
                                         float x43, float y43) {
    float y13 = __fsub_rn(y1, y3);
    float x13 = __fsub_rn(x1, x3);
    float numa = __fsub_rn(__fmul_rn(x43, y13), __fmul_rn(y43, x13));
    float numb = __fsub_rn(__fmul_rn(x21, y13), __fmul_rn(y21, x13));
    float deno = __fsub_rn(__fmul_rn(y43, x21), __fmul_rn(x43, y21));
    float ua = __fdiv_rn(numa, deno);
    float ub = __fdiv_rn(numb, deno);
    return (ua >= 0.0f) && (ua <= 1.0f) && (ub >= 0.0f) && (ub <= 1.0f);
}

__global__ void k_line_segment_intersect(int T, const double* __restrict__ xy1,
                                         int G, const double* __restrict__ xy2,
                                         int* __restrict__ cross) {
    extern __shared__ float sseg[];   // 4*G: x3, y3, x43, y43
    for (int g = threadIdx.x; g < G; g += blockDim.x) {
        sseg[g] = (float)xy2[g];
        sseg[G + g] = (float)xy2[g + G];
        sseg[2 * G + g] = (float)(xy2[g + 2 * G] - xy2[g]);
        sseg[3 * G + g] = (float)(xy2[g + 3 * G] - xy2[g + G]);
    }
    __syncthreads();
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < T;
         t += gridDim.x * blockDim.x) {
        float x1 = (float)xy1[t], y1 = (float)xy1[t + T];
        float x21 = (float)(xy1[t + 2 * T] - xy1[t]);
        float y21 = (float)(xy1[t + 3 * T] - xy1[t + T]);
        int c = 0;
        for (int g = 0; g < G; ++g)
            c += seg_cross(x1, y1, x21, y21, sseg[g], sseg[G + g],
                           sseg[2 * G + g], sseg[3 * G + g]);
        cross[t] = c;
    }
}

// sqrt(d2) <= md, decided on d2 with an exact sqrt only within 1e-9 of the
// cut-off (identical to the reference's test on the distance itself)
__device__ __forceinline__ bool within(double d2, double md, double md2lo, double md2hi) {
    if (d2 < md2lo) return true;
    if (d2 > md2hi) return false;
    return sqrt(d2) <= md;
}

// One CTA per (road, species): the whole species-road model.
__global__ void __launch_bounds__(1024)
k_species_patches(to_model_args a) {
    extern __shared__ int smem[];
    const int rs = a.rs0 + blockIdx.x;         // road*S + species
    const int road = rs / a.S, sp = rs - road * a.S;
    const int W = a.W, H = a.H, n = W * H;
    int* s_tmp = smem;                         // 33 ints
    int* s_misc = s_tmp + 40;                  // counters
    int* par = smem + 64;                      // labels, later tables (8-byte aligned)
    int* s_list = par + (size_t)((a.W * a.H + 1) & ~1);   // block region lists
    const int* hab = a.hab_map;
    const int c0 = a.cell_off ? a.cell_off[road] : 0;
    const int c1 = a.cell_off ? a.cell_off[road + 1] : 0;
    const to_model_species& S = a.species[sp];
    const int NM = a.max_patches;
    double* area = a.area + (size_t)rs * NM;
    double* cap = a.cap + (size_t)rs * NM;
    double* popd = a.pop + (size_t)rs * NM;
    double* cx = a.cx + (size_t)rs * NM;
    double* cy = a.cy + (size_t)rs * NM;
    int* ptype = a.type + (size_t)rs * NM;
    const float* popmap = a.pop_map + (size_t)sp * n;

    if (threadIdx.x == 0) { s_misc[0] = 0; s_misc[1] = -1; }
    __syncthreads();
    bool ok = true;
    for (int h = 0; h < S.n_hab; ++h) {
        int typ = S.hab_type[h];
        if (typ == 3 || typ == 4) continue;      // CLEAR, ROAD
        for (int i = threadIdx.x; i < n; i += blockDim.x)
            par[i] = (hab[i] == typ) ? i : -1;
        __syncthreads();
        for (int q = c0 + threadIdx.x; q < c1; q += blockDim.x) {
            const int cc = a.cells[q];        // device inputs: checked here
            if ((unsigned)cc < (unsigned)n) par[cc] = -1;
            else if (a.d_flags) atomicExch(a.d_flags, TO_DEVERR_CELL);
        }
        __syncthreads();
        int nreg = cta_label(n, W, par, s_tmp, a.d_flags);
        if (nreg == 0) continue;
        float maxpop = (float)S.hab_max_pop[h];
        auto lab = [&](int c) { return par[c]; };
        auto popf = [&](int c) { return popmap[c]; };
        auto emit = [&](int o, int cnt, float pop, float sx, float sy, int bx, int by) {
            float v[5];
            finish_patch(cnt, pop, sx, sy, bx, by, a.skpx, a.skpy, a.xs, a.ys, a.spa, maxpop, v);
            area[o] = (double)v[0];
            cap[o] = (double)v[1];
            popd[o] = (double)v[2];
            cx[o] = (double)v[3];
            cy[o] = (double)v[4];
            ptype[o] = h;
        };
        ok &= cta_block_patches(W, H, a.skpx, a.skpy, a.xres, a.yres, NM, &s_misc[0], s_tmp,
                                s_list, lab, popf, emit);
        __syncthreads();
    }
    if (!ok && a.d_flags) atomicExch(a.d_flags, TO_DEVERR_PATCHES);
    __syncthreads();
    const int N = min(s_misc[0], NM);
    if (threadIdx.x == 0) a.n_patches[rs] = N;
}


// Labels of one (road, habitable type): the type's cells less the road's
// cells, labelled as LabelImage numbers into global memory.  The labels do
// not depend on the species, so every species of the road reads them.
__global__ void __launch_bounds__(1024)
k_road_labels(to_model_args a) {
    extern __shared__ int smem[];
    const int T = a.n_label_types;
    const int road = a.rs0 / a.S + (int)blockIdx.x / T, ti = (int)blockIdx.x % T;
    const int W = a.W, n = W * a.H;
    int* s_tmp = smem;                         // 33 ints
    int* par = smem + 64;
    const int typ = a.label_types[ti];
    const int* hab = a.hab_map;
    for (int i = threadIdx.x; i < n; i += blockDim.x) par[i] = (hab[i] == typ) ? i : -1;
    __syncthreads();
    const int c0 = a.cell_off ? a.cell_off[road] : 0;
    const int c1 = a.cell_off ? a.cell_off[road + 1] : 0;
    for (int q = c0 + threadIdx.x; q < c1; q += blockDim.x) {
        const int cc = a.cells[q];            // device inputs: checked here
        if ((unsigned)cc < (unsigned)n) par[cc] = -1;
        else if (a.d_flags) atomicExch(a.d_flags, TO_DEVERR_CELL);
    }
    __syncthreads();
    cta_label(n, W, par, s_tmp, a.d_flags);
    int* out = a.labels + ((size_t)road * T + ti) * n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = par[i];
}

// The patch pass of k_species_patches on labels from k_road_labels: same
// patch list (habitats in order, then coarse blocks, regions ascending,
// the same per-(block, region) sums).  All habitable types are worked on at
// once: warps over (type, block) items for the two region passes, one scan
// over the items in that order, and a thread per patch for the sums, so a
// CTA is not a chain of small per-type phases with a few threads busy.
__global__ void __launch_bounds__(512, 3)
k_species_patches_lab(to_model_args a) {
    extern __shared__ int smem[];
    const int rs = a.rs0 + blockIdx.x;
    const int road = rs / a.S, sp = rs - road * a.S;
    const int W = a.W, H = a.H, n = W * H, T = a.n_label_types;
    int* s_tmp = smem;                         // 33 ints
    int* s_hab = smem + 40;                    // [TO_MAX_HAB] habitat index of item type
    int* s_lt = s_hab + TO_MAX_HAB;            // [TO_MAX_HAB] its label type
    int* s_misc = s_lt + TO_MAX_HAB;           // [0] habitable types, [1] flag
    const int nblocks = a.xres * a.yres;
    int* s_off = smem + 64;                    // [TO_MAX_HAB * nblocks + 1]
    int* s_lab = s_off + TO_MAX_HAB * nblocks + 1;   // [max_patches]
    const to_model_species& S = a.species[sp];
    const int NM = a.max_patches;
    const float* popmap = a.pop_map + (size_t)sp * n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int skpx = a.skpx, skpy = a.skpy, xres = a.xres;

    if (threadIdx.x == 0) {
        int nh = 0, bad = 0;
        for (int h = 0; h < S.n_hab; ++h) {
            const int typ = S.hab_type[h];
            if (typ == 3 || typ == 4) continue;      // CLEAR, ROAD
            int ti = 0;
            while (ti < T && a.label_types[ti] != typ) ++ti;
            if (ti == T) { bad = 1; continue; }       // not planned for: flagged
            s_hab[nh] = h;
            s_lt[nh] = ti;
            ++nh;
        }
        s_misc[0] = nh;
        s_misc[1] = bad;
    }
    __syncthreads();
    const int nitems = s_misc[0] * nblocks;
    const int* labels = a.labels + (size_t)road * T * n;
    for (int pass = 0; pass < 2; ++pass) {
        for (int it = warp; it < nitems; it += nw) {
            const int hi = it / nblocks, b = it - hi * nblocks;
            const int* L = labels + (size_t)s_lt[hi] * n;
            const int by = b / xres, bx = b - by * xres;
            int bsx, bsy;
            block_extent(bx, by, W, H, skpx, skpy, bsx, bsy);
            const int ncell = (bsx > 0 && bsy > 0) ? bsx * bsy : 0;
            const int out = pass ? s_off[it] : 0;
            int lastr = 0, cnt = 0;
            for (;;) {
                int mn = 0x7fffffff;
                for (int e = lane; e < ncell; e += 32) {
                    const int ii = e / bsy, jj = e - ii * bsy;
                    const int r = L[(bx * skpx + ii) + (by * skpy + jj) * W];
                    if (r > lastr && r < mn) mn = r;
                }
                mn = __reduce_min_sync(0xffffffffu, mn);
                if (mn == 0x7fffffff) break;
                if (pass && lane == 0 && out + cnt < NM) s_lab[out + cnt] = mn;
                ++cnt;
                lastr = mn;
            }
            if (!pass && lane == 0) s_off[it] = cnt;
        }
        __syncthreads();
        if (!pass) {
            const int total = cta_scan_array(s_off, nitems, s_tmp);
            if (threadIdx.x == 0) s_off[nitems] = total;
            __syncthreads();
        }
    }
    const int total = s_off[nitems];
    const int nemit = min(total, NM);
    for (int t = threadIdx.x; t < nemit; t += blockDim.x) {
        int lo = 0, hi = nitems;                  // item: last one with s_off <= t
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (s_off[mid] <= t) lo = mid; else hi = mid;
        }
        const int it = lo, ht = it / nblocks, b = it - ht * nblocks;
        const int h = s_hab[ht];
        const int* L = labels + (size_t)s_lt[ht] * n;
        const int by = b / xres, bx = b - by * xres;
        int bsx, bsy;
        block_extent(bx, by, W, H, skpx, skpy, bsx, bsy);
        const int r = s_lab[t];
        int cnt = 0;
        float pop = 0.0f, sx = 0.0f, sy = 0.0f;
        // cells in the reference's order (x offset outer, y offset inner),
        // their loads issued four at a time before the in-order sums
        for (int ii = 0; ii < bsx; ++ii) {
            const int* Lc = L + (bx * skpx + ii) + (size_t)(by * skpy) * W;
            const float* Pc = popmap + (bx * skpx + ii) + (size_t)(by * skpy) * W;
            for (int j0 = 0; j0 < bsy; j0 += 4) {
                int lv[4];
                float pv[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const bool in = j0 + u < bsy;
                    lv[u] = in ? Lc[(size_t)(j0 + u) * W] : -1;
                    pv[u] = in ? Pc[(size_t)(j0 + u) * W] : 0.0f;
                }
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (lv[u] == r) {
                        cnt += 1;
                        pop = pop + pv[u];
                        sx = sx + (float)ii;
                        sy = sy + (float)(j0 + u);
                    }
            }
        }
        float v[5];
        finish_patch(cnt, pop, sx, sy, bx, by, skpx, skpy, a.xs, a.ys, a.spa,
                     (float)S.hab_max_pop[h], v);
        const size_t o = (size_t)rs * NM + t;
        a.area[o] = (double)v[0];
        a.cap[o] = (double)v[1];
        a.pop[o] = (double)v[2];
        a.cx[o] = (double)v[3];
        a.cy[o] = (double)v[4];
        a.type[o] = h;
    }
    if (threadIdx.x == 0) {
        if ((s_misc[1] || total > NM) && a.d_flags) atomicExch(a.d_flags, TO_DEVERR_PATCHES);
        a.n_patches[rs] = nemit;
    }
}

// Second half of the species-road model, one CTA per (road, species):
// patch-pair distances, road crossings, transition and survival
// probabilities and the migration matrices.  Small shared memory, so two
// CTAs share an SM and the FP64-bound transition rows of one overlap the
// integer work of the other.
__global__ void __launch_bounds__(512, 2)
k_species_links(to_model_args a) {
    extern __shared__ __align__(16) unsigned char sml[];
    __shared__ int s_last, s_cnt, s_npair;
    __shared__ int s_tmp[33];
    const int rs = a.rs0 + blockIdx.x;
    const int road = rs / a.S, sp = rs - road * a.S;
    const to_model_species& S = a.species[sp];
    const int NM = a.max_patches;
    const int N = a.n_patches[rs];
    const double* area = a.area + (size_t)rs * NM;
    const double* cap = a.cap + (size_t)rs * NM;
    const double* popd = a.pop + (size_t)rs * NM;
    const double* cx = a.cx + (size_t)rs * NM;
    const double* cy = a.cy + (size_t)rs * NM;
    const int* ptype = a.type + (size_t)rs * NM;

    // FP64 is scarce on this part, so every distance test is first decided
    // on a float d^2 (centroids are floats, so its relative error is below
    // 4e-7); only pairs within 1e-6 of a cut-off take the exact FP64 test.
    const double lam = S.lambda_mean + S.lambda_sd * S.lambda_mult;
    const double max_dist_x = log(0.05) / (-lam);
    const double mx2 = max_dist_x * max_dist_x;
    const double mx2lo = mx2 * (1.0 - 1e-9), mx2hi = mx2 * (1.0 + 1e-9);
    const float fx_lo = (float)(mx2 * (1.0 - 1e-6)), fx_hi = (float)(mx2 * (1.0 + 1e-6));
    int* cross = a.crossings_scratch + (size_t)rs * NM * NM;
    const int G = a.seg_off[road + 1] - a.seg_off[road];
    const double* rseg = a.segs + (size_t)a.seg_off[road] * 4;
    const bool seg_tab = G <= TO_SURV_TABLE_SEGS;
    constexpr int SC = TO_SURV_TABLE_SEGS;
    float* cxf = reinterpret_cast<float*>(sml);                 // [NM]
    float* cyf = cxf + NM;                                      // [NM]
    float* sgf = cyf + NM;                                      // [4][SC]
    double* s_attr = reinterpret_cast<double*>(sgf + 4 * SC);   // [TO_MAX_HAB]
    double* s_surv = s_attr + TO_MAX_HAB;                       // [C][SC+1]
    double* s_sum = s_surv + a.C * (SC + 1);                    // [NM] row sums
    int* s_off = reinterpret_cast<int*>(s_sum + NM);            // [NM+1] row offsets
    const double lda = S.lambda_mult * S.lambda_sd + S.lambda_mean;
    for (int k = threadIdx.x; k < N; k += blockDim.x) { cxf[k] = (float)cx[k]; cyf[k] = (float)cy[k]; }
    if (seg_tab)
        for (int g = threadIdx.x; g < G; g += blockDim.x) {
            const double* sg = rseg + 4 * g;
            sgf[g] = (float)sg[0];
            sgf[SC + g] = (float)sg[1];
            sgf[2 * SC + g] = (float)(sg[2] - sg[0]);
            sgf[3 * SC + g] = (float)(sg[3] - sg[1]);
        }
    for (int h = threadIdx.x; h < S.n_hab; h += blockDim.x)
        s_attr[h] = exp(S.hab_pref_mean[h] + S.hab_pref_sd[h] * S.hab_pref_mult);
    if (seg_tab)
        for (int q = threadIdx.x; q < a.C * (G + 1); q += blockDim.x) {
            int c = q / (G + 1), cr = q - c * (G + 1);
            s_surv[q] = exp(-(double)cr * S.hazard[c]);
        }
    auto surv_of = [&](int c, int cr) {
        return seg_tab ? s_surv[c * (G + 1) + cr] : exp(-(double)cr * S.hazard[c]);
    };
    if (threadIdx.x == 0) { s_last = -1; s_cnt = 0; s_npair = 0; }
    // zero the crossing counts and the migration matrices (destination-major,
    // padded to NP); initial populations and capacities
    {
        int4* c4 = reinterpret_cast<int4*>(cross);
        const int n4 = (N * N) / 4;
        for (int q = threadIdx.x; q < n4; q += blockDim.x) c4[q] = make_int4(0, 0, 0, 0);
        for (int q = n4 * 4 + threadIdx.x; q < N * N; q += blockDim.x) cross[q] = 0;
    }
    const int NP = a.npad;
    float* mmm = a.mmm + (size_t)rs * a.C * NP * NP;
    const bool direct = a.csc_ptr != nullptr;
    if (!direct) {
        float4* m4 = reinterpret_cast<float4*>(mmm);
        const size_t n4 = (size_t)a.C * NP * NP / 4;
        for (size_t q = threadIdx.x; q < n4; q += blockDim.x) m4[q] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    float* ip = a.init_pops + (size_t)rs * NP;
    float* cp = a.caps + (size_t)rs * NP;
    for (int k = threadIdx.x; k < NP; k += blockDim.x) {
        ip[k] = (k < N) ? (float)popd[k] : 0.0f;
        cp[k] = (k < N) ? (float)cap[k] : 1.0f;
    }
    __syncthreads();
    auto in_range = [&](int i, int j, float flo, float fhi, double md, double lo2, double hi2) {
        float dxf = cxf[i] - cxf[j], dyf = cyf[i] - cyf[j];
        float d2f = dxf * dxf + dyf * dyf;
        if (d2f < flo) return true;
        if (d2f > fhi) return false;
        double dx = cx[i] - cx[j], dy = cy[i] - cy[j];
        return within(dx * dx + dy * dy, md, lo2, hi2);
    };
    // pass 1: valid pairs i < j (within the crossing distance) into a list;
    // the reference never tests its last valid pair (its counter starts at
    // -1), so the largest valid pair index is noted too
    int* plist = reinterpret_cast<int*>(a.trans_scratch + (size_t)rs * NM * NM);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    {
        int last = -1, cnt = 0;
        const int npair = N * N;
        for (int q0 = warp * 32; q0 < npair; q0 += blockDim.x) {
            const int q = q0 + lane;
            const int i = q / N, j = q - i * N;
            const bool v = q < npair && j > i && in_range(i, j, fx_lo, fx_hi, max_dist_x, mx2lo, mx2hi);
            const unsigned m = __ballot_sync(0xffffffffu, v);
            int pos = 0;
            if (lane == 0 && m) pos = atomicAdd(&s_npair, __popc(m));
            pos = __shfl_sync(0xffffffffu, pos, 0);
            if (v) {
                plist[pos + __popc(m & ((1u << lane) - 1u))] = q;
                last = max(last, q);
                ++cnt;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            last = max(last, __shfl_xor_sync(0xffffffffu, last, o));
            cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        }
        if (lane == 0) { atomicMax(&s_last, last); atomicAdd(&s_cnt, cnt); }
    }
    __syncthreads();
    // pass 2: road crossings of the listed pairs in float without
    // contraction (pathAdjacencyKernel, SimulateGPU.cu:454-493)
    const int last_pair = (a.sem == 0) ? s_last : -1;
    for (int t = threadIdx.x; t < s_npair; t += blockDim.x) {
        const int q = plist[t];
        if (q == last_pair) continue;
        const int i = q / N, j = q - i * N;
        const float x1 = cxf[i], y1 = cyf[i];
        const float x21 = cxf[j] - cxf[i];       // = (float)(cx[j] - cx[i]): one rounding
        const float y21 = cyf[j] - cyf[i];
        int c = 0;
        if (seg_tab) {
            for (int g = 0; g < G; ++g)
                c += seg_cross(x1, y1, x21, y21, sgf[g], sgf[SC + g], sgf[2 * SC + g], sgf[3 * SC + g]);
        } else {
            for (int g = 0; g < G; ++g) {
                const double* sg = rseg + 4 * g;
                c += seg_cross(x1, y1, x21, y21, (float)sg[0], (float)sg[1],
                               (float)(sg[2] - sg[0]), (float)(sg[3] - sg[1]));
            }
        }
        cross[(size_t)i * N + j] = c;
        cross[(size_t)j * N + i] = c;
    }
    if (threadIdx.x == 0) {
        const int cnt = s_cnt;
        a.n_transitions[rs] = (a.sem == 0 && cnt > 0) ? cnt - 1 : cnt;
    }
    __syncthreads();

    // Transition probabilities (SpeciesRoadPatches.cpp:383-426) and the
    // migration matrices.  FP64 issues at a small fraction of the FP32 rate
    // here, and a warp pays for a whole FP64 instruction however few lanes
    // are active, so the in-range pairs (a few per row) are listed first and
    // the FP64 work then runs over the list on full warps:
    //   T1  a warp per origin row i lists its in-range destinations j in
    //       ascending order (float tests; FP64 only within 1e-6 of the cut-off)
    //   T2  one thread per listed pair: the unnormalised weight
    //   T3  one thread per row: the row sum in j order (the reference's order)
    //   T4  one thread per listed pair: division by the row sum, survival,
    //       the migration matrices
    // Every value goes through the same operations in the same order as a
    // row-at-a-time evaluation, so the bits do not depend on the schedule.
    const double max_dist_t = (a.sem == 0)
        ? log(0.05) / (-(S.lambda_mean + S.lambda_sd * lda))
        : log(0.05) / (-lda);
    const double mt2 = max_dist_t * max_dist_t;
    const double mt2lo = mt2 * (1.0 - 1e-9), mt2hi = mt2 * (1.0 + 1e-9);
    const float ft_lo = (float)(mt2 * (1.0 - 1e-6)), ft_hi = (float)(mt2 * (1.0 + 1e-6));
    double* trans = a.trans ? a.trans + (size_t)rs * NM * NM : nullptr;
    double* surv = a.surv ? a.surv + (size_t)rs * a.C * NM * NM : nullptr;
    double* wv = a.trans_scratch + (size_t)rs * NM * NM;        // weights, [i][slot]
    uint16_t* dj = a.trans_dest + (size_t)rs * NM * NM;         // destinations, [i][slot]
    // T1
    for (int i = warp; i < N; i += nwarp) {
        uint16_t* rowj = dj + (size_t)i * NM;
        int cnt = 0;
        for (int j0 = 0; j0 < N; j0 += 32) {
            const int j = j0 + lane;
            const bool inr = (j < N) && in_range(i, j, ft_lo, ft_hi, max_dist_t, mt2lo, mt2hi);
            const unsigned m = __ballot_sync(0xffffffffu, inr);
            if (inr) rowj[cnt + __popc(m & ((1u << lane) - 1u))] = (uint16_t)j;
            cnt += __popc(m);
        }
        if (lane == 0) s_off[i] = cnt;
    }
    __syncthreads();
    {   // row offsets: exclusive scan of the counts, s_off[N] = total
        const int chunk = (N + (int)blockDim.x - 1) / (int)blockDim.x;
        const int lo = (int)threadIdx.x * chunk, hi = min(N, lo + chunk);
        int c = 0;
        for (int i = lo; i < hi; ++i) c += s_off[i];
        int total = 0;
        int base = cta_exclusive_scan(c, s_tmp, &total);
        for (int i = lo; i < hi; ++i) { const int v = s_off[i]; s_off[i] = base; base += v; }
        if (threadIdx.x == 0) s_off[N] = total;
    }
    __syncthreads();
    const int n_listed = s_off[N];
    auto row_of = [&](int f) {                 // s_off[i] <= f < s_off[i + 1]
        int lo = 0, hi = N;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (s_off[mid] <= f) lo = mid; else hi = mid;
        }
        return lo;
    };
    // T2
    for (int f = threadIdx.x; f < n_listed; f += blockDim.x) {
        const int i = row_of(f);
        const size_t at = (size_t)i * NM + (f - s_off[i]);
        const int j = dj[at];
        const double w = area[j] * lda * s_attr[ptype[j]];
        double v = w;
        if (i != j) {
            const double dx = cx[i] - cx[j], dy = cy[i] - cy[j];
            const double d = sqrt(dx * dx + dy * dy);
            v = (a.sem == 0) ? w / exp(-lda * d) : w * exp(-lda * d);
        }
        wv[at] = v;
    }
    __syncthreads();
    // T3
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const double* rowv = wv + (size_t)i * NM;
        const int n = s_off[i + 1] - s_off[i];
        double summ = 0.0;
        for (int q = 0; q < n; ++q) summ += rowv[q];
        s_sum[i] = summ;
    }
    __syncthreads();
    // T4
    for (int f = threadIdx.x; f < n_listed; f += blockDim.x) {
        const int i = row_of(f);
        const size_t at = (size_t)i * NM + (f - s_off[i]);
        const int j = dj[at];
        const double tr = wv[at] / s_sum[i];
        wv[at] = tr;                           // kept for the animals-at-risk sums
        const int cr = cross[(size_t)i * N + j];
        if (direct) {
            // the pair's place in destination j's list (in range is
            // symmetric, so row j lists its origins, ascending)
            const uint16_t* rj = dj + (size_t)j * NM;
            int lo = 0, hi = s_off[j + 1] - s_off[j];
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if ((int)rj[mid] < i) lo = mid + 1; else hi = mid;
            }
            const size_t ft = (size_t)s_off[j] + lo;
            for (int c = 0; c < a.C; ++c)
                mmm[(size_t)c * NP * NP + ft] = (float)(tr * surv_of(c, cr));
        } else {
            for (int c = 0; c < a.C; ++c) {
                const float mv = (float)(tr * surv_of(c, cr));
                if ((double)mv > 0.00001) mmm[((size_t)c * NP + j) * NP + i] = mv;
            }
        }
        if (trans) trans[(size_t)i * NM + j] = tr;
    }
    if (a.iar) {
        // initial animals at risk per control (SpeciesRoadPatches::
        // computeAAR / computeInitialAAR, SpeciesRoadPatches.cpp:453-490):
        // 1 - sum_i pop_i sum_j trans(i,j) surv_c(i,j) / sum_i pop_i, each
        // row over its listed destinations ascending, rows ascending
        __syncthreads();
        for (int c = 0; c < a.C; ++c) {
            for (int i = threadIdx.x; i < N; i += blockDim.x) {
                const double* rowv = wv + (size_t)i * NM;
                const uint16_t* rowj = dj + (size_t)i * NM;
                const int n = s_off[i + 1] - s_off[i];
                double acc = 0.0;
                for (int q = 0; q < n; ++q)
                    acc += rowv[q] * surv_of(c, cross[(size_t)i * N + rowj[q]]);
                s_sum[i] = popd[i] * acc;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                double tot = 0.0, init = 0.0;
                for (int i = 0; i < N; ++i) { tot += s_sum[i]; init += popd[i]; }
                a.iar[(size_t)rs * a.C + c] = 1.0 - tot / init;
            }
            __syncthreads();
        }
    }
    if (direct) {
        // packed matrices: destination j's entries are the listed origins
        // whose value passes the reference's 1e-5 cut, ascending - the dense
        // matrix's non-zeros of row j in k_pack_csc's order
        __syncthreads();
        const unsigned lt = (1u << lane) - 1u;
        for (int c = 0; c < a.C; ++c) {
            const int mtx = rs * a.C + c;
            int* cp = a.csc_ptr + (size_t)mtx * (NP + 1);
            const float* mvT = mmm + (size_t)c * NP * NP;
            for (int j = warp; j < NP; j += nwarp) {
                int cnt = 0;
                if (j < N) {
                    const int f0 = s_off[j], n = s_off[j + 1] - f0;
                    for (int q0 = 0; q0 < n; q0 += 32) {
                        const bool keep = q0 + lane < n && (double)mvT[f0 + q0 + lane] > 0.00001;
                        cnt += __popc(__ballot_sync(0xffffffffu, keep));
                    }
                }
                if (lane == 0) cp[j] = cnt;
            }
            __syncthreads();
            {
                const int chunk = (NP + (int)blockDim.x - 1) / (int)blockDim.x;
                const int lo = (int)threadIdx.x * chunk, hi = min(NP, lo + chunk);
                int c0 = 0;
                for (int k = lo; k < hi; ++k) c0 += cp[k];
                int total = 0;
                int base = cta_exclusive_scan(c0, s_tmp, &total);
                for (int k = lo; k < hi; ++k) { const int v = cp[k]; cp[k] = base; base += v; }
                if (threadIdx.x == 0) {
                    cp[NP] = total;
                    a.csc_nnz[mtx] = (total <= a.csc_cap) ? total : -1;
                }
            }
            __syncthreads();
            if (cp[NP] <= a.csc_cap) {
                uint16_t* ix = a.csc_idx + (size_t)mtx * a.csc_cap;
                float* vv = a.csc_val + (size_t)mtx * a.csc_cap;
                for (int j = warp; j < N; j += nwarp) {
                    int o = cp[j];
                    const int f0 = s_off[j], n = s_off[j + 1] - f0;
                    for (int q0 = 0; q0 < n; q0 += 32) {
                        const bool in = q0 + lane < n;
                        const float mv = in ? mvT[f0 + q0 + lane] : 0.0f;
                        const bool keep = in && (double)mv > 0.00001;
                        const unsigned b = __ballot_sync(0xffffffffu, keep);
                        if (keep) {
                            const int q = o + __popc(b & lt);
                            ix[q] = dj[(size_t)j * NM + q0 + lane];
                            vv[q] = mv;
                        }
                        o += __popc(b);
                    }
                }
            }
            __syncthreads();
        }
    }
    // dense FP64 transition / survival outputs (single-road API only)
    if (trans || surv) {
        __syncthreads();
        for (int q = threadIdx.x; q < N * N; q += blockDim.x) {
            const int i = q / N, j = q - i * N;
            if (trans && !in_range(i, j, ft_lo, ft_hi, max_dist_t, mt2lo, mt2hi))
                trans[(size_t)i * NM + j] = 0.0;
            if (surv) {
                const int cr = cross[(size_t)i * N + j];
                for (int c = 0; c < a.C; ++c)
                    surv[((size_t)c * NM + i) * NM + j] = surv_of(c, cr);
            }
        }
    }
    if (a.crossings_out) {
        __syncthreads();
        int* co = a.crossings_out + (size_t)rs * NM * NM;
        for (int q = threadIdx.x; q < N * N; q += blockDim.x) {
            int i = q / N, j = q - i * N;
            co[(size_t)i * NM + j] = cross[q];
        }
    }
}

}  // namespace

namespace to_k {

to_status label_image(to_ctx ctx, int W, int H, const int* d_in, int* d_out,
                      int* d_nreg) {
    size_t smem = (size_t)W * H * sizeof(int) + 64 * sizeof(int);
    if (smem > ctx->smem_optin)
        return to_set_error(ctx, TO_ERR_UNSUPPORTED,
                            "label image of %d x %d exceeds shared memory", W, H);
    TO_CUDA(ctx, cudaFuncSetAttribute(k_label_image,
                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_label_image<<<1, 1024, smem, ctx->stream>>>(W, H, d_in, d_out, d_nreg,
                                                  ctx->d_flags);
    TO_LAUNCHED(ctx);
    return TO_OK;
}

to_status build_patches(to_ctx ctx, int W, int H, int skpx, int skpy, int xres,
                        int yres, int nreg, float xs, float ys, float spa,
                        float maxpop, const int* d_labels, const float* d_pops,
                        int max_patches, double* d_out5, int* d_count) {
    (void)nreg;
    const size_t smem = (size_t)(xres * yres + 1 + max_patches) * sizeof(int);
    if (smem > ctx->smem_optin)
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "%d blocks, %d patches exceed shared memory",
                            xres * yres, max_patches);
    TO_CUDA(ctx, cudaFuncSetAttribute(k_build_patches,
                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_build_patches<<<1, 256, smem, ctx->stream>>>(W, H, skpx, skpy, xres, yres,
        xs, ys, spa, maxpop, d_labels, d_pops, max_patches, d_out5, d_count,
        ctx->d_flags);
    TO_LAUNCHED(ctx);
    return TO_OK;
}

to_status line_segment_intersect(to_ctx ctx, int T, const double* d_xy1, int G,
                                 const double* d_xy2, int* d_cross) {
    if (T <= 0) return TO_OK;
    int threads = 256;
    int blocks = (T + threads - 1) / threads;
    if (blocks > 4 * ctx->sm_count) blocks = 4 * ctx->sm_count;
    size_t smem = (size_t)4 * (G > 0 ? G : 1) * sizeof(float);
    k_line_segment_intersect<<<blocks, threads, smem, ctx->stream>>>(
        T, d_xy1, G, d_xy2, d_cross);
    TO_LAUNCHED(ctx);
    return TO_OK;
}

to_status species_model(to_ctx ctx, const to_model_args& a, int n_rs) {
    // patches: labels (W*H ints) and the block region lists in shared memory
    size_t smem = (size_t)a.W * a.H * sizeof(int);
    smem = ((smem + 7) & ~(size_t)7) + (size_t)(a.xres * a.yres + 1 + a.max_patches) * sizeof(int);
    smem += 64 * sizeof(int);
    if (smem > ctx->smem_optin)
        return to_set_error(ctx, TO_ERR_UNSUPPORTED,
                            "grid of %d x %d exceeds shared memory", a.W, a.H);
    TO_CUDA(ctx, cudaFuncSetAttribute(k_species_patches,
                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // links: float centroids, segment and survival tables
    const size_t smem2 = (size_t)2 * a.max_patches * sizeof(float) +
                         (size_t)4 * TO_SURV_TABLE_SEGS * sizeof(float) +
                         (size_t)(TO_MAX_HAB + a.C * (TO_SURV_TABLE_SEGS + 1)) * sizeof(double) +
                         (size_t)a.max_patches * sizeof(double) +
                         (size_t)(a.max_patches + 1) * sizeof(int);
    if (smem2 > ctx->smem_optin || a.max_patches > 65535)
        return to_set_error(ctx, TO_ERR_UNSUPPORTED, "%d patches exceed shared memory",
                            a.max_patches);
    TO_CUDA(ctx, cudaFuncSetAttribute(k_species_links,
                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2));
    if (a.n_label_types > 0) {
        // labels once per (road, habitable type), then each species' patches
        const size_t smem_l = (size_t)(64 + a.W * a.H) * sizeof(int);
        const size_t smem_p =
            (size_t)(64 + TO_MAX_HAB * a.xres * a.yres + 1 + a.max_patches) * sizeof(int);
        if (smem_l > ctx->smem_optin || smem_p > ctx->smem_optin)
            return to_set_error(ctx, TO_ERR_UNSUPPORTED, "grid of %d x %d exceeds shared memory",
                                a.W, a.H);
        TO_CUDA(ctx, cudaFuncSetAttribute(k_road_labels,
                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_l));
        TO_CUDA(ctx, cudaFuncSetAttribute(k_species_patches_lab,
                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_p));
        const int roads = n_rs / a.S;
        to_prof_begin(ctx, "species_labels");
        k_road_labels<<<roads * a.n_label_types, 1024, smem_l, ctx->stream>>>(a);
        to_prof_end(ctx);
        TO_LAUNCHED(ctx);
        to_prof_begin(ctx, "species_patches");
        k_species_patches_lab<<<n_rs, 512, smem_p, ctx->stream>>>(a);
        to_prof_end(ctx);
        TO_LAUNCHED(ctx);
    } else {
        to_prof_begin(ctx, "species_patches");
        k_species_patches<<<n_rs, 1024, smem, ctx->stream>>>(a);
        to_prof_end(ctx);
        TO_LAUNCHED(ctx);
    }
    to_prof_begin(ctx, "species_links");
    k_species_links<<<n_rs, 512, smem2, ctx->stream>>>(a);
    to_prof_end(ctx);
    TO_LAUNCHED(ctx);
    return TO_OK;
}

}  // namespace to_k
