/*
 * to_grid.h - host-side check of the coarse-block layout of the patch
 * computation (plain C++, no CUDA; included by the entry points and by a CPU
 * test).
 *
 * patchComputation (SimulateGPU.cu:510-520) bounds a block's x extent by H
 * and its y extent by W.  On a square grid every visited cell is inside it;
 * on a W x H grid with W != H the last blocks can run past the grid (past the
 * label image for H < W), which the kernels must never read.  The entry
 * points refuse such layouts instead of reading past their buffers.
 */
#ifndef TO_GRID_H
#define TO_GRID_H

/* true when every cell the block loop visits, x = bx*skpx + ii and
 * y = by*skpy + jj over the extents below, lies inside the W x H grid */
static inline bool to_blocks_inside(int W, int H, int skpx, int skpy, int xres, int yres) {
    if (W <= 0 || H <= 0 || skpx < 0 || skpy < 0 || xres < 0 || yres < 0) return false;
    long long maxx = -1, maxy = -1;
    for (int bx = 0; bx < xres; ++bx) {
        const long long bsx = ((long long)(bx + 1) * skpx <= H) ? skpx
                                                                : (long long)H - (long long)bx * skpx;
        if (bsx > 0 && (long long)bx * skpx + bsx - 1 > maxx) maxx = (long long)bx * skpx + bsx - 1;
    }
    for (int by = 0; by < yres; ++by) {
        const long long bsy = ((long long)(by + 1) * skpy <= W) ? skpy
                                                                : (long long)W - (long long)by * skpy;
        if (bsy > 0 && (long long)by * skpy + bsy - 1 > maxy) maxy = (long long)by * skpy + bsy - 1;
    }
    /* blocks with an empty x or y extent hold no cell at all */
    if (maxx < 0 || maxy < 0) return true;
    return maxx < W && maxy < H;
}

#endif /* TO_GRID_H */
