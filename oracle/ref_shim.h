/*
 * ref_shim.h - lets the reference's CUDA kernels compile as host C++ so the
 * oracle can be pinned against the reference's own arithmetic.  Prepended by
 * oracle/build_ref.sh to the kernel source lines it streams out of the
 * reference tree; nothing here is product code.
 *
 * Each kernel launch becomes a sequential loop over the grid in
 * oracle/ref_harness.cpp, which sets the thread/block coordinates below
 * before calling the kernel body as a plain function.  Device malloc/free,
 * printf and the math functions map to their host counterparts.
 */
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
using namespace std;

#define __global__
#define __device__
#define __host__

struct to_dim3 { unsigned int x, y, z; };
extern thread_local to_dim3 blockIdx, threadIdx, blockDim, gridDim;

/* legacy 2-D texture reference of the vendored kNN (point filtering,
 * unnormalised coordinates): texel (x, y) = data[y * width + x] */
struct to_ref_texture { const float* data; int width; };
extern thread_local to_ref_texture texA;
static inline float tex2D(const to_ref_texture& t, float x, float y) {
    return t.data[(int)y * t.width + (int)x];
}

namespace SimulateGPU {
void dense2Sparse(float* denseIn, int rows, int cols, float* sparseOut,
                  int* elemsPerCol, int* rowIdx, int& totalElements);
}
