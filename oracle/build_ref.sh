#!/bin/sh
# Builds oracle/_ref/libtoref.so: the reference's own hot-path kernels
# (include/gpuCode/SimulateGPU.cu, include/gpuCode/knn_cuda_with_indexes.cu)
# and its LabelImage (include/utilities/labelmethod.cpp), compiled for the
# host CPU straight from the reference tree.  The kernel source lines are
# streamed from their files into g++ behind oracle/ref_shim.h, which turns
# each CUDA launch into a loop (oracle/ref_harness.cpp); no reference source
# is copied into this repository.  Used only to pin the oracle; skipped when
# the reference tree is absent.
set -e
REF=${TO_REFERENCE_DIR:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=$HERE/_ref
SG=$REF/include/gpuCode/SimulateGPU.cu
KNN=$REF/include/gpuCode/knn_cuda_with_indexes.cu
LAB=$REF/include/utilities/labelmethod.cpp
if [ ! -f "$SG" ] || [ ! -f "$KNN" ] || [ ! -f "$LAB" ]; then
    echo "build_ref: reference tree not found at $REF; skipped"
    exit 0
fi
mkdir -p "$OUT"
# kernel line ranges: solveLinearSystem, expPVPath, pathAdjacencyKernel +
# roadCrossingsKernel, patchComputation, mteKernel, randControls,
# forwardPathKernel .. createQueryPoints, firstPeriodInduction +
# backwardInduction, multiLocLinReg + rovCorrection, interpolateMulti,
# dense2Sparse; kNN distance (texture form), insertion sort, sqrt.
{
    cat "$HERE/ref_shim.h"
    sed -n '129,190p;256,279p;454,493p;498,573p;595,717p;720,730p;789,1195p;2210,2784p;2934,3073p' "$SG"
    # interpolateMulti reads its coefficient buffer after freeing it (device
    # heap memory keeps the value; the host allocator reuses it), so free is
    # a no-op inside it here
    echo '#define free(p) ((void)(p))'
    sed -n '3077,3155p' "$SG"
    echo '#undef free'
    sed -n '5973,5996p' "$SG"
    sed -n '77,90p;340,411p;424,429p' "$KNN"
} | g++ -x c++ -std=c++14 -O2 -fPIC -w -c - -o "$OUT/ref_kernels.o"
g++ -std=c++14 -O2 -fPIC -w -I "$REF/include/utilities" -c "$LAB" -o "$OUT/labelmethod.o"
g++ -std=c++14 -O2 -fPIC -c "$HERE/ref_harness.cpp" -o "$OUT/ref_harness.o"
g++ -shared -o "$OUT/libtoref.so" "$OUT/ref_kernels.o" "$OUT/labelmethod.o" "$OUT/ref_harness.o"
echo "build_ref: $OUT/libtoref.so"
