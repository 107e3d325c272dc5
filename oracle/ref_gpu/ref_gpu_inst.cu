// Test infrastructure (never the product): explicit instantiations of the
// reference's own GPU kernel, batched_lu_subwarp -- parallel_pivot
// (luBatchedInplace.cuh:127-198), serial_pivot (:104-170) and templated
// (:78-121), one cubin each, all with this file and the variant's directory
// on the include path -- compiled unchanged from the reference tree into
// device-only cubins (oracle/Makefile, target ref) so that they can be timed
// on the GPU beside this project's kernels (oracle/ref_gpu.py).  The template arguments follow the reference's driver
// (parallel_pivot/luBatchedInplace.cu:4-11: threads per matrix = n, matrices
// per block = NUMTHREADS / n) with NUMTHREADS from parallel_pivot/run.py:187-222
// (32 for n = 4, 8, 16; n for n > 16).  numMatrices is a template argument:
// a launch must cover exactly that many matrices, in whole blocks (the
// kernel's __syncthreads sit inside its `globalMatrixId < numMatrices` test).
#include "luBatchedInplace.cuh"

#define MI_REF_INST(N, MPB, COUNT) template __global__ void batched_lu_subwarp<float, N, N, MPB, COUNT>(float*);

MI_REF_INST(4, 8, 1000000)
MI_REF_INST(8, 4, 1000000)
MI_REF_INST(16, 2, 1000000)
MI_REF_INST(24, 1, 1000000)
MI_REF_INST(31, 1, 1000000)
MI_REF_INST(32, 1, 1000000)
MI_REF_INST(8, 4, 4096)
MI_REF_INST(16, 2, 4096)
MI_REF_INST(32, 1, 4096)
MI_REF_INST(32, 1, 1000)
