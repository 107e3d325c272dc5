// mi_refine64.cu -- one refinement step in FP64 for a listed subset of a
// batch (matrices flagged as ill-conditioned):  R = I - A X and
// X <- X + X R, both in FP64 from the FP32 A and X, rounded once to FP32.
// With the residual in FP64 the step takes the error from about kappa * u
// down to about u (while kappa * u < 1), which no FP32-accumulated residual
// can do.  One warp per matrix; lane j owns column j of X and of R.
#include <cuda_runtime.h>

#include <cstdint>

#include "mi_inverse.h"

namespace mi {

int set_cuda_error(cudaError_t e, const char* what);   // mi_api.cu
int device_sm_count();
long long resident_grid(const void* kernel, int threads, long long want, int* cache);

constexpr int kR64Warps = 2;                          // 2 x 16.9 KB of FP64 staging per block
constexpr int kR64Pitch = 33;                           // doubles per staged row (bank spread)

__global__ void __launch_bounds__(64) mi_refine64_kernel(const float* __restrict__ A, float* __restrict__ X,
                                                          const int32_t* __restrict__ list, long long count,
                                                          long long batch, int n) {
    __shared__ double sa[kR64Warps][32 * kR64Pitch];
    __shared__ double sx[kR64Warps][32 * kR64Pitch];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long nn = (long long)n * n;
    for (long long t = (long long)blockIdx.x * kR64Warps + warp; t < count; t += (long long)gridDim.x * kR64Warps) {
        const long long b = list[t];
        if (b < 0 || b >= batch) continue;              // out-of-range entries are skipped
        const float* a = A + b * nn;
        float* x = X + b * nn;
        for (int e = lane; e < n * n; e += 32) {
            const int i = e / n, j = e - i * n;
            sa[warp][i * kR64Pitch + j] = (double)a[e];
            sx[warp][i * kR64Pitch + j] = (double)x[e];
        }
        __syncwarp();
        const int j = lane;
        double xc[32], rc[32];
#pragma unroll
        for (int k = 0; k < 32; k++) xc[k] = (k < n && j < n) ? sx[warp][k * kR64Pitch + j] : 0.0;
        // column j of R = I - A X
#pragma unroll
        for (int i = 0; i < 32; i++) {
            double s = 0.0;
            if (i < n) {
#pragma unroll
                for (int k = 0; k < 32; k++)
                    if (k < n) s = fma(sa[warp][i * kR64Pitch + k], xc[k], s);
            }
            rc[i] = (i < n && j < n) ? ((i == j ? 1.0 : 0.0) - s) : 0.0;
        }
        // column j of X + X R
#pragma unroll
        for (int i = 0; i < 32; i++) {
            if (i < n && j < n) {
                double s = 0.0;
#pragma unroll
                for (int k = 0; k < 32; k++)
                    if (k < n) s = fma(sx[warp][i * kR64Pitch + k], rc[k], s);
                x[i * n + j] = (float)(sx[warp][i * kR64Pitch + j] + s);
            }
        }
        __syncwarp();
    }
}

}  // namespace mi

extern "C" int mi_refine_fp64_f32(const float* d_a, float* d_x, const int32_t* d_list, int64_t count, int64_t batch,
                                  int n, void* stream) {
    if (n < 1 || n > 32 || count < 0 || batch < 0) return MI_ERR_INVALID_VALUE;
    if (count == 0) return MI_OK;
    if (d_a == nullptr || d_x == nullptr || d_list == nullptr) return MI_ERR_NULL_POINTER;
    static int per_sm[64] = {0};
    const long long blocks = mi::resident_grid(reinterpret_cast<const void*>(mi::mi_refine64_kernel),
                                               32 * mi::kR64Warps, (count + mi::kR64Warps - 1) / mi::kR64Warps, per_sm);
    mi::mi_refine64_kernel<<<(unsigned)blocks, 32 * mi::kR64Warps, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        d_a, d_x, d_list, count, batch, n);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return mi::set_cuda_error(e, "fp64 refinement launch");
    return MI_OK;
}
