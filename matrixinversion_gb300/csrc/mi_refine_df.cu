// mi_refine_df.cu -- one refinement step for a listed subset of a batch with
// the residual in compensated float-float arithmetic on the FP32 pipes:
//   R = I - A X    each product split exactly (p = a*x, e = fma(a, x, -p))
//                  and summed with Knuth's TwoSum into a (hi, lo) pair,
//   X <- X + X R   in FP32 (R is small, so FP32 relative accuracy suffices).
// The residual carries about 44 significant bits, enough to take the error
// of an FP32 inverse from about kappa * u down to about u while kappa * u < 1;
// on GB300 this runs several times faster than the same step in FP64.
// One warp per matrix; lane j owns column j.
#include <cuda_runtime.h>

#include <cstdint>

#include "mi_inverse.h"

namespace mi {

int set_cuda_error(cudaError_t e, const char* what);   // mi_api.cu
int device_sm_count();

constexpr int kDfWarps = 2;                             // 3 x 4.2 KB of staging per warp
constexpr int kDfPitch = 33;                              // floats per staged row (bank spread)

// (s, c) += a * x, exactly up to the final rounding of c.  Explicit
// round-to-nearest intrinsics: none of these may be contracted into an FMA.
__device__ __forceinline__ void df_madd(float& s, float& c, float a, float x) {
    const float p = __fmul_rn(a, x);
    const float e = fmaf(a, x, -p);                               // a * x = p + e exactly
    const float t = __fadd_rn(s, p);                              // TwoSum(s, p) = t + r exactly
    const float z = __fsub_rn(t, s);
    const float r = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));
    s = t;
    c = __fadd_rn(c, __fadd_rn(r, e));
}

__global__ void __launch_bounds__(64) mi_refine_df_kernel(const float* __restrict__ A, float* __restrict__ X,
                                                           const int32_t* __restrict__ list, long long count,
                                                           long long batch, int n) {
    __shared__ float sa[kDfWarps][32 * kDfPitch];
    __shared__ float sx[kDfWarps][32 * kDfPitch];
    __shared__ float sr[kDfWarps][32 * kDfPitch];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long nn = (long long)n * n;
    float* ma = sa[warp];
    float* mx = sx[warp];
    float* mr = sr[warp];
    for (long long t = (long long)blockIdx.x * kDfWarps + warp; t < count; t += (long long)gridDim.x * kDfWarps) {
        const long long b = list[t];
        if (b < 0 || b >= batch) continue;                // out-of-range entries are skipped
        const float* a = A + b * nn;
        float* x = X + b * nn;
        for (int e = lane; e < 32 * 32; e += 32) {
            const int i = e >> 5, j = e & 31;
            const bool in = i < n && j < n;
            ma[i * kDfPitch + j] = in ? a[i * n + j] : 0.0f;
            mx[i * kDfPitch + j] = in ? x[i * n + j] : 0.0f;
        }
        __syncwarp();
        const int j = lane;
        // column j of R = I - A X, accumulated as -(A X) + I in float-float
        for (int i = 0; i < n; i++) {
            float s = 0.0f, c = 0.0f;
#pragma unroll 8
            for (int k = 0; k < 32; k++) df_madd(s, c, -ma[i * kDfPitch + k], mx[k * kDfPitch + j]);
            const float d = (i == j) ? 1.0f : 0.0f;
            const float t2 = __fadd_rn(s, d);
            const float z = __fsub_rn(t2, s);
            const float r = __fadd_rn(__fsub_rn(s, __fsub_rn(t2, z)), __fsub_rn(d, z));
            mr[i * kDfPitch + j] = __fadd_rn(t2, __fadd_rn(c, r));
        }
        __syncwarp();
        // column j of X + X R in FP32
        if (j < n) {
            for (int i = 0; i < n; i++) {
                float s = 0.0f;
#pragma unroll 8
                for (int k = 0; k < 32; k++) s = fmaf(mx[i * kDfPitch + k], mr[k * kDfPitch + j], s);
                x[i * n + j] = mx[i * kDfPitch + j] + s;
            }
        }
        __syncwarp();
    }
}

}  // namespace mi

extern "C" int mi_refine_df_f32(const float* d_a, float* d_x, const int32_t* d_list, int64_t count, int64_t batch,
                                int n, void* stream) {
    if (n < 1 || n > 32 || count < 0 || batch < 0) return MI_ERR_INVALID_VALUE;
    if (count == 0) return MI_OK;
    if (d_a == nullptr || d_x == nullptr || d_list == nullptr) return MI_ERR_NULL_POINTER;
    long long blocks = (count + mi::kDfWarps - 1) / mi::kDfWarps;
    const long long cap = 8LL * mi::device_sm_count();
    if (blocks > cap) blocks = cap;
    mi::mi_refine_df_kernel<<<(unsigned)blocks, 32 * mi::kDfWarps, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        d_a, d_x, d_list, count, batch, n);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return mi::set_cuda_error(e, "float-float refinement launch");
    return MI_OK;
}
