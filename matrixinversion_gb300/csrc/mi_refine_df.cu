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
long long resident_grid(const void* kernel, int threads, long long want, int* cache);

constexpr int kDfWarps = 2;                             // 3 staged 32 x 32 tiles per warp (about 13 KB)
constexpr int kDfPitch = 33;                            // row-major tiles: column reads conflict-free
constexpr int kDfPitchT = 34;                           // transposed tiles: 8-byte row-pair loads

__device__ __forceinline__ float2 neg2(float2 v) { return make_float2(-v.x, -v.y); }

// Two independent float-float accumulators (rows i and i + 1 of one column):
// (s, c) += a * x with a = (a_i, a_i+1), x duplicated.  Packed FP32x2
// arithmetic with explicit rounding (nothing contracted into an FMA).
__device__ __forceinline__ void df_madd2(float2& s, float2& c, float2 a, float2 x) {
    const float2 p = __fmul2_rn(a, x);
    const float2 e = __ffma2_rn(a, x, neg2(p));                         // a * x = p + e exactly
    const float2 t = __fadd2_rn(s, p);                                  // TwoSum(s, p) = t + r exactly
    const float2 z = __fadd2_rn(t, neg2(s));
    const float2 r = __fadd2_rn(__fadd2_rn(s, neg2(__fadd2_rn(t, neg2(z)))), __fadd2_rn(p, neg2(z)));
    s = t;
    c = __fadd2_rn(c, __fadd2_rn(r, e));
}

__device__ __forceinline__ float df_round(float s, float c, float d) {
    const float t = __fadd_rn(s, d);
    const float z = __fsub_rn(t, s);
    const float r = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(d, z));
    return __fadd_rn(t, __fadd_rn(c, r));
}

__global__ void __launch_bounds__(64) mi_refine_df_kernel(const float* __restrict__ A, float* __restrict__ X,
                                                          const int32_t* list, long long count, long long batch,
                                                          int n, float tol, int32_t* next) {
    __shared__ float sat[kDfWarps][32 * kDfPitchT];    // A^T (row pair i, i+1 adjacent), then the correction D^T
    __shared__ float sxt[kDfWarps][32 * kDfPitchT];    // X^T
    __shared__ float sr[kDfWarps][32 * kDfPitch];      // R
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long nn = (long long)n * n;
    float* at = sat[warp];
    float* xt = sxt[warp];
    float* mr = sr[warp];
    for (long long t = (long long)blockIdx.x * kDfWarps + warp; t < count; t += (long long)gridDim.x * kDfWarps) {
        // lane 0 alone reads list[t] and writes next[t], in that order, so the
        // two may be one array
        const long long b = __shfl_sync(0xffffffffu, lane == 0 ? (long long)list[t] : 0LL, 0);
        if (b < 0 || b >= batch) {                        // out-of-range entries are skipped
            if (next != nullptr && lane == 0) next[t] = -1;
            continue;
        }
        const float* a = A + b * nn;
        float* x = X + b * nn;
        for (int e = lane; e < 32 * 32; e += 32) {
            const int i = e >> 5, j = e & 31;
            const bool in = i < n && j < n;
            at[j * kDfPitchT + i] = in ? a[i * n + j] : 0.0f;
            xt[j * kDfPitchT + i] = in ? x[i * n + j] : 0.0f;
        }
        __syncwarp();
        const int j = lane;
        // my column of X, each entry duplicated in a register pair
        float2 xc[32];
        float xmax = 0.0f;
#pragma unroll
        for (int k = 0; k < 32; k += 2) {
            const float2 v = *reinterpret_cast<const float2*>(xt + j * kDfPitchT + k);
            xc[k] = make_float2(v.x, v.x);
            xc[k + 1] = make_float2(v.y, v.y);
            xmax = fmaxf(xmax, fmaxf(fabsf(v.x), fabsf(v.y)));
        }
        // column j of R = I - A X, rows in pairs, accumulated as -(A X) + I in
        // float-float; two row pairs at a time, so two TwoSum chains overlap
        for (int i = 0; i < 32; i += 4) {
            float2 s0 = make_float2(0.0f, 0.0f), c0 = make_float2(0.0f, 0.0f);
            float2 s1 = make_float2(0.0f, 0.0f), c1 = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int k = 0; k < 32; k++) {
                const float2 a0 = *reinterpret_cast<const float2*>(at + k * kDfPitchT + i);
                const float2 a1 = *reinterpret_cast<const float2*>(at + k * kDfPitchT + i + 2);
                df_madd2(s0, c0, neg2(a0), xc[k]);
                df_madd2(s1, c1, neg2(a1), xc[k]);
            }
            mr[i * kDfPitch + j] = df_round(s0.x, c0.x, (i == j) ? 1.0f : 0.0f);
            mr[(i + 1) * kDfPitch + j] = df_round(s0.y, c0.y, (i + 1 == j) ? 1.0f : 0.0f);
            mr[(i + 2) * kDfPitch + j] = df_round(s1.x, c1.x, (i + 2 == j) ? 1.0f : 0.0f);
            mr[(i + 3) * kDfPitch + j] = df_round(s1.y, c1.y, (i + 3 == j) ? 1.0f : 0.0f);
        }
        __syncwarp();                                      // R complete, A^T no longer read
        // column j of X + X R in FP32, rows in pairs; the correction D = X R
        // goes to the A^T tile (transposed) when the next-step estimate is wanted
        float2 rc[32];
#pragma unroll
        for (int k = 0; k < 32; k++) {
            const float v = mr[k * kDfPitch + j];
            rc[k] = make_float2(v, v);
        }
        for (int i = 0; i < 32; i += 2) {
            float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int k = 0; k < 32; k++)
                acc = __ffma2_rn(*reinterpret_cast<const float2*>(xt + k * kDfPitchT + i), rc[k], acc);
            const float2 xo = *reinterpret_cast<const float2*>(xt + j * kDfPitchT + i);   // X[i][j], X[i+1][j]
            if (j < n) {
                if (i < n) x[i * n + j] = xo.x + acc.x;
                if (i + 1 < n) x[(i + 1) * n + j] = xo.y + acc.y;
            }
            if (next != nullptr) *reinterpret_cast<float2*>(at + j * kDfPitchT + i) = acc;
        }
        if (next != nullptr) {
            __syncwarp();
            // column j of D R = X R^2; the error left is about max|X R^2| / max|X|
            float emax = 0.0f;
            bool nan = false;
            for (int i = 0; i < 32; i += 2) {
                float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
                for (int k = 0; k < 32; k++)
                    acc = __ffma2_rn(*reinterpret_cast<const float2*>(at + k * kDfPitchT + i), rc[k], acc);
                nan = nan || isnan(acc.x) || isnan(acc.y);
                emax = fmaxf(emax, fmaxf(fabsf(acc.x), fabsf(acc.y)));
            }
            float xm = xmax;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) xm = fmaxf(xm, __shfl_xor_sync(0xffffffffu, xm, o));
            const bool bad = nan || !(emax <= tol * xm);   // inf fails the comparison too
            const unsigned any = __ballot_sync(0xffffffffu, bad);
            if (lane == 0) next[t] = any ? (int32_t)b : -1;
        }
        __syncwarp();
    }
}

// list[b] = b if ||A_b||_1 * ||X_b||_1 >= threshold (a cheap estimate of the
// condition number from the inverse itself), else -1.  One warp per matrix,
// lane = column (coalesced rows), max of the column sums over the warp.
__global__ void mi_flag_condition_kernel(const float* __restrict__ A, const float* __restrict__ X, long long batch,
                                         int n, float threshold, int32_t* __restrict__ list) {
    const int lane = threadIdx.x & 31;
    const long long nn = (long long)n * n;
    for (long long b = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; b < batch;
         b += ((long long)gridDim.x * blockDim.x) >> 5) {
        float ca = 0.0f, cx = 0.0f;
        if (lane < n) {
            const float* a = A + b * nn + lane;
            const float* x = X + b * nn + lane;
            for (int i = 0; i < n; i++) {
                ca += fabsf(a[(long long)i * n]);
                cx += fabsf(x[(long long)i * n]);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            ca = fmaxf(ca, __shfl_xor_sync(0xffffffffu, ca, o));
            cx = fmaxf(cx, __shfl_xor_sync(0xffffffffu, cx, o));
        }
        const float est = ca * cx;
        // a non-finite estimate (inf or NaN in the inverse) is flagged too
        if (lane == 0) list[b] = (!(est < threshold)) ? (int32_t)b : -1;
    }
}

}  // namespace mi

extern "C" int mi_flag_condition_f32(const float* d_a, const float* d_x, int64_t batch, int n, float threshold,
                                     int32_t* d_list, void* stream) {
    if (n < 1 || n > 32 || batch < 0) return MI_ERR_INVALID_VALUE;
    if (batch == 0) return MI_OK;
    if (d_a == nullptr || d_x == nullptr || d_list == nullptr) return MI_ERR_NULL_POINTER;
    long long blocks = (batch + 7) / 8;                   // 8 warps per block
    const long long cap = 16LL * mi::device_sm_count();
    if (blocks > cap) blocks = cap;
    mi::mi_flag_condition_kernel<<<(unsigned)blocks, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        d_a, d_x, batch, n, threshold, d_list);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return mi::set_cuda_error(e, "condition flag launch");
    return MI_OK;
}

extern "C" int mi_refine_df_next_f32(const float* d_a, float* d_x, const int32_t* d_list, int64_t count,
                                     int64_t batch, int n, float tol, int32_t* d_next, void* stream) {
    if (n < 1 || n > 32 || count < 0 || batch < 0) return MI_ERR_INVALID_VALUE;
    if (d_next != nullptr && !(tol >= 0.0f)) return MI_ERR_INVALID_VALUE;
    if (count == 0) return MI_OK;
    if (d_a == nullptr || d_x == nullptr || d_list == nullptr) return MI_ERR_NULL_POINTER;
    static int per_sm[64] = {0};
    const long long blocks = mi::resident_grid(reinterpret_cast<const void*>(mi::mi_refine_df_kernel),
                                               32 * mi::kDfWarps, (count + mi::kDfWarps - 1) / mi::kDfWarps, per_sm);
    mi::mi_refine_df_kernel<<<(unsigned)blocks, 32 * mi::kDfWarps, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        d_a, d_x, d_list, count, batch, n, tol, d_next);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return mi::set_cuda_error(e, "float-float refinement launch");
    return MI_OK;
}

extern "C" int mi_refine_df_f32(const float* d_a, float* d_x, const int32_t* d_list, int64_t count, int64_t batch,
                                int n, void* stream) {
    return mi_refine_df_next_f32(d_a, d_x, d_list, count, batch, n, 0.0f, nullptr, stream);
}
