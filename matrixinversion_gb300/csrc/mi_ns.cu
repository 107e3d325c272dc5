// mi_ns.cu -- Newton-Schulz refinement of batched 32 x 32 inverses on the
// tensor cores:  X <- X + X (I - A X),  1 or 2 steps.
//
// A CTA of 128 threads takes 4 matrices per tile, stacked into the M = 128
// rows of tcgen05.mma (kind::tf32, N = 128, K = 32 in four k-steps).  The
// product of the stacked A with the side-by-side X's holds every A_i X_j;
// only the four diagonal 32 x 32 blocks are read back (tcgen05.ld), so the
// tensor cores do 4x the useful work -- still far below their rate.  Each
// operand is split into a TF32 head and an FP32 remainder and every product
// is formed as hi*hi + hi*lo + lo*hi (3xTF32, FP32 accumulation in tensor
// memory), which keeps FP32-level accuracy in the residual.
//
// Shared-memory operands use the no-swizzle K-major layout: 8-row x 16-byte
// core matrices, with padded pitches (144 bytes between the two core
// matrices of a k-step, 288 between 8-row groups, 4640 between k-steps) so
// that the transposed stores of X^T and R^T hit 32 distinct banks.
#include <cuda_runtime.h>

#include <cstdint>

#include "mi_inverse.h"
#include "mi_kernel.cuh"
#include "mi_ptx.cuh"
#include "mi_tc.cuh"

namespace mi {

int set_cuda_error(cudaError_t e, const char* what);   // mi_api.cu
int device_sm_count();

namespace ns {

constexpr int kLbo = 144, kSbo = 288, kStep = 4640;          // bytes
constexpr int kOpFloats = 4 * kStep / 4;                     // one operand buffer (4 k-steps)
constexpr uint32_t kIdesc = tc_idesc_tf32(128, 128);

// float index of element (row m, column k) of a 128 x 32 K-major operand
__device__ __forceinline__ int off(int m, int k) {
    return (k >> 3) * (kStep / 4) + (m >> 3) * (kSbo / 4) + ((k >> 2) & 1) * (kLbo / 4) + (m & 7) * 4 + (k & 3);
}

struct Smem {
    float ah[kOpFloats], al[kOpFloats];     // A (operand A of A X)
    float xah[kOpFloats], xal[kOpFloats];   // X (operand A of X R)
    float bh[kOpFloats], bl[kOpFloats];     // X^T (operand B of A X), then R^T (of X R), then the output stage
    uint64_t bar;
    uint32_t tmem;
};

__device__ __forceinline__ void put(float* h, float* l, int o, float v) {
    const float hv = tf32_head(v);
    h[o] = hv;
    l[o] = v - hv;
}

__device__ __forceinline__ void put4(float* h, float* l, int o, float4 v) {
    const float4 hv = make_float4(tf32_head(v.x), tf32_head(v.y), tf32_head(v.z), tf32_head(v.w));
    *reinterpret_cast<float4*>(h + o) = hv;
    *reinterpret_cast<float4*>(l + o) = make_float4(v.x - hv.x, v.y - hv.y, v.z - hv.z, v.w - hv.w);
}

// D (tensor memory) = Ah Bh^T + Ah Bl^T + Al Bh^T over K = 32.
__device__ __forceinline__ void mma3(uint32_t tmem, const float* ah, const float* al, const float* bh,
                                     const float* bl) {
    const float* as[3] = {ah, ah, al};
    const float* bs[3] = {bh, bl, bh};
#pragma unroll
    for (int p = 0; p < 3; p++)
#pragma unroll
        for (int s = 0; s < 4; s++)
            tc_mma_tf32(tmem, tc_desc(smem_addr(as[p]) + s * kStep, kLbo, kSbo),
                        tc_desc(smem_addr(bs[p]) + s * kStep, kLbo, kSbo), kIdesc, p > 0 || s > 0);
}

}  // namespace ns

__global__ void __launch_bounds__(128, 2) mi_ns_kernel(const float* __restrict__ A, float* __restrict__ X,
                                                       long long batch, int steps) {
    using namespace ns;
    extern __shared__ unsigned char smem_raw[];
    Smem& sm = *reinterpret_cast<Smem*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~static_cast<uintptr_t>(127));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        mbar_init(&sm.bar, 1);
        fence_mbar_init();
    }
    if (warp == 0) {
        tc_alloc(&sm.tmem, 128);
        tc_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = sm.tmem;
    // this warp's TMEM lanes (rows 32w ..), columns of its diagonal block
    const uint32_t tblk = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(32 * warp);
    uint32_t phase = 0;
    bool failed = false;
    const long long tiles = (batch + 3) / 4;
    for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const long long mat = tile * 4 + warp;
        const bool valid = mat < batch;
        const float4* ga = reinterpret_cast<const float4*>(A + mat * 1024);
        const float4* gx = reinterpret_cast<const float4*>(X + mat * 1024);
        // all of this tile's loads in flight at once, before waiting for the
        // previous tile's output stage (bh) to be read by its bulk store
        float4 ra[8], rx[8];
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
            ra[q] = valid ? ga[lane + 32 * q] : zero;
            rx[q] = valid ? gx[lane + 32 * q] : zero;
        }
        if (tid == 0) bulk_wait_read_all();
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int f = lane + 32 * q;               // float4 index within the matrix
            const int r = f >> 3, c = (f & 7) * 4;
            const float4 a = ra[q];
            const float4 x = rx[q];
            const int m = 32 * warp + r;
            put4(sm.ah, sm.al, off(m, c), a);
            put4(sm.xah, sm.xal, off(m, c), x);
            // X^T: operand-B row n = 32w + column, k = row
            put(sm.bh, sm.bl, off(32 * warp + c + 0, r), x.x);
            put(sm.bh, sm.bl, off(32 * warp + c + 1, r), x.y);
            put(sm.bh, sm.bl, off(32 * warp + c + 2, r), x.z);
            put(sm.bh, sm.bl, off(32 * warp + c + 3, r), x.w);
        }
        float xn[32];
        for (int it = 0; it < steps; it++) {
            // ---- P = A X
            fence_proxy_async();
            tc_fence_before();
            __syncthreads();
            bool ok = true;
            if (tid == 0) {
                tc_fence_after();
                ns::mma3(tmem, sm.ah, sm.al, sm.bh, sm.bl);
                tc_commit(&sm.bar);
                ok = mbar_wait(&sm.bar, phase & 1u, kWaitLimit);
                // a product still running when the CTA gives up writes TMEM that
                // is freed on the way out: wait for it once more, bounded
                if (!ok) mbar_wait(&sm.bar, phase & 1u, kWaitLimit);
            }
            // one thread waits; the whole CTA learns the outcome at the barrier
            if (__syncthreads_or(!ok)) { failed = true; break; }
            phase++;
            tc_fence_after();
            float p[32];
            tc_ld32(tblk, p);
            // ---- R = I - P, stored as R^T (operand B): row n = 32w + j, k = my row
#pragma unroll
            for (int j = 0; j < 32; j++) put(sm.bh, sm.bl, off(32 * warp + j, lane), (j == lane ? 1.0f : 0.0f) - p[j]);
            // ---- D = X R
            fence_proxy_async();
            tc_fence_before();
            __syncthreads();
            ok = true;
            if (tid == 0) {
                tc_fence_after();
                ns::mma3(tmem, sm.xah, sm.xal, sm.bh, sm.bl);
                tc_commit(&sm.bar);
                ok = mbar_wait(&sm.bar, phase & 1u, kWaitLimit);
                // a product still running when the CTA gives up writes TMEM that
                // is freed on the way out: wait for it once more, bounded
                if (!ok) mbar_wait(&sm.bar, phase & 1u, kWaitLimit);
            }
            if (__syncthreads_or(!ok)) { failed = true; break; }
            phase++;
            tc_fence_after();
            float d[32];
            tc_ld32(tblk, d);
            const int m = 32 * warp + lane;
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const float4 h = *reinterpret_cast<const float4*>(sm.xah + off(m, 4 * q));
                const float4 l = *reinterpret_cast<const float4*>(sm.xal + off(m, 4 * q));
                xn[4 * q + 0] = (h.x + l.x) + d[4 * q + 0];
                xn[4 * q + 1] = (h.y + l.y) + d[4 * q + 1];
                xn[4 * q + 2] = (h.z + l.z) + d[4 * q + 2];
                xn[4 * q + 3] = (h.w + l.w) + d[4 * q + 3];
            }
            if (it + 1 < steps) {
                // the next step's operands: my row of X (operand A) and my column of X^T
                // (operand B; R^T there has been consumed by the completed product)
                tc_fence_before();
                __syncthreads();
#pragma unroll
                for (int q = 0; q < 8; q++)
                    put4(sm.xah, sm.xal, off(m, 4 * q),
                         make_float4(xn[4 * q], xn[4 * q + 1], xn[4 * q + 2], xn[4 * q + 3]));
#pragma unroll
                for (int j = 0; j < 32; j++) put(sm.bh, sm.bl, off(32 * warp + j, lane), xn[j]);
            }
        }
        if (failed) break;                // uniform: decided at a barrier
        // ---- output: rows to a row-major stage (bh), 16-byte chunks rotated by
        // the row against bank conflicts, then one bulk store for the tile
        tc_fence_before();
        __syncthreads();
        float* stage = sm.bh;
#pragma unroll
        for (int q0 = 0; q0 < 8; q0++) {
            const int q = (q0 + lane) & 7;
            float4 v;
            // static register indexing: select chunk q
            v = make_float4(xn[0], xn[1], xn[2], xn[3]);
#pragma unroll
            for (int t = 1; t < 8; t++)
                if (q == t) v = make_float4(xn[4 * t], xn[4 * t + 1], xn[4 * t + 2], xn[4 * t + 3]);
            *reinterpret_cast<float4*>(stage + (32 * warp + lane) * 32 + 4 * q) = v;
        }
        fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            const long long left = batch - tile * 4;
            const int cnt = left < 4 ? (int)left : 4;
            bulk_store(X + tile * 4 * 1024, stage, (uint32_t)(cnt * 4096));
            bulk_commit();
        }
    }
    if (failed && tid == 0) atomicOr(&g_device_error, 2);   // a tensor-core wait timed out
    if (tid == 0) bulk_wait_all();
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tc_dealloc(tmem, 128);
}

}  // namespace mi

extern "C" int mi_newton_schulz_f32(const float* d_a, float* d_x, int64_t batch, int n, int steps, void* stream) {
    if (n != 32 || batch < 0 || steps < 1 || steps > 4) return MI_ERR_INVALID_VALUE;
    if (batch == 0) return MI_OK;
    if (d_a == nullptr || d_x == nullptr) return MI_ERR_NULL_POINTER;
    if ((reinterpret_cast<uintptr_t>(d_a) & 15u) != 0 || (reinterpret_cast<uintptr_t>(d_x) & 15u) != 0)
        return MI_ERR_MISALIGNED;
    const size_t smem = sizeof(mi::ns::Smem) + 128;
    static size_t smem_set[mi::kMaxDevices] = {};
    {
        const cudaError_t e = mi::opt_in_smem(mi::mi_ns_kernel, smem, smem_set);
        if (e != cudaSuccess) return mi::set_cuda_error(e, "newton-schulz attributes");
    }
    const long long tiles = (batch + 3) / 4;
    long long grid = 2LL * mi::device_sm_count();
    if (grid > tiles) grid = tiles;
    mi::mi_ns_kernel<<<(unsigned)grid, 128, smem, reinterpret_cast<cudaStream_t>(stream)>>>(d_a, d_x, batch, steps);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return mi::set_cuda_error(e, "newton-schulz launch");
    return MI_OK;
}
