// mi_descr_persist.cu -- the single persistent launch of a descriptor call
// (mi_persist.cuh): the plan of chunks, the work loop and its launch.
// Relocatable device code: the walks it calls are in mi_pwalk_*.cu.
#include <cuda_runtime.h>

#include <cstdint>

#include "mi_persist.cuh"

namespace mi {

constexpr int kPlanEntries = 128;   // (n, mode) buckets
constexpr int kMaxChunkGroups = 8;

// Bucket at position i of the plan: n from 32 down to 1 (the costliest
// groups first, so the last chunks handed out are the cheapest), modes 0..3.
__host__ __device__ constexpr int plan_bucket(int i) { return (31 - i / 4) * 4 + (i & 3); }

__device__ __forceinline__ bool persist_dispatch(int bucket, MI_PWALK_PARAMS) {
    switch (bucket) {
#define MI_PCASE(M, N) \
    case (N - 1) * 4 + M: return pwalk_##M##_##N(MI_PWALK_ARGS);
        MI_PWALK_EACH_N(MI_PCASE, 0)
        MI_PWALK_EACH_N(MI_PCASE, 1)
        MI_PWALK_EACH_N(MI_PCASE, 2)
        MI_PWALK_EACH_N(MI_PCASE, 3)
#undef MI_PCASE
        default: return true;
    }
}

// Every block first lays out the plan: plan entry i (bucket plan_bucket(i),
// count from `ranges`, zero when the masks leave it out) is cut into chunks
// of k_i groups, k_i = chunk_floats / (group matrices x n^2) -- about
// chunk_floats input floats per chunk -- clamped to 1 .. kMaxChunkGroups,
// and s_first[i] is its first chunk in the global order.  Then each warp
// takes chunk numbers from `counter` (zero at launch) until they run out and
// walks the groups of each one.
//
// The clamp matters at small n: a group there costs about one copy latency
// whatever its size, so a chunk of the float budget (n = 2: 128 groups) ran
// as one long serial chain on one warp at the end of the launch (measured:
// 131,072 matrices of n = 2 in 0.140 ms at 128 groups per chunk, 0.047 ms at
// one).
__global__ void __launch_bounds__(kPersistWarps * 32, 1)
    mi_descr_persistent_kernel(float* __restrict__ base, const long long* __restrict__ offsets,
                               const int* __restrict__ list, const long long* __restrict__ ranges, uint32_t n_mask,
                               uint32_t mode_mask, int chunk_floats, unsigned int* __restrict__ counter,
                               int32_t* __restrict__ perm_out, int32_t* __restrict__ info_out) {
    __shared__ int s_first[kPlanEntries + 1];
    __shared__ int s_k[kPlanEntries];
    __shared__ int s_wsum[kPlanEntries / 32];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if (t < kPlanEntries) {                              // warps 0..3, whole
        const int b = plan_bucket(t), n = b / 4 + 1, mode = b & 3;
        const bool on = ((n_mask >> (n - 1)) & 1u) != 0u && ((mode_mask >> mode) & 1u) != 0u;
        const long long cnt = on ? ranges[2 * b + 1] : 0;
        const int m = persist_group(n, mode);
        const long long groups = (cnt + m - 1) / m;
        int k = chunk_floats / (m * n * n);
        k = k < 1 ? 1 : (k > kMaxChunkGroups ? kMaxChunkGroups : k);
        int v = (int)((groups + k - 1) / k);
        s_k[t] = k;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(kFull, v, o);
            if (lane >= o) v += u;
        }
        if (lane == 31) s_wsum[warp] = v;
        s_first[t + 1] = v;
    }
    __syncthreads();
    if (t < kPlanEntries) {
        int add = 0;
        for (int w = 0; w < warp; w++) add += s_wsum[w];
        s_first[t + 1] += add;
    }
    if (t == 0) s_first[0] = 0;
    __syncthreads();

    const int total = s_first[kPlanEntries];
    int i = 0;
    while (true) {
        int c = 0;
        if (lane == 0) c = (int)atomicAdd(counter, 1u);
        c = __shfl_sync(kFull, c, 0);
        if (c >= total) break;
        while (s_first[i + 1] <= c) i++;                 // chunk numbers only grow within a warp
        const int b = plan_bucket(i), n = b / 4 + 1, mode = b & 3;
        const long long start = ranges[2 * b], cnt = ranges[2 * b + 1];
        const int m = persist_group(n, mode);
        const long long groups = (cnt + m - 1) / m;
        const long long g0 = (long long)(c - s_first[i]) * s_k[i];
        const long long g1 = g0 + s_k[i] < groups ? g0 + s_k[i] : groups;
        // a wait that ran out leaves the warp's region in an unknown state:
        // the warp takes no more work (the device error word records it)
        if (!persist_dispatch(b, base, offsets, list, start, cnt, g0, g1, perm_out, info_out)) break;
    }
}

cudaError_t launch_descr_persistent(float* base, const long long* offsets, const int* list, const long long* ranges,
                                    uint32_t n_mask, uint32_t mode_mask, int chunk_floats, unsigned int* counter,
                                    int32_t* perm, int32_t* info, cudaStream_t stream) {
    auto kern = mi_descr_persistent_kernel;
    const size_t smem = persist_smem_bytes();
    static size_t smem_set[kMaxDevices] = {};
    cudaError_t e = opt_in_smem(kern, smem, smem_set);
    if (e != cudaSuccess) return e;
    static int per_sm_cached[kMaxDevices] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) dev = 0;
    int& per_sm = per_sm_cached[dev];
    if (per_sm == 0) {
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPersistWarps * 32, smem);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
    }
    kern<<<per_sm * device_sm_count(), kPersistWarps * 32, smem, stream>>>(base, offsets, list, ranges, n_mask,
                                                                           mode_mask, chunk_floats, counter, perm,
                                                                           info);
    return cudaGetLastError();
}

}  // namespace mi
