// mi_descr.cu -- mixed sizes in one call: an (offset, n, pivot flag)
// descriptor table is bucketed by (n, flag) on the GPU (count, scan, scatter
// into caller-provided workspace), then either one persistent launch walks
// every bucket (mi_descr_persist.cu) or one persistent indexed launch per
// bucket (the default) walks that bucket's matrices.  Nothing waits on the host
// between the steps, so the whole call can be captured into one CUDA graph.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "mi_inverse.h"
#include "mi_launch.cuh"

namespace mi {

constexpr int kBuckets = 32 * 4;                 // (n - 1) * 4 + mode
constexpr size_t kOffCounts = 0;                 // uint32[128]
constexpr size_t kOffCounter = 512;              // uint32: chunk counter of the persistent launch
constexpr size_t kOffCursors = 1024;             // uint32[128]
constexpr size_t kOffRanges = 2048;              // long long[128][2]: start, count
constexpr size_t kOffList = 4096;                // int32[count]
constexpr size_t kZeroed = 1024;                 // counts and counter, cleared per call

cudaError_t launch_descr_persistent(float* base, const long long* offsets, const int* list, const long long* ranges,
                                    uint32_t n_mask, uint32_t mode_mask, int chunk_floats, unsigned int* counter,
                                    int32_t* perm, int32_t* info, cudaStream_t stream);   // mi_descr_persist.cu

// Input floats per chunk of the single persistent launch; 0 (the default)
// selects one launch per bucket (mi_set_descr_chunk).  The per-bucket form
// is the default because it measured faster: the persistent kernel runs
// every body at one block of 8 warps per SM (the largest walk needs 255
// registers) and its walks are separately compiled functions, so each body
// ran 1.5-2.4x slower than as its own kernel (131,072 matrices of one size:
// n = 32 reference rule 0.67 against 0.46 ms).
std::atomic<int> g_descr_chunk{0};

// Bucket counts: a shared-memory histogram per block, then one global
// atomic per non-empty bucket per block (a million descriptors land on a few
// dozen buckets, so per-descriptor global atomics would serialise).
// A descriptor is well-formed when n is 1..32, the flag a pivot mode, and its
// matrix lies inside the packed buffer of `packed` floats.
__device__ __forceinline__ bool descr_ok(int n, int f, long long off, long long packed) {
    return n >= 1 && n <= 32 && f >= 0 && f <= 3 && off >= 0 && off <= packed - (long long)n * n;
}

__global__ void descr_count(const int32_t* __restrict__ ns, const int32_t* __restrict__ flags,
                            const long long* __restrict__ offsets, long long packed, long long count,
                            unsigned int* __restrict__ counts, int32_t* __restrict__ info) {
    __shared__ unsigned int hist[kBuckets];
    for (int b = threadIdx.x; b < kBuckets; b += blockDim.x) hist[b] = 0u;
    __syncthreads();
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        const int n = ns[i], f = flags[i];
        if (descr_ok(n, f, offsets[i], packed)) atomicAdd(&hist[(n - 1) * 4 + f], 1u);
        else if (info != nullptr) info[i] = -1;   // malformed descriptor: reported, not processed
    }
    __syncthreads();
    for (int b = threadIdx.x; b < kBuckets; b += blockDim.x)
        if (hist[b] != 0u) atomicAdd(&counts[b], hist[b]);
}

__global__ void descr_scan(const unsigned int* __restrict__ counts, unsigned int* __restrict__ cursors,
                           long long* __restrict__ ranges) {
    __shared__ unsigned int c[kBuckets];
    const int t = threadIdx.x;
    c[t] = counts[t];
    __syncthreads();
    if (t == 0) {
        unsigned int run = 0;                    // at most the descriptor count (< 2^31)
        for (int b = 0; b < kBuckets; b++) {
            const unsigned int v = c[b];
            c[b] = run;
            run += v;
        }
    }
    __syncthreads();
    cursors[t] = c[t];
    ranges[2 * t] = (long long)c[t];
    ranges[2 * t + 1] = (long long)counts[t];
}

// List scatter in chunks of blockDim descriptors: the block ranks each
// descriptor within its bucket in shared memory, reserves the chunk's range
// of every bucket with one global atomic, then writes the indices.  (Order
// within a bucket is not significant: each matrix is independent.)
__global__ void descr_scatter(const int32_t* __restrict__ ns, const int32_t* __restrict__ flags,
                              const long long* __restrict__ offsets, long long packed, long long count,
                              unsigned int* __restrict__ cursors, int32_t* __restrict__ list) {
    __shared__ unsigned int hist[kBuckets];
    __shared__ unsigned int base[kBuckets];
    for (long long c0 = (long long)blockIdx.x * blockDim.x; c0 < count; c0 += (long long)gridDim.x * blockDim.x) {
        for (int b = threadIdx.x; b < kBuckets; b += blockDim.x) hist[b] = 0u;
        __syncthreads();
        const long long i = c0 + threadIdx.x;
        int bucket = -1;
        unsigned int rank = 0u;
        if (i < count) {
            const int n = ns[i], f = flags[i];
            if (descr_ok(n, f, offsets[i], packed)) {
                bucket = (n - 1) * 4 + f;
                rank = atomicAdd(&hist[bucket], 1u);
            }
        }
        __syncthreads();
        for (int b = threadIdx.x; b < kBuckets; b += blockDim.x)
            if (hist[b] != 0u) base[b] = atomicAdd(&cursors[b], hist[b]);
        __syncthreads();
        if (bucket >= 0) list[base[bucket] + rank] = (int32_t)i;
        __syncthreads();
    }
}

int tuned_threads(int n, int mode);   // mi_api.cu
int set_cuda_error(cudaError_t e, const char* what);

}  // namespace mi

extern "C" {

size_t mi_descr_workspace_bytes(int64_t count) {
    if (count < 0) return 0;
    return (mi::kOffList + 4 * (size_t)count + 255) & ~(size_t)255;
}

int mi_inverse_descr_f32(float* d_packed, int64_t packed_floats, const int64_t* d_offsets, const int32_t* d_n,
                         const int32_t* d_flags, int32_t* d_perm, int32_t* d_info, int64_t count, uint32_t n_mask,
                         uint32_t mode_mask, void* d_workspace, size_t workspace_bytes, void* stream) {
    if (count < 0 || count > 0x7fffffffLL || packed_floats < 0) return MI_ERR_INVALID_VALUE;
    if (count == 0) return MI_OK;
    if (d_packed == nullptr || d_offsets == nullptr || d_n == nullptr || d_flags == nullptr || d_workspace == nullptr)
        return MI_ERR_NULL_POINTER;
    if ((reinterpret_cast<uintptr_t>(d_packed) & 3u) != 0 || (reinterpret_cast<uintptr_t>(d_workspace) & 255u) != 0)
        return MI_ERR_MISALIGNED;
    if (workspace_bytes < mi_descr_workspace_bytes(count)) return MI_ERR_INVALID_VALUE;
    if (n_mask == 0) n_mask = 0xffffffffu;
    if (mode_mask == 0) mode_mask = 0xfu;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    unsigned char* ws = static_cast<unsigned char*>(d_workspace);
    auto* counts = reinterpret_cast<unsigned int*>(ws + mi::kOffCounts);
    auto* counter = reinterpret_cast<unsigned int*>(ws + mi::kOffCounter);
    auto* cursors = reinterpret_cast<unsigned int*>(ws + mi::kOffCursors);
    auto* ranges = reinterpret_cast<long long*>(ws + mi::kOffRanges);
    auto* list = reinterpret_cast<int32_t*>(ws + mi::kOffList);

    cudaError_t e = cudaMemsetAsync(ws, 0, mi::kZeroed, st);
    if (e != cudaSuccess) return mi::set_cuda_error(e, "descriptor bucketing");
    const int sms = mi::device_sm_count();
    long long blocks = (count + 255) / 256;
    if (blocks > 4LL * sms) blocks = 4LL * sms;
    const long long* off64 = reinterpret_cast<const long long*>(d_offsets);
    mi::descr_count<<<(unsigned)blocks, 256, 0, st>>>(d_n, d_flags, off64, packed_floats, count, counts, d_info);
    mi::descr_scan<<<1, mi::kBuckets, 0, st>>>(counts, cursors, ranges);
    mi::descr_scatter<<<(unsigned)blocks, 256, 0, st>>>(d_n, d_flags, off64, packed_floats, count, cursors, list);
    e = cudaGetLastError();
    if (e != cudaSuccess) return mi::set_cuda_error(e, "descriptor bucketing");

    const int chunk = mi::g_descr_chunk.load(std::memory_order_relaxed);
    if (chunk > 0) {
        e = mi::launch_descr_persistent(d_packed, off64, list, ranges, n_mask, mode_mask, chunk, counter, d_perm,
                                        d_info, st);
        return e == cudaSuccess ? MI_OK : mi::set_cuda_error(e, "descriptor persistent launch");
    }
    const mi::ilaunch_fn* tables[4] = {mi::kITableNone, mi::kITableReference, mi::kITableReferenceSerial,
                                       mi::kITablePartial};
    for (int n = 1; n <= 32; n++) {
        if (!((n_mask >> (n - 1)) & 1u)) continue;
        for (int mode = 0; mode < 4; mode++) {
            if (!((mode_mask >> mode) & 1u)) continue;
            const int b = (n - 1) * 4 + mode;
            e = tables[mode][n](d_packed, off64, list, ranges + 2 * b, d_perm, d_info, mi::tuned_threads(n, mode), 0,
                                st);
            if (e != cudaSuccess) return mi::set_cuda_error(e, "descriptor bucket launch");
        }
    }
    return MI_OK;
}

int mi_set_descr_chunk(int chunk_floats) {
    if (chunk_floats < 0) return MI_ERR_INVALID_VALUE;
    mi::g_descr_chunk.store(chunk_floats, std::memory_order_relaxed);
    return MI_OK;
}

int mi_get_descr_chunk(void) { return mi::g_descr_chunk.load(std::memory_order_relaxed); }

}  // extern "C"
