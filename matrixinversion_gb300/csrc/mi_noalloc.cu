// mi_noalloc.cu -- descriptor batches whose bucketing scratch lives in a
// fixed file-scope device array, for callers that cannot allocate device
// memory at call time (see mi_inverse_descr_noalloc_f32 in mi_inverse.h).
//
// The per-call work is exactly mi_inverse_descr_f32's: this file only
// supplies the workspace pointer.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "mi_inverse.h"

namespace mi {

int set_cuda_error(cudaError_t e, const char* what);   // mi_api.cu

// Same layout as the caller-provided workspace: 4 KB of bucket counters,
// cursors and ranges, then one int32 list entry per descriptor.
constexpr size_t kNoAllocBytes = 4096 + 4 * (size_t)MI_NOALLOC_MAX_COUNT;
static_assert(kNoAllocBytes % 256 == 0, "scratch size must keep the 256-byte workspace rounding");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kNoAllocMaxDevices = 64;
static void* g_noalloc_ptr[kNoAllocMaxDevices];
static std::mutex g_noalloc_mu;

// Device address of the scratch on the current device, looked up once per
// device (cudaGetSymbolAddress with that device current).
static int noalloc_scratch(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_cuda_error(e, "no-allocation scratch: current device");
    if (dev < 0 || dev >= kNoAllocMaxDevices) return MI_ERR_INVALID_VALUE;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (g_noalloc_ptr[dev] == nullptr) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return set_cuda_error(e, "no-allocation scratch: symbol address");
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return MI_OK;
}

}  // namespace mi

extern "C" int mi_inverse_descr_noalloc_f32(float* d_packed, const int64_t* d_offsets, const int32_t* d_n,
                                            const int32_t* d_flags, int32_t* d_perm, int32_t* d_info, int64_t count,
                                            uint32_t n_mask, uint32_t mode_mask, void* stream) {
    if (count > MI_NOALLOC_MAX_COUNT) return MI_ERR_SCRATCH_LIMIT;
    if (count <= 0) return count < 0 ? MI_ERR_INVALID_VALUE : MI_OK;
    void* scratch = nullptr;
    const int status = mi::noalloc_scratch(&scratch);
    if (status != MI_OK) return status;
    // the workspace entry point clears the bucket counters on `stream` before use
    return mi_inverse_descr_f32(d_packed, d_offsets, d_n, d_flags, d_perm, d_info, count, n_mask, mode_mask, scratch,
                                mi::kNoAllocBytes, stream);
}
