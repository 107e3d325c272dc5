// mi_noalloc.cu -- descriptor batches whose bucketing scratch lives in a
// fixed file-scope device array, for callers that cannot allocate device
// memory at call time (see mi_inverse_descr_noalloc_f32 in mi_inverse.h).
//
// The per-call work is exactly mi_inverse_descr_f32's: this file only
// supplies the workspace pointer.
#include <cuda.h>
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
static CUcontext g_noalloc_ctx[kNoAllocMaxDevices];   // the context each address belongs to
static std::mutex g_noalloc_mu;

using ctx_get_fn = CUresult (*)(CUcontext*);

// The driver's cuCtxGetCurrent, found once through the runtime (the library
// does not link the driver library).
static ctx_get_fn ctx_get_current() {
    static ctx_get_fn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<ctx_get_fn>(p);
    });
    return fn;
}

// Device address of the scratch on the current device, looked up once per
// device and context (cudaGetSymbolAddress with that device current).  A new
// context on the device -- after cudaDeviceReset, say, which unloads the
// library's device code with the old one -- gets a fresh look-up.
static int noalloc_scratch(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_cuda_error(e, "no-allocation scratch: current device");
    if (dev < 0 || dev >= kNoAllocMaxDevices) return MI_ERR_INVALID_VALUE;
    // the current context, or none yet (then the look-up below creates it
    // and the next call records it)
    CUcontext ctx = nullptr;
    const ctx_get_fn get = ctx_get_current();
    if (get != nullptr && get(&ctx) != CUDA_SUCCESS) ctx = nullptr;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (g_noalloc_ptr[dev] == nullptr || g_noalloc_ctx[dev] != ctx || ctx == nullptr) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return set_cuda_error(e, "no-allocation scratch: symbol address");
        g_noalloc_ptr[dev] = p;
        g_noalloc_ctx[dev] = ctx;
    }
    *out = g_noalloc_ptr[dev];
    return MI_OK;
}

}  // namespace mi

extern "C" int mi_inverse_descr_noalloc_f32(float* d_packed, int64_t packed_floats, const int64_t* d_offsets,
                                            const int32_t* d_n, const int32_t* d_flags, int32_t* d_perm,
                                            int32_t* d_info, int64_t count, uint32_t n_mask, uint32_t mode_mask,
                                            void* stream) {
    if (count > MI_NOALLOC_MAX_COUNT) return MI_ERR_SCRATCH_LIMIT;
    if (count <= 0 || packed_floats < 0) return (count < 0 || packed_floats < 0) ? MI_ERR_INVALID_VALUE : MI_OK;
    void* scratch = nullptr;
    const int status = mi::noalloc_scratch(&scratch);
    if (status != MI_OK) return status;
    // the workspace entry point clears the bucket counters on `stream` before use
    return mi_inverse_descr_f32(d_packed, packed_floats, d_offsets, d_n, d_flags, d_perm, d_info, count, n_mask,
                                mode_mask, scratch, mi::kNoAllocBytes, stream);
}
