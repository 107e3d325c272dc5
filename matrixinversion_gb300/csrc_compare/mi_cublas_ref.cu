// mi_cublas_ref.cu -- the comparison point for measurements: cuBLAS
// getrfBatched + getriBatched on the same device buffers (the benchmark the
// reference describes in README.md:63-69 but does not ship).  Not part of
// the product path; built as its own library, libmi_cublas_ref.so.
//
// cuBLAS is column-major, so a row-major batch is handed over as its
// transpose: the column-major inverse of A^T read back row-major is A^-1.
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <vector>

namespace {
thread_local char g_err[256] = "";

struct Ctx {
    cublasHandle_t h = nullptr;
    float** dAarr = nullptr;
    float** dCarr = nullptr;
    long long cap = 0;
};
thread_local Ctx g_ctx;

__global__ void fill_ptrs(float** out, float* base, long long stride, long long count) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) out[i] = base + i * stride;
}

int fail(const char* what, int code) {
    std::snprintf(g_err, sizeof(g_err), "%s failed (%d)", what, code);
    return -1;
}
}  // namespace

extern "C" {

const char* mi_cublas_last_error(void) { return g_err; }

// dA: batch row-major n x n (overwritten by the LU factors); dC: output
// inverses; dPiv: int32[batch * n]; dInfo: int32[batch].  ms_getrf /
// ms_getri (nullable) receive the two phases' device times.
int mi_cublas_inverse_f32(float* dA, float* dC, int32_t* dPiv, int32_t* dInfo, int64_t batch, int n, void* stream,
                          float* ms_getrf, float* ms_getri) {
    if (batch <= 0 || n < 1 || batch > 0x7fffffffLL) return fail("arguments", 0);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    Ctx& c = g_ctx;
    if (c.h == nullptr && cublasCreate(&c.h) != CUBLAS_STATUS_SUCCESS) return fail("cublasCreate", 0);
    cublasSetStream(c.h, st);
    if (batch > c.cap) {
        cudaFree(c.dAarr);
        cudaFree(c.dCarr);
        if (cudaMalloc(&c.dAarr, batch * sizeof(float*)) != cudaSuccess) return fail("cudaMalloc", 0);
        if (cudaMalloc(&c.dCarr, batch * sizeof(float*)) != cudaSuccess) return fail("cudaMalloc", 0);
        c.cap = batch;
    }
    const int tpb = 256;
    const long long blocks = (batch + tpb - 1) / tpb;
    fill_ptrs<<<(unsigned)blocks, tpb, 0, st>>>(c.dAarr, dA, (long long)n * n, batch);
    fill_ptrs<<<(unsigned)blocks, tpb, 0, st>>>(c.dCarr, dC, (long long)n * n, batch);
    cudaEvent_t e0, e1, e2;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventCreate(&e2);
    cudaEventRecord(e0, st);
    cublasStatus_t s1 = cublasSgetrfBatched(c.h, n, c.dAarr, n, dPiv, dInfo, (int)batch);
    cudaEventRecord(e1, st);
    cublasStatus_t s2 = cublasSgetriBatched(c.h, n, (const float* const*)c.dAarr, n, dPiv, c.dCarr, n, dInfo,
                                            (int)batch);
    cudaEventRecord(e2, st);
    int rc = 0;
    if (s1 != CUBLAS_STATUS_SUCCESS) rc = fail("cublasSgetrfBatched", s1);
    else if (s2 != CUBLAS_STATUS_SUCCESS) rc = fail("cublasSgetriBatched", s2);
    if (ms_getrf != nullptr || ms_getri != nullptr) {
        cudaEventSynchronize(e2);
        if (ms_getrf) cudaEventElapsedTime(ms_getrf, e0, e1);
        if (ms_getri) cudaEventElapsedTime(ms_getri, e1, e2);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    cudaError_t ce = cudaGetLastError();
    if (rc == 0 && ce != cudaSuccess) rc = fail(cudaGetErrorString(ce), ce);
    return rc;
}

}  // extern "C"
