// mi_launch.cuh -- host-side launch of one (n, pivot mode) instantiation of
// mi_inverse_kernel, and the per-mode dispatch tables the C ABI indexes.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "mi_kernel.cuh"

namespace mi {

using launch_fn = cudaError_t (*)(float*, int32_t*, int32_t*, long long, int, int, cudaStream_t);

constexpr int kMaxThreadsPerBlock = 256;
constexpr int kDefaultThreadsPerBlock = 128;

int device_sm_count();   // cached per device (mi_api.cu)

template <int N, int MODE>
cudaError_t launch(float* a, int32_t* perm, int32_t* info, long long batch, int tpb, int grid,
                   cudaStream_t stream) {
    using G = Geom<N>;
    const int warps = tpb / 32;
    const size_t smem = (size_t)warps * G::kPerWarp * sizeof(float);
    auto kern = mi_inverse_kernel<N, MODE>;
    static size_t smem_set = 0;   // largest dynamic size opted in so far
    if (smem > 48 * 1024 && smem > smem_set) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        smem_set = smem;
    }
    const long long groups = (batch + G::M - 1) / G::M;
    const long long need = (groups + warps - 1) / warps;
    if (grid <= 0) {
        int per_sm = 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, tpb, smem);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
        long long cap = (long long)per_sm * device_sm_count();
        grid = (int)(need < cap ? need : cap);
    }
    if (grid < 1) grid = 1;
    kern<<<grid, tpb, smem, stream>>>(a, perm, info, batch);
    return cudaGetLastError();
}

extern const launch_fn kTableNone[33];
extern const launch_fn kTableReference[33];
extern const launch_fn kTableReferenceSerial[33];
extern const launch_fn kTablePartial[33];

}  // namespace mi

#define MI_TABLE(NAME, MODE)                                                                      \
    const launch_fn NAME[33] = {                                                                  \
        nullptr,                launch<1, MODE>,  launch<2, MODE>,  launch<3, MODE>,  launch<4, MODE>,  \
        launch<5, MODE>,  launch<6, MODE>,  launch<7, MODE>,  launch<8, MODE>,  launch<9, MODE>,  \
        launch<10, MODE>, launch<11, MODE>, launch<12, MODE>, launch<13, MODE>, launch<14, MODE>, \
        launch<15, MODE>, launch<16, MODE>, launch<17, MODE>, launch<18, MODE>, launch<19, MODE>, \
        launch<20, MODE>, launch<21, MODE>, launch<22, MODE>, launch<23, MODE>, launch<24, MODE>, \
        launch<25, MODE>, launch<26, MODE>, launch<27, MODE>, launch<28, MODE>, launch<29, MODE>, \
        launch<30, MODE>, launch<31, MODE>, launch<32, MODE>}
