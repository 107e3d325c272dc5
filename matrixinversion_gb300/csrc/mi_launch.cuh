// mi_launch.cuh -- host-side launch of one (n, pivot mode) instantiation of
// mi_inverse_kernel, and the per-mode dispatch tables the C ABI indexes.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <cstring>

#include "mi_inverse.h"
#include "mi_kernel.cuh"

namespace mi {

using launch_fn = cudaError_t (*)(float*, int32_t*, int32_t*, long long, int, int, cudaStream_t);

constexpr int kMaxThreadsPerBlock = 256;
constexpr int kDefaultThreadsPerBlock = 128;

int device_sm_count();                                  // cached per device (mi_api.cu)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder();  // driver entry point (mi_api.cu)

}  // namespace mi

#include "mi_tiny.cuh"
#include "mi_rows.cuh"
#include "mi_wide.cuh"

namespace mi {

// 3-D tensor map over the batch: {column, row, matrix}, box of one warp's
// group of matrices; the 128-byte swizzle for n = 32 (rows are 128 bytes).
inline bool make_tensor_map(CUtensorMap* map, float* a, int n, long long batch, int box_rows, int box_matrices) {
    auto encode = tensor_map_encoder();
    if (encode == nullptr) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)n, (cuuint64_t)n, (cuuint64_t)batch};
    const cuuint64_t strides[2] = {(cuuint64_t)n * 4u, (cuuint64_t)n * n * 4u};
    const cuuint32_t box[3] = {(cuuint32_t)n, (cuuint32_t)box_rows, (cuuint32_t)box_matrices};
    const cuuint32_t estr[3] = {1u, 1u, 1u};
    const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, a, dims, strides, box, estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE,
                              n == 32 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

// n = 32 without partial pivoting: the eight-lane form (mi_wide.cuh), with
// tensor copies.  Sets *used = false, launching nothing, when the batch does
// not allow them (pointer not 16-byte aligned, more than 2^31 - 1 matrices).
template <int MODE>
cudaError_t launch_wide(float* a, int32_t* perm, int32_t* info, long long batch, int tpb, int grid,
                        cudaStream_t stream, bool* used) {
    using G = WideGeom;
    *used = false;
    CUtensorMap map, map_out;
    std::memset(&map, 0, sizeof(map));
    std::memset(&map_out, 0, sizeof(map_out));
    if ((reinterpret_cast<uintptr_t>(a) & 15u) != 0 || batch > 0x7fffffffLL ||
        !make_tensor_map(&map, a, G::N, batch, G::N, G::M) || !make_tensor_map(&map_out, a, G::N, batch, G::ORows, G::M))
        return cudaSuccess;
    *used = true;
    if (tpb > G::kThreadsMax) tpb = G::kThreadsMax;
    const int warps = tpb / 32;
    const size_t smem = wide_smem_bytes(warps);
    auto kern = mi_wide_kernel<MODE>;
    static size_t smem_set[kMaxDevices] = {};
    {
        const cudaError_t e = opt_in_smem(kern, smem, smem_set);
        if (e != cudaSuccess) return e;
    }
    const long long groups = (batch + G::M - 1) / G::M;
    const long long need = (groups + warps - 1) / warps;
    if (grid <= 0) {
        int per_sm = 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, tpb, smem);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
        const long long cap = (long long)per_sm * device_sm_count();
        grid = (int)(need < cap ? need : cap);
    }
    if (grid < 1) grid = 1;
    kern<<<grid, tpb, smem, stream>>>(a, perm, info, batch, map, map_out);
    return cudaGetLastError();
}

// The eight-lane form for descriptor buckets (IDX) and for contiguous batches
// the tensor copies cannot take (matrix b at a + 1024 b).
template <int MODE, bool IDX>
cudaError_t launch_wide_gather(float* a, const long long* offsets, const int* list, const long long* range,
                               long long batch, int32_t* perm, int32_t* info, int tpb, int grid,
                               cudaStream_t stream) {
    using G = WideGeom;
    if (tpb > G::kThreadsMax) tpb = G::kThreadsMax;
    const int warps = tpb / 32;
    const size_t smem = wide_smem_bytes(warps);
    auto kern = mi_wide_gather_kernel<MODE, IDX>;
    static size_t smem_set[kMaxDevices] = {};
    {
        const cudaError_t e = opt_in_smem(kern, smem, smem_set);
        if (e != cudaSuccess) return e;
    }
    if (grid <= 0) {
        static int per_sm_cached[kMaxDevices][G::kThreadsMax / 32 + 1] = {};
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) dev = 0;
        int& per_sm = per_sm_cached[dev][warps];
        if (per_sm == 0) {
            cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, tpb, smem);
            if (e != cudaSuccess) return e;
            if (per_sm < 1) per_sm = 1;
        }
        long long cap = (long long)per_sm * device_sm_count();
        if (!IDX) {
            const long long need = ((batch + G::M - 1) / G::M + warps - 1) / warps;
            if (need < cap) cap = need;
        }
        grid = (int)(cap < 1 ? 1 : cap);
    }
    kern<<<grid, tpb, smem, stream>>>(a, offsets, list, range, batch, perm, info);
    return cudaGetLastError();
}

// Lanes per matrix installed for (n, mode): the tuned table or its run-time
// override (mi_api.cu, mi_set_launch_lanes); default_lanes when unset.
int tuned_lanes(int n, int mode);

// The lane-group kernel (mi_inverse_kernel) for a contiguous batch.
template <int N, int MODE, int L = default_lanes(N, MODE)>
cudaError_t launch_lanes(float* a, int32_t* perm, int32_t* info, long long batch, int tpb, int grid,
                         cudaStream_t stream) {
    using G = Geom<N, L>;
    const int warps = tpb / 32;
    const size_t smem = smem_bytes<N, L, MODE>(warps);
    auto kern = mi_inverse_kernel<N, L, MODE>;
    static size_t smem_set[kMaxDevices] = {};       // largest dynamic size opted in, per device
    {
        const cudaError_t e = opt_in_smem(kern, smem, smem_set);
        if (e != cudaSuccess) return e;
    }

    // how each warp's group of M matrices moves in: tensor copies (rows of a
    // multiple of 16 bytes), 1-D bulk copies (16-byte aligned groups), or
    // per-element asynchronous copies; results leave with 16-byte stores when
    // rows allow
    CUtensorMap map, map_out;
    std::memset(&map, 0, sizeof(map));
    std::memset(&map_out, 0, sizeof(map_out));
    int copy_mode = kCopyPlain;
    const bool aligned16 = (reinterpret_cast<uintptr_t>(a) & 15u) == 0;
    if (aligned16) {
        if (N % 4 == 0 && batch <= 0x7fffffffLL && make_tensor_map(&map, a, N, batch, N, G::M) &&
            make_tensor_map(&map_out, a, N, batch, KGeom<N, L, MODE>::OBR, G::M))
            copy_mode = kCopyTensor;
        else if (N % 4 != 0)
            copy_mode = kCopyWindow;
        else if (((long long)G::M * N * N) % 4 == 0)
            copy_mode = kCopyBulk;
    }
    const int vec_out = (aligned16 && N % 4 == 0) ? 1 : 0;
    if (N == 32 && copy_mode != kCopyTensor) copy_mode = kCopyPlain;   // the swizzled layout needs the tensor copy

    const long long groups = (batch + G::M - 1) / G::M;
    const long long need = (groups + warps - 1) / warps;
    if (grid <= 0) {
        int per_sm = 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, tpb, smem);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
        const long long cap = (long long)per_sm * device_sm_count();
        grid = (int)(need < cap ? need : cap);
    }
    if (grid < 1) grid = 1;
    kern<<<grid, tpb, smem, stream>>>(a, perm, info, batch, copy_mode, vec_out, map, map_out);
    return cudaGetLastError();
}

// The lane-group kernel at the lanes per matrix installed for (n, mode) --
// from MI_LANES_ALT_MIN_BATCH matrices up; smaller batches run at the
// default width (measured on GB300: eight lanes, one block of eight warps per
// SM, win on batches of 262,144 and 1,000,000 matrices and lose on batches of
// about 16,000, where sixteen warps per SM hide more of each step's latency).
template <int N, int MODE>
cudaError_t launch_lanes_tuned(float* a, int32_t* perm, int32_t* info, long long batch, int tpb, int grid,
                               cudaStream_t stream) {
    constexpr int alt = alt_lanes(N, MODE);
    if constexpr (alt != 0)
        if (batch >= MI_LANES_ALT_MIN_BATCH && tuned_lanes(N, MODE) == alt)
            return launch_lanes<N, MODE, alt>(a, perm, info, batch, tpb, grid, stream);
    return launch_lanes<N, MODE>(a, perm, info, batch, tpb, grid, stream);
}

template <int N, int MODE>
cudaError_t launch(float* a, int32_t* perm, int32_t* info, long long batch, int tpb, int grid,
                   cudaStream_t stream) {
    if constexpr (N == WideGeom::N && MODE != kModePartial) {
        bool used = false;
        const cudaError_t e = launch_wide<MODE>(a, perm, info, batch, tpb, grid, stream, &used);
        if (used) return e;
        return launch_wide_gather<MODE, false>(a, nullptr, nullptr, nullptr, batch, perm, info, tpb, grid, stream);
    } else {
        if constexpr (N <= kTinyMax) {
            return launch_tiny<N, MODE>(a, perm, info, batch, tpb, grid, stream);
        } else if constexpr (N <= tiny_max_contig<MODE>()) {
            if (batch >= tiny_min_batch<N, MODE>())
                return launch_tiny<N, MODE>(a, perm, info, batch, tpb, grid, stream);
        }
        if constexpr (MODE == kModePartial && N >= kRowsMin && rows_partial_enabled<N>())
            return launch_rows_partial<N>(a, perm, info, batch, grid, stream);
        else
            return launch_lanes_tuned<N, MODE>(a, perm, info, batch, tpb, grid, stream);
    }
}

// What launch<N, MODE> runs for a contiguous batch: the kernel form (the
// MI_FORM_* codes of mi_inverse.h), lanes per matrix, matrices per warp and
// threads per block.  The branches are launch<N, MODE>'s, in its order; only
// the lane-group form launches with the resolved threads-per-block knob
// `tpb`, the other two have a fixed block.
enum : int { kFormThread = 1, kFormLanes = 2, kFormRows = 3 };

struct LaunchForm {
    int form, lanes, mpw, threads;
};

template <int N, int MODE>
LaunchForm launch_form(long long batch, int tpb) {
    if constexpr (N <= kTinyMax) {
        return {kFormThread, 1, 32, tiny_threads<N>()};
    } else if constexpr (N <= tiny_max_contig<MODE>()) {
        if (batch >= tiny_min_batch<N, MODE>()) return {kFormThread, 1, 32, tiny_threads<N>()};
    }
    if constexpr (MODE == kModePartial && N >= kRowsMin && rows_partial_enabled<N>())
        return {kFormRows, RowsGeom<N>::kLanes, RowsGeom<N>::kMats, 32 * kRowsWarps};
    if constexpr (N == WideGeom::N && MODE != kModePartial)
        return {kFormLanes, WideGeom::L, WideGeom::M, tpb < WideGeom::kThreadsMax ? tpb : WideGeom::kThreadsMax};
    constexpr int L = default_lanes(N, MODE), alt = alt_lanes(N, MODE);
    if constexpr (alt != 0)
        if (batch >= MI_LANES_ALT_MIN_BATCH && tuned_lanes(N, MODE) == alt)
            return {kFormLanes, alt, Geom<N, alt>::M, tpb};
    return {kFormLanes, L, Geom<N, L>::M, tpb};
}

// Indexed bucket launch: the kernel reads its bucket's [start, count) from
// `range` on the device, so the grid is fixed (persistent warps) and the
// launch needs no host round trip -- it can be captured in a CUDA graph.
using ilaunch_fn = cudaError_t (*)(float*, const long long*, const int*, const long long*, int32_t*, int32_t*, int,
                                   int, cudaStream_t);

// The lane-group kernel of a descriptor bucket at L lanes per matrix.
template <int N, int MODE, int L>
cudaError_t launch_indexed_lanes(float* base, const long long* offsets, const int* list, const long long* range,
                                 int32_t* perm, int32_t* info, int tpb, int grid, cudaStream_t stream) {
    const int warps = tpb / 32;
    const size_t smem = smem_bytes<N, L, MODE>(warps);
    auto kern = mi_inverse_indexed_kernel<N, L, MODE>;
    static size_t smem_set[kMaxDevices] = {};
    {
        const cudaError_t e = opt_in_smem(kern, smem, smem_set);
        if (e != cudaSuccess) return e;
    }
    if (grid <= 0) {
        static int per_sm_cached[9] = {0};
        int& per_sm = per_sm_cached[warps];
        if (per_sm == 0) {
            cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, tpb, smem);
            if (e != cudaSuccess) return e;
            if (per_sm < 1) per_sm = 1;
        }
        grid = per_sm * device_sm_count();
    }
    kern<<<grid, tpb, smem, stream>>>(base, offsets, list, range, perm, info);
    return cudaGetLastError();
}

template <int N, int MODE>
cudaError_t launch_indexed(float* base, const long long* offsets, const int* list, const long long* range,
                           int32_t* perm, int32_t* info, int tpb, int grid, cudaStream_t stream) {
    if constexpr (N <= tiny_max_indexed<MODE>())
        return launch_tiny_indexed<N, MODE>(base, offsets, list, range, perm, info, tpb, grid, stream);
    if constexpr (N == WideGeom::N && MODE != kModePartial)
        return launch_wide_gather<MODE, true>(base, offsets, list, range, 0, perm, info, tpb, grid, stream);
    // the default width: a bucket's size is known only on the device, and
    // buckets are typically below MI_LANES_ALT_MIN_BATCH (either width gives
    // the same bits)
    return launch_indexed_lanes<N, MODE, default_lanes(N, MODE)>(base, offsets, list, range, perm, info, tpb, grid,
                                                                 stream);
}

extern const ilaunch_fn kITableNone[33];
extern const ilaunch_fn kITableReference[33];
extern const ilaunch_fn kITableReferenceSerial[33];
extern const ilaunch_fn kITablePartial[33];

extern const launch_fn kTableNone[33];
extern const launch_fn kTableReference[33];
extern const launch_fn kTableReferenceSerial[33];
extern const launch_fn kTablePartial[33];

}  // namespace mi

#define MI_TABLE(NAME, MODE)                                                                          \
    const launch_fn NAME[33] = {                                                                      \
        nullptr,          launch<1, MODE>,  launch<2, MODE>,  launch<3, MODE>,  launch<4, MODE>,  \
        launch<5, MODE>,  launch<6, MODE>,  launch<7, MODE>,  launch<8, MODE>,  launch<9, MODE>,  \
        launch<10, MODE>, launch<11, MODE>, launch<12, MODE>, launch<13, MODE>, launch<14, MODE>, \
        launch<15, MODE>, launch<16, MODE>, launch<17, MODE>, launch<18, MODE>, launch<19, MODE>, \
        launch<20, MODE>, launch<21, MODE>, launch<22, MODE>, launch<23, MODE>, launch<24, MODE>, \
        launch<25, MODE>, launch<26, MODE>, launch<27, MODE>, launch<28, MODE>, launch<29, MODE>, \
        launch<30, MODE>, launch<31, MODE>, launch<32, MODE>}

#define MI_ITABLE(NAME, MODE)                                                                                 \
    const ilaunch_fn NAME[33] = {                                                                             \
        nullptr,                  launch_indexed<1, MODE>,  launch_indexed<2, MODE>,  launch_indexed<3, MODE>,  \
        launch_indexed<4, MODE>,  launch_indexed<5, MODE>,  launch_indexed<6, MODE>,  launch_indexed<7, MODE>,  \
        launch_indexed<8, MODE>,  launch_indexed<9, MODE>,  launch_indexed<10, MODE>, launch_indexed<11, MODE>, \
        launch_indexed<12, MODE>, launch_indexed<13, MODE>, launch_indexed<14, MODE>, launch_indexed<15, MODE>, \
        launch_indexed<16, MODE>, launch_indexed<17, MODE>, launch_indexed<18, MODE>, launch_indexed<19, MODE>, \
        launch_indexed<20, MODE>, launch_indexed<21, MODE>, launch_indexed<22, MODE>, launch_indexed<23, MODE>, \
        launch_indexed<24, MODE>, launch_indexed<25, MODE>, launch_indexed<26, MODE>, launch_indexed<27, MODE>, \
        launch_indexed<28, MODE>, launch_indexed<29, MODE>, launch_indexed<30, MODE>, launch_indexed<31, MODE>, \
        launch_indexed<32, MODE>}
