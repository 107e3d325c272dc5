// mi_persist.cuh -- the single persistent launch of a descriptor call (the
// form selected by mi_set_descr_chunk(c > 0); one launch per bucket is the
// default, measured faster).
//
// One kernel (mi_descr_persistent_kernel, mi_descr_persist.cu) inverts every
// bucket of a bucketed descriptor table: its warps take chunks of groups from
// one global counter, in an order that visits the buckets from n = 32 down
// to n = 1, and run each chunk through the walk of that bucket's (n, mode) --
// the same per-warp code the per-bucket kernels run, so every matrix gets
// the bits of the contiguous call.  The 128 walks are separate device
// functions in four units (one per pivot mode, mi_pwalk_*.cu) compiled as
// relocatable device code and linked with the kernel, so they compile in
// parallel; the kernel's register count is the largest walk's (the n = 32
// eight-lane form and the one-thread-per-matrix forms at n = 13, 14 use up to
// 255), so a block of 8 warps per SM runs them all, each warp in a region of
// kPersistRegion floats.
//
// Bodies per (n, mode):
//   n = 1, 2          one thread per matrix in registers (tiny_indexed_walk)
//   n = 3 .. 14       one thread per matrix in a shared-memory slot (tiny_slot_walk)
//   n = 15, 16        lane groups at the default width
//   n = 17 .. 31      lane groups, eight lanes per matrix (8 x 16 blocks, four
//                     matrices per warp; the same bits as sixteen) without
//                     partial pivoting, the default width with it
//   n = 32            the eight-lane 16 x 8 form (wide_gather_walk) without
//                     partial pivoting, lane groups with it
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "mi_launch.cuh"

namespace mi {

constexpr int kPersistWarps = 8;                     // one block of 256 threads per SM
constexpr int kPersistRegion = WideGeom::kWarp;      // floats per warp (26 KB, a 1 KB multiple)
static_assert(kPersistRegion % 256 == 0, "per-warp regions keep the 1 KB alignment of the swizzled forms");

constexpr size_t persist_smem_bytes() { return 1024 + (size_t)kPersistWarps * kPersistRegion * sizeof(float); }

// Lanes per matrix of the lane-group body of (n, mode).
__host__ __device__ constexpr int persist_lanes(int n, int mode) {
    return (mode != kModePartial && n >= 17 && n <= 31) ? 8 : default_lanes(n, mode);
}

// Matrices per group of the body of (n, mode): the unit a warp takes.
__host__ __device__ constexpr int persist_group(int n, int mode) {
    return n <= 14 ? 32 : ((n == 32 && mode != kModePartial) ? WideGeom::M : 32 / persist_lanes(n, mode));
}

// One warp's walk over groups [g0, g1) of a bucket (descriptor indices
// list[start .. start + count)).  Returns false when a copy wait ran out.
template <int N, int MODE>
__device__ __forceinline__ bool persist_body(float* __restrict__ base, const long long* __restrict__ offsets,
                                             const int* __restrict__ list, long long start, long long count,
                                             long long g0, long long g1, int32_t* __restrict__ perm_out,
                                             int32_t* __restrict__ info_out) {
    extern __shared__ unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if constexpr (N < kTinySlotMinIndexed) {
        tiny_indexed_walk<N, MODE>(lane, base, offsets, list, start, count, g0, g1, 1, perm_out, info_out);
        return true;
    } else if constexpr (N <= 14) {
        static_assert(tiny_slot_floats<N>() <= kPersistRegion, "slot stage must fit the region");
        const uintptr_t sb = (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023);
        float* st = reinterpret_cast<float*>(sb) + (size_t)warp * kPersistRegion;
        tiny_slot_walk<N, MODE>(st, lane, base, offsets, list, start, count, g0, g1, 1, perm_out, info_out);
        return true;
    } else if constexpr (N == WideGeom::N && MODE != kModePartial) {
        const uintptr_t sb = (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023);
        float* slot = reinterpret_cast<float*>(sb) + (size_t)warp * kPersistRegion;
        wide_gather_walk<MODE, true>(slot, lane, base, offsets, list, start, count, g0, g1, 1, perm_out, info_out);
        return true;
    } else {
        constexpr int L = persist_lanes(N, MODE);
        static_assert(KGeom<N, L, MODE>::kWarp <= kPersistRegion, "lane-group region must fit");
        static_assert(GeomN<N, L, MODE>::M == persist_group(N, MODE), "group size of the plan");
        return indexed_walk<N, L, MODE>(WarpSmem<N, L, MODE>(smem_raw, warp, kPersistRegion), lane, base, offsets,
                                        list, start, count, g0, g1, 1, perm_out, info_out);
    }
}

#define MI_PWALK_PARAMS                                                                                         \
    float *__restrict__ base, const long long *__restrict__ offsets, const int *__restrict__ list, long long start, \
        long long count, long long g0, long long g1, int32_t *__restrict__ perm_out, int32_t *__restrict__ info_out
#define MI_PWALK_ARGS base, offsets, list, start, count, g0, g1, perm_out, info_out

// Apply F(MODE, N) for N = 1..32.
#define MI_PWALK_EACH_N(F, M)                                                                                  \
    F(M, 1) F(M, 2) F(M, 3) F(M, 4) F(M, 5) F(M, 6) F(M, 7) F(M, 8) F(M, 9) F(M, 10) F(M, 11) F(M, 12) F(M, 13) \
        F(M, 14) F(M, 15) F(M, 16) F(M, 17) F(M, 18) F(M, 19) F(M, 20) F(M, 21) F(M, 22) F(M, 23) F(M, 24)     \
            F(M, 25) F(M, 26) F(M, 27) F(M, 28) F(M, 29) F(M, 30) F(M, 31) F(M, 32)

// Walk of bucket (n, mode), defined in mi_pwalk_<mode>.cu.
#define MI_PWALK_DECL(M, N) __device__ bool pwalk_##M##_##N(MI_PWALK_PARAMS);
#define MI_PWALK_DEF(M, N) \
    __device__ __noinline__ bool pwalk_##M##_##N(MI_PWALK_PARAMS) { return persist_body<N, M>(MI_PWALK_ARGS); }

MI_PWALK_EACH_N(MI_PWALK_DECL, 0)
MI_PWALK_EACH_N(MI_PWALK_DECL, 1)
MI_PWALK_EACH_N(MI_PWALK_DECL, 2)
MI_PWALK_EACH_N(MI_PWALK_DECL, 3)

}  // namespace mi
