// mi_rows.cuh -- partial pivoting for n = 16..32 with whole rows per lane.
//
// 16 lanes per matrix, two matrices per warp; lane s of a group owns the
// rows (slots) s and s + 16 in registers, every column of them.  A step of
// partial pivoting then needs no exchange of column values between lanes:
// each lane keys column k of its own rows, one 16-lane maximum over a packed
// (key, logical row, slot) word picks getrf's pivot (largest |x|, ties to the
// lowest logical row), the winning lane stores its row to a small
// shared-memory buffer and every lane reads it back as broadcast 16-byte
// loads.  Rows stay in their slots (no exchanges); as in gj_step_partial each
// slot carries its logical position, the output row of a slot is the step
// that chose it, and the columns leave through the pivot permutation.  The
// arithmetic of every element (m = c * (1/pivot), a = fma(-m, w, a), column k
// zeroed first with w[k] = 1, rows scaled by 1/pivot at the end) is that of
// gj_step_partial, so the results are the same bits.
//
// The warp's two matrices move between HBM and a padded shared-memory stage
// (row pitch an odd number of 16-byte chunks: conflict-free row reads) with
// asynchronous copies, 16 bytes at a time when rows allow.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "mi_kernel.cuh"

namespace mi {

constexpr int kRowsWarps = 4;       // warps per block
constexpr int kRowsMin = 16;        // smallest n of this kernel (partial pivoting)

// Lanes per matrix at size n: 16 (two matrices per warp, two rows per lane)
// or 8 (four matrices per warp, up to four rows per lane).  Measured on GB300
// at 1,000,000 matrices, same bits, with each step's search inside the
// previous step: 8 lanes at n = 17 1.69 against 2.09 ms, 18 1.82 against
// 2.30, 19 2.02 against 2.70, 20 1.95 against 2.35, 21 2.75 against 3.20,
// 22 2.93 against 3.38, 23 3.27 against 3.67, 24 3.10 against 3.79; at
// n = 25 (four rows per lane) 4.47 against 4.24.  (Before that change 8
// lanes won only at n = 18; from n = 25 up four whole rows per lane spilled:
// n = 32 12.04 against 6.74 ms.)
template <int N>
__host__ __device__ constexpr int rows_lanes() { return (N >= 17 && N <= 24) ? 8 : 16; }

template <int N, int LN = rows_lanes<N>()>
struct RowsGeom {
    static_assert(N >= 1 && N <= 32, "n must be in 1..32");
    static_assert(LN == 8 || LN == 16, "8 or 16 lanes per matrix");
    static constexpr int kLanes = LN;                               // lanes per matrix
    static constexpr int kMats = 32 / LN;                           // matrices per warp
    static constexpr int R = (N + LN - 1) / LN;                     // rows per lane
    static constexpr int NC = (N + 3) & ~3;                         // register columns
    static constexpr int SP = (((N + 3) / 4) | 1) * 4;              // stage row pitch (floats)
    static constexpr int kMat = N * SP;                             // stage floats per matrix
    // per-matrix scratch (floats): two pivot-row buffers, pivots, pivot slots,
    // output row of each slot
    static constexpr int oRow = 0;
    static constexpr int oD = oRow + 2 * NC;
    static constexpr int oWin = oD + 32;
    static constexpr int oMap = oWin + 32;
    static constexpr int kScr = oMap + 32;
    static constexpr int oScr = kMats * kMat;                       // scratch after the stage
    static constexpr int kWarp = (oScr + kMats * kScr + 31) & ~31;  // floats per warp (128-byte multiple)
    static_assert(kMat % 4 == 0 && kScr % 4 == 0 && NC % 4 == 0, "16-byte alignment of rows and buffers");
};

__device__ __forceinline__ void cp_async_16(float* dst, const float* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}

// Partial-pivoting key of one entry: |x| bits + 2 (a NaN never beats a
// number: key 1), as gj_step_partial.
__device__ __forceinline__ unsigned rows_key(float x) {
    const unsigned b = __float_as_uint(x) & 0x7fffffffu;
    return (b > 0x7f800000u) ? 1u : b + 2u;
}

// Maximum over the LN lanes of this lane's group (xor offsets < LN stay in
// the group).  Measured: one redux.sync per group mask instead (both groups
// of a warp in one instruction) is 6-10% slower here at 16 lanes.
template <int LN>
__device__ __forceinline__ unsigned rows_group_max(unsigned v) {
#pragma unroll
    for (int o = LN / 2; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(kFull, v, o));
    return v;
}

// The same over 64-bit words: two shuffles per level, one dependent chain.
template <int LN>
__device__ __forceinline__ unsigned long long rows_group_max64(unsigned long long v) {
#pragma unroll
    for (int o = LN / 2; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(kFull, v, o);
        v = w > v ? w : v;
    }
    return v;
}

template <int N, int LN = rows_lanes<N>()>
__global__ void __launch_bounds__(32 * kRowsWarps, LN == 16 ? 3 : 2) mi_rows_partial_kernel(
    float* __restrict__ A, int32_t* __restrict__ perm_out, int32_t* __restrict__ info_out, long long batch, int vec) {
    using G = RowsGeom<N, LN>;
    constexpr int R = G::R, NC = G::NC, SP = G::SP, NN = N * N;
    constexpr int kRowsLanes = G::kLanes, kRowsMats = G::kMats;
    constexpr unsigned kGroupMask = (1u << kRowsLanes) - 1u;
    extern __shared__ float4 rows_smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float* ws = reinterpret_cast<float*>(rows_smem) + warp * G::kWarp;
    const int mslot = lane / kRowsLanes, s = lane % kRowsLanes, gbase = mslot * kRowsLanes;
    float* st = ws + mslot * G::kMat;                    // this lane's matrix in the stage
    float* scr = ws + G::oScr + mslot * G::kScr;
    int* win = reinterpret_cast<int*>(scr + G::oWin);
    int* omap = reinterpret_cast<int*>(scr + G::oMap);
    const long long groups = (batch + kRowsMats - 1) / kRowsMats;
    const long long wstride = (long long)gridDim.x * kRowsWarps;
    for (long long grp = (long long)blockIdx.x * kRowsWarps + warp; grp < groups; grp += wstride) {
        const long long b0 = grp * kRowsMats;
        const int cnt = (batch - b0 < kRowsMats) ? (int)(batch - b0) : kRowsMats;
        float* g = A + b0 * NN;
        // ---- in: the group's cnt * n * n floats into the padded stage
        if (vec) {                                       // n % 4 == 0, 16-byte-aligned batch
            constexpr int Q4 = (N / 4 > 0) ? N / 4 : 1;  // chunks per row
            const int total = cnt * (NN / 4);
#pragma unroll 4
            for (int c = lane; c < total; c += 32) {
                const int m = c / (NN / 4), rem = c - m * (NN / 4);
                const int row = rem / Q4, c4 = rem - row * Q4;
                cp_async_16(ws + m * G::kMat + row * SP + 4 * c4, g + 4 * c);
            }
        } else {
            const int total = cnt * NN;
#pragma unroll 4
            for (int e = lane; e < total; e += 32) {
                const int m = e / NN, rem = e - m * NN;
                const int row = rem / N, col = rem - row * N;
                cp_async_4(ws + m * G::kMat + row * SP + col, g + e, true);
            }
        }
        cp_async_commit();
        cp_async_wait_all();
        __syncwarp();
        const bool valid = mslot < cnt;
        // ---- my rows to registers (padding rows and columns are zero)
        float a[R][NC];
#pragma unroll
        for (int ri = 0; ri < R; ri++) {
            const int slot = s + kRowsLanes * ri;
            const bool in = valid && slot < N;
#pragma unroll
            for (int q = 0; q < NC / 4; q++) {
                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                if (in) v = *reinterpret_cast<const float4*>(st + slot * SP + 4 * q);
                a[ri][4 * q] = v.x;
                a[ri][4 * q + 1] = v.y;
                a[ri][4 * q + 2] = v.z;
                a[ri][4 * q + 3] = v.w;
            }
#pragma unroll
            for (int j = N; j < NC; j++) a[ri][j] = 0.0f;
        }
        // ---- n steps of partial pivoting.  The search of step k + 1 runs
        // inside step k: as soon as the pivot row of step k is in the buffer,
        // column k + 1 takes its update (the same fma the full update would
        // give it), the keys of that column go into the two 16-lane maxima,
        // and only then does the rest of step k's update run -- so the
        // shuffle latency of the search overlaps the update's FMAs instead of
        // heading the next step.
        int lp[R];
        bool placed[R];
#pragma unroll
        for (int ri = 0; ri < R; ri++) {
            lp[ri] = s + kRowsLanes * ri;
            placed[ri] = (s + kRowsLanes * ri >= N);
        }
        // getrf's pivot of column kk over the rows not yet placed: the
        // largest key, then the lowest logical row.  Each candidate is one
        // word key << 16 | (255 - logical row) << 8 | slot (0 for none), so a
        // single maximum over the group picks it; the low 16 bits of the
        // result are (255 - logical row) << 8 | slot of the winner.  At
        // n = 30, 31 (168 registers, at the limit of three blocks per SM)
        // the 64-bit words measured 4-7% slower than two 32-bit maxima --
        // the largest key, then the best candidate among the lanes holding
        // it -- which pick the same winner.
        auto search = [&](int kk) -> unsigned long long {
            if constexpr (N == 30 || N == 31) {
                unsigned bk = 0u;
                int bl = 255, bs = 0;
#pragma unroll
                for (int ri = 0; ri < R; ri++) {
                    const unsigned key = placed[ri] ? 0u : rows_key(a[ri][kk]);
                    if (key > bk || (key == bk && key != 0u && lp[ri] < bl)) {
                        bk = key;
                        bl = lp[ri];
                        bs = s + kRowsLanes * ri;
                    }
                }
                const unsigned mx = rows_group_max<kRowsLanes>(bk);
                const unsigned cand = (bk != 0u && bk == mx) ? (((unsigned)(255 - bl) << 8) | (unsigned)bs) : 0u;
                return rows_group_max<kRowsLanes>(cand);
            } else {
                unsigned long long bp = 0ull;
#pragma unroll
                for (int ri = 0; ri < R; ri++) {
                    const unsigned key = placed[ri] ? 0u : rows_key(a[ri][kk]);
                    const unsigned long long cand =
                        key == 0u ? 0ull
                                  : ((unsigned long long)key << 16) |
                                        (unsigned long long)(((255 - lp[ri]) << 8) | (s + kRowsLanes * ri));
                    bp = cand > bp ? cand : bp;
                }
                return rows_group_max64<kRowsLanes>(bp);
            }
        };
        unsigned long long best = search(0);
#pragma unroll
        for (int k = 0; k < N; k++) {
            const int r = (int)(best & 0xffull);             // pivot slot
            const int lw = 255 - (int)((best >> 8) & 0xffull);   // its logical row
#pragma unroll
            for (int ri = 0; ri < R; ri++) {
                if (s + kRowsLanes * ri == r) {
                    lp[ri] = k;
                    placed[ri] = true;
                } else if (lp[ri] == k) {
                    lp[ri] = lw;                             // the row at logical k takes the winner's place
                }
            }
            // the pivot row, from its owner through a double-buffered row buffer
            float* rb = scr + G::oRow + (k & 1) * NC;
#pragma unroll
            for (int ri = 0; ri < R; ri++)
                if (s + kRowsLanes * ri == r) {
#pragma unroll
                    for (int q = 0; q < NC / 4; q++)
                        *reinterpret_cast<float4*>(rb + 4 * q) =
                            make_float4(a[ri][4 * q], a[ri][4 * q + 1], a[ri][4 * q + 2], a[ri][4 * q + 3]);
                }
            __syncwarp();
            const float d = rb[k];
            const float p = recip(d);
            if (s == 0) {
                scr[G::oD + k] = d;
                win[k] = r;
            }
            float2 nm[R];
#pragma unroll
            for (int ri = 0; ri < R; ri++) {
                const bool piv = (s + kRowsLanes * ri == r);
                const float c = piv ? 0.0f : a[ri][k];       // the pivot row takes no update
                a[ri][k] = piv ? 1.0f : 0.0f;                // column k becomes -multiplier (w[k] = 1)
                const float m = c * p;
                nm[ri] = make_float2(-m, -m);
            }
            // column k + 1 first, then the search of step k + 1
            const int k1 = k + 1;
            if (k1 < N) {
                const float w1 = rb[k1];
#pragma unroll
                for (int ri = 0; ri < R; ri++) a[ri][k1] = fmaf(nm[ri].x, w1, a[ri][k1]);
                best = search(k1);
            }
            // the rest of the update: the pivot row streams through in 16-byte
            // chunks (4 values live); column k + 1 is done
#pragma unroll
            for (int q = 0; q < NC / 4; q++) {
                float4 v = *reinterpret_cast<const float4*>(rb + 4 * q);
                if (k == 4 * q) v.x = 1.0f;
                if (k == 4 * q + 1) v.y = 1.0f;
                if (k == 4 * q + 2) v.z = 1.0f;
                if (k == 4 * q + 3) v.w = 1.0f;
                const bool d0 = k1 < N && k1 == 4 * q, d1 = k1 < N && k1 == 4 * q + 1;
                const bool d2 = k1 < N && k1 == 4 * q + 2, d3 = k1 < N && k1 == 4 * q + 3;
#pragma unroll
                for (int ri = 0; ri < R; ri++) {
                    if (!d0 && !d1) {
                        float2 x0 = make_float2(a[ri][4 * q], a[ri][4 * q + 1]);
                        x0 = __ffma2_rn(nm[ri], make_float2(v.x, v.y), x0);
                        a[ri][4 * q] = x0.x;
                        a[ri][4 * q + 1] = x0.y;
                    } else if (d0) {
                        a[ri][4 * q + 1] = fmaf(nm[ri].y, v.y, a[ri][4 * q + 1]);
                    } else {
                        a[ri][4 * q] = fmaf(nm[ri].x, v.x, a[ri][4 * q]);
                    }
                    if (!d2 && !d3) {
                        float2 x1 = make_float2(a[ri][4 * q + 2], a[ri][4 * q + 3]);
                        x1 = __ffma2_rn(nm[ri], make_float2(v.z, v.w), x1);
                        a[ri][4 * q + 2] = x1.x;
                        a[ri][4 * q + 3] = x1.y;
                    } else if (d2) {
                        a[ri][4 * q + 3] = fmaf(nm[ri].y, v.w, a[ri][4 * q + 3]);
                    } else {
                        a[ri][4 * q + 2] = fmaf(nm[ri].x, v.z, a[ri][4 * q + 2]);
                    }
                }
            }
        }
        __syncwarp();
        // output row of each slot = the step that chose it; row scale = 1 / its pivot
#pragma unroll
        for (int ri = 0; ri < R; ri++) {
            const int t = s + kRowsLanes * ri;
            if (t < N) omap[win[t]] = t;
        }
        __syncwarp();
#pragma unroll
        for (int ri = 0; ri < R; ri++) {
            const int slot = s + kRowsLanes * ri;
            const float ps = (slot < N) ? recip(scr[G::oD + omap[slot]]) : 1.0f;
#pragma unroll
            for (int q = 0; q < NC / 2; q++) {
                const float2 x = __fmul2_rn(make_float2(a[ri][2 * q], a[ri][2 * q + 1]), make_float2(ps, ps));
                a[ri][2 * q] = x.x;
                a[ri][2 * q + 1] = x.y;
            }
        }
        // ---- rows to the stage in output order, columns through the pivot
        // permutation: A^-1[omap[slot]][win[j]] = X[slot][j]
        if (valid) {
#pragma unroll
            for (int ri = 0; ri < R; ri++) {
                const int slot = s + kRowsLanes * ri;
                if (slot < N) {
                    float* orow = st + omap[slot] * SP;
#pragma unroll
                    for (int j = 0; j < N; j++) orow[win[j]] = a[ri][j];
                }
            }
        }
        __syncwarp();
        // ---- out
        if (vec) {
            constexpr int Q4 = (N / 4 > 0) ? N / 4 : 1;
            const int total = cnt * (NN / 4);
#pragma unroll 4
            for (int c = lane; c < total; c += 32) {
                const int m = c / (NN / 4), rem = c - m * (NN / 4);
                const int row = rem / Q4, c4 = rem - row * Q4;
                *reinterpret_cast<float4*>(g + 4 * c) =
                    *reinterpret_cast<const float4*>(ws + m * G::kMat + row * SP + 4 * c4);
            }
        } else {
            const int total = cnt * NN;
#pragma unroll 4
            for (int e = lane; e < total; e += 32) {
                const int m = e / NN, rem = e - m * NN;
                const int row = rem / N, col = rem - row * N;
                g[e] = ws[m * G::kMat + row * SP + col];
            }
        }
        // ---- pivots and info (first exactly-zero pivot, 1-based)
        unsigned zmask = 0u;
#pragma unroll
        for (int ri = 0; ri < R; ri++) {
            const int t = s + kRowsLanes * ri;
            const bool z = valid && t < N && scr[G::oD + t] == 0.0f;
            zmask |= ((__ballot_sync(kFull, z) >> gbase) & kGroupMask) << (kRowsLanes * ri);
            if (valid && t < N && perm_out != nullptr) perm_out[(b0 + mslot) * N + t] = win[t];
        }
        if (valid && s == 0 && info_out != nullptr) info_out[b0 + mslot] = zmask ? __ffs(zmask) : 0;
        __syncwarp();
    }
}

// Launch over a contiguous batch: persistent warps, as many blocks as are
// resident.
template <int N>
cudaError_t launch_rows_partial(float* a, int32_t* perm, int32_t* info, long long batch, int grid,
                                cudaStream_t stream) {
    using G = RowsGeom<N>;
    constexpr int kRowsMats = G::kMats;
    constexpr int threads = 32 * kRowsWarps;
    constexpr size_t smem = (size_t)kRowsWarps * G::kWarp * sizeof(float);
    auto kern = mi_rows_partial_kernel<N>;
    static size_t smem_set[kMaxDevices] = {};
    {
        const cudaError_t e = opt_in_smem(kern, smem, smem_set);
        if (e != cudaSuccess) return e;
    }
    static int per_sm = 0;
    if (per_sm == 0) {
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
    }
    const long long groups = (batch + kRowsMats - 1) / kRowsMats;
    if (grid <= 0) {
        const long long need = (groups + kRowsWarps - 1) / kRowsWarps;
        const long long cap = (long long)per_sm * device_sm_count();
        grid = (int)(need < cap ? need : cap);
    }
    if (grid < 1) grid = 1;
    const int vec = (N % 4 == 0 && (reinterpret_cast<uintptr_t>(a) & 15u) == 0) ? 1 : 0;
    kern<<<grid, threads, smem, stream>>>(a, perm, info, batch, vec);
    return cudaGetLastError();
}

// Whether partial pivoting at size n uses this kernel (contiguous batches).
// Measured on GB300 at 1,000,000 matrices against the lane-block kernel
// (gj_step_partial, one matrix per warp above n = 16), same bits: n = 16
// 1.63 -> 1.20 ms, 17 3.68 -> 2.59, 20 4.20 -> 2.65, 24 4.99 -> 4.21, 28
// 6.33 -> 5.27, 32 6.99 -> 6.76.  At n = 29..31 it spilled registers until
// the search of each step moved into the previous one (154-158 registers
// since, no spills).
template <int N>
__host__ __device__ constexpr bool rows_partial_enabled() { return N >= kRowsMin; }

}  // namespace mi
