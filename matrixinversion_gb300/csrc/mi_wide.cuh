// mi_wide.cuh -- n = 32 without partial pivoting (modes none, reference,
// reference_serial): eight lanes per matrix, 16 x 8 register blocks.
//
// The inverse of a 32 x 32 matrix is 32 rank-1 updates of the whole matrix
// (product-form Gauss-Jordan, the same step as mi_kernel.cuh's gj_step).
// Every step each lane needs column k for its rows and row k for its columns
// from the lanes that hold them: R + C values by warp shuffle for the R x C
// FMAs of its block.  Shuffles and shared-memory accesses share one data path
// that moves one 128-byte wavefront per clock per SM, and at n = 32 that path,
// not HBM, sets the pace.  Eight lanes per matrix with 16 x 8 blocks need
// 24 broadcast values per 128 FMAs (16 lanes with 8 x 8 blocks: 16 per 64),
// so a warp of four matrices moves 25 shuffles per step where two 16-lane
// groups moved 34.  The block takes 128 registers, so an SM holds 8 warps
// (32 matrices), as many as the 16-lane form held.
//
//   * Lane s = 2 cg + rg of a group holds rows 2 ri + rg (ri = 0..15, cyclic)
//     and columns 8 cg .. 8 cg + 7.  Rows are loaded in pivot order (the
//     reference rules' pivot sequence is replayed first, as in mi_kernel.cuh),
//     so the elimination itself has no pivoting.  All 32 steps are unrolled:
//     every register index is a constant.
//   * Deferred column scaling.  Step k leaves column k as it is (c_i for every
//     row i != k) instead of overwriting it with the multipliers -c_i / d, and
//     stores -d in place of the pivot.  Later steps update that column like
//     any other (the update is linear in the column, so a column scaled by a
//     constant stays scaled by it), and at the end element (i, j) is scaled by
//     -(1/d_i)(1/d_j): the row scale of the unnormalised pivot row and the
//     column scale the step left out.  A step therefore writes no zeros into
//     column k; its only per-lane fix-ups are one multiplier (the pivot row
//     takes no update), one broadcast value (column k takes none) and the
//     pivot itself.
//   * Packed FMAs pair rows: (a[2q][j], a[2q+1][j]) += (c_2q, c_2q+1) (w_j,
//     w_j) with w = -a[k][j] / d, so the column values arrive as natural pairs
//     and only the eight row values are duplicated into pairs.
//   * Data movement as mi_inverse_kernel: one shared-memory slot per warp
//     (four matrices, TMA 3-D tensor load with the 128-byte swizzle), the next
//     group's load issued as soon as the block is in registers, and results
//     leaving in four rounds of 8 rows through two alternating buffers by TMA
//     tensor stores.  Cyclic rows put the two lanes that store one column in
//     one instruction on rows of different swizzle phase, so they never share
//     a bank.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "mi_kernel.cuh"

namespace mi {

struct WideGeom {
    static constexpr int N = 32, L = 8, M = 4, R = 16, C = 8;
    static constexpr int kMat = N * N;
    static constexpr int kSlot = M * kMat;              // input slot: 4 matrices, 16 KB
    static constexpr int ORows = 8;                     // matrix rows per output round
    static constexpr int Rounds = N / ORows;
    static constexpr int kOutT = M * ORows * N;         // one output buffer: 4 KB
    // per matrix: 32 pivots, 32 pivot rows, 8 floats of skew so that the four
    // matrices' entries of one step fall in different banks
    static constexpr int kScr = 72;
    static constexpr int oD = 0, oWin = 32;
    static constexpr int oOut = kSlot;
    static constexpr int oScr = oOut + 2 * kOutT;
    static constexpr int oBar = oScr + M * kScr;
    static constexpr int kWarp = (oBar + 4 + 255) / 256 * 256;   // floats per warp, 1 KB multiple
    static constexpr int kThreadsMax = 256;
    // matrix row held in register row ri by row group rg
    __host__ __device__ static constexpr int row(int ri, int rg) { return 2 * ri + rg; }
    static_assert(Rounds % 2 == 0, "output buffers alternate by round parity within a group");
    static_assert(kSlot % 256 == 0 && oOut % 256 == 0 && kOutT % 256 == 0,
                  "128-byte-swizzled tensor-copy buffers need 1 KB alignment");
    static_assert(kScr % 4 == 0 && kScr % 32 != 0, "16-byte aligned, bank-skewed per-matrix scratch");
};

constexpr size_t wide_smem_bytes(int warps) { return 1024 + (size_t)warps * WideGeom::kWarp * sizeof(float); }

// -1/d: the reciprocal of recip() with the sign folded into its last FMA.
__device__ __forceinline__ float neg_recip(float d) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(d));
    const float e = fmaf(-d, r, 1.0f);
    return fmaf(-r, e, -r);
}

__device__ __forceinline__ void sts_u32addr(uint32_t addr, float v) {
    asm volatile("st.shared.f32 [%0], %1;" ::"r"(addr), "f"(v) : "memory");
}

// Register block of one matrix from the warp's slot (128-byte swizzle), row
// i = 2 ri + rg taken from input row src(i): the pivot order (reference rules)
// or i itself (no pivoting).
template <int MODE>
__device__ __forceinline__ void wide_load(float (&a)[16][8], const float* st, const int* win, int rg, int cg) {
#pragma unroll
    for (int ri = 0; ri < 16; ri++) {
        const int i = WideGeom::row(ri, rg);
        const int src = (MODE == kModeNone) ? i : win[i];
        const float* row = st + src * 32;
        const int x = src & 7;
        const float4 v0 = *reinterpret_cast<const float4*>(row + (((2 * cg) ^ x) << 2));
        const float4 v1 = *reinterpret_cast<const float4*>(row + (((2 * cg + 1) ^ x) << 2));
        a[ri][0] = v0.x; a[ri][1] = v0.y; a[ri][2] = v0.z; a[ri][3] = v0.w;
        a[ri][4] = v1.x; a[ri][5] = v1.y; a[ri][6] = v1.z; a[ri][7] = v1.w;
    }
}

// The 32 elimination steps and the final scaling.  Lane s of the group whose
// first lane is gb; the pivot of every step goes to scr[oD + k].
__device__ __forceinline__ void wide_eliminate(float (&a)[16][8], float* scr, int s, int gb) {
    using G = WideGeom;
    const int rg = s & 1, cg = s >> 1;
#pragma unroll
    for (int k = 0; k < 32; ++k) {
        const int kr = k & 1, kri = k >> 1;      // pivot row: owner row group, register row
        const int kc = k >> 3, kci = k & 7;      // pivot column: owner column group, register column
        float c[16], w[8];
        // column k for my rows from lane (rg, kc), row k for my columns from
        // lane (kr, cg), -1/pivot from lane (kr, kc); row k is then scaled,
        // w = -a[k][j] / pivot
#pragma unroll
        for (int ri = 0; ri < 16; ri++) c[ri] = __shfl_sync(kFull, a[ri][kci], gb + 2 * kc + rg);
#pragma unroll
        for (int ci = 0; ci < 8; ci++) w[ci] = __shfl_sync(kFull, a[kri][ci], gb + 2 * cg + kr);
        const float pn = __shfl_sync(kFull, neg_recip(a[kri][kci]), gb + 2 * kc + kr);
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const float2 t = __fmul2_rn(make_float2(w[2 * q], w[2 * q + 1]), make_float2(pn, pn));
            w[2 * q] = t.x;
            w[2 * q + 1] = t.y;
        }
        if (s == 2 * kc + kr) {
            scr[G::oD + k] = a[kri][kci];
            a[kri][kci] = -a[kri][kci];          // the pivot's place holds -pivot (deferred column scale)
        }
        if (rg == kr) c[kri] = 0.0f;             // the pivot row takes no update
        if (cg == kc) w[kci] = 0.0f;             // column k takes no update
#pragma unroll
        for (int ci = 0; ci < 8; ci++) {
            const float2 wd = make_float2(w[ci], w[ci]);
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const float2 x = __ffma2_rn(make_float2(c[2 * q], c[2 * q + 1]), wd,
                                            make_float2(a[2 * q][ci], a[2 * q + 1][ci]));
                a[2 * q][ci] = x.x;
                a[2 * q + 1][ci] = x.y;
            }
        }
    }
    __syncwarp();
    // element (i, j) *= -(1/d_i)(1/d_j), both scales formed from the recorded
    // pivots (carrying the row scales through the steps would hold 16 more
    // registers there)
    float ps[16], cs[8];
#pragma unroll
    for (int ri = 0; ri < 16; ri++) ps[ri] = -recip(scr[G::oD + G::row(ri, rg)]);
    {
        const float4 d0 = *reinterpret_cast<const float4*>(scr + G::oD + 8 * cg);
        const float4 d1 = *reinterpret_cast<const float4*>(scr + G::oD + 8 * cg + 4);
        cs[0] = recip(d0.x); cs[1] = recip(d0.y); cs[2] = recip(d0.z); cs[3] = recip(d0.w);
        cs[4] = recip(d1.x); cs[5] = recip(d1.y); cs[6] = recip(d1.z); cs[7] = recip(d1.w);
    }
#pragma unroll
    for (int ci = 0; ci < 8; ci++) {
        const float2 cd = make_float2(cs[ci], cs[ci]);
#pragma unroll
        for (int q = 0; q < 8; q++) {
            float2 x = __fmul2_rn(make_float2(a[2 * q][ci], a[2 * q + 1][ci]), make_float2(ps[2 * q], ps[2 * q + 1]));
            x = __fmul2_rn(x, cd);
            a[2 * q][ci] = x.x;
            a[2 * q + 1][ci] = x.y;
        }
    }
}

// Pivots and info of the group's matrix at output index idx (negative: no
// matrix): lane s writes perm entries s, s + 8, s + 16, s + 24 from win; info
// = the first step whose pivot is exactly zero (1-based), else 0.
__device__ __forceinline__ void wide_perm_info(const float* scr, int s, int gb, long long idx, int32_t* perm_out,
                                               int32_t* info_out, const int* win) {
    using G = WideGeom;
    unsigned zmask = 0u;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int t = s + 8 * q;
        zmask |= ((__ballot_sync(kFull, scr[G::oD + t] == 0.0f) >> gb) & 0xffu) << (8 * q);
        if (perm_out != nullptr && idx >= 0) perm_out[idx * 32 + t] = win[t];
    }
    if (info_out != nullptr && s == 0 && idx >= 0) info_out[idx] = zmask ? __ffs(zmask) : 0;
    __syncwarp();
}

// Shared address of every (register row within a round, register column) of
// this lane in an output buffer: buffer row lr = 2h + rg (matrix row 8q + lr
// of round q), column win[8cg + ci] (A^-1[i][win[j]] = X[i][j]) under the
// 128-byte swizzle (column ^ 4 (lr & 7)).
template <int MODE>
__device__ __forceinline__ void wide_out_addrs(uint32_t (&addr)[4][8], const float* outb, const int* win, int ms,
                                               int rg, int cg) {
    const uint32_t base = smem_addr(outb) + (uint32_t)(ms * WideGeom::ORows * 32) * 4u;
#pragma unroll
    for (int ci = 0; ci < 8; ci++) {
        const int dc = (MODE == kModeNone) ? 8 * cg + ci : win[8 * cg + ci];
#pragma unroll
        for (int h = 0; h < 4; h++) {
            const int lr = 2 * h + rg;
            addr[h][ci] = base + (uint32_t)(lr * 32 + (dc ^ (lr << 2))) * 4u;
        }
    }
}

// Matrix rows 8q .. 8q + 7 (register rows 4q .. 4q + 3) into the buffer at
// byte offset boff from the addresses of wide_out_addrs.
__device__ __forceinline__ void wide_write_round(const float (&a)[16][8], const uint32_t (&addr)[4][8], int q,
                                                 uint32_t boff) {
#pragma unroll
    for (int h = 0; h < 4; h++)
#pragma unroll
        for (int ci = 0; ci < 8; ci++) sts_u32addr(addr[h][ci] + boff, a[4 * q + h][ci]);
}

// Results leave in four rounds of 8 rows, each round one TMA tensor store of
// the four matrices from one of two alternating buffers.
template <int MODE>
__device__ __forceinline__ void wide_store(const float (&a)[16][8], float* outb, const int* win, int ms, int rg,
                                           int cg, int lane, const CUtensorMap* tmap_out, long long first) {
    using G = WideGeom;
    uint32_t addr[4][8];
    wide_out_addrs<MODE>(addr, outb, win, ms, rg, cg);
#pragma unroll
    for (int q = 0; q < G::Rounds; q++) {
        if (lane == 0) bulk_wait_read_one();     // this buffer's store from two rounds ago has read it
        __syncwarp();
        wide_write_round(a, addr, q, (uint32_t)((q & 1) * G::kOutT) * 4u);
        fence_proxy_async();
        __syncwarp();
        if (lane == 0) {
            tma_store_3d(tmap_out, 0, q * G::ORows, (int)first, outb + (q & 1) * G::kOutT);
            bulk_commit();
        }
    }
}

// Pivot order of the four matrices in the slot: the reference rules replayed
// (lane = input row of each matrix), or the identity without pivoting.
template <int MODE>
__device__ __forceinline__ void wide_pivot_order(const float* slot, float* scr0, int scr_pitch, int win_off,
                                                 int lane) {
    using G = WideGeom;
    if constexpr (MODE == kModeReference || MODE == kModeReferenceSerial) {
        const float* stm[G::M];
        int* winm[G::M];
#pragma unroll
        for (int q = 0; q < G::M; q++) {
            stm[q] = slot + q * G::kMat;
            winm[q] = reinterpret_cast<int*>(scr0 + q * scr_pitch + win_off);
        }
        replay_fast_multi<32, 32, G::M, MODE, true>(stm, winm, lane, 0);
    } else {
        const int ms = lane >> 3;
        for (int t = lane & 7; t < 32; t += 8) reinterpret_cast<int*>(scr0 + ms * scr_pitch + win_off)[t] = t;
    }
}

// The per-group work shared by both kernels once the group is in the slot:
// pivot order, register block, and -- after `next()` has issued the copy of
// the warp's next group into the slot -- elimination.
template <int MODE, class Next>
__device__ __forceinline__ void wide_compute(float (&a)[16][8], const float* slot, float* scr0, int lane,
                                             Next&& next) {
    using G = WideGeom;
    const int ms = lane >> 3, s = lane & 7, gb = lane & ~7;
    const int rg = s & 1, cg = s >> 1;
    float* scr = scr0 + ms * G::kScr;
    wide_pivot_order<MODE>(slot, scr0, G::kScr, G::oWin, lane);
    __syncwarp();
    wide_load<MODE>(a, slot + ms * G::kMat, reinterpret_cast<const int*>(scr + G::oWin), rg, cg);
    __syncwarp();
    next();
    wide_eliminate(a, scr, s, gb);
}

// Contiguous batch, n = 32: persistent warps walk groups of four matrices.
template <int MODE>
__global__ void __launch_bounds__(WideGeom::kThreadsMax, 1)
    mi_wide_kernel(float* __restrict__ A, int32_t* __restrict__ perm_out, int32_t* __restrict__ info_out,
                   long long batch, const __grid_constant__ CUtensorMap tmap,
                   const __grid_constant__ CUtensorMap tmap_out) {
    using G = WideGeom;
    static_assert(MODE != kModePartial, "partial pivoting has its own kernels");
    extern __shared__ unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int W = blockDim.x >> 5;
    const uintptr_t base = (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023);
    float* slot = reinterpret_cast<float*>(base) + (size_t)warp * G::kWarp;
    float* outb = slot + G::oOut;
    float* scr0 = slot + G::oScr;
    uint64_t* bar = reinterpret_cast<uint64_t*>(slot + G::oBar);
    const int ms = lane >> 3, s = lane & 7;
    const int rg = s & 1, cg = s >> 1;
    const int* win = reinterpret_cast<const int*>(scr0 + ms * G::kScr + G::oWin);

    if (lane == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
        tma_prefetch_map(&tmap);
        tma_prefetch_map(&tmap_out);
    }
    __syncwarp();

    const long long groups = (batch + G::M - 1) / G::M;
    const long long gstride = (long long)gridDim.x * W;
    auto issue = [&](long long g) {
        if (lane == 0) {
            mbar_arrive_expect_tx(bar, (uint32_t)(G::kSlot * 4));
            if (g_wait_arm_only == 0) tma_load_3d(slot, &tmap, 0, 0, (int)(g * G::M), bar);
        }
    };

    long long g = (long long)blockIdx.x * W + warp;
    uint32_t phase = 0;
    bool timed_out = false;
    if (g < groups) issue(g);
    while (g < groups) {
        const long long first = g * G::M;
        // lanes time their waits separately, so the warp decides together
        if (!__all_sync(kFull, mbar_wait_copy(bar, phase & 1u))) {
            timed_out = true;
            break;
        }
        phase++;
        __syncwarp();

        float a[16][8];
        const long long gn = g + gstride;
        wide_compute<MODE>(a, slot, scr0, lane, [&] {
            // the slot is free: bring in this warp's next group now
            if (gn < groups) {
                if (lane == 0) fence_proxy_async();
                issue(gn);
            }
        });
        wide_store<MODE>(a, outb, win, ms, rg, cg, lane, &tmap_out, first);
        const long long mb = first + ms;
        wide_perm_info(scr0 + ms * G::kScr, s, lane & ~7, mb < batch ? mb : -1, perm_out, info_out, win);
        g = gn;
    }
    if (timed_out) {
        atomicOr(&g_device_error, 1);
        // the copy may still land in this warp's slot: wait for it once more,
        // bounded, before the warp leaves
        mbar_wait_copy(bar, phase & 1u);
    }
    if (lane == 0) bulk_wait_all();
}

__device__ __forceinline__ void cp_async_16_cg(float* dst, const float* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}

// Batches the tensor copies cannot take -- descriptor buckets (IDX: the
// bucket's matrices are list[start ..] of the descriptor table, matrix idx at
// base + offsets[idx]) and contiguous batches whose pointer is not 16-byte
// aligned (matrix b at base + 1024 b) -- with the same arithmetic as
// mi_wide_kernel, so every matrix gets the same bits either way.  Each
// matrix moves into the slot's swizzled layout by asynchronous copies (16
// bytes when its address allows, else 4) and its rows leave from one output
// buffer by plain stores (16 bytes when aligned).  Pivots go to
// perm_out[idx * 32 ..], info to info_out[idx].
//
// wide_gather_walk is one warp's walk over the groups g, g + gstride, ...
// (< g_end) of four matrices, in the warp's region `slot` (WideGeom::kWarp
// floats, 1 KB aligned); mi_wide_gather_kernel runs it on persistent warps.
template <int MODE, bool IDX>
__device__ __forceinline__ void wide_gather_walk(float* slot, int lane, float* __restrict__ base,
                                                 const long long* __restrict__ offsets, const int* __restrict__ list,
                                                 long long start, long long count, long long g, long long g_end,
                                                 long long gstride, int32_t* __restrict__ perm_out,
                                                 int32_t* __restrict__ info_out) {
    using G = WideGeom;
    static_assert(MODE != kModePartial, "partial pivoting has its own kernels");
    float* outb = slot + G::oOut;
    float* scr0 = slot + G::oScr;
    const int ms = lane >> 3, s = lane & 7;
    const int rg = s & 1, cg = s >> 1;
    const int* win = reinterpret_cast<const int*>(scr0 + ms * G::kScr + G::oWin);
    const long long groups = g_end;

    // descriptor index of matrix m of group g (-1 past the end) and its address
    auto index_of = [&](long long g, int m) -> long long {
        const long long p = g * G::M + m;
        return p < count ? (IDX ? (long long)list[start + p] : p) : -1;
    };
    auto matrix = [&](long long idx) -> float* { return base + (IDX ? offsets[idx] : idx * G::kMat); };
    auto issue = [&](long long g) {
#pragma unroll
        for (int m = 0; m < G::M; m++) {
            const long long idx = index_of(g, m);
            const float* src = idx >= 0 ? matrix(idx) : base;
            float* dst = slot + m * G::kMat;
            if (idx >= 0 && (reinterpret_cast<uintptr_t>(src) & 15u) == 0) {
                // 16-byte chunk c of row r lands at chunk c ^ (r & 7)
                for (int t = lane; t < 256; t += 32) {
                    const int r = t >> 3, c = t & 7;
                    cp_async_16_cg(dst + r * 32 + ((c ^ (r & 7)) << 2), src + 4 * t);
                }
            } else {
                // element by element (zero-filled past the end of the batch)
                for (int e = lane; e < G::kMat; e += 32)
                    cp_async_4(dst + stage_off<32>(e >> 5, e & 31), idx >= 0 ? src + e : base, idx >= 0);
            }
        }
        cp_async_commit();
    };

    if (g < groups) issue(g);
    while (g < groups) {
        cp_async_wait_all();
        __syncwarp();
        long long idx[G::M];
#pragma unroll
        for (int m = 0; m < G::M; m++) idx[m] = index_of(g, m);
        float a[16][8];
        const long long gn = g + gstride;
        wide_compute<MODE>(a, slot, scr0, lane, [&] {
            if (gn < groups) issue(gn);
        });
        uint32_t addr[4][8];
        wide_out_addrs<MODE>(addr, outb, win, ms, rg, cg);
#pragma unroll
        for (int q = 0; q < G::Rounds; q++) {
            __syncwarp();                             // the previous round's rows have left the buffer
            wide_write_round(a, addr, q, 0u);
            __syncwarp();
#pragma unroll
            for (int m = 0; m < G::M; m++) {
                if (idx[m] < 0) continue;
                float* dst = matrix(idx[m]) + q * G::ORows * 32;
                const float* ob = outb + m * G::ORows * 32;
                if ((reinterpret_cast<uintptr_t>(dst) & 15u) == 0) {
                    for (int t = lane; t < 64; t += 32) {
                        const int r = t >> 3, c = t & 7;
                        *reinterpret_cast<float4*>(dst + 4 * t) =
                            *reinterpret_cast<const float4*>(ob + r * 32 + ((c ^ r) << 2));
                    }
                } else {
                    for (int e = lane; e < G::ORows * 32; e += 32) {
                        const int r = e >> 5, c = e & 31;
                        dst[e] = ob[r * 32 + (c ^ (r << 2))];
                    }
                }
            }
        }
        wide_perm_info(scr0 + ms * G::kScr, s, lane & ~7, index_of(g, ms), perm_out, info_out, win);
        g = gn;
    }
}

template <int MODE, bool IDX>
__global__ void __launch_bounds__(WideGeom::kThreadsMax, 1)
    mi_wide_gather_kernel(float* __restrict__ base, const long long* __restrict__ offsets,
                          const int* __restrict__ list, const long long* __restrict__ range, long long batch,
                          int32_t* __restrict__ perm_out, int32_t* __restrict__ info_out) {
    using G = WideGeom;
    extern __shared__ unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int W = blockDim.x >> 5;
    const uintptr_t sbase = (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023);
    float* slot = reinterpret_cast<float*>(sbase) + (size_t)warp * G::kWarp;
    const long long start = IDX ? range[0] : 0;
    const long long count = IDX ? range[1] : batch;
    if (count <= 0) return;
    wide_gather_walk<MODE, IDX>(slot, lane, base, offsets, list, start, count, (long long)blockIdx.x * W + warp,
                                (count + G::M - 1) / G::M, (long long)gridDim.x * W, perm_out, info_out);
}

}  // namespace mi
