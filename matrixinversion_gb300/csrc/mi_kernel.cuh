// mi_kernel.cuh -- batched in-place inverse of n x n FP32 matrices (n <= 32)
// for sm_103a.
//
// Method (the reference's: LU with optional row pivoting, then the inverse
// from the triangular factors and the row permutation), scheduled for warps
// instead of the reference's one-thread-per-column shared-memory sweep
// (parallel_pivot/luBatchedInplace.cuh:127-199):
//
//   * Data movement: a CTA of W warps works on tiles of W*M matrices.  Tiles
//     stream HBM -> shared memory through the TMA engine (a 3-D tensor copy
//     with the 128-byte swizzle for n = 32, a 1-D bulk copy otherwise), two
//     tiles in flight per CTA (the next tile loads while this one computes),
//     and results leave the same way, so the SMs issue no per-element loads
//     or stores.  Ragged tails and unaligned pointers use plain loads.
//   * One sub-warp of L lanes owns a matrix (a warp holds M = 32/L).  Lane
//     (rg, cg) keeps an R x C register block: rows rg, rg+RG, ... (cyclic),
//     columns cg*C .. cg*C+C-1.
//   * Step k applies the k-th LU elimination to the rows below the pivot and
//     the k-th triangular-inverse update to the rows above it, in product
//     (Gauss-Jordan) form, a[i][j] -= (a[i][k] / a[k][k]) a[k][j].  Below the
//     pivot this is exactly right-looking LU's Schur-complement update, so the
//     pivot values, info and the partial-pivoting argmax see the numbers getrf
//     sees; after n steps the block holds (PA)^-1, and A^-1 = (PA)^-1 P is
//     stored by permuting columns.  Every step is one full rank-1 update
//     (n^2 FMAs): n^3 FMAs in all, the 2n^3 flops of getrf + getri, with no
//     lanes idling on triangular shapes.
//   * The pivot row is kept unscaled (its diagonal entry set to 1) and every
//     row is scaled by its 1/pivot once at the end, so a step is: column k and
//     row k broadcast through shared memory, one reciprocal, R/2 packed
//     multiplies and R*C/2 packed FMAs (fma.rn.f32x2).
//   * Pivoting:
//       reference        -- the reference's parallel argmax (find_pivot_parallel,
//                           parallel_pivot/luBatchedInplace.cuh:12-44, with
//                           T = n slots).  It compares raw input entries only
//                           (columns k, rows >= k are never written before step
//                           k), so the whole pivot sequence is replayed before
//                           the elimination, lane = row, with warp max
//                           reductions; when the maximum is unique no position
//                           bookkeeping is needed, and ties or NaNs fall back to
//                           an exact replay of the tree (slot order, dropped
//                           slots of non-power-of-two n).  Rows are then loaded
//                           in pivot order.
//       reference_serial -- serial_pivot's sequential argmax
//                           (serial_pivot/luBatchedInplace.cuh:22-36).
//       partial          -- textbook partial pivoting on the updated column
//                           (getrf: first maximum, rows exchanged in place).
//       none             -- templated/luBatchedInplace.cuh:78-126's plain LU.
//   * Outputs: A^-1 in place, optional perm[b][i] (input row that ends at row
//     i, the reference's shared pivots[]) and info[b] (0, or the 1-based step
//     of the first exactly-zero pivot, as getrf's info).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "mi_ptx.cuh"

namespace mi {

enum : int { kModeNone = 0, kModeReference = 1, kModeReferenceSerial = 2, kModePartial = 3 };
enum : int { kCopyPlain = 0, kCopyBulk = 1, kCopyTensor = 2, kCopyWindow = 3 };

// Dynamic shared memory above the 48 KB default needs an opt-in per kernel,
// and the opt-in holds for one device only.  `done` has one zero-initialised
// entry per device and records the largest size opted in there; sizes only
// grow, so a launch never finds its kernel's limit lowered by another.
constexpr int kMaxDevices = 64;

template <typename Kernel>
inline cudaError_t opt_in_smem(Kernel kern, size_t smem, size_t* done) {
    if (smem <= 48 * 1024) return cudaSuccess;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) dev = -1;
    if (dev >= 0 && done[dev] >= smem) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess && dev >= 0) done[dev] = smem;
    return e;
}

constexpr unsigned kFull = 0xffffffffu;
// Longest wait for one tile copy (SM clocks, about 2 s) before the kernel
// gives up, records an error and returns.
constexpr long long kWaitLimit = 4000000000LL;

// Sticky device error word: bit 0 = a tile-copy wait timed out, bit 1 = a
// tensor-core wait timed out (the MI_DEVERR_* flags of mi_inverse.h).  Every
// translation unit that includes this header is a module of its own with its
// own copy, so each registers a host reader of its copy when the library
// loads; mi_device_error() reads them all.  (Internal linkage: units
// compiled as relocatable device code and linked together keep one copy
// each as well.)
static __device__ int g_device_error;

using device_error_reader = cudaError_t (*)(int* flags, bool clear);
bool register_device_error_reader(device_error_reader fn);   // mi_api.cu

namespace {
cudaError_t read_device_error(int* flags, bool clear) {
    int v = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_device_error, sizeof(int));
    if (e != cudaSuccess) return e;
    if (clear && v != 0) {
        const int zero = 0;
        e = cudaMemcpyToSymbol(g_device_error, &zero, sizeof(int));
        if (e != cudaSuccess) return e;
    }
    *flags |= v;
    return cudaSuccess;
}
[[maybe_unused]] const bool g_device_error_registered = register_device_error_reader(&read_device_error);
}  // namespace

// Test hook of the bounded tile-copy waits (per module, like the error word):
// the longest wait in SM clocks, and a switch under which a warp arms its copy
// barrier with the expected bytes but issues no copy -- the barrier then never
// completes, nothing is in flight, and the wait runs out after the limit.
// Read once per launch by mi_inverse_kernel and mi_wide_kernel; set through
// mi_set_wait_test.
static __device__ long long g_wait_limit = kWaitLimit;
static __device__ int g_wait_arm_only = 0;

using wait_test_setter = cudaError_t (*)(long long limit, int arm_only);
bool register_wait_test_setter(wait_test_setter fn);   // mi_api.cu

// Bounded wait on a tile-copy barrier with the limit of the test hook, read
// only once the barrier is found incomplete (no register held across the
// kernel's loop).
__device__ __forceinline__ bool mbar_wait_copy(uint64_t* bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    return mbar_wait(bar, parity, *(volatile long long*)&g_wait_limit);
}

namespace {
cudaError_t set_wait_test(long long limit, int arm_only) {
    cudaError_t e = cudaMemcpyToSymbol(g_wait_limit, &limit, sizeof(limit));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_wait_arm_only, &arm_only, sizeof(arm_only));
    return e;
}
[[maybe_unused]] const bool g_wait_test_registered = register_wait_test_setter(&set_wait_test);
}  // namespace

__host__ __device__ constexpr int pow2_at_least(int n) { return n <= 4 ? 4 : (n <= 8 ? 8 : (n <= 16 ? 16 : 32)); }

// Lanes per matrix used by default (n <= 8 runs one thread per matrix):
// 16 lanes for n > 16 keeps 8 x 8 register blocks (n = 32), i.e. 16 broadcast
// values per 64 FMAs; 8 lanes for n = 11..16 and 4 for n = 9, 10 (measured on
// GB300: 4 lanes lose from n = 12 up).
__host__ __device__ constexpr int default_lanes(int n, int mode) {
    return mode == kModePartial ? pow2_at_least(n) : (n > 16 ? 16 : (n > 10 ? 8 : 4));
}

// The other lanes-per-matrix a size can run at (0: none), chosen per
// (n, mode) at run time from the tuned table: eight lanes for n = 17..31
// without partial pivoting -- 8 x 16 register blocks, four matrices per warp,
// the same bits as sixteen lanes.  Measured on GB300 at 1,000,000 matrices:
// faster at n = 17..28 in most modes (no pivoting, n = 20: 0.87 against
// 1.09 ms), slower at n = 29..31 (the reference rule, n = 30: 4.82 against
// 3.83 ms).
__host__ __device__ constexpr int alt_lanes(int n, int mode) {
    return (mode != kModePartial && n > 16 && n < 32) ? 8 : 0;
}

// Blocks of 256 threads per SM the lane-group kernels are compiled for: two
// (at most 128 registers), or one for eight lanes above n = 16, whose 8 x 16
// register blocks need up to 255.
__host__ __device__ constexpr int lane_min_blocks(int n, int lanes) { return (lanes == 8 && n > 16) ? 1 : 2; }

// ---------------------------------------------------------------------------
// Geometry per (n, lanes per matrix).
// ---------------------------------------------------------------------------
template <int N, int L>
struct Geom {
    static_assert(N >= 1 && N <= 32, "n must be in 1..32");
    static_assert(L == 4 || L == 8 || L == 16 || L == 32, "lanes per matrix");
    static constexpr int M = 32 / L;                                    // matrices per warp
    static constexpr int RG = (L == 32) ? 8 : (L == 16 ? 4 : (L == 8 ? 4 : 2));
    static constexpr int CG = L / RG;
    static constexpr int R = (N + RG - 1) / RG;                        // rows per lane (cyclic)
    static constexpr int C = (((N + CG - 1) / CG) + 1) & ~1;           // columns per lane (even)
    static constexpr int PR = R * RG;
    static constexpr int PC = C * CG;
    static constexpr int P = pow2_at_least(N);                          // pivot-replay lanes per matrix
    static_assert(P % L == 0 || L == 32 || true, "");
    static constexpr int pad4(int x) { return (x + 3) & ~3; }
    static constexpr int kMat = N * N;                                  // stage floats per matrix
    // per-matrix scratch (floats)
    static constexpr int kCol = pad4(PR);
    static constexpr int kRow = pad4(PC);
    static constexpr int oCol = 0;
    static constexpr int oRow = oCol + 2 * kCol;
    static constexpr int oD = oRow + 2 * kRow;                          // pivot value of every step
    static constexpr int oWin = oD + 32;                                // input row placed at each step
    static constexpr int oMap = oWin + 32;                              // partial: output row of each slot
    static constexpr int kScratch = oMap + 32;
};

// Stage layout of one matrix: row-major, with the TMA 128-byte swizzle
// (16-byte chunk index XOR row & 7) for n = 32 so that both row-wise and
// column-block accesses from a warp are free of bank conflicts.
template <int N, bool SW = (N == 32)>
__device__ __forceinline__ int stage_off(int r, int c) {
    if constexpr (SW) return r * 32 + ((((c >> 2) ^ (r & 7)) << 2) | (c & 3));
    else return r * N + c;
}

// ---------------------------------------------------------------------------
// The reference's argmax tree (strides T/2, T/4, ..., 1; strict '<' so the
// lower slot keeps ties).  survive_mask: slots whose value can reach slot 0.
// prio: rank of each surviving slot when values tie (higher wins), 0 if the
// slot is dropped.  Derived by running the tree on tie-only inputs.
// ---------------------------------------------------------------------------
__host__ __device__ constexpr unsigned survive_mask(int T) {
    unsigned m = 0;
    for (int t = 0; t < T; t++) {
        int p = t;
        bool alive = true;
        for (int s = T / 2; s > 0; s >>= 1) {
            if (p >= 2 * s) { alive = false; break; }
            if (p >= s) p -= s;
        }
        if (alive && p == 0) m |= 1u << t;
    }
    return m;
}

struct PrioTable { unsigned char v[33][32]; };

__host__ __device__ constexpr PrioTable make_prio_table() {
    PrioTable tab{};
    for (int T = 1; T <= 32; T++) {
        bool alive[32] = {};
        for (int t = 0; t < T; t++) alive[t] = true;
        for (int rank = 32; rank > 0; rank--) {
            int val[32] = {}, idx[32] = {};
            for (int t = 0; t < T; t++) { val[t] = alive[t] ? 1 : 0; idx[t] = t; }
            for (int s = T / 2; s > 0; s >>= 1)
                for (int t = 0; t < s; t++)
                    if (val[t] < val[t + s]) { val[t] = val[t + s]; idx[t] = idx[t + s]; }
            if (val[0] == 0) break;
            tab.v[T][idx[0]] = (unsigned char)rank;
            alive[idx[0]] = false;
        }
    }
    return tab;
}

static __constant__ PrioTable c_prio = make_prio_table();

// ---------------------------------------------------------------------------
// Small helpers.
// ---------------------------------------------------------------------------
template <int P>
__device__ __forceinline__ unsigned group_max(unsigned x) {
    if constexpr (P == 32) {
        return __reduce_max_sync(kFull, x);
    } else {
#pragma unroll
        for (int o = P / 2; o > 0; o >>= 1) x = max(x, __shfl_xor_sync(kFull, x, o));
        return x;
    }
}

template <int P>
__device__ __forceinline__ unsigned group_min(unsigned x) {
    if constexpr (P == 32) {
        return __reduce_min_sync(kFull, x);
    } else {
#pragma unroll
        for (int o = P / 2; o > 0; o >>= 1) x = min(x, __shfl_xor_sync(kFull, x, o));
        return x;
    }
}

template <int P>
__device__ __forceinline__ unsigned group_ballot(bool p, int gbase) {
    const unsigned b = __ballot_sync(kFull, p);
    if constexpr (P == 32) return b;
    else return (b >> gbase) & ((1u << P) - 1u);
}

// Exact pivot-compare key: |x| as ordered bits, subnormals flushed to zero
// (the reference is built with --use_fast_math, parallel_pivot/run.py:47),
// NaN -> 0xffffffff (as the diagonal it blocks every exchange; as a candidate
// it fails the <= +inf test).
__device__ __forceinline__ unsigned pivot_key(float x) {
    const unsigned a = __float_as_uint(x) & 0x7fffffffu;
    const unsigned k = (a < 0x00800000u) ? 0u : a;
    return (a > 0x7f800000u) ? 0xffffffffu : k;
}

// Fast key: one max.NaN.ftz of |x| with 0: subnormals and zero -> 0, NaN ->
// 0x7fffffff (above +inf, so a NaN anywhere in the candidates shows up in the
// maximum and sends the step to the exact path).
__device__ __forceinline__ unsigned fast_key(float x) {
    float r;
    asm("max.NaN.ftz.f32 %0, %1, 0f00000000;" : "=f"(r) : "f"(fabsf(x)));
    return __float_as_uint(r);
}

// 1/d: hardware approximation refined by one Newton-Raphson step,
// r' = r + r (1 - d r).  A zero pivot yields a non-finite reciprocal.
__device__ __forceinline__ float recip(float d) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(d));
    const float e = fmaf(-d, r, 1.0f);
    return fmaf(r, e, r);
}

template <int CNT>
__device__ __forceinline__ void lds_vec(const float* p, float (&v)[CNT]) {
    if constexpr (CNT % 4 == 0) {
#pragma unroll
        for (int q = 0; q < CNT / 4; q++) {
            const float4 t = reinterpret_cast<const float4*>(p)[q];
            v[4 * q] = t.x; v[4 * q + 1] = t.y; v[4 * q + 2] = t.z; v[4 * q + 3] = t.w;
        }
    } else if constexpr (CNT % 2 == 0) {
#pragma unroll
        for (int q = 0; q < CNT / 2; q++) {
            const float2 t = reinterpret_cast<const float2*>(p)[q];
            v[2 * q] = t.x; v[2 * q + 1] = t.y;
        }
    } else {
#pragma unroll
        for (int q = 0; q < CNT; q++) v[q] = p[q];
    }
}

template <int CNT>
__device__ __forceinline__ void sts_vec(float* p, const float (&v)[CNT]) {
    if constexpr (CNT % 4 == 0) {
#pragma unroll
        for (int q = 0; q < CNT / 4; q++)
            reinterpret_cast<float4*>(p)[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    } else if constexpr (CNT % 2 == 0) {
#pragma unroll
        for (int q = 0; q < CNT / 2; q++) reinterpret_cast<float2*>(p)[q] = make_float2(v[2 * q], v[2 * q + 1]);
    } else {
#pragma unroll
        for (int q = 0; q < CNT; q++) p[q] = v[q];
    }
}

// a[*] -= m * w[*] on packed pairs.
template <int C>
__device__ __forceinline__ void row_update(float (&a)[C], float m, const float (&w)[C]) {
    const float2 nm = make_float2(-m, -m);
#pragma unroll
    for (int q = 0; q < C / 2; q++) {
        float2 x = make_float2(a[2 * q], a[2 * q + 1]);
        x = __ffma2_rn(nm, make_float2(w[2 * q], w[2 * q + 1]), x);
        a[2 * q] = x.x;
        a[2 * q + 1] = x.y;
    }
}

// ---------------------------------------------------------------------------
// Pivot replay of the reference rules.  A group of P lanes handles one
// matrix, lane s = input row s.  Writes win[k] = input row placed at step k.
// ---------------------------------------------------------------------------

// Exact rule for one step k, from scratch: positions after steps 0..k-1 are
// rebuilt from win[], then the reference's tree (or serial scan) runs on the
// raw entries with its own tie order and dropped slots.  Returns the row.
template <int N, int P, int MODE, bool SW = (N == 32)>
__device__ __noinline__ int exact_pivot(const float* st, const int* win, int k, int s, int gbase) {
    __syncwarp();
    int pos = (s < N) ? s : 0x7fff;
    for (int j = 0; j < k; ++j) {
        const int wj = win[j];
        const int pw = __shfl_sync(kFull, pos, gbase + wj);
        if (s == wj) pos = j;
        else if (pos == j) pos = pw;
    }
    const unsigned kraw = (s < N) ? pivot_key(st[stage_off<N, SW>(s, k)]) : 0u;
    const int dl = __ffs(group_ballot<P>(pos == k, gbase)) - 1;
    const unsigned kd = __shfl_sync(kFull, kraw, gbase + dl);
    const int slot = pos - k - 1;
    bool ok = (slot >= 0) && (pos < N) && (kraw > kd) && (kraw <= 0x7f800000u);
    if (MODE == kModeReference) ok = ok && ((survive_mask(N) >> (slot & 31)) & 1u);
    const unsigned cand = ok ? kraw : 0u;
    const unsigned mx = group_max<P>(cand);
    const bool top = ok && (cand == mx);
    unsigned pr = 0u;
    if (top) pr = (MODE == kModeReference) ? (unsigned)c_prio.v[N][slot] : (unsigned)(64 - pos);
    const unsigned pm = group_max<P>(pr);
    const unsigned tb = group_ballot<P>(top && pr == pm, gbase);
    return tb ? (__ffs(tb) - 1) : dl;   // nothing beats the diagonal: it stays
}

// Keys of row r, columns k0..k0+3 (0 past the matrix).
template <int N, bool SW = (N == 32)>
__device__ __forceinline__ void load_keys4(const float* st, int r, int k0, unsigned (&kv)[4]) {
    if (r >= N) {
#pragma unroll
        for (int t = 0; t < 4; t++) kv[t] = 0u;
        return;
    }
    if constexpr (N % 4 == 0) {
        const float4 v = *reinterpret_cast<const float4*>(st + (SW ? (r * 32 + ((((k0 >> 2) ^ (r & 7))) << 2))
                                                                  : (r * N + k0)));
        kv[0] = fast_key(v.x); kv[1] = fast_key(v.y); kv[2] = fast_key(v.z); kv[3] = fast_key(v.w);
    } else {
#pragma unroll
        for (int t = 0; t < 4; t++) kv[t] = (k0 + t < N) ? fast_key(st[r * N + k0 + t]) : 0u;
    }
}

// Maximum over the P-lane group that starts at lane gbase: one warp
// reduction, each group naming its own lanes.
// Groups of 8 or fewer lanes use a shuffle butterfly instead (reductions over
// several disjoint lane masks in one instruction were measured slower there).
template <int P>
__device__ __forceinline__ unsigned group_max_redux(unsigned x, int gbase) {
    if constexpr (P == 32) return __reduce_max_sync(kFull, x);
    else if constexpr (P >= 16) return __reduce_max_sync(((1u << P) - 1u) << gbase, x);
    else return group_max<P>(x);
}

// The fast replay for IM matrices at once, one independent chain each, so
// the reduction latencies of the chains overlap; keys are read from the
// stage four columns at a time (a compact, rolled loop).  A step costs one
// group maximum: the lane holding it takes the step, with no per-step vote or
// branch.  A matrix whose maximum ever tied (found at the end: two rows on one
// step) or where a NaN competed is replayed afterwards with the exact rule.
template <int N, int P, int IM, int MODE, bool SW = (N == 32)>
__device__ __forceinline__ void replay_fast_multi(const float* const (&st)[IM], int* const (&win)[IM], int s,
                                                  int gbase) {
    bool placed[IM];
    int step[IM];
    unsigned top[IM];
#pragma unroll
    for (int m = 0; m < IM; m++) {
        placed[m] = (s >= N);
        step[m] = 0;
        top[m] = 0u;
    }
#pragma unroll 1
    for (int k0 = 0; k0 < N; k0 += 4) {
        unsigned kv[IM][4];
#pragma unroll
        for (int m = 0; m < IM; m++) load_keys4<N, SW>(st[m], s, k0, kv[m]);
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const int k = k0 + t;
            if (N % 4 == 0 || k < N) {
#pragma unroll
                for (int m = 0; m < IM; m++) {
                    const unsigned cand = placed[m] ? 0u : kv[m][t];
                    const unsigned mx = group_max_redux<P>(cand, gbase);
                    const bool hit = (cand == mx);
                    top[m] = max(top[m], mx);
                    if (hit) {
                        placed[m] = true;
                        step[m] = k;
                    }
                }
            }
        }
    }
#pragma unroll
    for (int m = 0; m < IM; m++) {
        // every row takes exactly one step unless a maximum tied (two rows in
        // one step, or placed rows taking a later step where only keys 0
        // remain): rows that ended on one step are found by one match
        const int tag = ((s < N) ? step[m] : 64 + s) | (gbase << 8);
        const unsigned same = __match_any_sync(kFull, tag);   // every lane takes part
        const bool dup = (s < N) && (__popc(same) > 1);
        const bool bad = (group_ballot<P>(dup, gbase) != 0u) || (top[m] > 0x7f800000u);
        if (!bad && s < N) win[m][step[m]] = s;
        if (__any_sync(kFull, bad)) {
#pragma unroll 1
            for (int k = 0; k < N; ++k) {
                const int w = exact_pivot<N, P, MODE, SW>(st[m], win[m], k, s, gbase);
                if (bad && s == 0) win[m][k] = w;
            }
        }
    }
}

// Non-power-of-two n under the reference rule: some tree slots are dropped,
// so positions are tracked every step (lane = row).
template <int N, int P, int MODE, bool SW = (N == 32)>
__device__ __noinline__ void replay_tracked(const float* st, int* win, int s, int gbase) {
    constexpr unsigned kSurv = survive_mask(N);
    unsigned key[N];
#pragma unroll
    for (int k = 0; k < N; k++) key[k] = (s < N) ? pivot_key(st[stage_off<N, SW>(s, k)]) : 0u;
    int pos = (s < N) ? s : 0x7fff;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const unsigned bd = group_ballot<P>(pos == k, gbase);
        const int dl = __ffs(bd) - 1;
        const unsigned kd = __shfl_sync(kFull, key[k], gbase + dl);
        const int slot = pos - k - 1;
        bool ok = (slot >= 0) && (pos < N) && (key[k] > kd) && (key[k] <= 0x7f800000u);
        ok = ok && ((kSurv >> (slot & 31)) & 1u);
        const unsigned cand = ok ? key[k] : 0u;
        const unsigned mx = group_max<P>(cand);
        const bool top = ok && (cand == mx);
        unsigned tb = group_ballot<P>(top, gbase);
        if (__any_sync(kFull, (tb & (tb - 1u)) != 0u)) {
            unsigned pr = 0u;
            if (top) pr = (unsigned)c_prio.v[N][slot];
            const unsigned pm = group_max<P>(pr);
            tb = group_ballot<P>(top && pr == pm, gbase);
        }
        const int wl = tb ? (__ffs(tb) - 1) : dl;
        const int pw = __shfl_sync(kFull, pos, gbase + wl);
        if (s == wl) pos = k;
        else if (pos == k) pos = pw;
        if (s == 0) win[k] = wl;
    }
}

// The tracked replay for IM matrices at once (independent chains that
// overlap).  Keys are encoded 2|x| for a candidate and 2|x| + 1 for the row on
// the diagonal (|x| from fast_key: subnormals 0, NaN above every number), so
// one group maximum decides the step: an odd maximum means no surviving
// candidate beats the diagonal strictly (it stays), an even one names the
// winner.  A second maximum brings the winner's old position to the row it
// displaces.  A placed row never moves again, so its final position is the
// step that placed it; a tie between candidates leaves two rows at one
// position, found by one match after the last step.  Such a matrix, or one
// where a NaN competed (codes above 2 * inf + 1), is replayed again by
// replay_tracked with the exact keys and the tree's tie order.
template <int N, int P, int IM, int MODE, bool SW = (N == 32)>
__device__ __forceinline__ void replay_tracked_multi(const float* const (&st)[IM], int* const (&win)[IM], int s,
                                                     int gbase) {
    constexpr unsigned kSurv = survive_mask(N);
    constexpr unsigned kInfCode = 0x7f800000u << 1;
    unsigned ek[IM][N];
#pragma unroll
    for (int m = 0; m < IM; m++)
#pragma unroll
        for (int k = 0; k < N; k++) ek[m][k] = (s < N) ? (fast_key(st[m][stage_off<N, SW>(s, k)]) << 1) : 0u;
    int pos[IM];
    unsigned top[IM];
#pragma unroll
    for (int m = 0; m < IM; m++) {
        pos[m] = (s < N) ? s : 31;     // padding lanes: key 0, never on the diagonal
        top[m] = 0u;
    }
#pragma unroll
    for (int k = 0; k < N; ++k) {
        // positions whose tree slot (position - k - 1) survives at step k
        const unsigned surv = (k + 1 < 32) ? (unsigned)(((unsigned long long)kSurv << (k + 1)) & 0xffffffffull) : 0u;
#pragma unroll
        for (int m = 0; m < IM; m++) {
            const bool at = (pos[m] == k);
            const bool live = (surv >> pos[m]) & 1u;
            const unsigned e = at ? (ek[m][k] | 1u) : (live ? ek[m][k] : 0u);
            const unsigned mx = (P == 32) ? __reduce_max_sync(kFull, e) : group_max<P>(e);
            top[m] = max(top[m], mx);
            const bool hit = !at && (e == mx);
            int wpos;
            if constexpr (P == 32) {
                wpos = (int)__reduce_max_sync(kFull, hit ? (unsigned)pos[m] : 0u);
            } else {
                const unsigned tb = group_ballot<P>(hit, gbase);
                wpos = __shfl_sync(kFull, pos[m], gbase + (tb ? __ffs(tb) - 1 : 0));
            }
            if (hit) pos[m] = k;
            else if (at && !(mx & 1u)) pos[m] = wpos;
        }
    }
#pragma unroll
    for (int m = 0; m < IM; m++) {
        // rows of one matrix (tagged by group) that ended on the same position
        const unsigned same = __match_any_sync(kFull, pos[m] | (gbase << 8));
        const bool dup = (s < N) && (__popc(same) > 1);
        const bool bad = (group_ballot<P>(dup, gbase) != 0u) || (top[m] > kInfCode + 1u);
        if (!bad && s < N) win[m][pos[m]] = s;
        if (__any_sync(kFull, bad)) replay_tracked<N, P, MODE, SW>(st[m], win[m], s, gbase);
    }
}

// ---------------------------------------------------------------------------
// Elimination steps.  k is a constant after the step loop is unrolled.
// ---------------------------------------------------------------------------
template <class G>
__device__ __forceinline__ void gj_step(float (&a)[G::R][G::C], float (&ps)[G::R], const int k, int rg, int cg,
                                        int gb, float* scr) {
    constexpr int R = G::R, C = G::C;
    const int kr = k % G::RG, kri = k / G::RG;   // pivot-row owner group, register row
    const int kc = k / C, kci = k % C;           // column owner group, register column
    // column k for my rows from lane (rg, kc); row k for my columns from lane
    // (kr, cg); 1/pivot from lane (kr, kc) -- straight out of the owners'
    // registers, no shared-memory round trip
    const int src_c = gb + kc * G::RG + rg;
    const int src_w = gb + cg * G::RG + kr;
    float c[R], w[C];
#pragma unroll
    for (int ri = 0; ri < R; ri++) c[ri] = __shfl_sync(kFull, a[ri][kci], src_c);
#pragma unroll
    for (int ci = 0; ci < C; ci++) w[ci] = __shfl_sync(kFull, a[kri][ci], src_w);
    // the pivot's owner forms 1/pivot from its own register, off the
    // critical path of the broadcasts, and records the pivot for info
    const float pown = recip(a[kri][kci]);
    if (rg == kr && cg == kc) scr[G::oD + k] = a[kri][kci];
    const float p = __shfl_sync(kFull, pown, gb + kc * G::RG + kr);
    if (rg == kr) {
        c[kri] = 0.0f;                                // the pivot row takes no update
        ps[kri] = p;
    }
    if (cg == kc) {
        w[kci] = 1.0f;                                // column k becomes -multiplier
#pragma unroll
        for (int ri = 0; ri < R; ri++) a[ri][kci] = 0.0f;
        if (rg == kr) a[kri][kci] = 1.0f;
    }
    float m[R];
#pragma unroll
    for (int ri = 0; ri < R; ri += 2) {
        if (ri + 1 < R) {
            const float2 mm = __fmul2_rn(make_float2(c[ri], c[ri + 1]), make_float2(p, p));
            m[ri] = mm.x;
            m[ri + 1] = mm.y;
        } else {
            m[ri] = c[ri] * p;
        }
    }
#pragma unroll
    for (int ri = 0; ri < R; ri++) row_update<C>(a[ri], m[ri], w);
}

// Register row q of the block, selected by a runtime q through a static chain
// (no dynamically indexed register arrays).
template <class G>
__device__ __forceinline__ void get_row(const float (&a)[G::R][G::C], int q, float (&w)[G::C]) {
#pragma unroll
    for (int ci = 0; ci < G::C; ci++) w[ci] = a[0][ci];
#pragma unroll
    for (int r = 1; r < G::R; r++)
        if (q == r) {
#pragma unroll
            for (int ci = 0; ci < G::C; ci++) w[ci] = a[r][ci];
        }
}

template <class G>
__device__ __forceinline__ void set_row(float (&a)[G::R][G::C], int q, const float (&w)[G::C]) {
#pragma unroll
    for (int r = 0; r < G::R; r++)
        if (q == r) {
#pragma unroll
            for (int ci = 0; ci < G::C; ci++) a[r][ci] = w[ci];
        }
}

// Partial pivoting without row exchanges (L = P: lane t of the group keys
// slot t, i.e. input row t).  Rows stay in their slots; each slot carries the
// logical position lp it would have under getrf's physical exchanges, so the
// argmax of the updated column k over the unplaced slots breaks ties toward
// the lowest logical row exactly as LAPACK does.  The chosen slot's row is
// the pivot row of the step (broadcast through shared memory); the slot that
// holds logical row k takes over the winner's logical position.  The output
// rows are permuted at the store (output row of a slot = the step that chose
// it); the arithmetic of every row is that of the exchanging form.
template <class G>
__device__ __forceinline__ void gj_step_partial(float (&a)[G::R][G::C], const int k, int rg, int cg, int s, int gbase,
                                                float* scr, int& lp, bool& placed) {
    constexpr int R = G::R, C = G::C;
    const int kc = k / C, kci = k % C;
    float* cb = scr + G::oCol + (k & 1) * G::kCol;
    float* rb = scr + G::oRow + (k & 1) * G::kRow;
    if (cg == kc) {
        float v[R];
#pragma unroll
        for (int ri = 0; ri < R; ri++) v[ri] = a[ri][kci];
        sts_vec<R>(cb + rg * R, v);
    }
    __syncwarp();
    // column entry of slot t lives at cb[(t % RG) * R + t / RG]
    unsigned key = 0u;
    if (!placed && s < G::kN) {
        const unsigned b = __float_as_uint(cb[(s % G::RG) * R + s / G::RG]) & 0x7fffffffu;
        key = (b > 0x7f800000u) ? 1u : b + 2u;   // a NaN never beats a number
    }
    const unsigned mx = group_max<G::LL>(key);
    const bool top = (key != 0u) && (key == mx);
    const unsigned lw = group_min<G::LL>(top ? (unsigned)lp : 0xffu);   // lowest logical row among the maxima
    const int r = __ffs(group_ballot<G::LL>(top && (unsigned)lp == lw, gbase)) - 1;
    if (s == r) {
        lp = k;
        placed = true;
    } else if (lp == k) {
        lp = (int)lw;
    }
    // slot r's row is the pivot row: its owners store it straight from the
    // register row that holds it (one predicated store per row, no select)
    bool piv[R];
#pragma unroll
    for (int ri = 0; ri < R; ri++) piv[ri] = (rg + G::RG * ri == r);
#pragma unroll
    for (int ri = 0; ri < R; ri++)
        if (piv[ri]) sts_vec<C>(rb + cg * C, a[ri]);
    __syncwarp();
    float w[C];
    lds_vec<C>(rb + cg * C, w);
    const float d = cb[(r % G::RG) * R + r / G::RG];
    const float p = recip(d);
    // pivot value of the step (the row scales are formed from these at the end)
    if (s < G::kN) scr[G::oD + k] = d;    // every lane writes the same value
    if (s == 0) reinterpret_cast<int*>(scr + G::oWin)[k] = r;
    if (cg == kc) w[kci] = 1.0f;
    float c[R];
    lds_vec<R>(cb + rg * R, c);
#pragma unroll
    for (int ri = 0; ri < R; ri++) {
        c[ri] = piv[ri] ? 0.0f : c[ri];
        if (cg == kc) a[ri][kci] = piv[ri] ? 1.0f : 0.0f;
    }
#pragma unroll
    for (int ri = 0; ri < R; ri++) row_update<C>(a[ri], c[ri] * p, w);
}

// ---------------------------------------------------------------------------
// Per-warp pipeline.  Each warp owns one shared-memory slot for its M input
// matrices, a small row buffer for results and its own mbarrier:
//   wait for group g in the slot -> pivot replay + register block load ->
//   issue the copy of group g + (warps in grid) into the same slot (it lands
//   while this warp eliminates) -> n elimination steps in registers ->
//   results out through the row buffer with coalesced 16-byte stores.
// No CTA-wide barriers; occupancy is set by registers, not by staging memory.
// ---------------------------------------------------------------------------
template <int N, int L, int MODE>
struct KGeom {
    using G = Geom<N, L>;
    // register rows per output round; partial pivoting permutes its output
    // rows, so all of them leave in one round
    static constexpr int H = (MODE == kModePartial) ? G::R : ((G::RG >= 8) ? 1 : 8 / G::RG);
    static constexpr int ORows = G::RG * H;                      // matrix rows per output round
    static constexpr int Rounds = (G::R + H - 1) / H;
    // Output rows leave in rounds of ORows rows per matrix, either as tensor
    // stores from two alternating buffers in the stage layout (OBR x N per
    // matrix, dense or 128-byte swizzled) or, for odd n / unaligned pointers,
    // through one buffer with a padded pitch SB and 16-byte or scalar stores.
    static constexpr int OBR = ORows < N ? ORows : N;
    static constexpr int SB = (N % 4 == 0) ? (N <= 8 ? 8 : 40) : (N | 1);
    static constexpr int kSlot = G::M * G::kMat;
    // one tensor-store buffer, a multiple of 128 bytes so that the second of
    // the two alternating buffers starts on the alignment TMA tensor copies need
    static constexpr int kOutT = (G::M * OBR * N + 31) & ~31;
    static constexpr int kOutS = G::M * ORows * SB;
    // Window copies (n not a multiple of 4): the group arrives as one 1-D bulk
    // copy of the 16-byte-aligned window around it (up to 3 floats of shift
    // and 3 of rounding), and each output round of a matrix leaves from a
    // region placed at the same shift as its global range.
    // Measured on GB300 (1,000,000 matrices): the window store wins from
    // n = 10 up in the reference and no-pivot modes; below that, and in
    // partial mode, the rows leave faster by coalesced plain stores.
    static constexpr bool WinStore = (N % 4 != 0) && (N >= 10) && (MODE != kModePartial);
    static constexpr int kOWm = (ORows * N + 3 + 3) & ~3;
    static constexpr int kOutW = G::M * kOWm;
    static constexpr int kOut0 = (2 * kOutT > kOutS) ? 2 * kOutT : kOutS;
    static constexpr int kOut = (WinStore && 2 * kOutW > kOut0) ? 2 * kOutW : kOut0;
    static constexpr int kScr = (MODE == kModePartial) ? G::kScratch : 64;   // partial: column/row buffers, row map
    static constexpr int kScrTotal = G::M * kScr;
    static constexpr int r4(int x) { return (x + 3) & ~3; }
    // per-warp region (floats): slot | output rows | scratch | mbarrier; the
    // output buffers start on a 128-byte boundary (1 KB for n = 32, where one
    // buffer is a multiple of 1 KB)
    static constexpr int oOut = (N == 32) ? ((kSlot + 255) & ~255) : ((kSlot + 8 + 31) & ~31);
    static constexpr int oScr = oOut + r4(kOut);
    static constexpr int oBar = oScr + r4(kScrTotal);
    static constexpr int kWarp = (oBar + 4 + 255) / 256 * 256;   // 1 KB multiple
    static_assert(kOutT % 32 == 0 && oOut % 32 == 0, "TMA tensor-store buffers must start on 128-byte boundaries");
    static_assert(N != 32 || (kOutT % 256 == 0 && oOut % 256 == 0), "128-byte-swizzled buffers need 1 KB alignment");
};

// Offsets of the small per-matrix scratch: pivot values, then pivot rows.
template <class G, int MODE>
struct ScratchOff {
    static constexpr int oD = (MODE == kModePartial) ? G::oD : 0;
    static constexpr int oWin = (MODE == kModePartial) ? G::oWin : 32;
};

__device__ __forceinline__ void cp_async_4(float* dst, const float* src, bool valid) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_addr(dst)), "l"(src),
                 "r"(valid ? 4 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

template <int N, int L, int MODE>
struct GeomN : Geom<N, L> {
    static constexpr int kN = N;
    static constexpr int LL = L;
    static constexpr int oD = ScratchOff<Geom<N, L>, MODE>::oD;
    static constexpr int oWin = ScratchOff<Geom<N, L>, MODE>::oWin;
};

// ---- phase A: pivot order (reference rules) and the register block, rows in
// pivot order, from the warp's slot (stage layout SW).
template <int N, int L, int MODE, bool SW>
__device__ __forceinline__ void phase_load(float (&a)[GeomN<N, L, MODE>::R][GeomN<N, L, MODE>::C], const float* slot,
                                           float* scr0, int lane) {
    using G = GeomN<N, L, MODE>;
    using K = KGeom<N, L, MODE>;
    constexpr int R = G::R, C = G::C, M = G::M, P = G::P;
    const int mslot = lane / L, s = lane % L;
    const int rg = s % G::RG, cg = s / G::RG;
    const float* st = slot + mslot * G::kMat;
    int* win = reinterpret_cast<int*>(scr0 + mslot * K::kScr + G::oWin);
    if constexpr (MODE == kModeReference || MODE == kModeReferenceSerial) {
        constexpr int GP = 32 / P;      // replay groups per warp
        constexpr int IM = M / GP;      // matrices per replay group (= P / L)
        const int gi = lane / P, sp = lane % P;
        if constexpr (MODE == kModeReferenceSerial || (N & (N - 1)) == 0) {
            const float* stm[IM];
            int* winm[IM];
#pragma unroll
            for (int q = 0; q < IM; q++) {
                const int mm = q * GP + gi;
                stm[q] = slot + mm * G::kMat;
                winm[q] = reinterpret_cast<int*>(scr0 + mm * K::kScr + G::oWin);
            }
            replay_fast_multi<N, P, IM, MODE, SW>(stm, winm, sp, gi * P);
        } else {
            const float* stm[IM];
            int* winm[IM];
#pragma unroll
            for (int q = 0; q < IM; q++) {
                const int mm = q * GP + gi;
                stm[q] = slot + mm * G::kMat;
                winm[q] = reinterpret_cast<int*>(scr0 + mm * K::kScr + G::oWin);
            }
            replay_tracked_multi<N, P, IM, MODE, SW>(stm, winm, sp, gi * P);
        }
    } else if constexpr (MODE == kModeNone) {
        for (int t = s; t < N; t += L) win[t] = t;
    }
    __syncwarp();
#pragma unroll
    for (int ri = 0; ri < R; ri++) {
        const int i = rg + G::RG * ri;
        int src = i;
        if constexpr (MODE == kModeReference || MODE == kModeReferenceSerial) src = (i < N) ? win[i] : 0;
        if constexpr (N % 4 == 0 && C % 4 == 0) {
#pragma unroll
            for (int h = 0; h < C / 4; h++) {
                const int c0 = cg * C + 4 * h;
                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                if (c0 < N) v = *reinterpret_cast<const float4*>(st + stage_off<N, SW>(src, c0));
                a[ri][4 * h] = v.x; a[ri][4 * h + 1] = v.y; a[ri][4 * h + 2] = v.z; a[ri][4 * h + 3] = v.w;
            }
            if (i >= N) {
#pragma unroll
                for (int ci = 0; ci < C; ci++) a[ri][ci] = 0.0f;
            }
        } else {
#pragma unroll
            for (int ci = 0; ci < C; ci++) {
                const int j = cg * C + ci;
                a[ri][ci] = (i < N && j < N) ? st[stage_off<N, SW>(src, j)] : 0.0f;
            }
        }
    }
    __syncwarp();
}

// ---- phase B: n elimination steps and the final row scaling.
template <int N, int L, int MODE>
__device__ __forceinline__ void phase_eliminate(float (&a)[GeomN<N, L, MODE>::R][GeomN<N, L, MODE>::C], float* scr0,
                                                int lane) {
    using G = GeomN<N, L, MODE>;
    using K = KGeom<N, L, MODE>;
    constexpr int R = G::R, C = G::C;
    const int mslot = lane / L, s = lane % L;
    const int rg = s % G::RG, cg = s / G::RG;
    float* scr = scr0 + mslot * K::kScr;
    float ps[R];
#pragma unroll
    for (int ri = 0; ri < R; ri++) ps[ri] = 1.0f;
    if constexpr (MODE == kModePartial) {
        int lp = s;
        bool placed = (s >= N);
#pragma unroll
        for (int k = 0; k < N; ++k) gj_step_partial<G>(a, k, rg, cg, s, mslot * L, scr, lp, placed);
        __syncwarp();
        // output row of each slot = the step that chose it
        if (s < N) reinterpret_cast<int*>(scr + G::oMap)[reinterpret_cast<const int*>(scr + G::oWin)[s]] = s;
        __syncwarp();
        // scale of each row = 1 / the pivot of the step that chose its slot
        const int* omap = reinterpret_cast<const int*>(scr + G::oMap);
#pragma unroll
        for (int ri = 0; ri < R; ri++) {
            const int slot = rg + G::RG * ri;
            if (slot < N) ps[ri] = recip(scr[G::oD + omap[slot]]);
        }
    } else {
#pragma unroll
        for (int k = 0; k < N; ++k) gj_step<G>(a, ps, k, rg, cg, mslot * L, scr);
    }
#pragma unroll
    for (int ri = 0; ri < R; ri++) {
#pragma unroll
        for (int q = 0; q < C / 2; q++) {
            const float2 x = __fmul2_rn(make_float2(a[ri][2 * q], a[ri][2 * q + 1]), make_float2(ps[ri], ps[ri]));
            a[ri][2 * q] = x.x;
            a[ri][2 * q + 1] = x.y;
        }
    }
    __syncwarp();
}

// Destination column of each register column: A^-1[i][win[j]] = X[i][j].
template <int N, int L, int MODE>
__device__ __forceinline__ void dest_columns(int (&dst)[GeomN<N, L, MODE>::C], const float* scr0, int lane) {
    using G = GeomN<N, L, MODE>;
    using K = KGeom<N, L, MODE>;
    const int mslot = lane / L, s = lane % L;
    const int cg = s / G::RG;
    const int* win = reinterpret_cast<const int*>(scr0 + mslot * K::kScr + G::oWin);
#pragma unroll
    for (int ci = 0; ci < G::C; ci++) {
        const int j = cg * G::C + ci;
        dst[ci] = (j < N) ? win[j] : 0;
    }
}

// ---- phase C1: rows leave in rounds through two alternating buffers in the
// stage layout, each round one tensor store of ORows rows of the M matrices.
template <int N, int L, int MODE>
__device__ __forceinline__ void phase_store_tensor(const float (&a)[GeomN<N, L, MODE>::R][GeomN<N, L, MODE>::C],
                                                   float* outb, const float* scr0, int lane, const CUtensorMap* tmap_out,
                                                   long long first, unsigned& round) {
    using G = GeomN<N, L, MODE>;
    using K = KGeom<N, L, MODE>;
    constexpr int R = G::R, C = G::C;
    const int mslot = lane / L, s = lane % L;
    const int rg = s % G::RG, cg = s / G::RG;
    int dst[C];
    dest_columns<N, L, MODE>(dst, scr0, lane);
    // n = 32 (128-byte swizzle): with 4 row groups the swizzle of output row
    // rg + 4h takes two values, one per parity of h -- two column tables
    constexpr bool kTwoTables = (N == 32) && (G::RG == 4) && (MODE != kModePartial);
    int dsx[kTwoTables ? 2 : 1][C];
    if constexpr (kTwoTables) {
#pragma unroll
        for (int par = 0; par < 2; par++)
#pragma unroll
            for (int ci = 0; ci < C; ci++) dsx[par][ci] = dst[ci] ^ (((rg + 4 * par) & 7) << 2);
    }
#pragma unroll
    for (int q = 0; q < K::Rounds; q++) {
        // buffers alternate over the warp's whole sequence of rounds, so the
        // one written now is never the one of the most recent store (with an
        // even number of rounds per group that is the round's own parity)
        const unsigned par = (K::Rounds & 1) ? ((round + q) & 1u) : ((unsigned)q & 1u);
        float* obuf = outb + par * K::kOutT;
        float* ob = obuf + mslot * K::OBR * N;
        if (lane == 0) bulk_wait_read_one();   // this buffer's store from two rounds ago has read it
        __syncwarp();
        const int* omap = reinterpret_cast<const int*>(scr0 + mslot * K::kScr + G::oMap);
#pragma unroll
        for (int h = 0; h < K::H; h++) {
            const int ri = q * K::H + h;
            const int i = rg + G::RG * ri;
            const int lr = (MODE == kModePartial) ? ((ri < R && i < N) ? omap[i] : K::OBR) : rg + G::RG * h;
            if (ri < R && lr < K::OBR) {
                if (i < N) {
                    float* orow = ob + lr * N;
                    if constexpr (kTwoTables) {
#pragma unroll
                        for (int ci = 0; ci < C; ci++) orow[dsx[h & 1][ci]] = a[ri][ci];
                    } else {
                        const int x = (N == 32) ? ((lr & 7) << 2) : 0;
#pragma unroll
                        for (int ci = 0; ci < C; ci++)
                            if (cg * C + ci < N) orow[dst[ci] ^ x] = a[ri][ci];
                    }
                }
            }
        }
        fence_proxy_async();
        __syncwarp();
        if (lane == 0) {
            tma_store_3d(tmap_out, 0, q * K::ORows, (int)first, obuf);
            bulk_commit();
        }
    }
    round += K::Rounds;
}

// ---- phase C3 (n not a multiple of 4, 16-byte aligned batch): each output
// round of matrix m is the contiguous range [G0, G1) of A.  Its rows are
// written to a region at the shift G0 mod 4, the 16-byte-aligned interior
// leaves by a 1-D bulk store, and the at most 3 + 3 floats outside it by
// plain stores.  Buffers alternate over the warp's sequence of rounds.
template <int N, int L, int MODE>
__device__ __forceinline__ void phase_store_window(const float (&a)[GeomN<N, L, MODE>::R][GeomN<N, L, MODE>::C],
                                                   float* outb, const float* scr0, int lane, float* A,
                                                   const long long (&gbase)[GeomN<N, L, MODE>::M], unsigned& round) {
    using G = GeomN<N, L, MODE>;
    using K = KGeom<N, L, MODE>;
    constexpr int R = G::R, C = G::C, M = G::M;
    constexpr long long NN = (long long)N * N;
    const int mslot = lane / L, s = lane % L;
    const int rg = s % G::RG, cg = s / G::RG;
    int dst[C];
    dest_columns<N, L, MODE>(dst, scr0, lane);
#pragma unroll
    for (int q = 0; q < K::Rounds; q++) {
        const int row0 = q * K::ORows;
        const int rows = (N - row0 < K::ORows) ? (N - row0) : K::ORows;
        const unsigned par = (K::Rounds & 1) ? ((round + q) & 1u) : ((unsigned)q & 1u);
        float* obuf = outb + par * K::kOutW;
        if (lane == 0) bulk_wait_read_one();
        __syncwarp();
        const int e = (int)((gbase[mslot] + (long long)row0 * N) & 3);   // (gbase < 0: no matrix, value unused)
        float* ob = obuf + mslot * K::kOWm + e;
#pragma unroll
        for (int h = 0; h < K::H; h++) {
            const int ri = q * K::H + h;
            if (ri < R) {
                const int i = rg + G::RG * ri;
                if (i < N) {
                    float* orow = ob + (rg + G::RG * h) * N;
#pragma unroll
                    for (int ci = 0; ci < C; ci++)
                        if (cg * C + ci < N) orow[dst[ci]] = a[ri][ci];
                }
            }
        }
        fence_proxy_async();
        __syncwarp();
        if (lane == 0) {
#pragma unroll
            for (int m = 0; m < M; m++) {
                if (gbase[m] >= 0) {
                    const long long g0 = gbase[m] + (long long)row0 * N, g1 = g0 + (long long)rows * N;
                    const long long a0 = (g0 + 3) & ~3LL, a1 = g1 & ~3LL;
                    if (a1 > a0)
                        bulk_store(A + a0, obuf + m * K::kOWm + (int)(g0 & 3) + (int)(a0 - g0),
                                   (uint32_t)((a1 - a0) * 4));
                }
            }
            bulk_commit();
        }
        for (int t = lane; t < M * 6; t += 32) {
            const int m = t / 6, u = t - m * 6;
            long long gb = gbase[0];
#pragma unroll
            for (int q = 1; q < M; q++)
                if (m == q) gb = gbase[q];
            if (gb >= 0) {
                const long long g0 = gb + (long long)row0 * N, g1 = g0 + (long long)rows * N;
                const long long a0 = (g0 + 3) & ~3LL, a1 = g1 & ~3LL;
                const long long head_end = a0 < g1 ? a0 : g1;
                const long long x = (u < 3) ? g0 + u : ((a1 > a0 ? a1 : a0) + (u - 3));
                const bool valid = (u < 3) ? (x < head_end) : (x < g1);
                if (valid) A[x] = obuf[m * K::kOWm + (int)(g0 & 3) + (int)(x - g0)];
            }
        }
        __syncwarp();
    }
    round += K::Rounds;
}

// ---- phase C2: rows leave through one padded buffer with plain stores to the
// M matrices at gout[m] (nullptr = no matrix); 16-byte stores when `vec`.
template <int N, int L, int MODE>
__device__ __forceinline__ void phase_store_rows(const float (&a)[GeomN<N, L, MODE>::R][GeomN<N, L, MODE>::C],
                                                 float* outb, const float* scr0, int lane,
                                                 float* const (&gout)[GeomN<N, L, MODE>::M], bool vec) {
    using G = GeomN<N, L, MODE>;
    using K = KGeom<N, L, MODE>;
    constexpr int R = G::R, C = G::C, M = G::M;
    const int mslot = lane / L, s = lane % L;
    const int rg = s % G::RG, cg = s / G::RG;
    int dst[C];
    dest_columns<N, L, MODE>(dst, scr0, lane);
    float* ob = outb + mslot * K::ORows * K::SB;
#pragma unroll
    for (int q = 0; q < K::Rounds; q++) {
#pragma unroll
        for (int h = 0; h < K::H; h++) {
            const int ri = q * K::H + h;
            if (ri < R) {
                const int i = rg + G::RG * ri;
                if (i < N) {
                    const int lr = (MODE == kModePartial)
                                       ? reinterpret_cast<const int*>(scr0 + mslot * K::kScr + G::oMap)[i]
                                       : rg + G::RG * h;
                    float* orow = ob + lr * K::SB;
#pragma unroll
                    for (int ci = 0; ci < C; ci++)
                        if (cg * C + ci < N) orow[dst[ci]] = a[ri][ci];
                }
            }
        }
        __syncwarp();
        const int row0 = q * K::ORows;
        const int rows = (N - row0 < K::ORows) ? (N - row0) : K::ORows;
        if (rows > 0) {
            if (N % 4 == 0 && vec) {
                constexpr int Q = N / 4;               // 16-byte chunks per row
                const int per = rows * Q;
                for (int e = lane; e < M * per; e += 32) {
                    const int m = e / per, rem = e - m * per;
                    const int r = rem / Q, c4 = rem - r * Q;
                    if (gout[m] != nullptr) {
                        const float4 v = *reinterpret_cast<const float4*>(outb + (m * K::ORows + r) * K::SB + 4 * c4);
                        *reinterpret_cast<float4*>(gout[m] + (row0 + r) * N + 4 * c4) = v;
                    }
                }
            } else {
                const int per = rows * N;
                for (int e = lane; e < M * per; e += 32) {
                    const int m = e / per, rem = e - m * per;
                    const int r = rem / N, c = rem - r * N;
                    if (gout[m] != nullptr) gout[m][(row0 + r) * N + c] = outb[(m * K::ORows + r) * K::SB + c];
                }
            }
        }
        __syncwarp();
    }
}

// ---- phase D: pivots and info of this lane's matrix at output index `idx`
// (negative: no matrix); perm rows have pitch `perm_pitch`.
template <int N, int L, int MODE>
__device__ __forceinline__ void phase_perm_info(const float* scr0, int lane, long long idx, int32_t* perm_out,
                                                int perm_pitch, int32_t* info_out) {
    using G = GeomN<N, L, MODE>;
    using K = KGeom<N, L, MODE>;
    const int mslot = lane / L, s = lane % L;
    const float* scr = scr0 + mslot * K::kScr;
    const int* win = reinterpret_cast<const int*>(scr + G::oWin);
    unsigned zmask = 0u;
#pragma unroll
    for (int q = 0; q < (N + L - 1) / L; q++) {
        const int t = s + q * L;
        const bool z = (t < N) && (scr[G::oD + t] == 0.0f);
        zmask |= group_ballot<L>(z, mslot * L) << (q * L);
        if (perm_out != nullptr && t < N && idx >= 0) perm_out[idx * perm_pitch + t] = win[t];
    }
    if (info_out != nullptr && s == 0 && idx >= 0) info_out[idx] = zmask ? __ffs(zmask) : 0;
    __syncwarp();
}

// n = 32 stage that arrived row-major (1-D copies) -> the 128-byte swizzle of
// stage_off, in place: 16-byte chunk c of row r moves to c ^ (r & 7).  Each
// warp instruction reads and writes 4 whole rows, so neither side conflicts.
template <int M>
__device__ __forceinline__ void swizzle_stage32(float* slot, int lane) {
    constexpr int kPer = M * 32 * 8 / 32;      // 16-byte chunks per lane
    float4* s4 = reinterpret_cast<float4*>(slot);
    float4 v[kPer];
#pragma unroll
    for (int q = 0; q < kPer; q++) v[q] = s4[q * 32 + lane];
    __syncwarp();
#pragma unroll
    for (int q = 0; q < kPer; q++) {
        const int e = q * 32 + lane, row = e >> 3, c = e & 7;
        s4[(row << 3) | (c ^ (row & 7))] = v[q];
    }
    __syncwarp();
}

// Per-warp shared memory carving.
template <int N, int L, int MODE>
struct WarpSmem {
    float* slot;
    float* outb;
    float* scr0;
    uint64_t* bar;
    // warp `warp`'s region at a pitch of `pitch` floats (a multiple of 256)
    // from the first 1 KB boundary of the dynamic shared memory
    __device__ __forceinline__ WarpSmem(unsigned char* smem_raw, int warp, int pitch = KGeom<N, L, MODE>::kWarp) {
        using K = KGeom<N, L, MODE>;
        const uintptr_t base = (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023);
        slot = reinterpret_cast<float*>(base) + (size_t)warp * pitch;
        outb = slot + K::oOut;
        scr0 = slot + K::oScr;
        bar = reinterpret_cast<uint64_t*>(slot + K::oBar);
    }
};

// ---------------------------------------------------------------------------
// Contiguous batch: matrix b at A + b*n*n.  Persistent warps walk groups of M
// matrices; one slot per warp, the next group's copy issued right after the
// block load.
// ---------------------------------------------------------------------------
template <int N, int L, int MODE>
__global__ void __launch_bounds__(256, lane_min_blocks(N, L)) mi_inverse_kernel(float* __restrict__ A, int32_t* __restrict__ perm_out,
                                                            int32_t* __restrict__ info_out, long long batch,
                                                            int copy_mode, int vec_out,
                                                            const __grid_constant__ CUtensorMap tmap,
                                                            const __grid_constant__ CUtensorMap tmap_out) {
    using G = GeomN<N, L, MODE>;
    using K = KGeom<N, L, MODE>;
    constexpr int NN = N * N, R = G::R, C = G::C, M = G::M;
    extern __shared__ unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int W = blockDim.x >> 5;
    const WarpSmem<N, L, MODE> sm(smem_raw, warp);
    const int mslot = lane / L;

    if (lane == 0) {
        mbar_init(sm.bar, 1);
        fence_mbar_init();
        if (copy_mode == kCopyTensor) {
            tma_prefetch_map(&tmap);
            tma_prefetch_map(&tmap_out);
        }
    }
    __syncwarp();

    const long long groups = (batch + M - 1) / M;
    const long long gstride = (long long)gridDim.x * W;
    // window copies: the 16-byte-aligned float range [w0, w1) around the group,
    // used while it stays inside the batch
    auto window = [&](long long g, long long& w0, long long& w1) {
        const long long f0 = g * M * NN;
        const long long cnt = (batch - g * M < M) ? (batch - g * M) : M;
        w0 = f0 & ~3LL;
        w1 = (f0 + cnt * NN + 3) & ~3LL;
        return w1 <= batch * NN;
    };
    auto is_async = [&](long long g) {
        long long w0, w1;
        return copy_mode == kCopyTensor || (copy_mode == kCopyBulk && (g + 1) * M <= batch) ||
               (copy_mode == kCopyWindow && window(g, w0, w1));
    };
    auto issue = [&](long long g) {
        const long long first = g * M;
        if (is_async(g)) {
            if (lane == 0) {
                if (copy_mode == kCopyWindow) {
                    long long w0, w1;
                    window(g, w0, w1);
                    mbar_arrive_expect_tx(sm.bar, (uint32_t)((w1 - w0) * 4));
                    if (g_wait_arm_only == 0) bulk_load(sm.slot, A + w0, (uint32_t)((w1 - w0) * 4), sm.bar);
                } else {
                    mbar_arrive_expect_tx(sm.bar, (uint32_t)(K::kSlot * 4));
                    if (g_wait_arm_only != 0) {
                    } else if (copy_mode == kCopyTensor) {
                        tma_load_3d(sm.slot, &tmap, 0, 0, (int)first, sm.bar);
                    } else {
                        bulk_load(sm.slot, A + first * NN, (uint32_t)(K::kSlot * 4), sm.bar);
                    }
                }
            }
        } else {
            for (int e = lane; e < M * NN; e += 32) {
                const int m = e / NN, rem = e - m * NN;
                const int r = rem / N, c = rem - r * N;
                const bool valid = first + m < batch;
                cp_async_4(sm.slot + m * G::kMat + stage_off<N>(r, c), valid ? A + first * NN + e : A, valid);
            }
            cp_async_commit();
        }
    };

    long long g = (long long)blockIdx.x * W + warp;
    uint32_t phase = 0;
    unsigned round = 0;
    bool timed_out = false;
    if (g < groups) issue(g);
    while (g < groups) {
        const long long first = g * M;
        const bool async_g = is_async(g);
        // a window copy lands at the group's offset within its 16-byte granule
        const int shift = (copy_mode == kCopyWindow && async_g) ? (int)((first * NN) & 3) : 0;
        if (async_g) {
            // lanes time their waits separately, so the warp decides together
            if (!__all_sync(kFull, mbar_wait_copy(sm.bar, phase & 1u))) {
                timed_out = true;
                break;
            }
            phase++;
        } else {
            cp_async_wait_all();
        }
        __syncwarp();

        float a[R][C];
        phase_load<N, L, MODE, (N == 32)>(a, sm.slot + shift, sm.scr0, lane);

        // the slot is free: bring in this warp's next group now
        const long long gn = g + gstride;
        if (gn < groups) {
            if (lane == 0) fence_proxy_async();
            issue(gn);
        }

        phase_eliminate<N, L, MODE>(a, sm.scr0, lane);
        if (copy_mode == kCopyTensor) {
            phase_store_tensor<N, L, MODE>(a, sm.outb, sm.scr0, lane, &tmap_out, first, round);
        } else if (K::WinStore && copy_mode == kCopyWindow) {
            long long gbase[M];
#pragma unroll
            for (int m = 0; m < M; m++) gbase[m] = (first + m < batch) ? (first + m) * NN : -1;
            phase_store_window<N, L, MODE>(a, sm.outb, sm.scr0, lane, A, gbase, round);
        } else {
            float* gout[M];
#pragma unroll
            for (int m = 0; m < M; m++) gout[m] = (first + m < batch) ? A + (first + m) * NN : nullptr;
            phase_store_rows<N, L, MODE>(a, sm.outb, sm.scr0, lane, gout, vec_out != 0);
        }
        const long long mb = first + mslot;
        phase_perm_info<N, L, MODE>(sm.scr0, lane, mb < batch ? mb : -1, perm_out, N, info_out);
        g = gn;
    }
    if (timed_out) {
        atomicOr(&g_device_error, 1);
        // the copy may still land in this warp's slot: wait for it once more,
        // bounded, before the warp leaves
        mbar_wait_copy(sm.bar, phase & 1u);
    }
    if (lane == 0) bulk_wait_all();
}

// One warp's walk over the groups g, g + gstride, ... (< g_end) of one
// bucket, whose descriptor indices are list[start .. start + count).  The
// warp's region `sm` holds the copy mbarrier only for the walk: it is
// initialised here and invalidated before a normal return, so the region can
// take another geometry afterwards.  Returns false when a copy wait ran out
// (the device error word is set; the warp must take no more work).
template <int N, int L, int MODE>
__device__ __forceinline__ bool indexed_walk(const WarpSmem<N, L, MODE>& sm, int lane, float* __restrict__ base,
                                             const long long* __restrict__ offsets, const int* __restrict__ list,
                                             long long start, long long count, long long g, long long g_end,
                                             long long gstride, int32_t* __restrict__ perm_out,
                                             int32_t* __restrict__ info_out) {
    using G = GeomN<N, L, MODE>;
    using K = KGeom<N, L, MODE>;
    constexpr int NN = N * N, R = G::R, C = G::C, M = G::M;
    const int mslot = lane / L;
    __syncwarp();
    if (lane == 0) {
        mbar_init(sm.bar, 1);
        fence_mbar_init();
        // the region may hold data of an earlier walk, read and written
        // through the generic proxy, where the first bulk copy lands
        fence_proxy_async();
    }
    __syncwarp();
    const bool base16 = (reinterpret_cast<uintptr_t>(base) & 15u) == 0;
    const long long groups = g_end;

    // descriptor index of matrix m of group g (-1 past the end of the bucket)
    auto index_of = [&](long long g, int m) -> long long {
        const long long p = g * M + m;
        return p < count ? (long long)list[start + p] : -1;
    };
    auto bulk_ok = [&](long long idx) { return idx >= 0 && base16 && NN % 4 == 0 && (offsets[idx] & 3) == 0; };
    // returns whether the group used the mbarrier
    auto issue = [&](long long g) -> bool {
        long long idx[M];
        uint32_t bytes = 0;
#pragma unroll
        for (int m = 0; m < M; m++) {
            idx[m] = index_of(g, m);
            if (bulk_ok(idx[m])) bytes += NN * 4;
        }
        if (bytes != 0 && lane == 0) {
            mbar_arrive_expect_tx(sm.bar, bytes);
#pragma unroll
            for (int m = 0; m < M; m++)
                if (bulk_ok(idx[m])) bulk_load(sm.slot + m * G::kMat, base + offsets[idx[m]], NN * 4, sm.bar);
        }
#pragma unroll
        for (int m = 0; m < M; m++) {
            if (!bulk_ok(idx[m])) {
                const bool valid = idx[m] >= 0;
                const float* src = valid ? base + offsets[idx[m]] : base;
                for (int e = lane; e < NN; e += 32)
                    cp_async_4(sm.slot + m * G::kMat + e, valid ? src + e : base, valid);
            }
        }
        cp_async_commit();
        return bytes != 0;
    };

    uint32_t phase = 0;
    unsigned round = 0;
    bool timed_out = false;
    bool used_bar = false;
    if (g < groups) used_bar = issue(g);
    while (g < groups) {
        if (used_bar) {
            // lanes time their waits separately, so the warp decides together
            if (!__all_sync(kFull, mbar_wait(sm.bar, phase & 1u, kWaitLimit))) {
                timed_out = true;
                break;
            }
            phase++;
        }
        cp_async_wait_all();
        __syncwarp();

        float a[R][C];
        if constexpr (N == 32) {
            swizzle_stage32<M>(sm.slot, lane);
            phase_load<N, L, MODE, true>(a, sm.slot, sm.scr0, lane);
        } else {
            phase_load<N, L, MODE, false>(a, sm.slot, sm.scr0, lane);
        }

        long long idx[M];
        float* gout[M];
        bool vec = base16 && N % 4 == 0;
#pragma unroll
        for (int m = 0; m < M; m++) {
            idx[m] = index_of(g, m);
            gout[m] = idx[m] >= 0 ? base + offsets[idx[m]] : nullptr;
            if (idx[m] >= 0 && (offsets[idx[m]] & 3) != 0) vec = false;
        }
        const long long gn = g + gstride;
        if (gn < groups) {
            if (lane == 0) fence_proxy_async();
            used_bar = issue(gn);
        }
        phase_eliminate<N, L, MODE>(a, sm.scr0, lane);
        if (K::WinStore && base16) {
            long long gbase[M];
#pragma unroll
            for (int m = 0; m < M; m++) gbase[m] = idx[m] >= 0 ? offsets[idx[m]] : -1;
            phase_store_window<N, L, MODE>(a, sm.outb, sm.scr0, lane, base, gbase, round);
        } else {
            phase_store_rows<N, L, MODE>(a, sm.outb, sm.scr0, lane, gout, vec);
        }
        phase_perm_info<N, L, MODE>(sm.scr0, lane, idx[mslot], perm_out, 32, info_out);
        g = gn;
    }
    if (timed_out) {
        atomicOr(&g_device_error, 1);
        // the copy may still land in this warp's slot: wait for it once more,
        // bounded, before the warp leaves
        mbar_wait(sm.bar, phase & 1u, kWaitLimit);
    }
    if (lane == 0) bulk_wait_all();
    __syncwarp();
    if (!timed_out && lane == 0) mbar_inval(sm.bar);
    __syncwarp();
    return !timed_out;
}

// ---------------------------------------------------------------------------
// Indexed batch (descriptor buckets): the matrices of one (n, mode) bucket are
// list[range[0] .. range[0] + range[1]) -- descriptor indices -- at
// base + offsets[index].  Each matrix moves in by a 1-D bulk copy when its
// address allows (16-byte aligned, n*n a multiple of 4), else element by
// element with asynchronous copies; results leave with plain stores.  Pivots
// go to perm_out[index * 32 ..], info to info_out[index].
// ---------------------------------------------------------------------------
template <int N, int L, int MODE>
__global__ void __launch_bounds__(256, lane_min_blocks(N, L)) mi_inverse_indexed_kernel(float* __restrict__ base,
                                                                    const long long* __restrict__ offsets,
                                                                    const int* __restrict__ list,
                                                                    const long long* __restrict__ range,
                                                                    int32_t* __restrict__ perm_out,
                                                                    int32_t* __restrict__ info_out) {
    extern __shared__ unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int W = blockDim.x >> 5;
    const long long start = range[0], count = range[1];
    if (count <= 0) return;
    const long long groups = (count + GeomN<N, L, MODE>::M - 1) / GeomN<N, L, MODE>::M;
    const long long g = (long long)blockIdx.x * W + warp;
    if (g >= groups) return;
    indexed_walk<N, L, MODE>(WarpSmem<N, L, MODE>(smem_raw, warp), lane, base, offsets, list, start, count, g, groups,
                             (long long)gridDim.x * W, perm_out, info_out);
}

// Dynamic shared memory for a block of `warps` warps (1 KB of slack for the
// 1024-byte alignment the swizzled tensor copies need).
template <int N, int L, int MODE>
constexpr size_t smem_bytes(int warps) {
    return 1024 + (size_t)warps * KGeom<N, L, MODE>::kWarp * sizeof(float);
}

}  // namespace mi
