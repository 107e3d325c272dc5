// mi_tiny.cuh -- small n: one thread per matrix.
//
// At these sizes a matrix is 4 to 784 bytes, and the lane groups of the
// sub-warp kernel spend more instructions on coordination than on the
// arithmetic.  Here each thread loads its matrix into registers, evaluates
// the pivot rule serially (the reference's tree with T = n slots, the
// serial scan, or partial pivoting on the updated column) and runs the same
// Gauss-Jordan step as gj_step / gj_step_partial, element for element:
// m = c * (1/pivot), a = fma(-m, w, a) with column k zeroed first and w[k] = 1,
// the pivot row updated with c = 0, rows scaled by 1/pivot at the end.  So
// results are the sub-warp kernel's, bit for bit.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "mi_kernel.cuh"

namespace mi {

constexpr int kTinyMax = 8;        // one thread per matrix at any batch size
constexpr int kTinySlotMin = 3;    // smallest n of the shared-memory-slot form, contiguous batches
constexpr int kTinySlotMax = 15;   // largest n of the shared-memory-slot form (n = 16 spills)
constexpr int kTinySlotMinIndexed = 3;   // smallest n of the slot form, descriptor buckets (measured: the uneven call 1.98 -> 1.90 ms against 9)

// Largest n inverted one thread per matrix for contiguous batches, per pivot
// mode.  Measured on GB300 at 1,000,000 matrices against the sub-warp kernel
// (same results bit for bit): n = 9 .. 15 run 1.07-3.5x faster in the
// no-pivot and reference modes and 1.3-7.8x in partial mode; at n = 16 the
// 256-value matrix no longer fits in registers and the slot form is 1.4-2x
// slower.  Against the register form (select chains for the row order and
// the column permutation) the slot form is 1.1-1.8x faster at n = 3..8 and
// slower only at n = 2.
template <int MODE>
__host__ __device__ constexpr int tiny_max_contig() { return 15; }

// Smallest batch for which one thread per matrix beats the lane groups: a
// small batch leaves few warps per SM, each running one long serial chain.
// Measured crossovers (n = 12 and 15): 8,192 -> 16,384 matrices without
// pivoting and with the reference rule, 2,048 -> 8,192 in partial mode; at
// n = 9 one thread per matrix wins from 2,048 up.
template <int N, int MODE>
__host__ __device__ constexpr long long tiny_min_batch() {
    return N <= 10 ? 0 : (MODE == kModePartial ? 4096 : 12288);
}

// |x| with subnormals flushed to zero, NaN kept (compares as false): the
// reference's fast-math fabs in its pivot compares.
__device__ __forceinline__ float tiny_ref_key(float x) {
    const float a = fabsf(x);
    return (a < 1.17549435e-38f) ? 0.0f : a;
}

template <int N>
__device__ __forceinline__ float tiny_get(const float (&a)[N][N], int r, int c) {
    float v = a[0][c];
#pragma unroll
    for (int i = 1; i < N; i++)
        if (r == i) v = a[i][c];
    return v;
}

// Pivot sequence of the reference rules on the raw matrix: win[k] = input
// row placed at step k.  Parallel rule: per slot t, the diagonal against row
// k+1+t (strict '>'), then the tree with strides T/2 .. 1 (strict '<').
template <int N, int MODE, class Get>
__device__ __forceinline__ void tiny_pivots_by(Get get, int (&win)[N]) {
#pragma unroll
    for (int i = 0; i < N; i++) win[i] = i;
#pragma unroll
    for (int k = 0; k < N; k++) {
        int p = k;
        if constexpr (MODE == kModeReference) {
            float vals[N];
            int idxs[N];
            const float dk = tiny_ref_key(get(win[k], k));
#pragma unroll
            for (int t = 0; t < N; t++) {
                vals[t] = dk;
                idxs[t] = k;
                const int i = k + 1 + t;
                if (i < N) {
                    const float w = tiny_ref_key(get(win[i], k));
                    if (w > vals[t]) {
                        vals[t] = w;
                        idxs[t] = i;
                    }
                }
            }
#pragma unroll
            for (int s = N / 2; s > 0; s >>= 1)
#pragma unroll
                for (int t = 0; t < s; t++)
                    if (vals[t] < vals[t + s]) {
                        vals[t] = vals[t + s];
                        idxs[t] = idxs[t + s];
                    }
            p = idxs[0];
        } else {   // serial scan
            float mv = tiny_ref_key(get(win[k], k));
#pragma unroll
            for (int i = k + 1; i < N; i++) {
                const float w = tiny_ref_key(get(win[i], k));
                if (w > mv) {
                    mv = w;
                    p = i;
                }
            }
        }
        // swap win[k] and win[p] (p >= k, runtime)
        const int wk = win[k];
        int wp = win[k];
#pragma unroll
        for (int i = k + 1; i < N; i++)
            if (p == i) wp = win[i];
#pragma unroll
        for (int i = k + 1; i < N; i++)
            if (p == i) win[i] = wk;
        win[k] = wp;
    }
}

template <int N, int MODE>
__device__ __forceinline__ void tiny_pivots(const float (&a)[N][N], int (&win)[N]) {
    tiny_pivots_by<N, MODE>([&](int r, int c) { return tiny_get<N>(a, r, c); }, win);
}

// One Gauss-Jordan step on rows already in pivot order (as gj_step).
template <int N>
__device__ __forceinline__ void tiny_step(float (&b)[N][N], float (&ps)[N], float (&dv)[N], const int k) {
    float c[N], w[N];
#pragma unroll
    for (int i = 0; i < N; i++) c[i] = b[i][k];
#pragma unroll
    for (int j = 0; j < N; j++) w[j] = b[k][j];
    const float d = b[k][k];
    const float p = recip(d);
    dv[k] = d;
    ps[k] = p;
    c[k] = 0.0f;
    w[k] = 1.0f;
#pragma unroll
    for (int i = 0; i < N; i++) b[i][k] = 0.0f;
    b[k][k] = 1.0f;
#pragma unroll
    for (int i = 0; i < N; i++) {
        const float m = c[i] * p;
#pragma unroll
        for (int j = 0; j < N; j++) b[i][j] = fmaf(-m, w[j], b[i][j]);
    }
}

// Partial pivoting step (as gj_step_partial): argmax of |column k| over rows
// k.. (first maximum; a NaN never beats a number), rows k and r exchanged,
// then the step.  ra[s] = input row at logical row s.
template <int N>
__device__ __forceinline__ void tiny_step_partial(float (&b)[N][N], float (&ps)[N], float (&dv)[N], int (&ra)[N],
                                                  const int k) {
    unsigned best = 0u;
    int r = k;
#pragma unroll
    for (int s = k; s < N; s++) {
        const unsigned bits = __float_as_uint(b[s][k]) & 0x7fffffffu;
        const unsigned key = (bits > 0x7f800000u) ? 1u : bits + 2u;
        if (key > best) {
            best = key;
            r = s;
        }
    }
    // exchange rows k and r with selects (r is a runtime value)
#pragma unroll
    for (int j = 0; j < N; j++) {
        const float bk = b[k][j];
        float nk = bk;
#pragma unroll
        for (int s = k + 1; s < N; s++) {
            const bool hit = (r == s);
            nk = hit ? b[s][j] : nk;
            b[s][j] = hit ? bk : b[s][j];
        }
        b[k][j] = nk;
    }
    {
        const int rk = ra[k];
        int nk = rk;
#pragma unroll
        for (int s = k + 1; s < N; s++) {
            const bool hit = (r == s);
            nk = hit ? ra[s] : nk;
            ra[s] = hit ? rk : ra[s];
        }
        ra[k] = nk;
    }
    tiny_step<N>(b, ps, dv, k);
}

// Invert one matrix in registers.  a: rows as loaded; on return b holds the
// scaled inverse of the pivot-ordered matrix, win the pivot order, info the
// first exactly-zero pivot (1-based) or 0.
template <int N, int MODE>
__device__ __forceinline__ void tiny_invert(const float (&a)[N][N], float (&b)[N][N], int (&win)[N], int& info) {
    if constexpr (MODE == kModeReference || MODE == kModeReferenceSerial) {
        tiny_pivots<N, MODE>(a, win);
#pragma unroll
        for (int i = 0; i < N; i++)
#pragma unroll
            for (int j = 0; j < N; j++) b[i][j] = tiny_get<N>(a, win[i], j);
    } else {
#pragma unroll
        for (int i = 0; i < N; i++) {
            win[i] = i;
#pragma unroll
            for (int j = 0; j < N; j++) b[i][j] = a[i][j];
        }
    }
    float ps[N], dv[N];
#pragma unroll
    for (int k = 0; k < N; k++) {
        if constexpr (MODE == kModePartial) tiny_step_partial<N>(b, ps, dv, win, k);
        else tiny_step<N>(b, ps, dv, k);
    }
#pragma unroll
    for (int i = 0; i < N; i++)
#pragma unroll
        for (int j = 0; j < N; j++) b[i][j] = b[i][j] * ps[i];
    info = 0;
#pragma unroll
    for (int k = N - 1; k >= 0; k--)
        if (dv[k] == 0.0f) info = k + 1;
}

// n > 8: the matrix is read from and written back to this thread's
// shared-memory slot (row-major, pitch n), so the rows and columns chosen at
// run time (pivot order, output permutation) are addressed directly instead
// of through register select chains, which grow as n^3.  Same arithmetic as
// tiny_invert.
template <int N, int MODE>
__device__ __forceinline__ void tiny_invert_slot(float* sm, int (&win)[N], int& info) {
    float b[N][N];
    if constexpr (MODE == kModeReference || MODE == kModeReferenceSerial) {
        tiny_pivots_by<N, MODE>([&](int r, int c) { return sm[r * N + c]; }, win);
#pragma unroll
        for (int i = 0; i < N; i++) {
            const float* row = sm + win[i] * N;
#pragma unroll
            for (int j = 0; j < N; j++) b[i][j] = row[j];
        }
    } else {
#pragma unroll
        for (int i = 0; i < N; i++) {
            win[i] = i;
#pragma unroll
            for (int j = 0; j < N; j++) b[i][j] = sm[i * N + j];
        }
    }
    float ps[N], dv[N];
#pragma unroll
    for (int k = 0; k < N; k++) {
        if constexpr (MODE == kModePartial) tiny_step_partial<N>(b, ps, dv, win, k);
        else tiny_step<N>(b, ps, dv, k);
    }
    info = 0;
#pragma unroll
    for (int k = N - 1; k >= 0; k--)
        if (dv[k] == 0.0f) info = k + 1;
    // A^-1[i][win[j]] = b[i][j] * ps[i]
#pragma unroll
    for (int i = 0; i < N; i++) {
        float* row = sm + i * N;
#pragma unroll
        for (int j = 0; j < N; j++) row[win[j]] = b[i][j] * ps[i];
    }
}

template <int N>
__device__ __forceinline__ void tiny_load(const float* src, float (&a)[N][N]) {
    if constexpr ((N * N) % 4 == 0) {
        // n * n a multiple of 4: 16-byte aligned whenever the batch is (the launcher checks)
        const float4* s4 = reinterpret_cast<const float4*>(src);
#pragma unroll
        for (int q = 0; q < N * N / 4; q++) {
            const float4 v = s4[q];
            const float t[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int e = 0; e < 4; e++) a[(4 * q + e) / N][(4 * q + e) % N] = t[e];
        }
    } else {
#pragma unroll
        for (int e = 0; e < N * N; e++) a[e / N][e % N] = src[e];
    }
}

// Store with the column permutation A^-1[i][win[j]] = b[i][j].
template <int N>
__device__ __forceinline__ void tiny_store(float* dst, const float (&b)[N][N], const int (&win)[N], bool vec) {
    float o[N][N];
#pragma unroll
    for (int i = 0; i < N; i++)
#pragma unroll
        for (int c = 0; c < N; c++) {
            float v = b[i][0];
#pragma unroll
            for (int j = 1; j < N; j++)
                if (win[j] == c) v = b[i][j];
            o[i][c] = v;
        }
    if constexpr ((N * N) % 4 == 0) {
        if (vec) {
            float4* d4 = reinterpret_cast<float4*>(dst);
#pragma unroll
            for (int q = 0; q < N * N / 4; q++) {
                const int e = 4 * q;
                d4[q] = make_float4(o[e / N][e % N], o[(e + 1) / N][(e + 1) % N], o[(e + 2) / N][(e + 2) % N],
                                    o[(e + 3) / N][(e + 3) % N]);
            }
            return;
        }
    }
#pragma unroll
    for (int e = 0; e < N * N; e++) dst[e] = o[e / N][e % N];
}

// Contiguous batch, one matrix per thread.  n = 2: each thread moves its
// matrix with 16-byte loads and stores (16-byte-aligned batch) and inverts it
// in registers.  n = 1 and n >= kTinySlotMin: each warp's 32 consecutive
// matrices move between global and shared memory with coalesced copies and
// each thread works on its own matrix there at an odd pitch (conflict-free);
// from n = 3 up that slot is also where the row order and the column
// permutation are addressed (tiny_invert_slot).
template <int N>
__host__ __device__ constexpr int tiny_warps() { return N <= 8 ? 4 : (N <= 13 ? 2 : 1); }   // static staging <= 48 KB
template <int N>
__host__ __device__ constexpr int tiny_threads() { return 32 * tiny_warps<N>(); }

template <int N>
__host__ __device__ constexpr int tiny_pitch() { return (N * N) | 1; }

template <int N, int MODE>
__global__ void __launch_bounds__(tiny_threads<N>()) mi_tiny_kernel(float* __restrict__ A, int32_t* __restrict__ perm_out,
                                                                   int32_t* __restrict__ info_out, long long batch,
                                                                   int vec) {
    constexpr int NN = N * N, P = tiny_pitch<N>(), W = tiny_warps<N>();
    if constexpr (NN % 4 == 0 && N < kTinySlotMin) {
        for (long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x; b < batch;
             b += (long long)gridDim.x * blockDim.x) {
            float a[N][N], x[N][N];
            float* src = A + b * NN;
            if (vec) tiny_load<N>(src, a);
            else {
#pragma unroll
                for (int e = 0; e < NN; e++) a[e / N][e % N] = src[e];
            }
            int win[N], info;
            tiny_invert<N, MODE>(a, x, win, info);
            tiny_store<N>(src, x, win, vec != 0);
            if (perm_out != nullptr) {
#pragma unroll
                for (int i = 0; i < N; i++) perm_out[b * N + i] = win[i];
            }
            if (info_out != nullptr) info_out[b] = info;
        }
        return;
    }
    __shared__ float stage[W][32 * P];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float* st = stage[warp];
    const long long wstride = (long long)gridDim.x * W * 32;
    for (long long b0 = ((long long)blockIdx.x * W + warp) * 32; b0 < batch; b0 += wstride) {
        const int cnt = (batch - b0 < 32) ? (int)(batch - b0) : 32;
        float* g = A + b0 * NN;
        if (N >= kTinySlotMin && cnt == 32) {
            // a full group: every copy in flight at once (element e of the
            // group goes to slot e / NN at pitch P)
#pragma unroll
            for (int q = 0; q < NN; q++) {
                const int e = lane + 32 * q;
                cp_async_4(st + e + (P - NN) * (e / NN), g + e, true);
            }
            cp_async_commit();
            cp_async_wait_all();
        } else {
            for (int e = lane; e < cnt * NN; e += 32) st[(e / NN) * P + (e % NN)] = g[e];
        }
        __syncwarp();
        const bool mine = lane < cnt;
        int win[N], info = 0;
        if (mine) {
            float* sm = st + lane * P;
            if constexpr (N >= kTinySlotMin) {
                tiny_invert_slot<N, MODE>(sm, win, info);
            } else {
                float a[N][N], x[N][N];
#pragma unroll
                for (int e = 0; e < NN; e++) a[e / N][e % N] = sm[e];
                tiny_invert<N, MODE>(a, x, win, info);
                tiny_store<N>(sm, x, win, false);
            }
        }
        __syncwarp();
        if (N >= kTinySlotMin && cnt == 32) {
#pragma unroll
            for (int q = 0; q < NN; q++) {
                const int e = lane + 32 * q;
                g[e] = st[e + (P - NN) * (e / NN)];
            }
        } else {
            for (int e = lane; e < cnt * NN; e += 32) g[e] = st[(e / NN) * P + (e % NN)];
        }
        if (mine) {
            const long long b = b0 + lane;
            if (perm_out != nullptr) {
#pragma unroll
                for (int i = 0; i < N; i++) perm_out[b * N + i] = win[i];
            }
            if (info_out != nullptr) info_out[b] = info;
        }
        __syncwarp();
    }
}

// One matrix of a descriptor bucket in registers (n = 1, 2): descriptor
// index idx at base + offsets[idx].
template <int N, int MODE>
__device__ __forceinline__ void tiny_indexed_one(float* __restrict__ base, const long long* __restrict__ offsets,
                                                 int idx, int32_t* __restrict__ perm_out,
                                                 int32_t* __restrict__ info_out) {
    float* src = base + offsets[idx];
    float a[N][N], x[N][N];
#pragma unroll
    for (int e = 0; e < N * N; e++) a[e / N][e % N] = src[e];
    int win[N], info;
    tiny_invert<N, MODE>(a, x, win, info);
    tiny_store<N>(src, x, win, false);
    if (perm_out != nullptr) {
#pragma unroll
        for (int i = 0; i < N; i++) perm_out[(long long)idx * 32 + i] = win[i];
    }
    if (info_out != nullptr) info_out[idx] = info;
}

// Descriptor bucket: list[range[0] .. range[0] + range[1]) at base + offsets[i].
template <int N, int MODE>
__global__ void __launch_bounds__(256) mi_tiny_indexed_kernel(float* __restrict__ base,
                                                              const long long* __restrict__ offsets,
                                                              const int* __restrict__ list,
                                                              const long long* __restrict__ range,
                                                              int32_t* __restrict__ perm_out,
                                                              int32_t* __restrict__ info_out) {
    const long long start = range[0], count = range[1];
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < count;
         t += (long long)gridDim.x * blockDim.x)
        tiny_indexed_one<N, MODE>(base, offsets, list[start + t], perm_out, info_out);
}

// One warp's walk over the groups g, g + gstride, ... (< g_end) of 32 list
// entries of a bucket (lane = entry), n = 1, 2.
template <int N, int MODE>
__device__ __forceinline__ void tiny_indexed_walk(int lane, float* __restrict__ base,
                                                  const long long* __restrict__ offsets, const int* __restrict__ list,
                                                  long long start, long long count, long long g, long long g_end,
                                                  long long gstride, int32_t* __restrict__ perm_out,
                                                  int32_t* __restrict__ info_out) {
    for (; g < g_end; g += gstride) {
        const long long t = g * 32 + lane;
        if (t < count) tiny_indexed_one<N, MODE>(base, offsets, list[start + t], perm_out, info_out);
    }
}

template <int N>
__host__ __device__ constexpr int tiny_slot_floats() { return 32 * tiny_pitch<N>(); }

// One warp's walk over the groups g, g + gstride, ... (< g_end) of 32 list
// entries of a bucket through its stage `st` (tiny_slot_floats<N>() floats):
// the matrices arrive one after another as coalesced 4-byte copies of their
// n * n floats into the slots (pitch P), every copy in flight before the
// wait, and leave the same way after each thread has inverted its slot.
template <int N, int MODE>
__device__ __forceinline__ void tiny_slot_walk(float* st, int lane, float* __restrict__ base,
                                               const long long* __restrict__ offsets, const int* __restrict__ list,
                                               long long start, long long count, long long g, long long g_end,
                                               long long gstride, int32_t* __restrict__ perm_out,
                                               int32_t* __restrict__ info_out) {
    constexpr int NN = N * N, P = tiny_pitch<N>();
    constexpr int Q = (NN + 31) / 32;                   // copies per lane per matrix
    for (; g < g_end; g += gstride) {
        const long long t0 = g * 32;
        const long long t = t0 + lane;
        const bool mine = t < count;
        const int idx = mine ? list[start + t] : 0;
        const long long off = mine ? offsets[idx] : 0;
        const int cnt = (count - t0 < 32) ? (int)(count - t0) : 32;
        for (int m = 0; m < cnt; m++) {
            const float* src = base + __shfl_sync(kFull, off, m);
#pragma unroll
            for (int q = 0; q < Q; q++) {
                const int e = lane + 32 * q;
                if (e < NN) cp_async_4(st + m * P + e, src + e, true);
            }
        }
        cp_async_commit();
        cp_async_wait_all();
        __syncwarp();
        int win[N], info = 0;
        if (mine) tiny_invert_slot<N, MODE>(st + lane * P, win, info);
        __syncwarp();
        for (int m = 0; m < cnt; m++) {
            float* dst = base + __shfl_sync(kFull, off, m);
#pragma unroll
            for (int q = 0; q < Q; q++) {
                const int e = lane + 32 * q;
                if (e < NN) dst[e] = st[m * P + e];
            }
        }
        if (mine) {
            if (perm_out != nullptr) {
#pragma unroll
                for (int i = 0; i < N; i++) perm_out[(long long)idx * 32 + i] = win[i];
            }
            if (info_out != nullptr) info_out[idx] = info;
        }
        __syncwarp();
    }
}

// Descriptor bucket, n > 8: each warp takes 32 list entries at a time
// (tiny_slot_walk).
template <int N, int MODE>
__global__ void __launch_bounds__(tiny_threads<N>()) mi_tiny_slot_indexed_kernel(float* __restrict__ base,
                                                                                const long long* __restrict__ offsets,
                                                                                const int* __restrict__ list,
                                                                                const long long* __restrict__ range,
                                                                                int32_t* __restrict__ perm_out,
                                                                                int32_t* __restrict__ info_out) {
    constexpr int W = tiny_warps<N>();
    __shared__ float stage[W][tiny_slot_floats<N>()];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long start = range[0], count = range[1];
    tiny_slot_walk<N, MODE>(stage[warp], lane, base, offsets, list, start, count, (long long)blockIdx.x * W + warp,
                            (count + 31) / 32, (long long)gridDim.x * W, perm_out, info_out);
}

template <int N, int MODE>
cudaError_t launch_tiny(float* a, int32_t* perm, int32_t* info, long long batch, int /*tpb*/, int grid,
                        cudaStream_t stream) {
    static_assert(N <= kTinySlotMax, "one thread per matrix up to kTinySlotMax");
    // the block size is fixed by the static staging buffer
    constexpr int threads = tiny_threads<N>();
    if (grid <= 0) {
        const long long per_block = threads;           // one matrix per thread
        const long long need = (batch + per_block - 1) / per_block;
        long long cap = 16LL * device_sm_count();
        if constexpr (N >= kTinySlotMin) {              // as many blocks as are resident
            static int per_sm = 0;
            if (per_sm == 0) {
                cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mi_tiny_kernel<N, MODE>,
                                                                              threads, 0);
                if (e != cudaSuccess) return e;
                if (per_sm < 1) per_sm = 1;
            }
            cap = (long long)per_sm * device_sm_count();
        }
        grid = (int)(need < cap ? need : cap);
    }
    if (grid < 1) grid = 1;
    const int vec = ((N * N) % 4 == 0 && (reinterpret_cast<uintptr_t>(a) & 15u) == 0) ? 1 : 0;
    mi_tiny_kernel<N, MODE><<<grid, threads, 0, stream>>>(a, perm, info, batch, vec);
    return cudaGetLastError();
}

template <int N, int MODE>
cudaError_t launch_tiny_indexed(float* base, const long long* offsets, const int* list, const long long* range,
                                int32_t* perm, int32_t* info, int tpb, int grid, cudaStream_t stream) {
    if constexpr (N >= kTinySlotMinIndexed) {
        static_assert(N <= kTinySlotMax, "one thread per matrix up to kTinySlotMax");
        // persistent warps, as many blocks as are resident (the bucket size is
        // known only on the device)
        constexpr int threads = tiny_threads<N>();
        if (grid <= 0) {
            static int per_sm = 0;
            if (per_sm == 0) {
                cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                    &per_sm, mi_tiny_slot_indexed_kernel<N, MODE>, threads, 0);
                if (e != cudaSuccess) return e;
                if (per_sm < 1) per_sm = 1;
            }
            grid = per_sm * device_sm_count();
        }
        mi_tiny_slot_indexed_kernel<N, MODE><<<grid, threads, 0, stream>>>(base, offsets, list, range, perm, info);
        return cudaGetLastError();
    } else {
        if (grid <= 0) grid = 16 * device_sm_count();
        mi_tiny_indexed_kernel<N, MODE><<<grid, tpb, 0, stream>>>(base, offsets, list, range, perm, info);
        return cudaGetLastError();
    }
}

// Largest n of a descriptor bucket inverted one thread per matrix (measured:
// 1,000,000 mixed matrices, n ~ U{2..32}, graph-captured call 2.03 -> 1.98 ms
// with the slot form for n = 9..15; same bits as the contiguous call).
template <int MODE>
__host__ __device__ constexpr int tiny_max_indexed() { return 15; }

}  // namespace mi
