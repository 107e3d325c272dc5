// mi_kernel.cuh -- batched in-place inverse of n x n FP32 matrices (n <= 32)
// for sm_103a.
//
// Method (the reference's: LU with optional row pivoting, then the inverse
// from the triangular factors and the row permutation), scheduled for a GPU
// warp instead of the reference's shared-memory Doolittle sweep
// (parallel_pivot/luBatchedInplace.cuh:127-199):
//
//   * One sub-warp of L lanes (4/8/16/32, by n) owns a matrix; a warp holds
//     32/L matrices.  Lane (rg, cg) keeps an R x C register block of the
//     matrix (rows rg*R.., columns cg*C..), so every step is register FMAs.
//   * Step k applies the k-th LU elimination to the rows below the pivot and
//     the k-th triangular-inverse update to the rows above it, in the
//     product (Gauss-Jordan) form: a[i][j] -= (a[i][k]/a[k][k]) * a[k][j].
//     Below the pivot this is exactly the Schur-complement update of
//     right-looking LU, so pivot values, info and the partial-pivot argmax see
//     the same numbers as getrf; after n steps the block holds (PA)^-1 and
//     A^-1 = (PA)^-1 P is stored by permuting columns.  Each step is one full
//     rank-1 update (n^2 FMAs), n^3 FMAs in total = the 2n^3 flops of
//     getrf + getri, with no idle lanes on triangular shapes.
//   * The pivot row is kept unscaled (its diagonal set to 1) and every row is
//     scaled by its 1/pivot once at the end, so a step is: broadcast column k
//     and row k through shared memory, one reciprocal, 2 packed multiplies and
//     R*C/2 packed FMAs (fma.rn.f32x2).
//   * Pivoting:
//       reference         -- the reference's parallel-argmax rule
//                            (find_pivot_parallel, parallel_pivot/
//                            luBatchedInplace.cuh:12-44, T = n slots): it reads
//                            only raw input entries, so the whole pivot
//                            sequence is replayed first, lane = row, with
//                            warp max-reductions (ties broken in the tree's
//                            own order), and the rows are then loaded in
//                            pivot order.
//       reference_serial  -- serial_pivot's sequential argmax
//                            (serial_pivot/luBatchedInplace.cuh:22-36).
//       partial           -- textbook partial pivoting on the updated column
//                            (getrf: first maximum, rows exchanged in place).
//       none              -- templated/luBatchedInplace.cuh:78-126's plain LU.
//   * Outputs: A^-1 in place, optional perm[b][i] (input row that ends at row
//     i, the reference's shared pivots[] array) and info[b] (0, or the 1-based
//     step of the first exactly-zero pivot, as getrf's info).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace mi {

enum : int { kModeNone = 0, kModeReference = 1, kModeReferenceSerial = 2, kModePartial = 3 };

constexpr unsigned kFull = 0xffffffffu;

// ---------------------------------------------------------------------------
// Geometry per matrix size.
// ---------------------------------------------------------------------------
template <int N>
struct Geom {
    static_assert(N >= 1 && N <= 32, "n must be in 1..32");
    static constexpr int L = N > 16 ? 32 : (N > 8 ? 16 : (N > 4 ? 8 : 4));  // lanes per matrix
    static constexpr int M = 32 / L;                                          // matrices per warp
    static constexpr int RG = (L == 32) ? 8 : (L == 16 ? 4 : (L == 8 ? 4 : 2));
    static constexpr int CG = L / RG;
    static constexpr int R = (N + RG - 1) / RG;                  // rows per lane
    static constexpr int C = (((N + CG - 1) / CG) + 1) & ~1;     // columns per lane (even)
    static constexpr int PR = R * RG;                             // padded rows
    static constexpr int PC = C * CG;                             // padded columns
    static constexpr int S = N + 1;                               // stage row stride
    static constexpr int pad4(int x) { return (x + 3) & ~3; }
    // per-matrix shared-memory regions (floats), each 16-byte aligned
    static constexpr int kStage = pad4(N * S);
    static constexpr int kCol = pad4(PR);
    static constexpr int kRow = pad4(PC + 1);   // row buffer + pivot value at [PC]
    static constexpr int kSwap = pad4(PC);
    static constexpr int kPerm = 32;
    static constexpr int kPerMatrix = kStage + 2 * kCol + 2 * kRow + 2 * kSwap + kPerm;
    static constexpr int kPerWarp = M * kPerMatrix;               // floats
};

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

__constant__ PrioTable c_prio = make_prio_table();

// ---------------------------------------------------------------------------
// Small helpers.
// ---------------------------------------------------------------------------
template <int L>
__device__ __forceinline__ unsigned sub_max(unsigned x) {
    if constexpr (L == 32) {
        return __reduce_max_sync(kFull, x);
    } else {
#pragma unroll
        for (int o = L / 2; o > 0; o >>= 1) x = max(x, __shfl_xor_sync(kFull, x, o));
        return x;
    }
}

template <int L>
__device__ __forceinline__ unsigned sub_ballot(bool p, int base) {
    unsigned b = __ballot_sync(kFull, p);
    if constexpr (L == 32) return b;
    else return (b >> base) & ((1u << L) - 1u);
}

// Pivot-compare key of one entry: |x| as ordered bits, subnormals flushed to
// zero (the reference compiles with --use_fast_math, parallel_pivot/run.py:47),
// NaN -> 0xffffffff (as a diagonal it blocks every swap; as a candidate it is
// rejected by the <= +inf test).
__device__ __forceinline__ unsigned pivot_key(float x) {
    unsigned a = __float_as_uint(x) & 0x7fffffffu;
    unsigned k = (a < 0x00800000u) ? 0u : a;
    return (a > 0x7f800000u) ? 0xffffffffu : k;
}

// 1/d: hardware approximation refined by one Newton-Raphson step
// (r' = r + r(1 - d r)); zero and infinite pivots keep the approximation.
__device__ __forceinline__ float recip(float d) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(d));
    float e = fmaf(-d, r, 1.0f);
    float r1 = fmaf(r, e, r);
    return (fabsf(r) == __int_as_float(0x7f800000) || d == 0.0f) ? r : r1;
}

template <int CNT>
__device__ __forceinline__ void lds_vec(const float* p, float (&v)[CNT]) {
    if constexpr (CNT % 4 == 0) {
#pragma unroll
        for (int q = 0; q < CNT / 4; q++) {
            float4 t = reinterpret_cast<const float4*>(p)[q];
            v[4 * q] = t.x; v[4 * q + 1] = t.y; v[4 * q + 2] = t.z; v[4 * q + 3] = t.w;
        }
    } else if constexpr (CNT % 2 == 0) {
#pragma unroll
        for (int q = 0; q < CNT / 2; q++) {
            float2 t = reinterpret_cast<const float2*>(p)[q];
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
        for (int q = 0; q < CNT / 2; q++)
            reinterpret_cast<float2*>(p)[q] = make_float2(v[2 * q], v[2 * q + 1]);
    } else {
#pragma unroll
        for (int q = 0; q < CNT; q++) p[q] = v[q];
    }
}

// a[ri][*] -= m * w[*] on packed pairs.
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
// Pivot replay for the reference rules, lane s = input row s.  Reads the raw
// input rows from the stage, returns the final position of this lane's row
// (positions follow the reference's physical row swaps).
// ---------------------------------------------------------------------------
template <int N, int MODE>
__device__ __forceinline__ int replay_pivots(const float* stage, int s, int base) {
    using G = Geom<N>;
    constexpr int L = G::L;
    constexpr unsigned kSurv = survive_mask(N);
    unsigned key[N];
#pragma unroll
    for (int k = 0; k < N; k++) key[k] = (s < N) ? pivot_key(stage[s * G::S + k]) : 0u;
    int pos = (s < N) ? s : 0x7fff;
#pragma unroll
    for (int k = 0; k < N; k++) {
        // key of the row now at position k (the diagonal candidate)
        const unsigned bd = sub_ballot<L>(pos == k, base);
        const int dl = __ffs(bd) - 1;
        const unsigned kd = __shfl_sync(kFull, key[k], base + dl);
        const int slot = pos - k - 1;
        bool ok = (slot >= 0) && (pos < N) && (key[k] > kd) && (key[k] <= 0x7f800000u);
        if constexpr (MODE == kModeReference) ok = ok && ((kSurv >> (slot & 31)) & 1u);
        const unsigned cand = ok ? key[k] : 0u;
        const unsigned mx = sub_max<L>(cand);
        const bool top = ok && (cand == mx);
        unsigned tb = sub_ballot<L>(top, base);
        if (__any_sync(kFull, __popc(tb) > 1)) {
            // equal keys: the reference tree keeps its own order; the serial
            // scan keeps the lowest position
            unsigned pr = 0u;
            if (top) pr = (MODE == kModeReference) ? (unsigned)c_prio.v[N][slot] : (unsigned)(64 - pos);
            const unsigned pm = sub_max<L>(pr);
            tb = sub_ballot<L>(top && pr == pm, base);
        }
        const int wl = __ffs(tb) - 1;
        const int pw = __shfl_sync(kFull, pos, base + (wl < 0 ? 0 : wl));
        if (wl >= 0) {
            if (s == wl) pos = k;
            else if (pos == k) pos = pw;
        }
    }
    return pos;
}

// ---------------------------------------------------------------------------
// One elimination step with the pivot row already at logical row k.
// ---------------------------------------------------------------------------
template <int N, int K>
struct StepConst {
    using G = Geom<N>;
    static constexpr int kr = K / G::R, kri = K % G::R;   // pivot-row owner, register row
    static constexpr int kc = K / G::C, kci = K % G::C;   // column owner, register column
};

template <int N, int K>
__device__ __forceinline__ void gj_step(float (&a)[Geom<N>::R][Geom<N>::C], float (&ps)[Geom<N>::R],
                                        int rg, int cg, float* colb, float* rowb, int& info) {
    using G = Geom<N>;
    using SC = StepConst<N, K>;
    constexpr int R = G::R, C = G::C;
    float* cb = colb + (K & 1) * G::kCol;
    float* rb = rowb + (K & 1) * G::kRow;
    if (cg == SC::kc) {
        float v[R];
#pragma unroll
        for (int ri = 0; ri < R; ri++) v[ri] = a[ri][SC::kci];
        if (rg == SC::kr) v[SC::kri] = 0.0f;          // the pivot row takes no update
        sts_vec<R>(cb + rg * R, v);
    }
    if (rg == SC::kr) {
        float w[C];
#pragma unroll
        for (int ci = 0; ci < C; ci++) w[ci] = a[SC::kri][ci];
        if (cg == SC::kc) {
            rb[G::PC] = w[SC::kci];                     // pivot value
            w[SC::kci] = 1.0f;                          // column k becomes -m_i
        }
        sts_vec<C>(rb + cg * C, w);
    }
    __syncwarp();
    const float d = rb[G::PC];
    const float p = recip(d);
    if (d == 0.0f && info == 0) info = K + 1;
    float c[R], w[C];
    lds_vec<R>(cb + rg * R, c);
    lds_vec<C>(rb + cg * C, w);
    if (cg == SC::kc) {
#pragma unroll
        for (int ri = 0; ri < R; ri++) a[ri][SC::kci] = (ri == SC::kri && rg == SC::kr) ? 1.0f : 0.0f;
    }
    if (rg == SC::kr) ps[SC::kri] = p;
    float m[R];
#pragma unroll
    for (int ri = 0; ri < R; ri += 2) {
        if (ri + 1 < R) {
            float2 mm = __fmul2_rn(make_float2(c[ri], c[ri + 1]), make_float2(p, p));
            m[ri] = mm.x;
            m[ri + 1] = mm.y;
        } else {
            m[ri] = c[ri] * p;
        }
    }
#pragma unroll
    for (int ri = 0; ri < R; ri++) row_update<C>(a[ri], m[ri], w);
}

// Partial pivoting step: argmax of the updated column over rows k.., swap the
// winner into row k (register blocks exchanged through shared memory), then
// the same update.  ra: the input row held at logical row s (lane s < N).
template <int N, int K>
__device__ __forceinline__ void gj_step_partial(float (&a)[Geom<N>::R][Geom<N>::C], float (&ps)[Geom<N>::R],
                                                int rg, int cg, int s, int base, float* colb, float* rowb,
                                                float* swapb, int& ra, int& info) {
    using G = Geom<N>;
    using SC = StepConst<N, K>;
    constexpr int R = G::R, C = G::C, L = G::L;
    float* cb = colb + (K & 1) * G::kCol;
    float* rb = rowb + (K & 1) * G::kRow;
    float* sb = swapb + (K & 1) * G::kSwap;
    if (cg == SC::kc) {
        float v[R];
#pragma unroll
        for (int ri = 0; ri < R; ri++) v[ri] = a[ri][SC::kci];
        sts_vec<R>(cb + rg * R, v);
    }
    __syncwarp();
    // argmax over logical rows k..N-1, first maximum (lowest row) wins
    unsigned key = 0u;
    if (s >= K && s < N) {
        unsigned b = __float_as_uint(cb[s]) & 0x7fffffffu;
        key = (b > 0x7f800000u) ? 1u : b + 2u;   // NaN never beats a number
    }
    const unsigned mx = sub_max<L>(key);
    const int r = __ffs(sub_ballot<L>(key != 0u && key == mx, base)) - 1;   // lane K is always a candidate
    const int rr = r / R, rri = r % R;
    // exchange rows K and r: row r -> rb (the pivot row), row K -> sb
    if (rg == rr) {
        float w[C];
#pragma unroll
        for (int q = 0; q < R; q++)
            if (q == rri) {
#pragma unroll
                for (int ci = 0; ci < C; ci++) w[ci] = a[q][ci];
            }
        sts_vec<C>(rb + cg * C, w);
    }
    if (rg == SC::kr) {
        float w[C];
#pragma unroll
        for (int ci = 0; ci < C; ci++) w[ci] = a[SC::kri][ci];
        sts_vec<C>(sb + cg * C, w);
    }
    __syncwarp();
    float w[C];
    lds_vec<C>(rb + cg * C, w);
    if (rg == SC::kr) {
#pragma unroll
        for (int ci = 0; ci < C; ci++) a[SC::kri][ci] = w[ci];
    }
    if (rg == rr && r != K) {
        float t[C];
        lds_vec<C>(sb + cg * C, t);
#pragma unroll
        for (int q = 0; q < R; q++)
            if (q == rri) {
#pragma unroll
                for (int ci = 0; ci < C; ci++) a[q][ci] = t[ci];
            }
    }
    const float d = cb[r];
    const float ck = cb[K];
    const float p = recip(d);
    if (d == 0.0f && info == 0) info = K + 1;
    {   // the input row held at each logical row follows the exchange
        const int a_r = __shfl_sync(kFull, ra, base + r);
        const int a_k = __shfl_sync(kFull, ra, base + K);
        if (s == K) ra = a_r;
        else if (s == r) ra = a_k;
    }
    if (cg == SC::kc) w[SC::kci] = 1.0f;
    float c[R];
    lds_vec<R>(cb + rg * R, c);
#pragma unroll
    for (int ri = 0; ri < R; ri++) {
        const int row = rg * R + ri;
        c[ri] = (row == K) ? 0.0f : ((row == r) ? ck : c[ri]);
    }
    if (cg == SC::kc) {
#pragma unroll
        for (int ri = 0; ri < R; ri++) a[ri][SC::kci] = (ri == SC::kri && rg == SC::kr) ? 1.0f : 0.0f;
    }
    if (rg == SC::kr) ps[SC::kri] = p;
#pragma unroll
    for (int ri = 0; ri < R; ri++) row_update<C>(a[ri], c[ri] * p, w);
}

template <int N, int K, int MODE>
struct Steps {
    static __device__ __forceinline__ void run(float (&a)[Geom<N>::R][Geom<N>::C], float (&ps)[Geom<N>::R],
                                               int rg, int cg, int s, int base, float* colb, float* rowb,
                                               float* swapb, int& ra, int& info) {
        if constexpr (K < N) {
            if constexpr (MODE == kModePartial)
                gj_step_partial<N, K>(a, ps, rg, cg, s, base, colb, rowb, swapb, ra, info);
            else
                gj_step<N, K>(a, ps, rg, cg, colb, rowb, info);
            Steps<N, K + 1, MODE>::run(a, ps, rg, cg, s, base, colb, rowb, swapb, ra, info);
        }
    }
};

// ---------------------------------------------------------------------------
// The kernel: a grid-stride loop of warps over groups of M matrices.
// ---------------------------------------------------------------------------
template <int N, int MODE>
__global__ void __launch_bounds__(256) mi_inverse_kernel(float* __restrict__ A, int32_t* __restrict__ perm_out,
                                                         int32_t* __restrict__ info_out, long long batch) {
    using G = Geom<N>;
    constexpr int L = G::L, M = G::M, R = G::R, C = G::C, S = G::S;
    constexpr int NN = N * N;
    extern __shared__ float4 smem_raw[];
    float* smem = reinterpret_cast<float*>(smem_raw);

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int w = lane / L;          // matrix slot within the warp
    const int s = lane % L;          // lane within the matrix
    const int base = w * L;
    const int rg = s % G::RG;
    const int cg = s / G::RG;

    float* wsm = smem + (size_t)warp * G::kPerWarp;
    float* msm = wsm + w * G::kPerMatrix;
    float* stage = msm;
    float* colb = stage + G::kStage;
    float* rowb = colb + 2 * G::kCol;
    float* swapb = rowb + 2 * G::kRow;
    int* permb = reinterpret_cast<int*>(swapb + 2 * G::kSwap);

    const long long ngroups = (batch + M - 1) / M;
    const long long gstride = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long grp = (long long)blockIdx.x * (blockDim.x >> 5) + warp; grp < ngroups; grp += gstride) {
        const long long first = grp * M;
        const int count = (int)min((long long)M, batch - first);
        const long long mb = first + w;
        const bool active = w < count;
        float* gA = A + first * NN;

        // ---- stage the warp's matrices into shared memory (row stride N+1)
#pragma unroll 4
        for (int e = lane; e < M * NN; e += 32) {
            const int m = e / NN, rem = e - m * NN;
            const int row = rem / N, col = rem - row * N;
            const float v = (m < count) ? gA[e] : 0.0f;
            wsm[m * G::kPerMatrix + row * S + col] = v;
        }
        __syncwarp();

        // ---- pivot order
        int ra = s;   // input row that ends at logical row s
        if constexpr (MODE == kModeReference || MODE == kModeReferenceSerial) {
            const int pos = replay_pivots<N, MODE>(stage, s, base);
            if (s < N) permb[pos] = s;
            __syncwarp();
            ra = (s < N) ? permb[s] : s;
        }

        // ---- register block, rows in pivot order
        float a[R][C];
#pragma unroll
        for (int ri = 0; ri < R; ri++) {
            const int i = rg * R + ri;
            int src = i;
            if constexpr (MODE == kModeReference || MODE == kModeReferenceSerial) src = (i < N) ? permb[i] : 0;
#pragma unroll
            for (int ci = 0; ci < C; ci++) {
                const int j = cg * C + ci;
                a[ri][ci] = (i < N && j < N) ? stage[src * S + j] : 0.0f;
            }
        }

        // ---- n elimination steps
        float ps[R];
#pragma unroll
        for (int ri = 0; ri < R; ri++) ps[ri] = 1.0f;
        int info = 0;
        Steps<N, 0, MODE>::run(a, ps, rg, cg, s, base, colb, rowb, swapb, ra, info);

        // ---- scale each row by its 1/pivot
#pragma unroll
        for (int ri = 0; ri < R; ri++) {
#pragma unroll
            for (int q = 0; q < C / 2; q++) {
                float2 x = __fmul2_rn(make_float2(a[ri][2 * q], a[ri][2 * q + 1]), make_float2(ps[ri], ps[ri]));
                a[ri][2 * q] = x.x;
                a[ri][2 * q + 1] = x.y;
            }
        }

        // ---- A^-1[i][ra(j)] = X[i][j]: scatter columns into the stage
        if constexpr (MODE == kModePartial) {
            if (s < N) permb[s] = ra;
        }
        __syncwarp();
#pragma unroll
        for (int ci = 0; ci < C; ci++) {
            const int j = cg * C + ci;
            if (j < N) {
                const int dst = (MODE == kModeNone) ? j : permb[j];
#pragma unroll
                for (int ri = 0; ri < R; ri++) {
                    const int i = rg * R + ri;
                    if (i < N) stage[i * S + dst] = a[ri][ci];
                }
            }
        }
        if (active) {
            if (perm_out != nullptr && s < N) perm_out[mb * N + s] = (MODE == kModeNone) ? s : permb[s];
            if (info_out != nullptr && s == 0) info_out[mb] = info;
        }
        __syncwarp();
#pragma unroll 4
        for (int e = lane; e < count * NN; e += 32) {
            const int m = e / NN, rem = e - m * NN;
            const int row = rem / N, col = rem - row * N;
            gA[e] = wsm[m * G::kPerMatrix + row * S + col];
        }
        __syncwarp();
    }
}

}  // namespace mi
