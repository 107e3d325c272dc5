// mi_refine_tc.cu -- one refinement step for listed 32 x 32 matrices with the
// residual R = I - A X formed exactly on the tensor cores:
//
//   * Error-free splitting (the scheme of Ozaki, Ogita, Oishi and Rump,
//     "Error-free transformations of matrix multiplication by using fast
//     routines of matrix multiplication and its applications", Numer.
//     Algorithms 59, 2012, restated here for bf16 tensor cores).  Row i of A
//     is scaled by 2^(8 - ea_i), the power of two that brings its largest
//     entry below 256, and cut into digits: digit s is the remainder rounded
//     to a multiple of 2^(-8s), an integer in [-256, 256] (s = 0) or in
//     [-128, 128] times 2^(-8s), so 8 significant bits, exact in bf16.
//     Column j of X likewise with 2^(8 - ex_j).  Scalings and cuts are exact.
//   * Digit products summed over k = 0..31 stay below 2^21 units of their
//     grid 2^(-8(s+t)), and a group d = s + t of at most six of them below
//     2^22 units: every group is an exact number in the FP32 accumulators of
//     mma.sync (bf16 inputs, FP32 accumulation), whatever order the tensor
//     core adds in.  (A X)_ij = 2^(ea_i + ex_j - 16) sum_d G_d[i][j], less the
//     groups left out; R = (delta_ij - s hi) - s lo, rounded once, with
//     s = 2^(ea_i + ex_j - 16) and hi + lo the float-float sum of the groups.
//   * Groups 0..4 leave out less than about 2^-37 of max_i,j |A_i.| |X_.j|
//     (rows and columns); where max|A| max|X| may reach 2^16 the matrix takes
//     group 5 too (a warp-uniform branch), so most matrices pay 15 digit
//     products and very ill-conditioned ones 21.  Only G0 + G1 carry the
//     cancellation of A X against I and are summed by TwoSum; the smaller
//     groups are added to the low part, which rounds at about 2^-40 of the
//     scale.
//   * X <- X + C, C = X R with X and R each split into two bf16 terms
//     (hi*hi + hi*lo + lo*hi, FP32 accumulation): C is small, so its 16 bits
//     of relative accuracy are plenty.
//   * Optionally (next != NULL) the error left after the step, estimated as
//     max|C R| / max|X| (one more bf16 product), lists the matrix for a second
//     step when it exceeds tol.
//
// One warp per matrix, four warps per block.  Digit tiles live in shared
// memory as 32 x 32 bf16 with 64-byte rows and the 16-byte chunk index XOR
// (row / 2) & 3, so the eight row reads of every ldmatrix hit distinct banks.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "mi_inverse.h"
#include "mi_ptx.cuh"

namespace mi {

int set_cuda_error(cudaError_t e, const char* what);   // mi_api.cu
int device_sm_count();

namespace tcr {

constexpr int kWarps = 4;                // matrices per block
constexpr int kDigits = 6;               // base-256 digits per operand
constexpr int kLowGroups = 5;            // groups every matrix takes
constexpr int kDeepExp = 16;             // group 5 too when max|A| max|X| may reach 2^kDeepExp
constexpr int kTile = 32 * 32 * 2;       // bytes of one 32 x 32 bf16 tile

struct WarpSmem {
    unsigned char ad[kDigits][kTile];    // digits of A ([i][k]); then X hi, X lo, C hi
    unsigned char xd[kDigits][kTile];    // digits of X ([k][j]); then R hi, R lo
    float sa[32], sx[32];                // 2^(ea_i - 8), 2^(ex_j - 8)
    float sia[32], six[32];              // their reciprocals
};

constexpr size_t smem_bytes() { return 128 + sizeof(WarpSmem) * kWarps; }

// byte offset of element (r, c) of a swizzled 32 x 32 bf16 tile
__device__ __forceinline__ uint32_t tofs(int r, int c) {
    return (uint32_t)(r * 64 + (((c >> 3) ^ ((r >> 1) & 3)) << 4) + (c & 7) * 2);
}

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t (&v)[4]) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3])
                 : "r"(addr));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t (&v)[4]) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3])
                 : "r"(addr));
}
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// d = A B with no accumulator input (C = 0)
__device__ __forceinline__ void mma_bf16_z(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    const float z = 0.0f;
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%10,%10,%10,%10};"
        : "=f"(d[0]), "=f"(d[1]), "=f"(d[2]), "=f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1), "f"(z));
}

typedef float Frag[2][4][4];             // a lane's share of a 32 x 32 FP32 accumulator

// acc (+)= A_tile * B_tile, both swizzled 32 x 32 bf16 tiles in shared
// memory, A row-major [i][k], B row-major [k][j]; kInit: acc = the product
// (its old value is not read).
template <bool kInit = false>
__device__ __forceinline__ void tile_mma(Frag& acc, uint32_t a, uint32_t b, int lane) {
    const int q = lane >> 3, r8 = lane & 7;
#pragma unroll
    for (int kc = 0; kc < 2; kc++) {
        uint32_t af[2][4];
#pragma unroll
        for (int mt = 0; mt < 2; mt++) ldsm_x4(a + tofs(16 * mt + r8 + (q & 1) * 8, 16 * kc + (q >> 1) * 8), af[mt]);
#pragma unroll
        for (int np = 0; np < 2; np++) {
            uint32_t bf[4];
            ldsm_x4_t(b + tofs(16 * kc + r8 + (q & 1) * 8, 16 * np + (q >> 1) * 8), bf);
#pragma unroll
            for (int mt = 0; mt < 2; mt++) {
                if (kInit && kc == 0) {
                    mma_bf16_z(acc[mt][2 * np], af[mt], bf[0], bf[1]);
                    mma_bf16_z(acc[mt][2 * np + 1], af[mt], bf[2], bf[3]);
                } else {
                    mma_bf16(acc[mt][2 * np], af[mt], bf[0], bf[1]);
                    mma_bf16(acc[mt][2 * np + 1], af[mt], bf[2], bf[3]);
                }
            }
        }
    }
}

// acc = group d: the sum over u = 0..d of A digit u times X digit d - u
__device__ __forceinline__ void group_sum(Frag& acc, uint32_t ad0, uint32_t xd0, int d, int lane) {
    tile_mma<true>(acc, ad0, xd0 + d * kTile, lane);
#pragma unroll 1
    for (int u = 1; u <= d; u++) tile_mma(acc, ad0 + u * kTile, xd0 + (d - u) * kTile, lane);
}

__device__ __forceinline__ void zero(Frag& acc) {
#pragma unroll
    for (int mt = 0; mt < 2; mt++)
#pragma unroll
        for (int nt = 0; nt < 4; nt++)
#pragma unroll
            for (int e = 0; e < 4; e++) acc[mt][nt][e] = 0.0f;
}

// element e of accumulator tile (mt, nt) of this lane: row, column
__device__ __forceinline__ int erow(int mt, int e, int lane) { return 16 * mt + (lane >> 2) + ((e >> 1) << 3); }
__device__ __forceinline__ int ecol(int nt, int e, int lane) { return 8 * nt + 2 * (lane & 3) + (e & 1); }

__device__ __forceinline__ uint32_t bf2_bits(__nv_bfloat162 v) { return *reinterpret_cast<const uint32_t*>(&v); }

__device__ __forceinline__ void put_bf16x2(unsigned char* tile, int r, int c, float v0, float v1) {
    *reinterpret_cast<__nv_bfloat162*>(tile + tofs(r, c)) = __floats2bfloat162_rn(v0, v1);
}

__device__ __forceinline__ uint32_t bf2_of(float2 v) { return bf2_bits(__floats2bfloat162_rn(v.x, v.y)); }

__device__ __forceinline__ float2 neg2(float2 v) { return make_float2(-v.x, -v.y); }

// 2^k for |k| <= 126, by its bits
__device__ __forceinline__ float pow2(int k) { return __int_as_float((127 + k) << 23); }

// 1.5 * 2^(23 - 8s): adding and subtracting it rounds to a multiple of 2^(-8s)
__host__ __device__ constexpr float magic(int s) {
    return s == 0 ? 12582912.0f : s == 1 ? 49152.0f : s == 2 ? 192.0f : s == 3 ? 0.75f
         : s == 4 ? 0.0029296875f : 1.1444091796875e-05f;
}

// (hi, lo) += p by Knuth's TwoSum on packed pairs; hi + p = s + r exactly
__device__ __forceinline__ void two_sum2(float2& hi, float2& lo, float2 p) {
    const float2 s = __fadd2_rn(hi, p);
    const float2 z = __fadd2_rn(s, neg2(hi));
    const float2 r = __fadd2_rn(__fadd2_rn(hi, neg2(__fadd2_rn(s, neg2(z)))), __fadd2_rn(p, neg2(z)));
    hi = s;
    lo = __fadd2_rn(lo, r);
}

// exponent e with |max| < 2^e (0 for 0), kept within [-100, 120] so that the
// scale 2^(e - 8) and its reciprocal stay normal FP32 numbers
__device__ __forceinline__ int line_exp(float mx) {
    int e = 0;
    frexpf(mx, &e);
    return e < -100 ? -100 : (e > 120 ? 120 : e);
}

// Work item t: the list's entry, or t itself when the kernel walks the whole
// batch (list == NULL); -1 past the end.  Lane 0 alone reads the list.
__device__ __forceinline__ long long work_item(const int32_t* list, long long t, long long count, int lane) {
    if (t >= count) return -1;
    if (list == nullptr) return t;
    return __shfl_sync(0xffffffffu, lane == 0 ? (long long)list[t] : 0LL, 0);
}

// a 32 x 32 FP32 matrix, lane's share in row order: row 4q + lane / 8,
// columns 4 (lane & 7) .. + 3
__device__ __forceinline__ void load_rows(float4 (&v)[8], const float* m, int lane) {
#pragma unroll
    for (int q = 0; q < 8; q++) v[q] = reinterpret_cast<const float4*>(m)[lane + 32 * q];
}

// float index of (r, c) in a swizzled 32 x 32 FP32 tile: fragment-order
// float2 writes and row-order float4 reads are both free of bank conflicts
__device__ __forceinline__ int fofs(int r, int c) { return r * 32 + (c ^ ((r & 7) << 2)); }

// max_j sum_i |M_ij| over the warp's row-order share (the same value in every lane)
__device__ __forceinline__ float norm1(const float4 (&v)[8]) {
    float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int q = 0; q < 8; q++) {
        c[0] += fabsf(v[q].x);
        c[1] += fabsf(v[q].y);
        c[2] += fabsf(v[q].z);
        c[3] += fabsf(v[q].w);
    }
    float m = 0.0f;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        c[k] += __shfl_xor_sync(0xffffffffu, c[k], 8);
        c[k] += __shfl_xor_sync(0xffffffffu, c[k], 16);
        m = k == 0 ? c[0] : fmaxf(m, c[k]);
    }
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    return m;
}

}  // namespace tcr

// kFlag: walk the whole batch and refine only the matrices whose condition
// estimate ||A||_1 ||X||_1 is at least `flag` (or not finite); otherwise
// refine the listed matrices.  The next matrix's A is loaded while the digit
// products run, its X once this one's X is written.
template <bool kFlag>
__global__ void __launch_bounds__(32 * tcr::kWarps) mi_refine_tc_kernel(const float* __restrict__ A, float* X,
                                                                        const int32_t* list, long long count,
                                                                        long long batch, float flag, float tol,
                                                                        int32_t* next) {
    using namespace tcr;
    extern __shared__ unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    WarpSmem& sm = reinterpret_cast<WarpSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~(uintptr_t)127)[warp];
    const uint32_t ad0 = smem_addr(sm.ad[0]), xd0 = smem_addr(sm.xd[0]);
    const long long stride = (long long)gridDim.x * kWarps;
    long long t = (long long)blockIdx.x * kWarps + warp;
    // lane 0 alone reads list[t] and writes next[t], and it reads list[t]
    // before it writes next[t], so the two may be one array
    long long b = work_item(list, t, count, lane);
    bool live = b >= 0 && b < batch;                      // out-of-range entries are skipped
    float4 va[8], vx[8];
    if (live) {
        load_rows(va, A + b * 1024, lane);
        load_rows(vx, X + b * 1024, lane);
    }
    for (; t < count; t += stride) {
        const long long bn = work_item(list, t + stride, count, lane);
        const bool live_n = bn >= 0 && bn < batch;
        bool run = live;
        if (kFlag && run) run = __shfl_sync(0xffffffffu, !(norm1(va) * norm1(vx) < flag), 0);
        if (!run) {
            if (next != nullptr && lane == 0) next[t] = -1;
            if (live_n) {
                load_rows(va, A + bn * 1024, lane);
                load_rows(vx, X + bn * 1024, lane);
            }
            b = bn;
            live = live_n;
            continue;
        }
        // exponents: rows of A (8 lanes share a row), columns of X (lanes
        // lane, lane ^ 8, ^ 16, ^ 24 share 4 columns, 8 rows each)
        float cm[4] = {0.f, 0.f, 0.f, 0.f};
        int ea_max = -1000;
#pragma unroll
        for (int q = 0; q < 8; q++) {
            float rm = fmaxf(fmaxf(fabsf(va[q].x), fabsf(va[q].y)), fmaxf(fabsf(va[q].z), fabsf(va[q].w)));
#pragma unroll
            for (int o = 1; o < 8; o <<= 1) rm = fmaxf(rm, __shfl_xor_sync(0xffffffffu, rm, o));
            const int e = line_exp(rm);
            ea_max = max(ea_max, e);
            if ((lane & 7) == 0) {
                sm.sa[4 * q + (lane >> 3)] = pow2(e - 8);
                sm.sia[4 * q + (lane >> 3)] = pow2(8 - e);
            }
            cm[0] = fmaxf(cm[0], fabsf(vx[q].x));
            cm[1] = fmaxf(cm[1], fabsf(vx[q].y));
            cm[2] = fmaxf(cm[2], fabsf(vx[q].z));
            cm[3] = fmaxf(cm[3], fabsf(vx[q].w));
        }
        int ex_max = -1000;
#pragma unroll
        for (int c = 0; c < 4; c++) {
            cm[c] = fmaxf(cm[c], __shfl_xor_sync(0xffffffffu, cm[c], 8));
            cm[c] = fmaxf(cm[c], __shfl_xor_sync(0xffffffffu, cm[c], 16));
            const int e = line_exp(cm[c]);
            ex_max = max(ex_max, e);
            if (lane < 8) {
                sm.sx[4 * lane + c] = pow2(e - 8);
                sm.six[4 * lane + c] = pow2(8 - e);
            }
        }
        // lanes hold rows of A in groups of 8 (lane / 8) and columns of X in
        // groups of 4 (lane & 7): reduce both maxima over the whole warp
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            ea_max = max(ea_max, __shfl_xor_sync(0xffffffffu, ea_max, o));
            ex_max = max(ex_max, __shfl_xor_sync(0xffffffffu, ex_max, o));
        }
        // the digit and group counts must be the same in every lane (mma.sync
        // and ldmatrix are warp-collective): the vote makes them so by construction
        const bool deep = __any_sync(0xffffffffu, ea_max + ex_max >= kDeepExp);
        const int ndig = deep ? kDigits : kLowGroups;
        __syncwarp();
        // digits: v = M 2^(8 - e) (exact, |v| < 256); digit s is the remainder
        // rounded to a multiple of 2^(-8s) by adding and subtracting
        // 1.5 * 2^(23 - 8s) (|remainder| < 2^(22 - 8s), so the sum stays in
        // the binade whose unit is 2^(-8s)), then taken off the remainder,
        // exactly.  Digit 0 is an integer in [-256, 256], digit s >= 1 an
        // integer in [-128, 128] times 2^(-8s): 8 significant bits, exact in
        // bf16.  Rows and columns in pairs on packed FP32x2 arithmetic.
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int r = 4 * q + (lane >> 3), c0 = 4 * (lane & 7);
            const float ia = sm.sia[r];
            const float2 ia2 = make_float2(ia, ia);
            float2 v01 = __fmul2_rn(make_float2(va[q].x, va[q].y), ia2);
            float2 v23 = __fmul2_rn(make_float2(va[q].z, va[q].w), ia2);
            float2 w01 = __fmul2_rn(make_float2(vx[q].x, vx[q].y), *reinterpret_cast<const float2*>(&sm.six[c0]));
            float2 w23 = __fmul2_rn(make_float2(vx[q].z, vx[q].w), *reinterpret_cast<const float2*>(&sm.six[c0 + 2]));
#pragma unroll
            for (int s = 0; s < kDigits; s++) {
                if (s >= ndig) break;
                const float2 c2 = make_float2(magic(s), magic(s)), n2 = make_float2(-magic(s), -magic(s));
                const float2 a01 = __fadd2_rn(__fadd2_rn(v01, c2), n2), a23 = __fadd2_rn(__fadd2_rn(v23, c2), n2);
                const float2 x01 = __fadd2_rn(__fadd2_rn(w01, c2), n2), x23 = __fadd2_rn(__fadd2_rn(w23, c2), n2);
                if (s + 1 < kDigits) {
                    v01 = __fadd2_rn(v01, neg2(a01));
                    v23 = __fadd2_rn(v23, neg2(a23));
                    w01 = __fadd2_rn(w01, neg2(x01));
                    w23 = __fadd2_rn(w23, neg2(x23));
                }
                *reinterpret_cast<uint2*>(sm.ad[s] + tofs(r, c0)) = make_uint2(bf2_of(a01), bf2_of(a23));
                *reinterpret_cast<uint2*>(sm.xd[s] + tofs(r, c0)) = make_uint2(bf2_of(x01), bf2_of(x23));
            }
        }
        __syncwarp();
        if (live_n) load_rows(va, A + bn * 1024, lane);   // in flight during the products
        // the sum of the groups in float-float, element pairs of the fragments
        // on packed FP32x2 arithmetic (in units of the row's and column's
        // scales).  G0 and G1 (below 2^22 units, exact) carry the cancellation
        // of A X against I: TwoSum(G0, G1) = hi + lo exactly.  G2 (exact,
        // below 2^6 units) is added to lo (rounding at 2^-18 units, about
        // 2^-40 of the scale), and the groups from 3 up (below 2^-2 units)
        // share one accumulator, whose additions round at 2^-26 units or less.
        float2 hi[2][4][2], lo[2][4][2];
        Frag acc;
        group_sum(acc, ad0, xd0, 0, lane);                                         // G0
#pragma unroll
        for (int mt = 0; mt < 2; mt++)
#pragma unroll
            for (int nt = 0; nt < 4; nt++)
#pragma unroll
                for (int h = 0; h < 2; h++) hi[mt][nt][h] = make_float2(acc[mt][nt][2 * h], acc[mt][nt][2 * h + 1]);
        group_sum(acc, ad0, xd0, 1, lane);                                         // G1
#pragma unroll
        for (int mt = 0; mt < 2; mt++)
#pragma unroll
            for (int nt = 0; nt < 4; nt++)
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    lo[mt][nt][h] = make_float2(0.0f, 0.0f);
                    two_sum2(hi[mt][nt][h], lo[mt][nt][h], make_float2(acc[mt][nt][2 * h], acc[mt][nt][2 * h + 1]));
                }
        group_sum(acc, ad0, xd0, 2, lane);                                         // G2
#pragma unroll
        for (int mt = 0; mt < 2; mt++)
#pragma unroll
            for (int nt = 0; nt < 4; nt++)
#pragma unroll
                for (int h = 0; h < 2; h++)
                    lo[mt][nt][h] = __fadd2_rn(lo[mt][nt][h], make_float2(acc[mt][nt][2 * h], acc[mt][nt][2 * h + 1]));
        group_sum(acc, ad0, xd0, 3, lane);                                         // G3 + G4 (+ G5)
#pragma unroll 1
        for (int d = 4; d < ndig; d++)
#pragma unroll 1
            for (int u = 0; u <= d; u++) tile_mma(acc, ad0 + u * kTile, xd0 + (d - u) * kTile, lane);
#pragma unroll
        for (int mt = 0; mt < 2; mt++)
#pragma unroll
            for (int nt = 0; nt < 4; nt++)
#pragma unroll
                for (int h = 0; h < 2; h++)
                    lo[mt][nt][h] = __fadd2_rn(lo[mt][nt][h], make_float2(acc[mt][nt][2 * h], acc[mt][nt][2 * h + 1]));
        __syncwarp();                                     // every digit read: the tiles are free
        // R = (delta - s hi) - s lo, s = 2^(ea_i + ex_j - 16) (exact products),
        // as two bf16 terms (operand B of X R); X as two bf16 terms (operand
        // A), from the registers
        unsigned char* rh = sm.xd[0];
        unsigned char* rl = sm.xd[1];
        unsigned char* xh = sm.ad[0];
        unsigned char* xl = sm.ad[1];
#pragma unroll
        for (int mt = 0; mt < 2; mt++)
#pragma unroll
            for (int nt = 0; nt < 4; nt++) {
                const float2 sc = *reinterpret_cast<const float2*>(&sm.sx[ecol(nt, 0, lane)]);
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int i = erow(mt, 2 * h, lane), j = ecol(nt, 0, lane);
                    const float sr = sm.sa[i];
                    const float2 s2 = __fmul2_rn(make_float2(sr, sr), sc);
                    const float2 dl = make_float2(i == j ? 1.0f : 0.0f, i == j + 1 ? 1.0f : 0.0f);
                    const float2 r = __fadd2_rn(__fadd2_rn(dl, neg2(__fmul2_rn(hi[mt][nt][h], s2))),
                                                neg2(__fmul2_rn(lo[mt][nt][h], s2)));
                    const __nv_bfloat162 r2 = __floats2bfloat162_rn(r.x, r.y);
                    *reinterpret_cast<__nv_bfloat162*>(rh + tofs(i, j)) = r2;
                    const float2 rr = __fadd2_rn(r, neg2(__bfloat1622float2(r2)));
                    *reinterpret_cast<__nv_bfloat162*>(rl + tofs(i, j)) = __floats2bfloat162_rn(rr.x, rr.y);
                }
            }
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int r = 4 * q + (lane >> 3), c0 = 4 * (lane & 7);
            const float2 v01 = make_float2(vx[q].x, vx[q].y), v23 = make_float2(vx[q].z, vx[q].w);
            const __nv_bfloat162 h01 = __floats2bfloat162_rn(v01.x, v01.y), h23 = __floats2bfloat162_rn(v23.x, v23.y);
            *reinterpret_cast<uint2*>(xh + tofs(r, c0)) = make_uint2(bf2_bits(h01), bf2_bits(h23));
            *reinterpret_cast<uint2*>(xl + tofs(r, c0)) =
                make_uint2(bf2_of(__fadd2_rn(v01, neg2(__bfloat1622float2(h01)))),
                           bf2_of(__fadd2_rn(v23, neg2(__bfloat1622float2(h23)))));
        }
        __syncwarp();
        // C = X R (three bf16 products), X <- X + C: C goes through shared
        // memory (FP32, swizzled) into row order, so that X + C is formed from
        // the registers and written as whole 512-byte rows
        tile_mma<true>(acc, smem_addr(xh), smem_addr(rh), lane);
        tile_mma(acc, smem_addr(xh), smem_addr(rl), lane);
        tile_mma(acc, smem_addr(xl), smem_addr(rh), lane);
        float* cf = reinterpret_cast<float*>(sm.ad[2]);  // 4 KB: tiles 2 and 3
#pragma unroll
        for (int mt = 0; mt < 2; mt++)
#pragma unroll
            for (int nt = 0; nt < 4; nt++)
#pragma unroll
                for (int e = 0; e < 4; e += 2) {
                    const int i = erow(mt, e, lane), j = ecol(nt, e, lane);
                    *reinterpret_cast<float2*>(cf + fofs(i, j)) = make_float2(acc[mt][nt][e], acc[mt][nt][e + 1]);
                }
        __syncwarp();
        float xmax = 0.0f;
        float4* xo = reinterpret_cast<float4*>(X + b * 1024);
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int r = 4 * q + (lane >> 3), c0 = 4 * (lane & 7);
            const float4 c = *reinterpret_cast<const float4*>(cf + fofs(r, c0));
            const float4 x = vx[q];
            xmax = fmaxf(xmax, fmaxf(fmaxf(fabsf(x.x), fabsf(x.y)), fmaxf(fabsf(x.z), fabsf(x.w))));
            xo[lane + 32 * q] = make_float4(x.x + c.x, x.y + c.y, x.z + c.z, x.w + c.w);
        }
        if (next != nullptr) {
            // the error left: about max|C R| / max|X|
            unsigned char* ch = sm.ad[4];
#pragma unroll
            for (int mt = 0; mt < 2; mt++)
#pragma unroll
                for (int nt = 0; nt < 4; nt++)
#pragma unroll
                    for (int e = 0; e < 4; e += 2)
                        put_bf16x2(ch, erow(mt, e, lane), ecol(nt, e, lane), acc[mt][nt][e], acc[mt][nt][e + 1]);
            __syncwarp();
            Frag e2;
            tile_mma<true>(e2, smem_addr(ch), smem_addr(rh), lane);
            float emax = 0.0f;
            bool nan = false;
#pragma unroll
            for (int mt = 0; mt < 2; mt++)
#pragma unroll
                for (int nt = 0; nt < 4; nt++)
#pragma unroll
                    for (int e = 0; e < 4; e++) {
                        nan = nan || isnan(e2[mt][nt][e]);
                        emax = fmaxf(emax, fabsf(e2[mt][nt][e]));
                    }
            float xm = xmax;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) xm = fmaxf(xm, __shfl_xor_sync(0xffffffffu, xm, o));
            const bool bad = nan || !(emax <= tol * xm);   // inf fails the comparison too
            const unsigned any = __ballot_sync(0xffffffffu, bad);
            if (lane == 0) next[t] = any ? (int32_t)b : -1;
        }
        // tiles are reused by the next matrix, and X written above is read
        // back below if the list names this matrix again
        __syncwarp();
        if (live_n) load_rows(vx, X + bn * 1024, lane);
        b = bn;
        live = live_n;
    }
}

}  // namespace mi

namespace {

template <bool kFlag>
int launch_tc(const float* d_a, float* d_x, const int32_t* d_list, int64_t count, int64_t batch, float flag,
              float tol, int32_t* d_next, void* stream) {
    constexpr size_t smem = mi::tcr::smem_bytes();
    constexpr int threads = 32 * mi::tcr::kWarps;
    static int per_sm[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
    if (per_sm[dev] == 0) {
        cudaError_t e = cudaFuncSetAttribute(mi::mi_refine_tc_kernel<kFlag>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return mi::set_cuda_error(e, "tensor-core refinement set-up");
        int p = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p, mi::mi_refine_tc_kernel<kFlag>, threads, smem);
        if (e != cudaSuccess) return mi::set_cuda_error(e, "tensor-core refinement occupancy");
        per_sm[dev] = p < 1 ? 1 : p;
    }
    long long blocks = (count + mi::tcr::kWarps - 1) / mi::tcr::kWarps;
    const long long cap = (long long)per_sm[dev] * mi::device_sm_count();
    if (blocks > cap) blocks = cap;
    mi::mi_refine_tc_kernel<kFlag><<<(unsigned)blocks, threads, smem, reinterpret_cast<cudaStream_t>(stream)>>>(
        d_a, d_x, d_list, count, batch, flag, tol, d_next);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return mi::set_cuda_error(e, "tensor-core refinement launch");
    return MI_OK;
}

int check_tc(const float* d_a, const float* d_x, int n) {
    if (n != 32) return MI_ERR_INVALID_VALUE;
    if (d_a == nullptr || d_x == nullptr) return MI_ERR_NULL_POINTER;
    if (((reinterpret_cast<uintptr_t>(d_a) | reinterpret_cast<uintptr_t>(d_x)) & 15u) != 0) return MI_ERR_MISALIGNED;
    return MI_OK;
}

}  // namespace

extern "C" int mi_refine_tc_next_f32(const float* d_a, float* d_x, const int32_t* d_list, int64_t count,
                                     int64_t batch, int n, float tol, int32_t* d_next, void* stream) {
    if (n != 32 || count < 0 || batch < 0) return MI_ERR_INVALID_VALUE;
    if (d_next != nullptr && !(tol >= 0.0f)) return MI_ERR_INVALID_VALUE;
    if (count == 0) return MI_OK;
    if (d_list == nullptr) return MI_ERR_NULL_POINTER;
    const int st = check_tc(d_a, d_x, n);
    if (st != MI_OK) return st;
    return launch_tc<false>(d_a, d_x, d_list, count, batch, 0.0f, tol, d_next, stream);
}

extern "C" int mi_refine_tc_f32(const float* d_a, float* d_x, const int32_t* d_list, int64_t count, int64_t batch,
                                int n, void* stream) {
    return mi_refine_tc_next_f32(d_a, d_x, d_list, count, batch, n, 0.0f, nullptr, stream);
}

extern "C" int mi_refine_tc_flagged_f32(const float* d_a, float* d_x, int64_t batch, int n, float flag_threshold,
                                        float tol, int32_t* d_next, void* stream) {
    if (n != 32 || batch < 0 || !(flag_threshold >= 0.0f)) return MI_ERR_INVALID_VALUE;
    if (d_next != nullptr && !(tol >= 0.0f)) return MI_ERR_INVALID_VALUE;
    if (batch == 0) return MI_OK;
    const int st = check_tc(d_a, d_x, n);
    if (st != MI_OK) return st;
    return launch_tc<true>(d_a, d_x, nullptr, batch, batch, flag_threshold, tol, d_next, stream);
}
