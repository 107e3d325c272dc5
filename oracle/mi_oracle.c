/*
 * mi_oracle.c -- CPU restatement of the reference's batched LU-inverse path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: the parity tests, the
 * smoke check and the CPU-baseline leg of the benchmark link it to check (or,
 * for the baseline, time) the CUDA path against it.
 * The product path (matrixinversion_gb300 + its CUDA library) never calls it.
 *
 * What it restates (paths are relative to the reference project root):
 *   - mi_or_pivots_reference: the pivot rule of parallel_pivot's kernel,
 *     find_pivot_parallel (parallel_pivot/luBatchedInplace.cuh:12-44) plus the
 *     bookkeeping and row swap of the k-loop (:145-148, :157-172).  The rule
 *     compares only raw input entries (columns k, rows >= k are never written
 *     before step k: comp_U writes row l < k, comp_L writes column l < k,
 *     :60-82), so it is replayed on the input without any arithmetic.
 *   - mi_or_pivots_reference_serial: serial_pivot's find_pivot + swap_rows
 *     (serial_pivot/luBatchedInplace.cuh:12-36, :132-141).
 *   - mi_or_ref_inverse_f32: the whole reference algorithm in FP32:
 *     Doolittle comp_U / comp_L (parallel_pivot/luBatchedInplace.cuh:60-82,
 *     :175-185), then comp_inv's forward/back substitution against the
 *     permuted identity (:84-125).  Every column is solved from the factors
 *     before any column is stored, which is what the reference's single-warp
 *     lockstep execution gives.  This is the "port" CPU baseline.
 *   - mi_or_inverse_f64: FP64 LU-inverse (getrf/getri semantics) used as the
 *     error oracle, with the row order either fixed by a given permutation or
 *     chosen by textbook partial pivoting (argmax of the updated column, first
 *     maximum wins, rows physically swapped as LAPACK getrf does).
 *   - mi_or_residual: ||A X - I|| in FP64 (infinity norm and max-abs entry;
 *     the max-abs entry against 1e-3 is verifyInv's criterion,
 *     parallel_pivot/verify.hpp:50-104).
 *   - mi_or_gen_uniform: MT19937 (seed s) -> float in [-1, 1) as
 *     ((u >> 8) - 2^23) * 2^-23, the seeded generator for every workload.
 *
 * Compare semantics: the reference is built with --use_fast_math
 * (parallel_pivot/run.py:47), so fabs/compare flush subnormal inputs to zero.
 * pivot_key() reproduces that; for normal numbers it is plain |x|.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MI_MAXN 32

enum { OR_PIVOT_NONE = 0, OR_PIVOT_REFERENCE = 1, OR_PIVOT_REFERENCE_SERIAL = 2, OR_PIVOT_PARTIAL = 3 };

/* ------------------------------------------------------------------ */
/* MT19937 (Matsumoto & Nishimura 1998), 32-bit output.                */
/* ------------------------------------------------------------------ */
typedef struct { uint32_t mt[624]; int idx; } mt19937_t;

static void mt_seed(mt19937_t *s, uint32_t seed) {
    s->mt[0] = seed;
    for (int i = 1; i < 624; i++)
        s->mt[i] = 1812433253u * (s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) + (uint32_t)i;
    s->idx = 624;
}

static uint32_t mt_next(mt19937_t *s) {
    if (s->idx >= 624) {
        for (int i = 0; i < 624; i++) {
            uint32_t y = (s->mt[i] & 0x80000000u) | (s->mt[(i + 1) % 624] & 0x7fffffffu);
            uint32_t v = s->mt[(i + 397) % 624] ^ (y >> 1);
            if (y & 1u) v ^= 0x9908b0dfu;
            s->mt[i] = v;
        }
        s->idx = 0;
    }
    uint32_t y = s->mt[s->idx++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

/* count floats uniform in [-1, 1) on the 2^-23 grid, from one MT19937 stream. */
void mi_or_gen_uniform(uint32_t seed, int64_t count, float *out) {
    mt19937_t s;
    mt_seed(&s, seed);
    for (int64_t i = 0; i < count; i++) {
        int32_t q = (int32_t)(mt_next(&s) >> 8) - (1 << 23);
        out[i] = (float)q * (1.0f / 8388608.0f);
    }
}

/* ------------------------------------------------------------------ */
/* Pivot rules on the raw input (no arithmetic).                       */
/* ------------------------------------------------------------------ */
static inline float pivot_key(float x) {
    float a = fabsf(x);
    /* flush-to-zero compare semantics of the reference build */
    if (a < 1.17549435e-38f) return 0.0f;   /* also leaves NaN untouched */
    return a;
}

/* perm[i] = input row that ends at row i (the reference's shared pivots[]). */
void mi_or_pivots_reference(const float *A, int n, int T, int32_t *perm) {
    float vals[64];
    int idxs[64];
    for (int i = 0; i < n; i++) perm[i] = i;
    for (int k = 0; k < n; k++) {
        /* find_pivot_parallel: per-thread strided scan, strict '>' against the
         * diagonal-initialised candidate (luBatchedInplace.cuh:17-30) */
        for (int t = 0; t < T; t++) {
            float v = pivot_key(A[perm[k] * n + k]);
            int idx = k;
            for (int i = k + 1 + t; i < n; i += T) {
                float w = pivot_key(A[perm[i] * n + k]);
                if (w > v) { v = w; idx = i; }
            }
            vals[t] = v;
            idxs[t] = idx;
        }
        /* tree with strides T/2, T/4, ..., 1 and strict '<' (:34-42);
         * slots outside the power-of-two tree never reach slot 0. */
        for (int s = T / 2; s > 0; s >>= 1)
            for (int t = 0; t < s; t++)
                if (vals[t] < vals[t + s]) { vals[t] = vals[t + s]; idxs[t] = idxs[t + s]; }
        int p = idxs[0];
        if (p != k) { int tmp = perm[k]; perm[k] = perm[p]; perm[p] = tmp; }
    }
}

void mi_or_pivots_reference_serial(const float *A, int n, int32_t *perm) {
    for (int i = 0; i < n; i++) perm[i] = i;
    for (int k = 0; k < n; k++) {
        int p = k;
        float mv = pivot_key(A[perm[k] * n + k]);
        for (int i = k + 1; i < n; i++) {
            float w = pivot_key(A[perm[i] * n + k]);
            if (w > mv) { mv = w; p = i; }
        }
        if (p != k) { int tmp = perm[k]; perm[k] = perm[p]; perm[p] = tmp; }
    }
}

/* ------------------------------------------------------------------ */
/* FP64 LU-inverse oracle.                                             */
/* mode NONE: no row exchange; REFERENCE / REFERENCE_SERIAL: rows      */
/* ordered by the replayed rule; PARTIAL: argmax of the updated column */
/* (first maximum, physical swaps, LAPACK getrf).  Returns info (0 or  */
/* first zero pivot step, 1-based) and writes perm.                    */
/* ------------------------------------------------------------------ */
int mi_or_inverse_f64(const float *A, int n, int mode, double *X, int32_t *perm) {
    double lu[MI_MAXN * MI_MAXN];
    int32_t p[MI_MAXN];
    int info = 0;
    if (mode == OR_PIVOT_REFERENCE) mi_or_pivots_reference(A, n, n, p);
    else if (mode == OR_PIVOT_REFERENCE_SERIAL) mi_or_pivots_reference_serial(A, n, p);
    else for (int i = 0; i < n; i++) p[i] = i;
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) lu[i * n + j] = (double)A[p[i] * n + j];
    /* right-looking LU */
    for (int k = 0; k < n; k++) {
        if (mode == OR_PIVOT_PARTIAL) {
            int q = k;
            double mv = fabs(lu[k * n + k]);
            for (int i = k + 1; i < n; i++) {
                double w = fabs(lu[i * n + k]);
                if (w > mv) { mv = w; q = i; }
            }
            if (q != k) {
                for (int j = 0; j < n; j++) { double t = lu[k * n + j]; lu[k * n + j] = lu[q * n + j]; lu[q * n + j] = t; }
                int t = p[k]; p[k] = p[q]; p[q] = t;
            }
        }
        double d = lu[k * n + k];
        if (d == 0.0 && info == 0) info = k + 1;
        for (int i = k + 1; i < n; i++) {
            double l = lu[i * n + k] / d;
            lu[i * n + k] = l;
            for (int j = k + 1; j < n; j++) lu[i * n + j] -= l * lu[k * n + j];
        }
    }
    /* column c of (PA)^-1 from L U x = e_c; A^-1 = (PA)^-1 P, i.e.
     * A^-1[:, p[c]] = (PA)^-1[:, c] */
    double y[MI_MAXN];
    for (int c = 0; c < n; c++) {
        for (int i = 0; i < n; i++) {
            double s = (i == c) ? 1.0 : 0.0;
            for (int j = 0; j < i; j++) s -= lu[i * n + j] * y[j];
            y[i] = s;
        }
        for (int i = n - 1; i >= 0; i--) {
            double s = y[i];
            for (int j = i + 1; j < n; j++) s -= lu[i * n + j] * y[j];
            y[i] = s / lu[i * n + i];
        }
        for (int i = 0; i < n; i++) X[i * n + p[c]] = y[i];
    }
    if (perm) memcpy(perm, p, sizeof(int32_t) * (size_t)n);
    return info;
}

/* ------------------------------------------------------------------ */
/* FP32 port of the reference kernel's arithmetic (Doolittle order).   */
/* In place: A becomes A^-1.  Returns info.                            */
/* ------------------------------------------------------------------ */
int mi_or_ref_inverse_f32(float *A, int n, int mode, int32_t *perm) {
    float a[MI_MAXN * MI_MAXN];
    int32_t p[MI_MAXN];
    int info = 0;
    memcpy(a, A, sizeof(float) * (size_t)n * n);
    for (int i = 0; i < n; i++) p[i] = i;
    for (int k = 0; k < n; k++) {
        int q = k;
        if (mode == OR_PIVOT_REFERENCE || mode == OR_PIVOT_REFERENCE_SERIAL) {
            /* raw column k at rows >= k is still the input (see header) */
            if (mode == OR_PIVOT_REFERENCE) {
                float vals[64]; int idxs[64];
                for (int t = 0; t < n; t++) {
                    float v = pivot_key(a[k * n + k]); int idx = k;
                    for (int i = k + 1 + t; i < n; i += n) {
                        float w = pivot_key(a[i * n + k]);
                        if (w > v) { v = w; idx = i; }
                    }
                    vals[t] = v; idxs[t] = idx;
                }
                for (int s = n / 2; s > 0; s >>= 1)
                    for (int t = 0; t < s; t++)
                        if (vals[t] < vals[t + s]) { vals[t] = vals[t + s]; idxs[t] = idxs[t + s]; }
                q = idxs[0];
            } else {
                float mv = pivot_key(a[k * n + k]);
                for (int i = k + 1; i < n; i++) {
                    float w = pivot_key(a[i * n + k]);
                    if (w > mv) { mv = w; q = i; }
                }
            }
        } else if (mode == OR_PIVOT_PARTIAL) {
            /* Doolittle keeps column k un-eliminated until comp_L, so the
             * partial rule needs the updated column: form it first. */
            float mv = -1.0f;
            for (int i = k; i < n; i++) {
                float s = a[i * n + k];
                for (int l = 0; l < k; l++) s -= a[i * n + l] * a[l * n + k];
                float w = fabsf(s);
                if (w > mv) { mv = w; q = i; }
            }
        }
        if (q != k) {
            for (int j = 0; j < n; j++) { float t = a[k * n + j]; a[k * n + j] = a[q * n + j]; a[q * n + j] = t; }
            int t = p[k]; p[k] = p[q]; p[q] = t;
        }
        /* comp_U: row k, columns j >= k */
        for (int j = k; j < n; j++) {
            float s = 0.0f;
            for (int l = 0; l < k; l++) s += a[k * n + l] * a[l * n + j];
            a[k * n + j] = a[k * n + j] - s;
        }
        if (a[k * n + k] == 0.0f && info == 0) info = k + 1;
        /* comp_L: column k, rows i > k */
        for (int i = k + 1; i < n; i++) {
            float s = 0.0f;
            for (int l = 0; l < k; l++) s += a[i * n + l] * a[l * n + k];
            a[i * n + k] = (a[i * n + k] - s) / a[k * n + k];
        }
    }
    /* comp_inv: column c solves L y = P e_c (b_i = [p[i] == c]), U x = y */
    float y[MI_MAXN], x[MI_MAXN];
    for (int c = 0; c < n; c++) {
        for (int i = 0; i < n; i++) {
            float b = (p[i] == c) ? 1.0f : 0.0f;
            float s = 0.0f;
            for (int j = 0; j < i; j++) s += a[i * n + j] * y[j];
            y[i] = b - s;
        }
        for (int i = n - 1; i >= 0; i--) {
            float s = 0.0f;
            for (int j = i + 1; j < n; j++) s += a[i * n + j] * x[j];
            x[i] = (y[i] - s) / a[i * n + i];
        }
        for (int i = 0; i < n; i++) A[i * n + c] = x[i];
    }
    if (perm) memcpy(perm, p, sizeof(int32_t) * (size_t)n);
    return info;
}

/* ------------------------------------------------------------------ */
/* Residuals in FP64: res[0] = ||A X - I||_inf (max row sum),          */
/* res[1] = max |(A X - I)_ij|.                                        */
/* ------------------------------------------------------------------ */
void mi_or_residual(const float *A, const float *X, int n, double *res) {
    double rinf = 0.0, rmax = 0.0;
    for (int i = 0; i < n; i++) {
        double row = 0.0;
        for (int j = 0; j < n; j++) {
            double s = (i == j) ? -1.0 : 0.0;
            for (int l = 0; l < n; l++) s += (double)A[i * n + l] * (double)X[l * n + j];
            double a = fabs(s);
            if (isnan(s)) a = INFINITY;
            row += a;
            if (a > rmax) rmax = a;
        }
        if (row > rinf) rinf = row;
    }
    res[0] = rinf;
    res[1] = rmax;
}

/* ------------------------------------------------------------------ */
/* Batched entry points (OpenMP over independent matrices).            */
/* ------------------------------------------------------------------ */
int mi_or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void mi_or_set_num_threads(int t) {
#ifdef _OPENMP
    if (t > 0) omp_set_num_threads(t);
#else
    (void)t;
#endif
}

void mi_or_batch_pivots(const float *A, int64_t batch, int n, int mode, int T, int32_t *perm) {
    int64_t nn = (int64_t)n * n;
#pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < batch; b++) {
        if (mode == OR_PIVOT_REFERENCE) mi_or_pivots_reference(A + b * nn, n, T, perm + b * n);
        else if (mode == OR_PIVOT_REFERENCE_SERIAL) mi_or_pivots_reference_serial(A + b * nn, n, perm + b * n);
        else for (int i = 0; i < n; i++) perm[b * n + i] = i;
    }
}

void mi_or_batch_inverse_f64(const float *A, int64_t batch, int n, int mode, double *X, int32_t *perm, int32_t *info) {
    int64_t nn = (int64_t)n * n;
#pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < batch; b++) {
        int r = mi_or_inverse_f64(A + b * nn, n, mode, X + b * nn, perm ? perm + b * n : NULL);
        if (info) info[b] = r;
    }
}

/* In place over the batch: the reference algorithm in FP32 (CPU baseline). */
void mi_or_batch_ref_inverse_f32(float *A, int64_t batch, int n, int mode, int32_t *perm, int32_t *info) {
    int64_t nn = (int64_t)n * n;
#pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < batch; b++) {
        int r = mi_or_ref_inverse_f32(A + b * nn, n, mode, perm ? perm + b * n : NULL);
        if (info) info[b] = r;
    }
}

void mi_or_batch_residual(const float *A, const float *X, int64_t batch, int n, double *res) {
    int64_t nn = (int64_t)n * n;
#pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < batch; b++) mi_or_residual(A + b * nn, X + b * nn, n, res + 2 * b);
}
