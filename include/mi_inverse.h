/*
 * mi_inverse.h -- C ABI of the GB300 batched small-matrix inverter.
 *
 * Plain pointers and sizes only.  All device pointers are caller-owned CUDA
 * device memory; every call is stream-ordered on `stream` (a cudaStream_t, or
 * NULL for the legacy default stream), returns a status code and never exits
 * the process.
 *
 * What each entry point replaces in the reference (sumukhashridhar/
 * matrixInversion; paths relative to its root):
 *   mi_inverse_f32      batched_lu_subwarp<float, n, T, mpb, N><<<ceil(N/mpb),
 *                       NUMTHREADS, smem>>>(d_A) -- parallel_pivot/
 *                       luBatchedInplace.cu:127 (pivot = MI_PIVOT_REFERENCE),
 *                       serial_pivot/luBatchedInplace.cu:105
 *                       (MI_PIVOT_REFERENCE_SERIAL), templated/
 *                       luBatchedInplace.cu:76 (MI_PIVOT_NONE).  In place,
 *                       row-major, matrix b at offset b*n*n, as there.  The
 *                       reference keeps its pivots in shared memory
 *                       (parallel_pivot/luBatchedInplace.cuh:140); here they
 *                       can be written out (d_perm).
 *   mi_inverse_cfg_f32  the same launch with the reference's NUMTHREADS knob
 *                       (threads per block; parallel_pivot/run.py:41, 187-224)
 *                       and an explicit grid size.
 *   mi_query_config     the launch geometry the reference derives in
 *                       luBatchedInplace.cu:8-11 (threads per matrix,
 *                       matrices per block) and :118 (shared memory).
 *   mi_error_string /   the reference's CUDA_CHECK, which prints and calls
 *   mi_last_cuda_error  exit(1) (parallel_pivot/luBatchedInplace.cuh:9).
 *   mi_inverse_descr_f32  no reference counterpart for mixed sizes in one
 *                       call; the per-matrix work is the same kernel, and the
 *                       runtime-n interface follows no_templ/
 *                       luBatchedInplace.cuh:82-85 (n, batch and threads as
 *                       runtime values).
 *   mi_set_launch_config / mi_get_launch_config  the NUMTHREADS table of
 *                       parallel_pivot/run.py:187-224, per (n, pivot), settable
 *                       at run time (by the autotuner).
 *   mi_set_launch_lanes / mi_get_launch_lanes  lanes per matrix per (n, pivot),
 *                       tuned likewise (no reference counterpart: its launch
 *                       uses one thread per column).
 */
#ifndef MI_INVERSE_H
#define MI_INVERSE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MI_ABI_VERSION 2

/* status codes */
#define MI_OK 0
#define MI_ERR_INVALID_VALUE (-1) /* n outside 1..32, batch < 0, unknown pivot mode, bad knob */
#define MI_ERR_NULL_POINTER (-2)  /* d_a is NULL while batch > 0 */
#define MI_ERR_MISALIGNED (-3)    /* d_a not 4-byte aligned */
#define MI_ERR_CUDA (-4)          /* a CUDA call failed; see mi_last_cuda_error() */
#define MI_ERR_SCRATCH_LIMIT (-5) /* count above MI_NOALLOC_MAX_COUNT (no-allocation entry point) */

/* pivot modes */
#define MI_PIVOT_NONE 0             /* plain LU (templated/ kernel)                  */
#define MI_PIVOT_REFERENCE 1        /* parallel_pivot/ argmax tree, bit-exact pivots */
#define MI_PIVOT_REFERENCE_SERIAL 2 /* serial_pivot/ sequential argmax               */
#define MI_PIVOT_PARTIAL 3          /* textbook partial pivoting (getrf semantics)   */

/*
 * Invert `batch` row-major n x n FP32 matrices in place: d_a[b*n*n ...] is
 * replaced by its inverse.
 *   d_perm  (nullable) int32[batch][n]: d_perm[b][i] = input row that ends at
 *           row i after the pivoting (the reference's shared pivots[]); the
 *           inverse satisfies A^-1[:, perm[i]] = (P A)^-1[:, i].
 *   d_info  (nullable) int32[batch]: 0, or k (1-based) if the k-th pivot was
 *           exactly zero (the inverse then holds inf/NaN, as the reference's).
 */
int mi_inverse_f32(float* d_a, int32_t* d_perm, int32_t* d_info, int64_t batch, int n, int pivot,
                   void* stream);

/*
 * As mi_inverse_f32 with explicit launch knobs.
 *   threads_per_block  the NUMTHREADS knob; rounded up to a multiple of 32 and
 *                      capped at 256; 0 = default.  Used by the lane-group
 *                      kernel form only (mi_query_launch says which form a
 *                      call runs); the other forms have a fixed block.
 *   grid_blocks        0 = sized from the device's SM count and occupancy.
 */
int mi_inverse_cfg_f32(float* d_a, int32_t* d_perm, int32_t* d_info, int64_t batch, int n, int pivot,
                       int threads_per_block, int grid_blocks, void* stream);

/*
 * Launch geometry for size n without pivoting or with the reference rules on
 * large batches: lanes per matrix, matrices per warp, shared memory bytes per
 * warp, and the default threads per block.  Any out pointer may be NULL.
 * Needs no GPU.  mi_query_launch gives the geometry for any pivot mode and
 * batch size.
 */
int mi_query_config(int n, int* lanes_per_matrix, int* matrices_per_warp, int* smem_bytes_per_warp,
                    int* default_threads_per_block);

/*
 * Kernel forms of a contiguous call (mi_query_launch).  Only the lane-group
 * form launches with the NUMTHREADS knob (threads_per_block of
 * mi_inverse_cfg_f32, or the installed mi_set_launch_config entry); the other
 * two have a fixed block, and the knob changes nothing there.
 */
#define MI_FORM_THREAD 1 /* one thread per matrix (n <= 8; n = 9..15 on large batches)  */
#define MI_FORM_LANES 2  /* a group of lanes per matrix, register blocks              */
#define MI_FORM_ROWS 3   /* 16 lanes per matrix, whole rows per lane (partial pivoting) */

/*
 * The kernel a contiguous mi_inverse_cfg_f32(..., batch, n, pivot,
 * threads_per_block, ...) call launches (no counterpart in the reference,
 * whose launch geometry is its compile-time template arguments,
 * parallel_pivot/luBatchedInplace.cu:4-11): *form (MI_FORM_*), lanes per
 * matrix, matrices per warp, and the threads per block it launches with --
 * threads_per_block resolved as that call resolves it (0 = the installed
 * entry; rounded up to a multiple of 32, capped at 256) for MI_FORM_LANES,
 * the form's fixed block otherwise.  Any out pointer may be NULL.  Needs no
 * GPU.  Descriptor buckets (mi_inverse_descr_f32) choose their kernels per
 * bucket and are not covered.
 */
int mi_query_launch(int n, int pivot, int64_t batch, int threads_per_block, int* form, int* lanes_per_matrix,
                    int* matrices_per_warp, int* threads_per_block_used);

/*
 * Mixed sizes in one call.  Matrix i is n_i x n_i (1..32), row-major at
 * d_packed + d_offsets[i] (floats), pivot mode d_flags[i] (MI_PIVOT_*),
 * inverted in place.  packed_floats: the size of d_packed in floats; every
 * matrix must lie in [0, packed_floats).  d_perm (nullable) int32[count][32]:
 * pivots of matrix i at d_perm[i * 32 ..]; d_info (nullable) int32[count]: as
 * mi_inverse_f32, or -1 for a malformed descriptor (n or flag out of range,
 * or a matrix that is not inside d_packed; not processed, not touched).
 * n_mask: bit n-1 set if size n may occur (0 = all sizes); mode_mask: bit m
 * set if pivot mode m may occur (0 = all) -- buckets outside the masks are
 * not processed.  d_workspace: caller-owned device scratch of at least
 * mi_descr_workspace_bytes(count) bytes, 256-byte aligned.  The call issues
 * only stream-ordered work (no host synchronisation), so it can be captured
 * into a CUDA graph: a memset and three bucketing kernels (count, scan,
 * scatter), then either one persistent launch per (n, mode) bucket inside the
 * masks (the default) or, after mi_set_descr_chunk(c > 0), ONE persistent
 * launch whose warps take chunks of about c input floats (at most 8 groups)
 * from a device counter, largest n first, for every bucket (the runtime-n
 * counterpart of no_templ/luBatchedInplace.cuh:82-131).  Every matrix gets
 * the bits of the contiguous call either way.
 */
int mi_inverse_descr_f32(float* d_packed, int64_t packed_floats, const int64_t* d_offsets, const int32_t* d_n,
                         const int32_t* d_flags, int32_t* d_perm, int32_t* d_info, int64_t count, uint32_t n_mask,
                         uint32_t mode_mask, void* d_workspace, size_t workspace_bytes, void* stream);
size_t mi_descr_workspace_bytes(int64_t count);
/*
 * Form of mi_inverse_descr_f32: 0 (the default) = one launch per (n, mode)
 * bucket; c > 0 = the single persistent launch with chunks of about c input
 * floats (1 to 8 groups of matrices each).  Process-wide; the same bits
 * either way.  MI_ERR_INVALID_VALUE for a negative size.
 */
int mi_set_descr_chunk(int chunk_floats);
int mi_get_descr_chunk(void);

/*
 * mi_inverse_descr_f32 without a caller workspace -- no counterpart in the
 * reference, whose kernels need no scratch.  For callers that cannot
 * allocate device memory when they invert: a serving loop whose HBM is
 * carved up once at start-up under a fixed budget, code whose framework
 * allocator must see every device allocation, and latency-bound loops --
 * cudaMalloc and cudaFree synchronise the device and stall every stream.
 * The bucketing scratch is a fixed file-scope device array of
 * 4096 + 4 * MI_NOALLOC_MAX_COUNT bytes (about 1 MB) per device; the call
 * itself allocates nothing.
 *   count > MI_NOALLOC_MAX_COUNT  returns MI_ERR_SCRATCH_LIMIT and launches
 *                 nothing; use mi_inverse_descr_f32 with your own workspace.
 *   First call on each device: looks up the scratch's device address
 *                 (cudaGetSymbolAddress, with that device current), which also
 *                 loads the library's device code there if needed.  Make that
 *                 first call before any stream capture begins.  The address is
 *                 kept per device and context: the first call in a new context
 *                 on the device (after cudaDeviceReset) looks it up again, so
 *                 make that one before any capture too.
 *   Zeroing:      the caller clears nothing; each call resets the scratch's
 *                 bucket counters on `stream` before use, and the rest of the
 *                 scratch is written before it is read.
 *   Concurrency:  one scratch per device, so calls that overlap on the same
 *                 device (other streams or host threads, not ordered by the
 *                 same stream or by events) race on it and can return wrong
 *                 results.  Order them.
 * Arguments, results and other status codes as mi_inverse_descr_f32.
 */
#define MI_NOALLOC_MAX_COUNT 262144
int mi_inverse_descr_noalloc_f32(float* d_packed, int64_t packed_floats, const int64_t* d_offsets,
                                 const int32_t* d_n, const int32_t* d_flags, int32_t* d_perm, int32_t* d_info,
                                 int64_t count, uint32_t n_mask, uint32_t mode_mask, void* stream);

/*
 * Waits that ran out on the device (no counterpart in the reference, whose
 * kernels wait without a limit).  Every wait of the kernels on a tile copy or
 * a tensor-core product gives up after about two seconds; the warp (or CTA)
 * then records a flag and stops, leaving the rest of its matrices unwritten.
 * The call still returned MI_OK, so a caller that must know checks here:
 *   *flags  (nullable) the flags recorded since the last clear:
 *           MI_DEVERR_COPY_TIMEOUT  a tile copy did not arrive (inverse kernels)
 *           MI_DEVERR_MMA_TIMEOUT   a tensor-core product did not complete
 *                                   (mi_newton_schulz_f32)
 *   clear   != 0 resets the flags after reading them.
 * Per device (the current one).  Synchronous: it reads after the work already
 * issued to the legacy default stream; synchronise other streams first.
 */
#define MI_DEVERR_COPY_TIMEOUT 1
#define MI_DEVERR_MMA_TIMEOUT 2
int mi_device_error(int* flags, int clear);

/*
 * Test hook of the bounded waits (no counterpart in the reference): lets a
 * test make a tile-copy wait run out without a fault or a stalled copy.
 * wait_limit_cycles  the longest wait of the contiguous inverse kernels on
 *                    a tile copy, in SM clocks (<= 0 restores the default of
 *                    about two seconds);
 * arm_without_copy   != 0: each warp arms its copy barrier with the bytes it
 *                    expects but issues no copy, so every such wait runs out
 *                    (nothing is in flight, nothing lands late); the warps
 *                    then record MI_DEVERR_COPY_TIMEOUT and return with their
 *                    matrices unwritten.
 * Applies to later launches on the current device until reset with
 * mi_set_wait_test(0, 0).  Not for production use: a call in test mode
 * returns MI_OK and leaves its outputs unwritten.
 */
int mi_set_wait_test(int64_t wait_limit_cycles, int arm_without_copy);

/*
 * Newton-Schulz refinement of n = 32 inverses on the tensor cores (no
 * reference counterpart: the reference computes in FP32 only, with its FP64
 * switch commented out, verify.hpp:9):  X <- X + X (I - A X), `steps` times
 * (1..4).  Products are 3xTF32 (TF32 head and FP32 remainder, FP32
 * accumulation).  d_a, d_x: batch row-major 32 x 32 FP32 matrices, 16-byte
 * aligned; d_x is refined in place, d_a is only read.
 */
int mi_newton_schulz_f32(const float* d_a, float* d_x, int64_t batch, int n, int steps, void* stream);

/*
 * One refinement step in FP64 for the matrices listed in d_list[0 .. count)
 * (indices into a batch of `batch` n x n FP32 matrices, n <= 32): R = I - A X
 * and X <- X + X R evaluated in FP64, X rounded once to FP32.  For the
 * matrices a cheap test flags as ill-conditioned, where an FP32 residual is
 * no better than the inverse itself.  Out-of-range list entries are skipped.
 * No counterpart in the reference, which computes in FP32 only (its FP64
 * switch is commented out, parallel_pivot/verify.hpp:9).
 */
int mi_refine_fp64_f32(const float* d_a, float* d_x, const int32_t* d_list, int64_t count, int64_t batch, int n,
                       void* stream);

/*
 * As mi_refine_fp64_f32 with the residual R = I - A X in compensated
 * float-float arithmetic on the FP32 pipes (exact products, TwoSum
 * accumulation: about 44 significant bits) and X R in FP32 -- the same
 * accuracy gain where kappa * u < 1, several times faster on GPUs whose FP64
 * rate is low.  No counterpart in the reference.
 */
int mi_refine_df_f32(const float* d_a, float* d_x, const int32_t* d_list, int64_t count, int64_t batch, int n,
                     void* stream);

/*
 * As mi_refine_df_f32, and also writes d_next[t] = d_list[t] where the
 * error left after this step, estimated as max|X R^2| / max|X| (X and R
 * before the step: X (I + R) - A^-1 = -A^-1 R^2 to first order), exceeds tol
 * or is not finite, else -1 (also -1 for skipped entries).  d_next has count
 * entries and may be d_list itself; it is the list for a second step, so that
 * step runs only where the first does not suffice.  No counterpart in the
 * reference.
 */
int mi_refine_df_next_f32(const float* d_a, float* d_x, const int32_t* d_list, int64_t count, int64_t batch, int n,
                          float tol, int32_t* d_next, void* stream);

/*
 * As mi_refine_df_f32 for n = 32, with the residual R = I - A X formed on the
 * tensor cores by error-free splitting: rows of A and columns of X, scaled by
 * powers of two, cut into digits of 8 significant bits held exactly in bf16,
 * digit products grouped so that each group is exact in the FP32 accumulators
 * of mma.sync, the groups combined in float-float.  The residual carries about
 * 37 bits of the row-times-column scale (about 40 where max|A| max|X| may
 * reach 2^16 and a sixth digit is taken); the correction X R takes two-term
 * bf16 splits of X and R.  d_a and d_x 16-byte aligned; n other than
 * 32 -> MI_ERR_INVALID_VALUE.  No counterpart in the reference.
 */
int mi_refine_tc_f32(const float* d_a, float* d_x, const int32_t* d_list, int64_t count, int64_t batch, int n,
                     void* stream);

/*
 * As mi_refine_tc_f32, and also writes d_next[t] = d_list[t] where the error
 * left after this step, estimated as max|C R| / max|X| (C = X R, the
 * correction), exceeds tol or is not finite, else -1 (also -1 for skipped
 * entries).  d_next has count entries and may be d_list itself.  No
 * counterpart in the reference.
 */
int mi_refine_tc_next_f32(const float* d_a, float* d_x, const int32_t* d_list, int64_t count, int64_t batch, int n,
                          float tol, int32_t* d_next, void* stream);

/*
 * The flag and the first step of the refined form in one pass over the batch:
 * for every b in [0, batch) whose condition estimate ||A_b||_1 ||X_b||_1 is
 * at least flag_threshold (or not finite) -- the estimate
 * mi_flag_condition_f32 computes, summed in another order -- one step of
 * mi_refine_tc_next_f32; d_next[b] = b where that step leaves an estimated
 * error above tol, else -1 (also -1 for matrices not refined).  d_next (batch
 * entries, or NULL) is the list for a second mi_refine_tc_f32 step.  No
 * counterpart in the reference.
 */
int mi_refine_tc_flagged_f32(const float* d_a, float* d_x, int64_t batch, int n, float flag_threshold, float tol,
                             int32_t* d_next, void* stream);

/*
 * d_list[b] = b if ||A_b||_1 * ||X_b||_1 >= threshold (or is not finite),
 * else -1, for b in [0, batch): a list the two refinement calls take as it is
 * (count = batch; -1 entries are skipped), so flagging needs no host round
 * trip.  No counterpart in the reference (its host code computes a condition
 * number only for reporting, parallel_pivot/verify.hpp:246-338).
 */
int mi_flag_condition_f32(const float* d_a, const float* d_x, int64_t batch, int n, float threshold,
                          int32_t* d_list, void* stream);

/*
 * Threads per block used for size n and pivot mode whenever a call passes
 * threads_per_block = 0.  Ships with a table measured on GB300; set 0 to
 * restore that table's entry.
 */
int mi_set_launch_config(int n, int pivot, int threads_per_block);
int mi_get_launch_config(int n, int pivot, int* threads_per_block);

/*
 * Lanes per matrix for size n and pivot mode (the width of the sub-warp that
 * owns a matrix; the reference fixes one thread per column,
 * parallel_pivot/luBatchedInplace.cu:4-11).  Sizes 17..31 without partial
 * pivoting run at 16 or 8 lanes -- the same bits either way -- and ship with
 * the choice measured on GB300; every other (n, pivot) has one width.  Set
 * lanes_per_matrix to that width, the alternative, or 0 to restore the table's
 * entry; anything else -> MI_ERR_INVALID_VALUE.  mi_get_launch_lanes returns
 * the installed width and the other width the size can run at (0 if none).
 * Contiguous calls of at least MI_LANES_ALT_MIN_BATCH matrices follow the
 * entry; smaller ones and descriptor buckets run at the default width.
 */
#define MI_LANES_ALT_MIN_BATCH 131072
int mi_set_launch_lanes(int n, int pivot, int lanes_per_matrix);
int mi_get_launch_lanes(int n, int pivot, int* lanes_per_matrix, int* other);

const char* mi_error_string(int status);
/* Text of the last CUDA error seen by this thread ("" if none). */
const char* mi_last_cuda_error(void);
/*
 * Serving loop (no counterpart in the reference, which inverts one pre-loaded
 * batch per process).  Serves num_requests requests -- request r: k[r]
 * matrices of size n[r] (1..32), pivot mode `pivot`, arriving arrival_s[r]
 * seconds after the call starts (non-decreasing) -- and returns when all have
 * completed, with latency_s[r] = completion - arrival.  Runs on the calling
 * thread; every launch and copy is issued from native code.
 *   Copies (d_ring == NULL): request r's matrices are read from the pinned
 *     host ring h_in + ring_off[r] (floats) and written back to h_out at the
 *     same offset.  d_pool: the device pool of pool_floats floats, carved by
 *     the caller once (the HBM budget); an arrived request is admitted, first
 *     come first served, as soon as a free extent of the pool holds it, and
 *     its extent is freed when its own results have reached h_out.  A request
 *     larger than the pool returns MI_ERR_SCRATCH_LIMIT.
 *   Resident (d_ring != NULL): the matrices already sit in device memory at
 *     d_ring + ring_off[r] and are inverted in place (no copies, d_pool and the
 *     host rings unused); a request completes with its batch's kernels.
 *   Batching: while fewer than two batches compute, every admitted request
 *     not yet computed (coalesce != 0; at most max_batch_matrices matrices)
 *     or the next one (coalesce == 0) goes out as one launch.
 *   d_scratch: device scratch of mi_serve_scratch_bytes(max_batch_matrices)
 *     bytes, 256-byte aligned.  The call makes its own streams, events and a
 *     pinned staging buffer for the descriptor tables at its start and frees
 *     them before it returns.
 *   stats (nullable) int64[2]: batches launched, peak pool floats in use.
 */
size_t mi_serve_scratch_bytes(int64_t max_batch_matrices);
int mi_serve_run(int64_t num_requests, const double* arrival_s, const int64_t* k, const int32_t* n,
                 const int64_t* ring_off, const float* h_in, float* h_out, float* d_ring, float* d_pool,
                 int64_t pool_floats, void* d_scratch, size_t scratch_bytes, int64_t max_batch_matrices, int pivot,
                 int coalesce, double* latency_s, double* wall_s, int64_t* stats);

/* MI_ABI_VERSION of the loaded library, to check against the header a
   caller was built with (no counterpart in the reference, which has no
   library). */
int mi_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* MI_INVERSE_H */
