// mi_api.cu -- the C ABI declared in include/mi_inverse.h.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "mi_inverse.h"
#include "mi_launch.cuh"

namespace mi {

static thread_local char g_last_cuda_error[256] = "";

static int cuda_fail(cudaError_t e, const char* what) {
    std::snprintf(g_last_cuda_error, sizeof(g_last_cuda_error), "%s: %s (%d)", what, cudaGetErrorString(e), (int)e);
    return MI_ERR_CUDA;
}

int set_cuda_error(cudaError_t e, const char* what) { return cuda_fail(e, what); }

// Readers of the per-module device error words, registered while the library
// loads (function-local statics: safe whatever the order of static
// initialisation across translation units).
static std::mutex& error_readers_mu() {
    static std::mutex m;
    return m;
}
static std::vector<device_error_reader>& error_readers() {
    static std::vector<device_error_reader> v;
    return v;
}
static std::vector<wait_test_setter>& wait_test_setters() {
    static std::vector<wait_test_setter> v;
    return v;
}
bool register_wait_test_setter(wait_test_setter fn) {
    std::lock_guard<std::mutex> lock(error_readers_mu());
    wait_test_setters().push_back(fn);
    return true;
}

bool register_device_error_reader(device_error_reader fn) {
    std::lock_guard<std::mutex> lock(error_readers_mu());
    error_readers().push_back(fn);
    return true;
}

// Threads per block per (n, pivot mode), measured on GB300 by the autotuner
// (matrixinversion_gb300/autotune.py: 262,144 uniform matrices per size, the
// fastest of 32..256; n = 17..31 at the lanes per matrix of kLanesGB300);
// 0 = the built-in default of 128.  mi_set_launch_config overrides entries at run
// time (0 restores this table's entry).
static const int kTunedGB300[33][4] = {
    {0, 0, 0, 0},
    {0, 0, 0, 0},
    {128, 128, 128, 256},
    {160, 64, 64, 64},
    {160, 128, 128, 64},
    {128, 256, 256, 256},
    {64, 256, 256, 256},
    {256, 256, 256, 256},
    {128, 32, 32, 256},
    {128, 256, 256, 256},
    {32, 256, 256, 256},
    {32, 256, 256, 256},
    {32, 256, 256, 256},
    {32, 256, 256, 256},
    {32, 256, 256, 256},
    {64, 256, 256, 256},
    {256, 32, 32, 256},
    {32, 256, 256, 256},
    {128, 256, 256, 256},
    {256, 256, 256, 256},
    {256, 256, 32, 256},
    {256, 256, 256, 256},
    {256, 256, 128, 256},
    {256, 256, 256, 256},
    {256, 256, 64, 256},
    {256, 256, 32, 256},
    {256, 256, 32, 256},
    {256, 256, 256, 256},
    {256, 256, 256, 256},
    {32, 256, 128, 256},
    {128, 256, 128, 256},
    {128, 256, 64, 256},
    {256, 256, 256, 256}};
static int g_tuned[33][4];
static bool g_tuned_init = [] {
    for (int n = 0; n < 33; n++)
        for (int m = 0; m < 4; m++) g_tuned[n][m] = kTunedGB300[n][m];
    return true;
}();

// Lanes per matrix per (n, pivot mode), measured on GB300 by the autotuner
// (262,144 uniform matrices per size, eight against sixteen lanes, the same
// bits either way; eight where they were at least 2% faster); 0 =
// default_lanes.  Only n = 17..31 without partial pivoting have a
// choice (alt_lanes); mi_set_launch_lanes overrides entries at run time.
static const int kLanesGB300[33][4] = {
    {0, 0, 0, 0},
    {0, 0, 0, 0},
    {0, 0, 0, 0},
    {0, 0, 0, 0},
    {0, 0, 0, 0},
    {0, 0, 0, 0},
    {0, 0, 0, 0},
    {0, 0, 0, 0},
    {0, 0, 0, 0},
    {0, 0, 0, 0},
    {0, 0, 0, 0},
    {0, 0, 0, 0},
    {0, 0, 0, 0},
    {0, 0, 0, 0},
    {0, 0, 0, 0},
    {0, 0, 0, 0},
    {0, 0, 0, 0},
    {8, 8, 0, 0},
    {8, 8, 0, 0},
    {8, 8, 0, 0},
    {8, 8, 8, 0},
    {8, 0, 0, 0},
    {0, 0, 0, 0},
    {8, 0, 0, 0},
    {8, 0, 0, 0},
    {8, 8, 8, 0},
    {8, 8, 8, 0},
    {8, 8, 8, 0},
    {8, 8, 8, 0},
    {0, 0, 0, 0},
    {0, 0, 0, 0},
    {0, 0, 0, 0},
    {0, 0, 0, 0}};
static int g_lanes[33][4];
static bool g_lanes_init = [] {
    for (int n = 0; n < 33; n++)
        for (int m = 0; m < 4; m++) g_lanes[n][m] = kLanesGB300[n][m];
    return true;
}();

int tuned_lanes(int n, int mode) {
    const int l = (n >= 1 && n <= 32 && mode >= 0 && mode < 4) ? g_lanes[n][mode] : 0;
    return l > 0 ? l : default_lanes(n, mode);
}

int tuned_threads(int n, int mode) {
    const int t = (n >= 1 && n <= 32 && mode >= 0 && mode < 4) ? g_tuned[n][mode] : 0;
    return t > 0 ? t : kDefaultThreadsPerBlock;
}

int device_sm_count() {
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    if (dev >= 0 && dev < 64 && cached[dev] > 0) return cached[dev];
    int sms = 1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 1;
    if (dev >= 0 && dev < 64) cached[dev] = sms;
    return sms;
}

// Grid of a grid-stride kernel: as many blocks as are resident at once on the
// current device (at most `want`), so that no partial second wave runs after
// the first.  cache: one entry per device, 0 = not queried yet.
long long resident_grid(const void* kernel, int threads, long long want, int* cache) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = -1;
    int per_sm = (dev >= 0 && dev < 64) ? cache[dev] : 0;
    if (per_sm <= 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) != cudaSuccess || per_sm < 1)
            per_sm = 1;
        if (dev >= 0 && dev < 64) cache[dev] = per_sm;
    }
    const long long cap = (long long)per_sm * device_sm_count();
    return want < cap ? want : cap;
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

template <int N>
static void geom_of(int& lanes, int& mpw, int& smem_warp) {
    if constexpr (N <= tiny_max_contig<kModeReference>()) {     // one thread per matrix
        lanes = 1;
        mpw = 32;
        // staged through shared memory unless each thread moves its matrix
        // with 16-byte copies
        smem_warp = ((N * N) % 4 == 0 && N < kTinySlotMin) ? 0 : 32 * tiny_pitch<N>() * 4;
        return;
    }
    if constexpr (N == WideGeom::N) {                           // eight lanes, 16 x 8 register blocks
        lanes = WideGeom::L;
        mpw = WideGeom::M;
        smem_warp = WideGeom::kWarp * 4;
        return;
    }
    constexpr int L = default_lanes(N, kModeReference);
    lanes = L;
    mpw = Geom<N, L>::M;
    // two staged tiles plus the per-matrix scratch, per warp
    smem_warp = (int)(smem_bytes<N, L, kModeReference>(1) - 1024);
}

static bool query(int n, int& lanes, int& mpw, int& smem_warp) {
    switch (n) {
#define MI_Q(K) case K: geom_of<K>(lanes, mpw, smem_warp); return true;
        MI_Q(1) MI_Q(2) MI_Q(3) MI_Q(4) MI_Q(5) MI_Q(6) MI_Q(7) MI_Q(8)
        MI_Q(9) MI_Q(10) MI_Q(11) MI_Q(12) MI_Q(13) MI_Q(14) MI_Q(15) MI_Q(16)
        MI_Q(17) MI_Q(18) MI_Q(19) MI_Q(20) MI_Q(21) MI_Q(22) MI_Q(23) MI_Q(24)
        MI_Q(25) MI_Q(26) MI_Q(27) MI_Q(28) MI_Q(29) MI_Q(30) MI_Q(31) MI_Q(32)
#undef MI_Q
        default: return false;
    }
}

static_assert(kFormThread == MI_FORM_THREAD && kFormLanes == MI_FORM_LANES && kFormRows == MI_FORM_ROWS,
              "kernel form codes of the ABI");

// The threads-per-block knob as a contiguous call resolves it: 0 = the
// installed entry for (n, mode); rounded up to a multiple of 32, capped.
static int resolve_threads(int n, int mode, int threads_per_block) {
    int tpb = threads_per_block == 0 ? tuned_threads(n, mode) : threads_per_block;
    tpb = (tpb + 31) / 32 * 32;
    return tpb > kMaxThreadsPerBlock ? kMaxThreadsPerBlock : tpb;
}

template <int N>
static LaunchForm form_for_mode(int mode, long long batch, int tpb) {
    switch (mode) {
        case kModeNone: return launch_form<N, kModeNone>(batch, tpb);
        case kModeReference: return launch_form<N, kModeReference>(batch, tpb);
        case kModeReferenceSerial: return launch_form<N, kModeReferenceSerial>(batch, tpb);
        default: return launch_form<N, kModePartial>(batch, tpb);
    }
}

static bool query_launch(int n, int mode, long long batch, int tpb, LaunchForm& out) {
    switch (n) {
#define MI_L(K) case K: out = form_for_mode<K>(mode, batch, tpb); return true;
        MI_L(1) MI_L(2) MI_L(3) MI_L(4) MI_L(5) MI_L(6) MI_L(7) MI_L(8)
        MI_L(9) MI_L(10) MI_L(11) MI_L(12) MI_L(13) MI_L(14) MI_L(15) MI_L(16)
        MI_L(17) MI_L(18) MI_L(19) MI_L(20) MI_L(21) MI_L(22) MI_L(23) MI_L(24)
        MI_L(25) MI_L(26) MI_L(27) MI_L(28) MI_L(29) MI_L(30) MI_L(31) MI_L(32)
#undef MI_L
        default: return false;
    }
}

}  // namespace mi

extern "C" {

int mi_abi_version(void) { return MI_ABI_VERSION; }

const char* mi_error_string(int status) {
    switch (status) {
        case MI_OK: return "ok";
        case MI_ERR_INVALID_VALUE: return "invalid value (n outside 1..32, batch < 0, unknown pivot mode or bad knob)";
        case MI_ERR_NULL_POINTER: return "null matrix pointer with batch > 0";
        case MI_ERR_MISALIGNED: return "matrix pointer is not 4-byte aligned";
        case MI_ERR_CUDA: return "CUDA error (see mi_last_cuda_error)";
        case MI_ERR_SCRATCH_LIMIT: return "descriptor count above MI_NOALLOC_MAX_COUNT (262144) for the no-allocation entry point";
        default: return "unknown status";
    }
}

const char* mi_last_cuda_error(void) { return mi::g_last_cuda_error; }

int mi_query_config(int n, int* lanes_per_matrix, int* matrices_per_warp, int* smem_bytes_per_warp,
                    int* default_threads_per_block) {
    int lanes = 0, mpw = 0, smem = 0;
    if (!mi::query(n, lanes, mpw, smem)) return MI_ERR_INVALID_VALUE;
    if (lanes_per_matrix) *lanes_per_matrix = lanes;
    if (matrices_per_warp) *matrices_per_warp = mpw;
    if (smem_bytes_per_warp) *smem_bytes_per_warp = smem;
    if (default_threads_per_block) *default_threads_per_block = mi::kDefaultThreadsPerBlock;
    return MI_OK;
}

int mi_inverse_cfg_f32(float* d_a, int32_t* d_perm, int32_t* d_info, int64_t batch, int n, int pivot,
                       int threads_per_block, int grid_blocks, void* stream) {
    if (n < 1 || n > 32 || batch < 0 || threads_per_block < 0 || grid_blocks < 0) return MI_ERR_INVALID_VALUE;
    const mi::launch_fn* table = nullptr;
    switch (pivot) {
        case MI_PIVOT_NONE: table = mi::kTableNone; break;
        case MI_PIVOT_REFERENCE: table = mi::kTableReference; break;
        case MI_PIVOT_REFERENCE_SERIAL: table = mi::kTableReferenceSerial; break;
        case MI_PIVOT_PARTIAL: table = mi::kTablePartial; break;
        default: return MI_ERR_INVALID_VALUE;
    }
    if (batch == 0) return MI_OK;
    if (d_a == nullptr) return MI_ERR_NULL_POINTER;
    if ((reinterpret_cast<uintptr_t>(d_a) & 3u) != 0) return MI_ERR_MISALIGNED;
    const int tpb = mi::resolve_threads(n, pivot, threads_per_block);
    cudaError_t e = table[n](d_a, d_perm, d_info, (long long)batch, tpb, grid_blocks,
                             reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return mi::cuda_fail(e, "mi_inverse launch");
    return MI_OK;
}

int mi_device_error(int* flags, int clear) {
    int all = 0;
    std::lock_guard<std::mutex> lock(mi::error_readers_mu());
    for (mi::device_error_reader read : mi::error_readers()) {
        const cudaError_t e = read(&all, clear != 0);
        if (e != cudaSuccess) return mi::cuda_fail(e, "device error word");
    }
    if (flags) *flags = all;
    return MI_OK;
}

int mi_set_wait_test(int64_t wait_limit_cycles, int arm_without_copy) {
    const long long limit = wait_limit_cycles > 0 ? (long long)wait_limit_cycles : mi::kWaitLimit;
    std::lock_guard<std::mutex> lock(mi::error_readers_mu());
    for (mi::wait_test_setter set : mi::wait_test_setters()) {
        const cudaError_t e = set(limit, arm_without_copy != 0 ? 1 : 0);
        if (e != cudaSuccess) return mi::cuda_fail(e, "wait test hook");
    }
    return MI_OK;
}

int mi_query_launch(int n, int pivot, int64_t batch, int threads_per_block, int* form, int* lanes_per_matrix,
                    int* matrices_per_warp, int* threads_per_block_used) {
    if (n < 1 || n > 32 || pivot < MI_PIVOT_NONE || pivot > MI_PIVOT_PARTIAL || batch < 0 || threads_per_block < 0)
        return MI_ERR_INVALID_VALUE;
    mi::LaunchForm f{};
    if (!mi::query_launch(n, pivot, (long long)batch, mi::resolve_threads(n, pivot, threads_per_block), f))
        return MI_ERR_INVALID_VALUE;
    if (form) *form = f.form;
    if (lanes_per_matrix) *lanes_per_matrix = f.lanes;
    if (matrices_per_warp) *matrices_per_warp = f.mpw;
    if (threads_per_block_used) *threads_per_block_used = f.threads;
    return MI_OK;
}

int mi_inverse_f32(float* d_a, int32_t* d_perm, int32_t* d_info, int64_t batch, int n, int pivot,
                   void* stream) {
    return mi_inverse_cfg_f32(d_a, d_perm, d_info, batch, n, pivot, 0, 0, stream);
}

int mi_set_launch_config(int n, int pivot, int threads_per_block) {
    if (n < 1 || n > 32 || pivot < 0 || pivot > 3 || threads_per_block < 0 || threads_per_block > 256 ||
        threads_per_block % 32 != 0)
        return MI_ERR_INVALID_VALUE;
    mi::g_tuned[n][pivot] = threads_per_block ? threads_per_block : mi::kTunedGB300[n][pivot];
    return MI_OK;
}

int mi_get_launch_config(int n, int pivot, int* threads_per_block) {
    if (n < 1 || n > 32 || pivot < 0 || pivot > 3) return MI_ERR_INVALID_VALUE;
    if (threads_per_block) *threads_per_block = mi::tuned_threads(n, pivot);
    return MI_OK;
}

int mi_set_launch_lanes(int n, int pivot, int lanes_per_matrix) {
    if (n < 1 || n > 32 || pivot < 0 || pivot > 3 || lanes_per_matrix < 0) return MI_ERR_INVALID_VALUE;
    const int def = mi::default_lanes(n, pivot), alt = mi::alt_lanes(n, pivot);
    if (lanes_per_matrix != 0 && lanes_per_matrix != def && (alt == 0 || lanes_per_matrix != alt))
        return MI_ERR_INVALID_VALUE;
    mi::g_lanes[n][pivot] = lanes_per_matrix ? lanes_per_matrix : mi::kLanesGB300[n][pivot];
    return MI_OK;
}

int mi_get_launch_lanes(int n, int pivot, int* lanes_per_matrix, int* other) {
    if (n < 1 || n > 32 || pivot < 0 || pivot > 3) return MI_ERR_INVALID_VALUE;
    const int installed = mi::tuned_lanes(n, pivot), alt = mi::alt_lanes(n, pivot);
    if (lanes_per_matrix) *lanes_per_matrix = installed;
    if (other) *other = alt == 0 ? 0 : (installed == alt ? mi::default_lanes(n, pivot) : alt);
    return MI_OK;
}

}  // extern "C"
