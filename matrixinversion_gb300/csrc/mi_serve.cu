// mi_serve.cu -- the serving loop in native code (host side of the C ABI's
// mi_serve_run).  No counterpart in the reference, which inverts one
// pre-loaded batch per process.
//
// Requests (k matrices of one size n each) arrive at given times.  The loop
// runs on the calling thread without returning to the caller until every
// request has completed:
//
//   * admission: first come, first served; an arrived request is admitted
//     when the device pool (the HBM budget, carved once by the caller) has a
//     free extent for it (ExtentPool, first fit), and its host-to-device copy
//     goes out at once on the copy stream -- one copy for a run of requests
//     admitted together that follow each other both in the host ring and in
//     the pool;
//   * batching: whenever fewer than two batches are computing, every admitted
//     request not yet computed goes into one launch -- one descriptor call
//     over the pool (its matrices' offsets into the pool staged through a
//     pinned table), or one contiguous call for a batch of a single request;
//   * completion: results are copied back to their place in the host ring
//     on the copy-out stream, one copy (with an event of its own) per run of
//     a batch's requests that follow each other in the pool and in the ring;
//     when the loop sees that event it records those requests' completion
//     time and frees their extents, so a request's latency does not wait for
//     the rest of its batch to leave and its memory serves the next arrivals
//     at once.  (One copy per request made the loop issue-bound with host
//     copies.)
//
// With requests already in device memory (d_ring != NULL: an upstream device
// stage wrote them there; the caller counts that memory against its budget)
// there are no copies: batches are inverted in place and a request completes
// with its batch's kernels.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdint>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "mi_extents.h"
#include "mi_inverse.h"

namespace mi {
int set_cuda_error(cudaError_t e, const char* what);   // mi_api.cu
}

namespace {

constexpr int kInFlight = 2;   // batches computing at once (each owns one descriptor table)

size_t table_bytes(int64_t max_batch) { return ((size_t)max_batch * 16 + 255) & ~(size_t)255; }

// Pinned staging blocks kept across runs: pinning host memory just before a
// timed region was followed by stalled host-link copies in the bench's
// end-to-end steps, so a run takes a cached block that is large enough (or
// pins a new one) and returns it when it ends.  At most kStagingCache blocks
// stay pinned; the process's exit releases them.
constexpr size_t kStagingCache = 4;
std::mutex g_staging_mu;
std::vector<std::pair<void*, size_t>> g_staging;   // (block, bytes), free for reuse

cudaError_t staging_take(size_t bytes, void** out, size_t* got) {
    {
        std::lock_guard<std::mutex> lock(g_staging_mu);
        for (size_t i = 0; i < g_staging.size(); i++)
            if (g_staging[i].second >= bytes) {
                *out = g_staging[i].first;
                *got = g_staging[i].second;
                g_staging.erase(g_staging.begin() + (long)i);
                return cudaSuccess;
            }
    }
    *got = bytes;
    return cudaHostAlloc(out, bytes, cudaHostAllocPortable);   // any device's run may take it later
}

void staging_give(void* p, size_t bytes) {
    std::lock_guard<std::mutex> lock(g_staging_mu);
    if (g_staging.size() < kStagingCache) {
        g_staging.emplace_back(p, bytes);
        return;
    }
    cudaFreeHost(p);
}

// Streams, events and pinned staging of one run, released on every exit.
struct Resources {
    cudaStream_t h2d = nullptr, cmp = nullptr, d2h = nullptr;
    std::vector<cudaEvent_t> events;        // all events made, destroyed at the end
    std::vector<cudaEvent_t> spare;         // events free for reuse
    void* staging = nullptr;                // pinned: kInFlight descriptor tables
    size_t staging_bytes = 0;
    ~Resources() {
        for (cudaStream_t s : {h2d, cmp, d2h})
            if (s != nullptr) cudaStreamSynchronize(s);
        for (cudaEvent_t e : events) cudaEventDestroy(e);
        for (cudaStream_t s : {h2d, cmp, d2h})
            if (s != nullptr) cudaStreamDestroy(s);
        if (staging != nullptr) staging_give(staging, staging_bytes);
    }
    cudaError_t event(cudaEvent_t* out) {
        if (!spare.empty()) {
            *out = spare.back();
            spare.pop_back();
            return cudaSuccess;
        }
        cudaError_t e = cudaEventCreateWithFlags(out, cudaEventDisableTiming);
        if (e == cudaSuccess) events.push_back(*out);
        return e;
    }
};

struct Batch {
    int64_t first, last;    // requests [first, last), in arrival order
    cudaEvent_t done;       // the batch's kernels finished
};

}  // namespace

extern "C" {

size_t mi_serve_scratch_bytes(int64_t max_batch_matrices) {
    if (max_batch_matrices <= 0) return 0;
    return kInFlight * table_bytes(max_batch_matrices) + mi_descr_workspace_bytes(max_batch_matrices);
}

int mi_serve_run(int64_t num_requests, const double* arrival_s, const int64_t* k, const int32_t* n,
                 const int64_t* ring_off, const float* h_in, float* h_out, float* d_ring, float* d_pool,
                 int64_t pool_floats, void* d_scratch, size_t scratch_bytes, int64_t max_batch_matrices, int pivot,
                 int coalesce, double* latency_s, double* wall_s, int64_t* stats) {
    if (num_requests < 0 || max_batch_matrices <= 0 || pivot < MI_PIVOT_NONE || pivot > MI_PIVOT_PARTIAL)
        return MI_ERR_INVALID_VALUE;
    if (num_requests == 0) return MI_OK;
    const bool resident = d_ring != nullptr;
    if (arrival_s == nullptr || k == nullptr || n == nullptr || ring_off == nullptr || latency_s == nullptr ||
        d_scratch == nullptr || (!resident && (h_in == nullptr || h_out == nullptr || d_pool == nullptr)))
        return MI_ERR_NULL_POINTER;
    if (scratch_bytes < mi_serve_scratch_bytes(max_batch_matrices) ||
        (reinterpret_cast<uintptr_t>(d_scratch) & 255u) != 0)
        return MI_ERR_INVALID_VALUE;
    // every request must be well-formed, fit one batch, and (with copies) fit the pool
    std::vector<int64_t> len(num_requests);
    for (int64_t r = 0; r < num_requests; r++) {
        if (n[r] < 1 || n[r] > 32 || k[r] < 1 || k[r] > max_batch_matrices || ring_off[r] < 0 ||
            (r > 0 && arrival_s[r] < arrival_s[r - 1]))
            return MI_ERR_INVALID_VALUE;
        len[r] = (k[r] * n[r] * n[r] + 3) / 4 * 4;          // 16-byte aligned extents
        if (!resident && len[r] > pool_floats) return MI_ERR_SCRATCH_LIMIT;
    }

    Resources res;
    cudaError_t e = cudaStreamCreateWithFlags(&res.h2d, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&res.cmp, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&res.d2h, cudaStreamNonBlocking);
    const size_t tb = table_bytes(max_batch_matrices);
    if (e == cudaSuccess) e = staging_take(kInFlight * tb, &res.staging, &res.staging_bytes);
    if (e != cudaSuccess) return mi::set_cuda_error(e, "serving set-up");
    unsigned char* scratch = static_cast<unsigned char*>(d_scratch);
    void* workspace = scratch + kInFlight * tb;
    const size_t ws_bytes = scratch_bytes - kInFlight * tb;
    float* base = resident ? d_ring : d_pool;
    const int64_t base_floats = resident ? INT64_MAX / 2 : pool_floats;

    mi::ExtentPool pool(resident ? 0 : pool_floats);
    constexpr int64_t kRunFloats = int64_t(1) << 24;       // the longest copy in: 64 MB
    std::vector<int64_t> ext(num_requests, -1);            // pool extent of each admitted request
    std::vector<double> done(num_requests, -1.0);
    std::deque<Batch> computing;
    // results on their way to the host ring: requests [first, last) of one copy
    struct Leaving {
        int64_t first, last;
        cudaEvent_t home;
    };
    std::deque<Leaving> leaving;
    // inputs on their way in: requests before `end` are on the device once the event has fired
    std::deque<std::pair<int64_t, cudaEvent_t>> arriving;
    int64_t admitted = 0, launched = 0, completed = 0, batches = 0, tables_used = 0;

    const auto t0 = std::chrono::steady_clock::now();
    auto now = [&] { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); };

    auto fail = [&](cudaError_t err, const char* what) { return mi::set_cuda_error(err, what); };

    while (completed < num_requests) {
        const double t = now();
        bool idle = true;
        // ---- completions: results home (per request), batches finished
        while (!leaving.empty()) {
            const cudaError_t q = cudaEventQuery(leaving.front().home);
            if (q == cudaErrorNotReady) break;
            if (q != cudaSuccess) return fail(q, "serving: result copy");
            for (int64_t r = leaving.front().first; r < leaving.front().last; r++) {
                done[r] = t;
                pool.release(ext[r], len[r]);
                completed++;
            }
            res.spare.push_back(leaving.front().home);
            leaving.pop_front();
            idle = false;
        }
        while (!computing.empty()) {
            const cudaError_t q = cudaEventQuery(computing.front().done);
            if (q == cudaErrorNotReady) break;
            if (q != cudaSuccess) return fail(q, "serving: batch");
            if (resident) {
                for (int64_t r = computing.front().first; r < computing.front().last; r++) done[r] = t;
                completed += computing.front().last - computing.front().first;
            }
            res.spare.push_back(computing.front().done);
            computing.pop_front();
            idle = false;
        }
        // ---- admission: arrived requests, first come first served, as extents free.
        // Requests that follow each other both in the host ring and in the pool
        // (offset + padded length = the next offset, on both sides) go in by one
        // copy; the padding it carries lies inside the ring and the extent.
        // A copy covers at most kRunFloats (64 MB) and records an event, so a
        // batch waits only for the copies of its own requests.
        int64_t run = -1;                                    // first request of the pending copy
        auto flush_in = [&](int64_t end) -> cudaError_t {   // copy requests [run, end)
            if (run < 0 || end <= run) return cudaSuccess;
            const int64_t last = end - 1;
            const int64_t floats = ring_off[last] - ring_off[run] + k[last] * n[last] * n[last];
            cudaError_t err = cudaMemcpyAsync(d_pool + ext[run], h_in + ring_off[run], (size_t)floats * sizeof(float),
                                              cudaMemcpyHostToDevice, res.h2d);
            cudaEvent_t in = nullptr;
            if (err == cudaSuccess) err = res.event(&in);
            if (err == cudaSuccess) err = cudaEventRecord(in, res.h2d);
            if (err == cudaSuccess) arriving.emplace_back(end, in);
            run = -1;
            return err;
        };
        while (admitted < num_requests && arrival_s[admitted] <= t) {
            if (!resident) {
                const int64_t off = pool.alloc(len[admitted]);
                if (off < 0) break;                          // wait for memory, keep the order
                ext[admitted] = off;
                const int64_t prev = admitted - 1;
                const bool joins = run >= 0 && ring_off[admitted] == ring_off[prev] + len[prev] &&
                                   off == ext[prev] + len[prev] &&
                                   ring_off[admitted] + k[admitted] * n[admitted] * n[admitted] - ring_off[run] <=
                                       kRunFloats;
                if (!joins) {
                    if ((e = flush_in(admitted)) != cudaSuccess) return fail(e, "serving: request copy");
                    run = admitted;
                }
            } else {
                ext[admitted] = ring_off[admitted];
            }
            admitted++;
            idle = false;
        }
        if ((e = flush_in(admitted)) != cudaSuccess) return fail(e, "serving: request copy");
        // ---- batching: every admitted request not yet computed, into one launch
        if (launched < admitted && (int)computing.size() < kInFlight) {
            int64_t last = launched, mats = 0;
            uint32_t n_mask = 0;
            while (last < admitted && mats + k[last] <= max_batch_matrices && (coalesce || last == launched)) {
                mats += k[last];
                n_mask |= 1u << (n[last] - 1);
                last++;
            }
            if (!resident) {
                // the copy that brings in the batch's last request (the copies
                // before it precede it on the copy stream); copies that end at
                // or before this batch's end are not needed by later batches
                auto it = arriving.begin();
                while (it != arriving.end() && it->first < last) ++it;
                if (it == arriving.end()) return fail(cudaErrorUnknown, "serving: batch inputs");
                if ((e = cudaStreamWaitEvent(res.cmp, it->second, 0)) != cudaSuccess)
                    return fail(e, "serving: batch inputs");
                while (!arriving.empty() && arriving.front().first <= last) {
                    res.spare.push_back(arriving.front().second);   // waited on in stream order: free for reuse
                    arriving.pop_front();
                }
            }
            int status = MI_OK;
            if (last - launched == 1) {
                status = mi_inverse_f32(base + ext[launched], nullptr, nullptr, k[launched], n[launched], pivot, res.cmp);
            } else {
                const int buf = (int)(tables_used++ % kInFlight);   // free: its batch finished (at most 2 in flight)
                // the table of this batch's mats matrices, packed: offsets, sizes, flags
                unsigned char* hs = static_cast<unsigned char*>(res.staging) + buf * tb;
                int64_t* hoff = reinterpret_cast<int64_t*>(hs);
                int32_t* hn = reinterpret_cast<int32_t*>(hs + 8 * (size_t)mats);
                int32_t* hf = reinterpret_cast<int32_t*>(hs + 12 * (size_t)mats);
                int64_t m = 0;
                for (int64_t r = launched; r < last; r++) {
                    const int64_t nn = (int64_t)n[r] * n[r];
                    for (int64_t i = 0; i < k[r]; i++, m++) {
                        hoff[m] = ext[r] + i * nn;
                        hn[m] = n[r];
                        hf[m] = pivot;
                    }
                }
                unsigned char* ds = scratch + buf * tb;
                e = cudaMemcpyAsync(ds, hs, 16 * (size_t)m, cudaMemcpyHostToDevice, res.cmp);
                if (e != cudaSuccess) return fail(e, "serving: descriptor table");
                status = mi_inverse_descr_f32(base, base_floats, reinterpret_cast<int64_t*>(ds),
                                              reinterpret_cast<int32_t*>(ds + 8 * (size_t)m),
                                              reinterpret_cast<int32_t*>(ds + 12 * (size_t)m), nullptr, nullptr, m,
                                              n_mask, 1u << pivot, workspace, ws_bytes, res.cmp);
            }
            if (status != MI_OK) return status;
            Batch b{launched, last, nullptr};
            if ((e = res.event(&b.done)) != cudaSuccess || (e = cudaEventRecord(b.done, res.cmp)) != cudaSuccess)
                return fail(e, "serving: batch event");
            if (!resident) {
                if ((e = cudaStreamWaitEvent(res.d2h, b.done, 0)) != cudaSuccess) return fail(e, "serving: results");
                // results out by one copy per run of requests that follow each
                // other in the pool and in the ring; each run completes at its
                // copy's event
                for (int64_t r0 = launched; r0 < last;) {
                    int64_t r1 = r0 + 1;
                    while (r1 < last && ring_off[r1] == ring_off[r1 - 1] + len[r1 - 1] &&
                           ext[r1] == ext[r1 - 1] + len[r1 - 1])
                        r1++;
                    const int64_t floats = ring_off[r1 - 1] - ring_off[r0] + k[r1 - 1] * n[r1 - 1] * n[r1 - 1];
                    cudaEvent_t home = nullptr;
                    if ((e = cudaMemcpyAsync(h_out + ring_off[r0], d_pool + ext[r0], (size_t)floats * sizeof(float),
                                             cudaMemcpyDeviceToHost, res.d2h)) != cudaSuccess ||
                        (e = res.event(&home)) != cudaSuccess || (e = cudaEventRecord(home, res.d2h)) != cudaSuccess)
                        return fail(e, "serving: result copy");
                    leaving.push_back({r0, r1, home});
                    r0 = r1;
                }
            }
            computing.push_back(b);
            launched = last;
            batches++;
            idle = false;
        }
        if (idle) std::this_thread::yield();
    }
    double wall = 0.0;
    for (int64_t r = 0; r < num_requests; r++) {
        latency_s[r] = done[r] - arrival_s[r];
        wall = done[r] > wall ? done[r] : wall;
    }
    if (wall_s != nullptr) *wall_s = wall;
    if (stats != nullptr) {
        stats[0] = batches;
        stats[1] = pool.peak();
    }
    return MI_OK;
}

}  // extern "C"
