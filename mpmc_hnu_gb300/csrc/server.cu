// Flash server (include/mpmc_gb300_flash.h, "Flash server"): continuous
// batching of PT flash requests on one GPU.
//
// One worker thread owns the device side.  Each slot is a CUDA stream with
// device buffers for max_batch_cells cells (inputs, flash outputs, mixed-form
// workspace) and pinned host staging.  A request becomes one or more tasks:
// a request of at most policy.chunk_cells cells is one task, a larger one is
// cut into chunks of that size, so no launch keeps the device for long and the
// chunks of large requests interleave with other work.  Tasks of requests of
// at most policy.small_request_cells cells wait in the latency queue, the
// others in the throughput queue.  The worker loop
//   1. retires slots whose completion event has fired, scattering each task's
//      rows out of the batch into its request's buffers; a request completes
//      when its last task does;
//   2. drops waiting tasks whose request's deadline has passed (the request
//      completes with MPMC_ERR_DEADLINE, its outputs untouched);
//   3. fills free slots: the latency slots (the highest stream priority) take
//      only latency-queue tasks, the oldest first plus every other waiting
//      latency task of the same mixture that fits policy.latency_batch_cells;
//      the throughput slots take the oldest throughput task plus others of
//      its mixture up to max_batch_cells, or latency tasks when no throughput
//      work waits;
//   4. sleeps on the queue's condition variable when there is nothing to do,
//      or polls the busy slots at a short interval.
// With MPMC_SERVER_WARM_CACHE each mixture keeps, on the device, the ln K of
// recently solved two-phase cells in a table keyed by the cell's composition;
// a cell of a later request with the same composition and a nearby (p, T)
// starts from it (mpmc_gpu_flash_solve_device_warm's warm start).  Without
// it every cell's result depends only on its own inputs, so the batching
// never changes a result.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/mpmc_gb300_flash.h"
#include "launch.h"

namespace {

using Clock = std::chrono::steady_clock;
using pr76::host::cuda_fail;
using pr76::host::fail;

constexpr int kFlashFields = 10;  // status .. counters of mpmc_flash_outputs
constexpr int kMaxMixtures = 64;
// warm-start cache: entries per mixture (a power of two) and the (p, T)
// window in which a cached ln K is used as a start
constexpr int kCacheEntries = 1 << 16;
constexpr double kCacheLnP = 0.25;
constexpr double kCacheT = 15.0;

int field_rows(int k, int n) {
    switch (k) {
    case 0: case 1: case 7: case 8: return 1;
    case 9: return MPMC_COUNTER_COUNT;
    default: return n;
    }
}
size_t field_elem(int k) { return (k == 0 || k == 9) ? 4 : 8; }

struct Request {
    uint64_t ticket = 0;
    int mixture = 0;
    int64_t ncell = 0;
    const double *p = nullptr, *t = nullptr, *z = nullptr;
    void* out[kFlashFields] = {};
    Clock::time_point submitted, finished, deadline;
    bool has_deadline = false;
    int tasks_left = 0;
    int state = 0;  // 0 waiting, 1 on the device, 2 done
    int error = MPMC_OK;
};

// A range of a request's cells, solved in one batch.
struct Task {
    std::shared_ptr<Request> req;
    int64_t lo = 0, hi = 0;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    bool latency = false;  // serves the latency queue only
    double *d_p = nullptr, *d_t = nullptr, *d_z = nullptr, *d_warm = nullptr;
    void* d_out[kFlashFields] = {};
    void* d_ws = nullptr;
    size_t ws_bytes = 0;
    double *h_p = nullptr, *h_t = nullptr, *h_z = nullptr;
    void* h_out[kFlashFields] = {};
    unsigned long long* d_hits = nullptr;  // warm starts found in the cache (last batch)
    unsigned long long* h_hits = nullptr;
    bool warm_launched = false;
    std::vector<Task> batch;
    std::vector<int64_t> offsets;
    int mixture = -1;
    int64_t cells = 0;
    bool busy = false;
};

// One cached solution: the composition's hash (twice, written last and first,
// so a reader sees a consistent entry), p, T and ln K.
struct CacheTable {
    unsigned long long* key0 = nullptr;  // [kCacheEntries]
    unsigned long long* key1 = nullptr;  // [kCacheEntries]
    double* pt = nullptr;                // [2 * kCacheEntries]
    double* lnk = nullptr;               // [n * kCacheEntries]
};

struct MixtureEntry {
    int n = 0;
    pr76::Mixture* d_mix = nullptr;
    CacheTable cache;
};

}  // namespace

struct mpmc_flash_server {
    int device = 0;
    int form = MPMC_FORM_MIXED;
    int64_t cap = 65536;
    int nmax = MPMC_MAX_COMPONENTS;
    bool warm_cache = false;
    mpmc_server_policy policy{};
    std::vector<Slot> slots;
    size_t slot_bytes = 0;
    std::vector<MixtureEntry> mixtures;

    std::mutex mu;
    std::condition_variable work_cv;  // worker: new request or stop
    std::condition_variable done_cv;  // waiters: a request finished
    std::deque<Task> latency_q, throughput_q;
    std::unordered_map<uint64_t, std::shared_ptr<Request>> tickets;
    uint64_t next_ticket = 1;
    int64_t in_flight = 0;  // submitted and not completed
    bool stop = false;
    std::thread worker;

    int64_t submitted = 0, completed = 0, batches = 0, cells = 0, most_in_batch = 0, most_busy = 0;
    int64_t rejected_busy = 0, expired = 0, warm_cells = 0;
};

namespace {

// ---- warm-start cache kernels ----
__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// Hash of a cell's composition bits; never 0 (0 marks an empty entry).
__device__ __forceinline__ unsigned long long composition_key(const double* z, int n, int64_t ncell, int64_t c) {
    unsigned long long h = 0x632BE59BD9B4E019ull;
    for (int i = 0; i < n; ++i) h = mix64(h ^ static_cast<unsigned long long>(__double_as_longlong(z[i * ncell + c])));
    return h ? h : 1ull;
}

// ln K starts for a batch: a cell whose composition is in the table, solved at
// a (p, T) within the window, starts from the cached ln K; every other cell
// gets NaN (cold).
__global__ void cache_lookup_kernel(CacheTable tab, int n, int64_t ncell, const double* __restrict__ p,
                                    const double* __restrict__ t, const double* __restrict__ z, double* warm,
                                    unsigned long long* hits) {
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; c < ncell;
         c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const unsigned long long key = composition_key(z, n, ncell, c);
        const int e = static_cast<int>(key & (kCacheEntries - 1));
        bool use = false;
        double lk[MPMC_MAX_COMPONENTS];
        const unsigned long long k1 = *(volatile unsigned long long*)&tab.key1[e];
        if (k1 == key) {
            __threadfence();
            // L2 reads: entries are rewritten by other streams' insert kernels
            const double pe = __ldcg(&tab.pt[2 * e]), te = __ldcg(&tab.pt[2 * e + 1]);
            for (int i = 0; i < n; ++i) lk[i] = __ldcg(&tab.lnk[static_cast<int64_t>(i) * kCacheEntries + e]);
            __threadfence();
            const unsigned long long k0 = *(volatile unsigned long long*)&tab.key0[e];
            use = k0 == key && fabs(log(p[c] / pe)) <= kCacheLnP && fabs(t[c] - te) <= kCacheT;
        }
        for (int i = 0; i < n; ++i) warm[i * ncell + c] = use ? lk[i] : nan;
        if (use) atomicAdd(hits, 1ull);
    }
}

// Stores the ln K of every two-phase cell of a finished batch (overwriting
// whatever shared its entry): key1 is cleared first and key0 / key1 set last,
// so a concurrent lookup either sees the old entry, the new one, or a miss.
__global__ void cache_insert_kernel(CacheTable tab, int n, int64_t ncell, const double* __restrict__ p,
                                    const double* __restrict__ t, const double* __restrict__ z,
                                    const int32_t* __restrict__ status, const double* __restrict__ lnk) {
    for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; c < ncell;
         c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (status[c] != pr76::kTwoPhase) continue;
        const unsigned long long key = composition_key(z, n, ncell, c);
        const int e = static_cast<int>(key & (kCacheEntries - 1));
        *(volatile unsigned long long*)&tab.key1[e] = 0ull;
        *(volatile unsigned long long*)&tab.key0[e] = 0ull;
        __threadfence();
        tab.pt[2 * e] = p[c];
        tab.pt[2 * e + 1] = t[c];
        for (int i = 0; i < n; ++i) tab.lnk[static_cast<int64_t>(i) * kCacheEntries + e] = lnk[i * ncell + c];
        __threadfence();
        *(volatile unsigned long long*)&tab.key0[e] = key;
        __threadfence();
        *(volatile unsigned long long*)&tab.key1[e] = key;
    }
}

size_t cache_bytes(int n) {
    return static_cast<size_t>(kCacheEntries) * (2 * sizeof(unsigned long long) + 2 * sizeof(double) +
                                                 static_cast<size_t>(n) * sizeof(double));
}

void release_slot(Slot& s) {
    if (s.stream) cudaStreamSynchronize(s.stream);
    cudaFree(s.d_p);
    cudaFree(s.d_t);
    cudaFree(s.d_z);
    cudaFree(s.d_warm);
    cudaFree(s.d_hits);
    cudaFreeHost(s.h_hits);
    for (auto* ptr : s.d_out) cudaFree(ptr);
    cudaFree(s.d_ws);
    cudaFreeHost(s.h_p);
    cudaFreeHost(s.h_t);
    cudaFreeHost(s.h_z);
    for (auto* ptr : s.h_out) cudaFreeHost(ptr);
    if (s.done) cudaEventDestroy(s.done);
    if (s.stream) cudaStreamDestroy(s.stream);
    s = Slot{};
}

cudaError_t allocate_slot(mpmc_flash_server* sv, Slot& s, int priority) {
    const size_t cap = static_cast<size_t>(sv->cap), nmax = static_cast<size_t>(sv->nmax);
    cudaError_t e;
    if ((e = cudaStreamCreateWithPriority(&s.stream, cudaStreamNonBlocking, priority)) != cudaSuccess) return e;
    if ((e = cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&s.d_p, cap * 8)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&s.d_t, cap * 8)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&s.d_z, nmax * cap * 8)) != cudaSuccess) return e;
    if (sv->warm_cache) {
        if ((e = cudaMalloc(&s.d_warm, nmax * cap * 8)) != cudaSuccess) return e;
        if ((e = cudaMalloc(&s.d_hits, sizeof(unsigned long long))) != cudaSuccess) return e;
        if ((e = cudaMallocHost(&s.h_hits, sizeof(unsigned long long))) != cudaSuccess) return e;
    }
    if ((e = cudaMallocHost(&s.h_p, cap * 8)) != cudaSuccess) return e;
    if ((e = cudaMallocHost(&s.h_t, cap * 8)) != cudaSuccess) return e;
    if ((e = cudaMallocHost(&s.h_z, nmax * cap * 8)) != cudaSuccess) return e;
    for (int k = 0; k < kFlashFields; ++k) {
        const size_t bytes = static_cast<size_t>(field_rows(k, sv->nmax)) * cap * field_elem(k);
        if ((e = cudaMalloc(&s.d_out[k], bytes)) != cudaSuccess) return e;
        if ((e = cudaMallocHost(&s.h_out[k], bytes)) != cudaSuccess) return e;
    }
    if (sv->form == MPMC_FORM_MIXED) {
        s.ws_bytes = pr76::batched_workspace_bytes(sv->nmax, sv->cap);
        if ((e = cudaMalloc(&s.d_ws, s.ws_bytes)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

size_t slot_device_bytes(const mpmc_flash_server* sv) {
    const size_t cap = static_cast<size_t>(sv->cap);
    size_t bytes = (2 + static_cast<size_t>(sv->nmax)) * cap * 8;
    if (sv->warm_cache) bytes += static_cast<size_t>(sv->nmax) * cap * 8;
    for (int k = 0; k < kFlashFields; ++k) bytes += static_cast<size_t>(field_rows(k, sv->nmax)) * cap * field_elem(k);
    if (sv->form == MPMC_FORM_MIXED) bytes += pr76::batched_workspace_bytes(sv->nmax, sv->cap);
    return bytes;
}

// Copy a batch in, launch, copy out (worker thread, device current).
int launch_batch(mpmc_flash_server* sv, Slot& s) {
    const MixtureEntry& mx = sv->mixtures[s.mixture];
    const int n = mx.n;
    const int64_t C = s.cells;
    const size_t cb = static_cast<size_t>(C);
    for (size_t r = 0; r < s.batch.size(); ++r) {
        const Task& tk = s.batch[r];
        const Request& q = *tk.req;
        const size_t off = static_cast<size_t>(s.offsets[r]), nc = static_cast<size_t>(tk.hi - tk.lo);
        const size_t lo = static_cast<size_t>(tk.lo), rn = static_cast<size_t>(q.ncell);
        std::memcpy(s.h_p + off, q.p + lo, nc * 8);
        std::memcpy(s.h_t + off, q.t + lo, nc * 8);
        for (int i = 0; i < n; ++i) std::memcpy(s.h_z + static_cast<size_t>(i) * cb + off, q.z + i * rn + lo, nc * 8);
    }
    cudaError_t e;
    if ((e = cudaMemcpyAsync(s.d_p, s.h_p, cb * 8, cudaMemcpyHostToDevice, s.stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(s.d_t, s.h_t, cb * 8, cudaMemcpyHostToDevice, s.stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(s.d_z, s.h_z, static_cast<size_t>(n) * cb * 8, cudaMemcpyHostToDevice, s.stream)) !=
            cudaSuccess)
        return cuda_fail(e, "server copy-in");
    pr76::DeviceOutputs d{};
    d.status = static_cast<int32_t*>(s.d_out[0]);
    d.beta = static_cast<double*>(s.d_out[1]);
    d.x = static_cast<double*>(s.d_out[2]);
    d.y = static_cast<double*>(s.d_out[3]);
    d.lnk = static_cast<double*>(s.d_out[4]);
    d.lnphi_l = static_cast<double*>(s.d_out[5]);
    d.lnphi_v = static_cast<double*>(s.d_out[6]);
    d.z_l = static_cast<double*>(s.d_out[7]);
    d.z_v = static_cast<double*>(s.d_out[8]);
    d.counters = static_cast<int32_t*>(s.d_out[9]);
    const bool warm = sv->warm_cache && sv->form == MPMC_FORM_MIXED && mx.cache.key0;
    const unsigned grid = static_cast<unsigned>(std::min<int64_t>((C + 255) / 256, 1024));
    s.warm_launched = warm;
    if (warm) {
        if ((e = cudaMemsetAsync(s.d_hits, 0, sizeof(unsigned long long), s.stream)) != cudaSuccess)
            return cuda_fail(e, "server cache lookup");
        cache_lookup_kernel<<<grid, 256, 0, s.stream>>>(mx.cache, n, C, s.d_p, s.d_t, s.d_z, s.d_warm, s.d_hits);
    }
    if (sv->form == MPMC_FORM_MIXED) {
        pr76::BatchedShape shape{0, 0, 0, 0, 0, nullptr, 0, 0.0f, 0};
        shape.warm_lnk = warm ? s.d_warm : nullptr;
        e = pr76::launch_batched(n, mx.d_mix, C, s.d_p, s.d_t, s.d_z, d, s.d_ws, s.ws_bytes, shape, s.stream);
    } else {
        e = pr76::launch_plain(n, mx.d_mix, C, s.d_p, s.d_t, s.d_z, d, s.stream);
    }
    if (e != cudaSuccess) return cuda_fail(e, "server flash launch");
    if (warm) {
        cache_insert_kernel<<<grid, 256, 0, s.stream>>>(mx.cache, n, C, s.d_p, s.d_t, s.d_z, d.status, d.lnk);
        if ((e = cudaMemcpyAsync(s.h_hits, s.d_hits, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                 s.stream)) != cudaSuccess)
            return cuda_fail(e, "server cache counter");
    }
    for (int k = 0; k < kFlashFields; ++k) {
        const size_t bytes = static_cast<size_t>(field_rows(k, n)) * cb * field_elem(k);
        if ((e = cudaMemcpyAsync(s.h_out[k], s.d_out[k], bytes, cudaMemcpyDeviceToHost, s.stream)) != cudaSuccess)
            return cuda_fail(e, "server copy-out");
    }
    if ((e = cudaEventRecord(s.done, s.stream)) != cudaSuccess) return cuda_fail(e, "server event");
    return MPMC_OK;
}

// Scatter a finished task to its request (worker thread, no lock held).
void scatter(const mpmc_flash_server* sv, const Slot& s, size_t r) {
    const int n = sv->mixtures[s.mixture].n;
    const size_t cb = static_cast<size_t>(s.cells);
    const Task& tk = s.batch[r];
    const Request& q = *tk.req;
    const size_t off = static_cast<size_t>(s.offsets[r]), nc = static_cast<size_t>(tk.hi - tk.lo);
    const size_t lo = static_cast<size_t>(tk.lo), rn = static_cast<size_t>(q.ncell);
    for (int k = 0; k < kFlashFields; ++k) {
        if (!q.out[k]) continue;
        const size_t el = field_elem(k);
        const char* src = static_cast<const char*>(s.h_out[k]);
        char* dst = static_cast<char*>(q.out[k]);
        for (int row = 0; row < field_rows(k, n); ++row)
            std::memcpy(dst + (static_cast<size_t>(row) * rn + lo) * el, src + (static_cast<size_t>(row) * cb + off) * el,
                        nc * el);
    }
}

// A task of `q` finished (or was dropped) with `err`: the request completes
// with its last task.  Call with the lock held.
void finish_task(mpmc_flash_server* sv, const std::shared_ptr<Request>& q, int err, Clock::time_point now) {
    if (err != MPMC_OK && q->error == MPMC_OK) q->error = err;
    if (--q->tasks_left > 0) return;
    q->state = 2;
    q->finished = now;
    ++sv->completed;
    --sv->in_flight;
}

// Drops the waiting tasks of requests whose deadline has passed (lock held).
void expire(mpmc_flash_server* sv, std::deque<Task>& q, Clock::time_point now, bool& any) {
    for (auto it = q.begin(); it != q.end();) {
        if (it->req->has_deadline && now >= it->req->deadline) {
            const bool first = it->req->error == MPMC_OK;
            finish_task(sv, it->req, MPMC_ERR_DEADLINE, now);
            if (first) ++sv->expired;
            any = true;
            it = q.erase(it);
        } else {
            ++it;
        }
    }
}

// Takes the oldest task of `q` and every later task of its mixture that fits
// in `limit` cells into the slot (lock held).
void take_batch(Slot& s, std::deque<Task>& q, int64_t limit) {
    const int mix = q.front().req->mixture;
    int64_t cells = 0;
    for (auto it = q.begin(); it != q.end();) {
        const int64_t nc = it->hi - it->lo;
        if (it->req->mixture == mix && cells + nc <= limit) {
            s.offsets.push_back(cells);
            cells += nc;
            it->req->state = 1;
            s.batch.push_back(*it);
            it = q.erase(it);
        } else {
            ++it;
        }
    }
    s.mixture = mix;
    s.cells = cells;
}

void worker_loop(mpmc_flash_server* sv) {
    cudaSetDevice(sv->device);
    for (;;) {
        // 1. retire finished slots
        for (Slot& s : sv->slots) {
            if (!s.busy) continue;
            const cudaError_t q = cudaEventQuery(s.done);
            if (q == cudaErrorNotReady) continue;
            int err = MPMC_OK;
            if (q != cudaSuccess) err = cuda_fail(q, "server batch");
            const auto now = Clock::now();
            std::vector<int> late(s.batch.size(), 0);
            for (size_t r = 0; r < s.batch.size(); ++r) {
                const Request& rq = *s.batch[r].req;
                // the reference publishes nothing once the deadline has passed
                late[r] = rq.has_deadline && now >= rq.deadline;
                if (err == MPMC_OK && !late[r]) scatter(sv, s, r);
            }
            {
                std::lock_guard<std::mutex> lock(sv->mu);
                if (s.warm_launched && err == MPMC_OK) sv->warm_cells += static_cast<int64_t>(*s.h_hits);
                for (size_t r = 0; r < s.batch.size(); ++r) {
                    const auto& rq = s.batch[r].req;
                    if (late[r] && rq->error == MPMC_OK) ++sv->expired;
                    finish_task(sv, rq, err != MPMC_OK ? err : (late[r] ? MPMC_ERR_DEADLINE : MPMC_OK), now);
                }
            }
            sv->done_cv.notify_all();
            s.batch.clear();
            s.offsets.clear();
            s.busy = false;
        }
        // 2-3. drop expired tasks, fill free slots
        bool any_busy = false;
        {
            std::unique_lock<std::mutex> lock(sv->mu);
            bool dropped = false;
            const auto now = Clock::now();
            expire(sv, sv->latency_q, now, dropped);
            expire(sv, sv->throughput_q, now, dropped);
            if (dropped) sv->done_cv.notify_all();
            int busy = 0;
            for (const Slot& s : sv->slots) busy += s.busy;
            for (Slot& s : sv->slots) {
                if (s.busy) continue;
                if (s.latency) {
                    if (sv->latency_q.empty()) continue;
                    take_batch(s, sv->latency_q, std::min<int64_t>(sv->cap, sv->policy.latency_batch_cells));
                } else if (!sv->throughput_q.empty()) {
                    take_batch(s, sv->throughput_q, sv->cap);
                } else if (!sv->latency_q.empty()) {
                    take_batch(s, sv->latency_q, sv->cap);
                } else {
                    continue;
                }
                s.busy = true;
                ++busy;
                ++sv->batches;
                sv->cells += s.cells;
                sv->most_in_batch = std::max<int64_t>(sv->most_in_batch, static_cast<int64_t>(s.batch.size()));
                sv->most_busy = std::max<int64_t>(sv->most_busy, busy);
                lock.unlock();
                const int rc = launch_batch(sv, s);
                lock.lock();
                if (rc != MPMC_OK) {
                    // nothing is in flight on the stream's event: fail the batch now
                    for (auto& tk : s.batch) finish_task(sv, tk.req, rc, Clock::now());
                    s.batch.clear();
                    s.offsets.clear();
                    s.busy = false;
                    sv->done_cv.notify_all();
                }
            }
            for (const Slot& s : sv->slots) any_busy = any_busy || s.busy;
            const bool waiting = !sv->latency_q.empty() || !sv->throughput_q.empty();
            if (sv->stop && !waiting && !any_busy) return;
            if (!any_busy && !waiting) {
                sv->work_cv.wait(lock, [&] {
                    return sv->stop || !sv->latency_q.empty() || !sv->throughput_q.empty();
                });
                continue;
            }
        }
        // 4. slots busy or tasks waiting for a slot: poll again shortly
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

int submit_request(mpmc_flash_server* sv, int32_t mixture_id, int64_t n_cells, const double* p, const double* t,
                   const double* z, const mpmc_flash_outputs* out, int64_t deadline_us, uint64_t* ticket) {
    if (!sv || !ticket || !out) return fail(MPMC_ERR_INVALID_ARGUMENT, "null argument");
    if (n_cells < 1 || n_cells > sv->policy.max_request_cells)
        return fail(MPMC_ERR_INVALID_ARGUMENT, "request cell count must be in [1, max_request_cells]");
    if (!p || !t || !z) return fail(MPMC_ERR_INVALID_ARGUMENT, "p, t and z must not be null");
    const void* const* fields = reinterpret_cast<const void* const*>(out);
    for (int k = kFlashFields; k < static_cast<int>(sizeof(mpmc_flash_outputs) / sizeof(void*)); ++k)
        if (fields[k]) return fail(MPMC_ERR_UNSUPPORTED, "the server returns flash fields only (no sensitivities)");
    if (deadline_us == 0 || deadline_us < -1)
        return fail(MPMC_ERR_INVALID_ARGUMENT, "a deadline must be positive (or -1 for none)");
    if (deadline_us > 0 && sv->policy.max_deadline_us > 0 && deadline_us > sv->policy.max_deadline_us)
        return fail(MPMC_ERR_INVALID_ARGUMENT, "request deadline exceeds the server policy");
    auto r = std::make_shared<Request>();
    r->mixture = mixture_id;
    r->ncell = n_cells;
    r->p = p;
    r->t = t;
    r->z = z;
    for (int k = 0; k < kFlashFields; ++k) r->out[k] = const_cast<void*>(fields[k]);
    r->submitted = Clock::now();
    r->has_deadline = deadline_us > 0;
    if (r->has_deadline) r->deadline = r->submitted + std::chrono::microseconds(deadline_us);
    const int64_t chunk = sv->policy.chunk_cells;
    r->tasks_left = static_cast<int>((n_cells + chunk - 1) / chunk);
    {
        std::lock_guard<std::mutex> lock(sv->mu);
        if (mixture_id < 0 || mixture_id >= static_cast<int>(sv->mixtures.size()))
            return fail(MPMC_ERR_INVALID_ARGUMENT, "unknown mixture id");
        if (sv->stop) return fail(MPMC_ERR_INVALID_ARGUMENT, "server is shutting down");
        if (sv->policy.max_in_flight > 0 && sv->in_flight >= sv->policy.max_in_flight) {
            ++sv->rejected_busy;
            return fail(MPMC_ERR_BUSY, "maximum concurrent requests are already in flight");
        }
        r->ticket = sv->next_ticket++;
        sv->tickets[r->ticket] = r;
        std::deque<Task>& q = n_cells <= sv->policy.small_request_cells ? sv->latency_q : sv->throughput_q;
        for (int64_t lo = 0; lo < n_cells; lo += chunk) q.push_back(Task{r, lo, std::min(n_cells, lo + chunk)});
        ++sv->submitted;
        ++sv->in_flight;
        *ticket = r->ticket;
    }
    sv->work_cv.notify_one();
    return MPMC_OK;
}

}  // namespace

extern "C" {

int mpmc_flash_server_create(const mpmc_server_options* options, mpmc_flash_server** out) {
    if (!options || !out) return fail(MPMC_ERR_INVALID_ARGUMENT, "options and out must not be null");
    *out = nullptr;
    if (options->form != MPMC_FORM_MIXED && options->form != MPMC_FORM_PLAIN_FP64)
        return fail(MPMC_ERR_UNSUPPORTED, "server form must be MPMC_FORM_MIXED or MPMC_FORM_PLAIN_FP64");
    if (options->flags & ~MPMC_SERVER_WARM_CACHE) return fail(MPMC_ERR_INVALID_ARGUMENT, "unknown server flag");
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
    if (options->device < 0 || options->device >= count)
        return fail(MPMC_ERR_INVALID_ARGUMENT, "device ordinal out of range");
    if ((e = cudaSetDevice(options->device)) != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    auto* sv = new mpmc_flash_server();
    sv->device = options->device;
    sv->form = options->form;
    sv->warm_cache = (options->flags & MPMC_SERVER_WARM_CACHE) != 0 && options->form == MPMC_FORM_MIXED;
    sv->cap = options->max_batch_cells > 0 ? options->max_batch_cells : 65536;
    if (sv->cap >= (int64_t{1} << 24)) {
        delete sv;
        return fail(MPMC_ERR_INVALID_ARGUMENT, "max_batch_cells must be below 16,777,216");
    }
    // default policy: every request whole up to the batch size, no latency
    // class, no limits (mpmc_flash_server_set_policy changes it)
    sv->policy.small_request_cells = 0;
    sv->policy.latency_slots = 0;
    sv->policy.latency_batch_cells = sv->cap;
    sv->policy.chunk_cells = sv->cap;
    sv->policy.max_request_cells = sv->cap;
    sv->policy.max_in_flight = 0;
    sv->policy.max_deadline_us = 0;
    const int64_t budget = options->memory_budget_bytes > 0 ? options->memory_budget_bytes : (int64_t{40} << 30);
    const int wanted = options->slots > 0 ? options->slots : 4;
    sv->slot_bytes = slot_device_bytes(sv);
    const int64_t fit = budget / static_cast<int64_t>(sv->slot_bytes);
    const int nslots = static_cast<int>(std::min<int64_t>(wanted, fit));
    if (nslots < 1) {
        delete sv;
        return fail(MPMC_ERR_INVALID_ARGUMENT, "memory budget holds no slot of " + std::to_string(sv->slot_bytes) +
                                                   " bytes (max_batch_cells too large for the budget)");
    }
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    sv->slots.resize(nslots);
    for (Slot& s : sv->slots) {
        if ((e = allocate_slot(sv, s, least)) != cudaSuccess) {
            for (Slot& r : sv->slots) release_slot(r);
            delete sv;
            return cuda_fail(e, "server slot allocation");
        }
    }
    sv->worker = std::thread(worker_loop, sv);
    *out = sv;
    return MPMC_OK;
}

int mpmc_flash_server_set_policy(mpmc_flash_server* sv, const mpmc_server_policy* policy) {
    if (!sv || !policy) return fail(MPMC_ERR_INVALID_ARGUMENT, "null argument");
    mpmc_server_policy p = *policy;
    if (p.small_request_cells < 0 || p.latency_slots < 0 || p.latency_batch_cells < 0 || p.chunk_cells < 0 ||
        p.max_request_cells < 0 || p.max_in_flight < 0 || p.max_deadline_us < 0)
        return fail(MPMC_ERR_INVALID_ARGUMENT, "policy values must not be negative");
    if (p.chunk_cells == 0) p.chunk_cells = sv->cap;
    if (p.latency_batch_cells == 0) p.latency_batch_cells = sv->cap;
    if (p.max_request_cells == 0) p.max_request_cells = sv->cap;
    if (p.chunk_cells > sv->cap || p.latency_batch_cells > sv->cap)
        return fail(MPMC_ERR_INVALID_ARGUMENT, "chunk_cells and latency_batch_cells must not exceed max_batch_cells");
    if (p.max_request_cells > p.chunk_cells * int64_t{4096})
        return fail(MPMC_ERR_INVALID_ARGUMENT, "max_request_cells must not exceed 4096 chunks");
    if (p.small_request_cells > p.chunk_cells)
        return fail(MPMC_ERR_INVALID_ARGUMENT, "small_request_cells must not exceed chunk_cells");
    std::lock_guard<std::mutex> lock(sv->mu);
    if (p.latency_slots >= static_cast<int32_t>(sv->slots.size()))
        return fail(MPMC_ERR_INVALID_ARGUMENT, "latency_slots must leave at least one throughput slot");
    for (const Slot& s : sv->slots)
        if (s.busy) return fail(MPMC_ERR_INVALID_ARGUMENT, "set the policy before the first submit");
    if (!sv->latency_q.empty() || !sv->throughput_q.empty())
        return fail(MPMC_ERR_INVALID_ARGUMENT, "set the policy before the first submit");
    // the first latency_slots slots serve the latency queue, on streams of the
    // highest priority
    cudaSetDevice(sv->device);
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    for (size_t k = 0; k < sv->slots.size(); ++k) {
        Slot& s = sv->slots[k];
        const bool lat = static_cast<int32_t>(k) < p.latency_slots;
        if (lat != s.latency) {
            cudaStream_t st = nullptr;
            const cudaError_t e = cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, lat ? greatest : least);
            if (e != cudaSuccess) return cuda_fail(e, "server stream");
            cudaStreamSynchronize(s.stream);
            cudaStreamDestroy(s.stream);
            s.stream = st;
            s.latency = lat;
        }
    }
    sv->policy = p;
    return MPMC_OK;
}

int mpmc_flash_server_add_mixture(mpmc_flash_server* sv, const mpmc_pr76_mixture* mixture, int32_t* id) {
    if (!sv || !mixture || !id) return fail(MPMC_ERR_INVALID_ARGUMENT, "null argument");
    pr76::Mixture m;
    const int rc = pr76::host::prepare_mixture(mixture, m);
    if (rc != MPMC_OK) return rc;
    std::lock_guard<std::mutex> lock(sv->mu);
    if (static_cast<int>(sv->mixtures.size()) >= kMaxMixtures)
        return fail(MPMC_ERR_UNSUPPORTED, "at most 64 mixtures per server");
    cudaError_t e = cudaSetDevice(sv->device);
    MixtureEntry entry;
    entry.n = m.n;
    if (e == cudaSuccess) e = cudaMalloc(&entry.d_mix, sizeof(pr76::Mixture));
    if (e == cudaSuccess) e = cudaMemcpy(entry.d_mix, &m, sizeof(pr76::Mixture), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && sv->warm_cache) {
        void* base = nullptr;
        e = cudaMalloc(&base, cache_bytes(m.n));
        if (e == cudaSuccess) e = cudaMemset(base, 0, cache_bytes(m.n));
        if (e == cudaSuccess) {
            char* b = static_cast<char*>(base);
            entry.cache.key0 = reinterpret_cast<unsigned long long*>(b);
            entry.cache.key1 = entry.cache.key0 + kCacheEntries;
            entry.cache.pt = reinterpret_cast<double*>(entry.cache.key1 + kCacheEntries);
            entry.cache.lnk = entry.cache.pt + 2 * kCacheEntries;
        }
    }
    if (e != cudaSuccess) {
        cudaFree(entry.d_mix);
        cudaFree(entry.cache.key0);
        return cuda_fail(e, "server mixture upload");
    }
    *id = static_cast<int32_t>(sv->mixtures.size());
    sv->mixtures.push_back(entry);
    return MPMC_OK;
}

int mpmc_flash_server_submit(mpmc_flash_server* sv, int32_t mixture_id, int64_t n_cells, const double* p,
                             const double* t, const double* z, const mpmc_flash_outputs* out, uint64_t* ticket) {
    return submit_request(sv, mixture_id, n_cells, p, t, z, out, -1, ticket);
}

int mpmc_flash_server_submit_deadline(mpmc_flash_server* sv, int32_t mixture_id, int64_t n_cells, const double* p,
                                      const double* t, const double* z, const mpmc_flash_outputs* out,
                                      int64_t deadline_us, uint64_t* ticket) {
    if (deadline_us <= 0) return fail(MPMC_ERR_INVALID_ARGUMENT, "a finite, positive deadline is required");
    return submit_request(sv, mixture_id, n_cells, p, t, z, out, deadline_us, ticket);
}

int mpmc_flash_server_wait(mpmc_flash_server* sv, uint64_t ticket, int64_t timeout_us, double* latency_s) {
    if (!sv) return fail(MPMC_ERR_INVALID_ARGUMENT, "null server");
    std::unique_lock<std::mutex> lock(sv->mu);
    auto it = sv->tickets.find(ticket);
    if (it == sv->tickets.end()) return fail(MPMC_ERR_INVALID_ARGUMENT, "unknown ticket");
    std::shared_ptr<Request> r = it->second;
    auto ready = [&] { return r->state == 2; };
    if (timeout_us < 0) {
        sv->done_cv.wait(lock, ready);
    } else if (!sv->done_cv.wait_for(lock, std::chrono::microseconds(timeout_us), ready)) {
        return fail(MPMC_ERR_TIMEOUT, "request still in progress");
    }
    sv->tickets.erase(ticket);
    if (latency_s) *latency_s = std::chrono::duration<double>(r->finished - r->submitted).count();
    if (r->error == MPMC_ERR_DEADLINE) return fail(MPMC_ERR_DEADLINE, "request deadline elapsed before publication");
    if (r->error != MPMC_OK) return fail(r->error, "request failed on the device");
    return MPMC_OK;
}

int mpmc_flash_server_stats(mpmc_flash_server* sv, int64_t* out, int capacity) {
    if (!sv || !out) return 0;
    std::lock_guard<std::mutex> lock(sv->mu);
    const int64_t v[12] = {sv->submitted, sv->completed, sv->batches, sv->cells,
                           static_cast<int64_t>(sv->slots.size()), static_cast<int64_t>(sv->slot_bytes),
                           sv->most_in_batch, sv->most_busy, sv->rejected_busy, sv->expired, sv->in_flight,
                           sv->warm_cells};
    const int k = std::min(capacity, 12);
    for (int i = 0; i < k; ++i) out[i] = v[i];
    return k;
}

int mpmc_flash_server_destroy(mpmc_flash_server* sv) {
    if (!sv) return MPMC_OK;
    {
        std::lock_guard<std::mutex> lock(sv->mu);
        sv->stop = true;
    }
    sv->work_cv.notify_all();
    if (sv->worker.joinable()) sv->worker.join();
    cudaSetDevice(sv->device);
    for (Slot& s : sv->slots) release_slot(s);
    for (auto& m : sv->mixtures) {
        cudaFree(m.d_mix);
        cudaFree(m.cache.key0);
    }
    delete sv;
    return MPMC_OK;
}

}  // extern "C"
