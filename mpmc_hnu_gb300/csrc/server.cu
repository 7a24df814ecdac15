// Flash server (include/mpmc_gb300_flash.h, "Flash server"): continuous
// batching of PT flash requests on one GPU.
//
// One worker thread owns the device side.  Each slot is a CUDA stream with
// device buffers for max_batch_cells cells (inputs, flash outputs, mixed-form
// workspace) and pinned host staging.  The worker loop
//   1. retires slots whose completion event has fired, scattering each
//      request's rows out of the batch into the caller's buffers;
//   2. fills every free slot with the oldest waiting request plus the other
//      waiting requests of the same mixture that still fit, stages them into
//      the slot's pinned buffers, and enqueues copy-in, flash, copy-out and
//      the completion event on the slot's stream;
//   3. sleeps on the queue's condition variable when there is nothing to do,
//      or polls the busy slots at a short interval.
// Every cell's result depends only on its own inputs, so the batching never
// changes a result.
#include <cuda_runtime.h>

#include <algorithm>
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
    Clock::time_point submitted, finished;
    int state = 0;  // 0 waiting, 1 on the device, 2 done
    int error = MPMC_OK;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    double *d_p = nullptr, *d_t = nullptr, *d_z = nullptr;
    void* d_out[kFlashFields] = {};
    void* d_ws = nullptr;
    size_t ws_bytes = 0;
    double *h_p = nullptr, *h_t = nullptr, *h_z = nullptr;
    void* h_out[kFlashFields] = {};
    std::vector<std::shared_ptr<Request>> batch;
    std::vector<int64_t> offsets;
    int mixture = -1;
    int64_t cells = 0;
    bool busy = false;
};

struct MixtureEntry {
    int n = 0;
    pr76::Mixture* d_mix = nullptr;
};

}  // namespace

struct mpmc_flash_server {
    int device = 0;
    int form = MPMC_FORM_MIXED;
    int64_t cap = 65536;
    int nmax = MPMC_MAX_COMPONENTS;
    std::vector<Slot> slots;
    size_t slot_bytes = 0;
    std::vector<MixtureEntry> mixtures;

    std::mutex mu;
    std::condition_variable work_cv;  // worker: new request or stop
    std::condition_variable done_cv;  // waiters: a request finished
    std::deque<std::shared_ptr<Request>> waiting;
    std::unordered_map<uint64_t, std::shared_ptr<Request>> tickets;
    uint64_t next_ticket = 1;
    bool stop = false;
    std::thread worker;

    int64_t submitted = 0, completed = 0, batches = 0, cells = 0, most_in_batch = 0, most_busy = 0;
};

namespace {

void release_slot(Slot& s) {
    if (s.stream) cudaStreamSynchronize(s.stream);
    cudaFree(s.d_p);
    cudaFree(s.d_t);
    cudaFree(s.d_z);
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

cudaError_t allocate_slot(mpmc_flash_server* sv, Slot& s) {
    const size_t cap = static_cast<size_t>(sv->cap), nmax = static_cast<size_t>(sv->nmax);
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking)) != cudaSuccess) return e;
    if ((e = cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&s.d_p, cap * 8)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&s.d_t, cap * 8)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&s.d_z, nmax * cap * 8)) != cudaSuccess) return e;
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
    for (int k = 0; k < kFlashFields; ++k) bytes += static_cast<size_t>(field_rows(k, sv->nmax)) * cap * field_elem(k);
    if (sv->form == MPMC_FORM_MIXED) bytes += pr76::batched_workspace_bytes(sv->nmax, sv->cap);
    return bytes;
}

// Copy a batch in, launch, copy out (worker thread, device current).
int launch_batch(mpmc_flash_server* sv, Slot& s) {
    const int n = sv->mixtures[s.mixture].n;
    const int64_t C = s.cells;
    const size_t cb = static_cast<size_t>(C);
    for (size_t r = 0; r < s.batch.size(); ++r) {
        const Request& q = *s.batch[r];
        const size_t off = static_cast<size_t>(s.offsets[r]), nc = static_cast<size_t>(q.ncell);
        std::memcpy(s.h_p + off, q.p, nc * 8);
        std::memcpy(s.h_t + off, q.t, nc * 8);
        for (int i = 0; i < n; ++i) std::memcpy(s.h_z + static_cast<size_t>(i) * cb + off, q.z + i * nc, nc * 8);
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
    const pr76::Mixture* mix = sv->mixtures[s.mixture].d_mix;
    if (sv->form == MPMC_FORM_MIXED) {
        const pr76::BatchedShape shape{0, 0, 0, 0, 0, nullptr, 0, 0.0f, 0};
        e = pr76::launch_batched(n, mix, C, s.d_p, s.d_t, s.d_z, d, s.d_ws, s.ws_bytes, shape, s.stream);
    } else {
        e = pr76::launch_plain(n, mix, C, s.d_p, s.d_t, s.d_z, d, s.stream);
    }
    if (e != cudaSuccess) return cuda_fail(e, "server flash launch");
    for (int k = 0; k < kFlashFields; ++k) {
        const size_t bytes = static_cast<size_t>(field_rows(k, n)) * cb * field_elem(k);
        if ((e = cudaMemcpyAsync(s.h_out[k], s.d_out[k], bytes, cudaMemcpyDeviceToHost, s.stream)) != cudaSuccess)
            return cuda_fail(e, "server copy-out");
    }
    if ((e = cudaEventRecord(s.done, s.stream)) != cudaSuccess) return cuda_fail(e, "server event");
    return MPMC_OK;
}

// Scatter a finished batch to its requests (worker thread, no lock held).
void scatter(const mpmc_flash_server* sv, const Slot& s) {
    const int n = sv->mixtures[s.mixture].n;
    const size_t cb = static_cast<size_t>(s.cells);
    for (size_t r = 0; r < s.batch.size(); ++r) {
        const Request& q = *s.batch[r];
        const size_t off = static_cast<size_t>(s.offsets[r]), nc = static_cast<size_t>(q.ncell);
        for (int k = 0; k < kFlashFields; ++k) {
            if (!q.out[k]) continue;
            const size_t el = field_elem(k);
            const char* src = static_cast<const char*>(s.h_out[k]);
            char* dst = static_cast<char*>(q.out[k]);
            for (int row = 0; row < field_rows(k, n); ++row)
                std::memcpy(dst + static_cast<size_t>(row) * nc * el, src + (static_cast<size_t>(row) * cb + off) * el,
                            nc * el);
        }
    }
}

void worker_loop(mpmc_flash_server* sv) {
    cudaSetDevice(sv->device);
    for (;;) {
        // 1. retire finished slots
        bool any_busy = false;
        for (Slot& s : sv->slots) {
            if (!s.busy) continue;
            const cudaError_t q = cudaEventQuery(s.done);
            if (q == cudaErrorNotReady) {
                any_busy = true;
                continue;
            }
            int err = MPMC_OK;
            if (q != cudaSuccess) err = cuda_fail(q, "server batch");
            else scatter(sv, s);
            const auto now = Clock::now();
            {
                std::lock_guard<std::mutex> lock(sv->mu);
                for (auto& r : s.batch) {
                    r->state = 2;
                    r->error = err;
                    r->finished = now;
                    ++sv->completed;
                }
            }
            sv->done_cv.notify_all();
            s.batch.clear();
            s.offsets.clear();
            s.busy = false;
        }
        // 2. fill free slots
        {
            std::unique_lock<std::mutex> lock(sv->mu);
            int busy = 0;
            for (const Slot& s : sv->slots) busy += s.busy;
            for (Slot& s : sv->slots) {
                if (s.busy || sv->waiting.empty()) continue;
                const int mix = sv->waiting.front()->mixture;
                int64_t cells = 0;
                for (auto it = sv->waiting.begin(); it != sv->waiting.end();) {
                    if ((*it)->mixture == mix && cells + (*it)->ncell <= sv->cap) {
                        s.offsets.push_back(cells);
                        cells += (*it)->ncell;
                        (*it)->state = 1;
                        s.batch.push_back(*it);
                        it = sv->waiting.erase(it);
                    } else {
                        ++it;
                    }
                }
                s.mixture = mix;
                s.cells = cells;
                s.busy = true;
                ++busy;
                ++sv->batches;
                sv->cells += cells;
                sv->most_in_batch = std::max<int64_t>(sv->most_in_batch, static_cast<int64_t>(s.batch.size()));
                sv->most_busy = std::max<int64_t>(sv->most_busy, busy);
                lock.unlock();
                const int rc = launch_batch(sv, s);
                lock.lock();
                if (rc != MPMC_OK) {
                    // nothing is in flight on the stream's event: fail the batch now
                    for (auto& r : s.batch) {
                        r->state = 2;
                        r->error = rc;
                        r->finished = Clock::now();
                        ++sv->completed;
                    }
                    s.batch.clear();
                    s.offsets.clear();
                    s.busy = false;
                    sv->done_cv.notify_all();
                }
            }
            any_busy = false;
            for (const Slot& s : sv->slots) any_busy = any_busy || s.busy;
            if (sv->stop && sv->waiting.empty() && !any_busy) return;
            if (!any_busy && sv->waiting.empty()) {
                sv->work_cv.wait(lock, [&] { return sv->stop || !sv->waiting.empty(); });
                continue;
            }
            bool free_slot = false;
            for (const Slot& s : sv->slots) free_slot = free_slot || !s.busy;
            if (free_slot && !sv->waiting.empty()) continue;  // fill it at once
        }
        // 3. slots busy: poll again shortly
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

}  // namespace

extern "C" {

int mpmc_flash_server_create(const mpmc_server_options* options, mpmc_flash_server** out) {
    if (!options || !out) return fail(MPMC_ERR_INVALID_ARGUMENT, "options and out must not be null");
    *out = nullptr;
    if (options->form != MPMC_FORM_MIXED && options->form != MPMC_FORM_PLAIN_FP64)
        return fail(MPMC_ERR_UNSUPPORTED, "server form must be MPMC_FORM_MIXED or MPMC_FORM_PLAIN_FP64");
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
    if (options->device < 0 || options->device >= count)
        return fail(MPMC_ERR_INVALID_ARGUMENT, "device ordinal out of range");
    if ((e = cudaSetDevice(options->device)) != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    auto* sv = new mpmc_flash_server();
    sv->device = options->device;
    sv->form = options->form;
    sv->cap = options->max_batch_cells > 0 ? options->max_batch_cells : 65536;
    if (sv->cap >= (int64_t{1} << 24)) {
        delete sv;
        return fail(MPMC_ERR_INVALID_ARGUMENT, "max_batch_cells must be below 16,777,216");
    }
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
    sv->slots.resize(nslots);
    for (Slot& s : sv->slots) {
        if ((e = allocate_slot(sv, s)) != cudaSuccess) {
            for (Slot& r : sv->slots) release_slot(r);
            delete sv;
            return cuda_fail(e, "server slot allocation");
        }
    }
    sv->worker = std::thread(worker_loop, sv);
    *out = sv;
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
    if (e != cudaSuccess) {
        cudaFree(entry.d_mix);
        return cuda_fail(e, "server mixture upload");
    }
    *id = static_cast<int32_t>(sv->mixtures.size());
    sv->mixtures.push_back(entry);
    return MPMC_OK;
}

int mpmc_flash_server_submit(mpmc_flash_server* sv, int32_t mixture_id, int64_t n_cells, const double* p,
                             const double* t, const double* z, const mpmc_flash_outputs* out, uint64_t* ticket) {
    if (!sv || !ticket || !out) return fail(MPMC_ERR_INVALID_ARGUMENT, "null argument");
    if (n_cells < 1 || n_cells > sv->cap)
        return fail(MPMC_ERR_INVALID_ARGUMENT, "request cell count must be in [1, max_batch_cells]");
    if (!p || !t || !z) return fail(MPMC_ERR_INVALID_ARGUMENT, "p, t and z must not be null");
    const void* const* fields = reinterpret_cast<const void* const*>(out);
    for (int k = kFlashFields; k < static_cast<int>(sizeof(mpmc_flash_outputs) / sizeof(void*)); ++k)
        if (fields[k]) return fail(MPMC_ERR_UNSUPPORTED, "the server returns flash fields only (no sensitivities)");
    auto r = std::make_shared<Request>();
    r->mixture = mixture_id;
    r->ncell = n_cells;
    r->p = p;
    r->t = t;
    r->z = z;
    for (int k = 0; k < kFlashFields; ++k) r->out[k] = const_cast<void*>(fields[k]);
    r->submitted = Clock::now();
    {
        std::lock_guard<std::mutex> lock(sv->mu);
        if (mixture_id < 0 || mixture_id >= static_cast<int>(sv->mixtures.size()))
            return fail(MPMC_ERR_INVALID_ARGUMENT, "unknown mixture id");
        if (sv->stop) return fail(MPMC_ERR_INVALID_ARGUMENT, "server is shutting down");
        r->ticket = sv->next_ticket++;
        sv->tickets[r->ticket] = r;
        sv->waiting.push_back(r);
        ++sv->submitted;
        *ticket = r->ticket;
    }
    sv->work_cv.notify_one();
    return MPMC_OK;
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
    if (r->error != MPMC_OK) return fail(r->error, "request failed on the device");
    return MPMC_OK;
}

int mpmc_flash_server_stats(mpmc_flash_server* sv, int64_t* out, int capacity) {
    if (!sv || !out) return 0;
    std::lock_guard<std::mutex> lock(sv->mu);
    const int64_t v[8] = {sv->submitted, sv->completed, sv->batches, sv->cells,
                          static_cast<int64_t>(sv->slots.size()), static_cast<int64_t>(sv->slot_bytes),
                          sv->most_in_batch, sv->most_busy};
    const int k = std::min(capacity, 8);
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
    for (auto& m : sv->mixtures) cudaFree(m.d_mix);
    delete sv;
    return MPMC_OK;
}

}  // extern "C"
