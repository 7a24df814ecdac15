// C ABI of the GB300 PR76 PT flash (include/mpmc_gb300_flash.h).
//
// Owns the per-mixture device state, validates requests the way the reference
// contracts do, stages host buffers for the host-buffer entry point and
// dispatches to the kernels of the selected algorithm form.  No exception
// crosses the boundary; failures set a thread-local message.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/mpmc_gb300_flash.h"
#include "launch.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& what) {
    g_last_error = what;
    return code;
}

int cuda_fail(cudaError_t e, const char* where) {
    return fail(MPMC_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// Device buffer that only grows.
struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t need) {
        if (need <= bytes) return cudaSuccess;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        const cudaError_t e = cudaMalloc(&ptr, need);
        if (e == cudaSuccess) bytes = need;
        return e;
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
};

constexpr int kOutputFields = 21;
constexpr size_t kMaxGraphs = 4;

// One captured solve: the cell count and every buffer are baked into it.
struct GraphEntry {
    int64_t ncell = 0;
    bool sensitivity = true;  // the sensitivity stage is part of the graph
    const double *p = nullptr, *t = nullptr, *z = nullptr, *warm = nullptr;
    pr76::DeviceOutputs outputs{};
    cudaGraphExec_t exec = nullptr;
    uint64_t last_use = 0;
};

}  // namespace

struct mpmc_gpu_flash {
    int n = 0;
    int device = 0;
    int form = MPMC_FORM_PLAIN_FP64;
    int want_sensitivity = 0;
    pr76::Mixture host_mixture{};
    pr76::Mixture* d_mixture = nullptr;
    cudaStream_t stream = nullptr;
    DevBuf in_p, in_t, in_z;
    DevBuf outs[kOutputFields];
    DevBuf sens_inputs[7];
    DevBuf workspace;  // batched-form stage buffers and work queues
    bool stage_timing = false;
    cudaEvent_t events[24] = {};
    cudaEvent_t redo_events[24] = {};  // the cold pass after a warm pass
    cudaEvent_t exact_events[24] = {};  // the exact sub-solve of the mixed form
    int n_events = 0;   // events recorded by the last solve (stages + 1)
    bool timed_warm = false;  // the last timed solve ran a warm and a cold pass
    bool timed_exact = false; // the last timed solve ran the exact sub-solve
    DevBuf in_warm;     // host entry: staged ln K warm starts
    DevBuf outs3[5];    // host entry: staged three-phase outputs
    DevBuf in_hints[7];   // host hinted entry: staged counts, compositions, three-phase flags, fractions
    DevBuf chart_in[2];   // host property-chart entry: staged chart values, dependent components
    DevBuf chart_out[3];  // host property-chart entry: staged status, values, Jacobian
    // a large work-queue solve runs as cell ranges on these streams (fork/join
    // by events on the caller's stream), each with its own workspace
    cudaStream_t range_streams[8] = {};
    cudaEvent_t fork_event = nullptr;
    // the mixed form's exact sub-solve overlaps the main pass on this stream
    cudaStream_t side_stream = nullptr;
    cudaEvent_t side_fork = nullptr, side_join = nullptr;
    cudaEvent_t join_events[8] = {};
    int last_ranges = 1;          // ranges of the last work-queue solve and their workspace offsets
    size_t range_offset[8] = {};
    cudaStream_t copy_stream = nullptr;  // host entry: copy-out overlapped with the sensitivity stage
    cudaEvent_t flash_done = nullptr;
    cudaEvent_t chunk_done[1] = {};
    int32_t shape[10] = {};  // explicit launch shape (mpmc_gpu_flash_set_launch_shape), 0 = default
    bool use_graphs = false;
    bool sens_lanes = false;  // the lane-group sensitivity kernel (MPMC_FLAG_SENSITIVITY_LANES)
    bool max3_newton = false;  // Newton roots in the max-3-phase continuation (MPMC_FLAG_MAX3_NEWTON_ROOTS)
    bool polish_stream = false;  // the state-machine polish (MPMC_FLAG_POLISH_STREAM)
    std::vector<GraphEntry> graphs;
    uint64_t graph_clock = 0;
};

namespace {

// Build the prepared constants exactly as Pr76Pure's constructor does
// (modules/thermodynamics/include/mpmc/thermodynamics/pr76_pure.hpp:181-199)
// and the binary factors of Pr76Mixture (pr76_mixture.hpp:229-251).
int prepare_mixture(const mpmc_pr76_mixture* mix, pr76::Mixture& m) {
    const int n = mix->n_components;
    if (n < 1 || n > MPMC_MAX_COMPONENTS)
        return fail(MPMC_ERR_UNSUPPORTED, "component count must be in [1, " +
                                              std::to_string(MPMC_MAX_COMPONENTS) + "]");
    if (!mix->critical_temperature_k || !mix->critical_pressure_pa || !mix->acentric_factor || !mix->kij)
        return fail(MPMC_ERR_INVALID_ARGUMENT, "mixture arrays must not be null");
    std::memset(&m, 0, sizeof(m));
    m.n = n;
    for (int i = 0; i < n; ++i) {
        const double tc = mix->critical_temperature_k[i];
        const double pc = mix->critical_pressure_pa[i];
        const double omega = mix->acentric_factor[i];
        if (!std::isfinite(tc) || !(tc > 0) || !std::isfinite(pc) || !(pc > 0) || !std::isfinite(omega))
            return fail(MPMC_ERR_DOMAIN, "component " + std::to_string(i) +
                                             ": finite Tc > 0, Pc > 0 and finite omega required");
        m.sqrt_tc[i] = std::sqrt(tc);
        m.kappa[i] = 0.37464 + omega * (1.54226 - 0.26992 * omega);
        const double rtc = pr76::kR * tc;
        m.ac[i] = (0.45724 * rtc) * (rtc / pc);
        m.b[i] = (0.07780 * rtc) / pc;
        if (!std::isfinite(m.kappa[i]) || !std::isfinite(m.ac[i]) || !(m.ac[i] > 0) || !std::isfinite(m.b[i]) ||
            !(m.b[i] > 0))
            return fail(MPMC_ERR_DOMAIN, "component " + std::to_string(i) + ": coefficient outside range");
    }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            const double k = mix->kij[i * n + j];
            if (!std::isfinite(k)) return fail(MPMC_ERR_DOMAIN, "kij must be finite");
            if (i == j && k != 0.0) return fail(MPMC_ERR_DOMAIN, "kij diagonal must be zero");
            if (k != mix->kij[j * n + i]) return fail(MPMC_ERR_DOMAIN, "kij must be symmetric");
            m.factor[i * n + j] = 1.0 - k;
            m.factor32[i * n + j] = static_cast<float>(m.factor[i * n + j]);
        }
    for (int i = 0; i < n; ++i) m.b32[i] = static_cast<float>(m.b[i]);
    return MPMC_OK;
}

pr76::DeviceOutputs to_device_outputs(const mpmc_flash_outputs* o) {
    pr76::DeviceOutputs d{};
    if (!o) return d;
    d.status = o->status;
    d.beta = o->vapor_fraction;
    d.x = o->liquid;
    d.y = o->vapor;
    d.lnk = o->ln_k;
    d.lnphi_l = o->ln_phi_liquid;
    d.lnphi_v = o->ln_phi_vapor;
    d.z_l = o->z_liquid;
    d.z_v = o->z_vapor;
    d.counters = o->counters;
    d.sens_status = o->sensitivity_status;
    d.dlnk = o->d_ln_k;
    d.dbeta = o->d_vapor_fraction;
    d.dx = o->d_liquid;
    d.dy = o->d_vapor;
    d.dzl = o->d_z_liquid;
    d.dzv = o->d_z_vapor;
    d.drhol = o->d_rho_liquid;
    d.drhov = o->d_rho_vapor;
    d.jl = o->jac_liquid;
    d.jv = o->jac_vapor;
    return d;
}

// Element counts per cell of every output field, in mpmc_flash_outputs order.
void field_sizes(int n, size_t* per_cell, size_t* elem) {
    const size_t q = static_cast<size_t>(n) + 1;
    const size_t counts[kOutputFields] = {1, 1, (size_t)n, (size_t)n, (size_t)n, (size_t)n, (size_t)n, 1, 1,
                                          MPMC_COUNTER_COUNT, 1, n * q, q, n * q, n * q, q, q, q, q,
                                          (n + 1) * (q + 1), (n + 1) * (q + 1)};
    for (int k = 0; k < kOutputFields; ++k) {
        per_cell[k] = counts[k];
        elem[k] = (k == 0 || k == 9 || k == 10) ? 4 : 8;
    }
}

void** field_ptr(mpmc_flash_outputs* o, int k) {
    void** base = reinterpret_cast<void**>(o);
    return base + k;
}

// The sensitivity kernel reads the accepted pair back from the flash outputs;
// fields the caller did not request are routed to per-handle scratch.
int with_sensitivity_inputs(mpmc_gpu_flash* h, int64_t ncell, pr76::DeviceOutputs& d) {
    const size_t nc = static_cast<size_t>(ncell), n = static_cast<size_t>(h->n);
    struct Need {
        void** field;
        size_t bytes;
    } needs[] = {{reinterpret_cast<void**>(&d.status), 4 * nc}, {reinterpret_cast<void**>(&d.beta), 8 * nc},
                 {reinterpret_cast<void**>(&d.x), 8 * n * nc},  {reinterpret_cast<void**>(&d.y), 8 * n * nc},
                 {reinterpret_cast<void**>(&d.lnk), 8 * n * nc}, {reinterpret_cast<void**>(&d.z_l), 8 * nc},
                 {reinterpret_cast<void**>(&d.z_v), 8 * nc}};
    for (int k = 0; k < 7; ++k) {
        if (*needs[k].field) continue;
        const cudaError_t e = h->sens_inputs[k].ensure(needs[k].bytes);
        if (e != cudaSuccess) return cuda_fail(e, "sensitivity scratch allocation");
        *needs[k].field = h->sens_inputs[k].ptr;
    }
    return MPMC_OK;
}

// Launch shape of the mixed form: defaults, then the MPMC_* environment knobs
// (sweeps), then the handle's explicit shape (mpmc_gpu_flash_set_launch_shape).
pr76::BatchedShape batched_shape(const mpmc_gpu_flash* h, cudaEvent_t* events) {
    pr76::BatchedShape shape{0, 0, 0, 0, 0, events, 0, 0.0f, 0};
    const struct {
        const char* name;
        int* field;
    } knobs[] = {{"MPMC_TRIAL_BLOCKS_PER_SM", &shape.trial_blocks_per_sm},
                 {"MPMC_SPLIT_BLOCKS_PER_SM", &shape.split_blocks_per_sm},
                 {"MPMC_T64_BLOCKS_PER_SM", &shape.t64_blocks_per_sm},
                 {"MPMC_S64_BLOCKS_PER_SM", &shape.s64_blocks_per_sm},
                 {"MPMC_CELL_BLOCKS_PER_SM", &shape.cell_blocks_per_sm},
                 {"MPMC_ITEM_FORM", &shape.item_form}};
    for (const auto& k : knobs)
        if (const char* v = std::getenv(k.name)) *k.field = std::atoi(v);
    int* fields[6] = {&shape.trial_blocks_per_sm, &shape.split_blocks_per_sm, &shape.t64_blocks_per_sm,
                      &shape.s64_blocks_per_sm, &shape.cell_blocks_per_sm, &shape.item_form};
    for (int k = 0; k < 6; ++k)
        if (h->shape[k] > 0) *fields[k] = h->shape[k];
    if (h->shape[6] > 0) shape.ss_switch = 1e-6f * static_cast<float>(h->shape[6]);
    if (h->shape[8] > 0) shape.slow_projection = static_cast<float>(h->shape[8]);
    if (h->shape[9] > 0) shape.continue_limit = h->shape[9];
    shape.polish_stream = h->polish_stream ? 1 : 0;
    return shape;
}

constexpr int kMaxRanges = 8;
constexpr int64_t kMinRangeCells = 65536;

// Cell ranges of a work-queue solve: the handle's launch shape [7], else
// MPMC_RANGES, else 1; each range keeps at least 65,536 cells.  Ranges on
// separate streams let the long last items of one range overlap the bulk
// stages of the others.  Measured on a GB300 at 1,048,576 cells (N = 10, 30 %
// near a boundary, with sensitivities): 1 range 1097 ms, 2 1157 ms, 4 1140
// ms, 8 1196 ms, every output identical -- the stages already fill the GPU,
// so one range is the default.
int solve_ranges(const mpmc_gpu_flash* h, int64_t ncell) {
    int k = h->shape[7];
    if (k <= 0)
        if (const char* v = std::getenv("MPMC_RANGES")) k = std::atoi(v);
    if (k <= 0) k = 1;
    k = std::min(std::max(k, 1), kMaxRanges);
    while (k > 1 && ncell / k < kMinRangeCells) --k;
    return k;
}

// Range r of k over ncell cells: [c0, c1).
void range_of(int64_t ncell, int k, int r, int64_t& c0, int64_t& c1) {
    const int64_t step = (ncell + k - 1) / k;
    c0 = std::min<int64_t>(ncell, r * step);
    c1 = std::min<int64_t>(ncell, c0 + step);
}

// Workspace bytes of a solve in k ranges (each range's arrays 256-aligned);
// fills the offsets when `offsets` is given.
size_t ranged_workspace_bytes(int n, int64_t ncell, bool fp64_items, int k, size_t* offsets = nullptr) {
    size_t off = 0;
    for (int r = 0; r < k; ++r) {
        int64_t c0, c1;
        range_of(ncell, k, r, c0, c1);
        if (offsets) offsets[r] = off;
        off += (pr76::batched_workspace_bytes(n, c1 - c0, fp64_items) + 255) & ~static_cast<size_t>(255);
    }
    return off;
}

// Device scratch of a solve (allocated before any launch, so that a graph
// capture of the launches sees no allocation).
int prepare_device(mpmc_gpu_flash* h, int64_t ncell, pr76::DeviceOutputs& d) {
    if (h->want_sensitivity) {
        const int rc = with_sensitivity_inputs(h, ncell, d);
        if (rc != MPMC_OK) return rc;
    }
    if (h->form == MPMC_FORM_MIXED || h->form == MPMC_FORM_BATCHED) {
        if (ncell >= (int64_t{1} << 24))
            return fail(MPMC_ERR_INVALID_ARGUMENT, "batched forms: at most 16,777,215 cells per call");
        const int k = h->stage_timing ? 1 : solve_ranges(h, ncell);
        cudaError_t e = h->workspace.ensure(ranged_workspace_bytes(h->n, ncell, h->form == MPMC_FORM_BATCHED, k));
        if (e != cudaSuccess) return cuda_fail(e, "batched workspace allocation");
        if (h->form == MPMC_FORM_MIXED && !h->side_stream) {
            if ((e = cudaStreamCreateWithFlags(&h->side_stream, cudaStreamNonBlocking)) != cudaSuccess)
                return cuda_fail(e, "side stream");
            if ((e = cudaEventCreateWithFlags(&h->side_fork, cudaEventDisableTiming)) != cudaSuccess ||
                (e = cudaEventCreateWithFlags(&h->side_join, cudaEventDisableTiming)) != cudaSuccess)
                return cuda_fail(e, "cudaEventCreate");
        }
        if (k > 1 && !h->fork_event) {
            if ((e = cudaEventCreateWithFlags(&h->fork_event, cudaEventDisableTiming)) != cudaSuccess)
                return cuda_fail(e, "cudaEventCreate");
            for (int r = 0; r < kMaxRanges; ++r) {
                if ((e = cudaStreamCreateWithFlags(&h->range_streams[r], cudaStreamNonBlocking)) != cudaSuccess)
                    return cuda_fail(e, "range stream");
                if ((e = cudaEventCreateWithFlags(&h->join_events[r], cudaEventDisableTiming)) != cudaSuccess)
                    return cuda_fail(e, "cudaEventCreate");
            }
        }
    } else if (h->form != MPMC_FORM_PLAIN_FP64) {
        return fail(MPMC_ERR_UNSUPPORTED, "algorithm form not available in this library");
    }
    return MPMC_OK;
}

// The launches of one solve on `stream` (no allocation, no synchronisation).
cudaError_t enqueue_device(mpmc_gpu_flash* h, int64_t ncell, const double* p, const double* t, const double* z,
                           const double* warm, const pr76::DeviceOutputs& d, cudaStream_t stream, bool timing,
                           const pr76::Max3Outputs* max3 = nullptr, const pr76::Hints* hints = nullptr,
                           bool sensitivity = true) {
    cudaError_t e;
    int next_event = 0;
    auto record = [&]() {
        if (timing && next_event < 24) cudaEventRecord(h->events[next_event++], stream);
    };
    if (h->form == MPMC_FORM_PLAIN_FP64 || hints) {
        // caller start hints run the reference algorithm itself, for every form
        record();
        e = pr76::launch_plain(h->n, h->d_mixture, ncell, p, t, z, d, stream, hints ? *hints : pr76::Hints{});
        record();
    } else {
        pr76::BatchedShape shape = batched_shape(h, timing ? h->events : nullptr);
        shape.fp64_items = h->form == MPMC_FORM_BATCHED;
        shape.warm_lnk = warm;
        shape.redo_events = timing ? h->redo_events : nullptr;
        shape.exact_events = timing ? h->exact_events : nullptr;
        const bool fp64_items = h->form == MPMC_FORM_BATCHED;
        const int k = timing ? 1 : solve_ranges(h, ncell);
        h->last_ranges = k;
        ranged_workspace_bytes(h->n, ncell, fp64_items, k, h->range_offset);
        if (k == 1) {
            // the exact sub-solve on the side stream, except when the stages
            // are timed (then it runs after the main pass, with its own events)
            if (!timing && h->side_stream) {
                shape.side_stream = h->side_stream;
                shape.side_fork = h->side_fork;
                shape.side_join = h->side_join;
            }
            e = pr76::launch_batched(h->n, h->d_mixture, ncell, p, t, z, d, h->workspace.ptr, h->workspace.bytes,
                                     shape, stream);
        } else {
            // each range a solve of its own on its own stream: every pointer at
            // the range's start, rows at the whole batch's stride
            e = cudaEventRecord(h->fork_event, stream);
            for (int r = 0; r < k && e == cudaSuccess; ++r) {
                int64_t c0, c1;
                range_of(ncell, k, r, c0, c1);
                cudaStream_t rs = h->range_streams[r];
                if ((e = cudaStreamWaitEvent(rs, h->fork_event, 0)) != cudaSuccess) break;
                pr76::DeviceOutputs dr = d;
                void** f = reinterpret_cast<void**>(&dr);
                for (int q = 0; q < kOutputFields; ++q) {
                    if (!f[q]) continue;
                    const size_t el = (q == 0 || q == 9 || q == 10) ? 4 : 8;
                    f[q] = static_cast<char*>(f[q]) + static_cast<size_t>(c0) * el;
                }
                pr76::BatchedShape sr = shape;
                sr.io_stride = ncell;
                sr.warm_lnk = warm ? warm + c0 : nullptr;
                const size_t bytes = pr76::batched_workspace_bytes(h->n, c1 - c0, fp64_items);
                e = pr76::launch_batched(h->n, h->d_mixture, c1 - c0, p + c0, t + c0, z + c0, dr,
                                         static_cast<char*>(h->workspace.ptr) + h->range_offset[r], bytes, sr, rs);
                if (e == cudaSuccess) e = cudaEventRecord(h->join_events[r], rs);
                if (e == cudaSuccess) e = cudaStreamWaitEvent(stream, h->join_events[r], 0);
            }
        }
        next_event = timing ? pr76::kBatchedStages + 1 : 0;
    }
    if (e != cudaSuccess) return e;
    if (max3) {  // before the sensitivities: a fresh two-phase neighbor is differentiated too
        e = pr76::launch_max3(h->n, h->d_mixture, ncell, p, t, z, d, *max3, stream, hints ? *hints : pr76::Hints{},
                              h->max3_newton);
        if (e != cudaSuccess) return e;
    }
    if (h->want_sensitivity && sensitivity) {
        e = pr76::launch_sensitivity(h->n, h->d_mixture, ncell, p, t, z, d, stream, 0, -1, h->sens_lanes);
        if (e != cudaSuccess) return e;
    }
    record();  // end of the sensitivity stage (zero length without sensitivities)
    if (timing) {
        h->n_events = next_event;
        h->timed_warm = warm != nullptr && (h->form == MPMC_FORM_MIXED || h->form == MPMC_FORM_BATCHED);
        h->timed_exact = h->form == MPMC_FORM_MIXED && !hints;
    }
    return cudaSuccess;
}

bool same_key(const GraphEntry& g, int64_t ncell, const double* p, const double* t, const double* z,
              const double* warm, const pr76::DeviceOutputs& d, bool sensitivity) {
    return g.ncell == ncell && g.sensitivity == sensitivity && g.p == p && g.t == t && g.z == z && g.warm == warm &&
           std::memcmp(&g.outputs, &d, sizeof(pr76::DeviceOutputs)) == 0;
}

// `sensitivity` false leaves the sensitivity stage to the caller (the
// host-buffer entry runs it by cell ranges, overlapped with its copies).
int run_device(mpmc_gpu_flash* h, int64_t ncell, const double* p, const double* t, const double* z,
               const double* warm, const pr76::DeviceOutputs& d_in, cudaStream_t stream,
               const pr76::Max3Outputs* max3 = nullptr, const pr76::Hints* hints = nullptr,
               bool sensitivity = true) {
    if (warm && h->form == MPMC_FORM_PLAIN_FP64)
        return fail(MPMC_ERR_UNSUPPORTED,
                    "ln K warm starts need a work-queue form (MPMC_FORM_MIXED or MPMC_FORM_BATCHED); the plain "
                    "form is the reference algorithm, which has no warm start");
    pr76::DeviceOutputs d = d_in;
    int rc = prepare_device(h, ncell, d);
    if (rc != MPMC_OK) return rc;
    cudaError_t e;
    h->n_events = 0;
    if (h->stage_timing && !h->events[0]) {
        for (auto& ev : h->events)
            if ((e = cudaEventCreate(&ev)) != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
        for (auto& ev : h->redo_events)
            if ((e = cudaEventCreate(&ev)) != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
        for (auto& ev : h->exact_events)
            if ((e = cudaEventCreate(&ev)) != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
    }
    if (!h->use_graphs || h->stage_timing || max3) {
        e = enqueue_device(h, ncell, p, t, z, warm, d, stream, h->stage_timing, max3, hints, sensitivity);
        return e == cudaSuccess ? MPMC_OK : cuda_fail(e, "flash kernel launch");
    }
    // CUDA graph of the launch sequence, one per (cells, buffers): captured on
    // the handle's stream at the first call, replayed on `stream` afterwards
    for (GraphEntry& g : h->graphs) {
        if (!same_key(g, ncell, p, t, z, warm, d, sensitivity)) continue;
        g.last_use = ++h->graph_clock;
        e = cudaGraphLaunch(g.exec, stream);
        return e == cudaSuccess ? MPMC_OK : cuda_fail(e, "cudaGraphLaunch");
    }
    cudaGraph_t graph = nullptr;
    if ((e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
        return cuda_fail(e, "cudaStreamBeginCapture");
    const cudaError_t le = enqueue_device(h, ncell, p, t, z, warm, d, h->stream, false, nullptr, nullptr, sensitivity);
    e = cudaStreamEndCapture(h->stream, &graph);
    if (le != cudaSuccess || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return cuda_fail(le != cudaSuccess ? le : e, "graph capture of the flash launches");
    }
    GraphEntry entry;
    e = cudaGraphInstantiate(&entry.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    entry.ncell = ncell;
    entry.sensitivity = sensitivity;
    entry.p = p;
    entry.t = t;
    entry.z = z;
    entry.warm = warm;
    entry.outputs = d;
    entry.last_use = ++h->graph_clock;
    if (h->graphs.size() >= kMaxGraphs) {  // evict the least recently used
        auto oldest = std::min_element(h->graphs.begin(), h->graphs.end(),
                                       [](const GraphEntry& a, const GraphEntry& b) { return a.last_use < b.last_use; });
        cudaGraphExecDestroy(oldest->exec);
        h->graphs.erase(oldest);
    }
    h->graphs.push_back(entry);
    e = cudaGraphLaunch(entry.exec, stream);
    return e == cudaSuccess ? MPMC_OK : cuda_fail(e, "cudaGraphLaunch");
}

// ---- fixed scratch of the no-allocation entry point ----
// One array per device, reserved when the library's device code is loaded;
// its address is looked up once per device (with that device current).
__device__ __align__(256) unsigned char g_noalloc_scratch[MPMC_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_address[kMaxDevices] = {};

int noalloc_scratch(int device, void** out) {
    if (device < 0 || device >= kMaxDevices) return fail(MPMC_ERR_INVALID_ARGUMENT, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_address[device]) {
        void* ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) return cuda_fail(e, "cudaGetSymbolAddress (no-allocation scratch)");
        g_noalloc_address[device] = ptr;
    }
    *out = g_noalloc_address[device];
    return MPMC_OK;
}

}  // namespace

namespace pr76 {
namespace host {
int fail(int code, const std::string& what) { return ::fail(code, what); }
int cuda_fail(cudaError_t e, const char* where) { return ::cuda_fail(e, where); }
int prepare_mixture(const mpmc_pr76_mixture* mix, Mixture& m) { return ::prepare_mixture(mix, m); }
}  // namespace host

LaunchShape plain_launch_shape() {
    LaunchShape s{64, 2};
    if (const char* v = std::getenv("MPMC_PLAIN_BLOCK")) s.block = std::atoi(v);
    if (const char* v = std::getenv("MPMC_PLAIN_BLOCKS_PER_SM")) s.blocks_per_sm = std::atoi(v);
    if (s.block != 32 && s.block != 64 && s.block != 128) s.block = 64;
    if (s.blocks_per_sm < 1 || s.blocks_per_sm > 32) s.blocks_per_sm = 2;
    return s;
}

int capacity_for(int n) {
    if (n < 1) return 0;
    if (n <= 4) return 4;
    if (n <= 8) return 8;
    if (n <= 12) return 12;
    if (n <= 16) return 16;
    if (n <= 20) return 20;
    return 0;
}

size_t batched_workspace_bytes(int n, int64_t ncell, bool fp64_items, int s64_per_cell) {
    switch (capacity_for(n)) {
    case 4: return batched_workspace_bytes_nm4(n, ncell, fp64_items, s64_per_cell);
    case 8: return batched_workspace_bytes_nm8(n, ncell, fp64_items, s64_per_cell);
    case 12: return batched_workspace_bytes_nm12(n, ncell, fp64_items, s64_per_cell);
    case 16: return batched_workspace_bytes_nm16(n, ncell, fp64_items, s64_per_cell);
    case 20: return batched_workspace_bytes_nm20(n, ncell, fp64_items, s64_per_cell);
    default: return 0;
    }
}

cudaError_t launch_batched(int n, const Mixture* d_mix, int64_t ncell, const double* p, const double* t,
                           const double* z, const DeviceOutputs& out, void* scratch, size_t scratch_bytes,
                           const BatchedShape& shape, cudaStream_t stream) {
    switch (capacity_for(n)) {
    case 4: return launch_batched_nm4(d_mix, n, ncell, p, t, z, out, scratch, scratch_bytes, shape, stream);
    case 8: return launch_batched_nm8(d_mix, n, ncell, p, t, z, out, scratch, scratch_bytes, shape, stream);
    case 12: return launch_batched_nm12(d_mix, n, ncell, p, t, z, out, scratch, scratch_bytes, shape, stream);
    case 16: return launch_batched_nm16(d_mix, n, ncell, p, t, z, out, scratch, scratch_bytes, shape, stream);
    case 20: return launch_batched_nm20(d_mix, n, ncell, p, t, z, out, scratch, scratch_bytes, shape, stream);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_sensitivity(int n, const Mixture* d_mix, int64_t ncell, const double* p, const double* t,
                               const double* z, const DeviceOutputs& out, cudaStream_t stream, int64_t c0,
                               int64_t c1, bool lanes) {
    if (lanes) switch (capacity_for(n)) {
        case 4: return launch_sensitivity_lanes_nm4(d_mix, ncell, p, t, z, out, stream, c0, c1);
        case 8: return launch_sensitivity_lanes_nm8(d_mix, ncell, p, t, z, out, stream, c0, c1);
        case 12: return launch_sensitivity_lanes_nm12(d_mix, ncell, p, t, z, out, stream, c0, c1);
        case 16: return launch_sensitivity_lanes_nm16(d_mix, ncell, p, t, z, out, stream, c0, c1);
        case 20: return launch_sensitivity_lanes_nm20(d_mix, ncell, p, t, z, out, stream, c0, c1);
        default: return cudaErrorInvalidValue;
        }
    switch (capacity_for(n)) {
    case 4: return launch_sensitivity_nm4(d_mix, ncell, p, t, z, out, stream, c0, c1);
    case 8: return launch_sensitivity_nm8(d_mix, ncell, p, t, z, out, stream, c0, c1);
    case 12: return launch_sensitivity_nm12(d_mix, ncell, p, t, z, out, stream, c0, c1);
    case 16: return launch_sensitivity_nm16(d_mix, ncell, p, t, z, out, stream, c0, c1);
    case 20: return launch_sensitivity_nm20(d_mix, ncell, p, t, z, out, stream, c0, c1);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_max3(int n, const Mixture* d_mix, int64_t ncell, const double* p, const double* t,
                        const double* z, const DeviceOutputs& out, const Max3Outputs& out3, cudaStream_t stream,
                        const Hints& hints, bool newton_roots) {
    switch (capacity_for(n)) {
    case 4: return launch_max3_nm4(d_mix, ncell, p, t, z, out, out3, stream, hints, newton_roots);
    case 8: return launch_max3_nm8(d_mix, ncell, p, t, z, out, out3, stream, hints, newton_roots);
    case 12: return launch_max3_nm12(d_mix, ncell, p, t, z, out, out3, stream, hints, newton_roots);
    case 16: return launch_max3_nm16(d_mix, ncell, p, t, z, out, out3, stream, hints, newton_roots);
    case 20: return launch_max3_nm20(d_mix, ncell, p, t, z, out, out3, stream, hints, newton_roots);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_chart(int n, const Mixture* d_mix, const ChartParams& params, int64_t ncell, const double* q,
                         const int32_t* dep, const ChartOutputs& out, cudaStream_t stream) {
    switch (capacity_for(n)) {
    case 4: return launch_chart_nm4(d_mix, params, ncell, q, dep, out, stream);
    case 8: return launch_chart_nm8(d_mix, params, ncell, q, dep, out, stream);
    case 12: return launch_chart_nm12(d_mix, params, ncell, q, dep, out, stream);
    case 16: return launch_chart_nm16(d_mix, params, ncell, q, dep, out, stream);
    case 20: return launch_chart_nm20(d_mix, params, ncell, q, dep, out, stream);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_plain(int n, const Mixture* d_mix, int64_t ncell, const double* p, const double* t,
                         const double* z, const DeviceOutputs& out, cudaStream_t stream, const Hints& hints) {
    switch (capacity_for(n)) {
    case 4: return launch_plain_nm4(d_mix, ncell, p, t, z, out, stream, hints);
    case 8: return launch_plain_nm8(d_mix, ncell, p, t, z, out, stream, hints);
    case 12: return launch_plain_nm12(d_mix, ncell, p, t, z, out, stream, hints);
    case 16: return launch_plain_nm16(d_mix, ncell, p, t, z, out, stream, hints);
    case 20: return launch_plain_nm20(d_mix, ncell, p, t, z, out, stream, hints);
    default: return cudaErrorInvalidValue;
    }
}
}  // namespace pr76

namespace {
// Caller starts of either hinted entry, in the device's Hints layout (host or
// device pointers).
pr76::Hints hints_of(const mpmc_start_hints* h) {
    pr76::Hints d;
    d.count = h->count;
    d.x = h->composition;
    d.three = h->three_phase;
    d.fraction = h->fraction;
    return d;
}
pr76::Hints hints_of(const mpmc_start_hints_ex* h) {
    pr76::Hints d;
    d.count = h->initial_count;
    d.x = h->initial_composition;
    d.final_count = h->final_count;
    d.final_x = h->final_composition;
    d.three = h->three_phase;
    d.three_x = h->three_phase_composition;
    d.fraction = h->fraction;
    d.separate = 1;
    d.initial_automatic_starts = h->initial_automatic_starts != 0;
    d.max_split_attempts = h->max_split_attempts;
    return d;
}
int check_hints_ex(const mpmc_start_hints_ex* h) {
    if (!h) return fail(MPMC_ERR_INVALID_ARGUMENT, "hinted solve: null hints");
    if ((h->initial_count != nullptr) != (h->initial_composition != nullptr) ||
        (h->final_count != nullptr) != (h->final_composition != nullptr) ||
        (h->three_phase != nullptr) != (h->three_phase_composition != nullptr) ||
        (h->three_phase != nullptr) != (h->fraction != nullptr))
        return fail(MPMC_ERR_INVALID_ARGUMENT, "hinted solve: each start class needs its count (or flag) and "
                                               "composition arrays together, the three-phase start its fractions");
    if (h->max_split_attempts < 0 || h->max_split_attempts > 65536)
        return fail(MPMC_ERR_INVALID_ARGUMENT, "hinted solve: max_split_attempts must be in [0, 65536]");
    return MPMC_OK;
}

int solve_host(mpmc_gpu_flash* h, int64_t ncell, const double* p, const double* t, const double* z,
               const double* ln_k_warm, const mpmc_flash_outputs* out, const mpmc_three_phase_outputs* out3,
               bool max3, const pr76::Hints* hints = nullptr);

// Validates a property-chart call and fills the kernel's closure constants
// (the checks of the closure's constructor, pr76_selected_phase_property_closure.hpp:274-319,
// and of the chart's shape, :553-562).
int chart_params(const mpmc_gpu_flash* h, int64_t ncell, const mpmc_property_chart_spec* spec, const double* q,
                 pr76::ChartParams& params) {
    if (!h) return fail(MPMC_ERR_INVALID_ARGUMENT, "null handle");
    if (ncell < 0) return fail(MPMC_ERR_INVALID_ARGUMENT, "negative cell count");
    if (!spec) return fail(MPMC_ERR_INVALID_ARGUMENT, "property chart: null spec");
    if (spec->phase_count < 1 || spec->phase_count > 3)
        return fail(MPMC_ERR_INVALID_ARGUMENT, "property chart: phase_count must be 1, 2 or 3");
    if (h->n < 2) return fail(MPMC_ERR_INVALID_ARGUMENT, "property chart: at least two components required");
    if (!spec->molar_mass || !spec->viscosity || !spec->enthalpy)
        return fail(MPMC_ERR_INVALID_ARGUMENT, "property chart: molar_mass, viscosity and enthalpy must not be null");
    std::memset(&params, 0, sizeof(params));
    params.phases = spec->phase_count;
    for (int k = 0; k < spec->phase_count; ++k) {
        if (spec->root_index[k] < 0) return fail(MPMC_ERR_INVALID_ARGUMENT, "property chart: negative root index");
        params.root_index[k] = spec->root_index[k];
    }
    for (int i = 0; i < h->n; ++i) {
        const double mw = spec->molar_mass[i];
        if (!std::isfinite(mw) || !(mw > 0))
            return fail(MPMC_ERR_INVALID_ARGUMENT, "property chart: every molar mass must be finite and positive");
        params.molar_mass[i] = mw;
    }
    for (int k = 0; k < 7 + h->n; ++k) {
        if (!std::isfinite(spec->viscosity[k]) || !std::isfinite(spec->enthalpy[k]))
            return fail(MPMC_ERR_INVALID_ARGUMENT, "property chart: model coefficients must be finite");
        params.visc[k] = spec->viscosity[k];
        params.enth[k] = spec->enthalpy[k];
    }
    if (ncell > 0 && !q) return fail(MPMC_ERR_INVALID_ARGUMENT, "property chart: null chart values");
    return MPMC_OK;
}
}  // namespace

extern "C" {

int mpmc_gpu_flash_abi_version(void) { return MPMC_GB300_FLASH_ABI_VERSION; }

const char* mpmc_gpu_flash_last_error(void) { return g_last_error.c_str(); }

int mpmc_gpu_flash_components(const mpmc_gpu_flash* h) { return h ? h->n : 0; }

int mpmc_gpu_flash_batch_stats(mpmc_gpu_flash* h, int64_t* out, int capacity) {
    if (!h || (h->form != MPMC_FORM_MIXED && h->form != MPMC_FORM_BATCHED) || !h->workspace.ptr) return 0;
    // workspace counter slots (pr76_batched.cuh Slot) in the documented order
    // negative entries: a 64-bit total held in slots -s and -s + 1
    constexpr int kSlots[] = {8, 9, 10, 11, 12, 13, 14, 15, 16, 17, 18, 20, 22, 23, 24, 25, 27, 28, 29, 30, 31, 32, 33,
                              -34, -36, -38, -40, -42, 44, 45, 4, 46};
    constexpr int kCount = static_cast<int>(sizeof(kSlots) / sizeof(kSlots[0]));
    if (cudaSetDevice(h->device) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return 0;
    for (int k = 0; k < kCount && k < capacity; ++k)
        if (out) out[k] = 0;
    // the counters are the first array of each range's workspace; sums over ranges
    for (int r = 0; r < h->last_ranges; ++r) {
        int vals[48] = {};
        if (cudaMemcpy(vals, static_cast<char*>(h->workspace.ptr) + h->range_offset[r], sizeof(vals),
                       cudaMemcpyDeviceToHost) != cudaSuccess)
            return 0;
        for (int k = 0; k < kCount && k < capacity; ++k) {
            if (!out) continue;
            if (kSlots[k] >= 0) {
                out[k] += vals[kSlots[k]];
            } else {
                unsigned long long v = 0;
                std::memcpy(&v, vals - kSlots[k], sizeof(v));
                out[k] += static_cast<int64_t>(v);
            }
        }
    }
    return kCount;
}

int mpmc_gpu_flash_stage_timings(mpmc_gpu_flash* h, float* ms, int capacity) {
    if (!h || !h->stage_timing || h->n_events < 2) return 0;
    if (cudaEventSynchronize(h->events[h->n_events - 1]) != cudaSuccess) return 0;
    const int stages = h->n_events - 1;
    for (int k = 0; k < stages && k < capacity; ++k) {
        float v = 0.f;
        cudaEventElapsedTime(&v, h->events[k], h->events[k + 1]);
        // after a warm pass, each stage's time is that of both passes
        // each stage's time is that of every pass the solve ran (first, then
        // the cold pass after a warm pass, then the exact sub-solve)
        if (k < pr76::kBatchedStages) {
            float r = 0.f;
            if (h->timed_warm) {
                cudaEventElapsedTime(&r, h->redo_events[k], h->redo_events[k + 1]);
                v += r;
            }
            if (h->timed_exact) {
                cudaEventElapsedTime(&r, h->exact_events[k], h->exact_events[k + 1]);
                v += r;
            }
        } else if (k == pr76::kBatchedStages && (h->timed_warm || h->timed_exact)) {
            // the sensitivity stage follows the last pass
            cudaEventElapsedTime(&v, h->timed_exact ? h->exact_events[pr76::kBatchedStages]
                                                    : h->redo_events[pr76::kBatchedStages],
                                 h->events[k + 1]);
        }
        if (ms) ms[k] = v;
    }
    return stages;
}

int mpmc_gpu_flash_create(const mpmc_pr76_mixture* mixture, const mpmc_flash_options* options,
                          mpmc_gpu_flash** out) {
    if (!mixture || !out) return fail(MPMC_ERR_INVALID_ARGUMENT, "mixture and out must not be null");
    *out = nullptr;
    mpmc_flash_options opt{};
    if (options) opt = *options;
    if (opt.form != MPMC_FORM_PLAIN_FP64 && opt.form != MPMC_FORM_BATCHED && opt.form != MPMC_FORM_MIXED)
        return fail(MPMC_ERR_INVALID_ARGUMENT, "unknown algorithm form");
    pr76::Mixture m;
    const int rc = prepare_mixture(mixture, m);
    if (rc != MPMC_OK) return rc;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
    if (opt.device < 0 || opt.device >= count) return fail(MPMC_ERR_INVALID_ARGUMENT, "device ordinal out of range");
    e = cudaSetDevice(opt.device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    mpmc_gpu_flash* h = new mpmc_gpu_flash();
    h->n = m.n;
    h->device = opt.device;
    h->form = opt.form;
    h->want_sensitivity = opt.want_sensitivity;
    h->stage_timing = (opt.flags & MPMC_FLAG_STAGE_TIMING) != 0;
    h->use_graphs = (opt.flags & MPMC_FLAG_CUDA_GRAPH) != 0;
    h->sens_lanes = (opt.flags & MPMC_FLAG_SENSITIVITY_LANES) != 0;
    h->max3_newton = (opt.flags & MPMC_FLAG_MAX3_NEWTON_ROOTS) != 0;
    h->polish_stream = (opt.flags & MPMC_FLAG_POLISH_STREAM) != 0;
    h->host_mixture = m;
    e = cudaMalloc(&h->d_mixture, sizeof(pr76::Mixture));
    if (e == cudaSuccess) e = cudaMemcpy(h->d_mixture, &m, sizeof(pr76::Mixture), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        mpmc_gpu_flash_destroy(h);
        return cuda_fail(e, "mpmc_gpu_flash_create");
    }
    *out = h;
    g_last_error.clear();
    return MPMC_OK;
}

int mpmc_gpu_flash_destroy(mpmc_gpu_flash* h) {
    if (!h) return MPMC_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    h->in_p.release();
    h->in_t.release();
    h->in_z.release();
    h->in_warm.release();
    for (auto& b : h->outs3) b.release();
    for (auto& b : h->in_hints) b.release();
    for (auto& b : h->chart_in) b.release();
    for (auto& b : h->chart_out) b.release();
    for (auto& b : h->outs) b.release();
    for (auto& b : h->sens_inputs) b.release();
    h->workspace.release();
    for (auto& ev : h->events)
        if (ev) cudaEventDestroy(ev);
    for (auto& ev : h->redo_events)
        if (ev) cudaEventDestroy(ev);
    for (auto& ev : h->exact_events)
        if (ev) cudaEventDestroy(ev);
    if (h->copy_stream) {
        cudaStreamSynchronize(h->copy_stream);
        cudaStreamDestroy(h->copy_stream);
    }
    for (int r = 0; r < kMaxRanges; ++r) {
        if (h->range_streams[r]) {
            cudaStreamSynchronize(h->range_streams[r]);
            cudaStreamDestroy(h->range_streams[r]);
        }
        if (h->join_events[r]) cudaEventDestroy(h->join_events[r]);
    }
    if (h->fork_event) cudaEventDestroy(h->fork_event);
    if (h->side_stream) {
        cudaStreamSynchronize(h->side_stream);
        cudaStreamDestroy(h->side_stream);
    }
    if (h->side_fork) cudaEventDestroy(h->side_fork);
    if (h->side_join) cudaEventDestroy(h->side_join);
    if (h->flash_done) cudaEventDestroy(h->flash_done);
    for (auto& ev : h->chunk_done)
        if (ev) cudaEventDestroy(ev);
    for (auto& g : h->graphs) cudaGraphExecDestroy(g.exec);
    if (h->d_mixture) cudaFree(h->d_mixture);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return MPMC_OK;
}

int mpmc_gpu_flash_solve_device(mpmc_gpu_flash* h, int64_t ncell, const double* p, const double* t,
                                const double* z, const mpmc_flash_outputs* out, void* stream) {
    return mpmc_gpu_flash_solve_device_warm(h, ncell, p, t, z, nullptr, out, stream);
}

int mpmc_gpu_flash_solve_device_max3(mpmc_gpu_flash* h, int64_t ncell, const double* p, const double* t,
                                     const double* z, const mpmc_flash_outputs* out,
                                     const mpmc_three_phase_outputs* out3, void* stream) {
    if (!h) return fail(MPMC_ERR_INVALID_ARGUMENT, "null handle");
    if (ncell < 0) return fail(MPMC_ERR_INVALID_ARGUMENT, "negative cell count");
    if (ncell == 0) return MPMC_OK;
    if (!p || !t || !z) return fail(MPMC_ERR_INVALID_ARGUMENT, "p, t and z must not be null");
    if (!out || !out->status || !out->ln_k)
        return fail(MPMC_ERR_INVALID_ARGUMENT, "max-3-phase solve: the status and ln_k outputs are required");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    pr76::Max3Outputs m3{};
    if (out3) m3 = {out3->max3_status, out3->phase_fraction, out3->composition, out3->ln_phi, out3->z_factor};
    return run_device(h, ncell, p, t, z, nullptr, to_device_outputs(out), static_cast<cudaStream_t>(stream), &m3);
}

int mpmc_gpu_flash_solve_device_warm(mpmc_gpu_flash* h, int64_t ncell, const double* p, const double* t,
                                     const double* z, const double* ln_k_warm, const mpmc_flash_outputs* out,
                                     void* stream) {
    if (!h) return fail(MPMC_ERR_INVALID_ARGUMENT, "null handle");
    if (ncell < 0) return fail(MPMC_ERR_INVALID_ARGUMENT, "negative cell count");
    if (ncell == 0) return MPMC_OK;
    if (!p || !t || !z) return fail(MPMC_ERR_INVALID_ARGUMENT, "p, t and z must not be null");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    return run_device(h, ncell, p, t, z, ln_k_warm, to_device_outputs(out), static_cast<cudaStream_t>(stream));
}

int mpmc_gpu_flash_set_launch_shape(mpmc_gpu_flash* h, const int32_t* values, int count) {
    if (!h) return fail(MPMC_ERR_INVALID_ARGUMENT, "null handle");
    if (count < 0 || count > 10 || (count > 0 && !values))
        return fail(MPMC_ERR_INVALID_ARGUMENT, "launch shape: 0 to 10 values");
    for (int k = 0; k < count; ++k)
        if (values[k] < 0 || values[k] > (k == 6 ? 1000000 : (k == 5 ? 255 : (k >= 8 ? 512 : 64))))
            return fail(MPMC_ERR_INVALID_ARGUMENT, "launch shape value out of range");
    for (int k = 0; k < 10; ++k) h->shape[k] = k < count ? values[k] : 0;
    cudaSetDevice(h->device);
    for (auto& g : h->graphs) cudaGraphExecDestroy(g.exec);  // captured with the old shape
    h->graphs.clear();
    return MPMC_OK;
}

int mpmc_gpu_flash_solve_device_noalloc(mpmc_gpu_flash* h, int64_t ncell, const double* p, const double* t,
                                        const double* z, const mpmc_flash_outputs* out, void* stream) {
    if (!h) return fail(MPMC_ERR_INVALID_ARGUMENT, "null handle");
    if (h->form != MPMC_FORM_MIXED)
        return fail(MPMC_ERR_UNSUPPORTED, "the no-allocation entry point serves mixed-precision handles only");
    if (ncell < 0) return fail(MPMC_ERR_INVALID_ARGUMENT, "negative cell count");
    if (ncell == 0) return MPMC_OK;
    if (!p || !t || !z) return fail(MPMC_ERR_INVALID_ARGUMENT, "p, t and z must not be null");
    if (ncell >= (int64_t{1} << 24))
        return fail(MPMC_ERR_INVALID_ARGUMENT, "mixed form: at most 16,777,215 cells per call");
    // the least scratch that runs: one FP64 attempt item per cell
    const size_t need = pr76::batched_workspace_bytes(h->n, ncell, false, 1);
    if (need > MPMC_NOALLOC_SCRATCH_BYTES)
        return fail(MPMC_ERR_INVALID_ARGUMENT,
                    "no-allocation entry point: " + std::to_string(ncell) + " cells of " + std::to_string(h->n) +
                        " components need " + std::to_string(need) + " bytes of scratch, above the fixed " +
                        std::to_string(MPMC_NOALLOC_SCRATCH_BYTES) + " (use mpmc_gpu_flash_solve_device)");
    const pr76::DeviceOutputs d = to_device_outputs(out);
    if (h->want_sensitivity && (!d.status || !d.beta || !d.x || !d.y || !d.lnk || !d.z_l || !d.z_v))
        return fail(MPMC_ERR_INVALID_ARGUMENT,
                    "no-allocation entry point with sensitivities: status, vapor_fraction, liquid, vapor, ln_k, "
                    "z_liquid and z_vapor outputs are required");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    void* scratch = nullptr;
    const int rc = noalloc_scratch(h->device, &scratch);
    if (rc != MPMC_OK) return rc;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    const pr76::BatchedShape shape = batched_shape(h, nullptr);
    e = pr76::launch_batched(h->n, h->d_mixture, ncell, p, t, z, d, scratch, MPMC_NOALLOC_SCRATCH_BYTES, shape, s);
    if (e != cudaSuccess) return cuda_fail(e, "flash kernel launch");
    if (h->want_sensitivity) {
        e = pr76::launch_sensitivity(h->n, h->d_mixture, ncell, p, t, z, d, s, 0, -1, h->sens_lanes);
        if (e != cudaSuccess) return cuda_fail(e, "sensitivity kernel launch");
    }
    return MPMC_OK;
}

int mpmc_gpu_flash_solve(mpmc_gpu_flash* h, int64_t ncell, const double* p, const double* t, const double* z,
                         const mpmc_flash_outputs* out) {
    return mpmc_gpu_flash_solve_warm(h, ncell, p, t, z, nullptr, out);
}

int mpmc_gpu_flash_solve_max3(mpmc_gpu_flash* h, int64_t ncell, const double* p, const double* t, const double* z,
                              const mpmc_flash_outputs* out, const mpmc_three_phase_outputs* out3) {
    return solve_host(h, ncell, p, t, z, nullptr, out, out3, true);
}

int mpmc_gpu_flash_solve_warm(mpmc_gpu_flash* h, int64_t ncell, const double* p, const double* t, const double* z,
                              const double* ln_k_warm, const mpmc_flash_outputs* out) {
    return solve_host(h, ncell, p, t, z, ln_k_warm, out, nullptr, false);
}

int mpmc_gpu_flash_solve_hinted(mpmc_gpu_flash* h, int64_t ncell, const double* p, const double* t, const double* z,
                                const mpmc_start_hints* hints, const mpmc_flash_outputs* out,
                                const mpmc_three_phase_outputs* out3) {
    if (!h) return fail(MPMC_ERR_INVALID_ARGUMENT, "null handle");
    if (!hints || (ncell > 0 && (!hints->count || !hints->composition)) ||
        (hints->three_phase != nullptr) != (hints->fraction != nullptr))
        return fail(MPMC_ERR_INVALID_ARGUMENT, "hinted solve: count and composition required, three_phase and "
                                               "fraction together");
    const pr76::Hints hh = hints_of(hints);
    return solve_host(h, ncell, p, t, z, nullptr, out, out3, true, &hh);
}

int mpmc_gpu_flash_solve_hinted_ex(mpmc_gpu_flash* h, int64_t ncell, const double* p, const double* t,
                                   const double* z, const mpmc_start_hints_ex* hints, const mpmc_flash_outputs* out,
                                   const mpmc_three_phase_outputs* out3) {
    if (!h) return fail(MPMC_ERR_INVALID_ARGUMENT, "null handle");
    const int rc = check_hints_ex(hints);
    if (rc != MPMC_OK) return rc;
    const pr76::Hints hh = hints_of(hints);
    return solve_host(h, ncell, p, t, z, nullptr, out, out3, true, &hh);
}

int mpmc_gpu_flash_solve_device_hinted(mpmc_gpu_flash* h, int64_t ncell, const double* p, const double* t,
                                       const double* z, const mpmc_start_hints* hints,
                                       const mpmc_flash_outputs* out, const mpmc_three_phase_outputs* out3,
                                       void* stream) {
    if (!h) return fail(MPMC_ERR_INVALID_ARGUMENT, "null handle");
    if (ncell < 0) return fail(MPMC_ERR_INVALID_ARGUMENT, "negative cell count");
    if (ncell == 0) return MPMC_OK;
    if (!p || !t || !z) return fail(MPMC_ERR_INVALID_ARGUMENT, "p, t and z must not be null");
    if (!hints || !hints->count || !hints->composition ||
        (hints->three_phase != nullptr) != (hints->fraction != nullptr))
        return fail(MPMC_ERR_INVALID_ARGUMENT, "hinted solve: count and composition required, three_phase and "
                                               "fraction together");
    if (!out || !out->status || !out->ln_k)
        return fail(MPMC_ERR_INVALID_ARGUMENT, "hinted solve: the status and ln_k outputs are required");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    pr76::Max3Outputs m3{};
    if (out3) m3 = {out3->max3_status, out3->phase_fraction, out3->composition, out3->ln_phi, out3->z_factor};
    const pr76::Hints dh = hints_of(hints);
    return run_device(h, ncell, p, t, z, nullptr, to_device_outputs(out), static_cast<cudaStream_t>(stream), &m3,
                      &dh);
}

int mpmc_gpu_flash_solve_device_hinted_ex(mpmc_gpu_flash* h, int64_t ncell, const double* p, const double* t,
                                          const double* z, const mpmc_start_hints_ex* hints,
                                          const mpmc_flash_outputs* out, const mpmc_three_phase_outputs* out3,
                                          void* stream) {
    if (!h) return fail(MPMC_ERR_INVALID_ARGUMENT, "null handle");
    if (ncell < 0) return fail(MPMC_ERR_INVALID_ARGUMENT, "negative cell count");
    const int rc = check_hints_ex(hints);
    if (rc != MPMC_OK) return rc;
    if (ncell == 0) return MPMC_OK;
    if (!p || !t || !z) return fail(MPMC_ERR_INVALID_ARGUMENT, "p, t and z must not be null");
    if (!out || !out->status || !out->ln_k)
        return fail(MPMC_ERR_INVALID_ARGUMENT, "hinted solve: the status and ln_k outputs are required");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    pr76::Max3Outputs m3{};
    if (out3) m3 = {out3->max3_status, out3->phase_fraction, out3->composition, out3->ln_phi, out3->z_factor};
    const pr76::Hints dh = hints_of(hints);
    return run_device(h, ncell, p, t, z, nullptr, to_device_outputs(out), static_cast<cudaStream_t>(stream), &m3,
                      &dh);
}

int mpmc_gpu_flash_property_chart_device(mpmc_gpu_flash* h, int64_t ncell, const mpmc_property_chart_spec* spec,
                                         const double* q, const int32_t* dependent,
                                         const mpmc_property_chart_outputs* out, void* stream) {
    pr76::ChartParams params;
    const int rc = chart_params(h, ncell, spec, q, params);
    if (rc != MPMC_OK || ncell == 0) return rc;
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    pr76::ChartOutputs d{};
    if (out) d = {out->status, out->values, out->jacobian};
    e = pr76::launch_chart(h->n, h->d_mixture, params, ncell, q, dependent, d, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "property chart launch");
    return MPMC_OK;
}

int mpmc_gpu_flash_property_chart(mpmc_gpu_flash* h, int64_t ncell, const mpmc_property_chart_spec* spec,
                                  const double* q, const int32_t* dependent, const mpmc_property_chart_outputs* out) {
    pr76::ChartParams params;
    const int rc = chart_params(h, ncell, spec, q, params);
    if (rc != MPMC_OK || ncell == 0) return rc;
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    const size_t nc = static_cast<size_t>(ncell);
    const size_t cols = static_cast<size_t>(params.phases) * h->n + 1;
    const size_t rows = static_cast<size_t>(params.phases) * (5 + h->n) + static_cast<size_t>(params.phases - 1) * h->n;
    const size_t bytes_in[2] = {cols * nc * sizeof(double), dependent ? params.phases * nc * sizeof(int32_t) : 0};
    void* host_out[3] = {};
    if (out) {
        host_out[0] = out->status;
        host_out[1] = out->values;
        host_out[2] = out->jacobian;
    }
    const size_t bytes_out[3] = {nc * sizeof(int32_t), rows * nc * sizeof(double), rows * cols * nc * sizeof(double)};
    for (int k = 0; k < 2; ++k)
        if (bytes_in[k] && (e = h->chart_in[k].ensure(bytes_in[k])) != cudaSuccess)
            return cuda_fail(e, "property chart input staging allocation");
    void* dev_out[3] = {};
    for (int k = 0; k < 3; ++k) {
        if (!host_out[k]) continue;
        if ((e = h->chart_out[k].ensure(bytes_out[k])) != cudaSuccess)
            return cuda_fail(e, "property chart output staging allocation");
        dev_out[k] = h->chart_out[k].ptr;
    }
    cudaStream_t s = h->stream;
    if ((e = cudaMemcpyAsync(h->chart_in[0].ptr, q, bytes_in[0], cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return cuda_fail(e, "property chart input copy");
    if (dependent &&
        (e = cudaMemcpyAsync(h->chart_in[1].ptr, dependent, bytes_in[1], cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return cuda_fail(e, "property chart input copy");
    const pr76::ChartOutputs d{static_cast<int32_t*>(dev_out[0]), static_cast<double*>(dev_out[1]),
                               static_cast<double*>(dev_out[2])};
    e = pr76::launch_chart(h->n, h->d_mixture, params, ncell, static_cast<const double*>(h->chart_in[0].ptr),
                           dependent ? static_cast<const int32_t*>(h->chart_in[1].ptr) : nullptr, d, s);
    if (e != cudaSuccess) return cuda_fail(e, "property chart launch");
    for (int k = 0; k < 3; ++k) {
        if (!host_out[k]) continue;
        if ((e = cudaMemcpyAsync(host_out[k], dev_out[k], bytes_out[k], cudaMemcpyDeviceToHost, s)) != cudaSuccess)
            return cuda_fail(e, "property chart output copy");
    }
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e, "property chart execution");
    return MPMC_OK;
}

}  // extern "C"

namespace {

// The host-buffer entry: stage inputs, solve on the handle's stream, copy the
// requested outputs back, synchronise.
int solve_host(mpmc_gpu_flash* h, int64_t ncell, const double* p, const double* t, const double* z,
               const double* ln_k_warm, const mpmc_flash_outputs* out, const mpmc_three_phase_outputs* out3,
               bool max3, const pr76::Hints* hints) {
    if (!h) return fail(MPMC_ERR_INVALID_ARGUMENT, "null handle");
    if (max3 && (!out || !out->status || !out->ln_k))
        return fail(MPMC_ERR_INVALID_ARGUMENT, "max-3-phase solve: the status and ln_k outputs are required");
    if (ncell < 0) return fail(MPMC_ERR_INVALID_ARGUMENT, "negative cell count");
    if (ncell == 0) return MPMC_OK;
    if (!p || !t || !z) return fail(MPMC_ERR_INVALID_ARGUMENT, "p, t and z must not be null");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    const size_t nc = static_cast<size_t>(ncell);
    const size_t n = static_cast<size_t>(h->n);
    if ((e = h->in_p.ensure(nc * 8)) != cudaSuccess || (e = h->in_t.ensure(nc * 8)) != cudaSuccess ||
        (e = h->in_z.ensure(n * nc * 8)) != cudaSuccess)
        return cuda_fail(e, "input staging allocation");
    size_t per_cell[kOutputFields], elem[kOutputFields];
    field_sizes(h->n, per_cell, elem);
    mpmc_flash_outputs host_out{};
    if (out) host_out = *out;
    mpmc_flash_outputs dev_out{};
    for (int k = 0; k < kOutputFields; ++k) {
        void* hp = *field_ptr(&host_out, k);
        if (!hp) continue;
        if ((e = h->outs[k].ensure(per_cell[k] * elem[k] * nc)) != cudaSuccess)
            return cuda_fail(e, "output staging allocation");
        *field_ptr(&dev_out, k) = h->outs[k].ptr;
    }
    cudaStream_t s = h->stream;
    if ((e = cudaMemcpyAsync(h->in_p.ptr, p, nc * 8, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(h->in_t.ptr, t, nc * 8, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(h->in_z.ptr, z, n * nc * 8, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return cuda_fail(e, "input copy");
    const double* d_warm = nullptr;
    if (ln_k_warm) {
        if ((e = h->in_warm.ensure(n * nc * 8)) != cudaSuccess) return cuda_fail(e, "warm-start staging allocation");
        if ((e = cudaMemcpyAsync(h->in_warm.ptr, ln_k_warm, n * nc * 8, cudaMemcpyHostToDevice, s)) != cudaSuccess)
            return cuda_fail(e, "warm-start copy");
        d_warm = static_cast<const double*>(h->in_warm.ptr);
    }
    // three-phase outputs: staged like the others
    void* host3[5] = {};
    size_t bytes3[5] = {sizeof(int32_t), 3 * sizeof(double), 3 * n * sizeof(double), 3 * n * sizeof(double),
                        3 * sizeof(double)};
    pr76::Max3Outputs m3{};
    if (max3) {
        if (out3) {
            host3[0] = out3->max3_status;
            host3[1] = out3->phase_fraction;
            host3[2] = out3->composition;
            host3[3] = out3->ln_phi;
            host3[4] = out3->z_factor;
        }
        void* dev3[5] = {};
        for (int k = 0; k < 5; ++k) {
            if (!host3[k]) continue;
            if ((e = h->outs3[k].ensure(bytes3[k] * nc)) != cudaSuccess)
                return cuda_fail(e, "three-phase output staging allocation");
            dev3[k] = h->outs3[k].ptr;
        }
        m3 = {static_cast<int32_t*>(dev3[0]), static_cast<double*>(dev3[1]), static_cast<double*>(dev3[2]),
              static_cast<double*>(dev3[3]), static_cast<double*>(dev3[4])};
    }
    // caller start hints: every array present staged like the inputs
    pr76::Hints dh{};
    if (hints) {
        dh = *hints;
        int slot = 0;
        auto stage = [&](auto*& field, size_t bytes) -> cudaError_t {
            DevBuf& b = h->in_hints[slot++];
            if (!field) return cudaSuccess;
            cudaError_t err = b.ensure(bytes);
            if (err == cudaSuccess) err = cudaMemcpyAsync(b.ptr, field, bytes, cudaMemcpyHostToDevice, s);
            if (err == cudaSuccess) field = static_cast<std::remove_reference_t<decltype(field)>>(b.ptr);
            return err;
        };
        const size_t counts = nc * sizeof(int32_t), comps = 3 * n * nc * sizeof(double);
        if ((e = stage(dh.count, counts)) != cudaSuccess || (e = stage(dh.x, comps)) != cudaSuccess ||
            (e = stage(dh.final_count, counts)) != cudaSuccess || (e = stage(dh.final_x, comps)) != cudaSuccess ||
            (e = stage(dh.three, counts)) != cudaSuccess || (e = stage(dh.three_x, comps)) != cudaSuccess ||
            (e = stage(dh.fraction, 2 * nc * sizeof(double))) != cudaSuccess)
            return cuda_fail(e, "hint staging");
    }
    // With sensitivities requested, the copy-out of the flash fields overlaps
    // the sensitivity stage: a second stream copies them while `s` runs the
    // sensitivities, then copies the derivative fields.
    bool overlap = h->want_sensitivity && !max3 && !hints && !h->stage_timing;
    bool any_sens = false;
    for (int k = 10; k < kOutputFields; ++k) any_sens = any_sens || *field_ptr(&host_out, k) != nullptr;
    overlap = overlap && any_sens;
    const double* dp_ = static_cast<const double*>(h->in_p.ptr);
    const double* dt_ = static_cast<const double*>(h->in_t.ptr);
    const double* dz_ = static_cast<const double*>(h->in_z.ptr);
    const int rc = run_device(h, ncell, dp_, dt_, dz_, d_warm, to_device_outputs(&dev_out), s, max3 ? &m3 : nullptr,
                              hints ? &dh : nullptr, !overlap);
    if (rc != MPMC_OK) return rc;
    if (overlap) {
        if (!h->copy_stream) {
            if ((e = cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking)) != cudaSuccess)
                return cuda_fail(e, "copy stream");
            if ((e = cudaEventCreateWithFlags(&h->flash_done, cudaEventDisableTiming)) != cudaSuccess)
                return cuda_fail(e, "cudaEventCreate");
            for (auto& ev : h->chunk_done)
                if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess)
                    return cuda_fail(e, "cudaEventCreate");
        }
        cudaStream_t cs = h->copy_stream;
        pr76::DeviceOutputs d = to_device_outputs(&dev_out);
        const int irc = with_sensitivity_inputs(h, ncell, d);  // the scratch run_device routed them to
        if (irc != MPMC_OK) return irc;
        if ((e = cudaEventRecord(h->flash_done, s)) != cudaSuccess || (e = cudaStreamWaitEvent(cs, h->flash_done, 0)) !=
                                                                          cudaSuccess)
            return cuda_fail(e, "copy stream ordering");
        for (int k = 0; k < 10; ++k) {
            void* hp = *field_ptr(&host_out, k);
            if (!hp) continue;
            if ((e = cudaMemcpyAsync(hp, h->outs[k].ptr, per_cell[k] * elem[k] * nc, cudaMemcpyDeviceToHost, cs)) !=
                cudaSuccess)
                return cuda_fail(e, "output copy");
        }
        // the sensitivities in one launch, then every derivative field in one
        // contiguous copy: measured on a GB300 (1M cells, N = 10), 80 ms less
        // per call than eight cell ranges each copied as 2D row segments
        e = pr76::launch_sensitivity(h->n, h->d_mixture, ncell, dp_, dt_, dz_, d, s, 0, -1, h->sens_lanes);
        if (e != cudaSuccess) return cuda_fail(e, "sensitivity kernel launch");
        if ((e = cudaEventRecord(h->chunk_done[0], s)) != cudaSuccess ||
            (e = cudaStreamWaitEvent(cs, h->chunk_done[0], 0)) != cudaSuccess)
            return cuda_fail(e, "copy stream ordering");
        for (int k = 10; k < kOutputFields; ++k) {
            void* hp = *field_ptr(&host_out, k);
            if (!hp) continue;
            if ((e = cudaMemcpyAsync(hp, h->outs[k].ptr, per_cell[k] * elem[k] * nc, cudaMemcpyDeviceToHost, cs)) !=
                cudaSuccess)
                return cuda_fail(e, "output copy");
        }
        if ((e = cudaStreamSynchronize(cs)) != cudaSuccess || (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return cuda_fail(e, "flash execution");
        return MPMC_OK;
    }
    for (int k = 0; k < kOutputFields; ++k) {
        void* hp = *field_ptr(&host_out, k);
        if (!hp) continue;
        if ((e = cudaMemcpyAsync(hp, h->outs[k].ptr, per_cell[k] * elem[k] * nc, cudaMemcpyDeviceToHost, s)) !=
            cudaSuccess)
            return cuda_fail(e, "output copy");
    }
    for (int k = 0; k < 5; ++k) {
        if (!host3[k]) continue;
        if ((e = cudaMemcpyAsync(host3[k], h->outs3[k].ptr, bytes3[k] * nc, cudaMemcpyDeviceToHost, s)) !=
            cudaSuccess)
            return cuda_fail(e, "three-phase output copy");
    }
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e, "flash execution");
    return MPMC_OK;
}

}  // namespace
