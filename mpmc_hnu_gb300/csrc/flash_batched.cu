// Host orchestration of the batched mixed-precision flash (pr76_batched.cuh).
// Compiled once per component capacity (-DMPMC_NM).  Every stage is enqueued
// on one stream with fixed launch shapes; the work sizes live in device
// counters, so the sequence needs no host synchronisation and can be
// captured into a CUDA graph by the caller.
#include "launch.h"
#include "pr76_batched64.cuh"
#include "pr76_warp64.cuh"

#ifndef MPMC_NM
#error "compile with -DMPMC_NM=<capacity>"
#endif
#define MPMC_CAT2(a, b) a##b
#define MPMC_CAT(a, b) MPMC_CAT2(a, b)

namespace pr76 {
namespace MPMC_CAT(batched_host_nm, MPMC_NM) {

constexpr int NM = MPMC_NM;

size_t align256(size_t x) { return (x + 255) & ~static_cast<size_t>(255); }

// Carves the workspace arrays out of one scratch allocation; with base ==
// nullptr only computes the size.
// The exact sub-solve of the mixed form (cells FP32 could not screen, solved
// again with every trial and attempt in FP64): its packed inputs and outputs
// and the FP64 form's workspace for `cap` cells, carved after the main
// workspace.
struct ExactRegion {
    double *p = nullptr, *t = nullptr, *z = nullptr;
    DeviceOutputs out{};
    char* scratch = nullptr;
    size_t scratch_bytes = 0;
};

size_t carve(batched::Workspace& ws, char* base, int n, int64_t ncell, bool fp64_items, int s64_per_cell,
             int exact_cap = 0, ExactRegion* exact = nullptr);

// Cells the exact sub-solve holds for a batch of ncell: all of a small batch,
// an eighth of a large one (at least 65,536).
int exact_capacity(int64_t ncell) {
    return static_cast<int>(ncell <= 65536 ? ncell : std::max<int64_t>(65536, ncell / 8));
}

size_t carve(batched::Workspace& ws, char* base, int n, int64_t ncell, bool fp64_items, int s64_per_cell,
             int exact_cap, ExactRegion* exact) {
    const size_t nc = static_cast<size_t>(ncell);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char* p = base ? base + off : nullptr;
        off += align256(bytes);
        return p;
    };
    ws.ncell = ncell;
    ws.n = n;
    ws.counters = reinterpret_cast<int*>(take(sizeof(int) * batched::qSlots));
    ws.phase = reinterpret_cast<int*>(take(sizeof(int) * nc));
    ws.trial_cells = reinterpret_cast<int*>(take(sizeof(int) * nc));
    ws.attempt_items = reinterpret_cast<int*>(take(sizeof(int) * batched::kMaxAttempts * nc));
    ws.z = reinterpret_cast<double*>(take(sizeof(double) * NM * nc));
    ws.ref_lnphi = reinterpret_cast<double*>(take(sizeof(double) * NM * nc));
    ws.ref_z = reinterpret_cast<double*>(take(sizeof(double) * nc));
    ws.tw = reinterpret_cast<float*>(take(sizeof(float) * (NM + 4) * NM * nc));
    ws.tclass = reinterpret_cast<signed char*>(take((NM + 4) * nc));
    ws.titer = reinterpret_cast<short*>(take(sizeof(short) * (NM + 4) * nc));
    ws.att_lnk = reinterpret_cast<float*>(take(sizeof(float) * batched::kMaxAttempts * NM * nc));
    ws.att_gibbs = reinterpret_cast<float*>(take(sizeof(float) * batched::kMaxAttempts * nc));
    ws.att_class = reinterpret_cast<signed char*>(take(batched::kMaxAttempts * nc));
    ws.att_count = reinterpret_cast<int*>(take(sizeof(int) * nc));
    ws.att_iter = reinterpret_cast<short*>(take(sizeof(short) * batched::kMaxAttempts * nc));
    ws.att_lnk64 = reinterpret_cast<double*>(take(sizeof(double) * batched::kMaxAttempts * NM * nc));
    ws.fp64_items = fp64_items ? 1 : 0;
    ws.att_rate = reinterpret_cast<float*>(take(sizeof(float) * batched::kMaxAttempts * nc));
    ws.cand = reinterpret_cast<double*>(take(sizeof(double) * 7 * NM * nc));
    ws.cand_s = reinterpret_cast<double*>(take(sizeof(double) * 8 * nc));
    ws.counters_out = reinterpret_cast<int*>(take(sizeof(int) * cCount * nc));
    ws.c32 = reinterpret_cast<float*>(take(sizeof(float) * 4 * NM * nc));
    ws.ref32 = reinterpret_cast<float*>(take(sizeof(float) * NM * nc));
    ws.t64_items = reinterpret_cast<int*>(take(sizeof(int) * (NM + 4) * nc));
    ws.t64_status = reinterpret_cast<signed char*>(take((NM + 4) * nc));
    ws.tw64 = reinterpret_cast<double*>(take(sizeof(double) * (NM + 4) * NM * nc));
    // FP64 attempt items: every attempt of every cell in the FP64 form; the
    // unsettled attempts of the mixed form, s64_per_cell per cell (at least
    // 16384 items).  A cell whose items do not fit runs the plain fallback.
    const size_t per = static_cast<size_t>(s64_per_cell < 1 ? 1 : s64_per_cell);
    ws.s64_capacity = static_cast<int>(fp64_items ? batched::kMaxAttempts * nc
                                                  : (per * nc < 4 * 4096 ? 4 * 4096 : per * nc));
    const size_t cap = static_cast<size_t>(ws.s64_capacity);
    ws.s64_items = reinterpret_cast<int*>(take(sizeof(int) * cap));
    ws.s64_status = reinterpret_cast<signed char*>(take(cap));
    ws.s64_state = reinterpret_cast<double*>(take(sizeof(double) * batched::S64Stride<NM>() * cap));
    ws.split_cells = reinterpret_cast<int*>(take(sizeof(int) * nc));
    ws.warm_cell = reinterpret_cast<signed char*>(take(nc));
    ws.s64_cells = reinterpret_cast<int*>(take(sizeof(int) * nc));
    ws.s64_base = reinterpret_cast<int*>(take(sizeof(int) * nc));
    ws.s64_count = reinterpret_cast<int*>(take(sizeof(int) * nc));
    ws.exact_capacity = fp64_items ? 0 : exact_cap;
    ws.exact_list = reinterpret_cast<int*>(take(sizeof(int) * static_cast<size_t>(ws.exact_capacity)));
    if (ws.exact_capacity > 0) {
        const size_t cap = static_cast<size_t>(ws.exact_capacity);
        ExactRegion r;
        r.p = reinterpret_cast<double*>(take(sizeof(double) * cap));
        r.t = reinterpret_cast<double*>(take(sizeof(double) * cap));
        r.z = reinterpret_cast<double*>(take(sizeof(double) * NM * cap));
        r.out.status = reinterpret_cast<int32_t*>(take(sizeof(int32_t) * cap));
        r.out.beta = reinterpret_cast<double*>(take(sizeof(double) * cap));
        r.out.x = reinterpret_cast<double*>(take(sizeof(double) * NM * cap));
        r.out.y = reinterpret_cast<double*>(take(sizeof(double) * NM * cap));
        r.out.lnk = reinterpret_cast<double*>(take(sizeof(double) * NM * cap));
        r.out.lnphi_l = reinterpret_cast<double*>(take(sizeof(double) * NM * cap));
        r.out.lnphi_v = reinterpret_cast<double*>(take(sizeof(double) * NM * cap));
        r.out.z_l = reinterpret_cast<double*>(take(sizeof(double) * cap));
        r.out.z_v = reinterpret_cast<double*>(take(sizeof(double) * cap));
        r.out.counters = reinterpret_cast<int32_t*>(take(sizeof(int32_t) * cCount * cap));
        batched::Workspace sub;
        r.scratch_bytes = carve(sub, nullptr, n, ws.exact_capacity, true, kS64PerCell);
        r.scratch = take(r.scratch_bytes);
        if (exact) *exact = r;
    }
    return off;
}

template <typename K>
int resident_blocks(K kernel, int block) {
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kernel, block, 0) != cudaSuccess || blocks < 1) blocks = 1;
    return blocks;
}

}  // namespace batched_host_nm<NM>
using namespace MPMC_CAT(batched_host_nm, MPMC_NM);

size_t MPMC_CAT(batched_workspace_bytes_nm, MPMC_NM)(int n, int64_t ncell, bool fp64_items, int s64_per_cell) {
    batched::Workspace ws;
    // s64_per_cell below the full capacity: the least scratch that runs, with
    // no exact sub-solve (its cells take the plain fallback)
    return carve(ws, nullptr, n, ncell, fp64_items, s64_per_cell,
                 s64_per_cell >= kS64PerCell ? exact_capacity(ncell) : 0);
}

cudaError_t MPMC_CAT(launch_batched_nm, MPMC_NM)(const Mixture* d_mix, int n, int64_t ncell, const double* p,
                                                   const double* t, const double* z, const DeviceOutputs& out,
                                                   void* scratch, size_t scratch_bytes, const BatchedShape& shape,
                                                   cudaStream_t stream) {
    using namespace batched;
    if (ncell <= 0) return cudaSuccess;
    if (ncell >= (int64_t{1} << 24)) return cudaErrorInvalidValue;  // work-item encodings hold 24-bit cells
    Workspace ws;
    const bool fp64_items = shape.fp64_items != 0;
    // the largest FP64 attempt-item capacity and exact sub-solve the scratch holds
    int per = kS64PerCell, ecap = fp64_items ? 0 : exact_capacity(ncell);
    while (ecap > 0 && carve(ws, nullptr, n, ncell, fp64_items, per, ecap) > scratch_bytes) ecap /= 2;
    while (per > 1 && carve(ws, nullptr, n, ncell, fp64_items, per, ecap) > scratch_bytes) per /= 2;
    if (carve(ws, nullptr, n, ncell, fp64_items, per, ecap) > scratch_bytes || scratch == nullptr)
        return cudaErrorInvalidValue;
    ExactRegion exact;
    carve(ws, static_cast<char*>(scratch), n, ncell, fp64_items, per, ecap, &exact);
    ws.io_stride = shape.io_stride > 0 ? shape.io_stride : ncell;
    ws.slow_projection = shape.slow_projection > 0.f ? shape.slow_projection : kSlowProjection;
    ws.continue_limit = shape.continue_limit > 0 ? shape.continue_limit : kContinueLimit;
    int device = 0, sms = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int cell_block = 64;
    // per-cell FP64 kernels and FP64 work items run best at low residency
    // (their per-thread local state then stays in L1/L2)
    const int64_t cell_grid_max = static_cast<int64_t>(sms) * (shape.cell_blocks_per_sm > 0 ? shape.cell_blocks_per_sm : 2);
    auto cell_grid = [&](int64_t items) {
        int64_t g = (items + cell_block - 1) / cell_block;
        return static_cast<unsigned>(g < cell_grid_max ? (g > 0 ? g : 1) : cell_grid_max);
    };
    const int qblock = 128;
    const int trial_res = shape.trial_blocks_per_sm > 0 ? shape.trial_blocks_per_sm
                                                        : resident_blocks(trials32_kernel<NM>, qblock);
    const int split_res = shape.split_blocks_per_sm > 0 ? shape.split_blocks_per_sm
                                                        : resident_blocks(split32_kernel<NM>, qblock);
    const int t64_res = shape.t64_blocks_per_sm > 0 ? shape.t64_blocks_per_sm : 2;
    // FP64 trial and attempt items: 32 / kSeg per warp (kSeg the component
    // capacity rounded to a power of two), or one per warp.  Measured on a
    // GB300: packed trial items gain at every size (N = 4: 1.88 s -> 0.85 s of
    // feed trials on 1M cells; N = 10 bench: 147 -> 138 ms); packed attempt
    // items gain where many short items share a warp (N = 4: 3.30 -> 2.26 s)
    // and lose where a few long ones set the stage's tail (N = 10: 176 -> 198 ms).
    const bool packed_trials = (shape.item_form & 32) == 0;
    const bool packed_attempts = (shape.item_form & 64) ? false : ((shape.item_form & 128) ? true : NM <= 8);
    const int s64_res = shape.s64_blocks_per_sm > 0 ? shape.s64_blocks_per_sm : 2;
    // one pass of the launch sequence over the cells `ws.pass` selects
    // The exact sub-solve: the marked cells gathered, solved by the FP64
    // work-queue form on their own workspace, written back.  On a side stream
    // it overlaps the main pass's stages after the polish.
    const bool side = shape.side_stream != nullptr && shape.side_fork != nullptr && shape.side_join != nullptr;
    auto launch_exact = [&]() -> cudaError_t {
        const int cap = ws.exact_capacity;
        if (cap <= 0) return cudaSuccess;
        cudaStream_t es = side ? shape.side_stream : stream;
        cudaError_t err;
        if (side) {
            if ((err = cudaEventRecord(shape.side_fork, stream)) != cudaSuccess) return err;
            if ((err = cudaStreamWaitEvent(es, shape.side_fork, 0)) != cudaSuccess) return err;
        }
        const unsigned g = static_cast<unsigned>(std::min<int64_t>((cap + 127) / 128, sms * 8));
        gather_exact_kernel<NM><<<g, 128, 0, es>>>(ws, p, t, z, n, cap, exact.p, exact.t, exact.z);
        BatchedShape sub = shape;
        sub.fp64_items = 1;
        sub.warm_lnk = nullptr;
        sub.io_stride = 0;
        sub.events = shape.exact_events;
        sub.redo_events = nullptr;
        sub.exact_events = nullptr;
        sub.side_stream = nullptr;
        err = MPMC_CAT(launch_batched_nm, MPMC_NM)(d_mix, n, cap, exact.p, exact.t, exact.z, exact.out, exact.scratch,
                                                   exact.scratch_bytes, sub, es);
        if (err != cudaSuccess) return err;
        scatter_exact_kernel<NM><<<g, 128, 0, es>>>(ws, n, cap, exact.out, out);
        if (side && (err = cudaEventRecord(shape.side_join, es)) != cudaSuccess) return err;
        return cudaGetLastError();
    };
    auto run_pass = [&](cudaEvent_t* events, bool f64, bool fork_exact) -> cudaError_t {
        // the warm pass's statistics stay for the cold pass after it
        const int clear = ws.pass >= kPassRedo ? qPassSlots : qSlots;
        cudaError_t e = cudaMemsetAsync(ws.counters, 0, sizeof(int) * clear, stream);
        if (e != cudaSuccess) return e;
        e = cudaMemsetAsync(ws.s64_items, 0xff, sizeof(int) * static_cast<size_t>(ws.s64_capacity), stream);
        if (e != cudaSuccess) return e;
        int stage = 0;
        auto mark = [&]() {
            if (events) cudaEventRecord(events[stage], stream);
            ++stage;
        };
        mark();
        setup_kernel<NM><<<cell_grid(ncell), 128, 0, stream>>>(d_mix, ws, p, t, z, out);
        mark();
        // The FP64 form queues every trial and attempt as an exact FP64 item (the
        // FP32 screening stages become empty), on the same stage slots.
        if (f64) rerun_all_kernel<NM><<<cell_grid(ncell), 128, 0, stream>>>(ws, 0);
        else trials32_kernel<NM><<<sms * trial_res, qblock, 0, stream>>>(d_mix, ws, p, t, 0);
        mark();
        classify_kernel<NM><<<cell_grid(ncell), 128, 0, stream>>>(d_mix, ws, 0);
        mark();
        // one warp per trial item: items of slow descents dominate, so latency
        // matters more than packing several items into a warp (measured)
        if ((shape.item_form & 1) && !f64) trials64_kernel<NM><<<sms * t64_res, 64, 0, stream>>>(d_mix, ws, p, t);
        else if (packed_trials) w64::trials64w_kernel<NM, w64::kSeg<NM>><<<sms * t64_res, 128, 0, stream>>>(d_mix, ws, p, t);
        else w64::trials64w_kernel<NM, 32><<<sms * t64_res, 128, 0, stream>>>(d_mix, ws, p, t);
        mark();
        decide_kernel<NM><<<cell_grid(ncell), cell_block, 0, stream>>>(d_mix, ws, p, t, out);
        mark();
        // FP32 successive substitution hands over to the FP64 Newton polish at
        // |r| <= ss_switch (default 2e-5, a few times the FP32 rounding floor)
        const float ss_switch = shape.ss_switch > 0.f ? shape.ss_switch : 2e-5f;
        if (!f64) split32_kernel<NM><<<sms * split_res, qblock, 0, stream>>>(d_mix, ws, p, t, ss_switch, 0);
        mark();
        // polish: one cell per thread up to 12 components (its per-cell arrays
        // still fit the cache), one cell per lane group above
        const bool lane_polish = (shape.item_form & 8) ? true : ((shape.item_form & 16) ? false : NM <= 12);
        if (lane_polish && shape.polish_stream)
            polish_stream_kernel<NM><<<cell_grid(ncell), cell_block, 0, stream>>>(d_mix, ws, p, t, out);
        else if (lane_polish) polish_kernel<NM><<<cell_grid(ncell), cell_block, 0, stream>>>(d_mix, ws, p, t, out);
        else w64::polishw_kernel<NM, w64::kSeg<NM>><<<sms * s64_res, 128, 0, stream>>>(d_mix, ws, p, t, out);
        mark();
        // every cell the exact sub-solve takes is marked by now (in this
        // pass's polish, or an earlier pass's)
        if (fork_exact && side) {
            const cudaError_t err = launch_exact();
            if (err != cudaSuccess) return err;
        }
        // attempts FP32 left open beside a polished pair: their FP32 prediction,
        // then the pair's review or the FP64 continuation of what stays open
        if (!f64) split32_kernel<NM><<<sms * split_res, qblock, 0, stream>>>(d_mix, ws, p, t, ss_switch, 1);
        mark();
        compete_kernel<NM><<<cell_grid(ncell), cell_block, 0, stream>>>(d_mix, ws, p, t);
        mark();
        if ((shape.item_form & 4) && !f64) split64_kernel<NM><<<sms * s64_res, 64, 0, stream>>>(d_mix, ws, p, t);
        else if (packed_attempts) w64::split64w_kernel<NM, w64::kSeg<NM>><<<sms * s64_res, 128, 0, stream>>>(d_mix, ws, p, t);
        else w64::split64w_kernel<NM, 32><<<sms * s64_res, 128, 0, stream>>>(d_mix, ws, p, t);
        mark();
        select64_kernel<NM><<<cell_grid(ncell), cell_block, 0, stream>>>(d_mix, ws, p, t, out);
        mark();
        relist_kernel<NM><<<1, 1024, 0, stream>>>(ws);
        cudaMemsetAsync(ws.counters + qT64Items, 0, 2 * sizeof(int), stream);
        mark();
        if (f64) rerun_all_kernel<NM><<<cell_grid(ncell), 128, 0, stream>>>(ws, 1);
        else trials32_kernel<NM><<<sms * trial_res, qblock, 0, stream>>>(d_mix, ws, p, t, 1);
        mark();
        classify_kernel<NM><<<cell_grid(ncell), 128, 0, stream>>>(d_mix, ws, 1);
        mark();
        if ((shape.item_form & 2) && !f64) trials64_kernel<NM><<<sms * t64_res, 64, 0, stream>>>(d_mix, ws, p, t);
        else if (packed_trials) w64::trials64w_kernel<NM, w64::kSeg<NM>><<<sms * t64_res, 128, 0, stream>>>(d_mix, ws, p, t);
        else w64::trials64w_kernel<NM, 32><<<sms * t64_res, 128, 0, stream>>>(d_mix, ws, p, t);
        mark();
        finish_kernel<NM><<<cell_grid(ncell), cell_block, 0, stream>>>(d_mix, ws, p, t, out);
        mark();
        fallback_kernel<NM><<<cell_grid(ncell), cell_block, 0, stream>>>(d_mix, ws, p, t, z, out);
        mark();
        return cudaGetLastError();
    };
    ws.warm_lnk = shape.warm_lnk;
    ws.pass = shape.warm_lnk ? kPassWarm : kPassCold;
    cudaError_t e = run_pass(shape.events, fp64_items, !shape.warm_lnk);
    if (e != cudaSuccess) return e;
    if (shape.warm_lnk) {
        // the warm cells whose pair was not accepted: the full cold solve (a
        // nearly empty pass when the warm starts are good)
        ws.pass = kPassRedo;
        e = run_pass(shape.redo_events, fp64_items, true);
        if (e != cudaSuccess) return e;
    }
    if (!fp64_items) {
        // the cells FP32 could not screen (mark_exact): without a side stream
        // the sub-solve runs here, after the main passes; with one, the main
        // stream waits for it (a nearly empty sub-solve on most batches)
        if (!side) e = launch_exact();
        else e = cudaStreamWaitEvent(stream, shape.side_join, 0);
        if (e != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

}  // namespace pr76
