// Batched mixed-precision PR76 flash: device workspace, work queues and the
// stage kernels.
//
// Execution model (one stream, no host synchronisation between stages, so
// the whole sequence can be captured in a CUDA graph):
//   setup       per cell   FP64 feed phase (reference phase of the TPD test),
//                          enqueue the cell's N+2 automatic TPD trials
//   trials32    per trial  persistent FP32 TPD descent; each loop iteration
//                          of every lane performs exactly one property
//                          evaluation, lanes whose trial ended refill from
//                          the queue, so warps stay full (work queue with
//                          implicit compaction)
//   decide      per cell   FP64 re-run of every trial FP32 could not decide;
//                          phase-set decision of the feed test; enqueue split
//                          attempts (witness order x {vapor, liquid}, <= 16)
//   split32     per attempt persistent FP32 ln K successive substitution
//   polish      per cell   minimum-Gibbs attempt, FP64 Newton polish of ln K
//                          (closed-form FP64 Jacobian, chord iterations),
//                          reference acceptance rules in FP64, enqueue the
//                          N+4 common-tangent review trials
//   open32      per attempt attempts FP32 left open near a pair beside a
//                          polished one: FP32 prediction of where they
//                          converge, pruning those that cannot change the
//                          minimum-Gibbs selection
//   compete     per cell   review the polished pair, or continue the attempts
//                          still open exactly in FP64 (split64) and select
//                          among them and the pair (select64)
//   trials32    per trial  review trials against the FP64 common tangent
//   finish      per cell   FP64 re-run of undecided review trials, final
//                          status, outputs
//   fallback    per cell   cells flagged by any stage rerun the plain FP64
//                          reference algorithm
// The reference decisions these stages reproduce are cited in pr76_fp64.cuh.
#pragma once

#include "pr76_ad.cuh"
#include "pr76_fp32.cuh"

namespace pr76 {
namespace batched {

constexpr int kMaxAttempts = 16;
// In the mixed form, counter rows 0-2 hold FP32 property evaluations of the
// feed trials, split attempts and review trials, and this row (the plain
// form's cubic-iteration row) holds every FP64 property evaluation.
constexpr int kFp64EvalRow = cRootIters;
// Flag added to an FP32 trial class when its descent converges too slowly for
// the reference's FP64 run to be sure of finishing within 512 iterations.
constexpr int kSlowFlag = 8;
// A descent whose projected FP64 iteration count (from its FP32 contraction)
// exceeds this is re-run exactly from its start.  Below it, an undecided
// trial continues in FP64 from its FP32 end point with the iterations left of
// the reference's 512; the projection overstates the count near the FP32
// rounding floor, so the margin to the limit is on the safe side.
#ifndef MPMC_SLOW_PROJECTION
#define MPMC_SLOW_PROJECTION 448.f
#endif
constexpr float kSlowProjection = MPMC_SLOW_PROJECTION;
// FP32 iterations from which an undecided trial or an unsettled attempt is run
// from its start in FP64 rather than continued from its FP32 end point.
constexpr int kContinueLimit = 512;

// Queue/counter slots in Workspace::counters.
enum Slot : int {
    qTrialCells = 0,   // cells listed for the current trial stage
    qTrialCursor = 1,  // next trial item to fetch
    qAttempts = 2,     // attempt items listed
    qAttemptCursor = 3,
    qFallback = 4,     // cells listed for the FP64 fallback
    qOpenItems = 5,    // open attempts listed for the FP32 prediction (open32)
    qOpenCursor = 6,
    qCompeteCells = 7, // cells whose polished pair awaits the open attempts' outcome
    // diagnostic statistics of the last batch
    sFeedContinued = 8,    // feed trials finished in FP64 from the FP32 end point
    sFeedRerun = 9,        // feed trials re-run exactly in FP64
    sReviewContinued = 10,
    sReviewRerun = 11,
    sFbNonsmooth = 12,     // fallback: nonsmooth feed reference
    sFbNoAttempt = 13,     // fallback: no FP32 attempt converged, some failed
    sFbPolish = 14,        // fallback: FP64 polish did not converge
    sFbRejected = 15,      // fallback: polished pair failed the acceptance rules
    sFbLoad = 16,          // fallback: cell constants unrepresentable
    sCandidates2 = 17,     // cells whose two best attempts were both polished
    qT64Items = 18,        // FP64 trial items listed
    qT64Cursor = 19,
    qS64Items = 20,        // FP64 attempt items listed
    qS64Cursor = 21,
    qSplitCells = 22,      // cells listed for the polish stage
    qS64Cells = 23,        // cells listed for the FP64 attempt selection
    sSlowSkipped = 24,     // slow trials whose outcome could not change the cell's status
    sLimitAttempts = 25,   // attempts classified as ending at the iteration limit
    qPolishCursor = 26,    // warp queue over the polish list
    qPassSlots = 27,       // slots above are cleared at the start of every pass
    sWarmCells = 27,       // cells run from their warm start (warm pass)
    sWarmRedo = 28,        // of those, cells whose pair was not accepted (cold pass)
    sWarmNoPair = 29,      // ... because no attempt converged to an accepted pair
    sWarmUnstable = 30,    // ... because the review found a negative TPD
    sCompeting = 31,       // cells whose polished pair waited on attempts FP32 left open
    sCompeteFp64 = 32,     // ... of those, cells with open attempts left for the FP64 continuation
    sReplayRisk = 33,      // cells whose polished attempt may stop short in the reference (replay_linear)
    // 64-bit totals (two slots each) of the FP64 work per stage, for the
    // algorithmic flop count of each stage: property evaluations ...
    tE64Setup = 34,        // ... of the feed phase (setup)
    tE64FeedTrials = 36,   // ... of the FP64 feed-test trial items
    tE64ReviewTrials = 38, // ... of the FP64 review trial items
    tE64Polish = 40,       // ... of the Newton polish (first state and chord steps)
    tE64Split64 = 42,      // ... of the FP64 attempt continuations
    sPolishJacobians = 44, // closed-form Jacobians built and factorised by the polish
    sPolishSolves = 45,    // LU solves of the polish's chord steps
    sExactCells = 46,      // cells marked for the exact sub-solve (every trial and attempt in FP64)
    qSlots = 48
};

// FP64 attempt items are (cell << 5) | flags | order, order < kMaxAttempts:
// kFromSeed runs the attempt from its FP64 seed with the whole 512-iteration
// budget, else it continues from its FP32 end point.
constexpr int kFromSeed = 16;
constexpr int kOrderMask = 15;

// Doubles per FP64 attempt result: gibbs, guard, fug, beta, z_l, z_v, 2 spare,
// then x, y, ln K, ln phi_L, ln phi_V, common log activity.
template <int NM>
__host__ __device__ constexpr int S64Stride() { return 8 + 6 * NM; }

// Cell phases kept in Workspace::phase.
enum Phase : int {
    pInvalid = -1, pSingle = 0, pTwo = 1, pUnstable = 2, pIndeterminate = 3,
    pPending = 10, pSplit = 11, pReview = 12, pFallback = 13, pSplit64 = 14,
    pRedo = 15,  // warm pass: the warm pair was not accepted, the cell runs the cold pass
    pCompete = 16,  // a polished pair waits on the open attempts' predicted ends
    pExact = 17     // FP32 could not screen the cell: the exact sub-solve solves it again in FP64
};

// Passes of the launch sequence: the cold solve of every cell; the warm pass
// (each cell with a usable ln K warm start runs one split attempt from it and
// the common-tangent review, no feed test, while the other cells take the
// cold path in the same pass); the cold solve of the warm cells whose pair was
// not accepted.
enum Pass : int { kPassCold = 0, kPassWarm = 1, kPassRedo = 2 };

// Device workspace for one batch (all arrays entry-major, cell fastest).
struct Workspace {
    int64_t ncell;
    int n;
    int* counters;          // [qSlots]
    int* phase;             // [ncell]
    int* trial_cells;       // [ncell] compacted cell list of the current trial stage
    int* attempt_items;     // [kMaxAttempts * ncell] (cell << 5 | order)
    double* z;              // [NM * ncell] normalised feed
    double* ref_lnphi;      // [NM * ncell] feed phase ln phi (FP64)
    double* ref_z;          // [ncell]
    float* tw;              // [(NM+4) * NM * ncell] trial end compositions
    signed char* tclass;    // [(NM+4) * ncell] trial classes
    short* titer;           // [(NM+4) * ncell] FP32 descent iterations of the trial
    float* att_lnk;         // [kMaxAttempts * NM * ncell]
    float* att_gibbs;       // [kMaxAttempts * ncell]
    signed char* att_class; // [kMaxAttempts * ncell]
    int* att_count;         // [ncell]
    double* cand;           // [7 * NM * ncell]: x, y, lnk, lnphi_l, lnphi_v, common, imposed
    double* cand_s;         // [8 * ncell]: beta, z_l, z_v, fug, gibbs_change, gibbs_guard, tpd_tol, pair guard;
                            // while FP64 continuations compete with a polished pair (phase pSplit64),
                            // slots 4 and 6 hold that pair's Gibbs energy (NaN: none) and attempt order
    int* counters_out;      // [cCount * ncell] work counters (FP32 evaluations are in row 1/0/2)
    float* c32;             // [4 * NM * ncell] FP32 cell constants: z, ln z, a_i(T), sqrt(a_i)
    float* ref32;           // [NM * ncell] feed-phase ln phi rounded to FP32
    int* t64_items;         // [(NM+4) * ncell] FP64 trial items (cell << 7 | k << 2 | mode)
    signed char* t64_status;// [(NM+4) * ncell] FP64 trial statuses (fp64::TrialStatus)
    double* tw64;           // [(NM+4) * NM * ncell] FP64 witnesses of negative feed trials
    int* s64_items;         // [s64_capacity] FP64 attempt items (cell << 5 | order)
    signed char* s64_status;// [s64_capacity]
    double* s64_state;      // [s64_capacity * S64Stride] converged attempt states
    short* att_iter;        // [kMaxAttempts * ncell] FP32 SS iterations of the attempt
    double* att_lnk64;      // [kMaxAttempts * NM * ncell] FP64 seeds of the attempts
    const double* warm_lnk; // [n * ncell] caller's ln K warm starts (NaN = cold), warm pass only
    signed char* warm_cell; // [ncell] 1 = the cell runs from its warm start in the warm pass
    int pass;               // Pass
    float* att_rate;        // [kMaxAttempts * ncell] FP32 SS contraction per iteration, ln(|r| ratio)
    int* split_cells;       // [ncell] cells that reached the split stage
    int* s64_cells;         // [ncell] cells whose attempts were continued in FP64
    int* s64_base;          // [ncell] first FP64 attempt item of the cell
    int* s64_count;         // [ncell]
    int s64_capacity;
    int fp64_items;         // FP64 work-queue form: every attempt item runs from its FP64 seed
    float slow_projection;  // projected FP64 iterations above which a trial is re-run exactly
    int continue_limit;     // FP32 iterations from which an undecided trial or unsettled attempt
                            // runs from its start in FP64 instead of from its FP32 end point
    int* exact_list;        // [exact_capacity] cells for the exact sub-solve, in marking order
    int exact_capacity;     // cells the exact sub-solve holds (beyond it: the plain fallback)
    int64_t io_stride;      // stride of the caller's z and output rows (the whole batch when this
                            // solve is one cell range of it; the pointers start at the range)
};

// A cell of the warm pass that runs from its warm start: a rejected pair sends
// it to the cold pass instead of settling its status.
__device__ __forceinline__ bool warm_cell(const Workspace& ws, int64_t c) {
    return ws.pass == kPassWarm && ws.warm_cell[c] != 0;
}

__device__ __forceinline__ int64_t idx(int k, int64_t ncell, int64_t c) { return static_cast<int64_t>(k) * ncell + c; }

// Adds each calling lane's `v` to the 64-bit total at counter slot `slot`,
// one atomic per warp (the lanes of the warp that call it together).
__device__ __forceinline__ void add_total(const Workspace& ws, int slot, int v) {
    const unsigned mask = __activemask();
    const unsigned sum = __reduce_add_sync(mask, static_cast<unsigned>(v));
    if ((threadIdx.x & 31) == __ffs(mask) - 1)
        atomicAdd(reinterpret_cast<unsigned long long*>(ws.counters + slot), static_cast<unsigned long long>(sum));
}
// 32-bit variant for counts
__device__ __forceinline__ void add_count(const Workspace& ws, int slot, int v) {
    const unsigned mask = __activemask();
    const unsigned sum = __reduce_add_sync(mask, static_cast<unsigned>(v));
    if ((threadIdx.x & 31) == __ffs(mask) - 1) atomicAdd(ws.counters + slot, static_cast<int>(sum));
}

// Number of automatic TPD starts for `active` components (pt_stability.hpp:254).
__device__ __forceinline__ int auto_starts(int active) { return active == 1 ? 1 : active + 2; }

// ---------------------------------------------------------------------------
// Loading a cell's FP32 and FP64 context.
template <int NM>
__device__ bool load_cell32(const Mixture& m, const Workspace& ws, int64_t c, const double* p, const double* t,
                            fp32::Cell<NM>& cf, int& active) {
    cf.n = m.n;
    cf.p = static_cast<float>(p[c]);
    cf.t = static_cast<float>(t[c]);
    cf.evals = 0;
    active = 0;
    for (int i = 0; i < cf.n; ++i) {
        cf.z[i] = ws.c32[idx(0 * NM + i, ws.ncell, c)];
        cf.lz[i] = ws.c32[idx(1 * NM + i, ws.ncell, c)];
        cf.a[i] = ws.c32[idx(2 * NM + i, ws.ncell, c)];
        cf.root[i] = ws.c32[idx(3 * NM + i, ws.ncell, c)];
        cf.b[i] = m.b32[i];
        active += cf.z[i] > 0.f;
    }
    return cf.a[0] > 0.f;
}

template <int NM>
__device__ bool load_cell64(const Mixture& m, const Workspace& ws, int64_t c, const double* p, const double* t,
                            fp64::Cell<NM>& c64) {
    c64.n = m.n;
    c64.newton = true;
    c64.p = p[c];
    c64.t = t[c];
    for (int k = 0; k < cCount; ++k) c64.counters[k] = 0;
    for (int i = 0; i < c64.n; ++i) {
        c64.z[i] = ws.z[idx(i, ws.ncell, c)];
        c64.lz[i] = c64.z[i] > 0.0 ? log(c64.z[i]) : 0.0;
    }
    return fp64::temp_setup(m, c64);
}

// ---------------------------------------------------------------------------
// Stage 1: per-cell setup and the FP64 feed phase.
template <int NM>
__global__ void __launch_bounds__(128) setup_kernel(const Mixture* __restrict__ mix_g, Workspace ws,
                                                    const double* __restrict__ p, const double* __restrict__ t,
                                                    const double* __restrict__ z, DeviceOutputs out) {
    __shared__ Mixture m;
    stage_mixture(mix_g, m);
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t c = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; c < ws.ncell; c += stride) {
        if (ws.pass == kPassRedo && ws.phase[c] != pRedo) continue;  // settled by the warm pass
        fp64::Cell<NM> cell;
        cell.n = m.n;
        cell.newton = true;
        cell.p = p[c];
        cell.t = t[c];
        for (int k = 0; k < cCount; ++k) cell.counters[k] = 0;
        double feed[NM];
        for (int i = 0; i < cell.n; ++i) feed[i] = z[idx(i, ws.io_stride, c)];
        int ph = pPending;
        if (!isfinite(cell.p) || cell.p <= 0.0 || !isfinite(cell.t) || cell.t <= 0.0 ||
            !fp64::normalise_feed(cell, feed) || !fp64::temp_setup(m, cell)) {
            ph = pInvalid;
        } else {
            for (int i = 0; i < cell.n; ++i)
                if (feed[i] > 0.0 && cell.z[i] == 0.0) ph = pIndeterminate;
        }
        for (int i = 0; i < cell.n; ++i) ws.z[idx(i, ws.ncell, c)] = ph == pInvalid ? 0.0 : cell.z[i];
        bool warm = false;
        if (ph == pPending && ws.pass == kPassWarm) {
            // a usable warm start: finite on every component present, not all zero
            warm = true;
            double contrast = 0.0;
            for (int i = 0; i < cell.n; ++i) {
                if (cell.z[i] == 0.0) continue;
                const double v = ws.warm_lnk[idx(i, ws.io_stride, c)];
                warm = warm && isfinite(v) && fabs(v) < 700.0;
                contrast = fmax(contrast, fabs(v));
            }
            warm = warm && contrast > 0.0;  // else: the cold path in this pass
        }
        if (ws.pass < kPassRedo) ws.warm_cell[c] = warm ? 1 : 0;
        if (warm) atomicAdd(&ws.counters[sWarmCells], 1);
        if (ph == pPending) {
            double lp[NM], zref = 0.0;
            bool smooth;
            const int is = fp64::stability_provider(m, cell, cell.z, lp, smooth, &zref, cInitEvals);
            if (is != kOk) {
                ph = is == kDomain ? pInvalid : pIndeterminate;
            } else {
                for (int i = 0; i < cell.n; ++i) {
                    ws.ref_lnphi[idx(i, ws.ncell, c)] = lp[i];
                    ws.ref32[idx(i, ws.ncell, c)] = static_cast<float>(lp[i]);
                    ws.c32[idx(0 * NM + i, ws.ncell, c)] = static_cast<float>(cell.z[i]);
                    ws.c32[idx(1 * NM + i, ws.ncell, c)] = static_cast<float>(cell.lz[i]);
                    ws.c32[idx(2 * NM + i, ws.ncell, c)] = static_cast<float>(cell.a[i]);
                    ws.c32[idx(3 * NM + i, ws.ncell, c)] = static_cast<float>(cell.root[i]);
                }
                ws.ref_z[c] = zref;
                // a nonsmooth feed reference makes every trial ambiguous: reference rules in FP64
                if (!smooth) {
                    ph = pFallback;
                    atomicAdd(&ws.counters[sFbNonsmooth], 1);
                }
            }
        }
        ws.att_count[c] = 0;
        if (ph == pPending && warm) {
            // One split attempt from the caller's ln K, entered as attempt 0.
            // A guess near the phase boundary (beta near 0 or 1) whose
            // Rachford-Rice function has no root in (0, 1) (rachford_rice.hpp:
            // 86-92: ln sum z K > 0 and ln sum z / K > 0) is moved by the
            // smallest common shift of ln K that puts the root inside again.
            double ls[2];
            for (int k = 0; k < 2; ++k) {
                const double sign = k == 0 ? 1.0 : -1.0;
                double largest = -INFINITY, sum = 0.0;
                for (int i = 0; i < cell.n; ++i)
                    if (cell.z[i] > 0.0) largest = fmax(largest, cell.lz[i] + sign * ws.warm_lnk[idx(i, ws.io_stride, c)]);
                for (int i = 0; i < cell.n; ++i)
                    if (cell.z[i] > 0.0) sum += exp(cell.lz[i] + sign * ws.warm_lnk[idx(i, ws.io_stride, c)] - largest);
                ls[k] = largest + log(sum);
            }
            double shift = 0.0;
            const double room = ls[0] + ls[1];  // >= 0 (Cauchy-Schwarz), 0 only for equal K
            if (isfinite(room) && room > 1e-9) {
                const double margin = fmin(1e-2, 0.25 * room);
                if (ls[0] < margin) shift = margin - ls[0];
                else if (ls[1] < margin) shift = ls[1] - margin;
            }
            for (int i = 0; i < cell.n; ++i) {
                const double v = cell.z[i] > 0.0 ? ws.warm_lnk[idx(i, ws.io_stride, c)] + shift : 0.0;
                ws.att_lnk[idx(i, ws.ncell, c)] = static_cast<float>(v);
                if (ws.att_lnk64) ws.att_lnk64[idx(i, ws.ncell, c)] = v;
            }
            ws.att_class[idx(0, ws.ncell, c)] = fp32::aFailed;  // overwritten by split32
            ws.att_iter[idx(0, ws.ncell, c)] = 0;
            ws.att_count[c] = 1;
            ws.attempt_items[atomicAdd(&ws.counters[qAttempts], 1)] = static_cast<int>(c) << 5;
            ws.split_cells[atomicAdd(&ws.counters[qSplitCells], 1)] = static_cast<int>(c);
            ph = pSplit;
        }
        ws.phase[c] = ph;
        add_total(ws, tE64Setup, cell.counters[cInitEvals]);
        if (ws.pass < kPassRedo) {
            for (int k = 0; k < cCount; ++k) ws.counters_out[idx(k, ws.ncell, c)] = 0;
            ws.counters_out[idx(kFp64EvalRow, ws.ncell, c)] = cell.counters[cInitEvals];
            if (ph == pSplit) ws.counters_out[idx(cAttempts, ws.ncell, c)] = 1;
        } else {
            // the earlier pass's work stays counted
            ws.counters_out[idx(kFp64EvalRow, ws.ncell, c)] += cell.counters[cInitEvals];
        }
        if (ph == pInvalid || ph == pIndeterminate) {
            const double nan = __longlong_as_double(0x7ff8000000000000LL);
            if (out.status) out.status[c] = ph == pInvalid ? static_cast<int>(kInvalid) : static_cast<int>(kIndeterminate);
            if (out.beta) out.beta[c] = nan;
            for (int i = 0; i < cell.n; ++i) {
                const int64_t k = idx(i, ws.io_stride, c);
                if (out.x) out.x[k] = nan;
                if (out.y) out.y[k] = nan;
                if (out.lnk) out.lnk[k] = nan;
                if (out.lnphi_l) out.lnphi_l[k] = nan;
                if (out.lnphi_v) out.lnphi_v[k] = nan;
            }
            if (out.z_l) out.z_l[c] = nan;
            if (out.z_v) out.z_v[c] = nan;
            if (out.counters)
                for (int k = 0; k < cCount; ++k) out.counters[idx(k, ws.io_stride, c)] = cell.counters[k];
        }
        if (ph == pPending) {
            const int slot = atomicAdd(&ws.counters[qTrialCells], 1);
            ws.trial_cells[slot] = static_cast<int>(c);
        } else if (ph == pFallback) {
            atomicAdd(&ws.counters[qFallback], 1);
        }
    }
}

// ---------------------------------------------------------------------------
// Stage 2/6: FP32 TPD trials as a flat per-lane state machine.
//
// review == false: feed test, reference = feed phase, starts = automatic.
// review == true:  common-tangent test, reference = imposed ln(x phi) of the
//                  polished pair, starts = automatic + x + y.
template <int NM>
struct TrialLane {
    fp32::Cell<NM> cell;
    fp32::TpdPoint<NM> point, next;
    float dir[NM], lnphi[NM], ref[NM], lrefs[2 * NM];
    int nrefs;
    int64_t item;
    int c, k, iter, bt, stage;  // stage: 0 = evaluate start, 1 = line search, 2 = finished
    float alpha, slope, scale;
    int result;
    // convergence-rate checkpoints: stationarity at the last two multiples of 8 iterations
    float ck_stat, ck_prev_stat, stat0;
    int ck_iter, ck_prev_iter;
};

template <int NM>
__device__ void trial_begin(const Mixture& m, const Workspace& ws, const double* p, const double* t, bool review,
                            int ntrial, TrialLane<NM>& L) {
    const int64_t c = ws.trial_cells[L.item / ntrial];
    const int k = static_cast<int>(L.item % ntrial);
    L.c = static_cast<int>(c);
    L.k = k;
    L.iter = 0;
    L.bt = 0;
    L.stage = 0;
    L.result = fp32::tRerun;
    L.ck_stat = L.ck_prev_stat = INFINITY;
    L.ck_iter = L.ck_prev_iter = 0;
    int active;
    if (!load_cell32(m, ws, c, p, t, L.cell, active)) {
        L.stage = 2;
        return;
    }
    const int n = L.cell.n;
    const int n_auto = auto_starts(active);
    if (k >= n_auto + (review ? 2 : 0)) {  // not a start of this cell (fewer active components)
        L.result = fp32::tTangent;  // neutral: an unused slot
        L.stage = 3;
        return;
    }
    if (!review) {
        for (int i = 0; i < n; ++i) L.ref[i] = ws.ref32[idx(i, ws.ncell, c)];
        L.nrefs = 1;
        for (int i = 0; i < n; ++i) L.lrefs[i] = L.cell.lz[i];
    } else {
        // imposed reference ln phi_eq = common - ln z (pt_stability.hpp:319-322), stored in FP64
        for (int i = 0; i < n; ++i) L.ref[i] = static_cast<float>(ws.cand[idx(6 * NM + i, ws.ncell, c)]);
        L.nrefs = 2;
        for (int i = 0; i < n; ++i) {
            const double x = ws.cand[idx(0 * NM + i, ws.ncell, c)], y = ws.cand[idx(1 * NM + i, ws.ncell, c)];
            L.lrefs[i] = x > 0.0 ? static_cast<float>(log(x)) : 0.f;
            L.lrefs[NM + i] = y > 0.0 ? static_cast<float>(log(y)) : 0.f;
        }
    }
    // start composition (pt_stability.hpp:294-311)
    float* w = L.next.w;
    if (k >= n_auto) {
        const int which = k - n_auto;
        for (int i = 0; i < n; ++i) w[i] = static_cast<float>(ws.cand[idx(which * NM + i, ws.ncell, c)]);
    } else if (k == 0) {
        for (int i = 0; i < n; ++i) w[i] = L.cell.z[i];
    } else if (k == 1) {
        for (int i = 0; i < n; ++i) w[i] = L.cell.z[i] > 0.f ? 1.f / static_cast<float>(active) : 0.f;
    } else {
        int target = k - 2, pick = 0;
        for (int i = 0; i < n; ++i)
            if (L.cell.z[i] > 0.f) {
                if (target == 0) {
                    pick = i;
                    break;
                }
                --target;
            }
        for (int i = 0; i < n; ++i) w[i] = 0.1f * L.cell.z[i];
        w[pick] += 0.9f;
    }
    float s = 0.f;
    for (int i = 0; i < n; ++i) s += w[i];
    for (int i = 0; i < n; ++i) w[i] /= s;
}

template <int NM>
__device__ __forceinline__ bool trial_prepare_candidate(TrialLane<NM>& L) {
    const int n = L.cell.n;
    float largest = -INFINITY;
    for (int i = 0; i < n; ++i)
        if (L.cell.z[i] > 0.f) {
            L.next.w[i] = fmaf(L.alpha, L.dir[i], L.point.lw[i]);
            largest = fmaxf(largest, L.next.w[i]);
        }
    float sum = 0.f;
    for (int i = 0; i < n; ++i) {
        L.next.w[i] = L.cell.z[i] > 0.f ? expf(L.next.w[i] - largest) : 0.f;
        sum += L.next.w[i];
    }
    const float inv = 1.f / sum;
    bool positive = isfinite(inv);
    for (int i = 0; i < n; ++i) {
        L.next.w[i] *= inv;
        positive = positive && (L.cell.z[i] == 0.f || L.next.w[i] > 0.f);
    }
    return positive;
}

// Decide at the current point or set up the next line search.
template <int NM>
__device__ void trial_step_or_finish(TrialLane<NM>& L) {
    const fp32::ScreenOptions so = fp32::screen_options();
    const int n = L.cell.n;
    const float margin = so.decide * L.point.mag;
    if (L.point.value < -margin) {
        L.result = fp32::tNegative;
        L.stage = 2;
        return;
    }
    if (L.point.stat <= so.stat_tol || L.iter >= 400) {
        L.stage = 2;
        L.result = -1;  // classify below
        return;
    }
    L.scale = fmaxf(1.f, L.point.stat / 4.f);
    float slope = 0.f;
    for (int i = 0; i < n; ++i) {
        L.dir[i] = 0.f;
        if (L.cell.z[i] == 0.f) continue;
        L.dir[i] = -L.point.res[i] / L.scale;
        slope = fmaf(L.point.w[i] * L.point.res[i], L.dir[i], slope);
    }
    if (!(slope < 0.f)) {
        L.stage = 2;
        L.result = -1;
        return;
    }
    L.slope = slope;
    L.alpha = 1.f;
    L.bt = 0;
    L.stage = 1;
}

// Iterations the reference's FP64 descent would still need to reach its
// stationarity tolerance 1e-8 (pt_stability.hpp:384), extrapolated from the
// linear contraction rate over the last checkpoint window.
template <int NM>
__device__ float projected_fp64_iterations(const TrialLane<NM>& L) {
    if (!(L.point.stat > 1e-8f)) return static_cast<float>(L.iter);
    // contraction per iteration over the last checkpoint window, or over the
    // whole descent when it was shorter than a window
    float from = L.ck_prev_stat;
    int span = L.iter - L.ck_prev_iter;
    if (span < 4 || !(from < INFINITY)) {
        from = L.stat0;
        span = L.iter;
    }
    if (span < 1) return static_cast<float>(L.iter);
    if (!(from > L.point.stat)) return 1e9f;  // no progress at all: let FP64 decide from the start
    const float rate = logf(from / L.point.stat) / static_cast<float>(span);
    return static_cast<float>(L.iter) + logf(L.point.stat / 1e-8f) / rate;
}

template <int NM>
__device__ int trial_classify(const TrialLane<NM>& L, float slow_projection) {
    const fp32::ScreenOptions so = fp32::screen_options();
    const int n = L.cell.n;
    const float margin = so.decide * L.point.mag;
    if (L.point.value < -margin) return fp32::tNegative;
    // a descent that would exhaust the reference's 512-iteration budget ends
    // "iteration_limit" there; the classify stage re-runs it exactly in FP64
    // whenever its outcome can matter
    // (the projection is only a screen: near the FP32 noise floor the measured
    // contraction understates the FP64 rate, so no trial is declared
    // "iteration_limit" from it without the FP64 run)
    const int slow = (L.iter >= 400 || projected_fp64_iterations(L) > slow_projection) ? kSlowFlag : 0;
    if (L.point.stat > 10.f * so.stat_tol) return fp32::tMarginal | slow;
    for (int r = 0; r < L.nrefs; ++r) {
        float dist = 0.f;
        for (int i = 0; i < n; ++i)
            if (L.cell.z[i] > 0.f) dist = fmaxf(dist, fabsf(L.point.lw[i] - L.lrefs[r * NM + i]));
        if (dist <= so.near_ref) return fp32::tTangent | slow;
    }
    if (L.point.value > margin) return fp32::tPositive | slow;
    return fp32::tMarginal | slow;
}

template <int NM>
__global__ void __launch_bounds__(128) trials32_kernel(const Mixture* __restrict__ mix_g, Workspace ws,
                                                       const double* __restrict__ p, const double* __restrict__ t,
                                                       int review) {
    __shared__ Mixture m;
    stage_mixture(mix_g, m);
    const int ntrial = m.n + 4;  // slots per cell (auto starts <= n + 2, review adds 2)
    const int64_t total = static_cast<int64_t>(ws.counters[qTrialCells]) * ntrial;
    TrialLane<NM> L;
    L.stage = 3;  // idle: fetch first
    L.item = -1;
    bool live = true;
    for (;;) {
        if (live && L.stage >= 2) {
            if (L.item >= 0 && L.stage == 2) {
                const int cls = L.result >= 0 ? L.result : trial_classify(L, ws.slow_projection);
                const int64_t c = L.c;
                ws.tclass[idx(L.k, ws.ncell, c)] = static_cast<signed char>(cls);
                ws.titer[idx(L.k, ws.ncell, c)] = static_cast<short>(L.iter);
                for (int i = 0; i < L.cell.n; ++i) ws.tw[idx(L.k * NM + i, ws.ncell, c)] = L.point.w[i];
                atomicAdd(&ws.counters_out[idx(review ? cFinalEvals : cInitEvals, ws.ncell, c)], L.cell.evals);
                atomicAdd(&ws.counters_out[idx(cTrialIters, ws.ncell, c)], L.iter);
            } else if (L.item >= 0 && L.stage == 3) {
                ws.tclass[idx(L.k, ws.ncell, L.c)] = static_cast<signed char>(-1);  // unused slot
            }
            L.item = atomicAdd(&ws.counters[qTrialCursor], 1);
            if (L.item >= total) {
                live = false;
            } else {
                trial_begin(m, ws, p, t, review != 0, ntrial, L);
            }
        }
        if (__all_sync(0xffffffffu, !live)) break;
        if (!live || L.stage >= 2) continue;
        // one property evaluation per lane per loop iteration
        bool ok = true;
        if (L.stage == 1) ok = trial_prepare_candidate(L);
        bool tie = false;
        if (ok) ok = fp32::stability_provider(m, L.cell, L.next.w, L.lnphi, tie) && !tie &&
                     fp32::tpd(L.cell, L.lnphi, L.ref, L.next);
        if (L.stage == 0) {
            if (!ok) {
                L.result = fp32::tRerun;
                L.stage = 2;
                for (int i = 0; i < L.cell.n; ++i) L.point.w[i] = L.next.w[i];
                continue;
            }
            L.point = L.next;
            L.stat0 = L.point.stat;
            trial_step_or_finish(L);
            continue;
        }
        // line search
        bool accept = false;
        if (ok) {
            const float predicted = -L.alpha * L.slope;
            const float guard = 64.f * fp32::kEpsF * (L.point.mag + L.next.mag);
            if (predicted <= guard)
                accept = L.next.value <= L.point.value + guard && L.next.stat < L.point.stat;
            else
                accept = L.next.value <= L.point.value - 1e-4f * predicted;
            if (L.next.value < -fp32::screen_options().decide * L.next.mag) accept = true;
        }
        if (accept) {
            L.point = L.next;
            ++L.iter;
            if ((L.iter & 7) == 0) {
                L.ck_prev_stat = L.ck_stat;
                L.ck_prev_iter = L.ck_iter;
                L.ck_stat = L.point.stat;
                L.ck_iter = L.iter;
            }
            trial_step_or_finish(L);
        } else if (++L.bt >= 24) {
            L.stage = 2;
            L.result = -1;
        } else {
            L.alpha *= 0.5f;
        }
    }
}


// ---------------------------------------------------------------------------
// Output helpers (layout of include/mpmc_gb300_flash.h).
template <int NM>
__device__ void write_single(const DeviceOutputs& out, const Workspace& ws, int64_t c) {
    const int n = ws.n;
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    if (out.status) out.status[c] = kSinglePhase;
    if (out.beta) out.beta[c] = nan;
    for (int i = 0; i < n; ++i) {
        const int64_t k = idx(i, ws.ncell, c), o = idx(i, ws.io_stride, c);
        if (out.x) out.x[o] = ws.z[k];
        if (out.y) out.y[o] = nan;
        if (out.lnk) out.lnk[o] = nan;
        if (out.lnphi_l) out.lnphi_l[o] = ws.ref_lnphi[k];
        if (out.lnphi_v) out.lnphi_v[o] = nan;
    }
    if (out.z_l) out.z_l[c] = ws.ref_z[c];
    if (out.z_v) out.z_v[c] = nan;
}

template <int NM>
__device__ void write_status_only(const DeviceOutputs& out, const Workspace& ws, int64_t c, int status,
                                  bool with_pair) {
    const int n = ws.n;
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    if (out.status) out.status[c] = status;
    if (out.beta) out.beta[c] = with_pair ? ws.cand_s[idx(0, ws.ncell, c)] : nan;
    for (int i = 0; i < n; ++i) {
        const int64_t k = idx(i, ws.io_stride, c);
        if (out.x) out.x[k] = with_pair ? ws.cand[idx(0 * NM + i, ws.ncell, c)] : nan;
        if (out.y) out.y[k] = with_pair ? ws.cand[idx(1 * NM + i, ws.ncell, c)] : nan;
        if (out.lnk) out.lnk[k] = with_pair ? ws.cand[idx(2 * NM + i, ws.ncell, c)] : nan;
        if (out.lnphi_l) out.lnphi_l[k] = with_pair ? ws.cand[idx(3 * NM + i, ws.ncell, c)] : nan;
        if (out.lnphi_v) out.lnphi_v[k] = with_pair ? ws.cand[idx(4 * NM + i, ws.ncell, c)] : nan;
    }
    if (out.z_l) out.z_l[c] = with_pair ? ws.cand_s[idx(1, ws.ncell, c)] : nan;
    if (out.z_v) out.z_v[c] = with_pair ? ws.cand_s[idx(2, ws.ncell, c)] : nan;
}

template <int NM>
__device__ void write_counters(const DeviceOutputs& out, const Workspace& ws, int64_t c) {
    if (!out.counters) return;
    for (int k = 0; k < cCount; ++k) out.counters[idx(k, ws.io_stride, c)] = ws.counters_out[idx(k, ws.ncell, c)];
}

// ---------------------------------------------------------------------------
// Batched FP64 form: instead of FP32 screening, every trial of the listed
// cells is queued as an exact FP64 run from its start.
template <int NM>
__global__ void __launch_bounds__(128) rerun_all_kernel(Workspace ws, int review) {
    const int cells = ws.counters[qTrialCells];
    for (int slot = blockIdx.x * blockDim.x + threadIdx.x; slot < cells; slot += gridDim.x * blockDim.x) {
        const int64_t c = ws.trial_cells[slot];
        int active = 0;
        for (int i = 0; i < ws.n; ++i) active += ws.z[idx(i, ws.ncell, c)] > 0.0;
        const int ntr = auto_starts(active) + (review ? 2 : 0);
        for (int k = 0; k < NM + 4; ++k) {
            ws.tclass[idx(k, ws.ncell, c)] = static_cast<signed char>(k < ntr ? fp32::tRerun : -1);
            ws.titer[idx(k, ws.ncell, c)] = 0;
        }
    }
}

// ---------------------------------------------------------------------------
// Stage 3: feed-test decision per cell and split-attempt enumeration.
template <int NM>
struct DecideScratch {
    fp64::TpdPoint<NM> pt, nx;
    double dir[NM], lp[NM], ref[NM], w[NM], other[NM], lk[NM];
};

template <int NM>
__global__ void __launch_bounds__(64) decide_kernel(const Mixture* __restrict__ mix_g, Workspace ws,
                                                    const double* __restrict__ p, const double* __restrict__ t,
                                                    DeviceOutputs out) {
    __shared__ Mixture m;
    stage_mixture(mix_g, m);
    const int cells = ws.counters[qTrialCells];
    const int n = m.n;
    for (int slot = blockIdx.x * blockDim.x + threadIdx.x; slot < cells; slot += gridDim.x * blockDim.x) {
        const int64_t c = ws.trial_cells[slot];
        fp64::Cell<NM> cell;
        DecideScratch<NM> s;
        if (!load_cell64(m, ws, c, p, t, cell)) {
            ws.phase[c] = pFallback;
            atomicAdd(&ws.counters[qFallback], 1);
            continue;
        }
        int active = 0;
        for (int i = 0; i < n; ++i) active += cell.z[i] > 0.0;
        const int n_auto = auto_starts(active);
        for (int i = 0; i < n; ++i) s.ref[i] = ws.ref_lnphi[idx(i, ws.ncell, c)];
        bool negative = false, all_stationary = true;
        int nattempt = 0;
        for (int k = 0; k < n_auto; ++k) {
            int cls = ws.tclass[idx(k, ws.ncell, c)];
            bool witness = false;
            if (cls == fp32::tMarginal || cls == fp32::tRerun) {
                // decided in FP64 by the trials64 stage
                const int ts = ws.t64_status[idx(k, ws.ncell, c)];
                if (ts == fp64::kNegativeTpd) {
                    witness = true;
                    for (int i = 0; i < n; ++i) s.w[i] = ws.tw64[idx(k * NM + i, ws.ncell, c)];
                } else if (ts != fp64::kStationary) {
                    all_stationary = false;
                }
            } else if (cls == fp32::tNegative) {
                witness = true;
                double sum = 0.0, cs = 0.0;
                for (int i = 0; i < n; ++i) {
                    s.w[i] = ws.tw[idx(k * NM + i, ws.ncell, c)];
                    kahan_add(s.w[i], sum, cs);
                }
                for (int i = 0; i < n; ++i) s.w[i] /= sum;
            }
            if (!witness) continue;
            negative = true;
            for (int role = 0; role < 2 && nattempt < kMaxAttempts; ++role) {
                // split_seed (pt_split.hpp:245-267) in FP64
                const bool ok = fp64::split_seed(cell, s.w, role == 0, s.other, s.lk);
                const int order = nattempt++;
                if (ok) {
                    for (int i = 0; i < n; ++i) ws.att_lnk[idx(order * NM + i, ws.ncell, c)] = static_cast<float>(s.lk[i]);
                    const int item = atomicAdd(&ws.counters[qAttempts], 1);
                    ws.attempt_items[item] = (static_cast<int>(c) << 5) | order;
                    ws.att_class[idx(order, ws.ncell, c)] = fp32::aFailed;  // overwritten by split32
                    // the exact seed: every attempt of the FP64 form runs from it, and in
                    // the mixed form the reference's own run of the attempt when needed
                    for (int i = 0; i < n; ++i) ws.att_lnk64[idx(order * NM + i, ws.ncell, c)] = s.lk[i];
                    if (ws.fp64_items) ws.att_iter[idx(order, ws.ncell, c)] = 0;
                } else {
                    ws.att_class[idx(order, ws.ncell, c)] = fp32::aTrivial;  // unrepresentable seed: not a candidate
                }
            }
        }
        ws.att_count[c] = nattempt;
        atomicAdd(&ws.counters_out[idx(kFp64EvalRow, ws.ncell, c)], cell.counters[cInitEvals]);
        if (negative) {
            ws.phase[c] = pSplit;
            ws.split_cells[atomicAdd(&ws.counters[qSplitCells], 1)] = static_cast<int>(c);
            atomicAdd(&ws.counters_out[idx(cAttempts, ws.ncell, c)], nattempt);
        } else if (all_stationary) {
            ws.phase[c] = pSingle;
            write_single<NM>(out, ws, c);
            write_counters<NM>(out, ws, c);
        } else {
            ws.phase[c] = pIndeterminate;
            write_status_only<NM>(out, ws, c, kIndeterminate, false);
            write_counters<NM>(out, ws, c);
        }
    }
}

// ---------------------------------------------------------------------------
// Stage 4: FP32 split attempts as a per-lane state machine.
template <int NM>
struct SplitLane {
    fp32::Cell<NM> cell;
    fp32::SplitState<NM> point, next;
    float lk[NM];
    int item, c, order, iter, bt, stage;  // stage 0 = evaluate seed, 1 = line search, 2 = finished
    float alpha, slope, scale;
    float fug0, ck_fug, rate;  // |r| at the seed, at the last checkpoint; contraction per iteration
    int ck_iter;
    int limit;  // iteration count at which the lane stops: the reference's 512, or the prediction's cap
};
// Iterations the open-attempt prediction runs beyond an attempt's FP32 end
// point: attempts near a pair converge within a few dozen (host runs of the
// bench distributions at 4-20 components); one that has not converged by then
// stays open for the FP64 continuation.
constexpr int kPredictionIterations = 96;
// Iteration count (FP32 iterations plus the replayed remainder) above which a
// polished attempt is sent to the exact FP64 continuation instead: the
// reference stops at 512, and the FP32 count and the replay are estimates.
constexpr int kReplayLimit = 480;

template <int NM>
__device__ void split_step_or_finish(SplitLane<NM>& L, float ss_switch) {
    const int n = L.cell.n;
    // contraction rate of the iteration over 16-iteration windows, measured
    // only while |r| is well above the FP32 rounding floor
    if (L.iter - L.ck_iter >= 16 && L.point.fug > 10.f * ss_switch) {
        if (L.ck_fug > L.point.fug) L.rate = logf(L.ck_fug / L.point.fug) / static_cast<float>(L.iter - L.ck_iter);
        L.ck_fug = L.point.fug;
        L.ck_iter = L.iter;
    }
    if (L.point.fug <= ss_switch || L.iter >= L.limit) {
        L.stage = 2;
        return;
    }
    L.scale = fmaxf(1.f, L.point.fug / 2.f);
    float h = 0.f, first = 0.f, second = 0.f;
    for (int i = 0; i < n; ++i) {
        if (L.cell.z[i] == 0.f) continue;
        const float cc = (L.point.x[i] / L.cell.z[i]) * L.point.y[i];
        const float d = L.point.y[i] - L.point.x[i];
        h += d * (d / L.cell.z[i]);
        first += cc * L.point.res[i];
        second += (cc * L.point.res[i]) * L.point.res[i];
    }
    const float slope = -(L.point.beta * (1.f - L.point.beta) * second + (first / h) * first) / L.scale;
    if (!(slope < 0.f) || !isfinite(slope)) {
        L.stage = 2;
        return;
    }
    L.slope = slope;
    L.alpha = 1.f;
    L.bt = 0;
    L.stage = 1;
}

// Prune decision of an open attempt at its predicted end (open pass of
// split32_kernel): true when the attempt cannot change the cell's selection,
// the first attempt of least Gibbs energy among those that converge
// (pt_split.hpp:459-486) -- its predicted pair is trivial (the reference's
// attempt would end indistinguishable, pt_split.hpp:351-362), is the polished
// pair of the cell, or has a Gibbs energy clearly above the polished pair's.
template <int NM>
__device__ bool prune_open(const Workspace& ws, const SplitLane<NM>& L) {
    const int n = L.cell.n;
    const int64_t c = L.c;
    float contrast = 0.f, dist = 0.f, big = 0.f;
    for (int i = 0; i < n; ++i) {
        if (L.cell.z[i] == 0.f) continue;
        const float ck = static_cast<float>(ws.cand[idx(2 * NM + i, ws.ncell, c)]);
        contrast = fmaxf(contrast, fabsf(L.point.lnk[i]));
        dist = fmaxf(dist, fabsf(L.point.lnk[i] - ck));
        big = fmaxf(big, fabsf(ck));
    }
    if (contrast < 1e-4f || L.point.z_v - L.point.z_l <= 1e-5f * fmaxf(L.point.z_v, L.point.z_l)) return true;
    if (dist <= 1e-3f * (1.f + big)) return true;
    const float gc = static_cast<float>(ws.cand_s[idx(4, ws.ncell, c)]);
    return L.point.gibbs > gc + 1e-4f * (1.f + fabsf(gc));
}

// FP32 ln K successive substitution over a persistent work queue of attempts.
// open == 0: every split attempt from its seed, with the reference's Gibbs
// line search, classified at its end (fp32::SplitClass).
// open == 1: the attempts the polish left open (class aFailed beside a
// polished pair), continued from their FP32 end point to predict where they
// converge.  Where FP32 cannot resolve the reference's Armijo test
// (predicted decrease below the rounding guard) the step is taken when the
// Gibbs energy does not rise beyond the guard, without the residual-decrease
// rule that stopped the first pass.  The prediction only prunes attempts
// (prune_open); the end point and class of a kept attempt stay as the first
// pass left them, and the FP64 continuation decides it exactly.
template <int NM>
__global__ void __launch_bounds__(128) split32_kernel(const Mixture* __restrict__ mix_g, Workspace ws,
                                                      const double* __restrict__ p, const double* __restrict__ t,
                                                      float ss_switch, int open) {
    __shared__ Mixture m;
    stage_mixture(mix_g, m);
    const int total = ws.counters[open ? qOpenItems : qAttempts];
    int* const cursor = &ws.counters[open ? qOpenCursor : qAttemptCursor];
    SplitLane<NM> L;
    L.stage = 3;
    L.item = -1;
    bool live = true;
    for (;;) {
        if (live && L.stage >= 2) {
            if (L.item >= 0 && L.stage == 2 && open) {
                const bool converged = L.iter >= 0 && L.point.fug <= ss_switch;
                if (converged && prune_open(ws, L))
                    ws.att_class[idx(L.order, ws.ncell, L.c)] = static_cast<signed char>(fp32::aPruned);
                atomicAdd(&ws.counters_out[idx(cSplitEvals, ws.ncell, L.c)], L.cell.evals);
            } else if (L.item >= 0 && L.stage == 2) {
                int cls = fp32::aFailed;
                const int n = L.cell.n;
                float contrast = 0.f;
                for (int i = 0; i < n; ++i) contrast = fmaxf(contrast, fabsf(L.point.lnk[i]));
                if (L.iter >= 0) {
                    // contraction per iteration: the last window above the FP32
                    // floor, else the whole descent from the seed
                    float rate = L.rate;
                    if (!(rate > 0.f) && L.iter > 0 && L.fug0 > L.point.fug)
                        rate = logf(L.fug0 / L.point.fug) / static_cast<float>(L.iter);
                    // iterations the reference's FP64 iteration still needs to |r| <= 1e-11
                    const float needed = rate > 0.f ? logf(fmaxf(L.point.fug, 1e-11f) / 1e-11f) / rate : 1e9f;
                    if (contrast < 1e-4f || L.point.z_v - L.point.z_l <= 1e-5f * fmaxf(L.point.z_v, L.point.z_l))
                        cls = fp32::aTrivial;
                    else if (L.iter >= 512)
                        cls = fp32::aLimit;  // FP32 and FP64 track each other far above the floor
                    else if (L.point.fug <= 1e-3f && static_cast<float>(L.iter) + needed <= 448.f)
                        cls = fp32::aConverged;  // converges well inside the 512-iteration budget
                    else if (L.point.fug >= fp32::kFarFailure)
                        cls = fp32::aFailedFar;  // stopped far from any pair
                    // else: unsettled, continued exactly in FP64 with the remaining budget
                    ws.att_rate[idx(L.order, ws.ncell, L.c)] = rate;
                }
                ws.att_iter[idx(L.order, ws.ncell, L.c)] = static_cast<short>(L.iter < 0 ? 0 : L.iter);
                const int64_t c = L.c;
                ws.att_class[idx(L.order, ws.ncell, c)] = static_cast<signed char>(cls);
                if (cls == fp32::aLimit) atomicAdd(&ws.counters[sLimitAttempts], 1);
                if (L.iter >= 0) {
                    ws.att_gibbs[idx(L.order, ws.ncell, c)] = L.point.gibbs;
                    for (int i = 0; i < n; ++i) ws.att_lnk[idx(L.order * NM + i, ws.ncell, c)] = L.point.lnk[i];
                } else {
                    // no FP32 state of this attempt (its seed or the cell's constants
                    // did not evaluate): the seed stays, and the FP64 continuation
                    // runs the attempt from its exact seed
                    ws.att_gibbs[idx(L.order, ws.ncell, c)] = INFINITY;
                }
                atomicAdd(&ws.counters_out[idx(cSplitEvals, ws.ncell, c)], L.cell.evals);
                atomicAdd(&ws.counters_out[idx(cSplitIters, ws.ncell, c)], L.iter);
            }
            L.item = atomicAdd(cursor, 1);
            if (L.item >= total) {
                live = false;
            } else {
                const int code = ws.attempt_items[L.item];
                L.c = code >> 5;
                L.order = code & 31;
                int active;
                L.iter = open ? ws.att_iter[idx(L.order, ws.ncell, L.c)] : 0;
                L.limit = open ? min(512, L.iter + kPredictionIterations) : 512;
                L.stage = 0;
                L.rate = 0.f;
                L.ck_iter = L.iter;
                if (!load_cell32(m, ws, L.c, p, t, L.cell, active)) {
                    L.iter = -1;
                    L.stage = 2;
                } else {
                    for (int i = 0; i < L.cell.n; ++i) L.lk[i] = ws.att_lnk[idx(L.order * NM + i, ws.ncell, L.c)];
                }
            }
        }
        if (__all_sync(0xffffffffu, !live)) break;
        if (!live || L.stage >= 2) continue;
        const int n = L.cell.n;
        if (L.stage == 1)
            for (int i = 0; i < n; ++i) L.lk[i] = fmaf(L.alpha / L.scale, L.point.res[i], L.point.lnk[i]);
        const bool ok = fp32::split_evaluate(m, L.cell, L.lk, L.next, L.stage == 1 ? L.point.beta : 0.5f);
        if (L.stage == 0) {
            if (!ok) {
                L.iter = -1;
                L.stage = 2;
                continue;
            }
            fp32::copy_state(L.point, L.next, n);
            L.fug0 = L.point.fug;
            L.ck_fug = L.point.fug;
            split_step_or_finish(L, ss_switch);
            continue;
        }
        bool accept = false;
        if (ok) {
            const float predicted = -L.alpha * L.slope;
            const float guard = 64.f * fp32::kEpsF * (L.point.mag + L.next.mag);
            accept = predicted > guard ? L.next.gibbs <= L.point.gibbs - 1e-4f * predicted
                                       : (L.next.gibbs <= L.point.gibbs + guard &&
                                          (open || L.point.fug - L.next.fug > 1e-4f * (L.alpha / L.scale) * L.point.fug));
        }
        if (accept) {
            fp32::copy_state(L.point, L.next, n);
            ++L.iter;
            split_step_or_finish(L, ss_switch);
        } else if (++L.bt >= 20) {
            L.stage = 2;
        } else {
            L.alpha *= 0.5f;
        }
    }
}

// ---------------------------------------------------------------------------
// Stage 5: FP64 polish of the minimum-Gibbs attempt and the acceptance rules.
template <int NM>
struct PolishScratch {
    fp64::SplitState<NM> st, nx;
    double lnk[NM], e[NM], num[NM], J[NM * NM], d[NM];
    double sl[NM], sv[NM];  // mixing row sums of the two phases
    int piv[NM];
    int jacobians, solves;  // closed-form Jacobians factorised, chord-step LU solves
};

// Closed-form full-chart d ln phi_i / d x_j = cs_i s_j + cb_i b_j + ca a_ij of
// one PR76 phase at composition x with root Z (mole fractions as independent
// variables, the chart of pr76_phase_ad.hpp:57-122): with r_i = b_i/b,
// q_i = 2 s_i/a - r_i, G = A ln((Z+(1+sqrt2)B)/(Z+(1-sqrt2)B)) / (2 sqrt2 B),
// ln phi_i = r_i (Z-1) - ln(Z-B) - q_i G, dA/dx_j = 2 s_j p/(RT)^2,
// dB/dx_j = b_j p/RT and dZ from the cubic's implicit derivative.
template <int NM>
__device__ bool phi_coefficients(const Mixture& m, fp64::Cell<NM>& c, const double* x, double Z, double* s_out,
                                 double* cs, double* cb, double& ca) {
    double amix, bmix, A, B;
    if (!fp64::mix(m, c, x, amix, bmix) || !fp64::coefficients(c.p, c.t, amix, bmix, A, B)) return false;
    const int n = c.n;
    const double sqrt2 = 1.4142135623730951;
    const double prt = c.p / (kR * c.t);
    const double p1 = prt / (kR * c.t), p2 = prt;
    const double d1 = Z + (1.0 + sqrt2) * B, d2 = Z + (1.0 - sqrt2) * B;
    const double L = log(d1 / d2);
    const double G = A * L / (2.0 * sqrt2 * B);
    const double fz = (3.0 * Z - 2.0 * (1.0 - B)) * Z + (A - 3.0 * B * B - 2.0 * B);
    const double fa = Z - B;
    const double fb = Z * Z - (6.0 * B + 2.0) * Z - A + 2.0 * B + 3.0 * B * B;
    const double zs = -2.0 * fa * p1 / fz, zb = -fb * p2 / fz;
    const double inv = 1.0 / d1 - 1.0 / d2;
    const double ls = zs * inv, lb = zb * inv + p2 * ((1.0 + sqrt2) / d1 - (1.0 - sqrt2) / d2);
    const double gs = (2.0 * p1 * L + A * ls) / (2.0 * sqrt2 * B), gb = A * lb / (2.0 * sqrt2 * B) - G * p2 / B;
    ca = -2.0 * G / amix;
    bool ok = isfinite(ca);
    for (int i = 0; i < n; ++i) {
        const double si = c.sums[i];
        s_out[i] = si;
        const double r = m.b[i] / bmix, q = 2.0 * si / amix - r;
        cs[i] = r * zs - zs / (Z - B) + 4.0 * G * si / (amix * amix) - q * gs;
        cb[i] = -r * (Z - 1.0) / bmix + r * zb - (zb - p2) / (Z - B) - G * r / bmix - q * gb;
        ok = ok && isfinite(cs[i]) && isfinite(cb[i]);
    }
    return ok;
}

// dF/dln K of F = ln x - ln y + ln phi_L(x) - ln phi_V(y) on the RR manifold at
// fixed feed (the RR linearisation of detail/pt_sensitivity_detail.hpp:291-345):
// dbeta_j = (x_j y_j / z_j)/h, h = sum_k (y_k - x_k)^2 / z_k, and
//   J_ij = -delta_ij - (x_j y_j / z_j) [(U^L_i - U^V_i)/h + beta PhiL_ij + (1-beta) PhiV_ij]
// with U^L_i = sum_k PhiL_ik x_k g_k, U^V_i = sum_k PhiV_ik y_k g_k,
// g_k = (y_k - x_k)/z_k, Phi the closed-form d ln phi / d x of each phase.
template <int NM>
__device__ bool equilibrium_jacobian(const Mixture& m, fp64::Cell<NM>& c, PolishScratch<NM>& s) {
    const int n = c.n;
    const fp64::SplitState<NM>& st = s.st;
    double csl[NM], cbl[NM], csv[NM], cbv[NM], cal, cav;
    if (!phi_coefficients(m, c, st.x, st.z_l, s.sl, csl, cbl, cal) ||
        !phi_coefficients(m, c, st.y, st.z_v, s.sv, csv, cbv, cav))
        return false;
    double h = 0.0, s1l = 0.0, s2l = 0.0, s1v = 0.0, s2v = 0.0;
    double xg[NM], yg[NM];
    for (int k = 0; k < n; ++k) {
        xg[k] = yg[k] = 0.0;
        if (c.z[k] == 0.0) continue;
        const double g = (st.y[k] - st.x[k]) / c.z[k];
        h += (st.y[k] - st.x[k]) * g;
        xg[k] = st.x[k] * g;
        yg[k] = st.y[k] * g;
        s1l += s.sl[k] * xg[k];
        s2l += m.b[k] * xg[k];
        s1v += s.sv[k] * yg[k];
        s2v += m.b[k] * yg[k];
    }
    if (!(h > 0.0) || !isfinite(h)) return false;
    for (int i = 0; i < n; ++i) {
        if (c.z[i] == 0.0) {
            for (int j = 0; j < n; ++j) s.J[i * n + j] = i == j ? 1.0 : 0.0;
            continue;
        }
        // row i of a_ij = sqrt(a_i a_j)(1 - k_ij), a_ii = a_i
        double tl = 0.0, tv = 0.0;
        for (int k = 0; k < n; ++k) {
            const double aik = k == i ? c.a[i] : (c.root[i] * m.factor[i * n + k]) * c.root[k];
            tl += aik * xg[k];
            tv += aik * yg[k];
        }
        const double u = ((csl[i] * s1l + cbl[i] * s2l + cal * tl) - (csv[i] * s1v + cbv[i] * s2v + cav * tv)) / h;
        for (int j = 0; j < n; ++j) {
            if (c.z[j] == 0.0) {
                s.J[i * n + j] = 0.0;
                continue;
            }
            const double aij = j == i ? c.a[i] : (c.root[i] * m.factor[i * n + j]) * c.root[j];
            const double phil = csl[i] * s.sl[j] + cbl[i] * m.b[j] + cal * aij;
            const double phiv = csv[i] * s.sv[j] + cbv[i] * m.b[j] + cav * aij;
            const double w = st.x[j] * st.y[j] / c.z[j];
            s.J[i * n + j] = (i == j ? -1.0 : 0.0) - w * (u + st.beta * phil + (1.0 - st.beta) * phiv);
        }
    }
    for (int k = 0; k < n * n; ++k)
        if (!isfinite(s.J[k])) return false;
    return true;
}

// The reference's ln K iteration (pt_split.hpp:364-405) replayed on the
// linearisation r' = r + (alpha / scale) J r around a pair, from the FP64
// residual r at an attempt's FP32 end point.  Returns the iterations to
// |r| <= 1e-11 (0 when |I + J| < 1 in the max norm: then every step of every
// length contracts |r|, so the reference's iteration cannot stall there), or
// -1 when every halving is rejected, or `budget` when it is reached.
//  * Where the Gibbs test is resolvable (predicted decrease above the round-off
//    guard) the step is the reference's Armijo test on the quadratic model of
//    the Gibbs energy its slope formula implies: grad G = -H r with
//    H = beta (1 - beta) diag(c) + c c^T / h, c_i = x_i y_i / z_i, so
//    dG(alpha) = -alpha q / s + alpha^2 p / (2 s^2), q = r^T H r, p = -r^T H J r.
//  * Below the guard it is the residual-decrease rule, up to 24 halvings.
// Two outcomes mark an FP32 attempt whose reference run ends elsewhere: a
// stall (two close slow modes of I + J keep the residual a mix whose max norm
// rises along the step; the reference ends line_search_failed just short of
// convergence), and the budget (I + J expands some direction: the FP32
// iteration stopped near a saddle that the reference's run leaves).
__device__ inline int replay_linear(int n, const double* J, const double* r0, const double* x, const double* y,
                                    const double* z, double beta, double guard64, int budget) {
    // FP32 arithmetic: the decisions compare relative changes of 1e-4 and
    // more, and FP32 keeps the replay off the FP64 pipe
    float Jf[kMaxC * kMaxC], r[kMaxC], jr[kMaxC], cw[kMaxC];
    float h = 0.f, norm = 0.f;
    for (int i = 0; i < n; ++i) {
        const bool act = z[i] > 0.0;
        r[i] = act ? static_cast<float>(r0[i]) : 0.f;
        cw[i] = act ? static_cast<float>((x[i] / z[i]) * y[i]) : 0.f;
        if (act) h += static_cast<float>((y[i] - x[i]) * ((y[i] - x[i]) / z[i]));
        float row = 0.f;
        for (int j = 0; j < n; ++j) {
            const bool on = act && z[j] > 0.0;
            Jf[i * n + j] = on ? static_cast<float>(J[i * n + j]) : 0.f;
            if (on) row += fabsf((i == j ? 1.f : 0.f) + Jf[i * n + j]);
        }
        norm = fmaxf(norm, row);
    }
    if (!(h > 0.f)) return -1;
    if (norm < 1.f - 1e-4f) return 0;
    const float bb = static_cast<float>(beta * (1.0 - beta));
    const float guard = static_cast<float>(guard64);
    for (int it = 0; it < budget; ++it) {
        float fug = 0.f, first = 0.f, second = 0.f;
        for (int i = 0; i < n; ++i) {
            fug = fmaxf(fug, fabsf(r[i]));
            first = fmaf(cw[i], r[i], first);
            second = fmaf(cw[i] * r[i], r[i], second);
        }
        if (fug <= 1e-11f) return it;
        const float scale = fmaxf(1.f, fug / 2.f);
        const float q = bb * second + (first / h) * first;
        float firstj = 0.f, mixed = 0.f;
        for (int i = 0; i < n; ++i) {
            float v = 0.f;
            for (int j = 0; j < n; ++j) v = fmaf(Jf[i * n + j], r[j], v);
            jr[i] = v;
            firstj = fmaf(cw[i], v, firstj);
            mixed = fmaf(cw[i] * r[i], v, mixed);
        }
        const float pq = -(bb * mixed + (first / h) * firstj);
        float alpha = 1.f;
        bool accepted = false;
        for (int bt = 0; bt < 24 && !accepted; ++bt) {
            if (alpha * q / scale > guard) {
                accepted = !(pq > 0.f) || alpha * pq <= 2.f * (1.f - 1e-4f) * scale * q;
            } else {
                float next = 0.f;
                for (int i = 0; i < n; ++i) next = fmaxf(next, fabsf(fmaf(alpha / scale, jr[i], r[i])));
                accepted = next <= 1e-11f || fug - next > 1e-4f * (alpha / scale) * fug;
            }
            if (!accepted) alpha *= 0.5f;
        }
        if (!accepted) return -1;
        for (int i = 0; i < n; ++i) r[i] = fmaf(alpha / scale, jr[i], r[i]);
    }
    return budget;
}

// Newton polish of ln K from the FP32 solution: FP64 residual F(ln K) (RR +
// role phases, pt_split.hpp:300-341) and the exact FP64 Jacobian in closed form
// taken at the first FP64 state (chord iterations).  On success `s.st` holds the FP64 state
// at |F| <= 1e-13, or at the point where F stopped decreasing below 1e-11.
// `replay` receives replay_linear's count from the FP32 end point within
// `budget` iterations (the reference's 512 less the FP32 iterations), or 0
// when that point is already converged.
template <int NM>
__device__ bool polish_split(const Mixture& m, fp64::Cell<NM>& c64, PolishScratch<NM>& s, int budget, int& replay) {
    const int n = c64.n;
    int evals = 0;
    replay = 0;
    if (fp64::split_evaluate(m, c64, s.lnk, s.st, evals, 1 << 30, s.e, s.num, true) != fp64::kConverged) return false;
    if (s.st.fug <= 1e-13) return true;
    if (!equilibrium_jacobian(m, c64, s)) return false;
    replay = replay_linear(n, s.J, s.st.res, s.st.x, s.st.y, c64.z, s.st.beta, 2.0 * s.st.guard, budget);
    double norm;
    if (!ad::lu_factor(s.J, s.piv, n, norm)) return false;
    ++s.jacobians;
    double prev = s.st.fug;
    for (int it = 0; it < 8; ++it) {
        for (int i = 0; i < n; ++i) s.d[i] = -s.st.res[i];
        ++s.solves;
        if (!ad::lu_solve(s.J, s.piv, n, s.d)) return false;
        for (int i = 0; i < n; ++i) s.lnk[i] = s.st.lnk[i] + s.d[i];
        // RR Newton from the current beta: a chord step moves ln K by |F| or less
        if (fp64::split_evaluate(m, c64, s.lnk, s.nx, evals, 1 << 30, s.e, s.num, true, s.st.beta, &s.st) !=
            fp64::kConverged)
            return prev <= 1e-11;
        if (!(s.nx.fug < prev)) return prev <= 1e-11;
        fp64::copy_state(s.st, s.nx, n);
        prev = s.st.fug;
        if (prev <= 1e-13) return true;
    }
    return prev <= 1e-11;
}

// Acceptance of a fugacity-converged state, pt_split.hpp:351-362.
// Attempts the FP64 continuation must settle: every one except those that
// collapsed to the trivial solution or provably end at the iteration limit.
__device__ __forceinline__ bool unsettled(int cls) { return cls != fp32::aTrivial && cls != fp32::aLimit; }

// Attempts of a cell that FP32 converged elsewhere the polish cannot skip: the
// reference keeps the first attempt of least Gibbs energy among all that
// converge (pt_split.hpp:459-486), and an attempt whose FP32 line search
// stopped near a pair, where FP32 rounding decides its tests (class aFailed),
// can still converge in the reference's FP64 iteration, to a pair of lower
// Gibbs energy than the polished one.  An attempt that stopped far from any
// pair (aFailedFar) stops there in FP64 too.
__device__ __forceinline__ bool open_attempt(int cls) { return cls == fp32::aFailed; }

// A cell FP32 cannot screen -- no FP32 attempt converged, or the replay of the
// reference's line search puts the polished attempt at risk -- is solved again
// by the exact sub-solve, every trial and attempt an FP64 item along the
// reference's own path from its start.  On such cells (hard near-critical
// states, N = 20 at 10-12 MPa and 365-375 K) FP32 descents stop early and the
// FP64 runs continued from there end differently from the reference's runs
// from the start.  Warm cells go to the cold pass instead.  Returns whether the
// cell was marked.
__device__ __forceinline__ bool mark_exact(const Workspace& ws, int64_t c) {
    if (ws.fp64_items || (ws.pass == kPassWarm && ws.warm_cell[c] != 0)) return false;
    const int slot = atomicAdd(&ws.counters[sExactCells], 1);
    if (slot < ws.exact_capacity) {
        ws.exact_list[slot] = static_cast<int>(c);
        ws.phase[c] = pExact;
    } else {
        // beyond the sub-solve's capacity: the plain FP64 solver, the same rules
        ws.phase[c] = pFallback;
        atomicAdd(&ws.counters[qFallback], 1);
    }
    return true;
}

// The exact sub-solve's inputs: the marked cells packed into `cap` slots
// (cell-fastest, stride cap); unused slots get an invalid pressure, which the
// sub-solve's setup turns into an invalid request at no cost.
template <int NM>
__global__ void gather_exact_kernel(Workspace ws, const double* __restrict__ p, const double* __restrict__ t,
                                    const double* __restrict__ z, int n, int cap, double* sp, double* st,
                                    double* sz) {
    const int count = min(ws.counters[sExactCells], cap);
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < cap; k += gridDim.x * blockDim.x) {
        const bool live = k < count;
        const int64_t c = live ? ws.exact_list[k] : 0;
        sp[k] = live ? p[c] : nan;
        st[k] = live ? t[c] : 300.0;
        for (int i = 0; i < n; ++i) sz[static_cast<int64_t>(i) * cap + k] = live ? z[idx(i, ws.io_stride, c)] : 1.0 / n;
    }
}

// The exact sub-solve's answers written back at the marked cells' places.
template <int NM>
__global__ void scatter_exact_kernel(Workspace ws, int n, int cap, DeviceOutputs sub, DeviceOutputs out) {
    const int count = min(ws.counters[sExactCells], cap);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        const int64_t c = ws.exact_list[k];
        auto row = [&](const double* from, double* to, int rows) {
            if (!to) return;
            for (int i = 0; i < rows; ++i) to[idx(i, ws.io_stride, c)] = from[static_cast<int64_t>(i) * cap + k];
        };
        if (out.status) out.status[c] = sub.status[k];
        row(sub.beta, out.beta, 1);
        row(sub.x, out.x, n);
        row(sub.y, out.y, n);
        row(sub.lnk, out.lnk, n);
        row(sub.lnphi_l, out.lnphi_l, n);
        row(sub.lnphi_v, out.lnphi_v, n);
        row(sub.z_l, out.z_l, 1);
        row(sub.z_v, out.z_v, 1);
        if (out.counters)
            for (int r = 0; r < cCount; ++r)
                out.counters[idx(r, ws.io_stride, c)] = sub.counters[static_cast<int64_t>(r) * cap + k];
        ws.phase[c] = sub.status[k];
    }
}

// Queues a cell's attempts for the FP64 continuation (split64) and lists the
// cell for select64: every unsettled attempt when no polished pair was
// accepted (cand_order < 0), else the open attempts, which then compete with
// the polished pair of attempt `cand_order` and Gibbs energy `cand_g` already
// stored in `cand`.  `from_seed`: the attempts run from their FP64 seeds with
// the full budget (the reference's own runs) instead of from their FP32 end
// points.  A cell whose items do not fit goes to the plain FP64 fallback.
template <int NM>
__device__ void queue_attempts64(const Workspace& ws, int64_t c, int na, int cnt, int cand_order, double cand_g,
                                 bool from_seed = false) {
    const int base = atomicAdd(&ws.counters[qS64Items], cnt);
    if (base + cnt > ws.s64_capacity) {
        ws.phase[c] = pFallback;
        atomicAdd(&ws.counters[qFallback], 1);
        return;
    }
    int k = 0;
    for (int a = 0; a < na; ++a) {
        const int cls = ws.att_class[idx(a, ws.ncell, c)];
        if (cand_order < 0 ? unsettled(cls) : open_attempt(cls))
            ws.s64_items[base + k++] = (static_cast<int>(c) << 5) | (from_seed ? kFromSeed : 0) | a;
    }
    ws.s64_base[c] = base;
    ws.s64_count[c] = cnt;
    ws.cand_s[idx(4, ws.ncell, c)] = cand_order >= 0 ? cand_g : __longlong_as_double(0x7ff8000000000000LL);
    ws.cand_s[idx(6, ws.ncell, c)] = static_cast<double>(cand_order);
    ws.phase[c] = pSplit64;
    ws.s64_cells[atomicAdd(&ws.counters[qS64Cells], 1)] = static_cast<int>(c);
}

// A polished pair of attempt `cand_order` (Gibbs energy `cand_g`, stored in
// `cand`) beside `open` attempts FP32 left open: the open attempts go to the
// FP32 prediction (the open pass of split32_kernel) and the cell waits for
// compete_kernel.  The feed-test cell list is free by now and holds these
// cells.
template <int NM>
__device__ void list_open(const Workspace& ws, int64_t c, int na, int open, int cand_order, double cand_g) {
    ws.cand_s[idx(4, ws.ncell, c)] = cand_g;
    ws.cand_s[idx(6, ws.ncell, c)] = static_cast<double>(cand_order);
    const int base = atomicAdd(&ws.counters[qOpenItems], open);
    int k = 0;
    for (int a = 0; a < na; ++a)
        if (open_attempt(ws.att_class[idx(a, ws.ncell, c)])) ws.attempt_items[base + k++] = (static_cast<int>(c) << 5) | a;
    ws.phase[c] = pCompete;
    ws.trial_cells[atomicAdd(&ws.counters[qCompeteCells], 1)] = static_cast<int>(c);
    atomicAdd(&ws.counters[sCompeting], 1);
}

template <int NM>
__device__ bool split_accepted(const fp64::SplitState<NM>& st, int n) {
    double contrast = 0.0;
    for (int i = 0; i < n; ++i) contrast = fmax(contrast, fabs(st.lnk[i]));
    return st.fug <= 1e-11 && st.mass_abs <= 1e-12 && st.mass_rel <= 1e-10 && st.beta > 1e-10 &&
           1.0 - st.beta > 1e-10 && contrast > 1e-7 && st.z_v - st.z_l > 1e-8 * fmax(st.z_v, st.z_l);
}

// Phase-set review set-up for the selected pair (pt_split.hpp:490-512):
// Gibbs change against the feed, its guard, the review tolerance and the
// imposed reference ln(phi_eq) = common - ln z on the twice-normalised feed.
template <int NM>
__device__ void begin_review(const Workspace& ws, int64_t c, fp64::Cell<NM>& c64, double best_g) {
    const int n = c64.n;
    double feed_g = 0.0, corr = 0.0, magnitude = 1.0;
    for (int i = 0; i < n; ++i) {
        if (c64.z[i] == 0.0) continue;
        const double phi = ws.ref_lnphi[idx(i, ws.ncell, c)];
        kahan_add(c64.z[i] * (c64.lz[i] + phi), feed_g, corr);
        magnitude += c64.z[i] * (fabs(c64.lz[i]) + fabs(phi));
    }
    const double fug = ws.cand_s[idx(3, ws.ncell, c)];
    ws.cand_s[idx(4, ws.ncell, c)] = best_g - feed_g;
    ws.cand_s[idx(5, ws.ncell, c)] = ws.cand_s[idx(7, ws.ncell, c)] + 256.0 * kEps * magnitude;
    ws.cand_s[idx(6, ws.ncell, c)] = 1e-10 + 0.5 * fug;
    double zz[NM];
    for (int i = 0; i < n; ++i) zz[i] = c64.z[i];
    fp64::normalise_feed(c64, zz);
    for (int i = 0; i < n; ++i)
        ws.cand[idx(6 * NM + i, ws.ncell, c)] = c64.z[i] > 0.0 ? ws.cand[idx(5 * NM + i, ws.ncell, c)] - c64.lz[i] : 0.0;
    ws.phase[c] = pReview;
}

template <int NM>
__device__ void store_candidate(const Workspace& ws, int64_t c, const fp64::SplitState<NM>& st, int n) {
    for (int i = 0; i < n; ++i) {
        ws.cand[idx(0 * NM + i, ws.ncell, c)] = st.x[i];
        ws.cand[idx(1 * NM + i, ws.ncell, c)] = st.y[i];
        ws.cand[idx(2 * NM + i, ws.ncell, c)] = st.lnk[i];
        ws.cand[idx(3 * NM + i, ws.ncell, c)] = st.lnphi_l[i];
        ws.cand[idx(4 * NM + i, ws.ncell, c)] = st.lnphi_v[i];
        ws.cand[idx(5 * NM + i, ws.ncell, c)] = st.common[i];
    }
    ws.cand_s[idx(0, ws.ncell, c)] = st.beta;
    ws.cand_s[idx(1, ws.ncell, c)] = st.z_l;
    ws.cand_s[idx(2, ws.ncell, c)] = st.z_v;
    ws.cand_s[idx(3, ws.ncell, c)] = st.fug;
    ws.cand_s[idx(7, ws.ncell, c)] = st.guard;
}

// The polish candidates of cell c (its na attempts): the minimum-Gibbs
// FP32-converged attempt, and the second one where FP32 cannot separate the
// two Gibbs energies at different compositions (FP64 arbitrates); -1 for none.
// Returns the first.
template <int NM>
__device__ __forceinline__ int polish_candidates(const Workspace& ws, int64_t c, int n, int na, int candidates[2]) {
    // rank converged attempts by FP32 Gibbs energy (ties in FP32 resolved in FP64)
    int best = -1, second = -1;
    for (int a = 0; a < na; ++a) {
        if (ws.att_class[idx(a, ws.ncell, c)] != fp32::aConverged) continue;
        const float g = ws.att_gibbs[idx(a, ws.ncell, c)];
        if (best < 0 || g < ws.att_gibbs[idx(best, ws.ncell, c)]) {
            second = best;
            best = a;
        } else if (second < 0 || g < ws.att_gibbs[idx(second, ws.ncell, c)]) {
            second = a;
        }
    }
    // a second converged attempt at a different composition with a Gibbs
    // energy FP32 cannot separate from the best: let FP64 arbitrate
    candidates[0] = best;
    candidates[1] = -1;
    if (best >= 0 && second >= 0) {
        const float gb = ws.att_gibbs[idx(best, ws.ncell, c)], gs = ws.att_gibbs[idx(second, ws.ncell, c)];
        float dist = 0.f;
        for (int i = 0; i < n; ++i)
            dist = fmaxf(dist, fabsf(ws.att_lnk[idx(best * NM + i, ws.ncell, c)] -
                                     ws.att_lnk[idx(second * NM + i, ws.ncell, c)]));
        if (gs - gb <= 1e-4f * (1.f + fabsf(gb)) && dist > 1e-2f) {
            candidates[1] = second;
            atomicAdd(&ws.counters[sCandidates2], 1);
        }
    }
    return best;
}

// A cell after its candidates' polishes: the work counters; then, on a replay
// risk, the exact sub-solve (or the FP64 runs of every attempt for a warm
// cell); without an accepted pair, the FP64 continuations of the unsettled
// attempts or the cell's status; with one, the competition of the attempts
// FP32 left open, or the review.
template <int NM>
__device__ __forceinline__ void polish_cell_next(const Workspace& ws, const DeviceOutputs& out, int64_t c,
                                                 fp64::Cell<NM>& c64, int na, int best, bool have, bool polish_failed,
                                                 bool replay_risk, double best_g, int cand_order, int jacobians,
                                                 int solves) {
    atomicAdd(&ws.counters_out[idx(kFp64EvalRow, ws.ncell, c)], c64.counters[cSplitEvals]);
    atomicAdd(&ws.counters_out[idx(cRrIters, ws.ncell, c)], c64.counters[cRrIters]);
    add_total(ws, tE64Polish, c64.counters[cSplitEvals]);
    add_count(ws, sPolishJacobians, jacobians);
    add_count(ws, sPolishSolves, solves);
    if (replay_risk) {
        atomicAdd(&ws.counters[sReplayRisk], 1);
        if (mark_exact(ws, c)) return;
        // (a warm cell) the reference's own runs of every attempt, from the FP64 seeds
        int cnt = 0;
        for (int a = 0; a < na; ++a) cnt += unsettled(ws.att_class[idx(a, ws.ncell, c)]);
        queue_attempts64<NM>(ws, c, na, cnt, -1, 0.0, true);
        return;
    }
    if (!have) {
        // FP64 continuation (reference ln K iteration, pt_split.hpp:275-408) of
        // every attempt FP32 left unsettled, from its FP32 end point: split64 items
        int cnt = 0;
        for (int a = 0; a < na; ++a) cnt += unsettled(ws.att_class[idx(a, ws.ncell, c)]);
        if (cnt == 0) {
            if (warm_cell(ws, c)) {  // the warm attempt collapsed: solve the cell cold
                ws.phase[c] = pRedo;
                atomicAdd(&ws.counters[sWarmRedo], 1);
                atomicAdd(&ws.counters[sWarmNoPair], 1);
                return;
            }
            ws.phase[c] = pIndeterminate;  // every attempt collapsed to the trivial solution
            write_status_only<NM>(out, ws, c, kIndeterminate, false);
            write_counters<NM>(out, ws, c);
            return;
        }
        atomicAdd(&ws.counters[best < 0 ? sFbNoAttempt : (polish_failed ? sFbPolish : sFbRejected)], 1);
        if (best < 0 && mark_exact(ws, c)) return;
        queue_attempts64<NM>(ws, c, na, cnt, -1, 0.0);
        return;
    }
    int open = 0;
    for (int a = 0; a < na; ++a) open += open_attempt(ws.att_class[idx(a, ws.ncell, c)]);
    if (open > 0) {
        list_open<NM>(ws, c, na, open, cand_order, best_g);
        return;
    }
    begin_review(ws, c, c64, best_g);
}

template <int NM>
__global__ void __launch_bounds__(64) polish_kernel(const Mixture* __restrict__ mix_g, Workspace ws,
                                                    const double* __restrict__ p, const double* __restrict__ t,
                                                    DeviceOutputs out) {
    __shared__ Mixture m;
    stage_mixture(mix_g, m);
    const int cells = ws.counters[qSplitCells];
    const int n = m.n;
    for (int slot = blockIdx.x * blockDim.x + threadIdx.x; slot < cells; slot += gridDim.x * blockDim.x) {
        const int64_t c = ws.split_cells[slot];
        fp64::Cell<NM> c64;
        PolishScratch<NM> s;
        s.jacobians = s.solves = 0;
        if (!load_cell64(m, ws, c, p, t, c64)) {
            ws.phase[c] = pFallback;
            atomicAdd(&ws.counters[qFallback], 1);
            atomicAdd(&ws.counters[sFbLoad], 1);
            continue;
        }
        const int na = ws.att_count[c];
        int candidates[2];
        const int best = polish_candidates<NM>(ws, c, n, na, candidates);
        bool have = false, polish_failed = false, replay_risk = false;
        double best_g = 0.0;
        int cand_order = -1;
        for (int k = 0; k < 2 && candidates[k] >= 0; ++k) {
            const int a = candidates[k];
            for (int i = 0; i < n; ++i) s.lnk[i] = ws.att_lnk[idx(a * NM + i, ws.ncell, c)];
            const int done = ws.att_iter[idx(a, ws.ncell, c)];
            int replay = 0;
            if (!polish_split(m, c64, s, 512 - done, replay)) {
                polish_failed = true;
                continue;
            }
            // the reference's attempt may stop short of this pair (a stalled line
            // search, or the iteration limit): the exact FP64 continuation decides
            if (replay < 0 || done + replay > kReplayLimit) {
                replay_risk = true;
                break;
            }
            if (!split_accepted(s.st, n)) continue;
            if (have && !(s.st.gibbs < best_g)) continue;
            have = true;
            best_g = s.st.gibbs;
            cand_order = a;
            store_candidate(ws, c, s.st, n);
        }
        polish_cell_next<NM>(ws, out, c, c64, na, best, have, polish_failed, replay_risk, best_g, cand_order,
                             s.jacobians, s.solves);
    }
}

// The per-thread polish as a state machine (opt-in, BatchedShape::polish_stream):
// the work of polish_kernel, cell by cell down the thread's grid-stride
// sequence and with the same arithmetic, but every loop iteration makes one
// FP64 property evaluation (split_evaluate, one call site) for every thread
// that has a cell, whatever step of its polish that cell is at -- a
// candidate's first FP64 state or one of its chord steps.  In polish_kernel a
// warp's lanes reach their evaluations at different points of the cell loop
// (one building a Jacobian, one in its fifth chord step, one starting its next
// cell) and run them one after another; here they evaluate together, and
// only the Jacobians, their factorisation and the per-cell bookkeeping
// diverge.
template <int NM>
__global__ void __launch_bounds__(64) polish_stream_kernel(const Mixture* __restrict__ mix_g, Workspace ws,
                                                           const double* __restrict__ p, const double* __restrict__ t,
                                                           DeviceOutputs out) {
    __shared__ Mixture m;
    stage_mixture(mix_g, m);
    const int cells = ws.counters[qSplitCells];
    const int n = m.n;
    const int stride = gridDim.x * blockDim.x;
    int slot = blockIdx.x * blockDim.x + threadIdx.x;
    enum Step : int { kFetch, kFirst, kChord, kDone };
    int step = kFetch;
    // the cell
    int64_t c = -1;
    fp64::Cell<NM> c64;
    PolishScratch<NM> s;
    int na = 0, best = -1, k = 0, cand_order = -1;
    int candidates[2] = {-1, -1};
    bool have = false, polish_failed = false, replay_risk = false;
    double best_g = 0.0;
    // the candidate being polished (polish_split's state)
    int done = 0, replay = 0, chord = 0, evals = 0;
    double prev = 0.0;
    auto start_candidate = [&]() {
        const int a = candidates[k];
        for (int i = 0; i < n; ++i) s.lnk[i] = ws.att_lnk[idx(a * NM + i, ws.ncell, c)];
        done = ws.att_iter[idx(a, ws.ncell, c)];
        replay = 0;
        evals = 0;
        step = kFirst;
    };
    // the candidate loop of polish_kernel after polish_split returned `ok`
    auto end_candidate = [&](bool ok) {
        const int a = candidates[k];
        bool stop = false;
        if (!ok) {
            polish_failed = true;
        } else if (replay < 0 || done + replay > kReplayLimit) {
            replay_risk = true;
            stop = true;
        } else if (split_accepted(s.st, n) && (!have || s.st.gibbs < best_g)) {
            have = true;
            best_g = s.st.gibbs;
            cand_order = a;
            store_candidate(ws, c, s.st, n);
        }
        ++k;
        if (!stop && k < 2 && candidates[k] >= 0) {
            start_candidate();
            return;
        }
        polish_cell_next<NM>(ws, out, c, c64, na, best, have, polish_failed, replay_risk, best_g, cand_order,
                             s.jacobians, s.solves);
        step = kFetch;
    };
    // the next chord step's ln K: J d = -F at the current state (false: the solve failed)
    auto chord_target = [&]() -> bool {
        for (int i = 0; i < n; ++i) s.d[i] = -s.st.res[i];
        ++s.solves;
        if (!ad::lu_solve(s.J, s.piv, n, s.d)) return false;
        for (int i = 0; i < n; ++i) s.lnk[i] = s.st.lnk[i] + s.d[i];
        return true;
    };
    for (;;) {
        while (step == kFetch) {
            if (slot >= cells) {
                step = kDone;
                break;
            }
            c = ws.split_cells[slot];
            slot += stride;
            s.jacobians = s.solves = 0;
            if (!load_cell64(m, ws, c, p, t, c64)) {
                ws.phase[c] = pFallback;
                atomicAdd(&ws.counters[qFallback], 1);
                atomicAdd(&ws.counters[sFbLoad], 1);
                continue;
            }
            na = ws.att_count[c];
            best = polish_candidates<NM>(ws, c, n, na, candidates);
            have = polish_failed = replay_risk = false;
            best_g = 0.0;
            cand_order = -1;
            k = 0;
            if (candidates[0] < 0) {
                polish_cell_next<NM>(ws, out, c, c64, na, best, have, polish_failed, replay_risk, best_g,
                                     cand_order, s.jacobians, s.solves);
                continue;
            }
            start_candidate();
        }
        if (step == kDone) break;
        // this iteration's evaluation: a candidate's first FP64 state, or a chord step
        const bool first = step == kFirst;
        const int r = fp64::split_evaluate(m, c64, s.lnk, first ? s.st : s.nx, evals, 1 << 30, s.e, s.num, true,
                                           first ? 0.5 : s.st.beta, first ? nullptr : &s.st);
        if (first) {
            if (r != fp64::kConverged) {
                end_candidate(false);
                continue;
            }
            if (s.st.fug <= 1e-13) {
                end_candidate(true);
                continue;
            }
            if (!equilibrium_jacobian(m, c64, s)) {
                end_candidate(false);
                continue;
            }
            replay = replay_linear(n, s.J, s.st.res, s.st.x, s.st.y, c64.z, s.st.beta, 2.0 * s.st.guard, 512 - done);
            double norm;
            if (!ad::lu_factor(s.J, s.piv, n, norm)) {
                end_candidate(false);
                continue;
            }
            ++s.jacobians;
            prev = s.st.fug;
            chord = 0;
            if (!chord_target()) {
                end_candidate(false);
                continue;
            }
            step = kChord;
            continue;
        }
        if (r != fp64::kConverged || !(s.nx.fug < prev)) {
            end_candidate(prev <= 1e-11);
            continue;
        }
        fp64::copy_state(s.st, s.nx, n);
        prev = s.st.fug;
        if (prev <= 1e-13) {
            end_candidate(true);
            continue;
        }
        if (++chord >= 8) {
            end_candidate(prev <= 1e-11);
            continue;
        }
        if (!chord_target()) end_candidate(false);
    }
}

// Cells whose polished pair waited on open attempts: the pair goes to the
// review when the FP32 prediction pruned every open attempt; otherwise the
// attempts left open continue exactly in FP64 (split64) and compete with the
// pair in select64.
template <int NM>
__global__ void __launch_bounds__(64) compete_kernel(const Mixture* __restrict__ mix_g, Workspace ws,
                                                     const double* __restrict__ p, const double* __restrict__ t) {
    __shared__ Mixture m;
    stage_mixture(mix_g, m);
    const int cells = ws.counters[qCompeteCells];
    for (int slot = blockIdx.x * blockDim.x + threadIdx.x; slot < cells; slot += gridDim.x * blockDim.x) {
        const int64_t c = ws.trial_cells[slot];
        const int na = ws.att_count[c];
        int open = 0;
        for (int a = 0; a < na; ++a) open += open_attempt(ws.att_class[idx(a, ws.ncell, c)]);
        const double cand_g = ws.cand_s[idx(4, ws.ncell, c)];
        if (open > 0) {
            queue_attempts64<NM>(ws, c, na, open, static_cast<int>(ws.cand_s[idx(6, ws.ncell, c)]), cand_g);
            atomicAdd(&ws.counters[sCompeteFp64], 1);
            continue;
        }
        fp64::Cell<NM> c64;
        if (!load_cell64(m, ws, c, p, t, c64)) {
            ws.phase[c] = pFallback;
            atomicAdd(&ws.counters[qFallback], 1);
            continue;
        }
        begin_review(ws, c, c64, cand_g);
    }
}

// Compacts the review cells into trial_cells (after the feed-test list is no
// longer needed) and resets the trial cursor.
template <int NM>
__global__ void relist_kernel(Workspace ws) {
    // single block: compaction order does not matter
    if (threadIdx.x == 0) {
        ws.counters[qTrialCells] = 0;
        ws.counters[qTrialCursor] = 0;
    }
    __syncthreads();
    for (int64_t c = threadIdx.x; c < ws.ncell; c += blockDim.x) {
        if (ws.phase[c] == pReview) {
            const int slot = atomicAdd(&ws.counters[qTrialCells], 1);
            ws.trial_cells[slot] = static_cast<int>(c);
        }
    }
}

// ---------------------------------------------------------------------------
// Stage 7: review decision, final status and outputs.
template <int NM>
__global__ void __launch_bounds__(64) finish_kernel(const Mixture* __restrict__ mix_g, Workspace ws,
                                                    const double* __restrict__ p, const double* __restrict__ t,
                                                    DeviceOutputs out) {
    __shared__ Mixture m;
    stage_mixture(mix_g, m);
    const int cells = ws.counters[qTrialCells];
    const int n = m.n;
    for (int slot = blockIdx.x * blockDim.x + threadIdx.x; slot < cells; slot += gridDim.x * blockDim.x) {
        const int64_t c = ws.trial_cells[slot];
        fp64::Cell<NM> cell;
        DecideScratch<NM> s;
        if (!load_cell64(m, ws, c, p, t, cell)) {
            ws.phase[c] = pFallback;
            atomicAdd(&ws.counters[qFallback], 1);
            continue;
        }
        // the review runs on the twice-normalised feed
        double zz[NM], ex0[NM], ex1[NM];
        for (int i = 0; i < n; ++i) zz[i] = cell.z[i];
        fp64::normalise_feed(cell, zz);
        for (int i = 0; i < n; ++i) {
            s.ref[i] = ws.cand[idx(6 * NM + i, ws.ncell, c)];
            ex0[i] = ws.cand[idx(0 * NM + i, ws.ncell, c)];
            ex1[i] = ws.cand[idx(1 * NM + i, ws.ncell, c)];
        }
        int active = 0;
        for (int i = 0; i < n; ++i) active += cell.z[i] > 0.0;
        const int ntr = auto_starts(active) + 2;
        const double tol = ws.cand_s[idx(6, ws.ncell, c)];
        bool negative = false, stationary = true;
        for (int k = 0; k < ntr; ++k) {
            const int cls = ws.tclass[idx(k, ws.ncell, c)];
            if (cls == fp32::tNegative) {
                negative = true;
            } else if (cls == fp32::tMarginal || cls == fp32::tRerun) {
                const int ts = ws.t64_status[idx(k, ws.ncell, c)];
                if (ts == fp64::kNegativeTpd) negative = true;
                else if (ts != fp64::kStationary) stationary = false;
            }
        }
        atomicAdd(&ws.counters_out[idx(kFp64EvalRow, ws.ncell, c)], cell.counters[cFinalEvals]);
        int status;
        if (negative) status = kPhaseSetUnstable;
        else if (ws.cand_s[idx(4, ws.ncell, c)] > ws.cand_s[idx(5, ws.ncell, c)]) status = kIndeterminate;
        else status = stationary ? kTwoPhase : kIndeterminate;
        if (warm_cell(ws, c) && status != kTwoPhase) {
            // only an accepted warm pair settles a cell; anything else gets the full cold solve
            ws.phase[c] = pRedo;
            atomicAdd(&ws.counters[sWarmRedo], 1);
            if (status == kPhaseSetUnstable) atomicAdd(&ws.counters[sWarmUnstable], 1);
            continue;
        }
        ws.phase[c] = status;
        write_status_only<NM>(out, ws, c, status, true);
        write_counters<NM>(out, ws, c);
    }
}

// ---------------------------------------------------------------------------
// Fallback: the plain FP64 reference algorithm for flagged cells.
template <int NM>
__global__ void __launch_bounds__(64) fallback_kernel(const Mixture* __restrict__ mix_g, Workspace ws,
                                                      const double* __restrict__ p, const double* __restrict__ t,
                                                      const double* __restrict__ z, DeviceOutputs out) {
    __shared__ Mixture m;
    stage_mixture(mix_g, m);
    if (ws.counters[qFallback] == 0) return;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t c = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; c < ws.ncell; c += stride) {
        if (ws.phase[c] != pFallback) continue;
        using namespace fp64;
        Cell<NM> cell;
        cell.n = m.n;
        cell.newton = true;
        cell.p = p[c];
        cell.t = t[c];
        for (int k = 0; k < cCount; ++k) cell.counters[k] = 0;
        double feed[NM];
        for (int i = 0; i < cell.n; ++i) feed[i] = z[idx(i, ws.io_stride, c)];
        Scratch<NM> w;
        CellResult<NM> r;
        const int status = solve_cell(m, cell, feed, w, r);
        ws.phase[c] = status;  // settled: a later pass of the same launch leaves it alone
        const int n = cell.n;
        const double nan = __longlong_as_double(0x7ff8000000000000LL);
        if (out.status) out.status[c] = status;
        const bool pair = r.has_pair && status != kSinglePhase && status != kInvalid;
        const SplitState<NM>& b = w.best;
        if (out.beta) out.beta[c] = pair ? b.beta : nan;
        for (int i = 0; i < n; ++i) {
            const int64_t k = idx(i, ws.io_stride, c);
            const bool single = status == kSinglePhase;
            if (out.x) out.x[k] = pair ? b.x[i] : (single ? cell.z[i] : nan);
            if (out.y) out.y[k] = pair ? b.y[i] : nan;
            if (out.lnk) out.lnk[k] = pair ? b.lnk[i] : nan;
            if (out.lnphi_l) out.lnphi_l[k] = pair ? b.lnphi_l[i] : (single ? r.ref_lnphi[i] : nan);
            if (out.lnphi_v) out.lnphi_v[k] = pair ? b.lnphi_v[i] : nan;
        }
        if (out.z_l) out.z_l[c] = pair ? b.z_l : (status == kSinglePhase ? r.ref_z : nan);
        if (out.z_v) out.z_v[c] = pair ? b.z_v : nan;
        if (out.counters)
            for (int k = 0; k < cCount; ++k)
                out.counters[idx(k, ws.io_stride, c)] = ws.counters_out[idx(k, ws.ncell, c)] + cell.counters[k];
    }
}

}  // namespace batched
}  // namespace pr76
