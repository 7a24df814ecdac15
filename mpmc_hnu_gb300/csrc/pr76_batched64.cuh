// FP64 work items of the mixed-precision flash, run as persistent per-lane
// state machines so that every lane of a warp performs one FP64 property
// evaluation per loop iteration (the same scheme as the FP32 stages).
//
//  trials64   a TPD trial with the reference's exact descent, line search and
//             stopping rules (pt_stability.hpp:343-457), started either at the
//             FP32 end point of the trial (continuation) or at the trial's
//             original start (exact re-run);
//  split64    a ln K split attempt with the reference's exact successive
//             substitution, Gibbs line search and acceptance rules
//             (pt_split.hpp:275-408), continued from the FP32 attempt's end
//             point.
// The evaluation budgets of the reference (100000 per stability test, 20000
// per flash for the split attempts) are applied per item; in the reference
// they only bind after thousands of iterations, far beyond the per-trial
// (512 x 32) and per-attempt (512 x 24) limits that are applied exactly.
#pragma once

#include "pr76_batched.cuh"

namespace pr76 {
namespace batched {

// Trial item modes.
enum TrialMode : int { mFeedContinue = 0, mFeedRerun = 1, mReviewContinue = 2, mReviewRerun = 3 };

__device__ __forceinline__ int trial_item(int64_t c, int k, int mode) {
    return (static_cast<int>(c) << 7) | (k << 2) | mode;
}

template <int NM>
struct Trial64Lane {
    fp64::Cell<NM> cell;
    fp64::TpdPoint<NM> point, next;
    double dir[NM], lnphi[NM], ref[NM];
    double tol, alpha, slope, scale;
    int64_t c;
    int item, k, mode, iter, bt, stage, status;  // stage 0 start, 1 line search, 2 done, 3 idle
    bool skip;  // current candidate not representable: count a backtrack without evaluating
};

template <int NM>
__device__ void t64_begin(const Mixture& m, const Workspace& ws, const double* p, const double* t, Trial64Lane<NM>& L) {
    const int code = ws.t64_items[L.item];
    L.c = code >> 7;
    L.k = (code >> 2) & 31;
    L.mode = code & 3;
    L.iter = 0;
    L.bt = 0;
    L.stage = 0;
    L.skip = false;
    L.status = fp64::kPropertyFailure;
    fp64::Cell<NM>& c = L.cell;
    if (!load_cell64(m, ws, L.c, p, t, c)) {
        L.stage = 2;
        return;
    }
    const int n = c.n;
    const bool review = L.mode >= mReviewContinue;
    int active = 0;
    for (int i = 0; i < n; ++i) active += c.z[i] > 0.0;
    double ex0[NM], ex1[NM];
    if (review) {
        double zz[NM];
        for (int i = 0; i < n; ++i) zz[i] = c.z[i];
        fp64::normalise_feed(c, zz);  // the review normalises the feed once more
        for (int i = 0; i < n; ++i) {
            L.ref[i] = ws.cand[idx(6 * NM + i, ws.ncell, L.c)];
            ex0[i] = ws.cand[idx(0 * NM + i, ws.ncell, L.c)];
            ex1[i] = ws.cand[idx(1 * NM + i, ws.ncell, L.c)];
        }
        L.tol = ws.cand_s[idx(6, ws.ncell, L.c)];
    } else {
        for (int i = 0; i < n; ++i) L.ref[i] = ws.ref_lnphi[idx(i, ws.ncell, L.c)];
        L.tol = 1e-10;
    }
    if (L.mode == mFeedRerun || L.mode == mReviewRerun) {
        fp64::make_start(c, L.k, active, ex0, ex1, auto_starts(active), L.next.w);
    } else {
        L.iter = ws.titer[idx(L.k, ws.ncell, L.c)];  // the FP32 iterations count against the 512
        double sum = 0.0, cs = 0.0;
        for (int i = 0; i < n; ++i) {
            L.next.w[i] = c.z[i] > 0.0 ? static_cast<double>(ws.tw[idx(L.k * NM + i, ws.ncell, L.c)]) : 0.0;
            kahan_add(L.next.w[i], sum, cs);
        }
        for (int i = 0; i < n; ++i) L.next.w[i] /= sum;
    }
    for (int i = 0; i < n; ++i)
        if (c.z[i] > 0.0 && L.next.w[i] == 0.0) {
            L.status = fp64::kUnrepresentableComposition;
            L.stage = 2;
        }
}

// Reference stopping rules at the current point, then the next line search.
template <int NM>
__device__ void t64_decide(Trial64Lane<NM>& L) {
    const int n = L.cell.n;
    if (fp64::tpd_negative(L.point, L.tol)) {
        L.status = fp64::kNegativeTpd;
        L.stage = 2;
        return;
    }
    if (!L.point.smooth) {
        L.status = fp64::kNonsmooth;
        L.stage = 2;
        return;
    }
    if (L.point.stat <= 1e-8) {
        L.status = fp64::kStationary;
        L.stage = 2;
        return;
    }
    if (L.iter >= 512) {
        L.status = fp64::kIterationLimit;
        L.stage = 2;
        return;
    }
    L.scale = fmax(1.0, L.point.stat / 4.0);
    double slope = 0.0, sc = 0.0;
    for (int i = 0; i < n; ++i) {
        L.dir[i] = 0.0;
        if (L.cell.z[i] == 0.0) continue;
        L.dir[i] = -L.point.res[i] / L.scale;
        kahan_add((L.point.w[i] * L.point.res[i]) * L.dir[i], slope, sc);
    }
    if (!isfinite(slope) || !(slope < 0.0)) {
        L.status = fp64::kLineSearchFailed;
        L.stage = 2;
        return;
    }
    L.slope = slope;
    L.alpha = 1.0;
    L.bt = 0;
    L.stage = 1;
}

template <int NM>
__device__ bool t64_candidate(Trial64Lane<NM>& L) {
    const int n = L.cell.n;
    double largest = -INFINITY;
    for (int i = 0; i < n; ++i)
        if (L.cell.z[i] > 0.0) {
            L.next.w[i] = L.point.lw[i] + L.alpha * L.dir[i];
            largest = fmax(largest, L.next.w[i]);
        }
    double sum = 0.0, cs = 0.0;
    for (int i = 0; i < n; ++i) {
        L.next.w[i] = L.cell.z[i] > 0.0 ? exp(L.next.w[i] - largest) : 0.0;
        kahan_add(L.next.w[i], sum, cs);
    }
    bool positive = isfinite(sum) && sum > 0.0;
    for (int i = 0; i < n; ++i) {
        L.next.w[i] /= sum;
        positive = positive && (L.cell.z[i] == 0.0 || L.next.w[i] > 0.0);
    }
    return positive;
}

template <int NM>
__device__ void t64_copy_point(fp64::TpdPoint<NM>& d, const fp64::TpdPoint<NM>& s, int n) {
    for (int i = 0; i < n; ++i) {
        d.w[i] = s.w[i];
        d.res[i] = s.res[i];
        d.lw[i] = s.lw[i];
    }
    d.value = s.value;
    d.guard = s.guard;
    d.stat = s.stat;
    d.smooth = s.smooth;
}

template <int NM>
__global__ void __launch_bounds__(64) trials64_kernel(const Mixture* __restrict__ mix_g, Workspace ws,
                                                      const double* __restrict__ p, const double* __restrict__ t) {
    __shared__ Mixture m;
    stage_mixture(mix_g, m);
    const int total = ws.counters[qT64Items];
    Trial64Lane<NM> L;
    L.stage = 3;
    L.item = -1;
    bool live = true;
    for (;;) {
        if (live && L.stage >= 2) {
            if (L.item >= 0 && L.stage == 2) {
                const int64_t c = L.c;
                const int n = L.cell.n;
                const bool review = L.mode >= mReviewContinue;
                ws.t64_status[idx(L.k, ws.ncell, c)] = static_cast<signed char>(L.status);
                if (!review && L.status == fp64::kNegativeTpd)
                    for (int i = 0; i < n; ++i) ws.tw64[idx(L.k * NM + i, ws.ncell, c)] = L.point.w[i];
                atomicAdd(&ws.counters_out[idx(kFp64EvalRow, ws.ncell, c)],
                          L.cell.counters[review ? cFinalEvals : cInitEvals]);
                add_total(ws, review ? tE64ReviewTrials : tE64FeedTrials, L.cell.counters[review ? cFinalEvals : cInitEvals]);
            }
            L.item = atomicAdd(&ws.counters[qT64Cursor], 1);
            if (L.item >= total) live = false;
            else t64_begin(m, ws, p, t, L);
        }
        if (__all_sync(0xffffffffu, !live)) break;
        if (!live || L.stage >= 2) continue;
        const int n = L.cell.n;
        const int row = L.mode >= mReviewContinue ? cFinalEvals : cInitEvals;
        bool ok = true;
        if (L.stage == 1) ok = t64_candidate(L);
        int is = kOk;
        if (ok) {
            bool smooth = true;
            is = fp64::stability_provider(m, L.cell, L.next.w, L.lnphi, smooth, nullptr, row);
            if (is == kOk) is = fp64::tpd(L.cell, L.lnphi, L.ref, L.next);
            L.next.smooth = smooth;
        }
        if (L.stage == 0) {
            if (!ok || is != kOk) {
                L.status = fp64::kPropertyFailure;
                L.stage = 2;
                continue;
            }
            t64_copy_point(L.point, L.next, n);
            t64_decide(L);
            continue;
        }
        bool accept = false;
        if (ok && is == kOk) {
            accept = fp64::tpd_negative(L.next, L.tol);
            if (!accept) {
                const double predicted = -L.alpha * L.slope;
                const double guard = L.point.guard + L.next.guard;
                if (predicted <= guard)
                    accept = L.next.value <= L.point.value + guard && L.alpha / L.scale > 0.0 &&
                             L.next.stat < L.point.stat;
                else
                    accept = L.next.value <= L.point.value - 1e-4 * predicted;
            }
        }
        if (accept) {
            t64_copy_point(L.point, L.next, n);
            ++L.iter;
            ++L.cell.counters[cTrialIters];
            t64_decide(L);
        } else if (++L.bt >= 32) {
            L.status = fp64::kLineSearchFailed;
            L.stage = 2;
        } else {
            L.alpha *= 0.5;
        }
    }
}

// ---------------------------------------------------------------------------
// FP64 split attempts.
template <int NM>
struct Split64Lane {
    fp64::Cell<NM> cell;
    fp64::SplitState<NM> point, next;
    double lk[NM], e[NM], num[NM];
    double alpha, slope, scale;
    int64_t c;
    int item, order, iter, bt, stage, status, evals, done;  // done: FP32 iterations already made
};

template <int NM>
__device__ void s64_check(Split64Lane<NM>& L) {
    const int n = L.cell.n;
    const fp64::SplitState<NM>& pt = L.point;
    if (pt.fug <= 1e-11) {  // pt_split.hpp:351-363
        double contrast = 0.0;
        for (int i = 0; i < n; ++i) contrast = fmax(contrast, fabs(pt.lnk[i]));
        if (!(pt.mass_abs <= 1e-12 && pt.mass_rel <= 1e-10)) L.status = fp64::kBalanceFailure;
        else if (pt.beta <= 1e-10 || 1.0 - pt.beta <= 1e-10) L.status = fp64::kPhaseDisappearance;
        else if (contrast <= 1e-7 || pt.z_v - pt.z_l <= 1e-8 * fmax(pt.z_v, pt.z_l)) L.status = fp64::kIndistinguishable;
        else L.status = fp64::kConverged;
        L.stage = 2;
        return;
    }
    if (L.done + L.iter >= 512) {
        L.status = fp64::kAttemptIterationLimit;
        L.stage = 2;
        return;
    }
    L.scale = fmax(1.0, pt.fug / 2.0);
    double h = 0.0, hc = 0.0, first = 0.0, fc = 0.0, second = 0.0, sc = 0.0;
    for (int i = 0; i < n; ++i) {
        if (L.cell.z[i] == 0.0) continue;
        const double x = pt.x[i], y = pt.y[i];
        const double cc = (x / L.cell.z[i]) * y;
        const double d = y - x;
        const double r = pt.res[i];
        kahan_add(d * (d / L.cell.z[i]), h, hc);
        kahan_add(cc * r, first, fc);
        kahan_add((cc * r) * r, second, sc);
    }
    double slope = NAN;
    if (h > 0.0 && isfinite(h) && isfinite(first) && isfinite(second))
        slope = -(pt.beta * (1.0 - pt.beta) * second + (first / h) * first) / L.scale;
    if (!isfinite(slope) || !(slope < 0.0)) {
        L.status = fp64::kAttemptLineSearchFailed;
        L.stage = 2;
        return;
    }
    L.slope = slope;
    L.alpha = 1.0;
    L.bt = 0;
    L.stage = 1;
    for (int i = 0; i < n; ++i) L.lk[i] = pt.lnk[i] + (L.alpha / L.scale) * pt.res[i];
}

template <int NM>
__global__ void __launch_bounds__(64) split64_kernel(const Mixture* __restrict__ mix_g, Workspace ws,
                                                     const double* __restrict__ p, const double* __restrict__ t) {
    __shared__ Mixture m;
    stage_mixture(mix_g, m);
    // the counter can run past the capacity when a cell's block did not fit
    // (that cell went to the fallback); unreserved slots hold -1
    const int total = min(ws.counters[qS64Items], ws.s64_capacity);
    Split64Lane<NM> L;
    L.stage = 3;
    L.item = -1;
    bool live = true;
    for (;;) {
        if (live && L.stage >= 2) {
            if (L.item >= 0 && L.stage == 2) {
                const int n = L.cell.n;
                ws.s64_status[L.item] = static_cast<signed char>(L.status);
                if (L.status == fp64::kConverged) {
                    double* r = ws.s64_state + static_cast<int64_t>(L.item) * S64Stride<NM>();
                    r[0] = L.point.gibbs;
                    r[1] = L.point.guard;
                    r[2] = L.point.fug;
                    r[3] = L.point.beta;
                    r[4] = L.point.z_l;
                    r[5] = L.point.z_v;
                    for (int i = 0; i < n; ++i) {
                        r[8 + 0 * NM + i] = L.point.x[i];
                        r[8 + 1 * NM + i] = L.point.y[i];
                        r[8 + 2 * NM + i] = L.point.lnk[i];
                        r[8 + 3 * NM + i] = L.point.lnphi_l[i];
                        r[8 + 4 * NM + i] = L.point.lnphi_v[i];
                        r[8 + 5 * NM + i] = L.point.common[i];
                    }
                }
                atomicAdd(&ws.counters_out[idx(kFp64EvalRow, ws.ncell, L.c)], L.cell.counters[cSplitEvals]);
                add_total(ws, tE64Split64, L.cell.counters[cSplitEvals]);
            }
            L.item = atomicAdd(&ws.counters[qS64Cursor], 1);
            if (L.item >= total) {
                live = false;
            } else {
                const int code = ws.s64_items[L.item];
                if (code < 0) {
                    // unreserved slot: stay idle this iteration (every lane must
                    // still reach the warp vote below) and fetch again next time
                    L.stage = 3;
                    L.item = -1;
                } else {
                    L.c = code >> 5;
                    L.order = code & kOrderMask;
                    const int done = ws.att_iter[idx(L.order, ws.ncell, L.c)];
                    const bool from_seed =
                        ws.fp64_items || (code & kFromSeed) || done == 0 || done >= ws.continue_limit;
                    L.iter = 0;
                    L.stage = 0;
                    L.evals = 0;
                    L.done = from_seed ? 0 : ws.att_iter[idx(L.order, ws.ncell, L.c)];
                    L.status = fp64::kAttemptPropertyFailure;
                    if (!load_cell64(m, ws, L.c, p, t, L.cell)) {
                        L.stage = 2;
                    } else {
                        for (int i = 0; i < L.cell.n; ++i)
                            L.lk[i] = from_seed ? ws.att_lnk64[idx(L.order * NM + i, ws.ncell, L.c)]
                                                : static_cast<double>(ws.att_lnk[idx(L.order * NM + i, ws.ncell, L.c)]);
                    }
                }
            }
        }
        if (__all_sync(0xffffffffu, !live)) break;
        if (!live || L.stage >= 2) continue;
        const int n = L.cell.n;
        const int st = fp64::split_evaluate(m, L.cell, L.lk, L.next, L.evals, 20000, L.e, L.num);
        if (L.stage == 0) {
            if (st != fp64::kConverged) {
                L.status = st;
                L.stage = 2;
                continue;
            }
            fp64::copy_state(L.point, L.next, n);
            s64_check(L);
            continue;
        }
        bool accept = false;
        if (st == fp64::kConverged) {
            const double predicted = -L.alpha * L.slope;
            const double guard = L.point.guard + L.next.guard;
            if (predicted > guard)
                accept = L.next.gibbs <= L.point.gibbs - 1e-4 * predicted;
            else
                accept = L.next.gibbs <= L.point.gibbs + guard &&
                         (L.next.fug <= 1e-11 || L.point.fug - L.next.fug > 1e-4 * (L.alpha / L.scale) * L.point.fug);
        } else if (st == fp64::kAttemptEvaluationLimit) {
            L.status = st;
            L.stage = 2;
            continue;
        }
        if (accept) {
            fp64::copy_state(L.point, L.next, n);
            ++L.iter;
            ++L.cell.counters[cSplitIters];
            s64_check(L);
        } else if (++L.bt >= 24) {
            L.status = fp64::kAttemptLineSearchFailed;
            L.stage = 2;
        } else {
            L.alpha *= 0.5;
            for (int i = 0; i < n; ++i) L.lk[i] = L.point.lnk[i] + (L.alpha / L.scale) * L.point.res[i];
        }
    }
}


// ---------------------------------------------------------------------------
// Per-cell classification of the FP32 trial outcomes: trials FP32 could not
// decide become FP64 items (continuation from the FP32 end point, or an exact
// re-run when the descent failed or would exhaust the reference's budget).
template <int NM>
__global__ void __launch_bounds__(128) classify_kernel(const Mixture* __restrict__ mix_g, Workspace ws, int review) {
    __shared__ Mixture m;
    stage_mixture(mix_g, m);
    const int cells = ws.counters[qTrialCells];
    const int n = m.n;
    for (int slot = blockIdx.x * blockDim.x + threadIdx.x; slot < cells; slot += gridDim.x * blockDim.x) {
        const int64_t c = ws.trial_cells[slot];
        int active = 0;
        for (int i = 0; i < n; ++i) active += ws.z[idx(i, ws.ncell, c)] > 0.0;
        const int ntr = auto_starts(active) + (review ? 2 : 0);
        bool fp32_negative = false;
        for (int k = 0; k < ntr; ++k) fp32_negative = fp32_negative || ws.tclass[idx(k, ws.ncell, c)] == fp32::tNegative;
        for (int k = 0; k < ntr; ++k) {
            const int raw = ws.tclass[idx(k, ws.ncell, c)];
            if (raw < 0) continue;
            const int cls = raw & (kSlowFlag - 1);
            const bool slow = (raw & kSlowFlag) != 0;
            bool rerun = cls == fp32::tRerun;
            // a long FP32 descent is not continued: its FP64 count from the
            // FP32 end point need not be the reference's from the start
            if (cls == fp32::tMarginal && ws.titer[idx(k, ws.ncell, c)] >= ws.continue_limit) rerun = true;
            if (slow) {
                // Another trial of this test is already negative, so the test is
                // "unstable" whatever this one does; its FP32 end point has a
                // nonnegative TPD (positive, or at a reference composition), so
                // a monotone descent cannot turn it into a witness either.
                if (fp32_negative && (cls == fp32::tPositive || cls == fp32::tTangent)) {
                    ws.tclass[idx(k, ws.ncell, c)] = static_cast<signed char>(cls);
                    atomicAdd(&ws.counters[sSlowSkipped], 1);
                    continue;
                }
                rerun = true;
            } else if (cls != fp32::tMarginal && cls != fp32::tRerun) {
                continue;
            }
            ws.tclass[idx(k, ws.ncell, c)] = static_cast<signed char>(rerun ? fp32::tRerun : fp32::tMarginal);
            const int mode = review ? (rerun ? mReviewRerun : mReviewContinue) : (rerun ? mFeedRerun : mFeedContinue);
            const int item = atomicAdd(&ws.counters[qT64Items], 1);
            ws.t64_items[item] = trial_item(c, k, mode);
            atomicAdd(&ws.counters[review ? (rerun ? sReviewRerun : sReviewContinued)
                                          : (rerun ? sFeedRerun : sFeedContinued)], 1);
        }
    }
}

// Minimum-Gibbs converged FP64 attempt per cell, in attempt order with a
// strict comparison (pt_split.hpp:480-483), then the review set-up.
template <int NM>
__global__ void __launch_bounds__(64) select64_kernel(const Mixture* __restrict__ mix_g, Workspace ws,
                                                      const double* __restrict__ p, const double* __restrict__ t,
                                                      DeviceOutputs out) {
    __shared__ Mixture m;
    stage_mixture(mix_g, m);
    const int cells = ws.counters[qS64Cells];
    const int n = m.n;
    for (int slot = blockIdx.x * blockDim.x + threadIdx.x; slot < cells; slot += gridDim.x * blockDim.x) {
        const int64_t c = ws.s64_cells[slot];
        const int base = ws.s64_base[c], cnt = ws.s64_count[c];
        // a polished pair already in `cand` (attempt order cand_order) competes
        // with the continued attempts: the first attempt of least Gibbs energy
        // in the reference's attempt order wins (pt_split.hpp:459-486)
        const double cand_g = ws.cand_s[idx(4, ws.ncell, c)];
        const int cand_order = isfinite(cand_g) ? static_cast<int>(ws.cand_s[idx(6, ws.ncell, c)]) : -1;
        int best = -1;  // -1 none yet, -2 the polished pair, else the FP64 item
        double best_g = 0.0;
        bool cand_seen = false;
        for (int k = 0; k <= cnt; ++k) {
            // items are queued in attempt order; the polished pair takes its
            // place before the first item of a later attempt
            const int order = k < cnt ? (ws.s64_items[base + k] & kOrderMask) : kMaxAttempts;
            if (cand_order >= 0 && !cand_seen && cand_order < order) {
                cand_seen = true;
                if (best == -1 || cand_g < best_g) {
                    best = -2;
                    best_g = cand_g;
                }
            }
            if (k == cnt) break;
            if (ws.s64_status[base + k] != fp64::kConverged) continue;
            const double g = ws.s64_state[static_cast<int64_t>(base + k) * S64Stride<NM>()];
            if (best == -1 || g < best_g) {
                best = base + k;
                best_g = g;
            }
        }
        const bool cand_wins = best == -2;
        if (cand_wins) {
            fp64::Cell<NM> c64;
            if (!load_cell64(m, ws, c, p, t, c64)) {
                ws.phase[c] = pFallback;
                atomicAdd(&ws.counters[qFallback], 1);
                continue;
            }
            begin_review(ws, c, c64, best_g);
            continue;
        }
        if (best < 0) {
            if (warm_cell(ws, c)) {  // no converged warm attempt: solve the cell cold
                ws.phase[c] = pRedo;
                atomicAdd(&ws.counters[sWarmRedo], 1);
                atomicAdd(&ws.counters[sWarmNoPair], 1);
                continue;
            }
            ws.phase[c] = pIndeterminate;
            write_status_only<NM>(out, ws, c, kIndeterminate, false);
            write_counters<NM>(out, ws, c);
            continue;
        }
        const double* r = ws.s64_state + static_cast<int64_t>(best) * S64Stride<NM>();
        for (int i = 0; i < n; ++i)
            for (int f = 0; f < 6; ++f) ws.cand[idx(f * NM + i, ws.ncell, c)] = r[8 + f * NM + i];
        ws.cand_s[idx(0, ws.ncell, c)] = r[3];
        ws.cand_s[idx(1, ws.ncell, c)] = r[4];
        ws.cand_s[idx(2, ws.ncell, c)] = r[5];
        ws.cand_s[idx(3, ws.ncell, c)] = r[2];
        ws.cand_s[idx(7, ws.ncell, c)] = r[1];
        fp64::Cell<NM> c64;
        if (!load_cell64(m, ws, c, p, t, c64)) {
            ws.phase[c] = pFallback;
            atomicAdd(&ws.counters[qFallback], 1);
            continue;
        }
        begin_review(ws, c, c64, best_g);
    }
}

}  // namespace batched
}  // namespace pr76
