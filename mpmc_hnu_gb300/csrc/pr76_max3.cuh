// Max-3-phase continuation of a phase_set_unstable two-phase answer, in FP64,
// one cell per warp (the reference's PR76 backend path for such cells).
//
//   orchestration        modules/flash/include/mpmc/flash/pr76_three_phase.hpp:328-561
//                        (backend defaults, pr76_pt_flash_backend.hpp:190-206:
//                        no caller hints, 16 automatic attempts, seed fraction 0.1)
//   phase evaluator      pr76_three_phase.hpp:26-106 (lower / upper admissible root)
//   witness root sides   pr76_three_phase.hpp:270-300
//   three-phase iteration modules/flash/include/mpmc/flash/pt_three_phase.hpp:399-676
//   generalized RR       pt_three_phase.hpp:176-340
//   publication          pt_phase_set.hpp:91-150
//
// The two-phase pair of the cell (its ln K from the flash outputs) is
// re-evaluated with the plain form's arithmetic, the final common-tangent
// review is re-run to recover its negative witnesses, and each witness seeds
// three-phase attempts in the reference's order.  Cells reach this path
// rarely (none of the 1M cells of the default bench workload), so the code
// is a direct restatement; its one concession to latency is the warp form of
// the attempts' line search (iterate_three), whose answers are the
// sequential ones.
#pragma once

#include "pr76_fp64.cuh"

namespace pr76 {
namespace fp64 {

enum Max3Status : int { kM3Single = 0, kM3Two = 1, kM3Three = 2, kM3Boundary = 3, kM3Higher = 4, kM3Indeterminate = 5 };

enum ThreeStatus : int {
    kTConverged = 0, kTNoBalance, kTBalanceDegenerate, kTBalanceIterLimit, kTBalanceLineSearch, kTBalanceFailure,
    kTPhaseDisappearance, kTIndistinguishable, kTPropertyFailure, kTIterationLimit, kTEvaluationLimit,
    kTLineSearchFailed
};

// An attempt's evaluation budget (pt_three_phase.hpp:459-565): at most 30000
// phase property evaluations, checked before each one.
constexpr int kThreeEvals = 30000;

template <int NM>
struct ThreeState {  // pt_three_phase.hpp:68-84
    double fraction[3];
    double x[3][NM], lnphi[3][NM];
    double zf[3];
    double lk1[NM], lk2[NM], r1[NM], r2[NM], common[NM];
    double cp_norm, gibbs, guard, rr_residual, mass_abs, mass_rel;
};

template <int NM>
__device__ __forceinline__ void copy_three(ThreeState<NM>& d, const ThreeState<NM>& s, int n) {
    for (int k = 0; k < 3; ++k) {
        d.fraction[k] = s.fraction[k];
        d.zf[k] = s.zf[k];
        for (int i = 0; i < n; ++i) {
            d.x[k][i] = s.x[k][i];
            d.lnphi[k][i] = s.lnphi[k][i];
        }
    }
    for (int i = 0; i < n; ++i) {
        d.lk1[i] = s.lk1[i];
        d.lk2[i] = s.lk2[i];
        d.r1[i] = s.r1[i];
        d.r2[i] = s.r2[i];
        d.common[i] = s.common[i];
    }
    d.cp_norm = s.cp_norm;
    d.gibbs = s.gibbs;
    d.guard = s.guard;
    d.rr_residual = s.rr_residual;
    d.mass_abs = s.mass_abs;
    d.mass_rel = s.mass_rel;
}

__device__ __forceinline__ bool rr3_feasible(double b0, double b1) {  // :176-181
    return isfinite(b0) && isfinite(b1) && b0 >= 0.0 && b1 >= 0.0 && b0 + b1 <= 1.0;
}

// rr3_evaluate, pt_three_phase.hpp:183-233
template <int NM>
__device__ bool rr3_evaluate(const Cell<NM>& c, const double* lk1, const double* lk2, double b0, double b1,
                             double comp[3][NM], double res[2], double jac[3]) {
    if (!rr3_feasible(b0, b1)) return false;
    const int n = c.n;
    const double beta0 = 1.0 - b0 - b1;
    double f0 = 0.0, c0 = 0.0, f1 = 0.0, c1 = 0.0, j00 = 0.0, k00 = 0.0, j01 = 0.0, k01 = 0.0, j11 = 0.0,
           k11 = 0.0;
    for (int i = 0; i < n; ++i) {
        comp[0][i] = comp[1][i] = comp[2][i] = 0.0;
        const double z = c.z[i];
        if (z == 0.0) continue;
        const double shift = fmax(fmax(0.0, lk1[i]), lk2[i]);
        const double e0 = exp(-shift), e1 = exp(lk1[i] - shift), e2 = exp(lk2[i] - shift);
        const double den = beta0 * e0 + b0 * e1 + b1 * e2;
        if (!isfinite(den) || !(den > 0.0)) return false;
        const double x0 = z * e0 / den, x1 = z * e1 / den, x2 = z * e2 / den;
        if (!isfinite(x0) || !isfinite(x1) || !isfinite(x2) || !(x0 > 0.0) || !(x1 > 0.0) || !(x2 > 0.0))
            return false;
        comp[0][i] = x0;
        comp[1][i] = x1;
        comp[2][i] = x2;
        const double d1 = x1 - x0, d2 = x2 - x0;
        kahan_add(d1, f0, c0);
        kahan_add(d2, f1, c1);
        kahan_add(-(d1 * d1) / z, j00, k00);
        kahan_add(-(d1 * d2) / z, j01, k01);
        kahan_add(-(d2 * d2) / z, j11, k11);
    }
    res[0] = f0;
    res[1] = f1;
    jac[0] = j00;
    jac[1] = j01;
    jac[2] = j11;
    return true;
}

// solve_generalized_rr3, pt_three_phase.hpp:235-340.  On success the state's
// fractions, normalised compositions, residual and balance errors are set.
template <int NM>
__device__ MPMC_FP64_CALL int solve_rr3(const Cell<NM>& c, const double* lk1, const double* lk2, const double init[2],
                         ThreeState<NM>& st, double cand[3][NM]) {
    const int n = c.n;
    if (!rr3_feasible(init[0], init[1])) return kTNoBalance;
    for (int i = 0; i < n; ++i)
        if (!isfinite(lk1[i]) || !isfinite(lk2[i])) return kTNoBalance;
    double beta[2] = {init[0], init[1]};
    double res[2], jac[3], nres[2], njac[3];
    double norm_at_success = 0.0;
    for (int iteration = 0;; ++iteration) {
        if (!rr3_evaluate(c, lk1, lk2, beta[0], beta[1], st.x, res, jac)) return kTNoBalance;
        const double norm = fmax(fabs(res[0]), fabs(res[1]));
        if (!isfinite(norm)) return kTNoBalance;
        if (norm <= 2e-13) {
            norm_at_success = norm;
            break;
        }
        if (iteration >= 192) return kTBalanceIterLimit;
        const double det = jac[0] * jac[2] - jac[1] * jac[1];
        const double det_scale = fabs(jac[0] * jac[2]) + fabs(jac[1] * jac[1]) + 1.0;
        if (!isfinite(det) || fabs(det) <= 256.0 * kEps * det_scale) return kTBalanceDegenerate;
        const double step0 = (-res[0] * jac[2] + jac[1] * res[1]) / det;
        const double step1 = (jac[1] * res[0] - jac[0] * res[1]) / det;
        if (!isfinite(step0) || !isfinite(step1)) return kTNoBalance;
        bool accepted = false;
        double alpha = 1.0;
        for (int bt = 0; bt < 48; ++bt, alpha *= 0.5) {
            const double b0 = beta[0] + alpha * step0, b1 = beta[1] + alpha * step1;
            if (!rr3_feasible(b0, b1)) continue;
            if (!rr3_evaluate(c, lk1, lk2, b0, b1, cand, nres, njac)) continue;
            const double next_norm = fmax(fabs(nres[0]), fabs(nres[1]));
            if (!isfinite(next_norm)) continue;
            if (next_norm < norm || next_norm <= 2e-13) {
                beta[0] = b0;
                beta[1] = b1;
                accepted = true;
                break;
            }
        }
        if (!accepted) return kTBalanceLineSearch;
    }
    if (!rr3_evaluate(c, lk1, lk2, beta[0], beta[1], st.x, res, jac)) return kTNoBalance;
    for (int k = 0; k < 3; ++k) {
        double sum = 0.0, cs = 0.0;
        for (int i = 0; i < n; ++i) kahan_add(st.x[k][i], sum, cs);
        if (!isfinite(sum) || !(sum > 0.0)) return kTNoBalance;
        for (int i = 0; i < n; ++i) st.x[k][i] /= sum;
    }
    st.fraction[0] = 1.0 - beta[0] - beta[1];
    st.fraction[1] = beta[0];
    st.fraction[2] = beta[1];
    const double fr[3] = {st.fraction[0], beta[0], beta[1]};
    double abs_err = 0.0, rel_err = 0.0;
    for (int i = 0; i < n; ++i) {
        const double recovered = fr[0] * st.x[0][i] + fr[1] * st.x[1][i] + fr[2] * st.x[2][i];
        const double err = fabs(recovered - c.z[i]);
        abs_err = fmax(abs_err, err);
        if (c.z[i] > 0.0)
            rel_err = fmax(rel_err, err / c.z[i]);
        else if (recovered != 0.0)
            rel_err = INFINITY;
    }
    st.rr_residual = norm_at_success;
    st.mass_abs = abs_err;
    st.mass_rel = rel_err;
    return kTConverged;
}

// The three-phase state at (ln K1, ln K2) (pt_three_phase.hpp:459-565):
// kTConverged for "evaluated", else the step-error or property status.
template <int NM>
__device__ MPMC_FP64_CALL int three_state(const Mixture& m, Cell<NM>& c, const double* lk1, const double* lk2, const double seed[2],
                           const bool upper[3], ThreeState<NM>& st, double scratch[3][NM], int& evals) {
    const int n = c.n;
    const int b = solve_rr3(c, lk1, lk2, seed, st, scratch);
    if (b != kTConverged) return b;
    for (int k = 0; k < 3; ++k) {
        if (evals >= kThreeEvals) return kTEvaluationLimit;
        ++evals;
        int branch;
        if (role_provider(m, c, st.x[k], upper[k], st.lnphi[k], st.zf[k], branch) != kOk) return kTPropertyFailure;
        for (int i = 0; i < n; ++i)
            if (!isfinite(st.lnphi[k][i])) return kTPropertyFailure;
    }
    st.cp_norm = 0.0;
    double gibbs = 0.0, gc = 0.0, magnitude = 1.0, mc = 0.0;
    for (int i = 0; i < n; ++i) {
        st.lk1[i] = st.lk2[i] = st.r1[i] = st.r2[i] = st.common[i] = 0.0;
        if (c.z[i] == 0.0) continue;
        const double l0 = log(st.x[0][i]), l1 = log(st.x[1][i]), l2 = log(st.x[2][i]);
        const double mu0 = l0 + st.lnphi[0][i], mu1 = l1 + st.lnphi[1][i], mu2 = l2 + st.lnphi[2][i];
        st.lk1[i] = l1 - l0;
        st.lk2[i] = l2 - l0;
        st.r1[i] = mu0 - mu1;
        st.r2[i] = mu0 - mu2;
        st.common[i] = (mu0 + mu1 + mu2) / 3.0;
        st.cp_norm = fmax(fmax(st.cp_norm, fabs(st.r1[i])), fabs(st.r2[i]));
        for (int k = 0; k < 3; ++k) {
            const double lx = log(st.x[k][i]);
            const double mu = lx + st.lnphi[k][i];
            kahan_add(st.fraction[k] * st.x[k][i] * mu, gibbs, gc);
            kahan_add(st.fraction[k] * st.x[k][i] * (fabs(lx) + fabs(st.lnphi[k][i])), magnitude, mc);
        }
    }
    st.gibbs = gibbs;
    st.guard = 256.0 * kEps * magnitude;
    if (!isfinite(st.cp_norm) || !isfinite(st.gibbs) || !isfinite(st.guard)) return kTPropertyFailure;
    return kTConverged;
}

// pt_three_phase_log_distance, :342-366
template <int NM>
__device__ double log_distance(const Cell<NM>& c, const double* a, const double* b) {
    double d = 0.0;
    for (int i = 0; i < c.n; ++i) {
        if (c.z[i] == 0.0) {
            if (a[i] != 0.0 || b[i] != 0.0) return INFINITY;
            continue;
        }
        if (!(a[i] > 0.0) || !(b[i] > 0.0)) return INFINITY;
        const double v = fabs(log(a[i]) - log(b[i]));
        if (!isfinite(v)) return INFINITY;
        d = fmax(d, v);
    }
    return d;
}

template <int NM>
struct ThreeScratch {
    ThreeState<NM> point, next;
    double lk1[NM], lk2[NM], nk1[NM], nk2[NM], rr[3][NM];
};

// Backtracking trial `bt` of the line search (alpha = 0.5^bt, exact) into
// s.next with its own evaluation count `used` (0-3; the shared budget is
// applied by line_walk).  Returns the state's status and sets `ok` when the
// trial passes the progress and Gibbs tests (pt_three_phase.hpp:600-650).
template <int NM>
__device__ __forceinline__ int line_trial(const Mixture& m, Cell<NM>& c, const bool upper[3], ThreeScratch<NM>& s,
                                          double scale, int bt, int& used, bool& ok) {
    const int n = c.n;
    const ThreeState<NM>& pt = s.point;
    const double alpha = ldexp(1.0, -bt);
    for (int i = 0; i < n; ++i) {
        s.nk1[i] = pt.lk1[i] + (alpha / scale) * pt.r1[i];
        s.nk2[i] = pt.lk2[i] + (alpha / scale) * pt.r2[i];
    }
    const double seed[2] = {pt.fraction[1], pt.fraction[2]};
    used = 0;
    ok = false;
    const int st = three_state(m, c, s.nk1, s.nk2, seed, upper, s.next, s.rr, used);
    if (st != kTConverged) return st;  // rejected evaluation
    const double required = 1e-4 * (alpha / scale) * pt.cp_norm;
    const bool progress = s.next.cp_norm <= 1e-11 || pt.cp_norm - s.next.cp_norm > required;
    const bool gibbs_ok = s.next.gibbs <= pt.gibbs + pt.guard + s.next.guard;
    ok = progress && gibbs_ok;
    return st;
}

enum LineWalk : int { kWalkNext = 0, kWalkAccept, kWalkLimit };

// The in-order line search's bookkeeping for one trial that used `used`
// evaluations: the reference checks the budget before each evaluation, so the
// trial runs out of it when its last evaluation would start at the limit.
__device__ __forceinline__ int line_walk(int& evals, int used, int st, bool ok) {
    if (used > 0 && evals + used - 1 >= kThreeEvals) return kWalkLimit;
    evals += used;
    return st == kTConverged && ok ? kWalkAccept : kWalkNext;
}

// The warp form of the line search builds for the device, and for the host
// under a warp emulation that provides __shfl_sync, __activemask and a
// per-lane threadIdx (a test build that runs the 32 lanes as threads).
#if defined(__CUDA_ARCH__) || defined(MPMC_WARP_EMULATION)
#define MPMC_MAX3_WARP 1
#endif

#ifdef MPMC_MAX3_WARP
// Every lane of the warp takes lane `src`'s state (the fields copy_three copies).
template <int NM>
__device__ __forceinline__ void shfl_three(ThreeState<NM>& d, const ThreeState<NM>& s, int n, int src) {
    constexpr unsigned kAll = 0xffffffffu;
    for (int k = 0; k < 3; ++k) {
        d.fraction[k] = __shfl_sync(kAll, s.fraction[k], src);
        d.zf[k] = __shfl_sync(kAll, s.zf[k], src);
        for (int i = 0; i < n; ++i) {
            d.x[k][i] = __shfl_sync(kAll, s.x[k][i], src);
            d.lnphi[k][i] = __shfl_sync(kAll, s.lnphi[k][i], src);
        }
    }
    for (int i = 0; i < n; ++i) {
        d.lk1[i] = __shfl_sync(kAll, s.lk1[i], src);
        d.lk2[i] = __shfl_sync(kAll, s.lk2[i], src);
        d.r1[i] = __shfl_sync(kAll, s.r1[i], src);
        d.r2[i] = __shfl_sync(kAll, s.r2[i], src);
        d.common[i] = __shfl_sync(kAll, s.common[i], src);
    }
    d.cp_norm = __shfl_sync(kAll, s.cp_norm, src);
    d.gibbs = __shfl_sync(kAll, s.gibbs, src);
    d.guard = __shfl_sync(kAll, s.guard, src);
    d.rr_residual = __shfl_sync(kAll, s.rr_residual, src);
    d.mass_abs = __shfl_sync(kAll, s.mass_abs, src);
    d.mass_rel = __shfl_sync(kAll, s.mass_rel, src);
}
#endif

// iterate_pt_three_phase, :399-676, on the cell's current (normalised) feed.
// `point` holds the last state; `disappearing` the phase that left.
//
// warp = true (device only): the 32 lanes of the warp run the same cell with
// the same state, and the line search's 32 backtracking trials run at once,
// trial bt on lane bt.  The in-order walk over their outcomes then picks the
// trial (and spends the evaluations) the reference's sequential loop would,
// and every lane takes that trial's state.  The answer is the sequential one;
// an iteration that backtracks k times costs one trial's latency, not k.
template <int NM>
__device__ MPMC_FP64_CALL int iterate_three(const Mixture& m, Cell<NM>& c, const double frac0[2], const bool upper[3],
                             ThreeScratch<NM>& s, int& disappearing, bool warp = false) {
    const int n = c.n;
    int evals = 0;
    {
        const int st = three_state(m, c, s.lk1, s.lk2, frac0, upper, s.point, s.rr, evals);
        if (st != kTConverged) return st;
    }
    int iterations = 0;
    for (;;) {
        ThreeState<NM>& pt = s.point;
        if (pt.cp_norm <= 1e-11) {
            if (pt.rr_residual > 2e-13 || pt.mass_abs > 1e-12 || pt.mass_rel > 1e-10) return kTBalanceFailure;
            for (int k = 0; k < 3; ++k)
                if (pt.fraction[k] <= 1e-10) {
                    disappearing = k;
                    return kTPhaseDisappearance;
                }
            const double d01 = log_distance(c, pt.x[0], pt.x[1]), d02 = log_distance(c, pt.x[0], pt.x[2]),
                         d12 = log_distance(c, pt.x[1], pt.x[2]);
            if (!(d01 > 1e-7) || !(d02 > 1e-7) || !(d12 > 1e-7)) return kTIndistinguishable;
            return kTConverged;
        }
        if (iterations >= 512) return kTIterationLimit;
        const double scale = fmax(1.0, pt.cp_norm / 2.0);
        int walk = kWalkNext;
#ifdef MPMC_MAX3_WARP
        // The lanes agree at every step, so they normally arrive here converged.
        // When the 32 are not all converged here, each lane searches in order on
        // its own below (the same answer, with no exchange between lanes).
        constexpr unsigned kAll = 0xffffffffu;
        if (warp && __activemask() == kAll) {
            int used;
            bool ok;
            const int st = line_trial(m, c, upper, s, scale, static_cast<int>(threadIdx.x & 31u), used, ok);
            int winner = 0;
            for (int bt = 0; bt < 32 && walk == kWalkNext; ++bt) {
                walk = line_walk(evals, __shfl_sync(kAll, used, bt), __shfl_sync(kAll, st, bt),
                                 __shfl_sync(kAll, static_cast<int>(ok), bt) != 0);
                winner = bt;
            }
            if (walk == kWalkLimit) return kTEvaluationLimit;
            if (walk != kWalkAccept) return kTLineSearchFailed;
            shfl_three(s.point, s.next, n, winner);
            ++iterations;
            continue;
        }
#endif
        for (int bt = 0; bt < 32 && walk == kWalkNext; ++bt) {
            int used;
            bool ok;
            const int st = line_trial(m, c, upper, s, scale, bt, used, ok);
            walk = line_walk(evals, used, st, ok);
        }
        if (walk == kWalkLimit) return kTEvaluationLimit;
        if (walk != kWalkAccept) return kTLineSearchFailed;
        copy_three(s.point, s.next, n);
        ++iterations;
    }
}

// pr76_witness_root_sides, pr76_three_phase.hpp:270-300: the root sides a
// witness at composition w (stability branch `branch`) may follow.
template <int NM>
__device__ int witness_sides(const Mixture& m, Cell<NM>& c, const double* w, int branch, bool sides[2]) {
    double amix, bmix, A, B;
    if (!mix(m, c, w, amix, bmix) || !coefficients(c.p, c.t, amix, bmix, A, B)) return 0;
    RootSet rs;
    int it = 0;
    solve_roots(A, B, rs, it, c.newton);
    if (rs.status != kRootSuccess) return 0;
    int adm[3], na = 0;
    bool found = false;
    for (int k = 0; k < rs.count; ++k)
        if (rs.r[k].slope_sign > 0) {
            adm[na++] = k;
            found = found || k == branch;
        }
    if (na == 0 || !found) return 0;
    if (na == 1) {
        sides[0] = false;
        sides[1] = true;
        return 2;
    }
    if (branch == adm[0]) {
        sides[0] = false;
        return 1;
    }
    if (branch == adm[na - 1]) {
        sides[0] = true;
        return 1;
    }
    return 0;
}

// ln(a_i / b_i) on the feed support, pr76_three_phase.hpp:246-268
template <int NM>
__device__ bool log_ratio(const Cell<NM>& c, const double* a, const double* b, double* out) {
    for (int i = 0; i < c.n; ++i) {
        out[i] = 0.0;
        if (c.z[i] == 0.0) {
            if (a[i] != 0.0 || b[i] != 0.0) return false;
            continue;
        }
        if (!(a[i] > 0.0) || !(b[i] > 0.0)) return false;
        out[i] = log(a[i]) - log(b[i]);
        if (!isfinite(out[i])) return false;
    }
    return true;
}

template <int NM>
struct Max3Scratch {
    Scratch<NM> w;             // trials and splits (the base review, the neighbor solve)
    ThreeScratch<NM> t;
    TpdPoint<NM> witness;      // the current base-review trial
    double z1[NM];             // the once-normalised feed
    double imposed[NM], direction[NM], lnphi[NM];
    double fr_x[NM], fr_y[NM];  // the base pair
    double beta_v;
};

struct Max3Result {
    int status;      // Max3Status, -1 invalid
    bool has_three;  // s.t.point holds the accepted three-phase set
    bool has_pair;   // a two-phase pair to publish (neighbor: s.w.best; higher: the base pair)
};

// Final three-phase review (pr76_three_phase.hpp:420-441: test_pt_stability_against
// with the common log activity, tolerance + |r|, starts = the three phases).
// Returns kUnstable-like codes: 0 unstable, 1 no instability, 2 indeterminate,
// -1 a domain error.
template <int NM>
__device__ MPMC_FP64_CALL int three_review(const Mixture& m, Cell<NM>& c, Max3Scratch<NM>& s) {
    const int n = c.n;
    const ThreeState<NM>& cand = s.t.point;
    // the feed of test_pt_stability_against: the once-normalised feed normalised again
    if (!normalise_feed(c, s.z1)) return -1;
    for (int k = 0; k < 3; ++k)
        if (!start_matches_feed(c, cand.x[k])) return -1;
    for (int i = 0; i < n; ++i) s.imposed[i] = c.z[i] > 0.0 ? cand.common[i] - c.lz[i] : 0.0;
    for (int i = 0; i < n; ++i)
        if (!isfinite(s.imposed[i])) return 2;  // property failure of every trial
    int active = 0;
    for (int i = 0; i < n; ++i) active += c.z[i] > 0.0;
    const int n_auto = active == 1 ? 1 : active + 2;
    const double* extra[3] = {cand.x[0], cand.x[1], cand.x[2]};
    StabilityOptions fo{1e-10 + cand.cp_norm, cFinalEvals};
    bool negative = false, stationary = true;
    int evals = 0;
    for (int k = 0; k < n_auto + 3; ++k) {
        make_start(c, k, active, extra, n_auto, s.w.point.w);
        const int ts = run_trial(m, c, s.imposed, fo, s.w.point, s.w.next, s.direction, s.lnphi, evals);
        if (ts < 0) return -1;
        stationary = stationary && ts == kStationary;
        negative = negative || ts == kNegativeTpd;
    }
    return negative ? 0 : (stationary ? 1 : 2);
}

// solve_pr76_pt_max3 from a phase_set_unstable two-phase answer with ln K `lnk`.
// `feed` is the raw feed; c.p, c.t and the temperature constants are set.
// Caller starts (pr76_three_phase.hpp:328-358): `hints` (n_hints <= 3) are
// the extra final-review starts the base solve ran with, ahead of the pair,
// and `three_hint` (3 n compositions, then the fractions of phases 1 and 2)
// is a three-phase start whose attempts run first, one per combination of
// root sides (:457-486), with their own quota of 16.  `opt` are the caller's
// two-phase options, which the fresh two-phase neighbour of a phase
// disappearance runs with (:413-415).  `warp`: the whole warp runs this cell
// (every lane with its own copy of the same state), and the attempts' line
// searches run their backtracking trials on the lanes (iterate_three).
// `newton_roots`: the cubic and the Rachford-Rice equation by bracketed Newton
// with the reference's stopping width, as the flash's FP64 items solve them,
// instead of the reference's bisection (fewer FP64 instructions per phase
// evaluation; the statuses of every recorded cell are unchanged).
template <int NM>
__device__ Max3Result max3_cell(const Mixture& m, Cell<NM>& c, const double* feed, const double* lnk,
                                Max3Scratch<NM>& s, const double* const* hints = nullptr, int n_hints = 0,
                                const double* three_hint = nullptr, const SolveOptions& opt = SolveOptions{},
                                bool warp = false, bool newton_roots = false) {
    const int n = c.n;
    Max3Result r{kM3Indeterminate, false, false};
    c.newton = newton_roots;  // false: the reference's bisection roots and RR
    if (!normalise_feed(c, feed)) {
        r.status = -1;
        return r;
    }
    for (int i = 0; i < n; ++i) s.z1[i] = c.z[i];
    // the base pair at its ln K (the state the base review was run on)
    int evals = 0;
    if (split_evaluate(m, c, lnk, s.w.best, evals, 1 << 30, s.w.e, s.w.num) != kConverged) return r;
    for (int i = 0; i < n; ++i) {
        s.fr_x[i] = s.w.best.x[i];
        s.fr_y[i] = s.w.best.y[i];
    }
    s.beta_v = s.w.best.beta;
    const double base_fug = s.w.best.fug;
    for (int i = 0; i < n; ++i) s.lnphi[i] = s.w.best.common[i];  // keep the pair's common log activity
    // the base review's feed: the once-normalised feed normalised again
    if (!normalise_feed(c, s.z1)) {
        r.status = -1;
        return r;
    }
    int active = 0;
    for (int i = 0; i < n; ++i) active += c.z[i] > 0.0;
    const int n_auto = active == 1 ? 1 : active + 2;
    double common[NM];
    for (int i = 0; i < n; ++i) common[i] = s.lnphi[i];
    const StabilityOptions fo{1e-10 + 0.5 * base_fug, cFinalEvals};
    if (n_hints > 3) n_hints = 3;
    const double* base_extra[5];
    int n_extra = 0;
    for (int k = 0; k < n_hints; ++k) base_extra[n_extra++] = hints[k];
    base_extra[n_extra++] = s.fr_x;
    base_extra[n_extra++] = s.fr_y;
    bool saw_higher = false, saw_boundary = false;
    // One three-phase attempt from the seeds in s.t.lk1 / lk2, run_attempt of
    // pr76_three_phase.hpp:379-455: true when it settles the cell (r is set).
    auto attempt = [&](const double fr[2], const bool upper[3]) -> bool {
        // the attempt iterates on the once-normalised feed normalised again
        if (!normalise_feed(c, s.z1)) {
            r.status = -1;
            return true;
        }
        int disappearing = -1;
        const int st = iterate_three(m, c, fr, upper, s.t, disappearing, warp);
        if (st == kTPhaseDisappearance) {
            saw_boundary = true;
            const double* starts[2];
            int ns2 = 0;
            for (int ph = 0; ph < 3; ++ph)
                if (ph != disappearing) starts[ns2++] = s.t.point.x[ph];
            if (ns2 == 2) {
                // fresh two-phase solve with the surviving phases as initial and final starts
                CellResult<NM> nb;
                double nfeed[NM];
                for (int i = 0; i < n; ++i) nfeed[i] = s.z1[i];
                // the surviving compositions are copied out: solve_cell reuses s.w
                double keep[2][NM];
                for (int i = 0; i < n; ++i) {
                    keep[0][i] = starts[0][i];
                    keep[1][i] = starts[1][i];
                }
                const double* kst[2] = {keep[0], keep[1]};
                // with the caller's two-phase options (pr76_three_phase.hpp:413-415)
                const int nst = solve_cell(m, c, nfeed, s.w, nb, kst, 2, kst, 2, opt);
                c.newton = newton_roots;
                if (nst == kTwoPhase) {
                    r.status = kM3Two;
                    r.has_pair = true;  // s.w.best
                    return true;
                }
            }
            // back to the base review's state for the next trials
            if (!normalise_feed(c, s.z1)) {
                r.status = -1;
                return true;
            }
            // solve_cell changed the temperature constants only by recomputing them
        } else if (st == kTConverged) {
            const int fin = three_review(m, c, s);
            if (fin < 0) {
                r.status = -1;
                return true;
            }
            if (fin == 1) {
                r.status = kM3Three;
                r.has_three = true;
                return true;
            }
            if (fin == 0) saw_higher = true;
        }
        // the base review continues on its own feed
        if (!normalise_feed(c, s.z1)) {
            r.status = -1;
            return true;
        }
        return false;
    };
    // the caller's three-phase start first, every combination of root sides
    if (three_hint != nullptr) {
        const double* x0 = three_hint;
        const double* x1 = three_hint + n;
        const double* x2 = three_hint + 2 * n;
        const double fr[2] = {three_hint[3 * n], three_hint[3 * n + 1]};
        if (log_ratio(c, x1, x0, s.t.lk1) && log_ratio(c, x2, x0, s.t.lk2)) {
            for (int side = 0; side < 8; ++side) {
                const bool upper[3] = {(side & 4) != 0, (side & 2) != 0, (side & 1) != 0};
                // the seeds stay in s.t.lk1 / lk2: iterate_three only reads them
                if (attempt(fr, upper)) return r;
            }
        }
    }
    int attempts = 0;
    bool limit = false;
    int review_evals = 0;
    const bool have_lk1 = log_ratio(c, s.fr_y, s.fr_x, s.t.lk1);
    for (int k = 0; k < n_auto + n_extra && !limit; ++k) {
        // base review trial k (pt_split.hpp:509-510), as the reference ran it
        for (int i = 0; i < n; ++i) s.imposed[i] = c.z[i] > 0.0 ? common[i] - c.lz[i] : 0.0;
        make_start(c, k, active, base_extra, n_auto, s.witness.w);
        const int ts = run_trial(m, c, s.imposed, fo, s.witness, s.w.next, s.direction, s.lnphi, review_evals);
        if (ts < 0) {
            r.status = -1;
            return r;
        }
        if (ts != kNegativeTpd || !have_lk1) continue;
        if (!log_ratio(c, s.witness.w, s.fr_x, s.t.lk2)) continue;
        bool sides[2];
        const int ns = witness_sides(m, c, s.witness.w, s.witness.branch, sides);
        for (int q = 0; q < ns; ++q) {
            if (attempts >= 16) {
                limit = true;
                break;
            }
            ++attempts;
            const double fr[2] = {(1.0 - 0.1) * s.beta_v, 0.1};
            const bool upper[3] = {false, true, sides[q]};
            // the seeds: source ln K1 = ln(y/x), ln K2 = ln(witness/x) (kept in s.t.lk1 / lk2)
            if (attempt(fr, upper)) return r;
        }
    }
    r.status = saw_higher ? kM3Higher : (saw_boundary ? kM3Boundary : kM3Indeterminate);
    r.has_pair = r.status == kM3Higher;
    return r;
}

}  // namespace fp64
}  // namespace pr76
