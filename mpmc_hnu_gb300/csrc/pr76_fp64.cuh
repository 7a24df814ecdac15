// PR76 two-phase PT flash in FP64, one cell per thread ("plain" form).
//
// The device restatement of MPMC_HNU's reference algorithm:
//   feed TPD stability   modules/flash/include/mpmc/flash/pt_stability.hpp:228-461
//   stability provider   modules/flash/include/mpmc/flash/pr76_stability.hpp:36-119
//   role provider        modules/flash/include/mpmc/flash/pr76_split.hpp:38-84
//   cubic roots          modules/thermodynamics/include/mpmc/thermodynamics/pr76_roots.hpp:77-173
//   ln phi               modules/thermodynamics/include/mpmc/thermodynamics/pr76_phase.hpp:193-258
//   Rachford-Rice        modules/flash/include/mpmc/flash/rachford_rice.hpp:70-147
//   ln K split (SSI)     modules/flash/include/mpmc/flash/pt_split.hpp:275-408
//   orchestration        modules/flash/include/mpmc/flash/pt_split.hpp:415-525
// with the same starts, tolerances, budgets and acceptance rules.  GPU-side
// changes that keep every iterate's arithmetic identical in exact arithmetic:
//  * a_i(T), sqrt(a_i) and the T-independent mixture data are formed once per
//    cell/block instead of once per property evaluation;
//  * exp(-|ln K|) and the expm1 numerators of the RR residual are formed once
//    per RR solve instead of once per bisection step;
//  * ln(w_i) of the current TPD point is kept from its evaluation and reused
//    by the line search;
//  * the split attempts of a negative TPD witness run as soon as that trial
//    ends, so one witness is stored at a time; attempts are still taken in
//    trial order with the same attempt and evaluation budgets, and no trial
//    depends on an attempt, so the selected pair is the same.
// Rounding differs from a CPU build only through FMA contraction and the
// device libm (log/exp/log1p/expm1 within 1-2 ulp).
#pragma once

#include "pr76_common.cuh"

// Call discipline of the large routines below: inlined by default; a
// translation unit may define MPMC_FP64_CALL as __noinline__ (the rare
// max-3-phase path) to keep its one kernel small and its build short.
#ifndef MPMC_FP64_CALL
#define MPMC_FP64_CALL
#endif

namespace pr76 {
namespace fp64 {

// ---------------------------------------------------------------------------
// Cell context: per-cell constants and scratch.
template <int NM>
struct Cell {
    int n;
    bool newton;              // bracketed Newton for the cubic and RR (mixed form's FP64 stages)
    double p, t;
    double a[NM], root[NM];   // a_i(T), sqrt(a_i(T))
    double z[NM], lz[NM];     // normalised feed and its log (0 where z_i = 0)
    double sums[NM];          // mixing row sums s_i = sum_j x_j a_ij
    double lnphi[2][NM];      // stability-provider scratch (<= 2 admissible roots)
    int counters[cCount];
};

// a_i(T) and sqrt(a_i), pr76_pure.hpp:146-165, pr76_mixture.hpp:172-188.
template <int NM>
__device__ bool temp_setup(const Mixture& m, Cell<NM>& c) {
    const double st = sqrt(c.t);
    for (int i = 0; i < c.n; ++i) {
        const double reduced_root = st / m.sqrt_tc[i];
        const double bracket = 1.0 + m.kappa[i] * (1.0 - reduced_root);
        const double attraction = (bracket * m.ac[i]) * bracket;
        if (!isfinite(attraction) || (attraction == 0.0 && bracket != 0.0)) return false;
        if (c.n > 1 && !(attraction > 0.0)) return false;
        c.a[i] = attraction;
        c.root[i] = sqrt(attraction);
    }
    return true;
}

// Mixing with row sums, pr76_mixture.hpp:170-218.
template <int NM>
__device__ bool mix(const Mixture& m, Cell<NM>& c, const double* x, double& amix, double& bmix) {
    const int n = c.n;
    double attraction = 0.0, covolume = 0.0;
    for (int i = 0; i < n; ++i) {
        attraction += (x[i] * c.a[i]) * x[i];
        covolume += x[i] * m.b[i];
        c.sums[i] = x[i] * c.a[i];
    }
    for (int i = 0; i < n; ++i) {
        const double xr_i = x[i] * c.root[i];
        const double r_i = c.root[i];
        const double x_i = x[i];
        double s_i = c.sums[i];
        for (int j = i + 1; j < n; ++j) {
            const double f = m.factor[i * n + j];
            const double cross = (xr_i * (x[j] * c.root[j])) * f;
            attraction += cross;
            attraction += cross;
            const double aij = (r_i * f) * c.root[j];
            s_i += x[j] * aij;
            c.sums[j] += x_i * aij;
        }
        c.sums[i] = s_i;
    }
    amix = attraction;
    bmix = covolume;
    if (!isfinite(attraction) || !isfinite(covolume) || !(covolume > 0.0)) return false;
    for (int i = 0; i < n; ++i)
        if (!isfinite(c.sums[i])) return false;
    return true;
}

// Reduced coefficients A, B, pr76_phase.hpp:175-191.
__device__ __forceinline__ bool coefficients(double p, double t, double amix, double bmix, double& A,
                                             double& B) {
    const double rt = kR * t;
    if (!isfinite(rt) || !(rt > 0.0)) return false;
    const double prt = p / rt;
    A = (amix / rt) * prt;
    B = bmix * prt;
    return isfinite(A) && isfinite(B) && B > 0.0 && !(A == 0.0 && amix != 0.0);
}

// ---------------------------------------------------------------------------
// Cubic roots by bisection per monotone interval, pr76_roots.hpp:77-173.
enum RootStatus : int { kRootSuccess = 0, kRootNearMultiple, kRootIterLimit, kRootUnrepresentable };
struct Root {
    double z, free_volume;
    bool derivative_valid;
    int slope_sign;
};
struct RootSet {
    Root r[3];
    int count;
    double scale;
    int status;
};
struct Cubic {
    double c2, c1, c0;
};
__device__ __forceinline__ double poly(double y, const Cubic& c) {
    return fma(fma(y + c.c2, y, c.c1), y, c.c0);
}
__device__ __forceinline__ double poly_scale(double y, const Cubic& c) {
    return ((fabs(y) + fabs(c.c2)) * fabs(y) + fabs(c.c1)) * fabs(y) + fabs(c.c0);
}

// `zhint` (nhint values): roots Z of a nearby evaluation.  Bracketed Newton
// on an interval starts from a hint inside it instead of its midpoint; the
// bracket, the bisection fallback and the stopping test are unchanged.
__device__ inline void solve_roots(double a, double b, RootSet& rs, int& iterations, bool newton = false,
                                   const double* zhint = nullptr, int nhint = 0) {
    rs.count = 0;
    rs.status = kRootUnrepresentable;
    rs.scale = 1.0;
    if (!isfinite(a) || !isfinite(b) || !(b > 0.0)) return;
    rs.scale = fmax(fmax(1.0, b), sqrt(fabs(a)));
    const double bs = b / rs.scale;
    const double inv = 1.0 / rs.scale;
    Cubic c;
    c.c2 = 4.0 * bs - inv;
    c.c1 = (a / rs.scale) / rs.scale + 2.0 * bs * bs - 4.0 * bs * inv;
    c.c0 = ((-2.0 * bs) * bs) * inv;
    if (!isfinite(c.c2) || !isfinite(c.c1) || !isfinite(c.c0) || !(c.c0 < 0.0)) return;
    const double upper = 1.0 + fmax(fmax(fabs(c.c2), fabs(c.c1)), fabs(c.c0));
    double ep[4] = {0.0, 0.0, 0.0, 0.0};
    int ne = 1;
    const double disc = fma(c.c2, c.c2, -3.0 * c.c1);
    if (disc > 0.0) {
        const double q = -c.c2 - copysign(sqrt(disc), c.c2);
        double s0 = q / 3.0, s1 = c.c1 / q;
        if (s1 < s0) {
            const double tmp = s0;
            s0 = s1;
            s1 = tmp;
        }
        const double st[2] = {s0, s1};
        for (int k = 0; k < 2; ++k) {
            const double point = st[k];
            if (point > 0.0 && point < upper) {
                const double value = poly(point, c);
                const double magnitude = poly_scale(point, c);
                if (!isfinite(value) || !(magnitude > 0.0)) return;
                if (fabs(value) <= 64.0 * kEps * magnitude) {
                    rs.status = kRootNearMultiple;
                    return;
                }
                ep[ne++] = point;
            }
        }
    }
    ep[ne++] = upper;
    for (int interval = 1; interval < ne; ++interval) {
        double left = ep[interval - 1], right = ep[interval];
        double fl = poly(left, c);
        const double fr = poly(right, c);
        if (!isfinite(fl) || !isfinite(fr)) return;
        if (signbit(fl) == signbit(fr)) continue;
        double y = 0.0;
        bool converged = false;
        int it = 0;
        if (newton) {
            // bracketed Newton on the same monotone interval: the iterate stays
            // inside [left, right], a step leaving it is replaced by bisection,
            // and the stopping test is the reference's 4 eps relative width
            const bool increasing = signbit(fl);  // H(left) < 0 <=> increasing on this interval
            y = (left + right) * 0.5;
            for (int h = 0; h < nhint; ++h) {
                const double yh = (zhint[h] - b) / rs.scale;
                if (yh > left && yh < right) {
                    y = yh;
                    break;
                }
            }
            for (; it < 100; ++it) {
                const double fy = poly(y, c);
                if (fy == 0.0) {
                    converged = true;
                    break;
                }
                if ((fy > 0.0) == increasing) right = y; else left = y;
                const double dh = fma(3.0 * y + 2.0 * c.c2, y, c.c1);
                double yn = y - fy / dh;
                if (!(yn > left && yn < right)) yn = (left + right) * 0.5;
                const bool done = fabs(yn - y) <= 2.0 * kEps * fmax(yn, kDblMin) ||
                                  right - left <= 4.0 * kEps * fmax(y, kDblMin);
                y = yn;
                if (done) {
                    converged = true;
                    break;
                }
            }
        }
        for (; it < 2048 && !converged; ++it) {
            y = (left + right) * 0.5;
            const double fy = poly(y, c);
            if (fy == 0.0 || y == left || y == right || right - left <= 4.0 * kEps * fmax(y, kDblMin)) {
                converged = true;
                break;
            }
            if (signbit(fy) == signbit(fl)) {
                left = y;
                fl = fy;
            } else {
                right = y;
            }
        }
        iterations += it + 1;
        if (!converged) {
            rs.count = 0;
            rs.status = kRootIterLimit;
            return;
        }
        const double xv = y * rs.scale;
        const double z = xv + b;
        const double magnitude = poly_scale(y, c);
        const double residual = fabs(poly(y, c)) / magnitude;
        const double dh = fma(3.0 * y + 2.0 * c.c2, y, c.c1);
        const double dh_scale = 3.0 * y * y + 2.0 * fabs(c.c2) * y + fabs(c.c1);
        const double slope_ratio = dh_scale > 0.0 ? fabs(dh) / dh_scale : 0.0;
        const double bz = b / z;
        const double repulsion = 1.0 / xv;
        const double attraction = ((a / z) / z) / (1.0 + 2.0 * bz - bz * bz);
        const double pres = fabs(repulsion - attraction - 1.0) / (1.0 + fabs(repulsion) + fabs(attraction));
        if (!isfinite(z) || !(z > b) || !isfinite(residual) || !isfinite(pres) || residual > 128.0 * kEps ||
            pres > 512.0 * kEps || rs.count == 3) {
            rs.count = 0;
            rs.status = kRootUnrepresentable;
            return;
        }
        if (rs.count != 0 && !(z > rs.r[rs.count - 1].z)) {
            rs.count = 0;
            rs.status = kRootNearMultiple;
            return;
        }
        Root& r = rs.r[rs.count++];
        r.z = z;
        r.free_volume = xv;
        r.derivative_valid = slope_ratio > 8.0 * 1.4901161193847656e-08;  // 8 sqrt(eps)
        r.slope_sign = dh > 0.0 ? 1 : (dh < 0.0 ? -1 : 0);
    }
    rs.status = rs.count > 0 ? kRootSuccess : kRootUnrepresentable;
}

__device__ __forceinline__ int root_issue(int s) {
    return s == kRootSuccess ? kOk : (s == kRootNearMultiple ? kRootTopology
                                      : (s == kRootIterLimit ? kRootIterationLimit : kRootRange));
}

// log1p(u)/u with the degree-19 series at |u| <= 1/8, pr76_phase.hpp:67-79.
__device__ __forceinline__ double log1p_over_x(double u) {
    if (fabs(u) <= 0.125) {
        double value = -1.0 / 20.0;
#pragma unroll
        for (int k = 18; k >= 0; --k) value = ((k % 2 == 0) ? 1.0 : -1.0) / static_cast<double>(k + 1) + u * value;
        return value;
    }
    return log1p(u) / u;
}

// ln phi at a resolved root, pr76_phase.hpp:223-253.
template <int NM>
__device__ bool ln_phi_of_root(const Mixture& m, const Cell<NM>& c, double amix, double bmix, double A,
                               double B, const Root& root, double* ln_phi) {
    const double free_volume = root.free_volume;
    const double z = free_volume + B;
    const double sqrt2 = 1.4142135623730951;
    const double denominator = free_volume + (2.0 - sqrt2) * B;
    const double u = (2.0 * sqrt2) * (B / denominator);
    const double log_factor = log1p_over_x(u) / denominator;
    double z_minus_one = z - 1.0;
    double log_free = log(free_volume);
    if (fabs(z_minus_one) < 0.25 && B < 0.125) {
        const double bz = B / z;
        z_minus_one = B / free_volume - (A / z) / (1.0 + 2.0 * bz - bz * bz);
        log_free = log1p(z_minus_one - B);
    }
    const double rt = kR * c.t;
    const double prt = c.p / rt;
    for (int i = 0; i < c.n; ++i) {
        const double ratio = m.b[i] / bmix;
        const double coefficient = ((2.0 * c.sums[i] - amix * ratio) / rt) * prt;
        ln_phi[i] = ratio * z_minus_one - log_free - coefficient * log_factor;
        if (!isfinite(ln_phi[i])) return false;
    }
    return isfinite(z);
}

// Stability provider (minimum-Gibbs admissible root), pr76_stability.hpp:36-119.
// Writes ln phi of the selected branch into `out`.
template <int NM>
__device__ MPMC_FP64_CALL int stability_provider(const Mixture& m, Cell<NM>& c, const double* x, double* out, bool& smooth,
                                  double* z_out, int counter_row, int* branch_out = nullptr) {
    ++c.counters[counter_row];
    double amix, bmix, A, B;
    if (!mix(m, c, x, amix, bmix)) return kRootRange;
    if (!coefficients(c.p, c.t, amix, bmix, A, B)) return kRootRange;
    RootSet rs;
    solve_roots(A, B, rs, c.counters[cRootIters], c.newton);
    if (rs.status != kRootSuccess) return root_issue(rs.status);
    int cand[3];
    int ncand = 0;
    for (int k = 0; k < rs.count; ++k) {
        if (rs.r[k].slope_sign <= 0) continue;
        if (ncand == 2) return kRootRange;  // cannot happen: admissible roots alternate with the middle one
        if (!ln_phi_of_root(m, c, amix, bmix, A, B, rs.r[k], c.lnphi[ncand])) return kRootRange;
        cand[ncand++] = k;
    }
    if (ncand == 0) return kNoAdmissibleBranch;
    const int n = c.n;
    int best = 0;
    smooth = true;
    if (ncand == 2) {
        double v = 0.0, cc = 0.0;
        for (int i = 0; i < n; ++i) kahan_add(x[i] * (c.lnphi[1][i] - c.lnphi[0][i]), v, cc);
        if (!isfinite(v)) return kNonfinite;
        if (v < 0.0) best = 1;
        const int other = 1 - best;
        double magnitude = 1.0;
        for (int i = 0; i < n; ++i) magnitude += x[i] * (fabs(c.lnphi[other][i]) + fabs(c.lnphi[best][i]));
        if (!isfinite(magnitude)) return kNonfinite;
        double d = 0.0, dc = 0.0;
        for (int i = 0; i < n; ++i) kahan_add(x[i] * (c.lnphi[other][i] - c.lnphi[best][i]), d, dc);
        if (!isfinite(d)) return kNonfinite;
        if (fabs(d) <= 256.0 * kEps * magnitude) smooth = false;
    }
    if (!rs.r[cand[best]].derivative_valid) return kIllConditionedRoot;
    for (int i = 0; i < n; ++i) out[i] = c.lnphi[best][i];
    if (z_out) *z_out = rs.r[cand[best]].z;
    if (branch_out) *branch_out = cand[best];
    return kOk;
}

// Role provider (liquid = smallest, vapor = largest admissible root),
// pr76_split.hpp:38-84 with split_check_phase (pt_split.hpp:197-203).
template <int NM>
__device__ MPMC_FP64_CALL int role_provider(const Mixture& m, Cell<NM>& c, const double* x, bool vapor, double* ln_phi,
                             double& z_out, int& branch, double* roots = nullptr, int* nroots = nullptr) {
    ++c.counters[cSplitEvals];
    double amix, bmix, A, B;
    if (!mix(m, c, x, amix, bmix)) return kRootRange;
    if (!coefficients(c.p, c.t, amix, bmix, A, B)) return kRootRange;
    RootSet rs;
    // roots (nroots of them) of this role's previous evaluation are the Newton starts;
    // on return they hold this evaluation's roots
    solve_roots(A, B, rs, c.counters[cRootIters], c.newton, roots, nroots ? *nroots : 0);
    if (roots && nroots) {
        *nroots = rs.status == kRootSuccess ? rs.count : 0;
        for (int k = 0; k < *nroots; ++k) roots[k] = rs.r[k].z;
    }
    if (rs.status != kRootSuccess) return root_issue(rs.status);
    int selected = -1;
    for (int k = 0; k < rs.count; ++k) {
        if (rs.r[k].slope_sign <= 0) continue;
        selected = k;
        if (!vapor) break;
    }
    if (selected < 0) return kNoAdmissibleBranch;
    if (!rs.r[selected].derivative_valid) return kIllConditionedRoot;
    if (!ln_phi_of_root(m, c, amix, bmix, A, B, rs.r[selected], ln_phi)) return kRootRange;
    z_out = rs.r[selected].z;
    branch = selected;
    if (!isfinite(z_out) || z_out <= 0.0) return kIllConditionedRoot;
    return kOk;
}

// ---------------------------------------------------------------------------
// Tangent-plane distance, pt_stability.hpp:178-220.
template <int NM>
struct TpdPoint {
    double w[NM], res[NM], lw[NM];
    double value, guard, stat;
    bool smooth;
    int branch;  // root branch of the stability phase at w
};

__device__ __forceinline__ bool check_composition(const double* x, int n, double& sum) {
    double s = 0.0, cc = 0.0;
    for (int i = 0; i < n; ++i) {
        if (!isfinite(x[i]) || x[i] < 0.0 || x[i] > 1.0) return false;
        kahan_add(x[i], s, cc);
    }
    sum = s;
    return fabs(s - 1.0) <= 64.0 * kEps;
}

template <int NM>
__device__ int tpd(const Cell<NM>& c, const double* lnphi_w, const double* lnphi_ref, TpdPoint<NM>& pt) {
    const int n = c.n;
    double sum;
    if (!check_composition(pt.w, n, sum)) return kDomain;
    double value = 0.0, correction = 0.0, magnitude = 1.0, mc = 0.0;
    bool boundary = false;
    for (int i = 0; i < n; ++i) {
        pt.res[i] = 0.0;
        if (c.z[i] == 0.0) {
            if (pt.w[i] != 0.0) return kDomain;
            continue;
        }
        if (pt.w[i] == 0.0) {
            boundary = true;
            continue;
        }
        const double w = pt.w[i], z = c.z[i];
        const double lw = log(w), lz = c.lz[i];
        pt.lw[i] = lw;
        const double log_ratio = fabs(w - z) < 0.5 * z ? log1p((w - z) / z) : lw - lz;
        const double q = log_ratio + (lnphi_w[i] - lnphi_ref[i]);
        pt.res[i] = q;
        kahan_add(w * q, value, correction);
        kahan_add(w * (fabs(lw) + fabs(lz) + fabs(lnphi_w[i]) + fabs(lnphi_ref[i])), magnitude, mc);
    }
    const double mean = value / sum;
    double stat = 0.0;
    for (int i = 0; i < n; ++i) {
        if (c.z[i] == 0.0) continue;
        pt.res[i] = pt.w[i] == 0.0 ? -INFINITY : pt.res[i] - mean;
        stat = fmax(stat, fabs(pt.res[i]));
    }
    pt.value = value;
    pt.stat = stat;
    pt.guard = 256.0 * kEps * magnitude;
    if (!isfinite(pt.value) || !isfinite(pt.guard) || (!boundary && !isfinite(stat))) return kNonfinite;
    return kOk;
}

struct StabilityOptions {  // pt_stability.hpp:44-56
    double tpd_tolerance;
    int eval_row;  // counter row charged for provider calls
};

enum TrialStatus : int { kNegativeTpd = 0, kStationary, kIterationLimit, kEvaluationLimit, kLineSearchFailed,
                         kPropertyFailure, kNonsmooth, kUnrepresentableComposition };

template <int NM>
__device__ __forceinline__ bool tpd_negative(const TpdPoint<NM>& p, double tol) {
    return p.value < -tol - p.guard;  // pt_stability.hpp:150-152
}

// One TPD trial from the composition already in `point.w`, pt_stability.hpp:343-457.
// `evals` counts provider calls of this stability test against the 100000 budget.
template <int NM>
__device__ MPMC_FP64_CALL int run_trial(const Mixture& m, Cell<NM>& c, const double* ref, const StabilityOptions& o,
                         TpdPoint<NM>& point, TpdPoint<NM>& next, double* direction, double* lnphi_scratch,
                         int& evals) {
    const int n = c.n;
    const int max_evals = 100000;
    for (int i = 0; i < n; ++i)
        if (c.z[i] > 0.0 && point.w[i] == 0.0) return kUnrepresentableComposition;
    if (evals >= max_evals) return kEvaluationLimit;
    {
        ++evals;
        bool smooth;
        int is = stability_provider(m, c, point.w, lnphi_scratch, smooth, nullptr, o.eval_row, &point.branch);
        if (is == kOk) is = tpd(c, lnphi_scratch, ref, point);
        if (is == kDomain) return -1;
        if (is != kOk) return kPropertyFailure;
        point.smooth = smooth;
    }
    int iterations = 0;
    for (;;) {
        if (tpd_negative(point, o.tpd_tolerance)) return kNegativeTpd;
        if (!point.smooth) return kNonsmooth;
        if (point.stat <= 1e-8) return kStationary;
        if (iterations >= 512) return kIterationLimit;
        const double scale = fmax(1.0, point.stat / 4.0);
        double slope = 0.0, sc = 0.0;
        for (int i = 0; i < n; ++i) {
            direction[i] = 0.0;
            if (c.z[i] == 0.0) continue;
            direction[i] = -point.res[i] / scale;
            kahan_add((point.w[i] * point.res[i]) * direction[i], slope, sc);
        }
        if (!isfinite(slope) || !(slope < 0.0)) return kLineSearchFailed;
        bool accepted = false;
        double alpha = 1.0;
        int status = kLineSearchFailed;
        for (int bt = 0; bt < 32; ++bt, alpha *= 0.5) {
            double largest = -INFINITY;
            for (int i = 0; i < n; ++i) {
                if (c.z[i] > 0.0) {
                    next.w[i] = point.lw[i] + alpha * direction[i];
                    largest = fmax(largest, next.w[i]);
                }
            }
            double sum = 0.0, cs = 0.0;
            for (int i = 0; i < n; ++i) {
                next.w[i] = c.z[i] > 0.0 ? exp(next.w[i] - largest) : 0.0;
                kahan_add(next.w[i], sum, cs);
            }
            bool positive = isfinite(sum) && sum > 0.0;
            for (int i = 0; i < n; ++i) {
                next.w[i] /= sum;
                positive = positive && (c.z[i] == 0.0 || next.w[i] > 0.0);
            }
            if (!positive) continue;
            if (evals >= max_evals) {
                status = kEvaluationLimit;
                break;
            }
            ++evals;
            bool smooth;
            int is = stability_provider(m, c, next.w, lnphi_scratch, smooth, nullptr, o.eval_row, &next.branch);
            if (is == kOk) is = tpd(c, lnphi_scratch, ref, next);
            if (is == kDomain) return -1;
            if (is != kOk) continue;
            next.smooth = smooth;
            bool accept = tpd_negative(next, o.tpd_tolerance);
            if (!accept) {
                const double predicted = -alpha * slope;
                const double guard = point.guard + next.guard;
                if (predicted <= guard)
                    accept = next.value <= point.value + guard && alpha / scale > 0.0 && next.stat < point.stat;
                else
                    accept = next.value <= point.value - 1e-4 * predicted;
            }
            if (accept) {
                // swap point <- next (copy; arrays are small)
                for (int i = 0; i < n; ++i) {
                    point.w[i] = next.w[i];
                    point.res[i] = next.res[i];
                    point.lw[i] = next.lw[i];
                }
                point.value = next.value;
                point.guard = next.guard;
                point.stat = next.stat;
                point.smooth = next.smooth;
                point.branch = next.branch;
                accepted = true;
                break;
            }
        }
        if (!accepted) return status;
        ++iterations;
        ++c.counters[cTrialIters];
    }
}

// ---------------------------------------------------------------------------
// Rachford-Rice, rachford_rice.hpp:70-147.
enum RrStatus : int { kRrInterior = 0, kRrNoInterior, kRrDegenerate, kRrIterLimit, kRrUnrepresentable };

template <int NM>
struct SplitState {
    double x[NM], y[NM], lnk[NM], res[NM], common[NM], lnphi_l[NM], lnphi_v[NM];
    double beta, z_l, z_v, gibbs, guard, fug, mass_abs, mass_rel;
    int branch_l, branch_v;
    double roots_l[3], roots_v[3];  // all cubic roots of each phase (Newton starts of a nearby state)
    int nroots_l, nroots_v;
};

// `newton` selects a bracketed Newton iteration on the same residual instead of
// bisection (used by the mixed form's polish; the plain form uses bisection,
// rachford_rice.hpp:93-107).  Both stop at the reference's width test
// 8 eps min(beta, 1 - beta) and apply the same residual and balance checks.
// Newton starts at `beta0` (the root of a nearby ln K, e.g. the previous
// chord step's) inside the bracket (0, 1), else at 1/2.
template <int NM>
__device__ int solve_rr(Cell<NM>& c, const double* lk, SplitState<NM>& s, double* e, double* num,
                        bool newton = false, double beta0 = 0.5) {
    const int n = c.n;
    double contrast = 0.0;
    for (int i = 0; i < n; ++i)
        if (c.z[i] > 0.0) contrast = fmax(contrast, fabs(lk[i]));
    if (contrast == 0.0) return kRrDegenerate;
    // log-sum-exp endpoint signs, :42-52 and :86-92
    double ls[2];
    for (int k = 0; k < 2; ++k) {
        const double sign = k == 0 ? 1.0 : -1.0;
        double largest = -INFINITY;
        for (int i = 0; i < n; ++i)
            if (c.z[i] > 0.0) largest = fmax(largest, c.lz[i] + sign * lk[i]);
        double sum = 0.0, cc = 0.0;
        for (int i = 0; i < n; ++i)
            if (c.z[i] > 0.0) kahan_add(exp(c.lz[i] + sign * lk[i] - largest), sum, cc);
        ls[k] = largest + log(sum);
    }
    if (!isfinite(ls[0]) || !isfinite(ls[1])) return kRrUnrepresentable;
    if (ls[0] <= 64.0 * kEps || ls[1] <= 64.0 * kEps) return kRrNoInterior;
    for (int i = 0; i < n; ++i) {
        if (c.z[i] == 0.0) continue;
        e[i] = exp(-fabs(lk[i]));
        num[i] = lk[i] >= 0.0 ? -expm1(-lk[i]) : expm1(lk[i]);
    }
    double left = 0.0, right = 1.0, beta = 0.5, value = 0.0;
    bool resolved = false;
    if (newton) {
        if (beta0 > 0.0 && beta0 < 1.0) beta = beta0;
        for (int it = 0; it < 64; ++it) {
            ++c.counters[cRrIters];
            double v = 0.0, dv = 0.0;
            for (int i = 0; i < n; ++i) {
                if (c.z[i] == 0.0) continue;
                const double den = lk[i] >= 0.0 ? beta + (1.0 - beta) * e[i] : (1.0 - beta) + beta * e[i];
                const double dd = lk[i] >= 0.0 ? 1.0 - e[i] : e[i] - 1.0;
                const double term = (c.z[i] / den) * num[i];
                v += term;
                dv -= term * dd / den;
            }
            value = v;
            if (!isfinite(value)) return kRrUnrepresentable;
            if (value == 0.0) {
                resolved = true;
                break;
            }
            if (value > 0.0) left = beta; else right = beta;
            double bn = beta - value / dv;
            if (!(bn > left && bn < right)) bn = (left + right) * 0.5;
            const double step = fabs(bn - beta);
            beta = bn;
            if (step <= 8.0 * kEps * fmin(beta, 1.0 - beta) || right - left <= 8.0 * kEps * fmin(beta, 1.0 - beta)) {
                double v2 = 0.0, cc = 0.0;
                for (int i = 0; i < n; ++i) {
                    if (c.z[i] == 0.0) continue;
                    const double den = lk[i] >= 0.0 ? beta + (1.0 - beta) * e[i] : (1.0 - beta) + beta * e[i];
                    kahan_add((c.z[i] / den) * num[i], v2, cc);
                }
                value = v2;
                resolved = true;
                break;
            }
        }
    }
    for (int it = 0; it < 192 && !resolved; ++it) {
        ++c.counters[cRrIters];
        beta = (left + right) * 0.5;
        if (!(beta > 0.0 && beta < 1.0)) break;
        double v = 0.0, cc = 0.0;
        for (int i = 0; i < n; ++i) {
            if (c.z[i] == 0.0) continue;
            const double den = lk[i] >= 0.0 ? beta + (1.0 - beta) * e[i] : (1.0 - beta) + beta * e[i];
            kahan_add((c.z[i] / den) * num[i], v, cc);
        }
        value = v;
        if (!isfinite(value)) return kRrUnrepresentable;
        if (value == 0.0 || beta == left || beta == right || right - left <= 8.0 * kEps * fmin(beta, 1.0 - beta)) {
            resolved = true;
            break;
        }
        if (value > 0.0) left = beta; else right = beta;
    }
    if (!resolved) return kRrIterLimit;
    if (fabs(value) > 64.0 * kEps) return kRrUnrepresentable;
    for (int i = 0; i < n; ++i) {
        s.x[i] = 0.0;
        s.y[i] = 0.0;
        if (c.z[i] == 0.0) continue;
        const double den = lk[i] >= 0.0 ? beta + (1.0 - beta) * e[i] : (1.0 - beta) + beta * e[i];
        const double larger = c.z[i] / den;
        s.x[i] = lk[i] >= 0.0 ? larger * e[i] : larger;
        s.y[i] = lk[i] >= 0.0 ? larger : larger * e[i];
        if (!isfinite(larger) || !(s.x[i] > 0.0 && s.y[i] > 0.0)) return kRrUnrepresentable;
    }
    double sx = 0.0, cx = 0.0, sy = 0.0, cy = 0.0;
    for (int i = 0; i < n; ++i) {
        kahan_add(s.x[i], sx, cx);
        kahan_add(s.y[i], sy, cy);
    }
    if (fabs(sx - 1.0) > 64.0 * kEps || fabs(sy - 1.0) > 64.0 * kEps) return kRrUnrepresentable;
    s.mass_abs = 0.0;
    s.mass_rel = 0.0;
    for (int i = 0; i < n; ++i) {
        s.x[i] /= sx;
        s.y[i] /= sy;
        const double recovered = fma(beta, s.y[i], (1.0 - beta) * s.x[i]);
        const double err = fabs(recovered - c.z[i]);
        s.mass_abs = fmax(s.mass_abs, err);
        if (c.z[i] > 0.0) {
            if (!(s.x[i] > 0.0 && s.y[i] > 0.0)) return kRrUnrepresentable;
            s.mass_rel = fmax(s.mass_rel, err / c.z[i]);
        } else if (recovered != 0.0) {
            return kRrUnrepresentable;
        }
    }
    s.beta = beta;
    return kRrInterior;
}

// ---------------------------------------------------------------------------
// Split iteration, pt_split.hpp:275-408.
enum AttemptStatus : int { kConverged = 0, kNoInteriorRr, kRrFailure, kIndistinguishable, kPhaseDisappearance,
                           kAttemptPropertyFailure, kAttemptIterationLimit, kAttemptEvaluationLimit,
                           kAttemptLineSearchFailed, kUnrepresentableSeed, kBalanceFailure };

// Split evaluation, pt_split.hpp:300-341.  Returns kConverged (= usable state)
// or the failure class.  `near` (optional): a nearby state whose beta and
// cubic roots start the Rachford-Rice and root Newton iterations (bracketed
// Newton only).
template <int NM>
__device__ MPMC_FP64_CALL int split_evaluate(const Mixture& m, Cell<NM>& c, const double* lk, SplitState<NM>& s, int& evals,
                              int budget, double* e, double* num, bool newton_rr = false, double beta0 = 0.5,
                              const SplitState<NM>* near = nullptr) {
    const int n = c.n;
    const int rr = solve_rr(c, lk, s, e, num, newton_rr || c.newton, beta0);
    if (rr != kRrInterior)
        return rr == kRrDegenerate ? kIndistinguishable : (rr == kRrNoInterior ? kNoInteriorRr : kRrFailure);
    s.nroots_l = s.nroots_v = 0;
    if (near && &s != near) {
        s.nroots_l = near->nroots_l;
        s.nroots_v = near->nroots_v;
        for (int k = 0; k < 3; ++k) {
            s.roots_l[k] = near->roots_l[k];
            s.roots_v[k] = near->roots_v[k];
        }
    }
    if (evals >= budget) return kAttemptEvaluationLimit;
    ++evals;
    if (role_provider(m, c, s.x, false, s.lnphi_l, s.z_l, s.branch_l, s.roots_l, &s.nroots_l) != kOk)
        return kAttemptPropertyFailure;
    if (evals >= budget) return kAttemptEvaluationLimit;
    ++evals;
    if (role_provider(m, c, s.y, true, s.lnphi_v, s.z_v, s.branch_v, s.roots_v, &s.nroots_v) != kOk)
        return kAttemptPropertyFailure;
    double correction = 0.0, magnitude = 1.0, mc = 0.0, gibbs = 0.0, fug = 0.0;
    const double beta = s.beta;
    for (int i = 0; i < n; ++i) {
        s.lnk[i] = 0.0;
        s.res[i] = 0.0;
        s.common[i] = 0.0;
        if (c.z[i] == 0.0) continue;
        const double lx = log(s.x[i]);
        const double ly = log(s.y[i]);
        const double mu_l = lx + s.lnphi_l[i];
        const double mu_v = ly + s.lnphi_v[i];
        s.lnk[i] = ly - lx;
        s.res[i] = (lx - ly) + (s.lnphi_l[i] - s.lnphi_v[i]);
        s.common[i] = (mu_l + mu_v) * 0.5;
        fug = fmax(fug, fabs(s.res[i]));
        kahan_add((1.0 - beta) * s.x[i] * mu_l + beta * s.y[i] * mu_v, gibbs, correction);
        kahan_add((1.0 - beta) * s.x[i] * (fabs(lx) + fabs(s.lnphi_l[i])) +
                      beta * s.y[i] * (fabs(ly) + fabs(s.lnphi_v[i])),
                  magnitude, mc);
        if (!isfinite(s.res[i]) || !isfinite(s.common[i])) return kAttemptPropertyFailure;
    }
    s.gibbs = gibbs;
    s.fug = fug;
    s.guard = 256.0 * kEps * magnitude;
    if (!isfinite(s.gibbs) || !isfinite(s.guard)) return kAttemptPropertyFailure;
    return kConverged;
}

template <int NM>
__device__ __forceinline__ void copy_state(SplitState<NM>& d, const SplitState<NM>& s, int n) {
    for (int i = 0; i < n; ++i) {
        d.x[i] = s.x[i];
        d.y[i] = s.y[i];
        d.lnk[i] = s.lnk[i];
        d.res[i] = s.res[i];
        d.common[i] = s.common[i];
        d.lnphi_l[i] = s.lnphi_l[i];
        d.lnphi_v[i] = s.lnphi_v[i];
    }
    d.beta = s.beta;
    d.z_l = s.z_l;
    d.z_v = s.z_v;
    d.gibbs = s.gibbs;
    d.guard = s.guard;
    d.fug = s.fug;
    d.mass_abs = s.mass_abs;
    d.mass_rel = s.mass_rel;
    d.branch_l = s.branch_l;
    d.branch_v = s.branch_v;
    d.nroots_l = s.nroots_l;
    d.nroots_v = s.nroots_v;
    for (int k = 0; k < 3; ++k) {
        d.roots_l[k] = s.roots_l[k];
        d.roots_v[k] = s.roots_v[k];
    }
}

// iterate_pt_split from ln K in `lk0`; the last accepted state ends in `point`.
template <int NM>
__device__ MPMC_FP64_CALL int iterate_split(const Mixture& m, Cell<NM>& c, const double* lk0, SplitState<NM>& point,
                             SplitState<NM>& next, double* next_lk, int& evals, int budget, double* e, double* num) {
    const int n = c.n;
    int st = split_evaluate(m, c, lk0, point, evals, budget, e, num);
    if (st != kConverged) return st;
    int iterations = 0;
    for (;;) {
        if (point.fug <= 1e-11) {  // :351-363
            double contrast = 0.0;
            for (int i = 0; i < n; ++i) contrast = fmax(contrast, fabs(point.lnk[i]));
            const double beta = point.beta;
            if (!(point.mass_abs <= 1e-12 && point.mass_rel <= 1e-10)) return kBalanceFailure;
            if (beta <= 1e-10 || 1.0 - beta <= 1e-10) return kPhaseDisappearance;
            if (contrast <= 1e-7 || point.z_v - point.z_l <= 1e-8 * fmax(point.z_v, point.z_l))
                return kIndistinguishable;
            return kConverged;
        }
        if (iterations >= 512) return kAttemptIterationLimit;
        const double scale = fmax(1.0, point.fug / 2.0);
        // Gibbs slope, :213-231
        double h = 0.0, hc = 0.0, first = 0.0, fc = 0.0, second = 0.0, sc = 0.0;
        for (int i = 0; i < n; ++i) {
            if (c.z[i] == 0.0) continue;
            const double x = point.x[i], y = point.y[i];
            const double cc = (x / c.z[i]) * y;
            const double d = y - x;
            const double r = point.res[i];
            kahan_add(d * (d / c.z[i]), h, hc);
            kahan_add(cc * r, first, fc);
            kahan_add((cc * r) * r, second, sc);
        }
        double slope = NAN;
        if (h > 0.0 && isfinite(h) && isfinite(first) && isfinite(second))
            slope = -(point.beta * (1.0 - point.beta) * second + (first / h) * first) / scale;
        if (!isfinite(slope) || !(slope < 0.0)) return kAttemptLineSearchFailed;
        bool accepted = false;
        double alpha = 1.0;
        for (int bt = 0; bt < 24; ++bt, alpha *= 0.5) {
            for (int i = 0; i < n; ++i) next_lk[i] = point.lnk[i] + (alpha / scale) * point.res[i];
            st = split_evaluate(m, c, next_lk, next, evals, budget, e, num);
            if (st == kConverged) {
                const double predicted = -alpha * slope;
                const double guard = point.guard + next.guard;
                bool accept;
                if (predicted > guard)
                    accept = next.gibbs <= point.gibbs - 1e-4 * predicted;
                else
                    accept = next.gibbs <= point.gibbs + guard &&
                             (next.fug <= 1e-11 || point.fug - next.fug > 1e-4 * (alpha / scale) * point.fug);
                if (accept) {
                    copy_state(point, next, n);
                    accepted = true;
                    break;
                }
            } else if (st == kAttemptEvaluationLimit) {
                return kAttemptEvaluationLimit;
            }
        }
        if (!accepted) return kAttemptLineSearchFailed;
        ++iterations;
        ++c.counters[cSplitIters];
    }
}

// split_seed, pt_split.hpp:245-267.
template <int NM>
__device__ bool split_seed(const Cell<NM>& c, const double* w, bool as_vapor, double* other, double* lk) {
    const int n = c.n;
    double amount = 0.1;
    for (int i = 0; i < n; ++i)
        if (c.z[i] > 0.0) amount = fmin(amount, 0.5 * (c.z[i] / w[i]));
    if (!(amount > 0.0 && amount < 1.0)) return false;
    double sum = 0.0, cs = 0.0;
    for (int i = 0; i < n; ++i) {
        other[i] = 0.0;
        lk[i] = 0.0;
        if (c.z[i] != 0.0) {
            other[i] = fma(-amount, w[i], c.z[i]) / (1.0 - amount);
            if (!(other[i] > 0.0)) return false;
        }
        kahan_add(other[i], sum, cs);
    }
    if (!isfinite(sum) || fabs(sum - 1.0) > 64.0 * kEps) return false;
    for (int i = 0; i < n; ++i) {
        if (c.z[i] == 0.0) continue;
        other[i] /= sum;
        lk[i] = (as_vapor ? 1.0 : -1.0) * (log(w[i]) - log(other[i]));
        if (!isfinite(lk[i])) return false;
    }
    return true;
}

// ---------------------------------------------------------------------------
// Whole cell: pt_split.hpp:415-525 (solve_pt_vle) without initial/final hints.
template <int NM>
struct CellResult {
    int status;
    bool has_pair;
    double ref_lnphi[NM];  // feed phase (single-phase result)
    double ref_z;
};

// Scratch bundle so the kernel frame holds one copy of everything.
template <int NM>
struct Scratch {
    TpdPoint<NM> point, next;
    double direction[NM], lnphi[NM], imposed[NM];
    SplitState<NM> s_point, s_next, best;
    double lk[NM], other[NM], e[NM], num[NM];
};

// Automatic start k of a stability test (pt_stability.hpp:294-310): 0 = feed,
// 1 = uniform over active components, 2.. = 0.1 z + 0.9 e_i for the (k-2)-th
// active component; then extra starts.  Normalised by its compensated sum.
template <int NM>
__device__ void make_start(const Cell<NM>& c, int k, int active, const double* const* extra, int n_auto, double* w) {
    const int n = c.n;
    if (k >= n_auto) {
        const double* src = extra[k - n_auto];
        for (int i = 0; i < n; ++i) w[i] = src[i];
    } else if (k == 0) {
        for (int i = 0; i < n; ++i) w[i] = c.z[i];
    } else if (k == 1) {
        for (int i = 0; i < n; ++i) w[i] = c.z[i] > 0.0 ? 1.0 / static_cast<double>(active) : 0.0;
    } else {
        int target = k - 2, idx = -1;
        for (int i = 0; i < n; ++i)
            if (c.z[i] > 0.0) {
                if (target == 0) {
                    idx = i;
                    break;
                }
                --target;
            }
        for (int i = 0; i < n; ++i) w[i] = c.z[i] * 0.1;
        w[idx] += 0.9;
    }
    double sum = 0.0, cs = 0.0;
    for (int i = 0; i < n; ++i) kahan_add(w[i], sum, cs);
    for (int i = 0; i < n; ++i) w[i] /= sum;
}

template <int NM>
__device__ void make_start(const Cell<NM>& c, int k, int active, const double* extra0, const double* extra1,
                           int n_auto, double* w) {
    const double* extra[2] = {extra0, extra1};
    make_start(c, k, active, extra, n_auto, w);
}

// An extra start of a stability test must be a composition with exactly the
// feed's support (pt_stability.hpp:263-272, a domain_error otherwise).
template <int NM>
__device__ bool start_matches_feed(const Cell<NM>& c, const double* s) {
    double ssum;
    if (!check_composition(s, c.n, ssum)) return false;
    for (int i = 0; i < c.n; ++i)
        if ((c.z[i] == 0.0) != (s[i] == 0.0)) return false;
    return true;
}

// Normalise the feed the way test_pt_stability_impl does (:242, :278).
template <int NM>
__device__ bool normalise_feed(Cell<NM>& c, const double* feed) {
    double sum;
    if (!check_composition(feed, c.n, sum)) return false;
    for (int i = 0; i < c.n; ++i) {
        c.z[i] = feed[i] / sum;
        c.lz[i] = c.z[i] > 0.0 ? log(c.z[i]) : 0.0;
    }
    return true;
}

// The two PtSplitOptions fields a caller may change (pt_split.hpp:45-50):
// initial_stability.automatic_starts and max_split_attempts.
struct SolveOptions {
    bool initial_automatic_starts = true;
    int max_split_attempts = 16;
};

// A caller start must be a composition with the raw feed's support (a
// domain_error in the reference: pt_stability.hpp:263-272, pt_split.hpp:436-443).
template <int NM>
__device__ bool start_on_support(const double* feed, int n, const double* s) {
    double ssum;
    if (!check_composition(s, n, ssum)) return false;
    for (int i = 0; i < n; ++i)
        if ((feed[i] > 0.0) != (s[i] > 0.0)) return false;
    return true;
}

// `init_extra` (n_init of them) join the automatic feed-test starts and
// `final_extra` (n_final, at most 3) precede the pair's x and y in the review,
// as solve_pt_vle's initial_starts / final_starts (pt_split.hpp:415-419, 512).
// Every caller start is checked before the first property call, final starts
// first (pt_split.hpp:436-443, pt_stability.hpp:254-272).
template <int NM>
__device__ MPMC_FP64_CALL int solve_cell(const Mixture& m, Cell<NM>& c, const double* feed_in, Scratch<NM>& w,
                          CellResult<NM>& out, const double* const* init_extra = nullptr, int n_init = 0,
                          const double* const* final_extra = nullptr, int n_final = 0,
                          const SolveOptions& opt = SolveOptions{}) {
    const int n = c.n;
    out.has_pair = false;
    if (!isfinite(c.p) || c.p <= 0.0 || !isfinite(c.t) || c.t <= 0.0) return kInvalid;
    if (!normalise_feed(c, feed_in)) return kInvalid;
    for (int k = 0; k < n_final && k < 3; ++k)
        if (!start_on_support<NM>(feed_in, n, final_extra[k])) return kInvalid;
    int active = 0;
    for (int i = 0; i < n; ++i) active += feed_in[i] > 0.0;
    const int n_auto = active == 1 ? 1 : active + 2;
    // the feed test's automatic starts, off on the caller's request; a test
    // with no start at all is a length_error in the reference
    const int n_auto_init = opt.initial_automatic_starts ? n_auto : 0;
    if (n_auto_init + n_init == 0) return kInvalid;
    for (int k = 0; k < n_init; ++k)
        if (!start_on_support<NM>(feed_in, n, init_extra[k])) return kInvalid;
    for (int i = 0; i < n; ++i)
        if (feed_in[i] > 0.0 && c.z[i] == 0.0) return kIndeterminate;
    if (!temp_setup(m, c)) return kInvalid;
    // ---- initial stability: reference phase at the feed
    int evals = 1;
    bool smooth_ref;
    {
        const int is = stability_provider(m, c, c.z, out.ref_lnphi, smooth_ref, &out.ref_z, cInitEvals);
        if (is == kDomain) return kInvalid;
        if (is != kOk) return kIndeterminate;  // every trial property_failure
    }
    StabilityOptions so{1e-10, cInitEvals};
    bool negative_found = false, all_stationary = true;
    int attempts = 0, split_evals = 0;
    bool limit = false;
    for (int k = 0; k < n_auto_init + n_init; ++k) {
        make_start(c, k, active, init_extra, n_auto_init, w.point.w);
        const int ts = run_trial(m, c, out.ref_lnphi, so, w.point, w.next, w.direction, w.lnphi, evals);
        if (ts < 0) return kInvalid;
        all_stationary = all_stationary && ts == kStationary;
        if (ts != kNegativeTpd) continue;
        negative_found = true;
        // split attempts of this witness, pt_split.hpp:459-486
        if (limit) continue;
        for (int role = 0; role < 2; ++role) {
            if (attempts >= opt.max_split_attempts || split_evals >= 20000) {
                limit = true;
                break;
            }
            const bool as_vapor = role == 0;
            int a_evals = 0;
            int st = kUnrepresentableSeed;
            if (split_seed(c, w.point.w, as_vapor, w.other, w.lk))
                st = iterate_split(m, c, w.lk, w.s_point, w.s_next, w.other, a_evals, 20000 - split_evals, w.e,
                                   w.num);
            split_evals += a_evals;
            ++attempts;
            if (st == kConverged && (!out.has_pair || w.s_point.gibbs < w.best.gibbs)) {
                copy_state(w.best, w.s_point, n);
                out.has_pair = true;
            }
        }
    }
    c.counters[cAttempts] = attempts;
    if (!negative_found) return all_stationary ? kSinglePhase : kIndeterminate;
    if (!out.has_pair) return kIndeterminate;
    // ---- phase-set review, pt_split.hpp:490-523
    const SplitState<NM>& cand = w.best;
    double feed_g = 0.0, correction = 0.0, magnitude = 1.0;
    for (int i = 0; i < n; ++i) {
        if (c.z[i] == 0.0) continue;
        const double lz = c.lz[i];
        const double phi = out.ref_lnphi[i];
        kahan_add(c.z[i] * (lz + phi), feed_g, correction);
        magnitude += c.z[i] * (fabs(lz) + fabs(phi));
    }
    const double gibbs_change = cand.gibbs - feed_g;
    const double gibbs_guard = cand.guard + 256.0 * kEps * magnitude;
    StabilityOptions fo{1e-10 + 0.5 * cand.fug, cFinalEvals};
    if (!isfinite(gibbs_change) || !isfinite(gibbs_guard) || !isfinite(fo.tpd_tolerance)) return kIndeterminate;
    // The review normalises the (already normalised) feed once more (:242, :278).
    double zz[NM];
    for (int i = 0; i < n; ++i) zz[i] = c.z[i];
    if (!normalise_feed(c, zz)) return kInvalid;
    // Extra starts (candidate x, y) must carry exactly the feed support (:263-272).
    for (int ph = 0; ph < 2; ++ph) {
        const double* s = ph == 0 ? cand.x : cand.y;
        double ssum;
        if (!check_composition(s, n, ssum)) return kInvalid;
        for (int i = 0; i < n; ++i)
            if ((c.z[i] == 0.0) != (s[i] == 0.0)) return kInvalid;
    }
    // imposed reference: ln phi_eq_i = common_i - ln z_i (pt_stability.hpp:319-322)
    for (int i = 0; i < n; ++i) w.imposed[i] = c.z[i] > 0.0 ? cand.common[i] - c.lz[i] : 0.0;
    bool final_negative = false, final_stationary = true;
    int fevals = 0;
    const double* review_extra[5];
    int n_review = 0;
    for (int k = 0; k < n_final && k < 3; ++k) review_extra[n_review++] = final_extra[k];
    review_extra[n_review++] = cand.x;
    review_extra[n_review++] = cand.y;
    for (int k = 0; k < n_auto + n_review; ++k) {
        make_start(c, k, active, review_extra, n_auto, w.point.w);
        const int ts = run_trial(m, c, w.imposed, fo, w.point, w.next, w.direction, w.lnphi, fevals);
        if (ts < 0) return kInvalid;
        final_stationary = final_stationary && ts == kStationary;
        final_negative = final_negative || ts == kNegativeTpd;
    }
    if (final_negative) return kPhaseSetUnstable;
    if (gibbs_change > gibbs_guard) return kIndeterminate;
    return final_stationary ? kTwoPhase : kIndeterminate;
}

}  // namespace fp64
}  // namespace pr76
