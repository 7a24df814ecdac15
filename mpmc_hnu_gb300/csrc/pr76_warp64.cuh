// Lane-group-cooperative FP64 work items of the mixed-precision flash.
//
// A group of S lanes (S = the component capacity rounded up to a power of two:
// 4, 8, 16 or 32, so a warp holds 32 / S groups) runs one item (a TPD trial, a
// ln K split attempt or a cell's Newton polish) to its end, with component i of
// the mixture on lane i of the group: mixing row sums, ln phi, the TPD terms,
// the Rachford-Rice terms and the ln K update are lane-parallel, the sums and
// maxima are group reductions, and the cubic is solved with one lane per
// monotone interval.  Control flow is uniform within a group (every branch
// depends on reduced, group-wide values); groups of one warp are independent.
//
// Why: a GB300 sub-partition retires an FP64 warp instruction in ~64 cycles
// whatever its active-lane count.  The lane-per-item form keeps 1-5 lanes of
// 32 busy on these long, uneven items (a few long attempts decided the
// stage's time); here an item's evaluation is ~5x fewer warp instructions.
//
// The rules are the reference's, as in the lane-per-item form:
//   TPD trial        pt_stability.hpp:343-457 (descent, 32-step line search,
//                    stopping at TPD < -tol - guard, stationarity 1e-8, 512 its)
//   stability root   pr76_stability.hpp:36-119 (minimum Gibbs admissible root)
//   role roots       pr76_split.hpp:38-84 (liquid smallest, vapor largest)
//   cubic            pr76_roots.hpp:77-173 (bracketed Newton per interval with
//                    the reference's stopping width and root checks)
//   Rachford-Rice    rachford_rice.hpp:70-147 (bracketed Newton)
//   ln K attempt     pt_split.hpp:275-408 (SS, Gibbs line search, 24 steps,
//                    |r| <= 1e-11 and the acceptance tests, 512 its)
// Sums are warp reductions instead of the reference's sequential compensated
// sums: they differ from it by rounding only.
#pragma once

#include "pr76_batched.cuh"
#include "pr76_lanes.cuh"

namespace pr76 {
namespace w64 {

// Per-lane view of one cell: lane i holds component i (lanes >= n hold zeros).
template <int NM, int S>
struct WCell {
    int n, lane;
    bool comp;     // lane < n
    bool act;      // lane < n and z_i > 0
    double p, t;
    double z, lz, b;
    double aij[NM];  // row i of a_ij = sqrt(a_i a_j)(1 - k_ij), a_ii = a_i
    int counters[cCount];  // warp-uniform
};

// Feed, a_i(T) and the a_ij row of one cell (pr76_pure.hpp:146-165,
// pr76_mixture.hpp:172-188).  False if the temperature terms are unusable.
template <int NM, int S>
__device__ bool load_cell(const Mixture& m, const batched::Workspace& ws, int64_t c, const double* p,
                          const double* t, WCell<NM, S>& w) {
    const int lane = seg_lane<S>();
    w.n = m.n;
    w.lane = lane;
    w.comp = lane < m.n;
    w.p = p[c];
    w.t = t[c];
    for (int k = 0; k < cCount; ++k) w.counters[k] = 0;
    w.z = w.comp ? ws.z[batched::idx(lane, ws.ncell, c)] : 0.0;
    w.act = w.comp && w.z > 0.0;
    w.lz = w.act ? log(w.z) : 0.0;
    w.b = w.comp ? m.b[lane] : 0.0;
    double a = 0.0, root = 0.0;
    bool bad = false;
    if (w.comp) {
        const double reduced_root = sqrt(w.t) / m.sqrt_tc[lane];
        const double bracket = 1.0 + m.kappa[lane] * (1.0 - reduced_root);
        a = (bracket * m.ac[lane]) * bracket;
        bad = !isfinite(a) || (a == 0.0 && bracket != 0.0) || (m.n > 1 && !(a > 0.0));
        root = sqrt(a);
    }
    if (wany<S>(bad)) return false;
#pragma unroll
    for (int j = 0; j < NM; ++j) {
        const double rj = bcast<S>(root, j);
        w.aij[j] = (w.comp && j < m.n) ? (j == lane ? a : (root * m.factor[lane * m.n + j]) * rj) : 0.0;
    }
    return true;
}

// Mixing with row sums (pr76_mixture.hpp:170-218): s_i on each lane, a and b
// warp-uniform.
template <int NM, int S>
__device__ bool mix(const WCell<NM, S>& c, double x, double& s, double& amix, double& bmix) {
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j < NM; ++j) {
        const double xj = bcast<S>(x, j);
        if (j < c.n) acc = fma(xj, c.aij[j], acc);
    }
    s = c.comp ? acc : 0.0;
    amix = wsum<S>(c.comp ? x * s : 0.0);
    bmix = wsum<S>(c.comp ? x * c.b : 0.0);
    return isfinite(amix) && isfinite(bmix) && bmix > 0.0 && !wany<S>(!isfinite(s));
}

// Cubic roots (pr76_roots.hpp:77-173) with one lane per monotone interval:
// the bracketed Newton iteration of the reference's stopping width on each
// interval runs concurrently, then the roots are checked and ordered exactly
// as in the sequential solver.
// `hint` (per lane, in/out): the root Z this lane's interval had in a nearby
// evaluation (NaN: none); Newton starts there when it lies inside the
// interval, else at the midpoint.  On return, the lane's root of this call
// (NaN where its interval holds none).
template <int S>
__device__ inline void roots_by_interval(double a, double b, fp64::RootSet& rs, int& iterations,
                                         double* hint = nullptr) {
    const double lane_hint = hint ? *hint : NAN;
    if (hint) *hint = NAN;
    using fp64::Cubic;
    const int lane = seg_lane<S>();
    rs.count = 0;
    rs.status = fp64::kRootUnrepresentable;
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
                const double value = fp64::poly(point, c);
                const double magnitude = fp64::poly_scale(point, c);
                if (!isfinite(value) || !(magnitude > 0.0)) return;
                if (fabs(value) <= 64.0 * kEps * magnitude) {
                    rs.status = fp64::kRootNearMultiple;
                    return;
                }
                ep[ne++] = point;
            }
        }
    }
    ep[ne++] = upper;
    // lane k (k < ne - 1) iterates on interval k + 1
    const int intervals = ne - 1;
    int state = 0;  // 0 no sign change, 1 root, 2 not converged, 3 nonfinite end value
    double y = 0.0;
    int it = 0;
    if (lane < intervals) {
        double left = ep[lane], right = ep[lane + 1];
        double fl = fp64::poly(left, c);
        const double fr = fp64::poly(right, c);
        if (!isfinite(fl) || !isfinite(fr)) {
            state = 3;
        } else if (signbit(fl) != signbit(fr)) {
            bool converged = false;
            const bool increasing = signbit(fl);
            y = (left + right) * 0.5;
            const double yh = (lane_hint - b) / rs.scale;
            if (yh > left && yh < right) y = yh;  // false for a NaN hint
            for (; it < 100; ++it) {
                const double fy = fp64::poly(y, c);
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
            for (; it < 2048 && !converged; ++it) {
                y = (left + right) * 0.5;
                const double fy = fp64::poly(y, c);
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
            state = converged ? 1 : 2;
        }
    }
    // per-lane root checks
    double z = 0.0, xv = 0.0;
    bool ok_root = false, dvalid = false;
    int sign = 0;
    if (state == 1) {
        xv = y * rs.scale;
        z = xv + b;
        const double magnitude = fp64::poly_scale(y, c);
        const double residual = fabs(fp64::poly(y, c)) / magnitude;
        const double dh = fma(3.0 * y + 2.0 * c.c2, y, c.c1);
        const double dh_scale = 3.0 * y * y + 2.0 * fabs(c.c2) * y + fabs(c.c1);
        const double slope_ratio = dh_scale > 0.0 ? fabs(dh) / dh_scale : 0.0;
        const double bz = b / z;
        const double repulsion = 1.0 / xv;
        const double attraction = ((a / z) / z) / (1.0 + 2.0 * bz - bz * bz);
        const double pres = fabs(repulsion - attraction - 1.0) / (1.0 + fabs(repulsion) + fabs(attraction));
        ok_root = isfinite(z) && z > b && isfinite(residual) && isfinite(pres) && residual <= 128.0 * kEps &&
                  pres <= 512.0 * kEps;
        dvalid = slope_ratio > 8.0 * 1.4901161193847656e-08;
        sign = dh > 0.0 ? 1 : (dh < 0.0 ? -1 : 0);
        if (hint && ok_root) *hint = z;
    }
    // sequential assembly in interval order
    for (int k = 0; k < intervals; ++k) {
        const int st = bcast<S>(state, k);
        const int itk = bcast<S>(it, k);
        const double zk = bcast<S>(z, k);
        const double xk = bcast<S>(xv, k);
        const bool okk = bcast<S>(ok_root ? 1 : 0, k) != 0;
        const bool dvk = bcast<S>(dvalid ? 1 : 0, k) != 0;
        const int sk = bcast<S>(sign, k);
        if (st == 3) {
            rs.count = 0;
            rs.status = fp64::kRootUnrepresentable;
            return;
        }
        if (st == 0) continue;
        iterations += itk + 1;
        if (st == 2) {
            rs.count = 0;
            rs.status = fp64::kRootIterLimit;
            return;
        }
        if (!okk || rs.count == 3) {
            rs.count = 0;
            rs.status = fp64::kRootUnrepresentable;
            return;
        }
        if (rs.count != 0 && !(zk > rs.r[rs.count - 1].z)) {
            rs.count = 0;
            rs.status = fp64::kRootNearMultiple;
            return;
        }
        fp64::Root& r = rs.r[rs.count++];
        r.z = zk;
        r.free_volume = xk;
        r.derivative_valid = dvk;
        r.slope_sign = sk;
    }
    rs.status = rs.count > 0 ? fp64::kRootSuccess : fp64::kRootUnrepresentable;
}

// ln phi_i at a resolved root (pr76_phase.hpp:223-253); true if every lane's
// value and Z are finite.
template <int NM, int S>
__device__ bool ln_phi(const WCell<NM, S>& c, double s, double amix, double bmix, double A, double B,
                       const fp64::Root& root, double& lnphi) {
    const double free_volume = root.free_volume;
    const double z = free_volume + B;
    const double sqrt2 = 1.4142135623730951;
    const double denominator = free_volume + (2.0 - sqrt2) * B;
    const double u = (2.0 * sqrt2) * (B / denominator);
    const double log_factor = fp64::log1p_over_x(u) / denominator;
    double z_minus_one = z - 1.0;
    double log_free = log(free_volume);
    if (fabs(z_minus_one) < 0.25 && B < 0.125) {
        const double bz = B / z;
        z_minus_one = B / free_volume - (A / z) / (1.0 + 2.0 * bz - bz * bz);
        log_free = log1p(z_minus_one - B);
    }
    const double rt = kR * c.t;
    const double prt = c.p / rt;
    lnphi = 0.0;
    if (c.comp) {
        const double ratio = c.b / bmix;
        const double coefficient = ((2.0 * s - amix * ratio) / rt) * prt;
        lnphi = ratio * z_minus_one - log_free - coefficient * log_factor;
    }
    return isfinite(z) && !wany<S>(c.comp && !isfinite(lnphi));
}

// Stability provider (pr76_stability.hpp:36-119): ln phi of the minimum-Gibbs
// admissible root at x.
template <int NM, int S>
__device__ int stability_provider(WCell<NM, S>& c, double x, double& out, bool& smooth, int counter_row,
                                  double* hint = nullptr) {
    ++c.counters[counter_row];
    double s, amix, bmix, A, B;
    if (!mix(c, x, s, amix, bmix)) return kRootRange;
    if (!fp64::coefficients(c.p, c.t, amix, bmix, A, B)) return kRootRange;
    fp64::RootSet rs;
    roots_by_interval<S>(A, B, rs, c.counters[cRootIters], hint);
    if (rs.status != fp64::kRootSuccess) return fp64::root_issue(rs.status);
    double phi[2] = {0.0, 0.0};
    int cand[2] = {0, 0};
    int ncand = 0;
    for (int k = 0; k < rs.count; ++k) {
        if (rs.r[k].slope_sign <= 0) continue;
        if (ncand == 2) return kRootRange;
        double v;
        if (!ln_phi(c, s, amix, bmix, A, B, rs.r[k], v)) return kRootRange;
        phi[ncand] = v;
        cand[ncand++] = k;
    }
    if (ncand == 0) return kNoAdmissibleBranch;
    int best = 0;
    smooth = true;
    if (ncand == 2) {
        const double v = wsum<S>(c.comp ? x * (phi[1] - phi[0]) : 0.0);
        if (!isfinite(v)) return kNonfinite;
        if (v < 0.0) best = 1;
        const double po = best == 1 ? phi[0] : phi[1];
        const double pb = best == 1 ? phi[1] : phi[0];
        const double magnitude = 1.0 + wsum<S>(c.comp ? x * (fabs(po) + fabs(pb)) : 0.0);
        if (!isfinite(magnitude)) return kNonfinite;
        const double d = wsum<S>(c.comp ? x * (po - pb) : 0.0);
        if (!isfinite(d)) return kNonfinite;
        if (fabs(d) <= 256.0 * kEps * magnitude) smooth = false;
    }
    if (!rs.r[cand[best]].derivative_valid) return kIllConditionedRoot;
    out = best == 1 ? phi[1] : phi[0];
    return kOk;
}

// Role provider (pr76_split.hpp:38-84): liquid = smallest, vapor = largest
// admissible root.
template <int NM, int S>
__device__ int role_provider(WCell<NM, S>& c, double x, bool vapor, double& lnphi, double& z_out, int& branch,
                             double* hint = nullptr) {
    ++c.counters[cSplitEvals];
    double s, amix, bmix, A, B;
    if (!mix(c, x, s, amix, bmix)) return kRootRange;
    if (!fp64::coefficients(c.p, c.t, amix, bmix, A, B)) return kRootRange;
    fp64::RootSet rs;
    roots_by_interval<S>(A, B, rs, c.counters[cRootIters], hint);
    if (rs.status != fp64::kRootSuccess) return fp64::root_issue(rs.status);
    int selected = -1;
    for (int k = 0; k < rs.count; ++k) {
        if (rs.r[k].slope_sign <= 0) continue;
        selected = k;
        if (!vapor) break;
    }
    if (selected < 0) return kNoAdmissibleBranch;
    if (!rs.r[selected].derivative_valid) return kIllConditionedRoot;
    if (!ln_phi(c, s, amix, bmix, A, B, rs.r[selected], lnphi)) return kRootRange;
    z_out = rs.r[selected].z;
    branch = selected;
    if (!isfinite(z_out) || z_out <= 0.0) return kIllConditionedRoot;
    return kOk;
}

// ---------------------------------------------------------------------------
// Tangent-plane distance (pt_stability.hpp:178-220).
struct Tpd {
    double w, res, lw;  // per lane
    double value, guard, stat;
    bool smooth;
    double root_hint;  // per lane: the cubic root of this lane's interval (Newton start of the next point)
};

template <int NM, int S>
__device__ int tpd(const WCell<NM, S>& c, double phiw, double phiref, Tpd& pt) {
    if (wany<S>(c.comp && (!isfinite(pt.w) || pt.w < 0.0 || pt.w > 1.0))) return kDomain;
    const double sum = wsum<S>(c.comp ? pt.w : 0.0);
    if (!(fabs(sum - 1.0) <= 64.0 * kEps)) return kDomain;
    pt.res = 0.0;
    bool domain = false, boundary = false;
    double wq = 0.0, mag = 0.0;
    if (c.comp) {
        if (c.z == 0.0) {
            domain = pt.w != 0.0;
        } else if (pt.w == 0.0) {
            boundary = true;
        } else {
            const double w = pt.w, z = c.z;
            const double lw = log(w);
            pt.lw = lw;
            const double log_ratio = fabs(w - z) < 0.5 * z ? log1p((w - z) / z) : lw - c.lz;
            const double q = log_ratio + (phiw - phiref);
            pt.res = q;
            wq = w * q;
            mag = w * (fabs(lw) + fabs(c.lz) + fabs(phiw) + fabs(phiref));
        }
    }
    if (wany<S>(domain)) return kDomain;
    const bool any_boundary = wany<S>(boundary);
    const double value = wsum<S>(wq);
    const double magnitude = 1.0 + wsum<S>(mag);
    const double mean = value / sum;
    double r = 0.0;
    if (c.act) {
        pt.res = pt.w == 0.0 ? -INFINITY : pt.res - mean;
        r = fabs(pt.res);
    }
    pt.value = value;
    pt.stat = wmax<S>(r);
    pt.guard = 256.0 * kEps * magnitude;
    if (!isfinite(pt.value) || !isfinite(pt.guard) || (!any_boundary && !isfinite(pt.stat))) return kNonfinite;
    return kOk;
}

__device__ __forceinline__ bool tpd_negative(const Tpd& p, double tol) { return p.value < -tol - p.guard; }

// A TPD trial from `start` with the reference's descent and stopping rules
// (pt_stability.hpp:343-457); provider calls are charged to `row`.  `done`
// iterations of the reference's 512 were already made (in FP32) to reach
// `start`.
template <int NM, int S>
__device__ int trial(WCell<NM, S>& c, double start, double ref, double tol, int row, Tpd& point, int done) {
    Tpd next;
    next.w = start;
    next.root_hint = NAN;
    {
        double phi;
        bool smooth = true;
        int is = stability_provider(c, next.w, phi, smooth, row, &next.root_hint);
        if (is == kOk) is = tpd(c, phi, ref, next);
        if (is != kOk) return fp64::kPropertyFailure;
        next.smooth = smooth;
        point = next;
    }
    int iter = done;
    for (;;) {
        if (tpd_negative(point, tol)) return fp64::kNegativeTpd;
        if (!point.smooth) return fp64::kNonsmooth;
        if (point.stat <= 1e-8) return fp64::kStationary;
        if (iter >= 512) return fp64::kIterationLimit;
        const double scale = fmax(1.0, point.stat / 4.0);
        const double dir = c.act ? -point.res / scale : 0.0;
        const double slope = wsum<S>(c.act ? (point.w * point.res) * dir : 0.0);
        if (!isfinite(slope) || !(slope < 0.0)) return fp64::kLineSearchFailed;
        double alpha = 1.0;
        bool accepted = false;
        for (int bt = 0; bt < 32; ++bt, alpha *= 0.5) {
            const double cand = c.act ? point.lw + alpha * dir : -INFINITY;
            const double largest = wmax<S>(cand);
            next.w = c.act ? exp(cand - largest) : 0.0;
            const double sum = wsum<S>(next.w);
            bool positive = isfinite(sum) && sum > 0.0;
            next.w /= sum;
            if (!c.act) next.w = 0.0;
            positive = positive && !wany<S>(c.act && !(next.w > 0.0));
            if (!positive) continue;
            double phi;
            bool smooth = true;
            next.root_hint = point.root_hint;
            int is = stability_provider(c, next.w, phi, smooth, row, &next.root_hint);
            if (is == kOk) is = tpd(c, phi, ref, next);
            if (is != kOk) continue;
            next.smooth = smooth;
            bool accept = tpd_negative(next, tol);
            if (!accept) {
                const double predicted = -alpha * slope;
                const double guard = point.guard + next.guard;
                if (predicted <= guard)
                    accept = next.value <= point.value + guard && alpha / scale > 0.0 && next.stat < point.stat;
                else
                    accept = next.value <= point.value - 1e-4 * predicted;
            }
            if (accept) {
                point = next;
                accepted = true;
                break;
            }
        }
        if (!accepted) return fp64::kLineSearchFailed;
        ++iter;
        ++c.counters[cTrialIters];
    }
}

// ---------------------------------------------------------------------------
// Split state (pt_split.hpp:300-341), per-lane components.
struct Split {
    double x, y, lnk, res, common, lnphi_l, lnphi_v;  // per lane
    double beta, z_l, z_v, gibbs, guard, fug, mass_abs, mass_rel;
    int branch_l, branch_v;
    double hint_l, hint_v;  // per lane: each phase's cubic root of this lane's interval
};

// Rachford-Rice by bracketed Newton (rachford_rice.hpp:70-147 checks).
template <int NM, int S>
__device__ int rachford_rice(WCell<NM, S>& c, double lk, Split& s, double beta0 = 0.5) {
    const double contrast = wmax<S>(c.act ? fabs(lk) : 0.0);
    if (contrast == 0.0) return fp64::kRrDegenerate;
    double ls[2];
    for (int k = 0; k < 2; ++k) {
        const double sign = k == 0 ? 1.0 : -1.0;
        const double arg = c.act ? c.lz + sign * lk : -INFINITY;
        const double largest = wmax<S>(arg);
        const double sum = wsum<S>(c.act ? exp(arg - largest) : 0.0);
        ls[k] = largest + log(sum);
    }
    if (!isfinite(ls[0]) || !isfinite(ls[1])) return fp64::kRrUnrepresentable;
    if (ls[0] <= 64.0 * kEps || ls[1] <= 64.0 * kEps) return fp64::kRrNoInterior;
    const double e = c.act ? exp(-fabs(lk)) : 0.0;
    const double num = c.act ? (lk >= 0.0 ? -expm1(-lk) : expm1(lk)) : 0.0;
    const bool pos = lk >= 0.0;
    auto den_at = [&](double beta) { return pos ? beta + (1.0 - beta) * e : (1.0 - beta) + beta * e; };
    // Newton from beta0 (the root of a nearby ln K: the previous iterate's)
    double left = 0.0, right = 1.0, beta = beta0 > 0.0 && beta0 < 1.0 ? beta0 : 0.5, value = 0.0;
    bool resolved = false;
    for (int it = 0; it < 64; ++it) {
        ++c.counters[cRrIters];
        double term = 0.0, dterm = 0.0;
        if (c.act) {
            const double den = den_at(beta);
            const double dd = pos ? 1.0 - e : e - 1.0;
            term = (c.z / den) * num;
            dterm = -term * dd / den;
        }
        value = wsum<S>(term);
        const double dv = wsum<S>(dterm);
        if (!isfinite(value)) return fp64::kRrUnrepresentable;
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
            value = wsum<S>(c.act ? (c.z / den_at(beta)) * num : 0.0);
            resolved = true;
            break;
        }
    }
    for (int it = 0; it < 192 && !resolved; ++it) {
        ++c.counters[cRrIters];
        beta = (left + right) * 0.5;
        if (!(beta > 0.0 && beta < 1.0)) break;
        value = wsum<S>(c.act ? (c.z / den_at(beta)) * num : 0.0);
        if (!isfinite(value)) return fp64::kRrUnrepresentable;
        if (value == 0.0 || beta == left || beta == right || right - left <= 8.0 * kEps * fmin(beta, 1.0 - beta)) {
            resolved = true;
            break;
        }
        if (value > 0.0) left = beta; else right = beta;
    }
    if (!resolved) return fp64::kRrIterLimit;
    if (fabs(value) > 64.0 * kEps) return fp64::kRrUnrepresentable;
    s.x = 0.0;
    s.y = 0.0;
    bool bad = false;
    if (c.act) {
        const double larger = c.z / den_at(beta);
        s.x = pos ? larger * e : larger;
        s.y = pos ? larger : larger * e;
        bad = !isfinite(larger) || !(s.x > 0.0 && s.y > 0.0);
    }
    if (wany<S>(bad)) return fp64::kRrUnrepresentable;
    const double sx = wsum<S>(s.x), sy = wsum<S>(s.y);
    if (fabs(sx - 1.0) > 64.0 * kEps || fabs(sy - 1.0) > 64.0 * kEps) return fp64::kRrUnrepresentable;
    s.x /= sx;
    s.y /= sy;
    double err_abs = 0.0, err_rel = 0.0;
    if (c.comp) {
        const double recovered = fma(beta, s.y, (1.0 - beta) * s.x);
        const double err = fabs(recovered - c.z);
        err_abs = err;
        if (c.z > 0.0) {
            bad = !(s.x > 0.0 && s.y > 0.0);
            err_rel = err / c.z;
        } else {
            bad = recovered != 0.0;
        }
    }
    if (wany<S>(bad)) return fp64::kRrUnrepresentable;
    s.mass_abs = wmax<S>(err_abs);
    s.mass_rel = wmax<S>(err_rel);
    s.beta = beta;
    return fp64::kRrInterior;
}

// Split evaluation at ln K (pt_split.hpp:300-341).  `near` (optional): a
// nearby state whose beta and cubic roots start the Rachford-Rice and root
// Newton iterations.
template <int NM, int S>
__device__ int split_evaluate(WCell<NM, S>& c, double lk, Split& s, int& evals, int budget, double beta0 = 0.5,
                              const Split* near = nullptr) {
    s.hint_l = near ? near->hint_l : NAN;
    s.hint_v = near ? near->hint_v : NAN;
    const int rr = rachford_rice(c, lk, s, beta0);
    if (rr != fp64::kRrInterior)
        return rr == fp64::kRrDegenerate ? fp64::kIndistinguishable
                                         : (rr == fp64::kRrNoInterior ? fp64::kNoInteriorRr : fp64::kRrFailure);
    if (evals >= budget) return fp64::kAttemptEvaluationLimit;
    ++evals;
    if (role_provider(c, s.x, false, s.lnphi_l, s.z_l, s.branch_l, &s.hint_l) != kOk)
        return fp64::kAttemptPropertyFailure;
    if (evals >= budget) return fp64::kAttemptEvaluationLimit;
    ++evals;
    if (role_provider(c, s.y, true, s.lnphi_v, s.z_v, s.branch_v, &s.hint_v) != kOk)
        return fp64::kAttemptPropertyFailure;
    s.lnk = 0.0;
    s.res = 0.0;
    s.common = 0.0;
    double g = 0.0, mag = 0.0, r = 0.0;
    bool bad = false;
    if (c.act) {
        const double lx = log(s.x), ly = log(s.y);
        const double mu_l = lx + s.lnphi_l, mu_v = ly + s.lnphi_v;
        s.lnk = ly - lx;
        s.res = (lx - ly) + (s.lnphi_l - s.lnphi_v);
        s.common = (mu_l + mu_v) * 0.5;
        r = fabs(s.res);
        g = (1.0 - s.beta) * s.x * mu_l + s.beta * s.y * mu_v;
        mag = (1.0 - s.beta) * s.x * (fabs(lx) + fabs(s.lnphi_l)) + s.beta * s.y * (fabs(ly) + fabs(s.lnphi_v));
        bad = !isfinite(s.res) || !isfinite(s.common);
    }
    if (wany<S>(bad)) return fp64::kAttemptPropertyFailure;
    s.fug = wmax<S>(r);
    s.gibbs = wsum<S>(g);
    s.guard = 256.0 * kEps * (1.0 + wsum<S>(mag));
    if (!isfinite(s.gibbs) || !isfinite(s.guard)) return fp64::kAttemptPropertyFailure;
    return fp64::kConverged;
}

// A ln K attempt continued from `lk0` (pt_split.hpp:349-407): the reference's
// convergence and acceptance tests, Gibbs line search with 24 halvings, and
// the iterations left of the reference's 512 after the `done` the attempt
// already made in FP32 (whose iterates track the FP64 ones far above the FP32
// floor).  `point` holds the last accepted state.
template <int NM, int S>
__device__ int attempt(WCell<NM, S>& c, double lk0, Split& point, int& evals, int done) {
    Split next;
    int st = split_evaluate(c, lk0, next, evals, 20000);
    if (st != fp64::kConverged) return st;
    point = next;
    int iter = 0;
    for (;;) {
        if (point.fug <= 1e-11) {
            const double contrast = wmax<S>(c.act ? fabs(point.lnk) : 0.0);
            if (!(point.mass_abs <= 1e-12 && point.mass_rel <= 1e-10)) return fp64::kBalanceFailure;
            if (point.beta <= 1e-10 || 1.0 - point.beta <= 1e-10) return fp64::kPhaseDisappearance;
            if (contrast <= 1e-7 || point.z_v - point.z_l <= 1e-8 * fmax(point.z_v, point.z_l))
                return fp64::kIndistinguishable;
            return fp64::kConverged;
        }
        if (done + iter >= 512) return fp64::kAttemptIterationLimit;
        const double scale = fmax(1.0, point.fug / 2.0);
        double hh = 0.0, f1 = 0.0, f2 = 0.0;
        if (c.act) {
            const double cc = (point.x / c.z) * point.y;
            const double d = point.y - point.x;
            hh = d * (d / c.z);
            f1 = cc * point.res;
            f2 = (cc * point.res) * point.res;
        }
        const double h = wsum<S>(hh), first = wsum<S>(f1), second = wsum<S>(f2);
        double slope = NAN;
        if (h > 0.0 && isfinite(h) && isfinite(first) && isfinite(second))
            slope = -(point.beta * (1.0 - point.beta) * second + (first / h) * first) / scale;
        if (!isfinite(slope) || !(slope < 0.0)) return fp64::kAttemptLineSearchFailed;
        double alpha = 1.0;
        bool accepted = false;
        for (int bt = 0; bt < 24; ++bt, alpha *= 0.5) {
            const double lk = c.act ? point.lnk + (alpha / scale) * point.res : 0.0;
            st = split_evaluate(c, lk, next, evals, 20000, point.beta, &point);
            if (st == fp64::kAttemptEvaluationLimit) return st;
            if (st != fp64::kConverged) continue;
            const double predicted = -alpha * slope;
            const double guard = point.guard + next.guard;
            bool accept;
            if (predicted > guard)
                accept = next.gibbs <= point.gibbs - 1e-4 * predicted;
            else
                accept = next.gibbs <= point.gibbs + guard &&
                         (next.fug <= 1e-11 || point.fug - next.fug > 1e-4 * (alpha / scale) * point.fug);
            if (accept) {
                point = next;
                accepted = true;
                break;
            }
        }
        if (!accepted) return fp64::kAttemptLineSearchFailed;
        ++iter;
        ++c.counters[cSplitIters];
    }
}

// ---------------------------------------------------------------------------
// Newton polish of ln K with the exact FP64 Jacobian in closed form.
//
// For one phase at composition x (mole fractions as independent variables,
// the full chart of pr76_phase_ad.hpp:57-122) the PR76 ln phi_i =
// r_i (Z - 1) - ln(Z - B) - q_i G, r_i = b_i/b, q_i = 2 s_i/a - r_i,
// G = A ln((Z + (1+sqrt2)B)/(Z + (1-sqrt2)B)) / (2 sqrt2 B), has
//     d ln phi_i / d x_j = cs_i s_j + cb_i b_j + ca a_ij
// (dA/dx_j = 2 s_j p/(RT)^2, dB/dx_j = b_j p/RT, dZ from the cubic's implicit
// derivative).  On the RR manifold at fixed feed (pt_sensitivity_detail.hpp:
// 291-345) dbeta_j = (x_j y_j / z_j) / h, h = sum_k (y_k - x_k)^2 / z_k, and
//     dF_i/dlnK_j = -delta_ij - (x_j y_j / z_j) [(U^L_i - U^V_i)/h
//                   + beta dlnphiL_ij/dx_j + (1 - beta) dlnphiV_ij/dy_j]
// with U^L_i = sum_k dlnphiL_i/dx_k x_k g_k, U^V_i = sum_k dlnphiV_i/dy_k y_k g_k,
// g_k = (y_k - x_k)/z_k.  Row i lives on lane i.
struct PhiCoeffs {
    double s, cs, cb, ca;  // s and the two row coefficients per lane; ca uniform
};

template <int NM, int S>
__device__ bool phi_coeffs(const WCell<NM, S>& c, double x, double Z, PhiCoeffs& f) {
    double amix, bmix, A, B;
    if (!mix(c, x, f.s, amix, bmix)) return false;
    if (!fp64::coefficients(c.p, c.t, amix, bmix, A, B)) return false;
    const double sqrt2 = 1.4142135623730951;
    const double prt = c.p / (kR * c.t);
    const double p1 = prt / (kR * c.t), p2 = prt;  // dA/da, dB/db
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
    f.ca = -2.0 * G / amix;
    f.cs = 0.0;
    f.cb = 0.0;
    if (c.comp) {
        const double r = c.b / bmix, q = 2.0 * f.s / amix - r;
        f.cs = r * zs - zs / (Z - B) + 4.0 * G * f.s / (amix * amix) - q * gs;
        f.cb = -r * (Z - 1.0) / bmix + r * zb - (zb - p2) / (Z - B) - G * r / bmix - q * gb;
    }
    return isfinite(f.ca) && !wany<S>(!isfinite(f.cs) || !isfinite(f.cb));
}

// batched::replay_linear with the component rows on the group's lanes: lane i
// holds row i of J, sums and maxima are group reductions.
template <int NM, int S>
__device__ int replay_rows(const WCell<NM, S>& c, const double* J, const Split& st, int budget) {
    float Jf[NM];
    float row = 0.f;
#pragma unroll
    for (int j = 0; j < NM; ++j) {
        // every lane of the group takes part in the broadcast
        const bool actj = bcast<S>(c.act ? 1 : 0, j) != 0;
        const bool on = c.act && j < c.n && actj;
        Jf[j] = on ? static_cast<float>(J[j]) : 0.f;
        if (on) row += fabsf((j == c.lane ? 1.f : 0.f) + Jf[j]);
    }
    float r = c.act ? static_cast<float>(st.res) : 0.f;
    const float cw = c.act ? static_cast<float>((st.x / c.z) * st.y) : 0.f;
    const float h = static_cast<float>(wsum<S>(c.act ? (st.y - st.x) * ((st.y - st.x) / c.z) : 0.0));
    if (!(h > 0.f)) return -1;
    if (static_cast<float>(wmax<S>(static_cast<double>(row))) < 1.f - 1e-4f) return 0;
    const float guard = static_cast<float>(2.0 * st.guard);
    const float bb = static_cast<float>(st.beta * (1.0 - st.beta));
    for (int it = 0; it < budget; ++it) {
        const float fug = fmax_group<S>(fabsf(r));
        if (fug <= 1e-11f) return it;
        const float first = fsum_group<S>(cw * r), second = fsum_group<S>((cw * r) * r);
        const float scale = fmaxf(1.f, fug / 2.f);
        const float q = bb * second + (first / h) * first;
        float jr = 0.f;
#pragma unroll
        for (int j = 0; j < NM; ++j) {
            const float rj = bcast<S>(r, j);
            if (j < c.n) jr = fmaf(Jf[j], rj, jr);
        }
        const float firstj = fsum_group<S>(cw * jr), mixed = fsum_group<S>((cw * r) * jr);
        const float pq = -(bb * mixed + (first / h) * firstj);
        float alpha = 1.f;
        bool accepted = false;
        for (int bt = 0; bt < 24 && !accepted; ++bt) {
            if (alpha * q / scale > guard) {
                accepted = !(pq > 0.f) || alpha * pq <= 2.f * (1.f - 1e-4f) * scale * q;
            } else {
                const float next = fmax_group<S>(fabsf(fmaf(alpha / scale, jr, r)));
                accepted = next <= 1e-11f || fug - next > 1e-4f * (alpha / scale) * fug;
            }
            if (!accepted) alpha *= 0.5f;
        }
        if (!accepted) return -1;
        r = fmaf(alpha / scale, jr, r);
    }
    return budget;
}

// Newton polish from ln K `lk` (the FP32 solution): FP64 residual (bracketed
// Newton RR and roots), the closed-form Jacobian at the first FP64 state, at
// most 8 chord steps while |F| decreases.  True with `st` at |F| <= 1e-13, or
// where |F| stopped decreasing below 1e-11.  `replay` receives replay_rows's
// count from the FP32 end point within `budget` iterations (0 when that point
// is already converged).
template <int NM, int S>
__device__ bool polish(WCell<NM, S>& c, double lk, Split& st, int budget, int& replay, int& jacobians, int& solves) {
    int evals = 0;
    replay = 0;
    if (split_evaluate(c, lk, st, evals, 1 << 30) != fp64::kConverged) return false;
    if (st.fug <= 1e-13) return true;
    PhiCoeffs fl, fv;
    if (!phi_coeffs(c, st.x, st.z_l, fl) || !phi_coeffs(c, st.y, st.z_v, fv)) return false;
    const double g = c.act ? (st.y - st.x) / c.z : 0.0;
    const double h = wsum<S>(c.act ? (st.y - st.x) * g : 0.0);
    if (!(h > 0.0) || !isfinite(h)) return false;
    const double xg = c.act ? st.x * g : 0.0, yg = c.act ? st.y * g : 0.0;
    const double s1l = wsum<S>(fl.s * xg), s2l = wsum<S>(c.b * xg);
    const double s1v = wsum<S>(fv.s * yg), s2v = wsum<S>(c.b * yg);
    double tl = 0.0, tv = 0.0;
#pragma unroll
    for (int j = 0; j < NM; ++j) {
        const double xgj = bcast<S>(xg, j), ygj = bcast<S>(yg, j);
        if (j < c.n) {
            tl = fma(c.aij[j], xgj, tl);
            tv = fma(c.aij[j], ygj, tv);
        }
    }
    const double u = ((fl.cs * s1l + fl.cb * s2l + fl.ca * tl) - (fv.cs * s1v + fv.cb * s2v + fv.ca * tv)) / h;
    const double w = c.act ? st.x * st.y / c.z : 0.0;
    const int lane = c.lane;
    double J[NM];
#pragma unroll
    for (int j = 0; j < NM; ++j) {
        const double wj = bcast<S>(w, j);
        const double slj = bcast<S>(fl.s, j), svj = bcast<S>(fv.s, j);
        const double bj = bcast<S>(c.b, j);
        const bool actj = bcast<S>(c.act ? 1 : 0, j) != 0;
        const double phil = fl.cs * slj + fl.cb * bj + fl.ca * c.aij[j];
        const double phiv = fv.cs * svj + fv.cb * bj + fv.ca * c.aij[j];
        double v = (j == lane) ? 1.0 : 0.0;  // identity rows/columns of absent components
        if (c.act && actj) v = (j == lane ? -1.0 : 0.0) - wj * (u + st.beta * phil + (1.0 - st.beta) * phiv);
        J[j] = j < c.n ? v : 0.0;
    }
    int piv[NM];
    if (wany<S>(c.comp && !isfinite(J[0]))) return false;
    replay = replay_rows<NM, S>(c, J, st, budget);
    if (!lu_rows<NM, S>(J, c.n, piv)) return false;
    ++jacobians;
    double prev = st.fug;
    Split nx;
    for (int it = 0; it < 8; ++it) {
        ++solves;
        const double d = lu_solve_rows<NM, S>(J, c.n, piv, c.act ? -st.res : 0.0);
        if (wany<S>(c.comp && !isfinite(d))) return prev <= 1e-11;
        const double next_lk = c.act ? st.lnk + d : 0.0;
        if (split_evaluate(c, next_lk, nx, evals, 1 << 30, st.beta, &st) != fp64::kConverged) return prev <= 1e-11;
        if (!(nx.fug < prev)) return prev <= 1e-11;
        st = nx;
        prev = st.fug;
        if (prev <= 1e-13) return true;
    }
    return prev <= 1e-11;
}

// Acceptance of a fugacity-converged state (pt_split.hpp:351-362).
template <int NM, int S>
__device__ bool accepted(const WCell<NM, S>& c, const Split& st) {
    const double contrast = wmax<S>(c.act ? fabs(st.lnk) : 0.0);
    return st.fug <= 1e-11 && st.mass_abs <= 1e-12 && st.mass_rel <= 1e-10 && st.beta > 1e-10 &&
           1.0 - st.beta > 1e-10 && contrast > 1e-7 && st.z_v - st.z_l > 1e-8 * fmax(st.z_v, st.z_l);
}

// ---------------------------------------------------------------------------
// Kernels: one warp per item, items taken from the stage's queue.
template <int S>
__device__ __forceinline__ int next_item(int* cursor) {
    int item = 0;
    if (seg_lane<S>() == 0) item = atomicAdd(cursor, 1);
    return bcast<S>(item, 0);
}

template <int NM, int S>
__global__ void __launch_bounds__(128) trials64w_kernel(const Mixture* __restrict__ mix_g, batched::Workspace ws,
                                                        const double* __restrict__ p, const double* __restrict__ t) {
    using namespace batched;
    __shared__ Mixture m;
    stage_mixture(mix_g, m);
    const int lane = seg_lane<S>();
    const int total = ws.counters[qT64Items];
    for (;;) {
        const int item = next_item<S>(&ws.counters[qT64Cursor]);
        if (item >= total) break;
        const int code = ws.t64_items[item];
        const int64_t c = code >> 7;
        const int k = (code >> 2) & 31;
        const int mode = code & 3;
        const bool review = mode >= mReviewContinue;
        const int row = review ? cFinalEvals : cInitEvals;
        WCell<NM, S> cell;
        int status = fp64::kPropertyFailure;
        Tpd point;
        point.w = 0.0;
        if (load_cell(m, ws, c, p, t, cell)) {
            const int active = __popc(seg_ballot<S>(cell.act));
            double ref, tol, ex0 = 0.0, ex1 = 0.0;
            bool ok = true;
            if (review) {
                // the review normalises the feed once more (pt_stability.hpp:242, :278)
                const bool bad = cell.comp && (!isfinite(cell.z) || cell.z < 0.0 || cell.z > 1.0);
                const double sum = wsum<S>(cell.comp ? cell.z : 0.0);
                ok = !wany<S>(bad) && fabs(sum - 1.0) <= 64.0 * kEps;
                if (ok && cell.comp) {
                    cell.z /= sum;
                    cell.lz = cell.z > 0.0 ? log(cell.z) : 0.0;
                    cell.act = cell.z > 0.0;
                }
                ref = cell.comp ? ws.cand[idx(6 * NM + lane, ws.ncell, c)] : 0.0;
                ex0 = cell.comp ? ws.cand[idx(0 * NM + lane, ws.ncell, c)] : 0.0;
                ex1 = cell.comp ? ws.cand[idx(1 * NM + lane, ws.ncell, c)] : 0.0;
                tol = ws.cand_s[idx(6, ws.ncell, c)];
            } else {
                ref = cell.comp ? ws.ref_lnphi[idx(lane, ws.ncell, c)] : 0.0;
                tol = 1e-10;
            }
            const bool rerun = mode == mFeedRerun || mode == mReviewRerun;
            // the trial's start (pt_stability.hpp:294-310, extra starts :263-272)
            double w0 = 0.0;
            {
                const int n_auto = auto_starts(active);
                if (k >= n_auto) {
                    w0 = (k - n_auto == 0) ? ex0 : ex1;
                } else if (k == 0) {
                    w0 = cell.z;
                } else if (k == 1) {
                    w0 = cell.act ? 1.0 / static_cast<double>(active) : 0.0;
                } else {
                    const unsigned mask = seg_ballot<S>(cell.act);
                    const int rank = __popc(mask & ((1u << lane) - 1u));
                    w0 = cell.z * 0.1 + ((cell.act && rank == k - 2) ? 0.9 : 0.0);
                }
                if (!cell.comp) w0 = 0.0;
                w0 /= wsum<S>(w0);
                if (!cell.comp) w0 = 0.0;
            }
            double w = w0;
            if (!rerun) {
                w = cell.act ? static_cast<double>(ws.tw[idx(k * NM + lane, ws.ncell, c)]) : 0.0;
                w /= wsum<S>(w);
                if (!cell.comp) w = 0.0;
            }
            if (!ok) {
                status = fp64::kPropertyFailure;
            } else if (wany<S>(cell.act && w == 0.0)) {
                status = fp64::kUnrepresentableComposition;
            } else {
                status = trial(cell, w, ref, tol, row, point, rerun ? 0 : ws.titer[idx(k, ws.ncell, c)]);
            }
        }
        if (lane == 0) ws.t64_status[idx(k, ws.ncell, c)] = static_cast<signed char>(status);
        if (!review && status == fp64::kNegativeTpd && lane < m.n)
            ws.tw64[idx(k * NM + lane, ws.ncell, c)] = point.w;
        if (lane == 0) {
            atomicAdd(&ws.counters_out[idx(kFp64EvalRow, ws.ncell, c)], cell.counters[row]);
            add_total(ws, review ? tE64ReviewTrials : tE64FeedTrials, cell.counters[row]);
        }
    }
}

template <int NM, int S>
__global__ void __launch_bounds__(128) split64w_kernel(const Mixture* __restrict__ mix_g, batched::Workspace ws,
                                                       const double* __restrict__ p, const double* __restrict__ t) {
    using namespace batched;
    __shared__ Mixture m;
    stage_mixture(mix_g, m);
    const int lane = seg_lane<S>();
    // the counter can run past the capacity when a cell's block did not fit
    // (that cell went to the fallback); unreserved slots hold -1
    const int total = min(ws.counters[qS64Items], ws.s64_capacity);
    for (;;) {
        const int item = next_item<S>(&ws.counters[qS64Cursor]);
        if (item >= total) break;
        const int code = ws.s64_items[item];
        if (code < 0) continue;
        const int64_t c = code >> 5;
        const int order = code & kOrderMask;
        // the FP64 seed with the whole budget, or the FP32 end point with what is left
        // (an attempt without FP32 progress also starts from its exact seed)
        // (and one whose FP32 run was long: its FP64 count from the FP32 end
        // point need not be the reference's from the seed)
        const int done = ws.att_iter[idx(order, ws.ncell, c)];
        const bool from_seed = ws.fp64_items || (code & kFromSeed) || done == 0 || done >= ws.continue_limit;
        WCell<NM, S> cell;
        Split point;
        int evals = 0;
        int status = fp64::kAttemptPropertyFailure;
        if (load_cell(m, ws, c, p, t, cell)) {
            const double lk0 = !cell.comp ? 0.0
                               : (from_seed ? ws.att_lnk64[idx(order * NM + lane, ws.ncell, c)]
                                            : static_cast<double>(ws.att_lnk[idx(order * NM + lane, ws.ncell, c)]));
            status = attempt(cell, lk0, point, evals, from_seed ? 0 : done);
        }
        if (lane == 0) ws.s64_status[item] = static_cast<signed char>(status);
        if (status == fp64::kConverged) {
            double* r = ws.s64_state + static_cast<int64_t>(item) * S64Stride<NM>();
            if (lane == 0) {
                r[0] = point.gibbs;
                r[1] = point.guard;
                r[2] = point.fug;
                r[3] = point.beta;
                r[4] = point.z_l;
                r[5] = point.z_v;
            }
            if (lane < m.n) {
                r[8 + 0 * NM + lane] = point.x;
                r[8 + 1 * NM + lane] = point.y;
                r[8 + 2 * NM + lane] = point.lnk;
                r[8 + 3 * NM + lane] = point.lnphi_l;
                r[8 + 4 * NM + lane] = point.lnphi_v;
                r[8 + 5 * NM + lane] = point.common;
            }
        }
        if (lane == 0) {
            atomicAdd(&ws.counters_out[idx(kFp64EvalRow, ws.ncell, c)], cell.counters[cSplitEvals]);
            add_total(ws, tE64Split64, cell.counters[cSplitEvals]);
        }
    }
}

// Polish of every cell that reached the split stage (mirrors the lane-per-cell
// polish_kernel of pr76_batched.cuh): the minimum-Gibbs FP32 attempt, or the
// two best when FP32 cannot separate them, polished and accepted in FP64; cells
// without an accepted pair queue their unsettled attempts for split64.
template <int NM, int S>
__global__ void __launch_bounds__(128) polishw_kernel(const Mixture* __restrict__ mix_g, batched::Workspace ws,
                                                      const double* __restrict__ p, const double* __restrict__ t,
                                                      DeviceOutputs out) {
    using namespace batched;
    __shared__ Mixture m;
    stage_mixture(mix_g, m);
    const int lane = seg_lane<S>();
    const int cells = ws.counters[qSplitCells];
    for (;;) {
        const int slot = next_item<S>(&ws.counters[qPolishCursor]);
        if (slot >= cells) break;
        const int64_t c = ws.split_cells[slot];
        WCell<NM, S> cell;
        if (!load_cell(m, ws, c, p, t, cell)) {
            if (lane == 0) {
                ws.phase[c] = pFallback;
                atomicAdd(&ws.counters[qFallback], 1);
                atomicAdd(&ws.counters[sFbLoad], 1);
            }
            continue;
        }
        const int n = m.n;
        const int na = ws.att_count[c];
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
        int candidates[2] = {best, -1};
        if (best >= 0 && second >= 0) {
            const float gb = ws.att_gibbs[idx(best, ws.ncell, c)], gs = ws.att_gibbs[idx(second, ws.ncell, c)];
            const float dl = lane < n ? fabsf(ws.att_lnk[idx(best * NM + lane, ws.ncell, c)] -
                                              ws.att_lnk[idx(second * NM + lane, ws.ncell, c)])
                                      : 0.f;
            const float dist = static_cast<float>(wmax<S>(dl));
            if (gs - gb <= 1e-4f * (1.f + fabsf(gb)) && dist > 1e-2f) {
                candidates[1] = second;
                if (lane == 0) atomicAdd(&ws.counters[sCandidates2], 1);
            }
        }
        bool have = false, polish_failed = false, replay_risk = false;
        double best_g = 0.0;
        int cand_order = -1, jacobians = 0, solves = 0;
        Split st;
        for (int k = 0; k < 2 && candidates[k] >= 0; ++k) {
            const int a = candidates[k];
            const double lk = cell.comp ? static_cast<double>(ws.att_lnk[idx(a * NM + lane, ws.ncell, c)]) : 0.0;
            const int done = ws.att_iter[idx(a, ws.ncell, c)];
            int replay = 0;
            if (!polish(cell, lk, st, 512 - done, replay, jacobians, solves)) {
                polish_failed = true;
                continue;
            }
            // the reference's attempt may stop short of this pair: FP64 decides
            if (replay < 0 || done + replay > kReplayLimit) {
                replay_risk = true;
                break;
            }
            if (!accepted(cell, st)) continue;
            if (have && !(st.gibbs < best_g)) continue;
            have = true;
            best_g = st.gibbs;
            cand_order = a;
            // store_candidate
            if (lane < n) {
                ws.cand[idx(0 * NM + lane, ws.ncell, c)] = st.x;
                ws.cand[idx(1 * NM + lane, ws.ncell, c)] = st.y;
                ws.cand[idx(2 * NM + lane, ws.ncell, c)] = st.lnk;
                ws.cand[idx(3 * NM + lane, ws.ncell, c)] = st.lnphi_l;
                ws.cand[idx(4 * NM + lane, ws.ncell, c)] = st.lnphi_v;
                ws.cand[idx(5 * NM + lane, ws.ncell, c)] = st.common;
            }
            if (lane == 0) {
                ws.cand_s[idx(0, ws.ncell, c)] = st.beta;
                ws.cand_s[idx(1, ws.ncell, c)] = st.z_l;
                ws.cand_s[idx(2, ws.ncell, c)] = st.z_v;
                ws.cand_s[idx(3, ws.ncell, c)] = st.fug;
                ws.cand_s[idx(7, ws.ncell, c)] = st.guard;
            }
        }
        if (lane == 0) {
            atomicAdd(&ws.counters_out[idx(kFp64EvalRow, ws.ncell, c)], cell.counters[cSplitEvals]);
            atomicAdd(&ws.counters_out[idx(cRrIters, ws.ncell, c)], cell.counters[cRrIters]);
            if (replay_risk) atomicAdd(&ws.counters[sReplayRisk], 1);
            add_total(ws, tE64Polish, cell.counters[cSplitEvals]);
            add_count(ws, sPolishJacobians, jacobians);
            add_count(ws, sPolishSolves, solves);
        }
        if (replay_risk) {  // the exact sub-solve, or (a warm cell) every attempt from its FP64 seed
            if (lane == 0 && !mark_exact(ws, c)) {
                int cnt = 0;
                for (int a = 0; a < na; ++a) cnt += unsettled(ws.att_class[idx(a, ws.ncell, c)]);
                queue_attempts64<NM>(ws, c, na, cnt, -1, 0.0, true);
            }
            continue;
        }
        if (!have) {
            if (lane == 0) {
                // FP64 continuation of every attempt FP32 left unsettled (split64 items)
                int cnt = 0;
                for (int a = 0; a < na; ++a) cnt += unsettled(ws.att_class[idx(a, ws.ncell, c)]);
                if (cnt == 0 && warm_cell(ws, c)) {
                    ws.phase[c] = pRedo;  // the warm attempt collapsed: solve the cell cold
                    atomicAdd(&ws.counters[sWarmRedo], 1);
                    atomicAdd(&ws.counters[sWarmNoPair], 1);
                } else if (cnt == 0) {
                    ws.phase[c] = pIndeterminate;  // every attempt collapsed or ended at the limit
                    write_status_only<NM>(out, ws, c, kIndeterminate, false);
                    write_counters<NM>(out, ws, c);
                } else {
                    atomicAdd(&ws.counters[best < 0 ? sFbNoAttempt : (polish_failed ? sFbPolish : sFbRejected)], 1);
                    if (!(best < 0 && mark_exact(ws, c))) queue_attempts64<NM>(ws, c, na, cnt, -1, 0.0);
                }
            }
            continue;
        }
        // attempts FP32 left open: predicted in FP32, then compete in FP64
        int open = 0;
        for (int a = 0; a < na; ++a) open += open_attempt(ws.att_class[idx(a, ws.ncell, c)]);
        if (open > 0) {
            if (lane == 0) list_open<NM>(ws, c, na, open, cand_order, best_g);
            continue;
        }
        // begin_review (pt_split.hpp:490-512): Gibbs change against the feed,
        // its guard, the review tolerance and the imposed reference on the
        // twice-normalised feed
        const double phi = lane < n ? ws.ref_lnphi[idx(lane, ws.ncell, c)] : 0.0;
        const double feed_g = wsum<S>(cell.act ? cell.z * (cell.lz + phi) : 0.0);
        const double magnitude = 1.0 + wsum<S>(cell.act ? cell.z * (fabs(cell.lz) + fabs(phi)) : 0.0);
        const double zsum = wsum<S>(cell.comp ? cell.z : 0.0);
        const double z2 = cell.z / zsum;
        const double lz2 = z2 > 0.0 ? log(z2) : 0.0;
        if (lane < n)
            ws.cand[idx(6 * NM + lane, ws.ncell, c)] = z2 > 0.0 ? ws.cand[idx(5 * NM + lane, ws.ncell, c)] - lz2 : 0.0;
        if (lane == 0) {
            const double fug = ws.cand_s[idx(3, ws.ncell, c)];
            ws.cand_s[idx(4, ws.ncell, c)] = best_g - feed_g;
            ws.cand_s[idx(5, ws.ncell, c)] = ws.cand_s[idx(7, ws.ncell, c)] + 256.0 * kEps * magnitude;
            ws.cand_s[idx(6, ws.ncell, c)] = 1e-10 + 0.5 * fug;
            ws.phase[c] = pReview;
        }
    }
}

}  // namespace w64
}  // namespace pr76
