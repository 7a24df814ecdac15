// Implicit two-phase sensitivities on a lane group: the quantity of
// ad::sensitivity_cell (pr76_ad.cuh; differentiate_pr76_pt_vle,
// modules/flash/include/mpmc/flash/pr76_sensitivity.hpp:51-390) with component
// i of the cell on lane i of a group of S lanes.
//
// The per-thread kernel holds a cell's Jacobians, LU, right-hand sides and
// RR derivatives in a 17 KB stack frame (NM = 12) and keeps a quarter of the
// warp's lanes busy.  Here row i of every matrix belongs to lane i: the phase
// Jacobian rows and dF/d ln K sit in the group's shared memory, the factored
// rows and the solutions in registers, and the LU is the row-distributed one
// of the FP64 polish (w64::lu_rows).  The group's sums follow the per-thread
// order (every lane adds the broadcast terms in component order), so up to
// the LU solves -- whose back substitution subtracts in the other order --
// every value is the per-thread kernel's.
//
//   base point, RR linearisation   pt_sensitivity_detail.hpp:257-355
//   phase Jacobians (closed form)  pr76_phase_ad.hpp:57-122 (ad::phase_jacobian_closed)
//   LU, rcond, backward error      pt_sensitivity_detail.hpp:364-471
//   totals and their checks        pr76_sensitivity.hpp:213-385
//   closure dZ, d rho              pr76_thermodynamic_closure.hpp:279-337
#pragma once

#include "launch.h"
#include "pr76_ad.cuh"
#include "pr76_lanes.cuh"

namespace pr76 {
namespace sensw {

// One group's shared scratch.  Row strides are odd multiples of a double where
// it matters, so that lane i reading row i column j spreads over the banks.
template <int NM>
struct GroupScratch {
    double xb[NM], yb[NM], z[NM], g[NM], w[NM];  // base pair, feed, (y-x)/z, x y / z
    double root[NM], uu[NM], s[2][NM];           // sqrt(a_i), a_i'/(2 a_i), mixing row sums per phase
    double db[2 * NM + 1];                        // d beta / d v, v = [ln K (n), p, T, z_0..z_{n-2}]
    double last_x[2 * NM + 1], last_y[2 * NM + 1];  // d x_{n-1}, d y_{n-1} along v
    double row0[2][NM + 2];                       // dZ / d[p, T, x] per phase
    double rows[2][NM][NM + 3];                   // d ln phi_i / d[p, T, x] per phase, row i
    double A[NM][NM + 1];                         // dF / d ln K before factoring, row i
};

template <int S>
__device__ __forceinline__ void group_sync() {
    __syncwarp(w64::seg_mask<S>());
}

// Sum of the lanes' v in component order (the per-thread loop's order).
template <int S>
__device__ __forceinline__ double ordered_sum(double v, int n, double start = 0.0) {
    double acc = start;
#pragma unroll
    for (int j = 0; j < S; ++j) {
        const double vj = w64::bcast<S>(v, j);
        if (j < n) acc += vj;
    }
    return acc;
}

// a_ij as fp64::mix forms it: the lower index's root first.
__device__ __forceinline__ double a_mix(const Mixture& m, const double* root, double ai, int i, int j, int n) {
    if (i == j) return ai;
    return i < j ? (root[i] * m.factor[i * n + j]) * root[j] : (root[j] * m.factor[j * n + i]) * root[i];
}
// a_ij as the closed-form Jacobian forms it: row i's root first.
__device__ __forceinline__ double a_row(const Mixture& m, const double* root, double ai, int i, int j, int n) {
    return i == j ? ai : (root[i] * m.factor[i * n + j]) * root[j];
}

// fp64::mix on the group: lane i's row sum s_i in fp64::mix's order (its own
// term, then the lower components, then the higher ones), amix and bmix by
// every lane in the sequential order.  x is the group's composition in
// shared memory; ai this lane's a_i.
template <int NM, int S>
__device__ bool mix(const Mixture& m, const GroupScratch<NM>& sh, const double* x, double ai, int n, double& s,
                    double& amix, double& bmix) {
    const int lane = w64::seg_lane<S>();
    s = 0.0;
    if (lane < n) {
        s = x[lane] * ai;
        for (int j = 0; j < lane; ++j) s += x[j] * a_mix(m, sh.root, 0.0, j, lane, n);
        for (int j = lane + 1; j < n; ++j) s += x[j] * a_mix(m, sh.root, 0.0, lane, j, n);
    }
    double attraction = 0.0, covolume = 0.0;
    // the diagonal terms need a_i of every component: broadcast in order
#pragma unroll
    for (int i = 0; i < S; ++i) {
        const double a_i = w64::bcast<S>(ai, i);
        if (i < n) {
            attraction += (x[i] * a_i) * x[i];
            covolume += x[i] * m.b[i];
        }
    }
    for (int i = 0; i < n; ++i) {
        const double xr_i = x[i] * sh.root[i];
        for (int j = i + 1; j < n; ++j) {
            const double cross = (xr_i * (x[j] * sh.root[j])) * m.factor[i * n + j];
            attraction += cross;
            attraction += cross;
        }
    }
    amix = attraction;
    bmix = covolume;
    if (!isfinite(attraction) || !isfinite(covolume) || !(covolume > 0.0)) return false;
    return !w64::wany<S>(lane < n && !isfinite(s));
}

// The root index of the role (liquid: smallest, vapor: largest admissible)
// and the roots, as ad::role_branch; -1 if none.
__device__ __forceinline__ int role_of(const fp64::RootSet& rs, bool vapor) {
    if (rs.status != fp64::kRootSuccess) return -1;
    int selected = -1;
    for (int k = 0; k < rs.count; ++k) {
        if (rs.r[k].slope_sign <= 0) continue;
        selected = k;
        if (!vapor) break;
    }
    return selected;
}

// ad::phase_jacobian_closed on the group: lane i writes row 1 + i into
// sh.rows[ph][i] and entry 2 + i of row 0; lane 0 the p and T entries of row
// 0.  s is lane i's mixing row sum (also in sh.s[ph]).
template <int NM, int S>
__device__ bool phase_jacobian(const Mixture& m, GroupScratch<NM>& sh, int ph, const double* x, double ai, int n,
                               double P, double T, double s, double amix, double bmix, double A, double B,
                               const fp64::RootSet& rs, int branch) {
    const int lane = w64::seg_lane<S>();
    const bool comp = lane < n;
    const int cols = n + 2;
    if (rs.status != fp64::kRootSuccess || branch >= rs.count || !rs.r[branch].derivative_valid) return false;
    const double Z = rs.r[branch].z;
    const double sqrt2 = 1.4142135623730951;
    const double rt = kR * T;
    const double prt = P / rt;
    const double p1 = prt / rt, p2 = prt;
    const double d1 = Z + (1.0 + sqrt2) * B, d2 = Z + (1.0 - sqrt2) * B;
    const double u = (2.0 * sqrt2) * (B / d2);
    const double L = fp64::log1p_over_x(u) * u;
    const double G = A * fp64::log1p_over_x(u) / d2;
    const double fz = (3.0 * Z - 2.0 * (1.0 - B)) * Z + (A - 3.0 * B * B - 2.0 * B);
    const double fa = Z - B;
    const double fb = Z * Z - (6.0 * B + 2.0) * Z - A + 2.0 * B + 3.0 * B * B;
    auto dz_of = [&](double dA, double dB) { return -(fa * dA + fb * dB) / fz; };
    auto dg_of = [&](double dA, double dB, double dZ) {
        const double dL = (dZ + (1.0 + sqrt2) * dB) / d1 - (dZ + (1.0 - sqrt2) * dB) / d2;
        return (dA * L + A * dL) / (2.0 * sqrt2 * B) - G * dB / B;
    };
    // temperature terms: u_i on lane i, t_i = sum_j a_ij u_j x_j, a' / 2
    const double st = sqrt(T);
    if (comp) {
        const double br = 1.0 + m.kappa[lane] * (1.0 - st / m.sqrt_tc[lane]);
        const double dbr = -m.kappa[lane] / (2.0 * st * m.sqrt_tc[lane]);
        sh.uu[lane] = dbr / br;
    }
    group_sync<S>();
    double ti = 0.0;
    if (comp)
        for (int j = 0; j < n; ++j) ti += a_row(m, sh.root, ai, lane, j, n) * sh.uu[j] * x[j];
    const double ap = ordered_sum<S>(comp ? 2.0 * sh.uu[lane] * x[lane] * s : 0.0, n);
    const double dAp = A / P, dBp = B / P;
    const double dAt = A * (ap / amix - 2.0 / T), dBt = -B / T;
    const double dZp = dz_of(dAp, dBp), dZt = dz_of(dAt, dBt);
    const double dGp = dg_of(dAp, dBp, dZp), dGt = dg_of(dAt, dBt, dZt);
    const double zs = -2.0 * fa * p1 / fz, zb = -fb * p2 / fz;
    if (lane == 0) {
        sh.row0[ph][0] = dZp;
        sh.row0[ph][1] = dZt;
    }
    if (comp) sh.row0[ph][2 + lane] = zs * s + zb * m.b[lane];
    const double inv = 1.0 / d1 - 1.0 / d2;
    const double ls = zs * inv, lb = zb * inv + p2 * ((1.0 + sqrt2) / d1 - (1.0 - sqrt2) / d2);
    const double gs = (2.0 * p1 * L + A * ls) / (2.0 * sqrt2 * B), gb = A * lb / (2.0 * sqrt2 * B) - G * p2 / B;
    const double ca = -2.0 * G / amix;
    bool bad = false;
    if (comp) {
        const double r = m.b[lane] / bmix, q = 2.0 * s / amix - r;
        double* row = sh.rows[ph][lane];
        row[0] = r * dZp - (dZp - dBp) / (Z - B) - q * dGp;
        const double dqt = 2.0 * (sh.uu[lane] * s + ti) / amix - 2.0 * s * ap / (amix * amix);
        row[1] = r * dZt - (dZt - dBt) / (Z - B) - dqt * G - q * dGt;
        const double cs = r * zs - zs / (Z - B) + 4.0 * G * s / (amix * amix) - q * gs;
        const double cb = -r * (Z - 1.0) / bmix + r * zb - (zb - p2) / (Z - B) - G * r / bmix - q * gb;
        for (int j = 0; j < n; ++j) row[2 + j] = cs * sh.s[ph][j] + cb * m.b[j] + ca * a_row(m, sh.root, ai, lane, j, n);
        for (int k = 0; k < cols; ++k) bad = bad || !isfinite(row[k]);
        bad = bad || !isfinite(sh.row0[ph][2 + lane]);
    }
    if (lane == 0) bad = bad || !isfinite(dZp) || !isfinite(dZt);
    group_sync<S>();
    return !w64::wany<S>(bad);
}

// d x_i / d v and d y_i / d v on the RR manifold for i < n - 1
// (pt_sensitivity_detail.hpp:291-345), as the per-thread loop forms them.
template <int NM>
__device__ __forceinline__ void rr_dxdy(const GroupScratch<NM>& sh, int n, double beta, int i, int v, double& dx,
                                        double& dy) {
    const double dlk = v == i ? 1.0 : 0.0;
    double dz = 0.0;
    if (v >= n + 2) {
        const int j = v - n - 2;
        dz = i == j ? 1.0 : (i == n - 1 ? -1.0 : 0.0);
    }
    const double dlx = dz / sh.z[i] - ((sh.yb[i] - sh.xb[i]) / sh.z[i]) * sh.db[v] - beta * (sh.yb[i] / sh.z[i]) * dlk;
    dx = sh.xb[i] * dlx;
    dy = sh.yb[i] * (dlx + dlk);
}

// One accepted two-phase cell on the group.  Every lane returns the same
// status; on success the cell's derivative outputs are written (a failure
// may leave some written: the caller NaN-fills the cell).
template <int NM, int S>
__device__ int cell(const Mixture& m, GroupScratch<NM>& sh, int64_t ncell, int64_t c, const double* p,
                    const double* t, const double* z, const DeviceOutputs& out) {
    using namespace ad;
    const int lane = w64::seg_lane<S>();
    const int n = m.n;
    const bool comp = lane < n;
    const int q = n + 1;
    const int nv = 2 * n + 1;
    const double P = p[c], T = t[c];
    const int64_t at = static_cast<int64_t>(lane) * ncell + c;
    const double feed = comp ? z[at] : 0.0;
    const double x_in = comp ? out.x[at] : 0.0, y_in = comp ? out.y[at] : 0.0, lnk = comp ? out.lnk[at] : 0.0;
    const double beta = out.beta[c], zl = out.z_l[c], zv = out.z_v[c];
    // fp64::normalise_feed: range checks, compensated sum in component order
    if (w64::wany<S>(comp && (!isfinite(feed) || feed < 0.0 || feed > 1.0))) return sArithmetic;
    double fsum = 0.0, fcomp = 0.0;
#pragma unroll
    for (int j = 0; j < S; ++j) {
        const double fj = w64::bcast<S>(feed, j);
        if (j < n) kahan_add(fj, fsum, fcomp);
    }
    if (!(fabs(fsum - 1.0) <= 64.0 * kEps)) return sArithmetic;
    const double zi = comp ? feed / fsum : 0.0;
    // fp64::temp_setup: a_i(T) and its root
    double ai = 0.0;
    bool bad = false;
    if (comp) {
        const double reduced_root = sqrt(T) / m.sqrt_tc[lane];
        const double bracket = 1.0 + m.kappa[lane] * (1.0 - reduced_root);
        ai = (bracket * m.ac[lane]) * bracket;
        bad = !isfinite(ai) || (ai == 0.0 && bracket != 0.0) || (n > 1 && !(ai > 0.0));
        sh.root[lane] = sqrt(ai);
        sh.z[lane] = zi;
    }
    if (w64::wany<S>(bad)) return sArithmetic;
    // sensitivity_cell's acceptance checks
    if (n < 2) return sNotAccepted;
    if (w64::wany<S>(comp && !(zi > 0.0))) return sUnsupportedFeed;
    const double contrast = w64::wmax<S>(comp ? fabs(lnk) : 0.0);
    if (!(contrast > 1e-7) || !(zv - zl > 1e-8 * fmax(zv, zl))) return sPhaseBoundary;
    const double guard = 1.490116119384765625e-8;
    if (!(beta > guard) || !(1.0 - beta > guard)) return sPhaseBoundary;
    // base RR point with dependent last fractions
    const double xs = ordered_sum<S>(lane < n - 1 ? x_in : 0.0, n - 1);
    const double ys = ordered_sum<S>(lane < n - 1 ? y_in : 0.0, n - 1);
    const double xb = lane == n - 1 ? 1.0 - xs : x_in;
    const double yb = lane == n - 1 ? 1.0 - ys : y_in;
    if (w64::wany<S>(comp && (!(xb > 0.0) || !(yb > 0.0) || !isfinite(xb) || !isfinite(yb)))) return sPhaseBoundary;
    if (comp) {
        sh.xb[lane] = xb;
        sh.yb[lane] = yb;
        sh.g[lane] = (yb - xb) / zi;
        sh.w[lane] = xb * yb / zi;
    }
    const double d = yb - xb;
    const double h = ordered_sum<S>(comp ? d * d / zi : 0.0, n);
    if (!isfinite(h) || !(h > 0.0)) return sIllConditioned;
    group_sync<S>();
    // the two phases: mixing, roots and role, closed-form Jacobian
    for (int ph = 0; ph < 2; ++ph) {
        const double* x = ph == 0 ? sh.xb : sh.yb;
        double s, amix, bmix, A, B;
        if (!mix<NM, S>(m, sh, x, ai, n, s, amix, bmix) || !fp64::coefficients(P, T, amix, bmix, A, B))
            return sPropertyFailure;
        fp64::RootSet rs;
        int dummy = 0;
        fp64::solve_roots(A, B, rs, dummy);
        const int branch = role_of(rs, ph == 1);
        if (branch < 0) return sPropertyFailure;
        if (comp) sh.s[ph][lane] = s;
        group_sync<S>();
        if (!phase_jacobian<NM, S>(m, sh, ph, x, ai, n, P, T, s, amix, bmix, A, B, rs, branch))
            return sPropertyFailure;
    }
    // RR linearisation: d beta / d v (every lane, the per-thread sum), then the
    // last component's d x, d y (lane 0 writes them)
    for (int v = lane; v < nv; v += S) {
        double num = 0.0;
        for (int i = 0; i < n; ++i) {
            const double dlk = v == i ? 1.0 : 0.0;
            double dz = 0.0;
            if (v >= n + 2) {
                const int j = v - n - 2;
                dz = i == j ? 1.0 : (i == n - 1 ? -1.0 : 0.0);
            }
            num += (sh.xb[i] * sh.yb[i] / sh.z[i]) * dlk + ((sh.yb[i] - sh.xb[i]) / sh.z[i]) * dz;
        }
        sh.db[v] = num / h;
    }
    group_sync<S>();
    for (int v = lane; v < nv; v += S) {
        double lsum = 0.0, vsum = 0.0;
        for (int i = 0; i + 1 < n; ++i) {
            double dx, dy;
            rr_dxdy(sh, n, beta, i, v, dx, dy);
            lsum += dx;
            vsum += dy;
        }
        sh.last_x[v] = -lsum;
        sh.last_y[v] = -vsum;
    }
    group_sync<S>();
    // dF/dv: row i on lane i, A (v < n) into registers and shared memory, B in registers
    double J[NM], Brow[NM + 1];
#pragma unroll
    for (int k = 0; k < NM; ++k) J[k] = 0.0;
#pragma unroll
    for (int k = 0; k <= NM; ++k) Brow[k] = 0.0;
    if (comp) {
        const double* rl = sh.rows[0][lane] + 2;
        const double* rv = sh.rows[1][lane] + 2;
        auto entry = [&](int v) {
            double e = v == lane ? -1.0 : 0.0;
            for (int j = 0; j + 1 < n; ++j) {
                double dx, dy;
                rr_dxdy(sh, n, beta, j, v, dx, dy);
                e += (rl[j] - rl[n - 1]) * dx - (rv[j] - rv[n - 1]) * dy;
            }
            if (v == n) e += sh.rows[0][lane][0] - sh.rows[1][lane][0];
            if (v == n + 1) e += sh.rows[0][lane][1] - sh.rows[1][lane][1];
            return e;
        };
#pragma unroll
        for (int k = 0; k < NM; ++k)
            if (k < n) {
                J[k] = entry(k);
                sh.A[lane][k] = J[k];
            }
#pragma unroll
        for (int k = 0; k <= NM; ++k)
            if (k < q) Brow[k] = entry(n + k);
    }
    group_sync<S>();
    // LU with partial pivoting, the reference's pivot guard
    double row_abs = 0.0;
#pragma unroll
    for (int k = 0; k < NM; ++k)
        if (k < n) row_abs += fabs(J[k]);
    const double norm_inf = w64::wmax<S>(comp ? row_abs : 0.0);
    if (!(norm_inf > 0.0) || !isfinite(norm_inf)) return sIllConditioned;
    const double pivot_guard = 64.0 * kEps * n * norm_inf;
    int piv[NM];
    if (!w64::lu_rows<NM, S>(J, n, piv)) return sIllConditioned;
    bool small = false;
#pragma unroll
    for (int k = 0; k < NM; ++k)
        if (k < n && lane == piv[k]) small = small || !(fabs(J[k]) > pivot_guard);
    if (w64::wany<S>(small)) return sIllConditioned;
    // reciprocal condition from the inverse's row sums
    double inv_row = 0.0;
    bool nonfinite = false;
#pragma unroll
    for (int col = 0; col < NM; ++col) {
        if (col >= n) break;
        const double e = w64::lu_solve_rows<NM, S>(J, n, piv, lane == col ? 1.0 : 0.0);
        nonfinite = nonfinite || (comp && !isfinite(e));
        inv_row += comp ? fabs(e) : 0.0;
    }
    if (w64::wany<S>(nonfinite)) return sIllConditioned;
    const double inv_norm = w64::wmax<S>(inv_row);
    const double prod = norm_inf * inv_norm;
    const double rcond = (prod > 0.0 && isfinite(prod)) ? 1.0 / prod : 0.0;
    if (!isfinite(rcond) || !(rcond > 256.0 * kEps * n)) return sIllConditioned;
    // X = -A^{-1} B, column by column
    double X[NM + 1];
#pragma unroll
    for (int col = 0; col <= NM; ++col) {
        X[col] = 0.0;
        if (col >= q) continue;
        const double xcol = w64::lu_solve_rows<NM, S>(J, n, piv, comp ? -Brow[col] : 0.0);
        nonfinite = nonfinite || (comp && !isfinite(xcol));
        X[col] = comp ? xcol : 0.0;
    }
    if (w64::wany<S>(nonfinite)) return sIllConditioned;
    // backward error of the solve against the unfactored A
    const double arithmetic_scale = 8192.0 * kEps * n;
    double backward = 0.0;
#pragma unroll
    for (int col = 0; col <= NM; ++col) {
        if (col >= q) continue;
        double res = Brow[col], sc = fabs(res);
#pragma unroll
        for (int j = 0; j < NM; ++j) {
            const double xj = w64::bcast<S>(X[col], j);
            if (j < n && comp) {
                const double term = sh.A[lane][j] * xj;
                res += term;
                sc += fabs(term);
            }
        }
        if (comp) backward = fmax(backward, fabs(res) / fmax(1.0, sc));
    }
    backward = w64::wmax<S>(backward);
    if (!isfinite(backward) || backward > arithmetic_scale) return sArithmetic;
    // totals, their consistency checks, the closure, and the outputs per column
    auto put = [&](double* arr, int k, double v) {
        if (arr) arr[static_cast<int64_t>(k) * ncell + c] = v;
    };
#pragma unroll
    for (int col = 0; col <= NM; ++col) {
        if (col >= q) continue;
        double dbq = sh.db[n + col];
        double dxq = 0.0, dyq = 0.0;
        if (lane < n - 1) rr_dxdy(sh, n, beta, lane, n + col, dxq, dyq);
        if (lane == n - 1) {
            dxq = sh.last_x[n + col];
            dyq = sh.last_y[n + col];
        }
#pragma unroll
        for (int j = 0; j < NM; ++j) {
            const double xj = w64::bcast<S>(X[col], j);
            if (j >= n) continue;
            dbq += sh.db[j] * xj;
            double dxj = 0.0, dyj = 0.0;
            if (lane < n - 1) rr_dxdy(sh, n, beta, lane, j, dxj, dyj);
            if (lane == n - 1) {
                dxj = sh.last_x[j];
                dyj = sh.last_y[j];
            }
            dxq += dxj * xj;
            dyq += dyj * xj;
        }
        if (!isfinite(dbq)) return sArithmetic;
        if (w64::wany<S>(comp && (!isfinite(dxq) || !isfinite(dyq)))) return sArithmetic;
        const double lsum = ordered_sum<S>(comp ? dxq : 0.0, n), vsum = ordered_sum<S>(comp ? dyq : 0.0, n);
        if (fabs(lsum) > arithmetic_scale || fabs(vsum) > arithmetic_scale) return sArithmetic;
        bool off = false;
        if (comp) {
            const double dz = col < 2 ? 0.0 : (lane == col - 2 ? 1.0 : (lane + 1 == n ? -1.0 : 0.0));
            const double der = (1.0 - beta) * dxq + beta * dyq + (sh.yb[lane] - sh.xb[lane]) * dbq - dz;
            const double sc = fmax(1.0, fabs(dxq) + fabs(dyq) + fabs(dbq) + fabs(dz));
            off = fabs(der) > arithmetic_scale * sc;
        }
        if (w64::wany<S>(off)) return sArithmetic;
        // closure: reduced dZ/dw_k = full column k - last column
        for (int ph = 0; ph < 2; ++ph) {
            const double* r0 = sh.row0[ph];
            const double dcomp = ph == 0 ? dxq : dyq;
            const double start = col == 0 ? r0[0] : (col == 1 ? r0[1] : 0.0);
            const double dz = ordered_sum<S>(lane < n - 1 ? (r0[2 + lane] - r0[2 + n - 1]) * dcomp : 0.0, n - 1, start);
            if (lane == 0) {
                const double zph = ph == 0 ? zl : zv;
                const double rho = P / (zph * kR * T);
                const double dp = col == 0 ? 1.0 / P : 0.0;
                const double dt = col == 1 ? 1.0 / T : 0.0;
                put(ph == 0 ? out.dzl : out.dzv, col, dz);
                put(ph == 0 ? out.drhol : out.drhov, col, rho * (dp - dz / zph - dt));
            }
        }
        if (comp) {
            put(out.dlnk, lane * q + col, X[col]);
            put(out.dx, lane * q + col, dxq);
            put(out.dy, lane * q + col, dyq);
        }
        if (lane == 0) put(out.dbeta, col, dbq);
    }
    // the phase Jacobians: row 0 and rows 1..n of each
    const int cols = n + 2;
    for (int k = lane; k < (n + 1) * cols; k += S) {
        const int r = k / cols, cc = k % cols;
        put(out.jl, k, r == 0 ? sh.row0[0][cc] : sh.rows[0][r - 1][cc]);
        put(out.jv, k, r == 0 ? sh.row0[1][cc] : sh.rows[1][r - 1][cc]);
    }
    return sSuccess;
}

}  // namespace sensw
}  // namespace pr76
