// Implicit two-phase sensitivities on the device.
//
//  * phase_jacobian_closed: d[Z, ln phi_0..]/d[p, T, x_0..x_{n-1}] of one phase
//    at a fixed root index, the quantity of
//    Pr76PhaseAdWorkspace::value_and_jacobian_full
//    (modules/thermodynamics/include/mpmc/thermodynamics/pr76_phase_ad.hpp:57-122),
//    in closed form (the reference evaluates it by forward AD with Dual
//    numbers through the same functions; the two agree to rounding).
//  * sensitivity_cell: differentiate_pr76_pt_vle
//    (modules/flash/include/mpmc/flash/pr76_sensitivity.hpp:51-390).  The
//    reference differentiates F(lnK, p, T, z) = ln x - ln y + ln phi_L(x) -
//    ln phi_V(y) through its RR linearisation
//    (detail/pt_sensitivity_detail.hpp:257-355) with Dual<double,4> blocks over
//    all 2n+1 variables; here the same derivatives are assembled by the chain
//    rule from the two per-phase Jacobians taken in the reference's reduced
//    chart (the last fraction x_{n-1} = 1 - sum x_j, i.e. "column minus last
//    column"), followed by the same LU with partial pivoting, reciprocal
//    condition, backward-error and normalisation checks
//    (pt_sensitivity_detail.hpp:364-471, pr76_sensitivity.hpp:213-385) and the
//    closure dZ, d(rho) of pr76_thermodynamic_closure.hpp:279-337.
#pragma once

#include "pr76_fp64.cuh"

namespace pr76 {
namespace ad {

// d[Z, ln phi_0..]/d[p, T, x_0..x_{n-1}] of one phase in closed form, at a
// fixed root index (the quantity of Pr76PhaseAdWorkspace::
// value_and_jacobian_full, pr76_phase_ad.hpp:57-122; rows Z, ln phi_i; mole
// fractions as independent variables).  With r_i = b_i/b, q_i = 2 s_i/a - r_i
// and G = A ln((Z+(1+sqrt2)B)/(Z+(1-sqrt2)B)) / (2 sqrt2 B),
//   ln phi_i = r_i (Z - 1) - ln(Z - B) - q_i G
// and Z from the cubic's implicit derivative dZ = -(F_A dA + F_B dB)/F_Z.
// Directions: p (dA = A/p, dB = B/p), T (dA = A (a'/a - 2/T), dB = -B/T,
// ds_i = u_i s_i + sum_j a_ij u_j x_j, a' = 2 sum_i u_i x_i s_i with
// u_i = a_i'/(2 a_i) from a_i = a_c,i (1 + kappa_i (1 - sqrt(T/Tc_i)))^2),
// x_j (dA = 2 s_j p/(RT)^2, dB = b_j p/RT, ds_i = a_ij, da = 2 s_j, db = b_j).
// Returns false if the roots no longer resolve or the root is not
// derivative-valid.
template <int NM>
__device__ bool phase_jacobian_closed(const Mixture& m, fp64::Cell<NM>& c, const double* x, int branch,
                                      double* jac) {
    const int n = c.n;
    const int cols = n + 2;
    double amix, bmix, A, B;
    if (!fp64::mix(m, c, x, amix, bmix) || !fp64::coefficients(c.p, c.t, amix, bmix, A, B)) return false;
    fp64::RootSet rs;
    int dummy = 0;
    fp64::solve_roots(A, B, rs, dummy);
    if (rs.status != fp64::kRootSuccess || branch >= rs.count || !rs.r[branch].derivative_valid) return false;
    const double Z = rs.r[branch].z;
    const double sqrt2 = 1.4142135623730951;
    const double rt = kR * c.t;
    const double prt = c.p / rt;
    const double p1 = prt / rt, p2 = prt;  // dA/da, dB/db
    const double d1 = Z + (1.0 + sqrt2) * B, d2 = Z + (1.0 - sqrt2) * B;
    const double u = (2.0 * sqrt2) * (B / d2);
    const double L = fp64::log1p_over_x(u) * u;  // ln(d1 / d2)
    const double G = A * fp64::log1p_over_x(u) / d2;  // A L / (2 sqrt2 B)
    const double fz = (3.0 * Z - 2.0 * (1.0 - B)) * Z + (A - 3.0 * B * B - 2.0 * B);
    const double fa = Z - B;
    const double fb = Z * Z - (6.0 * B + 2.0) * Z - A + 2.0 * B + 3.0 * B * B;
    // per-direction helpers (db = 0 for p and T)
    auto dz_of = [&](double dA, double dB) { return -(fa * dA + fb * dB) / fz; };
    auto dg_of = [&](double dA, double dB, double dZ) {
        const double dL = (dZ + (1.0 + sqrt2) * dB) / d1 - (dZ + (1.0 - sqrt2) * dB) / d2;
        return (dA * L + A * dL) / (2.0 * sqrt2 * B) - G * dB / B;
    };
    // temperature terms
    double uu[NM], tt[NM];
    double ap = 0.0;
    const double st = sqrt(c.t);
    for (int i = 0; i < n; ++i) {
        const double br = 1.0 + m.kappa[i] * (1.0 - st / m.sqrt_tc[i]);
        const double dbr = -m.kappa[i] / (2.0 * st * m.sqrt_tc[i]);
        uu[i] = dbr / br;
    }
    for (int i = 0; i < n; ++i) {
        double ti = 0.0;
        for (int j = 0; j < n; ++j) {
            const double aij = j == i ? c.a[i] : (c.root[i] * m.factor[i * n + j]) * c.root[j];
            ti += aij * uu[j] * x[j];
        }
        tt[i] = ti;
        ap += 2.0 * uu[i] * x[i] * c.sums[i];
    }
    const double dAp = A / c.p, dBp = B / c.p;
    const double dAt = A * (ap / amix - 2.0 / c.t), dBt = -B / c.t;
    const double dZp = dz_of(dAp, dBp), dZt = dz_of(dAt, dBt);
    const double dGp = dg_of(dAp, dBp, dZp), dGt = dg_of(dAt, dBt, dZt);
    const double zs = -2.0 * fa * p1 / fz, zb = -fb * p2 / fz;  // dZ/dx_j = zs s_j + zb b_j
    jac[0 * cols + 0] = dZp;
    jac[0 * cols + 1] = dZt;
    for (int j = 0; j < n; ++j) jac[0 * cols + 2 + j] = zs * c.sums[j] + zb * m.b[j];
    // composition row coefficients (the polish's closed form)
    const double inv = 1.0 / d1 - 1.0 / d2;
    const double ls = zs * inv, lb = zb * inv + p2 * ((1.0 + sqrt2) / d1 - (1.0 - sqrt2) / d2);
    const double gs = (2.0 * p1 * L + A * ls) / (2.0 * sqrt2 * B), gb = A * lb / (2.0 * sqrt2 * B) - G * p2 / B;
    const double ca = -2.0 * G / amix;
    for (int i = 0; i < n; ++i) {
        const double si = c.sums[i];
        const double r = m.b[i] / bmix, q = 2.0 * si / amix - r;
        double* row = jac + (1 + i) * cols;
        row[0] = r * dZp - (dZp - dBp) / (Z - B) - q * dGp;
        const double dqt = 2.0 * (uu[i] * si + tt[i]) / amix - 2.0 * si * ap / (amix * amix);
        row[1] = r * dZt - (dZt - dBt) / (Z - B) - dqt * G - q * dGt;
        const double cs = r * zs - zs / (Z - B) + 4.0 * G * si / (amix * amix) - q * gs;
        const double cb = -r * (Z - 1.0) / bmix + r * zb - (zb - p2) / (Z - B) - G * r / bmix - q * gb;
        for (int j = 0; j < n; ++j) {
            const double aij = j == i ? c.a[i] : (c.root[i] * m.factor[i * n + j]) * c.root[j];
            row[2 + j] = cs * c.sums[j] + cb * m.b[j] + ca * aij;
        }
    }
    for (int k = 0; k < (n + 1) * cols; ++k)
        if (!isfinite(jac[k])) return false;
    return true;
}

// Root index of the liquid (smallest) / vapor (largest) admissible root at x.
template <int NM>
__device__ int role_branch(const Mixture& m, fp64::Cell<NM>& c, const double* x, bool vapor) {
    double amix, bmix, A, B;
    if (!fp64::mix(m, c, x, amix, bmix) || !fp64::coefficients(c.p, c.t, amix, bmix, A, B)) return -1;
    fp64::RootSet rs;
    int dummy = 0;
    fp64::solve_roots(A, B, rs, dummy);
    if (rs.status != fp64::kRootSuccess) return -1;
    int selected = -1;
    for (int k = 0; k < rs.count; ++k) {
        if (rs.r[k].slope_sign <= 0) continue;
        selected = k;
        if (!vapor) break;
    }
    return selected;
}

// PtSensitivityStatus (modules/flash/include/mpmc/flash/pt_sensitivity.hpp:16-24)
enum SensStatus : int { sSuccess = 0, sNotAccepted = 1, sPhaseBoundary = 2, sUnsupportedFeed = 3,
                        sPropertyFailure = 4, sIllConditioned = 5, sArithmetic = 6 };

template <int NM>
struct SensScratch {
    double jl[(NM + 1) * (NM + 2)], jv[(NM + 1) * (NM + 2)];
    double A[NM * NM], B[NM * (NM + 1)], lu[NM * NM], X[NM * (NM + 1)];
    double dxl[NM * (2 * NM + 1)], dyv[NM * (2 * NM + 1)], dbeta[2 * NM + 1];
    int piv[NM];
};

// LU with partial pivoting, pt_sensitivity_detail.hpp:364-420.
__device__ inline bool lu_factor(double* v, int* piv, int n, double& norm_inf) {
    norm_inf = 0.0;
    for (int r = 0; r < n; ++r) {
        double s = 0.0;
        for (int c = 0; c < n; ++c) s += fabs(v[r * n + c]);
        norm_inf = fmax(norm_inf, s);
    }
    if (!(norm_inf > 0.0) || !isfinite(norm_inf)) return false;
    const double guard = 64.0 * kEps * n * norm_inf;
    for (int c = 0; c < n; ++c) {
        int p = c;
        double mag = fabs(v[c * n + c]);
        for (int r = c + 1; r < n; ++r)
            if (fabs(v[r * n + c]) > mag) {
                mag = fabs(v[r * n + c]);
                p = r;
            }
        if (!isfinite(mag) || !(mag > guard)) return false;
        piv[c] = p;
        if (p != c)
            for (int j = 0; j < n; ++j) {
                const double tmp = v[c * n + j];
                v[c * n + j] = v[p * n + j];
                v[p * n + j] = tmp;
            }
        const double diag = v[c * n + c];
        for (int r = c + 1; r < n; ++r) {
            const double mult = v[r * n + c] / diag;
            v[r * n + c] = mult;
            for (int j = c + 1; j < n; ++j) v[r * n + j] -= mult * v[c * n + j];
        }
    }
    return true;
}
__device__ inline bool lu_solve(const double* v, const int* piv, int n, double* rhs) {
    for (int c = 0; c < n; ++c)
        if (piv[c] != c) {
            const double tmp = rhs[c];
            rhs[c] = rhs[piv[c]];
            rhs[piv[c]] = tmp;
        }
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < r; ++c) rhs[r] -= v[r * n + c] * rhs[c];
    for (int r = n - 1; r >= 0; --r) {
        for (int c = r + 1; c < n; ++c) rhs[r] -= v[r * n + c] * rhs[c];
        rhs[r] /= v[r * n + r];
        if (!isfinite(rhs[r])) return false;
    }
    return true;
}

// Sensitivity of one accepted two-phase cell.  `z` is the normalised feed,
// x, y, lnk, beta, zl, zv the accepted pair.  Writes into the outputs at
// `cell` (NaN-filled by the caller on failure).  Returns the status.
template <int NM>
__device__ int sensitivity_cell(const Mixture& m, fp64::Cell<NM>& c, const double* x_in, const double* y_in,
                                const double* lnk, double beta, double zl, double zv, SensScratch<NM>& s,
                                const DeviceOutputs& out, int64_t ncell, int64_t cell) {
    const int n = c.n;
    const int q = n + 1;
    const int nv = 2 * n + 1;
    if (n < 2) return sNotAccepted;
    for (int i = 0; i < n; ++i)
        if (!(c.z[i] > 0.0)) return sUnsupportedFeed;
    double contrast = 0.0;
    for (int i = 0; i < n; ++i) contrast = fmax(contrast, fabs(lnk[i]));
    if (!(contrast > 1e-7) || !(zv - zl > 1e-8 * fmax(zv, zl))) return sPhaseBoundary;
    const double guard = 1.490116119384765625e-8;
    if (!(beta > guard) || !(1.0 - beta > guard)) return sPhaseBoundary;
    // base RR point with dependent last fractions, pt_sensitivity_detail.hpp:269-300
    double xb[NM], yb[NM];
    double xs = 0.0, ys = 0.0;
    for (int i = 0; i + 1 < n; ++i) {
        xb[i] = x_in[i];
        yb[i] = y_in[i];
        xs += xb[i];
        ys += yb[i];
    }
    xb[n - 1] = 1.0 - xs;
    yb[n - 1] = 1.0 - ys;
    for (int i = 0; i < n; ++i)
        if (!(xb[i] > 0.0) || !(yb[i] > 0.0) || !isfinite(xb[i]) || !isfinite(yb[i])) return sPhaseBoundary;
    double h = 0.0;
    for (int i = 0; i < n; ++i) {
        const double d = yb[i] - xb[i];
        h += d * d / c.z[i];
    }
    if (!isfinite(h) || !(h > 0.0)) return sIllConditioned;
    const int bl = role_branch(m, c, xb, false);
    const int bv = role_branch(m, c, yb, true);
    if (bl < 0 || bv < 0) return sPropertyFailure;
    if (!phase_jacobian_closed<NM>(m, c, xb, bl, s.jl) || !phase_jacobian_closed<NM>(m, c, yb, bv, s.jv))
        return sPropertyFailure;
    const int cols = n + 2;
    // RR linearisation for every variable v of [lnK (n), p, T, z_0..z_{n-2}]
    for (int v = 0; v < nv; ++v) {
        auto dlk = [&](int i) { return v == i ? 1.0 : 0.0; };
        auto dz = [&](int i) {
            if (v < n + 2) return 0.0;
            const int j = v - n - 2;
            return i == j ? 1.0 : (i == n - 1 ? -1.0 : 0.0);
        };
        double num = 0.0;
        for (int i = 0; i < n; ++i) num += (xb[i] * yb[i] / c.z[i]) * dlk(i) + ((yb[i] - xb[i]) / c.z[i]) * dz(i);
        const double db = num / h;
        s.dbeta[v] = db;
        double lsum = 0.0, vsum = 0.0;
        for (int i = 0; i + 1 < n; ++i) {
            const double dlx = dz(i) / c.z[i] - ((yb[i] - xb[i]) / c.z[i]) * db - beta * (yb[i] / c.z[i]) * dlk(i);
            s.dxl[i * nv + v] = xb[i] * dlx;
            s.dyv[i * nv + v] = yb[i] * (dlx + dlk(i));
            lsum += s.dxl[i * nv + v];
            vsum += s.dyv[i * nv + v];
        }
        s.dxl[(n - 1) * nv + v] = -lsum;
        s.dyv[(n - 1) * nv + v] = -vsum;
    }
    // dF/dv by the chain rule through the per-phase Jacobians taken in the
    // reduced chart of the reference's phase evaluation (evaluate_reduced:
    // x_{n-1} = 1 - sum of the others, pr76_sensitivity_local.hpp:70-79), i.e.
    // d/dx_j - d/dx_{n-1} for j < n-1.  Contracting the full-chart columns
    // with dx (whose entries sum to zero) instead would cancel large terms.
    double res_norm = 0.0;
    for (int i = 0; i < n; ++i) {
        const double* rl = s.jl + (1 + i) * cols + 2;
        const double* rv = s.jv + (1 + i) * cols + 2;
        for (int v = 0; v < nv; ++v) {
            // d ln x_i - d ln y_i = -d ln K_i on the RR manifold (y_i = K_i x_i),
            // taken exactly: the dependent last fractions would give it only up
            // to a cancellation error of eps * sum|dx| / x_{n-1}
            double d = v == i ? -1.0 : 0.0;
            for (int j = 0; j + 1 < n; ++j)
                d += (rl[j] - rl[n - 1]) * s.dxl[j * nv + v] - (rv[j] - rv[n - 1]) * s.dyv[j * nv + v];
            if (v == n) d += s.jl[(1 + i) * cols + 0] - s.jv[(1 + i) * cols + 0];
            if (v == n + 1) d += s.jl[(1 + i) * cols + 1] - s.jv[(1 + i) * cols + 1];
            if (v < n)
                s.A[i * n + v] = d;
            else
                s.B[i * q + (v - n)] = d;
        }
    }
    (void)res_norm;
    for (int k = 0; k < n * n; ++k) s.lu[k] = s.A[k];
    double norm_inf;
    if (!lu_factor(s.lu, s.piv, n, norm_inf)) return sIllConditioned;
    // reciprocal condition from the LU inverse, pt_sensitivity_detail.hpp:450-471
    double inv_norm = 0.0;
    {
        double rows[NM];
        for (int r = 0; r < n; ++r) rows[r] = 0.0;
        for (int col = 0; col < n; ++col) {
            double e[NM];
            for (int r = 0; r < n; ++r) e[r] = r == col ? 1.0 : 0.0;
            if (!lu_solve(s.lu, s.piv, n, e)) return sIllConditioned;
            for (int r = 0; r < n; ++r) rows[r] += fabs(e[r]);
        }
        for (int r = 0; r < n; ++r) inv_norm = fmax(inv_norm, rows[r]);
    }
    const double prod = norm_inf * inv_norm;
    const double rcond = (prod > 0.0 && isfinite(prod)) ? 1.0 / prod : 0.0;
    if (!isfinite(rcond) || !(rcond > 256.0 * kEps * n)) return sIllConditioned;
    for (int col = 0; col < q; ++col) {
        double rhs[NM];
        for (int r = 0; r < n; ++r) rhs[r] = -s.B[r * q + col];
        if (!lu_solve(s.lu, s.piv, n, rhs)) return sIllConditioned;
        for (int r = 0; r < n; ++r) s.X[r * q + col] = rhs[r];
    }
    const double arithmetic_scale = 8192.0 * kEps * n;
    double backward = 0.0;
    for (int col = 0; col < q; ++col)
        for (int r = 0; r < n; ++r) {
            double res = s.B[r * q + col], sc = fabs(res);
            for (int j = 0; j < n; ++j) {
                const double term = s.A[r * n + j] * s.X[j * q + col];
                res += term;
                sc += fabs(term);
            }
            backward = fmax(backward, fabs(res) / fmax(1.0, sc));
        }
    if (!isfinite(backward) || backward > arithmetic_scale) return sArithmetic;
    // totals, pr76_sensitivity.hpp:309-333
    auto total = [&](const double* rows_v, int i, int col) {
        double v = rows_v[i * nv + n + col];
        for (int j = 0; j < n; ++j) v += rows_v[i * nv + j] * s.X[j * q + col];
        return v;
    };
    double dbeta_q[NM + 1], dx_q[NM * (NM + 1)], dy_q[NM * (NM + 1)];
    for (int col = 0; col < q; ++col) {
        double v = s.dbeta[n + col];
        for (int j = 0; j < n; ++j) v += s.dbeta[j] * s.X[j * q + col];
        dbeta_q[col] = v;
        for (int i = 0; i < n; ++i) {
            dx_q[i * q + col] = total(s.dxl, i, col);
            dy_q[i * q + col] = total(s.dyv, i, col);
        }
    }
    for (int col = 0; col < q; ++col) {
        if (!isfinite(dbeta_q[col])) return sArithmetic;
        double ls = 0.0, vs = 0.0;
        for (int i = 0; i < n; ++i) {
            if (!isfinite(dx_q[i * q + col]) || !isfinite(dy_q[i * q + col])) return sArithmetic;
            ls += dx_q[i * q + col];
            vs += dy_q[i * q + col];
        }
        if (fabs(ls) > arithmetic_scale || fabs(vs) > arithmetic_scale) return sArithmetic;
        for (int i = 0; i < n; ++i) {
            const double dz = col < 2 ? 0.0 : (i == col - 2 ? 1.0 : (i + 1 == n ? -1.0 : 0.0));
            const double der = (1.0 - beta) * dx_q[i * q + col] + beta * dy_q[i * q + col] +
                               (yb[i] - xb[i]) * dbeta_q[col] - dz;
            const double sc = fmax(1.0, fabs(dx_q[i * q + col]) + fabs(dy_q[i * q + col]) + fabs(dbeta_q[col]) + fabs(dz));
            if (fabs(der) > arithmetic_scale * sc) return sArithmetic;
        }
    }
    // closure dZ and d(rho): reduced dZ/dw_c = full column c - last column
    auto put = [&](double* arr, int k, double v) {
        if (arr) arr[static_cast<int64_t>(k) * ncell + cell] = v;
    };
    for (int ph = 0; ph < 2; ++ph) {
        const double* jac = ph == 0 ? s.jl : s.jv;
        const double* dcomp = ph == 0 ? dx_q : dy_q;
        const double zph = ph == 0 ? zl : zv;
        const double rho = c.p / (zph * kR * c.t);
        for (int col = 0; col < q; ++col) {
            double dz = col == 0 ? jac[0] : (col == 1 ? jac[1] : 0.0);
            for (int k = 0; k + 1 < n; ++k) dz += (jac[2 + k] - jac[2 + n - 1]) * dcomp[k * q + col];
            const double dp = col == 0 ? 1.0 / c.p : 0.0;
            const double dt = col == 1 ? 1.0 / c.t : 0.0;
            put(ph == 0 ? out.dzl : out.dzv, col, dz);
            put(ph == 0 ? out.drhol : out.drhov, col, rho * (dp - dz / zph - dt));
        }
    }
    for (int k = 0; k < n * q; ++k) {
        put(out.dlnk, k, s.X[k]);
        put(out.dx, k, dx_q[k]);
        put(out.dy, k, dy_q[k]);
    }
    for (int k = 0; k < q; ++k) put(out.dbeta, k, dbeta_q[k]);
    for (int k = 0; k < (n + 1) * (n + 2); ++k) {
        put(out.jl, k, s.jl[k]);
        put(out.jv, k, s.jv[k]);
    }
    return sSuccess;
}

}  // namespace ad
}  // namespace pr76
