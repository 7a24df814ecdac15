// Forward-mode AD on the device and the implicit two-phase sensitivity.
//
//  * Dual<K>: value + K tangent lanes (the device counterpart of the
//    reference's mpmc::ad::Dual<T,N>, modules/ad/include/mpmc/ad/dual.hpp:80).
//  * phase_jacobian: d[Z, ln phi_0..]/d[p, T, x_0..x_{n-1}] of one phase at a
//    fixed root index, i.e. Pr76PhaseAdWorkspace::value_and_jacobian_full
//    (modules/thermodynamics/include/mpmc/thermodynamics/pr76_phase_ad.hpp:57-122),
//    computed in ceil((n+2)/K) passes of K lanes with the first-order root IFT
//    of pr76_phase.hpp:208-222.
//  * sensitivity: differentiate_pr76_pt_vle
//    (modules/flash/include/mpmc/flash/pr76_sensitivity.hpp:51-390).  The
//    reference differentiates F(lnK, p, T, z) = ln x - ln y + ln phi_L(x) -
//    ln phi_V(y) through its RR linearisation
//    (detail/pt_sensitivity_detail.hpp:257-355) with Dual<double,4> blocks over
//    all 2n+1 variables; here the same derivatives are assembled by the chain
//    rule from the two per-phase full-chart Jacobians (the reduced last
//    fraction x_{n-1} = 1 - sum x_j contributes exactly the "full column minus
//    last column" combination), followed by the same LU with partial pivoting,
//    reciprocal condition, backward-error and normalisation checks
//    (pt_sensitivity_detail.hpp:364-471, pr76_sensitivity.hpp:213-385) and the
//    closure dZ, d(rho) of pr76_thermodynamic_closure.hpp:279-337.
#pragma once

#include "pr76_fp64.cuh"

namespace pr76 {
namespace ad {

template <int K>
struct Dual {
    double v;
    double d[K];
};

template <int K>
__device__ __forceinline__ Dual<K> cst(double v) {
    Dual<K> r;
    r.v = v;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = 0.0;
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator+(const Dual<K>& a, const Dual<K>& b) {
    Dual<K> r;
    r.v = a.v + b.v;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator-(const Dual<K>& a, const Dual<K>& b) {
    Dual<K> r;
    r.v = a.v - b.v;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator*(const Dual<K>& a, const Dual<K>& b) {
    Dual<K> r;
    r.v = a.v * b.v;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator/(const Dual<K>& a, const Dual<K>& b) {
    Dual<K> r;
    r.v = a.v / b.v;
    const double inv = 1.0 / b.v;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * inv;
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> scale(const Dual<K>& a, double s) {
    Dual<K> r;
    r.v = a.v * s;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * s;
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> shift(const Dual<K>& a, double s) {
    Dual<K> r = a;
    r.v = a.v + s;
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> dsqrt(const Dual<K>& a) {
    Dual<K> r;
    r.v = sqrt(a.v);
    const double f = 0.5 / r.v;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * f;
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> dlog(const Dual<K>& a) {
    Dual<K> r;
    r.v = log(a.v);
    const double f = 1.0 / a.v;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * f;
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> dlog1p(const Dual<K>& a) {
    Dual<K> r;
    r.v = log1p(a.v);
    const double f = 1.0 / (1.0 + a.v);
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * f;
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> log1p_over_x(const Dual<K>& u) {
    if (fabs(u.v) <= 0.125) {
        Dual<K> value = cst<K>(-1.0 / 20.0);
        for (int k = 18; k >= 0; --k) value = shift(u * value, ((k % 2 == 0) ? 1.0 : -1.0) / static_cast<double>(k + 1));
        return value;
    }
    return dlog1p(u) / u;
}

// Columns [first, first + K) of d[Z, ln phi]/d[p, T, x_0..x_{n-1}] at a fixed
// root index; `jac` is row-major (n+1) x (n+2).  Returns false if the root set
// no longer resolves or the selected root is not derivative-valid.
// The primal of every chunk is the same, so the root set is solved by the
// first chunk and reused (`have_roots`).
template <int NM, int K>
__device__ bool phase_jacobian_chunk(const Mixture& m, int n, double p, double t, const double* x, int branch,
                                     int first, double* jac, fp64::RootSet& rs, bool have_roots) {
    const int cols = n + 2;
    auto seed = [&](int col, double v) {
        Dual<K> r = cst<K>(v);
#pragma unroll
        for (int k = 0; k < K; ++k) r.d[k] = (first + k == col) ? 1.0 : 0.0;
        return r;
    };
    const Dual<K> P = seed(0, p), T = seed(1, t);
    Dual<K> xs[NM], a[NM], root[NM], sums[NM];
    Dual<K> attraction = cst<K>(0.0), covolume = cst<K>(0.0);
    const Dual<K> st = dsqrt(T);
    for (int i = 0; i < n; ++i) {
        xs[i] = seed(2 + i, x[i]);
        const Dual<K> reduced_root = scale(st, 1.0 / m.sqrt_tc[i]);
        // pr76_pure.hpp:153-159: bracket = 1 + kappa (1 - sqrt(T)/sqrt(Tc)), a = (bracket ac) bracket
        Dual<K> bracket = shift(scale(reduced_root, -m.kappa[i]), 1.0 + m.kappa[i]);
        bracket.v = 1.0 + m.kappa[i] * (1.0 - st.v / m.sqrt_tc[i]);
        a[i] = scale(bracket, m.ac[i]) * bracket;
        attraction = attraction + (xs[i] * a[i]) * xs[i];
        covolume = covolume + scale(xs[i], m.b[i]);
        sums[i] = xs[i] * a[i];
        root[i] = dsqrt(a[i]);
    }
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j) {
            const double f = m.factor[i * n + j];
            const Dual<K> cross = scale((xs[i] * root[i]) * (xs[j] * root[j]), f);
            attraction = attraction + cross;
            attraction = attraction + cross;
            const Dual<K> aij = scale(root[i], f) * root[j];
            sums[i] = sums[i] + xs[j] * aij;
            sums[j] = sums[j] + xs[i] * aij;
        }
    const Dual<K> rt = scale(T, kR);
    const Dual<K> prt = P / rt;
    const Dual<K> A = (attraction / rt) * prt;
    const Dual<K> B = covolume * prt;
    if (!have_roots) {
        int dummy = 0;
        fp64::solve_roots(A.v, B.v, rs, dummy);
    }
    if (rs.status != fp64::kRootSuccess || branch >= rs.count || !rs.r[branch].derivative_valid) return false;
    // root IFT, pr76_phase.hpp:214-221
    const double sc = rs.scale;
    const double y0 = rs.r[branch].free_volume / sc;
    const Dual<K> bs = scale(B, 1.0 / sc);
    const double inv = 1.0 / sc;
    const Dual<K> c2 = shift(scale(bs, 4.0), -inv);
    const Dual<K> c1 = scale(scale(A, 1.0 / sc), 1.0 / sc) + scale(bs, 2.0) * bs - scale(bs, 4.0 * inv);
    const Dual<K> c0 = scale(scale(bs, -2.0) * bs, inv);
    const Dual<K> residual = scale(shift(scale(shift(c2, y0), y0) + c1, 0.0), y0) + c0;
    const double dh = (3.0 * y0 + 2.0 * c2.v) * y0 + c1.v;
    Dual<K> fv = cst<K>(rs.r[branch].free_volume);
#pragma unroll
    for (int k = 0; k < K; ++k) fv.d[k] = -(residual.d[k] / dh) * sc;
    const Dual<K> z = fv + B;
    const double sqrt2 = 1.4142135623730951;
    const Dual<K> denominator = fv + scale(B, 2.0 - sqrt2);
    const Dual<K> u = scale(B / denominator, 2.0 * sqrt2);
    const Dual<K> log_factor = log1p_over_x(u) / denominator;
    Dual<K> zm1 = shift(z, -1.0);
    Dual<K> log_free = dlog(fv);
    if (fabs(zm1.v) < 0.25 && B.v < 0.125) {
        const Dual<K> bz = B / z;
        zm1 = B / fv - (A / z) / (shift(scale(bz, 2.0), 1.0) - bz * bz);
        log_free = dlog1p(zm1 - B);
    }
#pragma unroll
    for (int k = 0; k < K; ++k)
        if (first + k < cols) jac[0 * cols + first + k] = z.d[k];
    for (int i = 0; i < n; ++i) {
        const Dual<K> ratio = cst<K>(m.b[i]) / covolume;
        const Dual<K> coefficient = ((scale(sums[i], 2.0) - attraction * ratio) / rt) * prt;
        const Dual<K> lp = ratio * zm1 - log_free - coefficient * log_factor;
        if (!isfinite(lp.v)) return false;
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (first + k < cols) jac[(1 + i) * cols + first + k] = lp.d[k];
    }
    return isfinite(z.v);
}

template <int NM>
__device__ bool phase_jacobian(const Mixture& m, int n, double p, double t, const double* x, int branch,
                               double* jac) {
    constexpr int K = 4;
    fp64::RootSet rs;
    for (int first = 0; first < n + 2; first += K)
        if (!phase_jacobian_chunk<NM, K>(m, n, p, t, x, branch, first, jac, rs, first > 0)) return false;
    for (int k = 0; k < (n + 1) * (n + 2); ++k)
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
    if (!phase_jacobian<NM>(m, n, c.p, c.t, xb, bl, s.jl) || !phase_jacobian<NM>(m, n, c.p, c.t, yb, bv, s.jv))
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
