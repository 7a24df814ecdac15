// Selected-phase property chart of one cell (FP64, one thread per cell):
// mpmc::flow::evaluate_pr76_selected_phase_property_chart
// (modules/flow/include/mpmc/flow/pr76_selected_phase_property_closure.hpp:533-822)
// over the fixed-selected-branch closure Pr76SelectedPhasePropertyClosure
// (:258-475).
//
// The reference differentiates the whole chart callback with Dual<double, 4>
// numbers, four chart columns per pass.  Here every property is first
// differentiated in the full coordinates (p, T, x_0 .. x_{n-1}) of its
// phase -- Z and ln phi by the closed form of phase_jacobian_closed, the
// density, molar mass and affine transport/caloric model by the chain rule --
// and a chart column is then read off: p and T directly, an independent mole
// fraction of phase k as the direction e_j - e_dependent (the dependent
// fraction is 1 - sum of the others, :115-157), and zero for the saturations
// and for the other phases' fractions.
//
// Checks and their classes follow the reference's order: non-finite chart
// entries (ad/runtime_differentiate.hpp:105-108), per phase the reconstructed
// fractions (:115-157), p, T and the mixture molar mass (:356-380), the EOS
// (pr76_mixture.hpp:125-219, pr76_phase.hpp:163-258: normalisation, A and B,
// the root set, the selected index, the root derivative, ln phi), then the
// densities, viscosity, enthalpy and internal energy (:382-459).
#pragma once

#include "launch.h"
#include "pr76_ad.cuh"

namespace pr76 {
namespace chart {

// mpmc_chart_status (include/mpmc_gb300_flash.h)
enum ChartStatus : int { cOk = 0, cInputDomain = 1, cEosDomain = 2, cRootUnresolved = 3, cRootIndex = 4,
                         cIllConditioned = 5, cPropertyDomain = 6 };

constexpr int kAffine = 7;  // affine model terms before the per-component ones

// Output rows of the cell: value row r at values[r * stride], derivative
// (r, column) at jac[(r * q + column) * stride]; either pointer may be null.
struct Sink {
    double* values;
    double* jac;
    int64_t stride;
    int q;
    __device__ __forceinline__ void value(int row, double v) const {
        if (values) values[static_cast<int64_t>(row) * stride] = v;
    }
    __device__ __forceinline__ void grad(int row, int col, double v) const {
        if (jac) jac[(static_cast<int64_t>(row) * q + col) * stride] = v;
    }
};

__host__ __device__ constexpr int chart_columns(int n, int phases) { return phases * n + 1; }
__host__ __device__ constexpr int chart_rows(int n, int phases) { return phases * (5 + n) + (phases - 1) * n; }

template <int NM>
struct ChartScratch {
    double x[NM];
    double jac[(NM + 1) * (NM + 2)];   // d[Z, ln phi]/d[p, T, x] of the current phase
    double lnphi[NM];
    double g[5][NM + 2];               // rho, rho_mass, mu, h, u by (p, T, x)
    double x0[NM], lnphi0[NM], dp0[NM], dt0[NM];  // phase 0, for the equilibrium rows
};

// Affine transport/caloric model of the closure's provider slot.
template <int NM>
__device__ __forceinline__ double affine(const double* c, int n, double p, double t, const double* x, double rho,
                                         double mm, double rhom, int root) {
    double f = c[0] + c[1] * p + c[2] * t;
    for (int i = 0; i < n; ++i) f += c[kAffine + i] * x[i];
    return f + c[3] * rho + c[4] * mm + c[5] * rhom + c[6] * static_cast<double>(root);
}

// Evaluates the chart of one cell and writes every value and derivative row
// through `out`.  On a failure the caller NaN-fills the cell (rows may be
// partly written).
template <int NM>
__device__ int chart_cell(const Mixture& m, const ChartParams& cp, const double* qv, const int* dep, const Sink& out,
                          ChartScratch<NM>& s) {
    const int n = m.n;
    const int P = cp.phases;
    const int q = chart_columns(n, P);
    const int prop_rows = P * (5 + n);
    const int first_block = 2 + (P - 1);
    for (int k = 0; k < q; ++k)
        if (!isfinite(qv[k])) return cInputDomain;
    const double p = qv[0], t = qv[1];
    fp64::Cell<NM> c;
    c.n = n;
    c.newton = false;
    c.p = p;
    c.t = t;
    bool temp_ready = false;
    const int cols = n + 2;
    for (int ph = 0; ph < P; ++ph) {
        const int d = dep[ph];
        if (d < 0 || d >= n) return cInputDomain;  // a pivot outside the components
        const int start = first_block + ph * (n - 1);
        // composition of the phase (:115-157)
        double sum = 0.0;
        for (int i = 0; i < n; ++i) {
            if (i == d) continue;
            const double v = qv[start + (i < d ? i : i - 1)];
            if (!(v > 0.0)) return cInputDomain;
            s.x[i] = v;
            sum += v;
        }
        s.x[d] = 1.0 - sum;
        if (!isfinite(s.x[d]) || !(s.x[d] > 0.0)) return cInputDomain;
        if (!(p > 0.0) || !(t > 0.0)) return cInputDomain;
        double mm = 0.0;
        for (int i = 0; i < n; ++i) mm += s.x[i] * cp.molar_mass[i];
        if (!isfinite(mm) || !(mm > 0.0)) return cInputDomain;
        // EOS at the selected root (pr76_mixture.hpp:125-165, pr76_phase.hpp:193-258)
        double xs = 0.0, xc = 0.0;
        for (int i = 0; i < n; ++i) {
            if (s.x[i] > 1.0) return cEosDomain;
            kahan_add(s.x[i], xs, xc);
        }
        if (fabs(xs - 1.0) > 64.0 * kEps) return cEosDomain;
        if (!temp_ready) {
            if (!fp64::temp_setup(m, c)) return cEosDomain;
            temp_ready = true;
        }
        double amix, bmix, A, B;
        if (!fp64::mix(m, c, s.x, amix, bmix) || !fp64::coefficients(p, t, amix, bmix, A, B)) return cEosDomain;
        fp64::RootSet rs;
        int iterations = 0;
        fp64::solve_roots(A, B, rs, iterations);
        if (rs.status != fp64::kRootSuccess) return cRootUnresolved;
        const int ri = cp.root_index[ph];
        if (ri < 0 || ri >= rs.count) return cRootIndex;
        if (!rs.r[ri].derivative_valid) return cIllConditioned;
        if (!fp64::ln_phi_of_root(m, c, amix, bmix, A, B, rs.r[ri], s.lnphi)) return cEosDomain;
        if (!ad::phase_jacobian_closed<NM>(m, c, s.x, ri, s.jac)) return cEosDomain;
        const double Z = rs.r[ri].z;
        // densities and the provider (:382-459)
        const double rho = p / ((Z * kR) * t);
        const double rhom = rho * mm;
        if (!isfinite(rho) || !(rho > 0.0) || !isfinite(rhom) || !(rhom > 0.0)) return cPropertyDomain;
        const double mu = affine<NM>(cp.visc, n, p, t, s.x, rho, mm, rhom, ri);
        const double h = affine<NM>(cp.enth, n, p, t, s.x, rho, mm, rhom, ri);
        if (!isfinite(mu) || !(mu > 0.0) || !isfinite(h)) return cPropertyDomain;
        const double u = h - p / rhom;
        if (!isfinite(u)) return cPropertyDomain;
        // gradients by (p, T, x_0..x_{n-1})
        for (int k = 0; k < cols; ++k) {
            const double dp = k == 0 ? 1.0 : 0.0;
            const double dt = k == 1 ? 1.0 : 0.0;
            const double dz = s.jac[k];
            const double drho = rho * (dp / p - dz / Z - dt / t);
            const double dmm = k >= 2 ? cp.molar_mass[k - 2] : 0.0;  // unit step of x_{k-2}
            const double drhom = mm * drho + rho * dmm;
            const double vx = k >= 2 ? cp.visc[kAffine + k - 2] : 0.0;
            const double hx = k >= 2 ? cp.enth[kAffine + k - 2] : 0.0;
            const double dmu =
                cp.visc[1] * dp + cp.visc[2] * dt + vx + cp.visc[3] * drho + cp.visc[4] * dmm + cp.visc[5] * drhom;
            const double dh =
                cp.enth[1] * dp + cp.enth[2] * dt + hx + cp.enth[3] * drho + cp.enth[4] * dmm + cp.enth[5] * drhom;
            s.g[0][k] = drho;
            s.g[1][k] = drhom;
            s.g[2][k] = dmu;
            s.g[3][k] = dh;
            s.g[4][k] = dh - dp / rhom + (p / rhom) * (drhom / rhom);
        }
        for (int r = 0; r < 5; ++r)
            for (int k = 0; k < cols; ++k)
                if (!isfinite(s.g[r][k])) return cPropertyDomain;
        // property rows of the phase
        const int base = ph * (5 + n);
        const double vals[5] = {rho, rhom, mu, h, u};
        const int own0 = start, own1 = start + (n - 1);  // own block [own0, own1)
        auto chart_of = [&](const double* g, int col) {
            if (col == 0) return g[0];
            if (col == 1) return g[1];
            if (col < own0 || col >= own1) return 0.0;
            const int rank = col - own0;
            const int j = rank < d ? rank : rank + 1;
            return g[2 + j] - g[2 + d];
        };
        for (int r = 0; r < 5; ++r) {
            out.value(base + r, vals[r]);
            for (int col = 0; col < q; ++col) out.grad(base + r, col, chart_of(s.g[r], col));
        }
        for (int i = 0; i < n; ++i) {
            out.value(base + 5 + i, s.lnphi[i]);
            const double* g = s.jac + (1 + i) * cols;
            for (int col = 0; col < q; ++col) out.grad(base + 5 + i, col, chart_of(g, col));
        }
        // equilibrium rows ln(x_0,i / x_k,i) + ln phi_0,i - ln phi_k,i (:660-681)
        if (ph == 0) {
            for (int i = 0; i < n; ++i) {
                s.x0[i] = s.x[i];
                s.lnphi0[i] = s.lnphi[i];
                s.dp0[i] = s.jac[(1 + i) * cols + 0];
                s.dt0[i] = s.jac[(1 + i) * cols + 1];
            }
            // every column of the rows except p, T and the other phase's own block
            for (int k = 1; k < P; ++k) {
                const int kstart = first_block + k * (n - 1);
                for (int i = 0; i < n; ++i) {
                    const int row = prop_rows + (k - 1) * n + i;
                    const double* g = s.jac + (1 + i) * cols;
                    for (int col = 2; col < q; ++col) {
                        if (col >= kstart && col < kstart + (n - 1)) continue;
                        double v = 0.0;
                        if (col >= own0 && col < own1) {
                            const int rank = col - own0;
                            const int j = rank < d ? rank : rank + 1;
                            const double dlog = (i == j ? 1.0 : 0.0) - (i == d ? 1.0 : 0.0);
                            v = dlog / s.x[i] + (g[2 + j] - g[2 + d]);
                        }
                        out.grad(row, col, v);
                    }
                }
            }
        } else {
            for (int i = 0; i < n; ++i) {
                const int row = prop_rows + (ph - 1) * n + i;
                const double* g = s.jac + (1 + i) * cols;
                const double v = (log(s.x0[i] / s.x[i]) + s.lnphi0[i]) - s.lnphi[i];
                const double gp = s.dp0[i] - g[0];
                const double gt = s.dt0[i] - g[1];
                if (!isfinite(v) || !isfinite(gp) || !isfinite(gt)) return cPropertyDomain;
                out.value(row, v);
                out.grad(row, 0, gp);
                out.grad(row, 1, gt);
                for (int rank = 0; rank < n - 1; ++rank) {
                    const int j = rank < d ? rank : rank + 1;
                    const double dlog = (i == j ? 1.0 : 0.0) - (i == d ? 1.0 : 0.0);
                    out.grad(row, own0 + rank, -(dlog / s.x[i]) - (g[2 + j] - g[2 + d]));
                }
            }
        }
    }
    return cOk;
}

// One cell of a batch: gathers its chart entries and pivots from the
// cell-fastest inputs, evaluates, and NaN-fills the cell on a failure.
template <int NM>
__device__ void run_cell(const Mixture& m, const ChartParams& cp, int64_t ncell, int64_t cell,
                         const double* __restrict__ qv, const int32_t* __restrict__ dep, const ChartOutputs& out) {
    const int n = m.n;
    const int P = cp.phases;
    const int q = chart_columns(n, P);
    const int rows = chart_rows(n, P);
    double qc[3 * NM + 1];
    for (int k = 0; k < q; ++k) qc[k] = qv[static_cast<int64_t>(k) * ncell + cell];
    int dc[3] = {n - 1, n - 1, n - 1};
    if (dep)
        for (int ph = 0; ph < P; ++ph) dc[ph] = dep[static_cast<int64_t>(ph) * ncell + cell];
    const Sink sink{out.values ? out.values + cell : nullptr, out.jacobian ? out.jacobian + cell : nullptr, ncell, q};
    ChartScratch<NM> s;
    const int st = chart_cell<NM>(m, cp, qc, dc, sink, s);
    if (st != cOk) {
        const double nan_value = nan("");
        for (int r = 0; r < rows; ++r) {
            sink.value(r, nan_value);
            for (int col = 0; col < q; ++col) sink.grad(r, col, nan_value);
        }
    }
    if (out.status) out.status[cell] = st;
}

}  // namespace chart
}  // namespace pr76
