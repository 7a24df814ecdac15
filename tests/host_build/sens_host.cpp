// Host build of the two sensitivity forms (test infrastructure only).
//
// Solves each cell with the plain flash's device function (fp64::solve_cell,
// pr76_fp64.cuh) and differentiates every accepted two-phase cell either with
// the per-thread device function ad::sensitivity_cell (pr76_ad.cuh; mode bit 0
// clear) or with the lane-group one, sensw::cell (pr76_sensw.cuh; bit 0 set), on
// an emulated group of S lanes (warp_emu.h) exactly as sensitivity_lanes_kernel
// runs it.  Cells without an accepted pair, and failed ones, are NaN-filled
// as the kernels fill them.  A lane group whose lanes diverge or end with
// different statuses gives the cell status -99.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>

using std::isfinite;
#include "warp_emu.h"

#include "launch.h"
#include "pr76_sensw.cuh"

namespace {

void prepare(int n, const double* tc, const double* pc, const double* omega, const double* kij, pr76::Mixture& m) {
    std::memset(&m, 0, sizeof(m));
    m.n = n;
    for (int i = 0; i < n; ++i) {
        m.sqrt_tc[i] = std::sqrt(tc[i]);
        m.kappa[i] = 0.37464 + omega[i] * (1.54226 - 0.26992 * omega[i]);
        const double rtc = pr76::kR * tc[i];
        m.ac[i] = (0.45724 * rtc) * (rtc / pc[i]);
        m.b[i] = (0.07780 * rtc) / pc[i];
    }
    for (int k = 0; k < n * n; ++k) m.factor[k] = 1.0 - kij[k];
}

void nan_fill(int n, int64_t ncell, int64_t cell, const pr76::DeviceOutputs& out) {
    const double nan = std::nan("");
    const int q = n + 1;
    auto put = [&](double* a, int k) { a[static_cast<int64_t>(k) * ncell + cell] = nan; };
    for (int k = 0; k < n * q; ++k) {
        put(out.dlnk, k);
        put(out.dx, k);
        put(out.dy, k);
    }
    for (int k = 0; k < q; ++k) {
        put(out.dbeta, k);
        put(out.dzl, k);
        put(out.dzv, k);
        put(out.drhol, k);
        put(out.drhov, k);
    }
    for (int k = 0; k < (n + 1) * (n + 2); ++k) {
        put(out.jl, k);
        put(out.jv, k);
    }
}

template <int NM>
void run(const pr76::Mixture& m, int64_t ncell, const double* p, const double* t, const double* z, int mode,
         const pr76::DeviceOutputs& out) {
    using namespace pr76;
    const bool lanes = (mode & 1) != 0, given = (mode & 2) != 0;
    const int n = m.n;
    auto w = std::make_unique<fp64::Scratch<NM>>();
    auto s = std::make_unique<ad::SensScratch<NM>>();
    auto sh = std::make_unique<sensw::GroupScratch<NM>>();
    for (int64_t cell = 0; cell < ncell; ++cell) {
        // the flash: the plain kernel's per-cell function
        fp64::Cell<NM> c;
        c.n = n;
        c.newton = false;
        c.p = p[cell];
        c.t = t[cell];
        for (int k = 0; k < cCount; ++k) c.counters[k] = 0;
        double feed[NM];
        for (int i = 0; i < n; ++i) feed[i] = z[i * ncell + cell];
        int status = out.status[cell];
        if (!given) {
            fp64::CellResult<NM> r;
            r.has_pair = false;
            status = fp64::solve_cell(m, c, feed, *w, r);
            out.status[cell] = status;
            const double nan = std::nan("");
            out.beta[cell] = status == kTwoPhase ? w->best.beta : nan;
            out.z_l[cell] = status == kTwoPhase ? w->best.z_l : nan;
            out.z_v[cell] = status == kTwoPhase ? w->best.z_v : nan;
            for (int i = 0; i < n; ++i) {
                out.x[i * ncell + cell] = status == kTwoPhase ? w->best.x[i] : nan;
                out.y[i * ncell + cell] = status == kTwoPhase ? w->best.y[i] : nan;
                out.lnk[i * ncell + cell] = status == kTwoPhase ? w->best.lnk[i] : nan;
            }
        }
        // the sensitivities
        int st = ad::sNotAccepted;
        if (status == kTwoPhase) {
            if (lanes) {
                constexpr int S = w64::kSeg<NM>;
                std::memset(sh.get(), 0xA5, sizeof(*sh));  // no read of stale scratch goes unnoticed
                int lane_status[S];
                const bool together = warp_emu::run(S, [&](int lane) {
                    lane_status[lane] = sensw::cell<NM, S>(m, *sh, ncell, cell, p, t, z, out);
                });
                bool agree = together;
                for (int lane = 1; lane < S; ++lane) agree = agree && lane_status[lane] == lane_status[0];
                st = agree ? lane_status[0] : -99;
            } else {
                fp64::Cell<NM> cs;
                cs.n = n;
                cs.newton = false;
                cs.p = p[cell];
                cs.t = t[cell];
                for (int k = 0; k < cCount; ++k) cs.counters[k] = 0;
                double x[NM], y[NM], lnk[NM];
                for (int i = 0; i < n; ++i) {
                    feed[i] = z[i * ncell + cell];
                    x[i] = out.x[i * ncell + cell];
                    y[i] = out.y[i * ncell + cell];
                    lnk[i] = out.lnk[i * ncell + cell];
                }
                st = ad::sArithmetic;
                if (fp64::normalise_feed(cs, feed) && fp64::temp_setup(m, cs))
                    st = ad::sensitivity_cell<NM>(m, cs, x, y, lnk, out.beta[cell], out.z_l[cell], out.z_v[cell], *s,
                                                  out, ncell, cell);
            }
        }
        if (st != ad::sSuccess) nan_fill(n, ncell, cell, out);
        out.sens_status[cell] = st;
    }
}

}  // namespace

// Flash fields: status [ncell]; beta, z_l, z_v [ncell]; x, y, lnk [n ncell].
// Sensitivity fields as in mpmc_flash_outputs.  mode bit 0: the lane-group
// form; bit 1: differentiate the flash fields given in the arrays (any pair,
// to reach the failure statuses) instead of solving the cells.
extern "C" int host_sensitivity_batch(int n, const double* tc, const double* pc, const double* omega,
                                      const double* kij, int64_t ncell, const double* p, const double* t,
                                      const double* z, int mode, int32_t* status, double* beta, double* x,
                                      double* y, double* lnk, double* z_l, double* z_v, int32_t* sens_status,
                                      double* dlnk, double* dbeta, double* dx, double* dy, double* dzl, double* dzv,
                                      double* drhol, double* drhov, double* jl, double* jv) {
    if (n < 2 || n > pr76::kMaxC) return 1;
    pr76::Mixture m;
    prepare(n, tc, pc, omega, kij, m);
    pr76::DeviceOutputs out{};
    out.status = status;
    out.beta = beta;
    out.x = x;
    out.y = y;
    out.lnk = lnk;
    out.z_l = z_l;
    out.z_v = z_v;
    out.sens_status = sens_status;
    out.dlnk = dlnk;
    out.dbeta = dbeta;
    out.dx = dx;
    out.dy = dy;
    out.dzl = dzl;
    out.dzv = dzv;
    out.drhol = drhol;
    out.drhov = drhov;
    out.jl = jl;
    out.jv = jv;
    if (n <= 4) run<4>(m, ncell, p, t, z, mode, out);
    else if (n <= 8) run<8>(m, ncell, p, t, z, mode, out);
    else if (n <= 12) run<12>(m, ncell, p, t, z, mode, out);
    else if (n <= 16) run<16>(m, ncell, p, t, z, mode, out);
    else run<20>(m, ncell, p, t, z, mode, out);
    return 0;
}
