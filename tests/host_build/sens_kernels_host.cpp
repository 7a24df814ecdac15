// Host build of the two sensitivity kernels themselves (sensitivity.cu, its
// launches rewritten for cuda_emu.h by the test and named MPMC_SENS_SOURCE):
// the per-thread sensitivity_kernel and the lane-group
// sensitivity_lanes_kernel with their launch shapes, grid-stride loops,
// NaN fills and status writes, on cells solved by the plain flash's device
// function (test infrastructure only).
#include "cuda_emu.h"

#include MPMC_SENS_SOURCE
#include "pr76_fp64.cuh"

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

}  // namespace

// Solves the cells with fp64::solve_cell, then runs one sensitivity kernel
// over them (lanes: the lane-group one).  Flash fields [.. ncell] as in
// mpmc_flash_outputs; derivative fields likewise.  Returns 0, a launch error,
// or -1 when emulated lanes diverged.
extern "C" int host_sensitivity_kernel(int n, const double* tc, const double* pc, const double* omega,
                                       const double* kij, int64_t ncell, const double* p, const double* t,
                                       const double* z, int lanes, int32_t* status, double* beta, double* x,
                                       double* y, double* lnk, double* z_l, double* z_v, int32_t* sens_status,
                                       double* dlnk, double* dbeta, double* dx, double* dy, double* dzl,
                                       double* dzv, double* drhol, double* drhov, double* jl, double* jv) {
    using namespace pr76;
    constexpr int NM = MPMC_NM;
    Mixture m;
    prepare(n, tc, pc, omega, kij, m);
    auto w = std::make_unique<fp64::Scratch<NM>>();
    const double nan = std::nan("");
    for (int64_t cell = 0; cell < ncell; ++cell) {
        fp64::Cell<NM> c;
        c.n = n;
        c.newton = false;
        c.p = p[cell];
        c.t = t[cell];
        for (int k = 0; k < cCount; ++k) c.counters[k] = 0;
        double feed[NM];
        for (int i = 0; i < n; ++i) feed[i] = z[i * ncell + cell];
        fp64::CellResult<NM> r;
        r.has_pair = false;
        const int st = fp64::solve_cell(m, c, feed, *w, r);
        status[cell] = st;
        const bool two = st == kTwoPhase;
        beta[cell] = two ? w->best.beta : nan;
        z_l[cell] = two ? w->best.z_l : nan;
        z_v[cell] = two ? w->best.z_v : nan;
        for (int i = 0; i < n; ++i) {
            x[i * ncell + cell] = two ? w->best.x[i] : nan;
            y[i * ncell + cell] = two ? w->best.y[i] : nan;
            lnk[i * ncell + cell] = two ? w->best.lnk[i] : nan;
        }
    }
    DeviceOutputs out{};
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
    cuda_emu::g_failed.store(false);
    const cudaError_t e =
        lanes ? MPMC_CAT(launch_sensitivity_lanes_nm, MPMC_NM)(&m, ncell, p, t, z, out, nullptr, 0, -1)
              : MPMC_CAT(launch_sensitivity_nm, MPMC_NM)(&m, ncell, p, t, z, out, nullptr, 0, -1);
    if (cuda_emu::g_failed.load()) return -1;
    return static_cast<int>(e);
}
