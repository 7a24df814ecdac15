// Host build of the plain flash kernel and the max-3-phase kernel as launched
// (flash_plain.cu and flash_max3.cu, their launches rewritten for cuda_emu.h
// by the test and named MPMC_PLAIN_SOURCE and MPMC_MAX3_SOURCE): launch
// shapes, grid-stride loops, the max3 kernel's warp per cell and lane-0
// writes (test infrastructure only).  Under the launch emulation
// __activemask() names the calling lane alone, so the max3 kernel's lanes
// take the in-order line search; tests/test_max3_warp_emulation.py checks the
// lane-parallel one.
#include "cuda_emu.h"

#include MPMC_MAX3_SOURCE
#include MPMC_PLAIN_SOURCE

namespace pr76 {
LaunchShape plain_launch_shape() { return LaunchShape{64, 2}; }  // the C ABI's default shape
}  // namespace pr76

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

// The plain kernel over the cells, then (max3 != 0) the max-3-phase kernel:
// the flash fields of mpmc_flash_outputs and the three-phase outputs.
// Returns 0, a launch error, or -1 when emulated lanes diverged.
extern "C" int host_plain_max3(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                               int64_t ncell, const double* p, const double* t, const double* z, int max3,
                               int newton_roots, int32_t* status, double* beta, double* x, double* y, double* lnk,
                               double* lnphi_l, double* lnphi_v, double* z_l, double* z_v, int32_t* counters,
                               int32_t* max3_status, double* fraction, double* x3, double* lnphi3, double* z3) {
    pr76::Mixture m;
    prepare(n, tc, pc, omega, kij, m);
    pr76::DeviceOutputs out{};
    out.status = status;
    out.beta = beta;
    out.x = x;
    out.y = y;
    out.lnk = lnk;
    out.lnphi_l = lnphi_l;
    out.lnphi_v = lnphi_v;
    out.z_l = z_l;
    out.z_v = z_v;
    out.counters = counters;
    cuda_emu::g_failed.store(false);
    cudaError_t e = MPMC_CAT(pr76::launch_plain_nm, MPMC_NM)(&m, ncell, p, t, z, out, nullptr, pr76::Hints{});
    if (e == cudaSuccess && max3) {
        const pr76::Max3Outputs out3{max3_status, fraction, x3, lnphi3, z3};
        e = MPMC_CAT(pr76::launch_max3_nm, MPMC_NM)(&m, ncell, p, t, z, out, out3, nullptr, pr76::Hints{},
                                                   newton_roots != 0);
    }
    if (cuda_emu::g_failed.load()) return -1;
    return static_cast<int>(e);
}
