// Host build of the batched flash pipeline (flash_batched.cu with
// pr76_batched.cuh, pr76_batched64.cuh, pr76_warp64.cuh) under the launch
// emulation of cuda_emu.h (test infrastructure only).  The test rewrites the
// kernel launches of flash_batched.cu into cuda_emu::launch calls and names
// the result MPMC_BATCHED_SOURCE; everything else is the product code as the
// GPU runs it, one launch after another on host threads.
#include "cuda_emu.h"

#include MPMC_BATCHED_SOURCE

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
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            m.factor[i * n + j] = 1.0 - kij[i * n + j];
            m.factor32[i * n + j] = static_cast<float>(m.factor[i * n + j]);
        }
    for (int i = 0; i < n; ++i) m.b32[i] = static_cast<float>(m.b[i]);
}

}  // namespace

// One solve of ncell cells by the mixed form (fp64_items = 0) or the FP64
// work-queue form (1), from ln K warm starts [n ncell] when warm_lnk is not
// null (a non-finite entry makes its cell cold), as
// mpmc_gpu_flash_solve_device_warm runs it; outputs as mpmc_flash_outputs'
// flash fields; polish_stream selects the state-machine polish; stats
// (optional) receives the batch's counter slots (batched::Slot).  Returns
// 0, a CUDA error code of the orchestration, or -1 when the emulated lanes
// diverged at an intrinsic.
extern "C" int host_batched_solve(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                                  int64_t ncell, const double* p, const double* t, const double* z,
                                  const double* warm_lnk, int fp64_items, int polish_stream,
                                  int32_t* status, double* beta, double* x, double* y, double* lnk, double* lnphi_l,
                                  double* lnphi_v, double* z_l, double* z_v, int32_t* counters,
                                  int32_t* stats) {
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
    pr76::BatchedShape shape{};
    shape.fp64_items = fp64_items;
    shape.warm_lnk = warm_lnk;
    shape.polish_stream = polish_stream;
    const size_t bytes = MPMC_CAT(pr76::batched_workspace_bytes_nm, MPMC_NM)(n, ncell, fp64_items != 0,
                                                                            pr76::kS64PerCell);
    std::vector<unsigned char> scratch(bytes + 256);
    void* base = reinterpret_cast<void*>((reinterpret_cast<uintptr_t>(scratch.data()) + 255) & ~uintptr_t(255));
    cuda_emu::g_failed.store(false);
    const cudaError_t e = MPMC_CAT(pr76::launch_batched_nm, MPMC_NM)(&m, n, ncell, p, t, z, out, base, bytes, shape,
                                                                      nullptr);
    if (cuda_emu::g_failed.load()) return -1;
    // the batch's queue and statistics slots (the workspace starts with them)
    if (stats) std::memcpy(stats, base, sizeof(int32_t) * pr76::batched::qSlots);
    return static_cast<int>(e);
}
