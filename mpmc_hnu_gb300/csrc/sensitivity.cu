// Implicit sensitivity kernel: one thread per cell, FP64, run after a flash
// kernel has written the accepted pairs (pr76_ad.cuh).  Compiled once per
// component capacity (-DMPMC_NM).
#include "launch.h"
#include "pr76_ad.cuh"
#include "pr76_sensw.cuh"

#ifndef MPMC_NM
#error "compile with -DMPMC_NM=<capacity>"
#endif

namespace pr76 {

template <int NM>
__device__ void nan_fill(int n, int64_t ncell, int64_t cell, const DeviceOutputs& out) {
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    const int q = n + 1;
    auto put = [&](double* a, int k) {
        if (a) a[static_cast<int64_t>(k) * ncell + cell] = nan;
    };
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

// Every lane walks its own grid-stride sequence of cells, NaN-filling the
// cells without an accepted pair, and stops at its next two-phase cell; then
// the warp differentiates those cells together.  A quarter of the cells are
// two-phase at the bench distribution, so a plain grid-stride loop would keep
// three lanes of four idle through the FP64 work.  Cells [c0, c1) of the
// ncell-cell batch.
template <int NM>
__global__ void __launch_bounds__(64) sensitivity_kernel(const Mixture* __restrict__ mix_g, int64_t ncell,
                                                         int64_t c0, int64_t c1, const double* __restrict__ p,
                                                         const double* __restrict__ t,
                                                         const double* __restrict__ z, DeviceOutputs out) {
    __shared__ Mixture m;
    stage_mixture(mix_g, m);
    const int n = m.n;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    int64_t next = c0 + static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    for (;;) {
        int64_t cell = -1;
        while (next < c1) {
            const int64_t c = next;
            next += stride;
            if (out.status[c] == kTwoPhase) {
                cell = c;
                break;
            }
            nan_fill<NM>(n, ncell, c, out);
            if (out.sens_status) out.sens_status[c] = ad::sNotAccepted;
        }
        if (__all_sync(0xffffffffu, cell < 0)) break;
        if (cell < 0) continue;
        fp64::Cell<NM> c;
        c.n = n;
        c.newton = false;
        c.p = p[cell];
        c.t = t[cell];
        double feed[NM], x[NM], y[NM], lnk[NM];
        for (int i = 0; i < n; ++i) {
            const int64_t k = static_cast<int64_t>(i) * ncell + cell;
            feed[i] = z[k];
            x[i] = out.x[k];
            y[i] = out.y[k];
            lnk[i] = out.lnk[k];
        }
        int st = ad::sArithmetic;
        if (fp64::normalise_feed(c, feed) && fp64::temp_setup(m, c)) {
            ad::SensScratch<NM> s;
            st = ad::sensitivity_cell<NM>(m, c, x, y, lnk, out.beta[cell], out.z_l[cell], out.z_v[cell], s, out,
                                          ncell, cell);
        }
        // a failure (possibly after partial writes) leaves no stale values
        if (st != ad::sSuccess) nan_fill<NM>(n, ncell, cell, out);
        if (out.sens_status) out.sens_status[cell] = st;
    }
}

// The lane-group form (pr76_sensw.cuh): one group of S lanes per cell, cells
// [c0, c1) in a grid-stride loop over the groups; cells without an accepted
// pair are NaN-filled by the group's lanes together.
constexpr int kSensLanesBlock = 64;

template <int NM>
__device__ void nan_fill_group(int n, int64_t ncell, int64_t cell, const DeviceOutputs& out, int lane, int lanes) {
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    const int q = n + 1;
    auto put = [&](double* a, int k) {
        if (a) a[static_cast<int64_t>(k) * ncell + cell] = nan;
    };
    for (int k = lane; k < n * q; k += lanes) {
        put(out.dlnk, k);
        put(out.dx, k);
        put(out.dy, k);
    }
    for (int k = lane; k < q; k += lanes) {
        put(out.dbeta, k);
        put(out.dzl, k);
        put(out.dzv, k);
        put(out.drhol, k);
        put(out.drhov, k);
    }
    for (int k = lane; k < (n + 1) * (n + 2); k += lanes) {
        put(out.jl, k);
        put(out.jv, k);
    }
}

template <int NM>
__global__ void __launch_bounds__(kSensLanesBlock) sensitivity_lanes_kernel(const Mixture* __restrict__ mix_g,
                                                                            int64_t ncell, int64_t c0, int64_t c1,
                                                                            const double* __restrict__ p,
                                                                            const double* __restrict__ t,
                                                                            const double* __restrict__ z,
                                                                            DeviceOutputs out) {
    constexpr int S = w64::kSeg<NM>;
    constexpr int kGroups = kSensLanesBlock / S;
    __shared__ Mixture m;
    __shared__ sensw::GroupScratch<NM> scratch[kGroups];
    stage_mixture(mix_g, m);
    const int group = threadIdx.x / S;
    const int lane = w64::seg_lane<S>();
    sensw::GroupScratch<NM>& sh = scratch[group];
    const int64_t stride = static_cast<int64_t>(gridDim.x) * kGroups;
    for (int64_t cell = c0 + static_cast<int64_t>(blockIdx.x) * kGroups + group; cell < c1; cell += stride) {
        int st = ad::sNotAccepted;
        if (out.status[cell] == kTwoPhase) st = sensw::cell<NM, S>(m, sh, ncell, cell, p, t, z, out);
        // the group's partial writes of a failed cell come before its NaN fill
        sensw::group_sync<S>();
        if (st != ad::sSuccess) nan_fill_group<NM>(m.n, ncell, cell, out, lane, S);
        if (out.sens_status && lane == 0) out.sens_status[cell] = st;
        sensw::group_sync<S>();  // the scratch is free for the next cell
    }
}

#define MPMC_CAT2(a, b) a##b
#define MPMC_CAT(a, b) MPMC_CAT2(a, b)

cudaError_t MPMC_CAT(launch_sensitivity_nm, MPMC_NM)(const Mixture* d_mix, int64_t ncell, const double* p,
                                                       const double* t, const double* z, const DeviceOutputs& out,
                                                       cudaStream_t stream, int64_t c0, int64_t c1) {
    if (c1 < 0) c1 = ncell;
    if (c1 <= c0) return cudaSuccess;
    int device = 0, sms = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int block = 64;  // a multiple of the warp: every lane reaches the warp vote
    int64_t grid = static_cast<int64_t>(sms) * 4;
    const int64_t needed = (c1 - c0 + block - 1) / block;
    if (grid > needed) grid = needed;
    sensitivity_kernel<MPMC_NM><<<static_cast<unsigned>(grid), block, 0, stream>>>(d_mix, ncell, c0, c1, p, t, z,
                                                                                   out);
    return cudaGetLastError();
}

cudaError_t MPMC_CAT(launch_sensitivity_lanes_nm, MPMC_NM)(const Mixture* d_mix, int64_t ncell, const double* p,
                                                             const double* t, const double* z,
                                                             const DeviceOutputs& out, cudaStream_t stream,
                                                             int64_t c0, int64_t c1) {
    if (c1 < 0) c1 = ncell;
    if (c1 <= c0) return cudaSuccess;
    int device = 0, sms = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    constexpr int groups = kSensLanesBlock / w64::kSeg<MPMC_NM>;
    int64_t grid = static_cast<int64_t>(sms) * 8;
    const int64_t needed = (c1 - c0 + groups - 1) / groups;
    if (grid > needed) grid = needed;
    sensitivity_lanes_kernel<MPMC_NM><<<static_cast<unsigned>(grid), kSensLanesBlock, 0, stream>>>(
        d_mix, ncell, c0, c1, p, t, z, out);
    return cudaGetLastError();
}

}  // namespace pr76
