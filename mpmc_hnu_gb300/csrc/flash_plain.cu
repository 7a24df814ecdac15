// Plain FP64 flash kernel: one thread per cell running the reference
// algorithm (pr76_fp64.cuh).  Structure-of-arrays inputs are read coalesced
// (cell index fastest); the mixture constants are staged into shared memory
// once per block.
#include "launch.h"
#include "pr76_hints.cuh"

namespace pr76 {

template <int NM>
__device__ void plain_cell(const Mixture& m, int64_t ncell, int64_t cell, const double* __restrict__ p,
                           const double* __restrict__ t, const double* __restrict__ z, const DeviceOutputs& out,
                           const Hints& hints);

// Persistent grid-stride launch: the grid is sized to the SM count times a
// residency target so that every thread's local state stays in L1/L2.
template <int NM>
__global__ void __launch_bounds__(128) flash_plain_kernel(const Mixture* __restrict__ mix_g, int64_t ncell,
                                                          const double* __restrict__ p,
                                                          const double* __restrict__ t,
                                                          const double* __restrict__ z, DeviceOutputs out,
                                                          Hints hints) {
    __shared__ Mixture m;
    stage_mixture(mix_g, m);
    using namespace fp64;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t cell = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; cell < ncell; cell += stride)
        plain_cell<NM>(m, ncell, cell, p, t, z, out, hints);
}

template <int NM>
__device__ void plain_cell(const Mixture& m, int64_t ncell, int64_t cell, const double* __restrict__ p,
                           const double* __restrict__ t, const double* __restrict__ z, const DeviceOutputs& out,
                           const Hints& hints) {
    using namespace fp64;
    Cell<NM> c;
    c.n = m.n;
    c.newton = false;
    c.p = p[cell];
    c.t = t[cell];
    for (int k = 0; k < cCount; ++k) c.counters[k] = 0;
    double feed[NM];
    for (int i = 0; i < c.n; ++i) feed[i] = z[static_cast<int64_t>(i) * ncell + cell];
    Scratch<NM> w;
    CellResult<NM> r;
    r.has_pair = false;
    // caller hints: extra starts of the feed test and of the final review
    // (solve_pt_vle's initial_starts and final_starts, pt_split.hpp:415-419)
    CellHints<NM> hs;
    const bool hints_ok = load_hints<NM>(hints, feed, c.n, ncell, cell, hs);
    const int status = hints_ok ? solve_cell(m, c, feed, w, r, hs.count > 0 ? hs.ptr : nullptr, hs.count,
                                             hs.fcount > 0 ? hs.fptr : nullptr, hs.fcount, hs.options)
                                : kInvalid;
    const int n = c.n;
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    auto put = [&](double* a, int k, double v) {
        if (a) a[static_cast<int64_t>(k) * ncell + cell] = v;
    };
    if (out.status) out.status[cell] = status;
    const bool pair = r.has_pair && status != kSinglePhase && status != kInvalid;
    const SplitState<NM>& b = w.best;
    put(out.beta, 0, pair ? b.beta : nan);
    for (int i = 0; i < n; ++i) {
        if (pair) {
            put(out.x, i, b.x[i]);
            put(out.y, i, b.y[i]);
            put(out.lnk, i, b.lnk[i]);
            put(out.lnphi_l, i, b.lnphi_l[i]);
            put(out.lnphi_v, i, b.lnphi_v[i]);
        } else if (status == kSinglePhase) {
            put(out.x, i, c.z[i]);
            put(out.y, i, nan);
            put(out.lnk, i, nan);
            put(out.lnphi_l, i, r.ref_lnphi[i]);
            put(out.lnphi_v, i, nan);
        } else {
            put(out.x, i, nan);
            put(out.y, i, nan);
            put(out.lnk, i, nan);
            put(out.lnphi_l, i, nan);
            put(out.lnphi_v, i, nan);
        }
    }
    put(out.z_l, 0, pair ? b.z_l : (status == kSinglePhase ? r.ref_z : nan));
    put(out.z_v, 0, pair ? b.z_v : nan);
    if (out.counters)
        for (int k = 0; k < cCount; ++k) out.counters[static_cast<int64_t>(k) * ncell + cell] = c.counters[k];
}

// One object per component capacity: this file is compiled once per
// MPMC_NM value (4, 8, 12, 16, 20) so the instantiations build in parallel.
#ifndef MPMC_NM
#error "compile with -DMPMC_NM=<capacity>"
#endif
#define MPMC_CAT2(a, b) a##b
#define MPMC_CAT(a, b) MPMC_CAT2(a, b)

cudaError_t MPMC_CAT(launch_plain_nm, MPMC_NM)(const Mixture* d_mix, int64_t ncell, const double* p,
                                                 const double* t, const double* z, const DeviceOutputs& out,
                                                 cudaStream_t stream, const Hints& hints) {
    if (ncell <= 0) return cudaSuccess;
    int device = 0, sms = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const LaunchShape shape = plain_launch_shape();
    const int block = shape.block;
    int64_t grid = static_cast<int64_t>(sms) * shape.blocks_per_sm;
    const int64_t needed = (ncell + block - 1) / block;
    if (grid > needed) grid = needed;
    flash_plain_kernel<MPMC_NM><<<static_cast<unsigned>(grid), block, 0, stream>>>(d_mix, ncell, p, t, z, out,
                                                                                   hints);
    return cudaGetLastError();
}

}  // namespace pr76
