// Implicit sensitivity kernel: one thread per cell, FP64, run after a flash
// kernel has written the accepted pairs (pr76_ad.cuh).  Compiled once per
// component capacity (-DMPMC_NM).
#include "launch.h"
#include "pr76_ad.cuh"

#ifndef MPMC_NM
#error "compile with -DMPMC_NM=<capacity>"
#endif

namespace pr76 {

template <int NM>
__global__ void __launch_bounds__(64) sensitivity_kernel(const Mixture* __restrict__ mix_g, int64_t ncell,
                                                         const double* __restrict__ p,
                                                         const double* __restrict__ t,
                                                         const double* __restrict__ z, DeviceOutputs out) {
    __shared__ Mixture m;
    stage_mixture(mix_g, m);
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    for (int64_t cell = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; cell < ncell; cell += stride) {
        const int n = m.n;
        const int q = n + 1;
        auto put = [&](double* a, int k, double v) {
            if (a) a[static_cast<int64_t>(k) * ncell + cell] = v;
        };
        // NaN-fill first; a successful cell overwrites everything
        for (int k = 0; k < n * q; ++k) {
            put(out.dlnk, k, nan);
            put(out.dx, k, nan);
            put(out.dy, k, nan);
        }
        for (int k = 0; k < q; ++k) {
            put(out.dbeta, k, nan);
            put(out.dzl, k, nan);
            put(out.dzv, k, nan);
            put(out.drhol, k, nan);
            put(out.drhov, k, nan);
        }
        for (int k = 0; k < (n + 1) * (n + 2); ++k) {
            put(out.jl, k, nan);
            put(out.jv, k, nan);
        }
        int st = ad::sNotAccepted;
        if (out.status[cell] == kTwoPhase) {
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
            if (fp64::normalise_feed(c, feed) && fp64::temp_setup(m, c)) {
                ad::SensScratch<NM> s;
                st = ad::sensitivity_cell<NM>(m, c, x, y, lnk, out.beta[cell], out.z_l[cell], out.z_v[cell], s, out,
                                              ncell, cell);
                if (st != ad::sSuccess) {
                    // a failure after partial writes must not leave stale values
                    for (int k = 0; k < n * q; ++k) {
                        put(out.dlnk, k, nan);
                        put(out.dx, k, nan);
                        put(out.dy, k, nan);
                    }
                    for (int k = 0; k < q; ++k) {
                        put(out.dbeta, k, nan);
                        put(out.dzl, k, nan);
                        put(out.dzv, k, nan);
                        put(out.drhol, k, nan);
                        put(out.drhov, k, nan);
                    }
                    for (int k = 0; k < (n + 1) * (n + 2); ++k) {
                        put(out.jl, k, nan);
                        put(out.jv, k, nan);
                    }
                }
            } else {
                st = ad::sArithmetic;
            }
        }
        if (out.sens_status) out.sens_status[cell] = st;
    }
}

#define MPMC_CAT2(a, b) a##b
#define MPMC_CAT(a, b) MPMC_CAT2(a, b)

cudaError_t MPMC_CAT(launch_sensitivity_nm, MPMC_NM)(const Mixture* d_mix, int64_t ncell, const double* p,
                                                       const double* t, const double* z, const DeviceOutputs& out,
                                                       cudaStream_t stream) {
    if (ncell <= 0) return cudaSuccess;
    int device = 0, sms = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int block = 64;
    int64_t grid = static_cast<int64_t>(sms) * 4;
    const int64_t needed = (ncell + block - 1) / block;
    if (grid > needed) grid = needed;
    sensitivity_kernel<MPMC_NM><<<static_cast<unsigned>(grid), block, 0, stream>>>(d_mix, ncell, p, t, z, out);
    return cudaGetLastError();
}

}  // namespace pr76
