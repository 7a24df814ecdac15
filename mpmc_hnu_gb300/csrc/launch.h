// Internal host-side interface between the C ABI (capi.cu) and the kernel
// translation units.  Not part of the public boundary.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "pr76_common.cuh"

namespace pr76 {

// Device pointers of every output (any may be null), layout a[k * ncell + c].
struct DeviceOutputs {
    int32_t* status;
    double* beta;
    double* x;
    double* y;
    double* lnk;
    double* lnphi_l;
    double* lnphi_v;
    double* z_l;
    double* z_v;
    int32_t* counters;
    int32_t* sens_status;
    double* dlnk;
    double* dbeta;
    double* dx;
    double* dy;
    double* dzl;
    double* dzv;
    double* drhol;
    double* drhov;
    double* jl;
    double* jv;
};

// Launch shape of the plain kernel: threads per block and resident blocks per
// SM.  Defaults to 64 x 2; MPMC_PLAIN_BLOCK / MPMC_PLAIN_BLOCKS_PER_SM override
// them for launch-shape sweeps.
struct LaunchShape {
    int block;
    int blocks_per_sm;
};
LaunchShape plain_launch_shape();

// Smallest compiled component capacity >= n (0 if unsupported).
int capacity_for(int n);

// Plain FP64 flash, one thread per cell (flash_plain.cu).
cudaError_t launch_plain(int n, const Mixture* d_mix, int64_t ncell, const double* p, const double* t,
                         const double* z, const DeviceOutputs& out, cudaStream_t stream);

#define MPMC_DECLARE_PLAIN(NM)                                                                         \
    cudaError_t launch_plain_nm##NM(const Mixture* d_mix, int64_t ncell, const double* p, const double* t, \
                                    const double* z, const DeviceOutputs& out, cudaStream_t stream);
MPMC_DECLARE_PLAIN(4)
MPMC_DECLARE_PLAIN(8)
MPMC_DECLARE_PLAIN(12)
MPMC_DECLARE_PLAIN(16)
MPMC_DECLARE_PLAIN(20)
#undef MPMC_DECLARE_PLAIN

}  // namespace pr76
