// Selected-phase property chart kernel: one thread per cell, FP64
// (pr76_chart.cuh).  Compiled once per component capacity (-DMPMC_NM).
//
// Every chart value and derivative of a cell is written exactly once, at
// a[(row * q + column) * ncell + cell]: for each (row, column) a warp writes
// 32 consecutive doubles.  A cell that fails is NaN-filled (chart::run_cell).
#include "launch.h"
#include "pr76_chart.cuh"

#ifndef MPMC_NM
#error "compile with -DMPMC_NM=<capacity>"
#endif

namespace pr76 {

template <int NM>
__global__ void __launch_bounds__(64) chart_kernel(const Mixture* __restrict__ mix_g, const ChartParams params,
                                                   int64_t ncell, const double* __restrict__ qv,
                                                   const int32_t* __restrict__ dep, ChartOutputs out) {
    __shared__ Mixture m;
    __shared__ ChartParams cp;
    if (threadIdx.x == 0) cp = params;
    stage_mixture(mix_g, m);  // ends with __syncthreads()
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t cell = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; cell < ncell; cell += stride)
        chart::run_cell<NM>(m, cp, ncell, cell, qv, dep, out);
}

#define MPMC_CAT2(a, b) a##b
#define MPMC_CAT(a, b) MPMC_CAT2(a, b)

cudaError_t MPMC_CAT(launch_chart_nm, MPMC_NM)(const Mixture* d_mix, const ChartParams& params, int64_t ncell,
                                                 const double* q, const int32_t* dep, const ChartOutputs& out,
                                                 cudaStream_t stream) {
    if (ncell <= 0) return cudaSuccess;
    int device = 0, sms = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int block = 64;
    // one wave: every SM holds as many blocks as its registers admit
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chart_kernel<MPMC_NM>, block, 0) != cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    int64_t grid = static_cast<int64_t>(sms) * per_sm;
    const int64_t needed = (ncell + block - 1) / block;
    if (grid > needed) grid = needed;
    chart_kernel<MPMC_NM><<<static_cast<unsigned>(grid), block, 0, stream>>>(d_mix, params, ncell, q, dep, out);
    return cudaGetLastError();
}

}  // namespace pr76
