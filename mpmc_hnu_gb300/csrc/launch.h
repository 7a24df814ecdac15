// Internal host-side interface between the C ABI (capi.cu) and the kernel
// translation units.  Not part of the public boundary.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/mpmc_gb300_flash.h"
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

// Persistent-kernel residency of the batched form (0 = from the occupancy
// calculator).
struct BatchedShape {
    int trial_blocks_per_sm;
    int split_blocks_per_sm;
    int t64_blocks_per_sm;    // FP64 trial items (64 threads per block)
    int s64_blocks_per_sm;    // FP64 attempt items (64 threads per block)
    int cell_blocks_per_sm;   // per-cell FP64 kernels (polish, decide, ...; 64 threads per block)
    cudaEvent_t* events;  // optional: kBatchedStages + 1 events recorded around the stages
    int item_form;        // FP64 item kernels: bit 0 feed trials, bit 1 review trials, bit 2 attempts
                          // run one item per thread when set, one per lane group when clear; the
                          // polish runs one cell per thread with bit 3, per lane group with bit 4,
                          // and by component capacity (thread up to 12) with neither
    float ss_switch;      // FP32 |r| at which successive substitution hands over to the FP64
                          // Newton polish (0 = 2e-5)
    int fp64_items;       // batched FP64 form: every trial and attempt as an exact FP64 item
    // per call: ln K warm starts (device, [n * ncell], a non-finite entry makes
    // the cell cold); null = cold solve of every cell
    const double* warm_lnk;
    cudaEvent_t* redo_events;  // optional: the events of the cold pass after a warm pass
    cudaEvent_t* exact_events; // optional: the stage events of the exact sub-solve (mixed form)
    // optional: a second stream and two events on which the exact sub-solve
    // overlaps the main pass (null: it runs on the solve's stream after it)
    cudaStream_t side_stream;
    cudaEvent_t side_fork, side_join;
    float slow_projection;     // projected FP64 iterations above which an FP32 trial is re-run exactly
                               // in FP64 (0 = the default)
    int continue_limit;        // FP32 iterations from which an undecided trial or unsettled attempt
                               // runs from its start in FP64 (0 = the default)
    int64_t io_stride;         // stride of z, the warm starts and the outputs (0 = ncell): a solve of one
                               // cell range of a larger batch, with every pointer at the range's start
    int polish_stream;         // nonzero: the per-thread polish as one evaluation per loop iteration
                               // (polish_stream_kernel) instead of cell by cell (polish_kernel)
};
constexpr int kBatchedStages = 17;

// FP64 attempt-item capacity of the mixed form per cell: every attempt of
// every cell (kMaxAttempts), so that no cell of a hard batch -- near-critical
// cells whose 16 attempts all stay unsettled in FP32 -- overflows to the
// one-thread-per-cell fallback.  A smaller scratch (the no-allocation entry)
// takes the largest of 16, 8, 4, 2, 1 per cell that fits.
constexpr int kS64PerCell = 16;

// Batched mixed-precision flash (flash_batched.cu): scratch bytes needed for
// ncell cells, and the launch sequence using that scratch.
size_t batched_workspace_bytes(int n, int64_t ncell, bool fp64_items = false, int s64_per_cell = kS64PerCell);
cudaError_t launch_batched(int n, const Mixture* d_mix, int64_t ncell, const double* p, const double* t,
                           const double* z, const DeviceOutputs& out, void* scratch, size_t scratch_bytes,
                           const BatchedShape& shape, cudaStream_t stream);

// Caller start hints of a solve (the hints of the reference's ordered-path
// continuation, pr76_pt_continuation.hpp:106-146): per cell count[c] (0..3)
// compositions at x[(k * n + i) * ncell + c], used as extra starts of the
// feed stability test and of the final review; where three[c] is nonzero the
// three compositions are also a three-phase start whose phase-1 and phase-2
// fractions are fraction[k * ncell + c].  Device pointers; count == null
// means no hints.
// Caller starts of solve_pr76_pt_max3 / solve_pt_vle, cell-fastest:
// composition k of cell c, component i at (k * n + i) * ncell + c.  With
// `separate` 0 (the continuation's hints) the `count` compositions are the
// initial and the final starts and, when three of them, the three-phase start;
// with `separate` 1 the final starts and the three-phase start have arrays of
// their own.
struct Hints {
    const int32_t* count = nullptr;  // initial starts (0..3 per cell)
    const double* x = nullptr;
    const int32_t* three = nullptr;  // nonzero: a three-phase start
    const double* fraction = nullptr;  // its phase_fraction_seed [2 * ncell]
    const int32_t* final_count = nullptr;
    const double* final_x = nullptr;
    const double* three_x = nullptr;
    int separate = 0;
    int initial_automatic_starts = 1;  // options.two_phase.initial_stability.automatic_starts
    int max_split_attempts = 16;       // options.two_phase.max_split_attempts
};

// Three-phase outputs of the max-3-phase continuation (layout a[k * ncell + c];
// phase-major compositions: phase q, component i at row q * n + i).
struct Max3Outputs {
    int32_t* max3_status;  // Pr76PtMax3Status (0 single, 1 two, 2 three, 3 boundary unresolved,
                           // 4 higher phase count, 5 indeterminate), -1 invalid
    double* fraction;      // [3] phase fractions
    double* x;             // [3 * n] compositions
    double* lnphi;         // [3 * n]
    double* z;             // [3] compressibility factors
};

// Max-3-phase continuation (flash_max3.cu) of the cells whose flash status in
// `out` is phase_set_unstable; every cell gets its max3_status.  Reads and
// rewrites the two-phase fields of `out` (status, pair) as the reference's
// publication does.  newton_roots: bracketed-Newton roots and Rachford-Rice
// in the continuation instead of the reference's bisection.
cudaError_t launch_max3(int n, const Mixture* d_mix, int64_t ncell, const double* p, const double* t,
                        const double* z, const DeviceOutputs& out, const Max3Outputs& out3, cudaStream_t stream,
                        const Hints& hints = Hints{}, bool newton_roots = false);

// Closure constants of a selected-phase property chart call (pr76_chart.cuh),
// passed to the kernel by value.
struct ChartParams {
    int phases;
    int root_index[3];
    double molar_mass[kMaxC];
    double visc[7 + kMaxC];  // affine model: constant, p, T, rho, M, rho_mass, root index, x_i
    double enth[7 + kMaxC];
};

// Device outputs of the chart (mpmc_property_chart_outputs), any may be null.
struct ChartOutputs {
    int32_t* status;
    double* values;    // [rows * ncell]
    double* jacobian;  // [rows * q * ncell]
};

// Selected-phase property chart of ncell cells (chart.cu): q [(P n + 1) *
// ncell] chart values, dep [P * ncell] dependent components or null (the last
// component).
cudaError_t launch_chart(int n, const Mixture* d_mix, const ChartParams& params, int64_t ncell, const double* q,
                         const int32_t* dep, const ChartOutputs& out, cudaStream_t stream);

// Smallest compiled component capacity >= n (0 if unsupported).
int capacity_for(int n);

// Plain FP64 flash, one thread per cell (flash_plain.cu).
cudaError_t launch_plain(int n, const Mixture* d_mix, int64_t ncell, const double* p, const double* t,
                         const double* z, const DeviceOutputs& out, cudaStream_t stream,
                         const Hints& hints = Hints{});

// Implicit sensitivity of accepted two-phase cells (sensitivity.cu) among the
// cells [c0, c1) of the batch (c1 < 0: to the end); reads the flash fields of
// `out` (status, beta, x, y, lnk, z_l, z_v), which must be set.
// lanes: the lane-group form (pr76_sensw.cuh) instead of one thread per cell.
cudaError_t launch_sensitivity(int n, const Mixture* d_mix, int64_t ncell, const double* p, const double* t,
                               const double* z, const DeviceOutputs& out, cudaStream_t stream, int64_t c0 = 0,
                               int64_t c1 = -1, bool lanes = false);

#define MPMC_DECLARE_PLAIN(NM)                                                                         \
    cudaError_t launch_plain_nm##NM(const Mixture* d_mix, int64_t ncell, const double* p, const double* t, \
                                    const double* z, const DeviceOutputs& out, cudaStream_t stream,       \
                                    const Hints& hints);                                                  \
    cudaError_t launch_sensitivity_nm##NM(const Mixture* d_mix, int64_t ncell, const double* p, const double* t, \
                                          const double* z, const DeviceOutputs& out, cudaStream_t stream,      \
                                          int64_t c0, int64_t c1);                                             \
    cudaError_t launch_sensitivity_lanes_nm##NM(const Mixture* d_mix, int64_t ncell, const double* p,          \
                                                const double* t, const double* z, const DeviceOutputs& out,      \
                                                cudaStream_t stream, int64_t c0, int64_t c1);                    \
    cudaError_t launch_max3_nm##NM(const Mixture* d_mix, int64_t ncell, const double* p, const double* t,      \
                                   const double* z, const DeviceOutputs& out, const Max3Outputs& out3,           \
                                   cudaStream_t stream, const Hints& hints, bool newton_roots);                   \
    cudaError_t launch_chart_nm##NM(const Mixture* d_mix, const ChartParams& params, int64_t ncell,           \
                                    const double* q, const int32_t* dep, const ChartOutputs& out,               \
                                    cudaStream_t stream);                                                        \
    size_t batched_workspace_bytes_nm##NM(int n, int64_t ncell, bool fp64_items, int s64_per_cell);           \
    cudaError_t launch_batched_nm##NM(const Mixture* d_mix, int n, int64_t ncell, const double* p,            \
                                      const double* t, const double* z, const DeviceOutputs& out, void* scratch, \
                                      size_t scratch_bytes, const BatchedShape& shape, cudaStream_t stream);
MPMC_DECLARE_PLAIN(4)
MPMC_DECLARE_PLAIN(8)
MPMC_DECLARE_PLAIN(12)
MPMC_DECLARE_PLAIN(16)
MPMC_DECLARE_PLAIN(20)
#undef MPMC_DECLARE_PLAIN

// Helpers of the C ABI shared with the flash server (capi.cu): the error
// message setters and the mixture preparation of mpmc_gpu_flash_create.
namespace host {
int fail(int code, const std::string& what);
int cuda_fail(cudaError_t e, const char* where);
int prepare_mixture(const mpmc_pr76_mixture* mix, Mixture& m);
}  // namespace host

}  // namespace pr76
