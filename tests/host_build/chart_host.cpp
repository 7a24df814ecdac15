// Host build of the device property-chart code (test infrastructure only).
//
// Compiles mpmc_hnu_gb300/csrc/pr76_chart.cuh -- the per-cell function the
// chart kernel runs, chart::run_cell, and everything it calls (the FP64 EOS,
// roots and closed-form phase Jacobian) -- with the host C++ compiler, so the
// device arithmetic and its output indexing can be checked against the
// oracle on a machine without a GPU.  The kernel itself only adds the
// grid-stride loop and the shared-memory staging of the constants.
// CUDA's headers mark __device__ functions with attributes that a host
// compiler ignores; the block-level names are stubbed for the one
// non-template helper that mentions them.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

using std::isfinite;
struct HostDim3 {
    unsigned x, y, z;
};
static HostDim3 threadIdx{0, 0, 0}, blockDim{1, 1, 1};
static inline void __syncthreads() {}

#include "launch.h"
#include "pr76_chart.cuh"

namespace {

// The prepared constants of mpmc_gpu_flash_create (pr76_pure.hpp:181-199).
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

template <int NM>
void run(const pr76::Mixture& m, const pr76::ChartParams& cp, int64_t ncell, const double* q, const int32_t* dep,
         const pr76::ChartOutputs& out) {
    for (int64_t c = 0; c < ncell; ++c) pr76::chart::run_cell<NM>(m, cp, ncell, c, q, dep, out);
}

}  // namespace

extern "C" int host_chart_batch(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                                int phases, const int* root_index, const double* molar_mass, const double* visc,
                                const double* enth, int64_t ncell, const double* q, const int32_t* dep,
                                int32_t* status, double* values, double* jac) {
    if (n < 2 || n > pr76::kMaxC || phases < 1 || phases > 3) return 1;
    pr76::Mixture m;
    prepare(n, tc, pc, omega, kij, m);
    pr76::ChartParams cp;
    std::memset(&cp, 0, sizeof(cp));
    cp.phases = phases;
    for (int k = 0; k < phases; ++k) cp.root_index[k] = root_index[k];
    for (int i = 0; i < n; ++i) cp.molar_mass[i] = molar_mass[i];
    for (int k = 0; k < 7 + n; ++k) {
        cp.visc[k] = visc[k];
        cp.enth[k] = enth[k];
    }
    const pr76::ChartOutputs out{status, values, jac};
    if (n <= 4) run<4>(m, cp, ncell, q, dep, out);
    else if (n <= 8) run<8>(m, cp, ncell, q, dep, out);
    else if (n <= 12) run<12>(m, cp, ncell, q, dep, out);
    else if (n <= 16) run<16>(m, cp, ncell, q, dep, out);
    else run<20>(m, cp, ncell, q, dep, out);
    return 0;
}
