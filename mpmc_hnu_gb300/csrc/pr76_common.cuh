// Shared device definitions for the GB300 PR76 PT flash kernels.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#ifndef MPMC_MAX_COMPONENTS
#define MPMC_MAX_COMPONENTS 20
#endif

namespace pr76 {

constexpr int kMaxC = MPMC_MAX_COMPONENTS;
constexpr double kEps = 2.220446049250313080847e-16;   // DBL_EPSILON
constexpr double kDblMin = 2.2250738585072013831e-308; // DBL_MIN
// R = N_A k_B in J/(mol K) (pr76_pure.hpp:115-117)
constexpr double kR = 8.31446261815324;

// Prepared mixture constants (pr76_pure.hpp:181-199, pr76_mixture.hpp:229-251).
// One copy lives in device global memory per handle; kernels stage it into
// shared memory once per block.
struct Mixture {
    int n;
    int pad;
    double sqrt_tc[kMaxC];
    double kappa[kMaxC];
    double ac[kMaxC];      // 0.45724 (R Tc)^2 / Pc
    double b[kMaxC];       // 0.07780 R Tc / Pc
    double factor[kMaxC * kMaxC];  // 1 - kij, row-major
    float factor32[kMaxC * kMaxC]; // the same, rounded to FP32 for the FP32 stages
    float b32[kMaxC];
};

// Failure classes standing in for the reference's exception/issue types
// (modules/flash/include/mpmc/flash/pt_stability.hpp:23-26).
enum Issue : int {
    kOk = 0, kRootTopology = 1, kRootIterationLimit = 2, kRootRange = 3,
    kIllConditionedRoot = 4, kNoAdmissibleBranch = 5, kNonfinite = 6, kDomain = 7
};

// Per-cell phase-set status (include/mpmc_gb300_flash.h).
enum FlashStatus : int { kSinglePhase = 0, kTwoPhase = 1, kPhaseSetUnstable = 2,
                         kIndeterminate = 3, kInvalid = -1 };
// accepted three-phase set (max-3-phase continuation only)
constexpr int MPMC_THREE_PHASE_STATUS = 4;

// Counter rows (include/mpmc_gb300_flash.h MPMC_COUNTER_*).
enum Counter : int { cInitEvals = 0, cSplitEvals, cFinalEvals, cSplitIters, cRrIters,
                     cRootIters, cAttempts, cTrialIters, cCount };

// Compensated summation step, pt_stability.hpp:99-104.
__device__ __forceinline__ void kahan_add(double term, double& sum, double& c) {
    const double inc = term - c;
    const double next = sum + inc;
    c = (next - sum) - inc;
    sum = next;
}

__device__ __forceinline__ void stage_mixture(const Mixture* g, Mixture& s) {
    const int words = static_cast<int>(sizeof(Mixture) / sizeof(double));
    const double* src = reinterpret_cast<const double*>(g);
    double* dst = reinterpret_cast<double*>(&s);
    for (int k = threadIdx.x; k < words; k += blockDim.x) dst[k] = src[k];
    __syncthreads();
}

}  // namespace pr76
