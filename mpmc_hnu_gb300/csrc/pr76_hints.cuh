// Per-cell caller start hints (launch.h Hints): the previous accepted
// phases of an ordered-path continuation, pr76_pt_continuation.hpp:106-146.
#pragma once

#include "pr76_max3.cuh"

namespace pr76 {
namespace fp64 {

template <int NM>
struct CellHints {
    double x[3][NM];
    const double* ptr[3];
    int count;
    double fx[3][NM];
    const double* fptr[3];
    int fcount;
    bool has_three;
    double three[3 * NM + 2];  // the three compositions, then the fractions of phases 1 and 2
    SolveOptions options;
};

template <int NM>
__device__ int load_set(const int32_t* count, const double* x, int n, int64_t ncell, int64_t cell,
                        double (&dst)[3][NM], const double* (&ptr)[3]) {
    if (count == nullptr || x == nullptr) return 0;
    int k = count[cell];
    k = k < 0 ? 0 : (k > 3 ? 3 : k);
    for (int q = 0; q < k; ++q) {
        for (int i = 0; i < n; ++i) dst[q][i] = x[(static_cast<int64_t>(q) * n + i) * ncell + cell];
        ptr[q] = dst[q];
    }
    return k;
}

// Loads cell `cell`'s hints.  False when its three-phase start fails the
// reference's start check (pr76_three_phase.hpp:211-244: fractions inside
// the simplex, compositions on the feed's support), a domain_error there.
template <int NM>
__device__ bool load_hints(const Hints& h, const double* feed, int n, int64_t ncell, int64_t cell,
                           CellHints<NM>& out) {
    out.has_three = false;
    out.options.initial_automatic_starts = h.initial_automatic_starts != 0;
    out.options.max_split_attempts = h.max_split_attempts;
    out.count = load_set<NM>(h.count, h.x, n, ncell, cell, out.x, out.ptr);
    if (h.separate) {
        out.fcount = load_set<NM>(h.final_count, h.final_x, n, ncell, cell, out.fx, out.fptr);
    } else {
        out.fcount = out.count;
        for (int q = 0; q < out.count; ++q) out.fptr[q] = out.ptr[q];
    }
    const double* tx = h.separate ? h.three_x : h.x;
    if (h.three == nullptr || h.fraction == nullptr || tx == nullptr || h.three[cell] == 0 ||
        (!h.separate && out.count != 3))
        return true;
    const double f1 = h.fraction[cell], f2 = h.fraction[ncell + cell];
    if (!rr3_feasible(f1, f2)) return false;
    for (int q = 0; q < 3; ++q) {
        for (int i = 0; i < n; ++i) out.three[q * n + i] = tx[(static_cast<int64_t>(q) * n + i) * ncell + cell];
        double sum;
        if (!check_composition(out.three + q * n, n, sum)) return false;
        for (int i = 0; i < n; ++i)
            if ((feed[i] > 0.0) != (out.three[q * n + i] > 0.0)) return false;
    }
    out.three[3 * n] = f1;
    out.three[3 * n + 1] = f2;
    out.has_three = true;
    return true;
}

}  // namespace fp64
}  // namespace pr76
