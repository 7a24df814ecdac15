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
    bool has_three;
    double three[3 * NM + 2];  // the three compositions, then the fractions of phases 1 and 2
};

// Loads cell `cell`'s hints.  False when its three-phase start fails the
// reference's start check (pr76_three_phase.hpp:211-244: fractions inside
// the simplex, compositions on the feed's support), a domain_error there.
template <int NM>
__device__ bool load_hints(const Hints& h, const double* feed, int n, int64_t ncell, int64_t cell,
                           CellHints<NM>& out) {
    out.count = 0;
    out.has_three = false;
    if (h.count == nullptr || h.x == nullptr) return true;
    int k = h.count[cell];
    k = k < 0 ? 0 : (k > 3 ? 3 : k);
    for (int q = 0; q < k; ++q) {
        for (int i = 0; i < n; ++i) out.x[q][i] = h.x[(static_cast<int64_t>(q) * n + i) * ncell + cell];
        out.ptr[q] = out.x[q];
    }
    out.count = k;
    if (h.three == nullptr || h.fraction == nullptr || h.three[cell] == 0 || k != 3) return true;
    const double f1 = h.fraction[cell], f2 = h.fraction[ncell + cell];
    if (!rr3_feasible(f1, f2)) return false;
    for (int q = 0; q < 3; ++q) {
        double sum;
        if (!check_composition(out.x[q], n, sum)) return false;
        for (int i = 0; i < n; ++i)
            if ((feed[i] > 0.0) != (out.x[q][i] > 0.0)) return false;
        for (int i = 0; i < n; ++i) out.three[q * n + i] = out.x[q][i];
    }
    out.three[3 * n] = f1;
    out.three[3 * n + 1] = f2;
    out.has_three = true;
    return true;
}

}  // namespace fp64
}  // namespace pr76
