// Lane-group primitives shared by the FP64 lane-group kernels: a group of S
// lanes (S a power of two, 4-32) works on one item with component i on lane
// i; sums and maxima are group reductions and broadcasts are shuffles within
// the group; the LU with partial pivoting keeps row i on lane i.
#pragma once

#include "pr76_common.cuh"

namespace pr76 {
namespace w64 {

// Lanes per item of the throughput-bound polish: the component capacity rounded
// up to a power of two, so a warp runs 32 / S cells side by side (8 at four
// components, 2 at ten, 1 at twenty).  The tail-latency-bound trial and attempt
// items run one per warp (S = 32): items sharing a warp would share its issue.
template <int NM>
constexpr int kSeg = NM <= 4 ? 4 : (NM <= 8 ? 8 : (NM <= 16 ? 16 : 32));

// first lane of this thread's item within the warp
template <int S>
__device__ __forceinline__ int seg_base() { return (threadIdx.x & 31) & ~(S - 1); }
template <int S>
__device__ __forceinline__ unsigned seg_mask() {
    if constexpr (S == 32) return 0xffffffffu;
    else return ((1u << S) - 1u) << seg_base<S>();
}
template <int S>
__device__ __forceinline__ int seg_lane() { return threadIdx.x & (S - 1); }
template <int S>
__device__ __forceinline__ double wsum(double v) {
    const unsigned m = seg_mask<S>();
#pragma unroll
    for (int o = S / 2; o > 0; o >>= 1) v += __shfl_xor_sync(m, v, o, S);
    return v;
}
template <int S>
__device__ __forceinline__ double wmax(double v) {
    const unsigned m = seg_mask<S>();
#pragma unroll
    for (int o = S / 2; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(m, v, o, S));
    return v;
}
template <int S>
__device__ __forceinline__ float fsum_group(float v) {
    const unsigned m = seg_mask<S>();
#pragma unroll
    for (int o = S / 2; o > 0; o >>= 1) v += __shfl_xor_sync(m, v, o, S);
    return v;
}
template <int S>
__device__ __forceinline__ float fmax_group(float v) {
    const unsigned m = seg_mask<S>();
#pragma unroll
    for (int o = S / 2; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(m, v, o, S));
    return v;
}
template <int S>
__device__ __forceinline__ bool wany(bool p) { return __any_sync(seg_mask<S>(), p); }
template <int S, typename T>
__device__ __forceinline__ T bcast(T v, int src) { return __shfl_sync(seg_mask<S>(), v, src, S); }
// ballot of the item's lanes, bit i = lane i of the item
template <int S>
__device__ __forceinline__ unsigned seg_ballot(bool p) {
    const unsigned b = __ballot_sync(seg_mask<S>(), p);
    if constexpr (S == 32) return b;
    else return (b >> seg_base<S>()) & ((1u << S) - 1u);
}

// Row-distributed LU with partial pivoting: lane i holds row i; pivot rows
// stay in their lanes (piv lists them in elimination order) and multipliers
// overwrite the eliminated entries.
template <int NM, int S>
__device__ bool lu_rows(double (&J)[NM], int n, int (&piv)[NM]) {
    const int lane = seg_lane<S>();
    bool used = lane >= n;
#pragma unroll
    for (int k = 0; k < NM; ++k) {
        if (k >= n) break;
        // pivot: largest |J_ik| among the rows not used yet (lowest lane on ties)
        double best = used ? -1.0 : fabs(J[k]);
        int who = lane;
#pragma unroll
        for (int o = S / 2; o > 0; o >>= 1) {
            const double ob = __shfl_xor_sync(seg_mask<S>(), best, o, S);
            const int ow = __shfl_xor_sync(seg_mask<S>(), who, o, S);
            if (ob > best || (ob == best && ow < who)) {
                best = ob;
                who = ow;
            }
        }
        if (!(best > 0.0) || !isfinite(best)) return false;
        piv[k] = who;
        const double pk = bcast<S>(J[k], who);
        const double f = (!used && lane != who) ? J[k] / pk : 0.0;
#pragma unroll
        for (int j = 0; j < NM; ++j) {
            const double rj = bcast<S>(J[j], who);
            if (j > k && !used && lane != who) J[j] -= f * rj;
        }
        if (!used && lane != who) J[k] = f;
        if (lane == who) used = true;
    }
    return true;
}

// Solve J d = rhs with the factors of lu_rows; rhs and d are per lane (row i /
// component i).
template <int NM, int S>
__device__ double lu_solve_rows(const double (&J)[NM], int n, const int (&piv)[NM], double rhs) {
    const int lane = seg_lane<S>();
    double y = rhs;
    // forward: lane piv[k] is final at step k; later rows subtract their multiplier
    int order = NM;  // this lane's elimination position
#pragma unroll
    for (int k = 0; k < NM; ++k)
        if (k < n && piv[k] == lane) order = k;
#pragma unroll
    for (int k = 0; k < NM; ++k) {
        if (k >= n) break;
        const double yk = bcast<S>(y, piv[k]);
        if (order > k && order < NM) y -= J[k] * yk;
    }
    double d = 0.0;
#pragma unroll
    for (int k = NM - 1; k >= 0; --k) {
        if (k >= n) continue;
        const double xk = bcast<S>(order == k ? y / J[k] : 0.0, piv[k]);
        if (order < k) y -= J[k] * xk;
        if (lane == k) d = xk;
    }
    return d;
}

}  // namespace w64
}  // namespace pr76
