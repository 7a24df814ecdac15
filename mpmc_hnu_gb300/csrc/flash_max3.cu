// Max-3-phase continuation kernel (pr76_max3.cuh).  A rare path (only cells
// whose two-phase answer is phase_set_unstable do work); its large FP64
// routines stay out of line (MPMC_FP64_CALL), which keeps the unit's build
// short.
#define MPMC_FP64_CALL __noinline__
#include "launch.h"
#include "pr76_hints.cuh"

namespace pr76 {

constexpr int kMax3Block = 64;  // two cells (warps) per block

// Max-3-phase continuation: one warp per cell over the whole batch; a cell
// whose two-phase status is phase_set_unstable runs fp64::max3_cell on all 32
// lanes (each lane with its own copy of the same state, so the lanes agree at
// every step; the attempts' line searches spread their trials over the
// lanes), every other cell only gets its max3 status
// (pr76_three_phase.hpp:336-358).  Lane 0 writes the outputs.
template <int NM>
__global__ void __launch_bounds__(kMax3Block) max3_kernel(const Mixture* __restrict__ mix_g, int64_t ncell,
                                                          const double* __restrict__ p, const double* __restrict__ t,
                                                          const double* __restrict__ z, DeviceOutputs out,
                                                          Max3Outputs out3, Hints hints, bool newton_roots) {
    __shared__ Mixture m;
    stage_mixture(mix_g, m);
    using namespace fp64;
    const int n = m.n;
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    const bool writer = (threadIdx.x & 31u) == 0;
    const int64_t warps = static_cast<int64_t>(gridDim.x) * (blockDim.x / 32);
    for (int64_t cell = static_cast<int64_t>(blockIdx.x) * (blockDim.x / 32) + threadIdx.x / 32; cell < ncell;
         cell += warps) {
        auto put = [&](double* a, int k, double v) {
            if (a && writer) a[static_cast<int64_t>(k) * ncell + cell] = v;
        };
        for (int q = 0; q < 3; ++q) {
            put(out3.fraction, q, nan);
            put(out3.z, q, nan);
            for (int i = 0; i < n; ++i) {
                put(out3.x, q * n + i, nan);
                put(out3.lnphi, q * n + i, nan);
            }
        }
        const int status = out.status[cell];
        __syncwarp();  // every lane has read the cell's status before lane 0 may rewrite it
                       // (the status is the same on all lanes: the branch below is uniform)
        int m3 = status == kSinglePhase ? kM3Single
                 : status == kTwoPhase  ? kM3Two
                 : status == kInvalid   ? -1
                                        : kM3Indeterminate;
        if (status == kPhaseSetUnstable) {
            Cell<NM> c;
            c.n = n;
            c.newton = false;
            c.p = p[cell];
            c.t = t[cell];
            for (int k = 0; k < cCount; ++k) c.counters[k] = 0;
            double feed[NM], lnk[NM];
            for (int i = 0; i < n; ++i) {
                feed[i] = z[static_cast<int64_t>(i) * ncell + cell];
                lnk[i] = out.lnk[static_cast<int64_t>(i) * ncell + cell];
            }
            Max3Scratch<NM> s;
            Max3Result r{kM3Indeterminate, false, false};
            // the caller's hints, as the base solve ran with them (the plain
            // kernel has already rejected a cell whose three-phase start fails)
            CellHints<NM> hs;
            load_hints<NM>(hints, feed, n, ncell, cell, hs);
            if (temp_setup(m, c))
                r = max3_cell(m, c, feed, lnk, s, hs.fcount > 0 ? hs.fptr : nullptr, hs.fcount,
                              hs.has_three ? hs.three : nullptr, hs.options, true, newton_roots);
            else
                r.status = -1;
            m3 = r.status;
            __syncwarp();  // every lane has read the cell's ln K before lane 0 may rewrite it
            // publication, pt_phase_set.hpp:91-150
            int published = kIndeterminate;
            bool clear_pair = true;
            if (m3 == kM3Three) {
                published = MPMC_THREE_PHASE_STATUS;
                const ThreeState<NM>& st = s.t.point;
                for (int q = 0; q < 3; ++q) {
                    put(out3.fraction, q, st.fraction[q]);
                    put(out3.z, q, st.zf[q]);
                    for (int i = 0; i < n; ++i) {
                        put(out3.x, q * n + i, st.x[q][i]);
                        put(out3.lnphi, q * n + i, st.lnphi[q][i]);
                    }
                }
            } else if (m3 == kM3Two && r.has_pair) {  // the fresh two-phase neighbor
                published = kTwoPhase;
                clear_pair = false;
                const SplitState<NM>& b = s.w.best;
                put(out.beta, 0, b.beta);
                for (int i = 0; i < n; ++i) {
                    put(out.x, i, b.x[i]);
                    put(out.y, i, b.y[i]);
                    put(out.lnk, i, b.lnk[i]);
                    put(out.lnphi_l, i, b.lnphi_l[i]);
                    put(out.lnphi_v, i, b.lnphi_v[i]);
                }
                put(out.z_l, 0, b.z_l);
                put(out.z_v, 0, b.z_v);
            } else if (m3 == kM3Higher) {  // the base pair stays published
                published = kPhaseSetUnstable;
                clear_pair = false;
            } else if (m3 < 0) {
                published = kInvalid;
            }
            if (writer) out.status[cell] = published;
            if (clear_pair) {
                put(out.beta, 0, nan);
                for (int i = 0; i < n; ++i) {
                    put(out.x, i, nan);
                    put(out.y, i, nan);
                    put(out.lnk, i, nan);
                    put(out.lnphi_l, i, nan);
                    put(out.lnphi_v, i, nan);
                }
                put(out.z_l, 0, nan);
                put(out.z_v, 0, nan);
            }
        }
        if (out3.max3_status && writer) out3.max3_status[cell] = m3;
    }
}

#ifndef MPMC_NM
#error "compile with -DMPMC_NM=<capacity>"
#endif
#define MPMC_CAT2(a, b) a##b
#define MPMC_CAT(a, b) MPMC_CAT2(a, b)

cudaError_t MPMC_CAT(launch_max3_nm, MPMC_NM)(const Mixture* d_mix, int64_t ncell, const double* p,
                                                const double* t, const double* z, const DeviceOutputs& out,
                                                const Max3Outputs& out3, cudaStream_t stream, const Hints& hints,
                                                bool newton_roots) {
    if (ncell <= 0) return cudaSuccess;
    if (!out.status || !out.lnk) return cudaErrorInvalidValue;
    int device = 0, sms = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    // one warp per cell, up to four blocks per SM at once
    int64_t grid = static_cast<int64_t>(sms) * 4;
    const int64_t needed = (ncell + kMax3Block / 32 - 1) / (kMax3Block / 32);
    if (grid > needed) grid = needed;
    max3_kernel<MPMC_NM><<<static_cast<unsigned>(grid), kMax3Block, 0, stream>>>(d_mix, ncell, p, t, z, out,
                                                                                  out3, hints, newton_roots);
    return cudaGetLastError();
}

}  // namespace pr76
