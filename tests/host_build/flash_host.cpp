// Host build of the plain FP64 flash and the max-3-phase continuation with
// caller start hints (test infrastructure only).
//
// Compiles the device functions the plain and max3 kernels run per cell --
// fp64::solve_cell (pr76_fp64.cuh), fp64::max3_cell (pr76_max3.cuh) and the
// hint loader (pr76_hints.cuh) -- with the host C++ compiler and applies the
// kernels' per-cell sequence: the plain flash with the cell's hints as extra
// feed-test and final-review starts, then, for a phase_set_unstable answer,
// the continuation with the same hints and the three-phase start, and the
// publication of pt_phase_set.hpp:91-150.  The tests check it against the
// reference's recorded max3 statuses and hint-seeded continuation.
//
// Built with -DMPMC_WARP_EMULATION, the continuation runs as the max3 kernel
// runs it: on the 32 lanes of an emulated warp (warp_emu.h), each lane with
// its own copy of the cell, the line-search trials spread over the lanes.
// Every lane must end with the same answer, and a cell whose lanes diverge or
// disagree gets max3 status -99.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>

using std::isfinite;
#ifdef MPMC_WARP_EMULATION
#include "warp_emu.h"
#else
struct HostDim3 {
    unsigned x, y, z;
};
static HostDim3 threadIdx{0, 0, 0}, blockDim{1, 1, 1};
static inline void __syncthreads() {}
#endif

#include "launch.h"
#include "pr76_hints.cuh"

namespace {

// The continuation's root solver: false, the reference's bisection; true,
// bracketed Newton (MPMC_FLAG_MAX3_NEWTON_ROOTS).  Set by host_set_max3_newton.
bool g_max3_newton = false;

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

struct Outputs {
    int32_t* published;  // MPMC_FLASH_* (4 = three phases)
    int32_t* max3;       // MPMC_MAX3_*, -1 invalid
    double* x;           // [n * ncell] the published pair, or the feed for one phase
    double* y;           // [n * ncell]
    double* x3;          // [3 * n * ncell] the three-phase set
    double* f3;          // [3 * ncell]
};

#ifdef MPMC_WARP_EMULATION
// The max3 kernel's per-cell work on an emulated warp: every lane runs
// max3_cell in warp mode on its own copy of the cell.  True when the lanes
// stayed together and agree bit for bit on everything the kernel publishes;
// lane 0's scratch and result are then returned in s and r.
template <int NM>
bool max3_on_warp(const pr76::Mixture& m, const pr76::fp64::Cell<NM>& c0, const double* feed, const double* lnk,
                  const pr76::fp64::CellHints<NM>& hs, const double* const* fin, pr76::fp64::Max3Scratch<NM>& s,
                  pr76::fp64::Max3Result& r) {
    using namespace pr76::fp64;
    const int n = c0.n;
    std::unique_ptr<Max3Scratch<NM>[]> lane_s(new Max3Scratch<NM>[warp_emu::kLanes]());
    Max3Result lane_r[warp_emu::kLanes];
    const bool together = warp_emu::run(warp_emu::kLanes, [&](int lane) {
        Cell<NM> c = c0;
        Max3Result res{kM3Indeterminate, false, false};
        if (temp_setup(m, c))
            res = max3_cell(m, c, feed, lnk, lane_s[lane], fin, hs.fcount, hs.has_three ? hs.three : nullptr,
                            hs.options, true, g_max3_newton);
        else
            res.status = -1;
        lane_r[lane] = res;
    });
    if (!together) {
        std::fprintf(stderr, "warp emulation: the lanes diverged\n");
        return false;
    }
    auto same = [](double a, double b) { return std::memcmp(&a, &b, sizeof(double)) == 0; };
    for (int lane = 1; lane < warp_emu::kLanes; ++lane) {
        const Max3Result& a = lane_r[0];
        const Max3Result& b = lane_r[lane];
        bool agree = a.status == b.status && a.has_pair == b.has_pair && a.has_three == b.has_three;
        const ThreeState<NM>& p0 = lane_s[0].t.point;
        const ThreeState<NM>& p1 = lane_s[lane].t.point;
        const SplitState<NM>& w0 = lane_s[0].w.best;
        const SplitState<NM>& w1 = lane_s[lane].w.best;
        for (int q = 0; q < 3 && agree; ++q) {
            agree = same(p0.fraction[q], p1.fraction[q]) && same(p0.zf[q], p1.zf[q]);
            for (int i = 0; i < n && agree; ++i)
                agree = same(p0.x[q][i], p1.x[q][i]) && same(p0.lnphi[q][i], p1.lnphi[q][i]);
        }
        if (agree && a.has_pair)
            for (int i = 0; i < n && agree; ++i) agree = same(w0.x[i], w1.x[i]) && same(w0.y[i], w1.y[i]);
        if (!agree) {
            std::fprintf(stderr, "warp emulation: lane %d disagrees with lane 0\n", lane);
            return false;
        }
    }
    s = lane_s[0];
    r = lane_r[0];
    return true;
}
#endif

template <int NM>
void run(const pr76::Mixture& m, int64_t ncell, const double* p, const double* t, const double* z,
         const pr76::Hints& hints, const Outputs& o) {
    using namespace pr76;
    using namespace pr76::fp64;
    const int n = m.n;
    auto w = std::make_unique<Scratch<NM>>();
    auto s = std::make_unique<Max3Scratch<NM>>();
    for (int64_t cell = 0; cell < ncell; ++cell) {
        const double nan = std::nan("");
        for (int i = 0; i < n; ++i) o.x[i * ncell + cell] = o.y[i * ncell + cell] = nan;
        for (int q = 0; q < 3; ++q) {
            o.f3[q * ncell + cell] = nan;
            for (int i = 0; i < n; ++i) o.x3[(q * n + i) * ncell + cell] = nan;
        }
        Cell<NM> c;
        c.n = n;
        c.newton = false;
        c.p = p[cell];
        c.t = t[cell];
        for (int k = 0; k < cCount; ++k) c.counters[k] = 0;
        double feed[NM];
        for (int i = 0; i < n; ++i) feed[i] = z[i * ncell + cell];
        CellResult<NM> r;
        r.has_pair = false;
        CellHints<NM> hs;
        const bool ok = load_hints<NM>(hints, feed, n, ncell, cell, hs);
        const double* const* fin = hs.fcount > 0 ? hs.fptr : nullptr;
        const int status = ok ? solve_cell(m, c, feed, *w, r, hs.count > 0 ? hs.ptr : nullptr, hs.count, fin,
                                           hs.fcount, hs.options)
                              : kInvalid;
        int published = status;
        int m3 = status == kSinglePhase ? kM3Single : status == kTwoPhase ? kM3Two : status == kInvalid ? -1
                                                                                                  : kM3Indeterminate;
        if (status == kSinglePhase)
            for (int i = 0; i < n; ++i) o.x[i * ncell + cell] = c.z[i];
        if (status == kTwoPhase || status == kPhaseSetUnstable)
            for (int i = 0; i < n; ++i) {
                o.x[i * ncell + cell] = w->best.x[i];
                o.y[i * ncell + cell] = w->best.y[i];
            }
        if (status == kPhaseSetUnstable) {
            double lnk[NM];
            for (int i = 0; i < n; ++i) lnk[i] = w->best.lnk[i];
            Cell<NM> c2;
            c2.n = n;
            c2.newton = false;
            c2.p = p[cell];
            c2.t = t[cell];
            for (int k = 0; k < cCount; ++k) c2.counters[k] = 0;
            Max3Result mr{kM3Indeterminate, false, false};
#ifdef MPMC_WARP_EMULATION
            if (!max3_on_warp(m, c2, feed, lnk, hs, fin, *s, mr)) mr.status = -99;
#else
            if (temp_setup(m, c2))
                mr = max3_cell(m, c2, feed, lnk, *s, fin, hs.fcount, hs.has_three ? hs.three : nullptr,
                               hs.options, false, g_max3_newton);
            else
                mr.status = -1;
#endif
            m3 = mr.status;
            published = kIndeterminate;
            bool clear = true;
            if (m3 == kM3Three) {
                published = MPMC_THREE_PHASE_STATUS;
                for (int q = 0; q < 3; ++q) {
                    o.f3[q * ncell + cell] = s->t.point.fraction[q];
                    for (int i = 0; i < n; ++i) o.x3[(q * n + i) * ncell + cell] = s->t.point.x[q][i];
                }
            } else if (m3 == kM3Two && mr.has_pair) {
                published = kTwoPhase;
                clear = false;
                for (int i = 0; i < n; ++i) {
                    o.x[i * ncell + cell] = s->w.best.x[i];
                    o.y[i * ncell + cell] = s->w.best.y[i];
                }
            } else if (m3 == kM3Higher) {
                published = kPhaseSetUnstable;
                clear = false;
            } else if (m3 < 0) {
                published = kInvalid;
            }
            if (clear)
                for (int i = 0; i < n; ++i) o.x[i * ncell + cell] = o.y[i * ncell + cell] = nan;
        }
        o.published[cell] = published;
        o.max3[cell] = m3;
    }
}

}  // namespace

extern "C" void host_set_max3_newton(int on) { g_max3_newton = on != 0; }

extern "C" int host_hinted_batch(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                                 int64_t ncell, const double* p, const double* t, const double* z,
                                 const int32_t* hint_count, const double* hint_x, const int32_t* three,
                                 const double* fraction, int32_t* published, int32_t* max3, double* x, double* y,
                                 double* x3, double* f3) {
    if (n < 2 || n > pr76::kMaxC) return 1;
    pr76::Mixture m;
    prepare(n, tc, pc, omega, kij, m);
    const pr76::Hints hints{hint_count, hint_x, three, fraction};
    const Outputs o{published, max3, x, y, x3, f3};
    if (n <= 4) run<4>(m, ncell, p, t, z, hints, o);
    else if (n <= 12) run<12>(m, ncell, p, t, z, hints, o);
    else run<20>(m, ncell, p, t, z, hints, o);
    return 0;
}

// The same with the general caller inputs of mpmc_start_hints_ex: separate
// initial starts, final starts and three-phase start, and the two split options.
extern "C" int host_hinted_ex_batch(int n, const double* tc, const double* pc, const double* omega,
                                    const double* kij, int64_t ncell, const double* p, const double* t,
                                    const double* z, const int32_t* initial_count, const double* initial_x,
                                    const int32_t* final_count, const double* final_x, const int32_t* three,
                                    const double* three_x, const double* fraction, int32_t initial_automatic_starts,
                                    int32_t max_split_attempts, int32_t* published, int32_t* max3, double* x,
                                    double* y, double* x3, double* f3) {
    if (n < 2 || n > pr76::kMaxC) return 1;
    pr76::Mixture m;
    prepare(n, tc, pc, omega, kij, m);
    pr76::Hints hints;
    hints.count = initial_count;
    hints.x = initial_x;
    hints.final_count = final_count;
    hints.final_x = final_x;
    hints.three = three;
    hints.three_x = three_x;
    hints.fraction = fraction;
    hints.separate = 1;
    hints.initial_automatic_starts = initial_automatic_starts;
    hints.max_split_attempts = max_split_attempts;
    const Outputs o{published, max3, x, y, x3, f3};
    if (n <= 4) run<4>(m, ncell, p, t, z, hints, o);
    else if (n <= 12) run<12>(m, ncell, p, t, z, hints, o);
    else run<20>(m, ncell, p, t, z, hints, o);
    return 0;
}
