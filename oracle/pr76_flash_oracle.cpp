// PR76 two-phase PT flash -- CPU oracle (test infrastructure, not product code).
//
// This file restates, in plain sequential C++20, the reference algorithm of
// MPMC_HNU's PR76 PT flash and its implicit sensitivity so that the GPU kernels
// can be checked against it on the GPU host, where the reference sources are
// not available.  It is only ever called by the tests, by the smoke check and
// by the CPU-baseline leg of the benchmark; the shipped library never links it.
//
// Parity is pinned: tests/golden holds fixtures produced by compiling the
// reference headers themselves (oracle/ref_harness.cpp, built into oracle/_ref
// by oracle/Makefile) together with the reference's own published golden
// vectors, and tests/test_oracle_golden.py checks this restatement against both.
//
// Every numbered step cites the reference file and line it restates
// (paths relative to the MPMC_HNU project root).  Exceptions of the reference
// are replaced by status codes with the same meaning.  Floating-point
// operations keep the reference's evaluation order; build with
// -ffp-contract=off so x86-64 and aarch64 hosts round identically.

#include <algorithm>
#include <atomic>
#include <array>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace oracle {

constexpr double kEps = std::numeric_limits<double>::epsilon();
constexpr double kR = 8.31446261815324;  // modules/thermodynamics/.../pr76_pure.hpp:115-117
constexpr double kNaN = std::numeric_limits<double>::quiet_NaN();

// ---------------------------------------------------------------------------
// Error codes standing in for the reference exception/issue classes.
// modules/flash/include/mpmc/flash/pt_stability.hpp:23-26
enum Issue {
    kOk = 0,
    kRootTopology = 1,        // near_multiple
    kRootIterationLimit = 2,  // iteration_limit
    kRootRange = 3,           // unrepresentable root / range_error
    kIllConditionedRoot = 4,
    kNoAdmissibleBranch = 5,
    kNonfinite = 6,
    kDomain = 7,              // std::domain_error (not caught by the flash)
};

// Kahan step, pt_stability.hpp:99-104
inline void kahan_add(double term, double& sum, double& c) {
    const double inc = term - c;
    const double next = sum + inc;
    c = (next - sum) - inc;
    sum = next;
}
inline double kahan_sum(const double* x, int n) {
    double s = 0, c = 0;
    for (int i = 0; i < n; ++i) kahan_add(x[i], s, c);
    return s;
}
inline double midpoint(double a, double b) { return (a + b) / 2; }

// ---------------------------------------------------------------------------
// Forward-mode number with one tangent direction; used only on the
// sensitivity path (the reference uses Dual<double,4> blocks,
// modules/ad/include/mpmc/ad/dual.hpp:80; one direction per pass gives the
// same first-order derivatives).
struct D1 {
    double v = 0, d = 0;
    D1() = default;
    explicit D1(double value, double tangent = 0) : v(value), d(tangent) {}
};
inline D1 operator+(D1 a, D1 b) { return D1(a.v + b.v, a.d + b.d); }
inline D1 operator-(D1 a, D1 b) { return D1(a.v - b.v, a.d - b.d); }
inline D1 operator*(D1 a, D1 b) { return D1(a.v * b.v, a.d * b.v + a.v * b.d); }
inline D1 operator/(D1 a, D1 b) {
    const double q = a.v / b.v;
    return D1(q, (a.d - q * b.d) / b.v);
}
inline D1 operator+(D1 a, double b) { return D1(a.v + b, a.d); }
inline D1 operator+(double a, D1 b) { return D1(a + b.v, b.d); }
inline D1 operator-(D1 a, double b) { return D1(a.v - b, a.d); }
inline D1 operator-(double a, D1 b) { return D1(a - b.v, -b.d); }
inline D1 operator*(D1 a, double b) { return D1(a.v * b, a.d * b); }
inline D1 operator*(double a, D1 b) { return D1(a * b.v, a * b.d); }
inline D1 operator/(D1 a, double b) { return D1(a.v / b, a.d / b); }
inline D1 operator/(double a, D1 b) {
    const double q = a / b.v;
    return D1(q, -q * b.d / b.v);
}
inline D1 sqrt(D1 a) {
    const double s = std::sqrt(a.v);
    return D1(s, a.d / (2 * s));
}
inline D1 log(D1 a) { return D1(std::log(a.v), a.d / a.v); }
inline D1 log1p(D1 a) { return D1(std::log1p(a.v), a.d / (1 + a.v)); }
inline double val(double a) { return a; }
inline double val(const D1& a) { return a.v; }
inline bool finite(double a) { return std::isfinite(a); }
inline bool finite(const D1& a) { return std::isfinite(a.v) && std::isfinite(a.d); }
using std::log;
using std::log1p;
using std::sqrt;

// ---------------------------------------------------------------------------
// Prepared mixture: pr76_pure.hpp:181-199 and pr76_mixture.hpp:229-251.
struct Model {
    int n = 0;
    std::vector<double> tc, sqrt_tc, kappa, ac, b, factor;  // factor = 1 - kij (row-major)
};

inline Model make_model(int n, const double* tc, const double* pc, const double* omega,
                        const double* kij) {
    Model m;
    m.n = n;
    m.tc.assign(tc, tc + n);
    m.sqrt_tc.resize(n);
    m.kappa.resize(n);
    m.ac.resize(n);
    m.b.resize(n);
    for (int i = 0; i < n; ++i) {
        m.sqrt_tc[i] = std::sqrt(tc[i]);
        // pr76_pure.hpp:189-190, Horner order
        m.kappa[i] = 0.37464 + omega[i] * (1.54226 - 0.26992 * omega[i]);
        const double rtc = kR * tc[i];
        m.ac[i] = (0.45724 * rtc) * (rtc / pc[i]);  // :193
        m.b[i] = (0.07780 * rtc) / pc[i];           // :194
    }
    m.factor.resize(static_cast<size_t>(n) * n);
    for (int k = 0; k < n * n; ++k) m.factor[k] = 1.0 - kij[k];
    return m;
}

// Per-temperature constants.  pr76_mixture.hpp:172-204 recomputes these on
// every call; they depend on T only, so computing them once per cell gives
// bit-identical values.
struct TempCache {
    std::vector<double> a, root, aij;  // a_i(T), sqrt(a_i), (root_i*f_ij)*root_j
};
inline bool make_temp_cache(const Model& m, double t, TempCache& c) {
    const int n = m.n;
    c.a.resize(n);
    c.root.resize(n);
    c.aij.assign(static_cast<size_t>(n) * n, 0.0);
    for (int i = 0; i < n; ++i) {
        // pr76_pure.hpp:153-163
        const double reduced_root = std::sqrt(t) / m.sqrt_tc[i];
        const double bracket = 1.0 + m.kappa[i] * (1.0 - reduced_root);
        const double attraction = (bracket * m.ac[i]) * bracket;
        if (!std::isfinite(attraction) || (attraction == 0 && bracket != 0)) return false;
        c.a[i] = attraction;
        if (n > 1) {
            if (!(attraction > 0)) return false;  // pr76_mixture.hpp:180-182
            c.root[i] = std::sqrt(attraction);
        }
    }
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j)
            c.aij[i * n + j] = (c.root[i] * m.factor[i * n + j]) * c.root[j];  // :198-199
    return true;
}

// Mixing with row sums, pr76_mixture.hpp:170-218 (WithSums=true order).
inline bool mix(const Model& m, const TempCache& c, const double* x, double& amix, double& bmix,
                double* sums) {
    const int n = m.n;
    double attraction = 0, covolume = 0;
    for (int i = 0; i < n; ++i) {
        attraction += (x[i] * c.a[i]) * x[i];
        covolume += x[i] * m.b[i];
        sums[i] = x[i] * c.a[i];
    }
    for (int i = 0; i < n; ++i) {
        for (int j = i + 1; j < n; ++j) {
            const double cross = ((x[i] * c.root[i]) * (x[j] * c.root[j])) * m.factor[i * n + j];
            attraction += cross;
            attraction += cross;
            const double aij = c.aij[i * n + j];
            sums[i] += x[j] * aij;
            sums[j] += x[i] * aij;
        }
    }
    amix = attraction;
    bmix = covolume;
    if (!std::isfinite(attraction) || !std::isfinite(covolume) || !(covolume > 0)) return false;
    for (int i = 0; i < n; ++i)
        if (!std::isfinite(sums[i])) return false;
    return true;
}

// ---------------------------------------------------------------------------
// Cubic roots, modules/thermodynamics/include/mpmc/thermodynamics/pr76_roots.hpp
enum RootStatus { kRootSuccess, kRootNearMultiple, kRootIterLimit, kRootUnrepresentable };
struct Root {
    double z, free_volume, slope_ratio;
    bool derivative_valid;
    int slope_sign;
};
struct RootSet {
    Root roots[3];
    int count = 0;
    double scale = 1;
    RootStatus status = kRootUnrepresentable;
    int iterations = 0;  // total bisection steps (work counter)
};
struct Cubic {
    double c2, c1, c0;
};
inline Cubic cubic_coefficients(double a, double b, double scale) {  // :50-58
    const double bs = b / scale;
    const double inv = 1.0 / scale;
    return {4.0 * bs - inv, (a / scale) / scale + 2.0 * bs * bs - 4.0 * bs * inv,
            ((-2.0 * bs) * bs) * inv};
}
inline double poly(double y, const Cubic& c) {  // :60-63
    return std::fma(std::fma(y + c.c2, y, c.c1), y, c.c0);
}
inline double poly_scale(double y, const Cubic& c) {  // :64-68
    return ((std::abs(y) + std::abs(c.c2)) * std::abs(y) + std::abs(c.c1)) * std::abs(y) +
           std::abs(c.c0);
}

inline RootSet solve_roots(double a, double b) {  // :77-173
    RootSet r;
    if (!std::isfinite(a) || !std::isfinite(b) || !(b > 0)) return r;
    r.scale = std::max({1.0, b, std::sqrt(std::abs(a))});
    const Cubic c = cubic_coefficients(a, b, r.scale);
    if (!std::isfinite(c.c2) || !std::isfinite(c.c1) || !std::isfinite(c.c0) || !(c.c0 < 0))
        return r;
    const double upper = 1.0 + std::max({std::abs(c.c2), std::abs(c.c1), std::abs(c.c0)});
    double endpoints[4] = {0, 0, 0, 0};
    int endpoint_count = 1;
    const double disc = std::fma(c.c2, c.c2, -3.0 * c.c1);
    if (disc > 0) {  // :95-112
        const double q = -c.c2 - std::copysign(std::sqrt(disc), c.c2);
        double st[2] = {q / 3.0, c.c1 / q};
        if (st[1] < st[0]) std::swap(st[0], st[1]);
        for (double point : st) {
            if (point > 0 && point < upper) {
                const double value = poly(point, c);
                const double magnitude = poly_scale(point, c);
                if (!std::isfinite(value) || !(magnitude > 0)) return r;
                if (std::abs(value) <= 64.0 * kEps * magnitude) {
                    r.status = kRootNearMultiple;
                    return r;
                }
                endpoints[endpoint_count++] = point;
            }
        }
    }
    endpoints[endpoint_count++] = upper;
    for (int interval = 1; interval < endpoint_count; ++interval) {  // :114-170
        double left = endpoints[interval - 1], right = endpoints[interval];
        double fl = poly(left, c);
        const double fr = poly(right, c);
        if (!std::isfinite(fl) || !std::isfinite(fr)) return r;
        if (std::signbit(fl) == std::signbit(fr)) continue;
        double y = 0;
        bool converged = false;
        int it = 0;
        for (; it < 2048; ++it) {
            y = midpoint(left, right);
            const double fy = poly(y, c);
            if (fy == 0 || y == left || y == right ||
                right - left <= 4.0 * kEps * std::max(y, std::numeric_limits<double>::min())) {
                converged = true;
                break;
            }
            if (std::signbit(fy) == std::signbit(fl)) {
                left = y;
                fl = fy;
            } else {
                right = y;
            }
        }
        r.iterations += it + 1;
        if (!converged) {
            r.count = 0;
            r.status = kRootIterLimit;
            return r;
        }
        const double xv = y * r.scale;
        const double z = xv + b;
        const double magnitude = poly_scale(y, c);
        const double residual = std::abs(poly(y, c)) / magnitude;
        const double dh = std::fma(3.0 * y + 2.0 * c.c2, y, c.c1);
        const double dh_scale = 3.0 * y * y + 2.0 * std::abs(c.c2) * y + std::abs(c.c1);
        const double slope_ratio = dh_scale > 0 ? std::abs(dh) / dh_scale : 0.0;
        const double bz = b / z;
        const double repulsion = 1.0 / xv;
        const double attraction = ((a / z) / z) / (1.0 + 2.0 * bz - bz * bz);
        const double pressure_residual = std::abs(repulsion - attraction - 1.0) /
                                         (1.0 + std::abs(repulsion) + std::abs(attraction));
        if (!std::isfinite(z) || !(z > b) || !std::isfinite(residual) ||
            !std::isfinite(pressure_residual) || residual > 128.0 * kEps ||
            pressure_residual > 512.0 * kEps || r.count == 3) {
            r.count = 0;
            r.status = kRootUnrepresentable;
            return r;
        }
        if (r.count != 0 && !(z > r.roots[r.count - 1].z)) {
            r.count = 0;
            r.status = kRootNearMultiple;
            return r;
        }
        r.roots[r.count++] = {z, xv, slope_ratio, slope_ratio > 8.0 * std::sqrt(kEps),
                              dh > 0 ? 1 : (dh < 0 ? -1 : 0)};
    }
    r.status = r.count > 0 ? kRootSuccess : kRootUnrepresentable;
    return r;
}

inline Issue root_issue(RootStatus s) {  // pr76_stability.hpp:42-53
    switch (s) {
    case kRootSuccess: return kOk;
    case kRootNearMultiple: return kRootTopology;
    case kRootIterLimit: return kRootIterationLimit;
    default: return kRootRange;
    }
}

// log1p(u)/u with the series branch, pr76_phase.hpp:67-79
template <class Num>
inline Num log1p_over_x(const Num& u) {
    if (std::abs(val(u)) <= 1.0 / 8.0) {
        constexpr int degree = std::numeric_limits<double>::digits / 3 + 2;
        Num value{(degree % 2 == 0 ? 1.0 : -1.0) / static_cast<double>(degree + 1)};
        for (int k = degree - 1; k >= 0; --k)
            value = (k % 2 == 0 ? 1.0 : -1.0) / static_cast<double>(k + 1) + u * value;
        return value;
    }
    return log1p(u) / u;
}

// Reduced coefficients A, B, pr76_phase.hpp:175-191
inline bool coefficients(double p, double t, double amix, double bmix, double& A, double& B) {
    const double rt = kR * t;
    if (!std::isfinite(rt) || !(rt > 0)) return false;
    const double prt = p / rt;
    A = (amix / rt) * prt;
    B = bmix * prt;
    if (!std::isfinite(A) || !std::isfinite(B) || !(B > 0) || (A == 0 && amix != 0)) return false;
    return true;
}

// ln(phi) of a resolved root, pr76_phase.hpp:223-253 (plain double path).
inline bool ln_phi_of_root(const Model& m, double p, double t, double amix, double bmix,
                           const double* sums, double A, double B, const Root& root,
                           double* ln_phi) {
    const double free_volume = root.free_volume;
    const double z = free_volume + B;
    const double sqrt2 = std::sqrt(2.0);
    const double denominator = free_volume + (2.0 - sqrt2) * B;
    const double u = (2.0 * sqrt2) * (B / denominator);
    const double log_factor = log1p_over_x(u) / denominator;
    double z_minus_one = z - 1.0;
    double log_free = std::log(free_volume);
    if (std::abs(z_minus_one) < 0.25 && B < 0.125) {
        const double bz = B / z;
        z_minus_one = B / free_volume - (A / z) / (1.0 + 2.0 * bz - bz * bz);
        log_free = std::log1p(z_minus_one - B);
    }
    const double rt = kR * t;
    const double prt = p / rt;
    for (int i = 0; i < m.n; ++i) {
        const double ratio = m.b[i] / bmix;
        const double coefficient = ((2.0 * sums[i] - amix * ratio) / rt) * prt;
        ln_phi[i] = ratio * z_minus_one - log_free - coefficient * log_factor;
        if (!std::isfinite(ln_phi[i])) return false;
    }
    return std::isfinite(z);
}

// ---------------------------------------------------------------------------
// Scratch for one cell.
struct Work {
    int n = 0;
    TempCache tc;
    std::vector<double> sums;
    std::vector<double> lnphi_tmp[3];
    long long evaluations = 0;     // provider calls
    long long root_bisections = 0; // cubic bisection steps
    long long rr_iterations = 0;
    void init(int nn) {
        n = nn;
        sums.resize(n);
        for (auto& v : lnphi_tmp) v.resize(n);
    }
};

struct StabilityPhase {
    std::vector<double> ln_phi;
    int branch = 0;
    bool smooth = true;
    double z = kNaN;  // Z of the selected branch (diagnostic output)
};

// Stability provider, modules/flash/include/mpmc/flash/pr76_stability.hpp:36-119
inline Issue stability_provider(const Model& m, Work& w, double p, double t, const double* x,
                                StabilityPhase& out) {
    const int n = m.n;
    ++w.evaluations;
    double amix, bmix, A, B;
    if (!mix(m, w.tc, x, amix, bmix, w.sums.data())) return kRootRange;
    if (!coefficients(p, t, amix, bmix, A, B)) return kRootRange;
    const RootSet roots = solve_roots(A, B);
    w.root_bisections += roots.iterations;
    if (roots.status != kRootSuccess) return root_issue(roots.status);
    int cand[3], ncand = 0;
    for (int k = 0; k < roots.count; ++k) {
        if (roots.roots[k].slope_sign <= 0) continue;  // :58
        if (!ln_phi_of_root(m, p, t, amix, bmix, w.sums.data(), A, B, roots.roots[k],
                            w.lnphi_tmp[ncand].data()))
            return kRootRange;
        cand[ncand++] = k;
    }
    if (ncand == 0) return kNoAdmissibleBranch;
    auto difference = [&](int a, int b, double& value) {  // :67-78
        double v = 0, c = 0;
        for (int i = 0; i < n; ++i)
            kahan_add(x[i] * (w.lnphi_tmp[a][i] - w.lnphi_tmp[b][i]), v, c);
        value = v;
        return std::isfinite(v);
    };
    int best = 0;
    for (int k = 1; k < ncand; ++k) {
        double d;
        if (!difference(k, best, d)) return kNonfinite;
        if (d < 0) best = k;
    }
    if (!roots.roots[cand[best]].derivative_valid) return kIllConditionedRoot;
    bool smooth = true;
    for (int k = 0; k < ncand; ++k) {  // :89-104
        if (k == best) continue;
        double magnitude = 1;
        for (int i = 0; i < n; ++i)
            magnitude += x[i] * (std::abs(w.lnphi_tmp[k][i]) + std::abs(w.lnphi_tmp[best][i]));
        if (!std::isfinite(magnitude)) return kNonfinite;
        double d;
        if (!difference(k, best, d)) return kNonfinite;
        if (std::abs(d) <= 256.0 * kEps * magnitude) smooth = false;
    }
    out.ln_phi.assign(w.lnphi_tmp[best].begin(), w.lnphi_tmp[best].end());
    out.branch = cand[best];
    out.smooth = smooth;
    out.z = roots.roots[cand[best]].z;
    return kOk;
}

struct SplitPhase {
    std::vector<double> ln_phi;
    int branch = 0;
    double z = 0;
};

// Role provider, modules/flash/include/mpmc/flash/pr76_split.hpp:38-84 plus
// split_check_phase, pt_split.hpp:197-203.
inline Issue role_provider(const Model& m, Work& w, double p, double t, const double* x,
                           bool vapor, SplitPhase& out) {
    ++w.evaluations;
    double amix, bmix, A, B;
    if (!mix(m, w.tc, x, amix, bmix, w.sums.data())) return kRootRange;
    if (!coefficients(p, t, amix, bmix, A, B)) return kRootRange;
    const RootSet roots = solve_roots(A, B);
    w.root_bisections += roots.iterations;
    if (roots.status != kRootSuccess) return root_issue(roots.status);
    int selected = -1;
    for (int k = 0; k < roots.count; ++k) {
        if (roots.roots[k].slope_sign <= 0) continue;
        selected = k;
        if (!vapor) break;
    }
    if (selected < 0) return kNoAdmissibleBranch;
    if (!roots.roots[selected].derivative_valid) return kIllConditionedRoot;
    out.ln_phi.resize(m.n);
    if (!ln_phi_of_root(m, p, t, amix, bmix, w.sums.data(), A, B, roots.roots[selected],
                        out.ln_phi.data()))
        return kRootRange;
    out.branch = selected;
    out.z = roots.roots[selected].z;
    if (!std::isfinite(out.z) || out.z <= 0) return kIllConditionedRoot;
    return kOk;
}

// ---------------------------------------------------------------------------
// TPD stability, modules/flash/include/mpmc/flash/pt_stability.hpp
struct StabilityOptions {  // :44-56
    double tpd_tolerance = 1e-10;
    double stationarity_tolerance = 1e-8;
    double armijo = 1e-4;
    double log_step_limit = 4.0;
    int max_iterations = 512;
    int max_backtracks = 32;
    long long max_evaluations = 100000;
    bool automatic_starts = true;  // :55, feed, uniform and 0.1 z + 0.9 e_i starts
};
enum TrialStatus {
    kNegativeTpd, kStationary, kIterationLimit, kEvaluationLimit, kLineSearchFailed,
    kPropertyFailure, kNonsmooth, kUnrepresentableComposition
};
struct TpdPoint {
    std::vector<double> w, residual;
    double value = 0, guard = 0, stationarity = 0;
    bool smooth = true;
    int branch = 0;  // root branch of the stability phase at w
};
struct Trial {
    std::vector<double> initial;
    TpdPoint point;
    bool has_point = false;
    TrialStatus status = kEvaluationLimit;
    int iterations = 0;
};
enum StabilityStatus { kUnstable, kNoInstabilityFound, kStabilityIndeterminate };
struct StabilityResult {
    StabilityStatus status = kStabilityIndeterminate;
    std::vector<double> feed;
    StabilityPhase reference;
    bool has_reference = false;
    std::vector<Trial> trials;
    long long evaluations = 0;
    int trial_iterations = 0;
};

// Composition check, pt_stability.hpp:110-122
inline bool check_composition(const double* x, int n, double& sum) {
    for (int i = 0; i < n; ++i)
        if (!std::isfinite(x[i]) || x[i] < 0 || x[i] > 1) return false;
    sum = kahan_sum(x, n);
    return std::abs(sum - 1.0) <= 64.0 * kEps;
}

inline bool stability_negative(const TpdPoint& p, const StabilityOptions& o) {  // :150-152
    return p.value < -o.tpd_tolerance - p.guard;
}
inline bool stability_accept(const TpdPoint& point, const TpdPoint& next, double predicted,
                             double armijo, double relative_step) {  // :157-171
    const double guard = point.guard + next.guard;
    if (predicted <= guard)
        return next.value <= point.value + guard && relative_step > 0 &&
               next.stationarity < point.stationarity;
    return next.value <= point.value - armijo * predicted;
}

// tangent_plane_distance, pt_stability.hpp:178-220
inline Issue tpd(const double* w, const std::vector<double>& z, const std::vector<double>& lnphi_w,
                 const std::vector<double>& lnphi_ref, int n, TpdPoint& out) {
    double sum;
    if (!check_composition(w, n, sum)) return kDomain;
    out.w.assign(w, w + n);
    out.residual.assign(n, 0.0);
    out.value = 0;
    out.stationarity = 0;
    double correction = 0, magnitude = 1, mc = 0;
    bool boundary = false;
    for (int i = 0; i < n; ++i) {
        if (z[i] == 0) {
            if (w[i] != 0) return kDomain;
            continue;
        }
        if (w[i] == 0) {
            boundary = true;
            continue;
        }
        const double lw = std::log(w[i]), lz = std::log(z[i]);
        const double log_ratio =
            std::abs(w[i] - z[i]) < 0.5 * z[i] ? std::log1p((w[i] - z[i]) / z[i]) : lw - lz;
        const double q = log_ratio + (lnphi_w[i] - lnphi_ref[i]);
        out.residual[i] = q;
        kahan_add(w[i] * q, out.value, correction);
        kahan_add(w[i] * (std::abs(lw) + std::abs(lz) + std::abs(lnphi_w[i]) +
                          std::abs(lnphi_ref[i])),
                  magnitude, mc);
    }
    const double mean = out.value / sum;
    for (int i = 0; i < n; ++i) {
        if (z[i] == 0) continue;
        out.residual[i] = w[i] == 0 ? -std::numeric_limits<double>::infinity() : out.residual[i] - mean;
        out.stationarity = std::max(out.stationarity, std::abs(out.residual[i]));
    }
    out.guard = 256.0 * kEps * magnitude;
    if (!std::isfinite(out.value) || !std::isfinite(out.guard) ||
        (!boundary && !std::isfinite(out.stationarity)))
        return kNonfinite;
    return kOk;
}

// test_pt_stability_impl, pt_stability.hpp:228-461.  `imposed` empty selects
// the feed-phase reference; otherwise it is the common log activity.
inline bool stability_test(const Model& m, Work& wk, double p, double t, const std::vector<double>& feed_in,
                           const StabilityOptions& o, const std::vector<std::vector<double>>& extra,
                           const std::vector<double>& imposed, StabilityResult& res) {
    const int n = m.n;
    double input_sum;
    if (!check_composition(feed_in.data(), n, input_sum)) return false;
    int active = 0;
    for (double v : feed_in) active += v > 0;
    // :254-262: no start at all is a length_error in the reference
    if ((o.automatic_starts ? (active == 1 ? 1 : active + 2) : 0) + extra.size() == 0) return false;
    for (const auto& s : extra) {  // :263-272, a domain_error in the reference
        double ssum;
        if (static_cast<int>(s.size()) != n || !check_composition(s.data(), n, ssum)) return false;
        for (int i = 0; i < n; ++i)
            if ((feed_in[i] == 0 && s[i] != 0) || (feed_in[i] > 0 && s[i] == 0)) return false;
    }
    res = StabilityResult();
    res.feed.resize(n);
    for (int i = 0; i < n; ++i) res.feed[i] = feed_in[i] / input_sum;
    for (int i = 0; i < n; ++i)
        if (feed_in[i] > 0 && res.feed[i] == 0) return true;  // indeterminate, :280-285
    auto add_start = [&](std::vector<double> s) {
        const double sum = kahan_sum(s.data(), n);
        for (double& v : s) v /= sum;
        Trial tr;
        tr.initial = std::move(s);
        res.trials.push_back(std::move(tr));
    };
    if (o.automatic_starts) add_start(res.feed);  // :294-310
    if (o.automatic_starts && active > 1) {
        std::vector<double> uniform(n, 0.0);
        for (int i = 0; i < n; ++i)
            if (res.feed[i] > 0) uniform[i] = 1.0 / static_cast<double>(active);
        add_start(uniform);
        for (int i = 0; i < n; ++i) {
            if (res.feed[i] == 0) continue;
            std::vector<double> s = res.feed;
            for (double& v : s) v *= 0.1;
            s[i] += 0.9;
            add_start(s);
        }
    }
    for (const auto& s : extra) add_start(s);
    StabilityPhase imposed_phase;
    const long long eval0 = wk.evaluations;
    if (imposed.empty()) {  // :313-335
        Issue is = stability_provider(m, wk, p, t, res.feed.data(), res.reference);
        if (is == kDomain) return false;
        if (is != kOk) {
            for (auto& tr : res.trials) tr.status = kPropertyFailure;
            res.evaluations = wk.evaluations - eval0;
            return true;
        }
        res.has_reference = true;
    } else {
        imposed_phase.ln_phi.resize(n);
        for (int i = 0; i < n; ++i)
            imposed_phase.ln_phi[i] = res.feed[i] > 0 ? imposed[i] - std::log(res.feed[i]) : 0.0;
        for (double v : imposed_phase.ln_phi)
            if (!std::isfinite(v)) {
                for (auto& tr : res.trials) tr.status = kPropertyFailure;
                return true;
            }
    }
    const std::vector<double>& ref = imposed.empty() ? res.reference.ln_phi : imposed_phase.ln_phi;
    bool negative_found = false, all_stationary = true;
    StabilityPhase phase;
    std::vector<double> direction(n), candidate(n);
    for (auto& tr : res.trials) {  // :343-457
        auto evaluate = [&](const double* w, TpdPoint& out) -> Issue {
            Issue is = stability_provider(m, wk, p, t, w, phase);
            if (is != kOk) return is;
            for (double v : phase.ln_phi)
                if (!std::isfinite(v)) return kNonfinite;
            is = tpd(w, res.feed, phase.ln_phi, ref, n, out);
            out.smooth = phase.smooth;
            out.branch = phase.branch;
            return is;
        };
        bool support_lost = false;
        for (int i = 0; i < n; ++i) support_lost = support_lost || (res.feed[i] > 0 && tr.initial[i] == 0);
        if (support_lost) {
            tr.status = kUnrepresentableComposition;
            all_stationary = false;
            continue;
        }
        if (wk.evaluations - eval0 >= o.max_evaluations) {
            tr.status = kEvaluationLimit;
            all_stationary = false;
            continue;
        }
        {
            Issue is = evaluate(tr.initial.data(), tr.point);
            if (is == kDomain) return false;
            if (is != kOk) {
                tr.status = kPropertyFailure;
                all_stationary = false;
                continue;
            }
            tr.has_point = true;
        }
        TpdPoint next;
        for (;;) {
            const TpdPoint& point = tr.point;
            if (stability_negative(point, o)) {
                tr.status = kNegativeTpd;
                negative_found = true;
                break;
            }
            if (!point.smooth) {
                tr.status = kNonsmooth;
                break;
            }
            if (point.stationarity <= o.stationarity_tolerance) {
                tr.status = kStationary;
                break;
            }
            if (tr.iterations >= o.max_iterations) {
                tr.status = kIterationLimit;
                break;
            }
            const double scale = std::max(1.0, point.stationarity / o.log_step_limit);
            double slope = 0, correction = 0;
            for (int i = 0; i < n; ++i) {
                direction[i] = 0;
                if (res.feed[i] == 0) continue;
                direction[i] = -point.residual[i] / scale;
                kahan_add((point.w[i] * point.residual[i]) * direction[i], slope, correction);
            }
            if (!std::isfinite(slope) || !(slope < 0)) {
                tr.status = kLineSearchFailed;
                break;
            }
            bool accepted = false;
            double alpha = 1;
            tr.status = kLineSearchFailed;
            for (int bt = 0; bt < o.max_backtracks; ++bt, alpha *= 0.5) {
                double largest = -std::numeric_limits<double>::infinity();
                for (int i = 0; i < n; ++i) {
                    if (res.feed[i] > 0) {
                        candidate[i] = std::log(point.w[i]) + alpha * direction[i];
                        largest = std::max(largest, candidate[i]);
                    }
                }
                for (int i = 0; i < n; ++i)
                    candidate[i] = res.feed[i] > 0 ? std::exp(candidate[i] - largest) : 0.0;
                const double sum = kahan_sum(candidate.data(), n);
                bool positive = std::isfinite(sum) && sum > 0;
                for (int i = 0; i < n; ++i) {
                    candidate[i] /= sum;
                    positive = positive && (res.feed[i] == 0 || candidate[i] > 0);
                }
                if (!positive) continue;
                if (wk.evaluations - eval0 >= o.max_evaluations) {
                    tr.status = kEvaluationLimit;
                    break;
                }
                Issue is = evaluate(candidate.data(), next);
                if (is == kDomain) return false;
                if (is != kOk) continue;  // rejected property evaluation
                if (stability_negative(next, o) ||
                    stability_accept(point, next, -alpha * slope, o.armijo, alpha / scale)) {
                    std::swap(tr.point, next);
                    accepted = true;
                    break;
                }
            }
            if (!accepted) break;
            ++tr.iterations;
        }
        res.trial_iterations += tr.iterations;
        all_stationary = all_stationary && tr.status == kStationary;
    }
    res.status = negative_found ? kUnstable : (all_stationary ? kNoInstabilityFound : kStabilityIndeterminate);
    res.evaluations = wk.evaluations - eval0;
    return true;
}

// ---------------------------------------------------------------------------
// Rachford-Rice, modules/flash/include/mpmc/flash/rachford_rice.hpp
enum RrStatus { kRrInterior, kRrNoInterior, kRrDegenerate, kRrIterLimit, kRrUnrepresentable };
struct RrResult {
    RrStatus status = kRrUnrepresentable;
    double beta = kNaN;
    std::vector<double> x, y;
    double mass_absolute = 0, mass_relative = 0;
};
inline double rr_log_sum(const std::vector<double>& z, const std::vector<double>& lk, double sign) {
    const int n = static_cast<int>(z.size());  // :42-52
    double largest = -std::numeric_limits<double>::infinity();
    for (int i = 0; i < n; ++i)
        if (z[i] > 0) largest = std::max(largest, std::log(z[i]) + sign * lk[i]);
    double sum = 0, c = 0;
    for (int i = 0; i < n; ++i)
        if (z[i] > 0) kahan_add(std::exp(std::log(z[i]) + sign * lk[i] - largest), sum, c);
    return largest + std::log(sum);
}
inline RrResult solve_rr(const std::vector<double>& z, const std::vector<double>& lk, Work& wk) {
    const int n = static_cast<int>(z.size());  // :70-147
    RrResult r;
    double contrast = 0;
    for (int i = 0; i < n; ++i)
        if (z[i] > 0) contrast = std::max(contrast, std::abs(lk[i]));
    if (contrast == 0) {
        r.status = kRrDegenerate;
        return r;
    }
    const double ls = rr_log_sum(z, lk, 1), rs = rr_log_sum(z, lk, -1);
    if (!std::isfinite(ls) || !std::isfinite(rs)) return r;
    if (ls <= 64 * kEps || rs <= 64 * kEps) {
        r.status = kRrNoInterior;
        return r;
    }
    // exp(-|lnK|) and the expm1 numerators do not depend on beta; they are
    // formed once here instead of once per bisection step (same values).
    std::vector<double> e(n), num(n);
    for (int i = 0; i < n; ++i) {
        if (z[i] == 0) continue;
        e[i] = std::exp(-std::abs(lk[i]));
        num[i] = lk[i] >= 0 ? -std::expm1(-lk[i]) : std::expm1(lk[i]);
    }
    double left = 0, right = 1, beta = 0.5, value = 0;
    bool resolved = false;
    for (int it = 0; it < 192; ++it) {
        ++wk.rr_iterations;
        beta = midpoint(left, right);
        if (!(beta > 0 && beta < 1)) break;
        double v = 0, c = 0;  // rr_value, :53-63
        for (int i = 0; i < n; ++i) {
            if (z[i] == 0) continue;
            const double den = lk[i] >= 0 ? beta + (1 - beta) * e[i] : (1 - beta) + beta * e[i];
            kahan_add((z[i] / den) * num[i], v, c);
        }
        value = v;
        if (!std::isfinite(value)) return r;
        if (value == 0 || beta == left || beta == right ||
            right - left <= 8 * kEps * std::min(beta, 1 - beta)) {
            resolved = true;
            break;
        }
        if (value > 0) left = beta; else right = beta;
    }
    if (!resolved) {
        r.status = kRrIterLimit;
        return r;
    }
    r.beta = beta;
    if (std::abs(value) > 64 * kEps) return r;
    r.x.assign(n, 0.0);
    r.y.assign(n, 0.0);
    for (int i = 0; i < n; ++i) {
        if (z[i] == 0) continue;
        const double den = lk[i] >= 0 ? beta + (1 - beta) * e[i] : (1 - beta) + beta * e[i];
        const double larger = z[i] / den;
        r.x[i] = lk[i] >= 0 ? larger * e[i] : larger;
        r.y[i] = lk[i] >= 0 ? larger : larger * e[i];
        if (!std::isfinite(larger) || !(r.x[i] > 0 && r.y[i] > 0)) return r;
    }
    const double sx = kahan_sum(r.x.data(), n), sy = kahan_sum(r.y.data(), n);
    if (std::abs(sx - 1) > 64 * kEps || std::abs(sy - 1) > 64 * kEps) return r;
    for (int i = 0; i < n; ++i) {
        r.x[i] /= sx;
        r.y[i] /= sy;
        const double recovered = std::fma(beta, r.y[i], (1 - beta) * r.x[i]);
        const double err = std::abs(recovered - z[i]);
        r.mass_absolute = std::max(r.mass_absolute, err);
        if (z[i] > 0) {
            if (!(r.x[i] > 0 && r.y[i] > 0)) return r;
            r.mass_relative = std::max(r.mass_relative, err / z[i]);
        } else if (recovered != 0) {
            return r;
        }
    }
    r.status = kRrInterior;
    return r;
}

// ---------------------------------------------------------------------------
// Split iteration, modules/flash/include/mpmc/flash/pt_split.hpp:275-408
enum AttemptStatus {
    kConverged, kNoInteriorRr, kRrFailure, kIndistinguishable, kPhaseDisappearance,
    kAttemptPropertyFailure, kAttemptIterationLimit, kAttemptEvaluationLimit,
    kAttemptLineSearchFailed, kUnrepresentableSeed, kBalanceFailure
};
struct SplitOptions {  // :30-44
    double fugacity_tolerance = 1e-11;
    double mass_absolute_tolerance = 1e-12;
    double mass_relative_tolerance = 1e-10;
    double minimum_phase_fraction = 1e-10;
    double log_k_separation = 1e-7;
    double relative_z_separation = 1e-8;
    double max_log_step = 2;
    double residual_decrease = 1e-4;
    int max_iterations = 512;
    int max_backtracks = 24;
    long long max_evaluations = 20000;
    double gibbs_armijo = 1e-4;
};
struct SplitState {
    RrResult rr;
    SplitPhase liquid, vapor;
    std::vector<double> log_k, residual, common;
    double fug_norm = 0, gibbs = 0, guard = 0;
};
struct Attempt {
    AttemptStatus status = kUnrepresentableSeed;
    SplitState point;
    bool has_point = false;
    int iterations = 0;
    long long evaluations = 0;
};

// Split evaluation, pt_split.hpp:300-341.  Returns false with `st` set to the
// failure class (SplitStepError or property failure).
inline bool split_evaluate(const Model& m, Work& wk, double p, double t, const std::vector<double>& z,
                           const std::vector<double>& lk, const SplitOptions& /*options*/, long long& evals,
                           long long budget, SplitState& s, AttemptStatus& st) {
    const int n = m.n;
    s.rr = solve_rr(z, lk, wk);
    if (s.rr.status != kRrInterior) {
        st = s.rr.status == kRrDegenerate ? kIndistinguishable
             : (s.rr.status == kRrNoInterior ? kNoInteriorRr : kRrFailure);
        return false;
    }
    for (int role = 0; role < 2; ++role) {
        if (evals >= budget) {
            st = kAttemptEvaluationLimit;
            return false;
        }
        ++evals;
        SplitPhase& ph = role == 0 ? s.liquid : s.vapor;
        Issue is = role_provider(m, wk, p, t, role == 0 ? s.rr.x.data() : s.rr.y.data(), role == 1, ph);
        if (is != kOk) {
            st = kAttemptPropertyFailure;
            return false;
        }
    }
    s.log_k.assign(n, 0.0);
    s.residual.assign(n, 0.0);
    s.common.assign(n, 0.0);
    s.fug_norm = 0;
    s.gibbs = 0;
    double correction = 0, magnitude = 1, mc = 0;
    const double beta = s.rr.beta;
    for (int i = 0; i < n; ++i) {
        if (z[i] == 0) continue;
        const double lx = std::log(s.rr.x[i]);
        const double ly = std::log(s.rr.y[i]);
        const double mu_l = lx + s.liquid.ln_phi[i];
        const double mu_v = ly + s.vapor.ln_phi[i];
        s.log_k[i] = ly - lx;
        s.residual[i] = (lx - ly) + (s.liquid.ln_phi[i] - s.vapor.ln_phi[i]);
        s.common[i] = midpoint(mu_l, mu_v);
        s.fug_norm = std::max(s.fug_norm, std::abs(s.residual[i]));
        kahan_add((1 - beta) * s.rr.x[i] * mu_l + beta * s.rr.y[i] * mu_v, s.gibbs, correction);
        kahan_add((1 - beta) * s.rr.x[i] * (std::abs(lx) + std::abs(s.liquid.ln_phi[i])) +
                      beta * s.rr.y[i] * (std::abs(ly) + std::abs(s.vapor.ln_phi[i])),
                  magnitude, mc);
        if (!std::isfinite(s.residual[i]) || !std::isfinite(s.common[i])) {
            st = kAttemptPropertyFailure;
            return false;
        }
    }
    s.guard = 256 * kEps * magnitude;
    if (!std::isfinite(s.gibbs) || !std::isfinite(s.guard)) {
        st = kAttemptPropertyFailure;
        return false;
    }
    return true;
}

inline double gibbs_slope(const SplitState& s, const std::vector<double>& z, double scale) {
    double h = 0, hc = 0, first = 0, fc = 0, second = 0, sc = 0;  // pt_split.hpp:213-231
    for (size_t i = 0; i < z.size(); ++i) {
        if (z[i] == 0) continue;
        const double x = s.rr.x[i], y = s.rr.y[i];
        const double c = (x / z[i]) * y;
        const double d = y - x;
        const double r = s.residual[i];
        kahan_add(d * (d / z[i]), h, hc);
        kahan_add(c * r, first, fc);
        kahan_add((c * r) * r, second, sc);
    }
    if (!(h > 0) || !std::isfinite(h) || !std::isfinite(first) || !std::isfinite(second) ||
        !std::isfinite(scale) || !(scale >= 1))
        return kNaN;
    const double beta = s.rr.beta;
    return -(beta * (1 - beta) * second + (first / h) * first) / scale;
}

inline bool split_accept(const SplitState& point, const SplitState& next, double predicted,
                         double relative_step, const SplitOptions& o) {  // :232-244
    const double guard = point.guard + next.guard;
    if (predicted > guard) return next.gibbs <= point.gibbs - o.gibbs_armijo * predicted;
    return next.gibbs <= point.gibbs + guard &&
           (next.fug_norm <= o.fugacity_tolerance ||
            point.fug_norm - next.fug_norm > o.residual_decrease * relative_step * point.fug_norm);
}

inline bool split_seed(const std::vector<double>& z, const std::vector<double>& w, bool as_vapor,
                       std::vector<double>& lk) {  // :245-267
    const int n = static_cast<int>(z.size());
    double amount = 0.1;
    for (int i = 0; i < n; ++i)
        if (z[i] > 0) amount = std::min(amount, 0.5 * (z[i] / w[i]));
    if (!(amount > 0 && amount < 1)) return false;
    std::vector<double> other(n, 0.0);
    lk.assign(n, 0.0);
    for (int i = 0; i < n; ++i) {
        if (z[i] == 0) continue;
        other[i] = std::fma(-amount, w[i], z[i]) / (1 - amount);
        if (!(other[i] > 0)) return false;
    }
    const double sum = kahan_sum(other.data(), n);
    if (!std::isfinite(sum) || std::abs(sum - 1) > 64 * kEps) return false;
    for (int i = 0; i < n; ++i) {
        if (z[i] == 0) continue;
        other[i] /= sum;
        lk[i] = (as_vapor ? 1.0 : -1.0) * (std::log(w[i]) - std::log(other[i]));
        if (!std::isfinite(lk[i])) return false;
    }
    return true;
}

inline Attempt iterate_split(const Model& m, Work& wk, double p, double t, const std::vector<double>& z,
                             const std::vector<double>& lk0, const SplitOptions& o, long long budget) {
    Attempt a;
    AttemptStatus st;
    if (!split_evaluate(m, wk, p, t, z, lk0, o, a.evaluations, budget, a.point, st)) {
        a.status = st;
        return a;
    }
    a.has_point = true;
    const int n = m.n;
    SplitState next;
    std::vector<double> next_lk(n);
    for (;;) {
        const SplitState& point = a.point;
        if (point.fug_norm <= o.fugacity_tolerance) {  // :351-363
            const double beta = point.rr.beta;
            double contrast = 0;
            for (double v : point.log_k) contrast = std::max(contrast, std::abs(v));
            if (!(point.rr.mass_absolute <= o.mass_absolute_tolerance &&
                  point.rr.mass_relative <= o.mass_relative_tolerance))
                a.status = kBalanceFailure;
            else if (beta <= o.minimum_phase_fraction || 1 - beta <= o.minimum_phase_fraction)
                a.status = kPhaseDisappearance;
            else if (contrast <= o.log_k_separation ||
                     point.vapor.z - point.liquid.z <=
                         o.relative_z_separation * std::max(point.vapor.z, point.liquid.z))
                a.status = kIndistinguishable;
            else
                a.status = kConverged;
            return a;
        }
        if (a.iterations >= o.max_iterations) {
            a.status = kAttemptIterationLimit;
            return a;
        }
        const double scale = std::max(1.0, point.fug_norm / o.max_log_step);
        const double slope = gibbs_slope(point, z, scale);
        if (!std::isfinite(slope) || !(slope < 0)) {
            a.status = kAttemptLineSearchFailed;
            return a;
        }
        bool accepted = false;
        double alpha = 1;
        a.status = kAttemptLineSearchFailed;
        for (int bt = 0; bt < o.max_backtracks; ++bt, alpha *= 0.5) {
            for (int i = 0; i < n; ++i) next_lk[i] = point.log_k[i] + (alpha / scale) * point.residual[i];
            if (split_evaluate(m, wk, p, t, z, next_lk, o, a.evaluations, budget, next, st)) {
                if (split_accept(point, next, -alpha * slope, alpha / scale, o)) {
                    std::swap(a.point, next);
                    accepted = true;
                    break;
                }
            } else if (st == kAttemptEvaluationLimit) {
                a.status = st;
                return a;
            }
        }
        if (!accepted) return a;
        ++a.iterations;
    }
}

// ---------------------------------------------------------------------------
// Full VLE, modules/flash/include/mpmc/flash/pt_split.hpp:415-525
enum FlashStatus { kSinglePhase = 0, kTwoPhase = 1, kPhaseSetUnstable = 2, kIndeterminate = 3, kInvalid = -1 };
struct FlashResult {
    FlashStatus status = kIndeterminate;
    StabilityResult initial, final_review;
    bool has_candidate = false;
    SplitState candidate;
    int attempts = 0;
    int split_iterations = 0;
    long long split_evaluations = 0;
};

// The two PtSplitOptions fields a caller changes here (pt_split.hpp:45-50):
// initial_stability.automatic_starts and max_split_attempts.
struct VleOptions {
    bool initial_automatic_starts = true;
    int max_split_attempts = 16;
};

// pt_split.hpp:415-525 with its optional extra starts: `initial_starts` join
// the automatic feed-test starts, `final_starts` precede the pair's x and y in
// the review.
inline FlashResult solve_vle(const Model& m, Work& wk, double p, double t, const std::vector<double>& feed,
                             const std::vector<std::vector<double>>& initial_starts = {},
                             const std::vector<std::vector<double>>& final_starts = {},
                             const VleOptions& vo = {}) {
    FlashResult res;
    const int n = m.n;
    double sum;
    if (!std::isfinite(p) || p <= 0 || !std::isfinite(t) || t <= 0 ||
        !check_composition(feed.data(), n, sum)) {
        res.status = kInvalid;
        return res;
    }
    // the final starts are checked before any property call (:436-443)
    for (const auto& w : final_starts) {
        double wsum;
        if (static_cast<int>(w.size()) != n || !check_composition(w.data(), n, wsum)) {
            res.status = kInvalid;
            return res;
        }
        for (int i = 0; i < n; ++i)
            if ((feed[i] > 0) != (w[i] > 0)) {
                res.status = kInvalid;
                return res;
            }
    }
    StabilityOptions so;
    so.automatic_starts = vo.initial_automatic_starts;
    SplitOptions sp;
    if (!stability_test(m, wk, p, t, feed, so, initial_starts, {}, res.initial)) {
        res.status = kInvalid;
        return res;
    }
    if (res.initial.status == kNoInstabilityFound) {
        res.status = kSinglePhase;
        return res;
    }
    if (res.initial.status != kUnstable) {
        res.status = kIndeterminate;
        return res;
    }
    const std::vector<double>& z = res.initial.feed;
    int selected = -1;
    bool limit = false;
    for (size_t k = 0; k < res.initial.trials.size() && !limit; ++k) {  // :459-486
        const Trial& wit = res.initial.trials[k];
        if (wit.status != kNegativeTpd || !wit.has_point || !stability_negative(wit.point, so)) continue;
        for (bool as_vapor : {true, false}) {
            if (res.attempts >= vo.max_split_attempts || res.split_evaluations >= sp.max_evaluations) {
                limit = true;
                break;
            }
            std::vector<double> seed;
            Attempt a;
            if (split_seed(z, wit.point.w, as_vapor, seed))
                a = iterate_split(m, wk, p, t, z, seed, sp, sp.max_evaluations - res.split_evaluations);
            res.split_evaluations += a.evaluations;
            res.split_iterations += a.iterations;
            ++res.attempts;
            if (a.status == kConverged && (selected < 0 || a.point.gibbs < res.candidate.gibbs)) {
                selected = res.attempts - 1;
                res.candidate = a.point;
                res.has_candidate = true;
            }
        }
    }
    if (selected < 0) {
        res.status = kIndeterminate;
        return res;
    }
    const SplitState& cand = res.candidate;
    double feed_g = 0, correction = 0, magnitude = 1;  // :491-500
    for (int i = 0; i < n; ++i) {
        if (z[i] == 0) continue;
        const double lz = std::log(z[i]);
        const double phi = res.initial.reference.ln_phi[i];
        kahan_add(z[i] * (lz + phi), feed_g, correction);
        magnitude += z[i] * (std::abs(lz) + std::abs(phi));
    }
    const double gibbs_change = cand.gibbs - feed_g;
    const double gibbs_guard = cand.guard + 256 * kEps * magnitude;
    StabilityOptions fo;  // final_stability: the defaults, automatic starts on
    fo.tpd_tolerance += 0.5 * cand.fug_norm;
    if (!std::isfinite(gibbs_change) || !std::isfinite(gibbs_guard) || !std::isfinite(fo.tpd_tolerance)) {
        res.status = kIndeterminate;
        return res;
    }
    std::vector<std::vector<double>> starts(final_starts.begin(), final_starts.end());
    starts.push_back(cand.rr.x);
    starts.push_back(cand.rr.y);
    if (!stability_test(m, wk, p, t, z, fo, starts, cand.common, res.final_review)) {
        res.status = kInvalid;
        return res;
    }
    if (res.final_review.status == kUnstable)
        res.status = kPhaseSetUnstable;
    else if (gibbs_change > gibbs_guard)
        res.status = kIndeterminate;
    else if (res.final_review.status == kNoInstabilityFound)
        res.status = kTwoPhase;
    else
        res.status = kIndeterminate;
    return res;
}

// ---------------------------------------------------------------------------
// Three-phase continuation, modules/flash/include/mpmc/flash/pt_three_phase.hpp
struct ThreeOptions {  // :23-38
    double cp_tolerance = 1e-11;
    double mass_absolute = 1e-12;
    double mass_relative = 1e-10;
    double balance_tolerance = 2e-13;
    double minimum_phase_fraction = 1e-10;
    double log_separation = 1e-7;
    double max_log_step = 2.0;
    double residual_decrease = 1e-4;
    int max_iterations = 512;
    int max_backtracks = 32;
    int max_balance_iterations = 192;
    int max_balance_backtracks = 48;
    long long max_evaluations = 30000;
};
enum ThreeStatus {  // :40-53
    kTConverged, kTNoBalance, kTBalanceDegenerate, kTBalanceIterLimit, kTBalanceLineSearch, kTBalanceFailure,
    kTPhaseDisappearance, kTIndistinguishable, kTPropertyFailure, kTIterationLimit, kTEvaluationLimit,
    kTLineSearchFailed
};
struct ThreeState {  // :68-84
    double fraction[3] = {0, 0, 0};
    std::vector<double> x[3], ln_phi[3];
    double zf[3] = {0, 0, 0};
    std::vector<double> lk1, lk2, r1, r2, common;
    double cp_norm = 0, gibbs = 0, guard = 0, rr_residual = 0, mass_abs = 0, mass_rel = 0;
    int balance_iterations = 0;
};
struct ThreeResult {
    ThreeStatus status = kTNoBalance;
    bool has_point = false;
    ThreeState point;
    int disappearing = -1;
    int iterations = 0;
    long long evaluations = 0;
};

inline bool rr3_feasible(double b0, double b1) {  // :176-181
    return std::isfinite(b0) && std::isfinite(b1) && b0 >= 0 && b1 >= 0 && b0 + b1 <= 1.0;
}

// rr3_evaluate, :183-233: compositions of the three phases at (beta_1, beta_2)
// and the two balance residuals with their symmetric Jacobian.
inline bool rr3_evaluate(const std::vector<double>& feed, const std::vector<double>& lk1,
                         const std::vector<double>& lk2, double b0, double b1, std::vector<double> comp[3],
                         double res[2], double jac[3]) {
    if (!rr3_feasible(b0, b1)) return false;
    const int n = static_cast<int>(feed.size());
    const double beta0 = 1.0 - b0 - b1;
    for (int k = 0; k < 3; ++k) comp[k].assign(n, 0.0);
    double f0 = 0, c0 = 0, f1 = 0, c1 = 0, j00 = 0, k00 = 0, j01 = 0, k01 = 0, j11 = 0, k11 = 0;
    for (int i = 0; i < n; ++i) {
        if (feed[i] == 0) continue;
        const double shift = std::max({0.0, lk1[i], lk2[i]});
        const double e0 = std::exp(-shift);
        const double e1 = std::exp(lk1[i] - shift);
        const double e2 = std::exp(lk2[i] - shift);
        const double den = beta0 * e0 + b0 * e1 + b1 * e2;
        if (!std::isfinite(den) || !(den > 0)) return false;
        const double x0 = feed[i] * e0 / den, x1 = feed[i] * e1 / den, x2 = feed[i] * e2 / den;
        if (!std::isfinite(x0) || !std::isfinite(x1) || !std::isfinite(x2) || !(x0 > 0) || !(x1 > 0) ||
            !(x2 > 0))
            return false;
        comp[0][i] = x0;
        comp[1][i] = x1;
        comp[2][i] = x2;
        const double d1 = x1 - x0, d2 = x2 - x0;
        kahan_add(d1, f0, c0);
        kahan_add(d2, f1, c1);
        kahan_add(-(d1 * d1) / feed[i], j00, k00);
        kahan_add(-(d1 * d2) / feed[i], j01, k01);
        kahan_add(-(d2 * d2) / feed[i], j11, k11);
    }
    res[0] = f0;
    res[1] = f1;
    jac[0] = j00;
    jac[1] = j01;
    jac[2] = j11;
    return true;
}

enum Rr3Status { kRr3Success, kRr3Degenerate, kRr3IterLimit, kRr3LineSearch, kRr3Unrepresentable };
struct Rr3Result {
    Rr3Status status = kRr3Unrepresentable;
    double fraction[2] = {0, 0};
    std::vector<double> comp[3];
    double residual = std::numeric_limits<double>::infinity();
    double mass_abs = 0, mass_rel = 0;
    int iterations = 0;
};

// solve_generalized_rr3, :235-340: damped Newton on the two independent phase
// fractions inside the closed simplex, then normalised compositions and the
// material-balance errors.
inline Rr3Result solve_rr3(const std::vector<double>& feed, const std::vector<double>& lk1,
                           const std::vector<double>& lk2, const double init[2], const ThreeOptions& o) {
    Rr3Result r;
    const int n = static_cast<int>(feed.size());
    if (n == 0 || !rr3_feasible(init[0], init[1])) return r;
    for (int i = 0; i < n; ++i)
        if (!std::isfinite(lk1[i]) || !std::isfinite(lk2[i])) return r;
    double beta[2] = {init[0], init[1]};
    std::vector<double> comp[3], ncomp[3];
    double res[2], jac[3], nres[2], njac[3];
    for (int iteration = 0;; ++iteration) {
        if (!rr3_evaluate(feed, lk1, lk2, beta[0], beta[1], comp, res, jac)) return r;
        r.iterations = iteration;
        const double norm = std::max(std::abs(res[0]), std::abs(res[1]));
        if (!std::isfinite(norm)) return r;
        if (norm <= o.balance_tolerance) {
            r.status = kRr3Success;
            r.residual = norm;
            break;
        }
        if (iteration >= o.max_balance_iterations) {
            r.status = kRr3IterLimit;
            return r;
        }
        const double det = jac[0] * jac[2] - jac[1] * jac[1];
        const double det_scale = std::abs(jac[0] * jac[2]) + std::abs(jac[1] * jac[1]) + 1.0;
        if (!std::isfinite(det) || std::abs(det) <= 256.0 * kEps * det_scale) {
            r.status = kRr3Degenerate;
            return r;
        }
        const double step[2] = {(-res[0] * jac[2] + jac[1] * res[1]) / det, (jac[1] * res[0] - jac[0] * res[1]) / det};
        if (!std::isfinite(step[0]) || !std::isfinite(step[1])) return r;
        bool accepted = false;
        double alpha = 1.0;
        for (int bt = 0; bt < o.max_balance_backtracks; ++bt, alpha *= 0.5) {
            const double cand[2] = {beta[0] + alpha * step[0], beta[1] + alpha * step[1]};
            if (!rr3_feasible(cand[0], cand[1])) continue;
            if (!rr3_evaluate(feed, lk1, lk2, cand[0], cand[1], ncomp, nres, njac)) continue;
            const double next_norm = std::max(std::abs(nres[0]), std::abs(nres[1]));
            if (!std::isfinite(next_norm)) continue;
            if (next_norm < norm || next_norm <= o.balance_tolerance) {
                beta[0] = cand[0];
                beta[1] = cand[1];
                accepted = true;
                break;
            }
        }
        if (!accepted) {
            r.status = kRr3LineSearch;
            return r;
        }
    }
    if (!rr3_evaluate(feed, lk1, lk2, beta[0], beta[1], comp, res, jac)) {
        r.status = kRr3Unrepresentable;
        return r;
    }
    r.fraction[0] = beta[0];
    r.fraction[1] = beta[1];
    for (int k = 0; k < 3; ++k) {
        const double sum = kahan_sum(comp[k].data(), n);
        if (!std::isfinite(sum) || !(sum > 0)) {
            r.status = kRr3Unrepresentable;
            return r;
        }
        for (double& v : comp[k]) v /= sum;
        r.comp[k] = comp[k];
    }
    const double fr[3] = {1.0 - beta[0] - beta[1], beta[0], beta[1]};
    double abs_err = 0, rel_err = 0;
    for (int i = 0; i < n; ++i) {
        const double recovered = fr[0] * r.comp[0][i] + fr[1] * r.comp[1][i] + fr[2] * r.comp[2][i];
        const double err = std::abs(recovered - feed[i]);
        abs_err = std::max(abs_err, err);
        if (feed[i] > 0)
            rel_err = std::max(rel_err, err / feed[i]);
        else if (recovered != 0)
            rel_err = std::numeric_limits<double>::infinity();
    }
    r.mass_abs = abs_err;
    r.mass_rel = rel_err;
    return r;
}

// pt_three_phase_log_distance, :342-366
inline double log_distance(const std::vector<double>& a, const std::vector<double>& b,
                           const std::vector<double>& feed) {
    double d = 0;
    for (size_t i = 0; i < feed.size(); ++i) {
        if (feed[i] == 0) {
            if (a[i] != 0 || b[i] != 0) return std::numeric_limits<double>::infinity();
            continue;
        }
        if (!(a[i] > 0) || !(b[i] > 0)) return std::numeric_limits<double>::infinity();
        const double v = std::abs(std::log(a[i]) - std::log(b[i]));
        if (!std::isfinite(v)) return std::numeric_limits<double>::infinity();
        d = std::max(d, v);
    }
    return d;
}

// iterate_pt_three_phase, :399-676.  `upper[k]` selects phase k's root side
// (pr76_three_phase.hpp:26-106: lower = smallest, upper = largest admissible
// root); `feed` is the caller's normalised feed, normalised once more here.
inline ThreeResult iterate_three(const Model& m, Work& wk, double p, double t, const std::vector<double>& feed_in,
                                 const std::vector<double>& lk1_0, const std::vector<double>& lk2_0,
                                 const double frac0[2], const bool upper[3], const ThreeOptions& o) {
    ThreeResult res;
    const int n = m.n;
    double input_sum = 1.0;
    if (!check_composition(feed_in.data(), n, input_sum)) return res;  // a domain_error in the reference
    std::vector<double> feed(n);
    for (int i = 0; i < n; ++i) feed[i] = feed_in[i] / input_sum;
    for (int i = 0; i < n; ++i)
        if (feed_in[i] > 0 && feed[i] == 0) {
            res.status = kTBalanceFailure;
            return res;
        }
    // the state at (ln K1, ln K2); returns kTConverged for "evaluated", a
    // step-error status, or kTPropertyFailure
    SplitPhase phase;
    auto evaluate_state = [&](const std::vector<double>& lk1, const std::vector<double>& lk2, const double seed[2],
                              ThreeState& st) -> ThreeStatus {
        const Rr3Result bal = solve_rr3(feed, lk1, lk2, seed, o);
        switch (bal.status) {
        case kRr3Success: break;
        case kRr3Degenerate: return kTBalanceDegenerate;
        case kRr3IterLimit: return kTBalanceIterLimit;
        case kRr3LineSearch: return kTBalanceLineSearch;
        case kRr3Unrepresentable: return kTNoBalance;
        }
        st.fraction[0] = 1.0 - bal.fraction[0] - bal.fraction[1];
        st.fraction[1] = bal.fraction[0];
        st.fraction[2] = bal.fraction[1];
        for (int k = 0; k < 3; ++k) {
            st.x[k] = bal.comp[k];
            if (res.evaluations >= o.max_evaluations) return kTEvaluationLimit;
            ++res.evaluations;
            if (role_provider(m, wk, p, t, st.x[k].data(), upper[k], phase) != kOk) return kTPropertyFailure;
            for (double v : phase.ln_phi)
                if (!std::isfinite(v)) return kTPropertyFailure;
            st.ln_phi[k] = phase.ln_phi;
            st.zf[k] = phase.z;
        }
        st.rr_residual = bal.residual;
        st.mass_abs = bal.mass_abs;
        st.mass_rel = bal.mass_rel;
        st.balance_iterations = bal.iterations;
        st.lk1.assign(n, 0.0);
        st.lk2.assign(n, 0.0);
        st.r1.assign(n, 0.0);
        st.r2.assign(n, 0.0);
        st.common.assign(n, 0.0);
        st.cp_norm = 0;
        st.gibbs = 0;
        double gc = 0, magnitude = 1, mc = 0;
        for (int i = 0; i < n; ++i) {
            if (feed[i] == 0) continue;
            const double l0 = std::log(st.x[0][i]), l1 = std::log(st.x[1][i]), l2 = std::log(st.x[2][i]);
            const double mu0 = l0 + st.ln_phi[0][i], mu1 = l1 + st.ln_phi[1][i], mu2 = l2 + st.ln_phi[2][i];
            st.lk1[i] = l1 - l0;
            st.lk2[i] = l2 - l0;
            st.r1[i] = mu0 - mu1;
            st.r2[i] = mu0 - mu2;
            st.common[i] = (mu0 + mu1 + mu2) / 3.0;
            st.cp_norm = std::max({st.cp_norm, std::abs(st.r1[i]), std::abs(st.r2[i])});
            for (int k = 0; k < 3; ++k) {
                const double lx = std::log(st.x[k][i]);
                const double mu = lx + st.ln_phi[k][i];
                kahan_add(st.fraction[k] * st.x[k][i] * mu, st.gibbs, gc);
                kahan_add(st.fraction[k] * st.x[k][i] * (std::abs(lx) + std::abs(st.ln_phi[k][i])), magnitude, mc);
            }
        }
        st.guard = 256.0 * kEps * magnitude;
        if (!std::isfinite(st.cp_norm) || !std::isfinite(st.gibbs) || !std::isfinite(st.guard))
            return kTPropertyFailure;
        return kTConverged;
    };
    {
        const ThreeStatus s = evaluate_state(lk1_0, lk2_0, frac0, res.point);
        if (s != kTConverged) {
            res.status = s;
            return res;
        }
        res.has_point = true;
    }
    ThreeState next;
    std::vector<double> nk1(n), nk2(n);
    for (;;) {
        ThreeState& pt = res.point;
        if (pt.cp_norm <= o.cp_tolerance) {
            if (pt.rr_residual > o.balance_tolerance || pt.mass_abs > o.mass_absolute || pt.mass_rel > o.mass_relative) {
                res.status = kTBalanceFailure;
                return res;
            }
            for (int k = 0; k < 3; ++k)
                if (pt.fraction[k] <= o.minimum_phase_fraction) {
                    res.status = kTPhaseDisappearance;
                    res.disappearing = k;
                    return res;
                }
            const double d01 = log_distance(pt.x[0], pt.x[1], feed), d02 = log_distance(pt.x[0], pt.x[2], feed),
                         d12 = log_distance(pt.x[1], pt.x[2], feed);
            if (!(d01 > o.log_separation) || !(d02 > o.log_separation) || !(d12 > o.log_separation)) {
                res.status = kTIndistinguishable;
                return res;
            }
            res.status = kTConverged;
            return res;
        }
        if (res.iterations >= o.max_iterations) {
            res.status = kTIterationLimit;
            return res;
        }
        const double scale = std::max(1.0, pt.cp_norm / o.max_log_step);
        bool accepted = false;
        double alpha = 1.0;
        for (int bt = 0; bt < o.max_backtracks; ++bt, alpha *= 0.5) {
            for (int i = 0; i < n; ++i) {
                nk1[i] = pt.lk1[i] + (alpha / scale) * pt.r1[i];
                nk2[i] = pt.lk2[i] + (alpha / scale) * pt.r2[i];
            }
            const double seed[2] = {pt.fraction[1], pt.fraction[2]};
            const ThreeStatus s = evaluate_state(nk1, nk2, seed, next);
            if (s == kTEvaluationLimit) {
                res.status = s;
                return res;
            }
            if (s != kTConverged) continue;  // rejected evaluation
            const double required = o.residual_decrease * (alpha / scale) * pt.cp_norm;
            const bool progress = next.cp_norm <= o.cp_tolerance || pt.cp_norm - next.cp_norm > required;
            const bool gibbs_ok = next.gibbs <= pt.gibbs + pt.guard + next.guard;
            if (progress && gibbs_ok) {
                std::swap(res.point, next);
                accepted = true;
                break;
            }
        }
        if (!accepted) {
            res.status = kTLineSearchFailed;
            return res;
        }
        ++res.iterations;
    }
}

// ---------------------------------------------------------------------------
// Max-3-phase orchestration, modules/flash/include/mpmc/flash/pr76_three_phase.hpp:328-561
// with the backend's default options (pr76_pt_flash_backend.hpp:190-206: no
// caller start hints, 16 automatic attempts, new-phase seed fraction 0.1).
enum Max3Status { kM3Single = 0, kM3Two = 1, kM3Three = 2, kM3Boundary = 3, kM3Higher = 4, kM3Indeterminate = 5 };
struct Max3Result {
    int status = kM3Indeterminate;  // Max3Status, or -1 for an invalid request
    FlashResult base;
    bool has_three = false;
    ThreeState three;
    bool has_neighbor = false;
    FlashResult neighbor;
    int attempts = 0;
};

// ln(a_i / b_i) on the feed support, pr76_three_phase.hpp:246-268
inline bool log_ratio(const std::vector<double>& a, const std::vector<double>& b, const std::vector<double>& feed,
                      std::vector<double>& out) {
    out.assign(feed.size(), 0.0);
    for (size_t i = 0; i < feed.size(); ++i) {
        if (feed[i] == 0) {
            if (a[i] != 0 || b[i] != 0) return false;
            continue;
        }
        if (!(a[i] > 0) || !(b[i] > 0)) return false;
        out[i] = std::log(a[i]) - std::log(b[i]);
        if (!std::isfinite(out[i])) return false;
    }
    return true;
}

// Root sides a witness may follow, pr76_three_phase.hpp:270-300: the side of
// the admissible root the witness sits on, both when there is only one.
inline int witness_sides(const Model& m, Work& wk, double p, double t, const std::vector<double>& w, int branch,
                         bool sides[2]) {
    double amix, bmix, A, B;
    if (!mix(m, wk.tc, w.data(), amix, bmix, wk.sums.data()) || !coefficients(p, t, amix, bmix, A, B)) return 0;
    const RootSet roots = solve_roots(A, B);
    if (roots.status != kRootSuccess) return 0;
    int adm[3], na = 0;
    for (int k = 0; k < roots.count; ++k)
        if (roots.roots[k].slope_sign > 0) adm[na++] = k;
    bool found = false;
    for (int k = 0; k < na; ++k) found = found || adm[k] == branch;
    if (na == 0 || !found) return 0;
    if (na == 1) {
        sides[0] = false;
        sides[1] = true;
        return 2;
    }
    if (branch == adm[0]) {
        sides[0] = false;
        return 1;
    }
    if (branch == adm[na - 1]) {
        sides[0] = true;
        return 1;
    }
    return 0;
}

// A caller's three-phase start (pr76_three_phase.hpp:110-116): three
// compositions and the independent fractions (beta_1, beta_2).
struct ThreeStart {
    std::vector<double> x[3];
    double fraction[2] = {1.0 / 3.0, 1.0 / 3.0};
};

// `initial_starts` / `final_starts` are the two-phase solve's extra stability
// starts and `three_starts` the caller's three-phase starts
// (pr76_three_phase.hpp:328-336, 457-486); each start class has its own
// quota of 16 attempts.
inline Max3Result solve_max3(const Model& m, Work& wk, double p, double t, const std::vector<double>& feed,
                             const std::vector<std::vector<double>>& initial_starts = {},
                             const std::vector<std::vector<double>>& final_starts = {},
                             const std::vector<ThreeStart>& three_starts = {}, const VleOptions& vo = {}) {
    Max3Result r;
    // pr76_pt_max3_check_starts, :211-244: a bad start is a domain_error
    for (const ThreeStart& st : three_starts) {
        if (!rr3_feasible(st.fraction[0], st.fraction[1])) {
            r.status = -1;
            return r;
        }
        for (int k = 0; k < 3; ++k) {
            double sum;
            if (static_cast<int>(st.x[k].size()) != m.n || !check_composition(st.x[k].data(), m.n, sum)) {
                r.status = -1;
                return r;
            }
            for (int i = 0; i < m.n; ++i)
                if ((feed[i] > 0) != (st.x[k][i] > 0)) {
                    r.status = -1;
                    return r;
                }
        }
    }
    r.base = solve_vle(m, wk, p, t, feed, initial_starts, final_starts, vo);
    switch (r.base.status) {
    case kInvalid: r.status = -1; return r;
    case kSinglePhase: r.status = kM3Single; return r;
    case kTwoPhase: r.status = kM3Two; return r;
    case kIndeterminate: r.status = kM3Indeterminate; return r;
    case kPhaseSetUnstable: break;
    }
    if (!r.base.has_candidate) {
        r.status = kM3Indeterminate;
        return r;
    }
    const SplitState& pair = r.base.candidate;
    const StabilityResult& review = r.base.final_review;
    const std::vector<double>& nfeed = r.base.initial.feed;
    const ThreeOptions to;
    bool saw_higher = false, saw_boundary = false, limit = false, hint_limit = false;
    int automatic = 0, supplied = 0;
    // run_attempt of pr76_three_phase.hpp:379-455; true when the cell is settled
    auto run_attempt = [&](const std::vector<double>& lk1, const std::vector<double>& lk2, const double fr[2],
                           const bool upper[3], bool from_hint = false) -> bool {
        int& used = from_hint ? supplied : automatic;
        if (used >= 16) {
            (from_hint ? hint_limit : limit) = true;
            return false;
        }
        ++used;
        ++r.attempts;
        const ThreeResult eq = iterate_three(m, wk, p, t, nfeed, lk1, lk2, fr, upper, to);
        if (eq.status == kTPhaseDisappearance) {
            saw_boundary = true;
            std::vector<std::vector<double>> starts;
            for (int k = 0; k < 3; ++k)
                if (k != eq.disappearing) starts.push_back(eq.point.x[k]);
            if (starts.size() == 2) {
                // options.two_phase again (pr76_three_phase.hpp:413-415)
                FlashResult nb = solve_vle(m, wk, p, t, nfeed, starts, starts, vo);
                if (nb.status == kTwoPhase) {
                    r.neighbor = nb;
                    r.has_neighbor = true;
                    r.status = kM3Two;
                    return true;
                }
            }
            return false;
        }
        const bool admissible = eq.status == kTConverged && eq.has_point && eq.point.cp_norm <= to.cp_tolerance &&
                                eq.point.rr_residual <= to.balance_tolerance &&
                                eq.point.mass_abs <= to.mass_absolute && eq.point.mass_rel <= to.mass_relative;
        if (!admissible) return false;
        const ThreeState& cand = eq.point;
        StabilityOptions fo;
        fo.tpd_tolerance += cand.cp_norm;
        std::vector<std::vector<double>> starts{cand.x[0], cand.x[1], cand.x[2]};
        StabilityResult fin;
        if (!stability_test(m, wk, p, t, nfeed, fo, starts, cand.common, fin)) {
            r.status = -1;  // a domain_error out of the reference's review
            return true;
        }
        if (fin.status == kUnstable) {
            saw_higher = true;
        } else if (fin.status == kNoInstabilityFound) {
            r.three = cand;
            r.has_three = true;
            r.status = kM3Three;
            return true;
        }
        return false;
    };
    std::vector<double> lk1, lk2;
    // caller starts first, every combination of root sides (:457-486)
    for (const ThreeStart& st : three_starts) {
        if (!log_ratio(st.x[1], st.x[0], nfeed, lk1) || !log_ratio(st.x[2], st.x[0], nfeed, lk2)) continue;
        for (int s0 = 0; s0 < 2 && !hint_limit; ++s0)
            for (int s1 = 0; s1 < 2 && !hint_limit; ++s1)
                for (int s2 = 0; s2 < 2 && !hint_limit; ++s2) {
                    const bool upper[3] = {s0 == 1, s1 == 1, s2 == 1};
                    if (run_attempt(lk1, lk2, st.fraction, upper, true)) return r;
                }
        if (hint_limit) break;
    }
    if (log_ratio(pair.rr.y, pair.rr.x, nfeed, lk1)) {
        for (const Trial& wit : review.trials) {
            if (wit.status != kNegativeTpd || !wit.has_point) continue;
            if (!log_ratio(wit.point.w, pair.rr.x, nfeed, lk2)) continue;
            bool sides[2];
            const int ns = witness_sides(m, wk, p, t, wit.point.w, wit.point.branch, sides);
            for (int k = 0; k < ns; ++k) {
                const double beta_v = pair.rr.beta;
                const double fr[2] = {(1.0 - 0.1) * beta_v, 0.1};
                const bool upper[3] = {false, true, sides[k]};
                if (run_attempt(lk1, lk2, fr, upper)) return r;
                if (limit) break;
            }
            if (limit) break;
        }
    }
    r.status = saw_higher ? kM3Higher : (saw_boundary ? kM3Boundary : kM3Indeterminate);
    return r;
}

// Ordered-path continuation, pr76_pt_continuation.hpp:183-306 (default
// options): every point is a max3 solve whose extra stability starts are the
// previous accepted point's phase compositions and whose three-phase start
// is the previous three-phase set; hints reset after an unresolved point.
// Writes each point's max3 status; false for an invalid path or feed (the
// reference throws).
inline bool solve_continuation(const Model& m, Work& wk, const double* p, const double* t, int npoint,
                               const std::vector<double>& feed_in, int* status) {
    for (int k = 0; k < npoint; ++k)
        if (!std::isfinite(p[k]) || !(p[k] > 0) || !std::isfinite(t[k]) || !(t[k] > 0)) return false;
    double sum;
    if (!check_composition(feed_in.data(), m.n, sum)) return false;
    std::vector<double> feed(m.n);
    for (int i = 0; i < m.n; ++i) feed[i] = feed_in[i] / sum;
    bool have_prev = false, have_three = false;
    std::vector<std::vector<double>> prev;
    ThreeStart three;
    for (int k = 0; k < npoint; ++k) {
        std::vector<std::vector<double>> starts;
        if (have_prev)
            for (const auto& c : prev) {  // pr76_pt_continuation_append_unique, :106-118
                bool dup = false;
                for (const auto& e : starts) dup = dup || e == c;
                if (!dup) starts.push_back(c);
            }
        std::vector<ThreeStart> hints;
        if (have_three) hints.push_back(three);
        if (!make_temp_cache(m, t[k], wk.tc)) return false;
        const Max3Result r = solve_max3(m, wk, p[k], t[k], feed, starts, starts, hints);
        if (r.status < 0) return false;
        status[k] = r.status;
        prev.clear();
        have_three = false;
        switch (r.status) {  // phase compositions of the accepted point, :118-146
        case kM3Single: prev.push_back(r.base.initial.feed); break;
        case kM3Two: {
            const FlashResult& src = r.has_neighbor ? r.neighbor : r.base;
            if (src.has_candidate) {
                prev.push_back(src.candidate.rr.x);
                prev.push_back(src.candidate.rr.y);
            }
            break;
        }
        case kM3Three:
            for (int q = 0; q < 3; ++q) prev.push_back(r.three.x[q]);
            for (int q = 0; q < 3; ++q) three.x[q] = r.three.x[q];
            three.fraction[0] = r.three.fraction[1];
            three.fraction[1] = r.three.fraction[2];
            have_three = true;
            break;
        default: break;
        }
        have_prev = r.status == kM3Single || r.status == kM3Two || r.status == kM3Three;
    }
    return true;
}

// ---------------------------------------------------------------------------
// Forward-mode phase evaluation (generic Number), pr76_mixture.hpp:125-219 and
// pr76_phase.hpp:193-258.  x holds all n fractions already in Number form.
// Returns 0 or the class of the reference's throw: 2 a range/domain error of
// the mixing or the coefficients, 3 an unresolved root set (Pr76PhaseError),
// 4 a root index out of range, 5 a root without a reliable derivative, 2 a
// non-representable ln phi or Z (the codes of the selected-phase chart).
enum EvalIssue { kEvalOk = 0, kEvalDomain = 2, kEvalRootSet = 3, kEvalRootIndex = 4, kEvalIllConditioned = 5 };
template <class Num>
inline int phase_eval_status(const Model& m, const Num& p, const Num& t, const std::vector<Num>& x,
                             int root_index, Num& z_out, std::vector<Num>& ln_phi) {
    const int n = m.n;
    std::vector<Num> a(n), root(n), sums(n);
    Num attraction(0.0), covolume(0.0);
    for (int i = 0; i < n; ++i) {
        const Num reduced_root = sqrt(t) / m.sqrt_tc[i];
        const Num bracket = 1.0 + m.kappa[i] * (1.0 - reduced_root);
        a[i] = (bracket * m.ac[i]) * bracket;
        attraction = attraction + (x[i] * a[i]) * x[i];
        covolume = covolume + x[i] * m.b[i];
        sums[i] = x[i] * a[i];
        if (n > 1) {
            if (!(val(a[i]) > 0.0)) return kEvalDomain;  // pr76_mixture.hpp:180-182
            root[i] = sqrt(a[i]);
        }
    }
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j) {
            const Num cross = ((x[i] * root[i]) * (x[j] * root[j])) * m.factor[i * n + j];
            attraction = attraction + cross;
            attraction = attraction + cross;
            const Num aij = (root[i] * m.factor[i * n + j]) * root[j];
            sums[i] = sums[i] + x[j] * aij;
            sums[j] = sums[j] + x[i] * aij;
        }
    if (!finite(attraction) || !finite(covolume) || !(val(covolume) > 0.0)) return kEvalDomain;
    const Num rt = kR * t;
    const Num prt = p / rt;
    const Num A = (attraction / rt) * prt;
    const Num B = covolume * prt;
    if (!finite(A) || !finite(B) || !(val(B) > 0.0) || (val(A) == 0.0 && val(attraction) != 0.0))
        return kEvalDomain;  // pr76_phase.hpp:175-191
    const RootSet roots = solve_roots(val(A), val(B));
    if (roots.status != kRootSuccess) return kEvalRootSet;
    if (root_index < 0 || root_index >= roots.count) return kEvalRootIndex;
    const Root& rootv = roots.roots[root_index];
    Num free_volume(rootv.free_volume);
    {
        // First-order implicit function theorem on the scaled cubic,
        // pr76_phase.hpp:208-222.
        if (!rootv.derivative_valid) return kEvalIllConditioned;
        const double y0 = rootv.free_volume / roots.scale;
        const double scale = roots.scale;
        const Num bs = B / scale;
        const double inv = 1.0 / scale;
        const Num c2 = 4.0 * bs - inv;
        const Num c1 = (A / scale) / scale + 2.0 * bs * bs - 4.0 * bs * inv;
        const Num c0 = ((-2.0 * bs) * bs) * inv;
        const Num residual = ((Num(y0) + c2) * y0 + c1) * y0 + c0;
        const double dh = (3.0 * y0 + 2.0 * val(c2)) * y0 + val(c1);
        free_volume = free_volume - ((residual - Num(val(residual))) / dh) * scale;
    }
    const Num z = free_volume + B;
    const double sqrt2 = std::sqrt(2.0);
    const Num denominator = free_volume + (2.0 - sqrt2) * B;
    const Num u = (2.0 * sqrt2) * (B / denominator);
    const Num log_factor = log1p_over_x(u) / denominator;
    Num z_minus_one = z - 1.0;
    Num log_free = log(free_volume);
    if (std::abs(val(z_minus_one)) < 0.25 && val(B) < 0.125) {
        const Num bz = B / z;
        z_minus_one = B / free_volume - (A / z) / (1.0 + 2.0 * bz - bz * bz);
        log_free = log1p(z_minus_one - B);
    }
    ln_phi.resize(n);
    for (int i = 0; i < n; ++i) {
        const Num ratio = Num(m.b[i]) / covolume;
        const Num coefficient = ((2.0 * sums[i] - attraction * ratio) / rt) * prt;
        ln_phi[i] = ratio * z_minus_one - log_free - coefficient * log_factor;
        if (!finite(ln_phi[i])) return kEvalDomain;
    }
    z_out = z;
    return finite(z) ? kEvalOk : kEvalDomain;
}

template <class Num>
inline bool phase_eval_ad(const Model& m, const Num& p, const Num& t, const std::vector<Num>& x,
                          int root_index, Num& z_out, std::vector<Num>& ln_phi) {
    return phase_eval_status(m, p, t, x, root_index, z_out, ln_phi) == kEvalOk;
}

// Sensitivity outputs (reduced chart q = p, T, z_0..z_{n-2}).
struct Sensitivity {
    int status = 6;  // PtSensitivityStatus; 0 = success
    std::vector<double> dlnk, dx, dy;  // n x (n+1), row-major
    std::vector<double> dbeta;         // n+1
    std::vector<double> dzl, dzv, drhol, drhov;  // n+1 (closure linearisation)
    std::vector<double> jl, jv;        // (n+1) x (n+2): d[Z, ln phi]/d[p, T, x_full]
    double rcond = 0.0;                // reciprocal condition estimate of dF/dln K (test diagnostics)
};

// LU with partial pivoting + rcond, pt_sensitivity_detail.hpp:364-471
struct Lu {
    int n = 0;
    std::vector<double> v;
    std::vector<int> piv;
    double norm_inf = 0;
};
inline bool lu_factor(const std::vector<double>& a, int n, Lu& f) {
    f.n = n;
    f.v = a;
    f.piv.assign(n, 0);
    f.norm_inf = 0;
    for (int r = 0; r < n; ++r) {
        double s = 0;
        for (int c = 0; c < n; ++c) s += std::abs(a[r * n + c]);
        f.norm_inf = std::max(f.norm_inf, s);
    }
    if (!(f.norm_inf > 0) || !std::isfinite(f.norm_inf)) return false;
    const double guard = 64.0 * kEps * n * f.norm_inf;
    for (int c = 0; c < n; ++c) {
        int piv = c;
        double mag = std::abs(f.v[c * n + c]);
        for (int r = c + 1; r < n; ++r) {
            const double cand = std::abs(f.v[r * n + c]);
            if (cand > mag) {
                mag = cand;
                piv = r;
            }
        }
        if (!std::isfinite(mag) || !(mag > guard)) return false;
        f.piv[c] = piv;
        if (piv != c)
            for (int j = 0; j < n; ++j) std::swap(f.v[c * n + j], f.v[piv * n + j]);
        const double diag = f.v[c * n + c];
        for (int r = c + 1; r < n; ++r) {
            const double mult = f.v[r * n + c] / diag;
            f.v[r * n + c] = mult;
            for (int j = c + 1; j < n; ++j) f.v[r * n + j] -= mult * f.v[c * n + j];
        }
    }
    return true;
}
inline bool lu_solve(const Lu& f, std::vector<double>& rhs) {
    const int n = f.n;
    for (int c = 0; c < n; ++c)
        if (f.piv[c] != c) std::swap(rhs[c], rhs[f.piv[c]]);
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < r; ++c) rhs[r] -= f.v[r * n + c] * rhs[c];
    for (int r = n - 1; r >= 0; --r) {
        for (int c = r + 1; c < n; ++c) rhs[r] -= f.v[r * n + c] * rhs[c];
        rhs[r] /= f.v[r * n + r];
        if (!std::isfinite(rhs[r])) return false;
    }
    return true;
}
inline double lu_rcond(const Lu& f) {
    const int n = f.n;
    std::vector<double> rows(n, 0.0);
    for (int c = 0; c < n; ++c) {
        std::vector<double> e(n, 0.0);
        e[c] = 1;
        if (!lu_solve(f, e)) return 0;
        for (int r = 0; r < n; ++r) rows[r] += std::abs(e[r]);
    }
    const double inv = *std::max_element(rows.begin(), rows.end());
    const double prod = f.norm_inf * inv;
    if (!(prod > 0) || !std::isfinite(prod)) return 0;
    return 1 / prod;
}

// differentiate_pr76_pt_vle, modules/flash/include/mpmc/flash/pr76_sensitivity.hpp:51-390,
// with the local system of detail/pr76_sensitivity_local.hpp:29-109 and the RR
// linearisation of detail/pt_sensitivity_detail.hpp:46-143; closure dZ/drho of
// modules/physics/include/mpmc/physics/pr76_thermodynamic_closure.hpp:279-337;
// per-phase full-chart Jacobians of pr76_phase_ad.hpp:57-122.
// Test diagnostics: when set, d(ln x_i - ln y_i) is taken as -d ln K_i, the
// exact value on the RR manifold (y_i = K_i x_i), instead of through the
// dependent last fractions of the reference's RR linearisation, whose
// cancellation error eps * sum|dx| / x_{n-1} is the reference's own rounding
// noise in the last component's row.  Off by default (the restatement).
inline std::atomic<int> g_manifold_identity{0};

inline void differentiate(const Model& m, const FlashResult& fr, double p, double t, Sensitivity& s) {
    const int n = m.n;
    const int q = n + 1;
    s = Sensitivity();
    if (fr.status != kTwoPhase || !fr.has_candidate) {
        s.status = 1;  // solution_not_accepted
        return;
    }
    const std::vector<double>& feed = fr.initial.feed;
    for (double v : feed)
        if (!(v > 0)) {
            s.status = 3;  // unsupported_feed_support
            return;
        }
    const SplitState& c = fr.candidate;
    double contrast = 0;
    for (double v : c.log_k) contrast = std::max(contrast, std::abs(v));
    if (!(contrast > 1e-7) || !(c.vapor.z - c.liquid.z > 1e-8 * std::max(c.vapor.z, c.liquid.z))) {
        s.status = 2;  // phase_boundary
        return;
    }
    const double beta = c.rr.beta;
    const double guard = std::max(1.490116119384765625e-8, 1e-10);
    if (!(beta > guard) || !(1 - beta > guard)) {
        s.status = 2;
        return;
    }
    if (!(c.fug_norm <= 1e-11)) {
        s.status = 1;
        return;
    }
    // Base RR point, pt_sensitivity_detail.hpp:269-300
    std::vector<double> xb(n), yb(n);
    double xs = 0, ys = 0;
    for (int i = 0; i + 1 < n; ++i) {
        xb[i] = c.rr.x[i];
        yb[i] = c.rr.y[i];
        xs += xb[i];
        ys += yb[i];
    }
    xb[n - 1] = 1.0 - xs;
    yb[n - 1] = 1.0 - ys;
    for (int i = 0; i < n; ++i)
        if (!(xb[i] > 0) || !(yb[i] > 0)) {
            s.status = 2;
            return;
        }
    double h = 0;
    for (int i = 0; i < n; ++i) {
        const double d = yb[i] - xb[i];
        h += d * d / feed[i];
    }
    if (!std::isfinite(h) || !(h > 0)) {
        s.status = 5;
        return;
    }
    // Local system Jacobian: variables [lnK(n), p, T, z_0..z_{n-2}],
    // outputs [F(n), beta, x(n), y(n)].  One tangent direction per pass.
    const int nv = 2 * n + 1, no = 3 * n + 1;
    std::vector<double> J(static_cast<size_t>(no) * nv), F(no);
    for (int v = 0; v < nv; ++v) {
        std::vector<D1> lk(n), zf(n);
        for (int i = 0; i < n; ++i) lk[i] = D1(c.log_k[i], v == i ? 1.0 : 0.0);
        D1 pd(p, v == n ? 1.0 : 0.0), td(t, v == n + 1 ? 1.0 : 0.0);
        D1 fsum(0.0);
        for (int i = 0; i + 1 < n; ++i) {
            zf[i] = D1(feed[i], v == n + 2 + i ? 1.0 : 0.0);
            fsum = fsum + zf[i];
        }
        zf[n - 1] = 1.0 - fsum;
        double num = 0;
        for (int i = 0; i < n; ++i) {
            const double zi = zf[i].v;
            num += (xb[i] * yb[i] / zi) * lk[i].d + ((yb[i] - xb[i]) / zi) * zf[i].d;
        }
        const double dbeta = num / h;
        std::vector<D1> xl(n), yv(n);
        D1 lsum(0.0), vsum(0.0);
        for (int i = 0; i + 1 < n; ++i) {
            const double zi = zf[i].v;
            const double dlx = zf[i].d / zi - ((yb[i] - xb[i]) / zi) * dbeta - beta * (yb[i] / zi) * lk[i].d;
            xl[i] = D1(xb[i], xb[i] * dlx);
            yv[i] = D1(yb[i], yb[i] * (dlx + lk[i].d));
            lsum = lsum + xl[i];
            vsum = vsum + yv[i];
        }
        xl[n - 1] = 1.0 - lsum;
        yv[n - 1] = 1.0 - vsum;
        D1 zl, zv;
        std::vector<D1> pl, pv;
        if (!phase_eval_ad(m, pd, td, xl, c.liquid.branch, zl, pl) ||
            !phase_eval_ad(m, pd, td, yv, c.vapor.branch, zv, pv)) {
            s.status = 4;  // property_failure
            return;
        }
        const bool identity = g_manifold_identity.load() != 0;
        for (int i = 0; i < n; ++i) {
            D1 fi = log(xl[i]) - log(yv[i]) + pl[i] - pv[i];
            if (identity) fi.d = -lk[i].d + pl[i].d - pv[i].d;
            J[i * nv + v] = fi.d;
            F[i] = fi.v;
        }
        J[n * nv + v] = dbeta;
        F[n] = beta;
        for (int i = 0; i < n; ++i) {
            J[(n + 1 + i) * nv + v] = xl[i].d;
            J[(2 * n + 1 + i) * nv + v] = yv[i].d;
            F[n + 1 + i] = xl[i].v;
            F[2 * n + 1 + i] = yv[i].v;
        }
    }
    const double arithmetic_scale = 8192.0 * kEps * n;  // pr76_sensitivity.hpp:219-229
    double res_norm = 0;
    for (int i = 0; i < n; ++i) res_norm = std::max(res_norm, std::abs(F[i]));
    if (res_norm > 1e-11 + arithmetic_scale) {
        s.status = 1;
        return;
    }
    std::vector<double> A(n * n), Bm(n * q);
    for (int r = 0; r < n; ++r) {
        for (int cc = 0; cc < n; ++cc) A[r * n + cc] = J[r * nv + cc];
        for (int cc = 0; cc < q; ++cc) Bm[r * q + cc] = J[r * nv + n + cc];
    }
    Lu f;
    if (!lu_factor(A, n, f)) {
        s.status = 5;
        return;
    }
    const double rc = lu_rcond(f);
    s.rcond = rc;
    if (!std::isfinite(rc) || !(rc > 256.0 * kEps * n)) {
        s.status = 5;
        return;
    }
    s.dlnk.assign(n * q, 0.0);
    for (int cc = 0; cc < q; ++cc) {
        std::vector<double> rhs(n);
        for (int r = 0; r < n; ++r) rhs[r] = -Bm[r * q + cc];
        if (!lu_solve(f, rhs)) {
            s.status = 5;
            return;
        }
        for (int r = 0; r < n; ++r) s.dlnk[r * q + cc] = rhs[r];
    }
    double backward = 0;
    for (int cc = 0; cc < q; ++cc)
        for (int r = 0; r < n; ++r) {
            double res = Bm[r * q + cc], sc = std::abs(res);
            for (int j = 0; j < n; ++j) {
                const double term = A[r * n + j] * s.dlnk[j * q + cc];
                res += term;
                sc += std::abs(term);
            }
            backward = std::max(backward, std::abs(res) / std::max(1.0, sc));
        }
    if (!std::isfinite(backward) || backward > arithmetic_scale) {
        s.status = 6;
        return;
    }
    auto total = [&](int out, int col) {
        double v = J[out * nv + n + col];
        for (int j = 0; j < n; ++j) v += J[out * nv + j] * s.dlnk[j * q + col];
        return v;
    };
    s.dbeta.assign(q, 0.0);
    s.dx.assign(n * q, 0.0);
    s.dy.assign(n * q, 0.0);
    for (int cc = 0; cc < q; ++cc) {
        s.dbeta[cc] = total(n, cc);
        for (int i = 0; i < n; ++i) {
            s.dx[i * q + cc] = total(n + 1 + i, cc);
            s.dy[i * q + cc] = total(2 * n + 1 + i, cc);
        }
    }
    for (double v : s.dbeta) if (!std::isfinite(v)) { s.status = 6; return; }
    for (double v : s.dx) if (!std::isfinite(v)) { s.status = 6; return; }
    for (double v : s.dy) if (!std::isfinite(v)) { s.status = 6; return; }
    for (int cc = 0; cc < q; ++cc) {  // :346-385
        double ls = 0, vs = 0;
        for (int i = 0; i < n; ++i) {
            ls += s.dx[i * q + cc];
            vs += s.dy[i * q + cc];
        }
        if (std::abs(ls) > arithmetic_scale || std::abs(vs) > arithmetic_scale) {
            s.status = 6;
            return;
        }
        for (int i = 0; i < n; ++i) {
            const double dz = cc < 2 ? 0.0 : (i == cc - 2 ? 1.0 : (i + 1 == n ? -1.0 : 0.0));
            const double xv = F[n + 1 + i], yv = F[2 * n + 1 + i];
            const double der = (1 - beta) * s.dx[i * q + cc] + beta * s.dy[i * q + cc] +
                               (yv - xv) * s.dbeta[cc] - dz;
            const double sc = std::max(1.0, std::abs(s.dx[i * q + cc]) + std::abs(s.dy[i * q + cc]) +
                                                std::abs(s.dbeta[cc]) + std::abs(dz));
            if (std::abs(der) > arithmetic_scale * sc) {
                s.status = 6;
                return;
            }
        }
    }
    s.status = 0;
    // Per-phase full-chart Jacobians d[Z, ln phi]/d[p, T, x_0..x_{n-1}].
    for (int ph = 0; ph < 2; ++ph) {
        const std::vector<double>& comp = ph == 0 ? c.rr.x : c.rr.y;
        const int branch = ph == 0 ? c.liquid.branch : c.vapor.branch;
        std::vector<double>& jac = ph == 0 ? s.jl : s.jv;
        jac.assign((n + 1) * (n + 2), 0.0);
        for (int v = 0; v < n + 2; ++v) {
            D1 pd(p, v == 0 ? 1.0 : 0.0), td(t, v == 1 ? 1.0 : 0.0);
            std::vector<D1> xs2(n);
            for (int i = 0; i < n; ++i) xs2[i] = D1(comp[i], v == 2 + i ? 1.0 : 0.0);
            D1 zz;
            std::vector<D1> lp;
            if (!phase_eval_ad(m, pd, td, xs2, branch, zz, lp)) {
                s.status = 4;
                return;
            }
            jac[0 * (n + 2) + v] = zz.d;
            for (int i = 0; i < n; ++i) jac[(1 + i) * (n + 2) + v] = lp[i].d;
        }
    }
    // Closure dZ and d(rho), pr76_thermodynamic_closure.hpp:81-118, 309-337.
    s.dzl.assign(q, 0.0);
    s.dzv.assign(q, 0.0);
    s.drhol.assign(q, 0.0);
    s.drhov.assign(q, 0.0);
    for (int ph = 0; ph < 2; ++ph) {
        const std::vector<double>& comp = ph == 0 ? c.rr.x : c.rr.y;
        const int branch = ph == 0 ? c.liquid.branch : c.vapor.branch;
        std::vector<double> grad(q);
        for (int v = 0; v < q; ++v) {
            D1 pd(p, v == 0 ? 1.0 : 0.0), td(t, v == 1 ? 1.0 : 0.0);
            std::vector<D1> xs2(n);
            D1 ssum(0.0);
            for (int i = 0; i + 1 < n; ++i) {
                xs2[i] = D1(comp[i], v == 2 + i ? 1.0 : 0.0);
                ssum = ssum + xs2[i];
            }
            xs2[n - 1] = 1.0 - ssum;
            D1 zz;
            std::vector<D1> lp;
            if (!phase_eval_ad(m, pd, td, xs2, branch, zz, lp)) {
                s.status = 4;
                return;
            }
            grad[v] = zz.d;
        }
        const double zph = ph == 0 ? c.liquid.z : c.vapor.z;
        const double rho = p / (zph * kR * t);
        const std::vector<double>& dcomp = ph == 0 ? s.dx : s.dy;
        for (int cc = 0; cc < q; ++cc) {
            double dz = cc == 0 ? grad[0] : (cc == 1 ? grad[1] : 0.0);
            for (int k = 0; k + 1 < n; ++k) dz += grad[2 + k] * dcomp[k * q + cc];
            const double dp = cc == 0 ? 1.0 / p : 0.0;
            const double dt = cc == 1 ? 1.0 / t : 0.0;
            (ph == 0 ? s.dzl : s.dzv)[cc] = dz;
            (ph == 0 ? s.drhol : s.drhov)[cc] = rho * (dp - dz / zph - dt);
        }
    }
}

// Index of the liquid (smallest) or vapor (largest) mechanically admissible
// root at composition x, pr76_split.hpp:54-59; -1 if none.
inline int role_branch(const Model& m, Work& wk, double p, double t, const double* x, bool vapor) {
    double amix, bmix, A, B;
    if (!mix(m, wk.tc, x, amix, bmix, wk.sums.data()) || !coefficients(p, t, amix, bmix, A, B)) return -1;
    const RootSet roots = solve_roots(A, B);
    if (roots.status != kRootSuccess) return -1;
    int selected = -1;
    for (int k = 0; k < roots.count; ++k) {
        if (roots.roots[k].slope_sign <= 0) continue;
        selected = k;
        if (!vapor) break;
    }
    return selected;
}

// Newton polish of the two-phase equilibrium equations
//   F_i(ln K) = ln x_i - ln y_i + ln phi_L,i(x) - ln phi_V,i(y) = 0
// with x, y from Rachford-Rice and the liquid/vapor root roles of the split.
// Test instrument only: two converged solutions of the same equilibrium
// (each stopped at the reference's |F| <= 1e-11) polish to the same point, so
// comparing polished states checks "same fixed point" independently of where
// each iteration happened to stop.  dF/dlnK uses the RR linearisation of
// detail/pt_sensitivity_detail.hpp:46-143 and forward-mode ln phi.  Returns
// false if RR or a phase evaluation fails.
inline bool polish(const Model& m, Work& wk, double p, double t, const std::vector<double>& z,
                   std::vector<double>& lnk, double& beta, std::vector<double>& x, std::vector<double>& y,
                   double& res_norm, double& ainv_norm) {
    const int n = m.n;
    res_norm = kNaN;
    ainv_norm = kNaN;
    for (int it = 0; it < 12; ++it) {
        RrResult rr = solve_rr(z, lnk, wk);
        if (rr.status != kRrInterior) return false;
        beta = rr.beta;
        x = rr.x;
        y = rr.y;
        const int bl = role_branch(m, wk, p, t, x.data(), false);
        const int bv = role_branch(m, wk, p, t, y.data(), true);
        if (bl < 0 || bv < 0) return false;
        double h = 0;
        for (int i = 0; i < n; ++i)
            if (z[i] > 0) h += (y[i] - x[i]) * (y[i] - x[i]) / z[i];
        std::vector<double> F(n), A(n * n);
        for (int v = 0; v < n; ++v) {
            double num = 0;
            for (int i = 0; i < n; ++i)
                if (z[i] > 0 && i == v) num += x[i] * y[i] / z[i];
            const double dbeta = num / h;
            std::vector<D1> xl(n), yv(n);
            for (int i = 0; i < n; ++i) {
                if (z[i] == 0) {
                    xl[i] = D1(0.0);
                    yv[i] = D1(0.0);
                    continue;
                }
                const double dlk = i == v ? 1.0 : 0.0;
                const double dlx = -((y[i] - x[i]) / z[i]) * dbeta - beta * (y[i] / z[i]) * dlk;
                xl[i] = D1(x[i], x[i] * dlx);
                yv[i] = D1(y[i], y[i] * (dlx + dlk));
            }
            D1 zl, zv;
            std::vector<D1> pl, pv;
            if (!phase_eval_ad(m, D1(p), D1(t), xl, bl, zl, pl) || !phase_eval_ad(m, D1(p), D1(t), yv, bv, zv, pv))
                return false;
            for (int i = 0; i < n; ++i) {
                if (z[i] == 0) {
                    F[i] = 0;
                    A[i * n + v] = i == v ? 1.0 : 0.0;
                    continue;
                }
                const D1 fi = log(xl[i]) - log(yv[i]) + pl[i] - pv[i];
                F[i] = fi.v;
                A[i * n + v] = fi.d;
            }
        }
        double fn = 0;
        for (double f : F) fn = std::max(fn, std::abs(f));
        res_norm = fn;
        Lu f;
        if (!lu_factor(A, n, f)) return false;
        const double rc = lu_rcond(f);
        ainv_norm = rc > 0 ? 1.0 / (rc * f.norm_inf) : kNaN;
        if (fn <= 4 * kEps) return true;
        std::vector<double> d(n);
        for (int i = 0; i < n; ++i) d[i] = -F[i];
        if (!lu_solve(f, d)) return false;
        for (int i = 0; i < n; ++i) lnk[i] += d[i];
        if (it >= 4) {
            double dn = 0;
            for (double v : d) dn = std::max(dn, std::abs(v));
            if (dn <= 1e-15 * 16) {
                RrResult r2 = solve_rr(z, lnk, wk);
                if (r2.status != kRrInterior) return false;
                beta = r2.beta;
                x = r2.x;
                y = r2.y;
                return true;
            }
        }
    }
    return true;
}

// ---------------------------------------------------------------------------
// Selected-phase property chart, evaluate_pr76_selected_phase_property_chart
// (modules/flow/include/mpmc/flow/pr76_selected_phase_property_closure.hpp:533-822)
// over Pr76SelectedPhasePropertyClosure::evaluate (:338-469), by forward mode
// with one chart column per pass (the reference runs four per pass; the
// first-order arithmetic per column is the same).  The closure's
// transport/caloric provider is the affine model of the C ABI:
//   f = c[0] + c[1] p + c[2] T + sum_i c[7+i] x_i + c[3] rho + c[4] M + c[5] rho_mass + c[6] root_index.
// Statuses: 0 ok, 1 chart input (non-finite entry, fractions, p, T, M),
// 2..5 the EOS classes of phase_eval_status, 6 a property check.
struct ChartSpec {
    int phases = 1;
    int root_index[3] = {0, 0, 0};
    std::vector<double> molar_mass, visc, enth;
};

template <class Num>
inline Num affine_model(const std::vector<double>& c, const Num& p, const Num& t, const std::vector<Num>& x,
                        const Num& rho, const Num& mm, const Num& rhom, int root) {
    Num f = Num(c[0]) + c[1] * p + c[2] * t;
    for (size_t i = 0; i < x.size(); ++i) f = f + c[7 + i] * x[i];
    return f + c[3] * rho + c[4] * mm + c[5] * rhom + c[6] * static_cast<double>(root);
}

inline int property_chart(const Model& m, const ChartSpec& spec, const double* qv, const int* dep, double* values,
                          double* jac) {
    const int n = m.n, P = spec.phases;
    const int q = P * n + 1;
    const int prop = P * (5 + n);
    const int rows = prop + (P - 1) * n;
    for (int k = 0; k < q; ++k)
        if (!std::isfinite(qv[k])) return 1;  // ad/runtime_differentiate.hpp:105-108
    for (int col = 0; col < q; ++col) {
        auto seed = [&](int k) { return D1(qv[k], k == col ? 1.0 : 0.0); };
        const D1 p = seed(0), t = seed(1);
        std::vector<std::vector<D1>> x(P, std::vector<D1>(n));
        std::vector<std::vector<D1>> lnphi(P);
        std::vector<D1> out(rows);
        for (int ph = 0; ph < P; ++ph) {
            // reconstruct_composition, :115-157
            const int d = dep[ph];
            if (d < 0 || d >= n) return 1;
            const int start = 2 + (P - 1) + ph * (n - 1);
            D1 sum(0.0);
            for (int i = 0; i < n; ++i) {
                if (i == d) continue;
                x[ph][i] = seed(start + (i < d ? i : i - 1));
                if (!(x[ph][i].v > 0.0)) return 1;
                sum = sum + x[ph][i];
            }
            x[ph][d] = 1.0 - sum;
            if (!std::isfinite(x[ph][d].v) || !(x[ph][d].v > 0.0)) return 1;
            // closure evaluate, :339-469
            if (!(p.v > 0.0) || !(t.v > 0.0)) return 1;
            D1 mm(0.0);
            for (int i = 0; i < n; ++i) mm = mm + x[ph][i] * spec.molar_mass[i];
            if (!std::isfinite(mm.v) || !(mm.v > 0.0)) return 1;
            // Pr76Mixture fraction checks, pr76_mixture.hpp:146-158 and :221-227
            long double xs = 0, xc = 0;
            for (int i = 0; i < n; ++i) {
                if (x[ph][i].v > 1.0) return 2;
                const long double inc = x[ph][i].v - xc;
                const long double next = xs + inc;
                xc = (next - xs) - inc;
                xs = next;
            }
            if (std::abs(xs - 1.0L) > static_cast<long double>(64.0 * kEps)) return 2;
            D1 z;
            const int ri = spec.root_index[ph];
            const int st = phase_eval_status(m, p, t, x[ph], ri, z, lnphi[ph]);
            if (st != kEvalOk) return st;
            const D1 rho = p / ((z * kR) * t);  // selected_phase_density.hpp:27-34
            const D1 rhom = rho * mm;
            if (!std::isfinite(rho.v) || !(rho.v > 0.0) || !std::isfinite(rhom.v) || !(rhom.v > 0.0)) return 6;
            const D1 mu = affine_model(spec.visc, p, t, x[ph], rho, mm, rhom, ri);
            const D1 h = affine_model(spec.enth, p, t, x[ph], rho, mm, rhom, ri);
            if (!std::isfinite(mu.v) || !(mu.v > 0.0) || !std::isfinite(h.v)) return 6;
            const D1 u = h - p / rhom;
            if (!std::isfinite(u.v)) return 6;
            const int base = ph * (5 + n);
            out[base + 0] = rho;
            out[base + 1] = rhom;
            out[base + 2] = mu;
            out[base + 3] = h;
            out[base + 4] = u;
            for (int i = 0; i < n; ++i) out[base + 5 + i] = lnphi[ph][i];
        }
        // equilibrium rows, :660-681
        for (int ph = 1; ph < P; ++ph)
            for (int i = 0; i < n; ++i)
                out[prop + (ph - 1) * n + i] =
                    (log(x[0][i] / x[ph][i]) + lnphi[0][i]) - lnphi[ph][i] + log(p / p);
        // the runtime Jacobian workspace's output checks, runtime_differentiate.hpp:138-156
        for (int r = 0; r < rows; ++r) {
            if (!finite(out[r])) return 6;
            if (col == 0 && values) values[r] = out[r].v;
            if (jac) jac[static_cast<size_t>(r) * q + col] = out[r].d;
        }
    }
    return 0;
}

}  // namespace oracle

// ===========================================================================
// C interface (ctypes).  Layout: every per-component or per-entry array is
// entry-major with the cell index fastest: a[k * ncell + c].
extern "C" {

struct OracleOutputs {
    int32_t* status;        // [ncell]
    double* beta;           // [ncell]
    double* x;              // [n*ncell]
    double* y;              // [n*ncell]
    double* ln_k;           // [n*ncell]
    double* ln_phi_l;       // [n*ncell]
    double* ln_phi_v;       // [n*ncell]
    double* z_l;            // [ncell]
    double* z_v;            // [ncell]
    int64_t* counters;      // [8*ncell]: init evals, split evals, final evals, split iters,
                            //  rr iters, root bisection steps, attempts, trial iterations
    int32_t* sens_status;   // [ncell]
    double* dlnk;           // [n*(n+1)*ncell]
    double* dbeta;          // [(n+1)*ncell]
    double* dx;             // [n*(n+1)*ncell]
    double* dy;             // [n*(n+1)*ncell]
    double* dzl;            // [(n+1)*ncell]
    double* dzv;            // [(n+1)*ncell]
    double* drhol;          // [(n+1)*ncell]
    double* drhov;          // [(n+1)*ncell]
    double* jl;             // [(n+1)*(n+2)*ncell]
    double* jv;             // [(n+1)*(n+2)*ncell]
    double* rcond;          // [ncell] reciprocal condition estimate of dF/dln K (NaN if not factored)
};

static void oracle_cell(const oracle::Model& m, int64_t ncell, int64_t c, const double* p, const double* t,
                        const double* z, int want_sens, const OracleOutputs* o) {
    using namespace oracle;
    const int n = m.n;
    const double nan = kNaN;
    Work wk;
    wk.init(n);
    std::vector<double> feed(n);
    for (int i = 0; i < n; ++i) feed[i] = z[i * ncell + c];
    FlashResult fr;
    if (!std::isfinite(t[c]) || !(t[c] > 0) || !make_temp_cache(m, t[c], wk.tc)) {
        fr.status = kInvalid;
    } else {
        fr = solve_vle(m, wk, p[c], t[c], feed);
    }
    auto put = [&](double* arr, int k, double v) {
        if (arr) arr[k * ncell + c] = v;
    };
    if (o->status) o->status[c] = fr.status;
    const bool pair = fr.has_candidate && fr.status != kSinglePhase && fr.status != kInvalid;
    put(o->beta, 0, pair ? fr.candidate.rr.beta : nan);
    for (int i = 0; i < n; ++i) {
        if (pair) {
            put(o->x, i, fr.candidate.rr.x[i]);
            put(o->y, i, fr.candidate.rr.y[i]);
            put(o->ln_k, i, fr.candidate.log_k[i]);
            put(o->ln_phi_l, i, fr.candidate.liquid.ln_phi[i]);
            put(o->ln_phi_v, i, fr.candidate.vapor.ln_phi[i]);
        } else if (fr.status == kSinglePhase) {
            put(o->x, i, fr.initial.feed[i]);
            put(o->y, i, nan);
            put(o->ln_k, i, nan);
            put(o->ln_phi_l, i, fr.initial.reference.ln_phi[i]);
            put(o->ln_phi_v, i, nan);
        } else {
            put(o->x, i, nan);
            put(o->y, i, nan);
            put(o->ln_k, i, nan);
            put(o->ln_phi_l, i, nan);
            put(o->ln_phi_v, i, nan);
        }
    }
    put(o->z_l, 0, pair ? fr.candidate.liquid.z : (fr.status == kSinglePhase ? fr.initial.reference.z : nan));
    put(o->z_v, 0, pair ? fr.candidate.vapor.z : nan);
    if (o->counters) {
        const int64_t cnt[8] = {fr.initial.evaluations, fr.split_evaluations, fr.final_review.evaluations,
                                fr.split_iterations, wk.rr_iterations, wk.root_bisections, fr.attempts,
                                fr.initial.trial_iterations + fr.final_review.trial_iterations};
        for (int k = 0; k < 8; ++k) o->counters[k * ncell + c] = cnt[k];
    }
    if (!want_sens) return;
    Sensitivity s;
    if (fr.status == kTwoPhase) differentiate(m, fr, p[c], t[c], s);
    else s.status = 1;
    if (o->sens_status) o->sens_status[c] = s.status;
    if (o->rcond) o->rcond[c] = s.rcond > 0.0 ? s.rcond : nan;
    const int q = n + 1;
    const bool ok = s.status == 0;
    for (int k = 0; k < n * q; ++k) {
        put(o->dlnk, k, ok ? s.dlnk[k] : nan);
        put(o->dx, k, ok ? s.dx[k] : nan);
        put(o->dy, k, ok ? s.dy[k] : nan);
    }
    for (int k = 0; k < q; ++k) {
        put(o->dbeta, k, ok ? s.dbeta[k] : nan);
        put(o->dzl, k, ok ? s.dzl[k] : nan);
        put(o->dzv, k, ok ? s.dzv[k] : nan);
        put(o->drhol, k, ok ? s.drhol[k] : nan);
        put(o->drhov, k, ok ? s.drhov[k] : nan);
    }
    for (int k = 0; k < (n + 1) * (n + 2); ++k) {
        put(o->jl, k, ok ? s.jl[k] : nan);
        put(o->jv, k, ok ? s.jv[k] : nan);
    }
}

// Flash `ncell` cells of one mixture with `threads` host threads (static
// partition, one scratch workspace per thread).  Returns 0, or -1 on invalid
// arguments.
int oracle_flash_batch(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                       int64_t ncell, const double* p, const double* t, const double* z, int threads,
                       int want_sensitivity, const OracleOutputs* out) {
    if (n < 1 || n > 256 || ncell < 0 || !tc || !pc || !omega || !kij || !p || !t || !z || !out) return -1;
    const oracle::Model m = oracle::make_model(n, tc, pc, omega, kij);
    if (threads < 1) threads = 1;
    if (threads > ncell) threads = static_cast<int>(std::max<int64_t>(ncell, 1));
    auto run = [&](int64_t lo, int64_t hi) {
        for (int64_t c = lo; c < hi; ++c) oracle_cell(m, ncell, c, p, t, z, want_sensitivity, out);
    };
    if (threads == 1) {
        run(0, ncell);
        return 0;
    }
    std::vector<std::thread> pool;
    const int64_t chunk = (ncell + threads - 1) / threads;
    for (int k = 0; k < threads; ++k) {
        const int64_t lo = k * chunk, hi = std::min<int64_t>(ncell, lo + chunk);
        if (lo < hi) pool.emplace_back(run, lo, hi);
    }
    for (auto& th : pool) th.join();
    return 0;
}

// Max-3-phase orchestration per cell (the reference's PR76 backend default:
// solve_pr76_pt_max3 with no start hints).  Same layout and codes as the
// harness's ref_max3_batch: max3_status 0 single, 1 two, 2 three, 3 boundary
// unresolved, 4 higher phase count or wrong candidate, 5 indeterminate, -1
// invalid; published 0 single, 1 two, 2 phase set unstable, 3 indeterminate,
// 4 three, -1 invalid (pt_phase_set.hpp:91-150).
struct Max3Outputs {
    int32_t* max3_status;
    int32_t* published;
    double* beta3;   // [3]
    double* x3;      // [3 * n], phase-major
    double* lnphi3;  // [3 * n]
    double* z3;      // [3]
    double* beta;    // published two-phase pair
    double* x;       // [n]
    double* y;       // [n]
    int32_t* attempts;
};

// Selected-phase property chart of `ncell` cells (oracle::property_chart).
// q [(P n + 1) * ncell] and dep [P * ncell] (null = the last component) in
// the cell-fastest layout; writes status [ncell], values [rows * ncell] and
// jac [rows * q * ncell] (element (r, col) of cell c at (r * q + col) * ncell
// + c), NaN for a failed cell.
int oracle_property_chart_batch(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                                int phases, const int* root_index, const double* molar_mass, const double* visc,
                                const double* enth, int64_t ncell, const double* q, const int* dep, int threads,
                                int* status, double* values, double* jac) {
    if (phases < 1 || phases > 3 || n < 2) return 1;
    const oracle::Model m = oracle::make_model(n, tc, pc, omega, kij);
    oracle::ChartSpec spec;
    spec.phases = phases;
    for (int k = 0; k < phases; ++k) spec.root_index[k] = root_index[k];
    spec.molar_mass.assign(molar_mass, molar_mass + n);
    spec.visc.assign(visc, visc + 7 + n);
    spec.enth.assign(enth, enth + 7 + n);
    const int cols = phases * n + 1;
    const int rows = phases * (5 + n) + (phases - 1) * n;
    auto run = [&](int64_t lo, int64_t hi) {
        std::vector<double> qc(cols), v(rows), j(static_cast<size_t>(rows) * cols);
        int dc[3];
        for (int64_t c = lo; c < hi; ++c) {
            for (int k = 0; k < cols; ++k) qc[k] = q[k * ncell + c];
            for (int k = 0; k < phases; ++k) dc[k] = dep ? dep[k * ncell + c] : n - 1;
            const int st = oracle::property_chart(m, spec, qc.data(), dc, v.data(), j.data());
            if (status) status[c] = st;
            for (int r = 0; r < rows; ++r) {
                if (values) values[r * ncell + c] = st == 0 ? v[r] : oracle::kNaN;
                if (jac)
                    for (int k = 0; k < cols; ++k)
                        jac[(static_cast<int64_t>(r) * cols + k) * ncell + c] =
                            st == 0 ? j[static_cast<size_t>(r) * cols + k] : oracle::kNaN;
            }
        }
    };
    if (threads <= 1 || ncell < 64) {
        run(0, ncell);
        return 0;
    }
    std::vector<std::thread> pool;
    const int64_t per = (ncell + threads - 1) / threads;
    for (int w = 0; w < threads; ++w) {
        const int64_t lo = w * per, hi = std::min<int64_t>(ncell, lo + per);
        if (lo < hi) pool.emplace_back(run, lo, hi);
    }
    for (auto& th : pool) th.join();
    return 0;
}

// Caller starts and options of solve_pr76_pt_max3 (pr76_three_phase.hpp:328-341;
// the split options of pt_split.hpp:45-50).  Compositions are cell-fastest:
// composition k of cell c, component i at (k * n + i) * ncell + c.
struct StartHints {
    const int32_t* initial_count;      // [ncell], 0..3 initial_starts (NULL: none)
    const double* initial_x;           // [3 n ncell]
    const int32_t* final_count;        // [ncell], 0..3 final_starts (NULL: none)
    const double* final_x;             // [3 n ncell]
    const int32_t* three_phase;        // [ncell], nonzero: one three-phase start (NULL: none)
    const double* three_x;             // [3 n ncell]
    const double* fraction;            // [2 ncell]: phase_fraction_seed of phases 1 and 2
    int32_t initial_automatic_starts;  // options.two_phase.initial_stability.automatic_starts
    int32_t max_split_attempts;        // options.two_phase.max_split_attempts
};

static void hint_set(const int32_t* count, const double* x, int n, int64_t ncell, int64_t c,
                     std::vector<std::vector<double>>& out) {
    out.clear();
    if (!count || !x) return;
    const int k = std::min(3, std::max(0, static_cast<int>(count[c])));
    for (int q = 0; q < k; ++q) {
        std::vector<double> w(n);
        for (int i = 0; i < n; ++i) w[i] = x[(static_cast<int64_t>(q) * n + i) * ncell + c];
        out.push_back(std::move(w));
    }
}

static int max3_batch(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                      int64_t ncell, const double* p, const double* t, const double* z, int threads,
                      const Max3Outputs* o, const StartHints* h) {
    if (n < 1 || n > 256 || ncell < 0 || !tc || !pc || !omega || !kij || !p || !t || !z || !o) return -1;
    const oracle::Model m = oracle::make_model(n, tc, pc, omega, kij);
    auto run = [&](int64_t lo, int64_t hi) {
        using namespace oracle;
        Work wk;
        wk.init(n);
        std::vector<double> feed(n);
        std::vector<std::vector<double>> init, fin;
        std::vector<ThreeStart> three;
        VleOptions vo;
        if (h) {
            vo.initial_automatic_starts = h->initial_automatic_starts != 0;
            vo.max_split_attempts = h->max_split_attempts;
        }
        for (int64_t c = lo; c < hi; ++c) {
            three.clear();
            if (h) {
                hint_set(h->initial_count, h->initial_x, n, ncell, c, init);
                hint_set(h->final_count, h->final_x, n, ncell, c, fin);
                if (h->three_phase && h->three_x && h->fraction && h->three_phase[c]) {
                    ThreeStart st;
                    for (int q = 0; q < 3; ++q) {
                        st.x[q].resize(n);
                        for (int i = 0; i < n; ++i) st.x[q][i] = h->three_x[(static_cast<int64_t>(q) * n + i) * ncell + c];
                    }
                    st.fraction[0] = h->fraction[c];
                    st.fraction[1] = h->fraction[ncell + c];
                    three.push_back(std::move(st));
                }
            }
            auto put = [&](double* arr, int k, double v) {
                if (arr) arr[k * ncell + c] = v;
            };
            for (int k = 0; k < 3; ++k) {
                put(o->beta3, k, kNaN);
                put(o->z3, k, kNaN);
                for (int i = 0; i < n; ++i) {
                    put(o->x3, k * n + i, kNaN);
                    put(o->lnphi3, k * n + i, kNaN);
                }
            }
            put(o->beta, 0, kNaN);
            for (int i = 0; i < n; ++i) {
                put(o->x, i, kNaN);
                put(o->y, i, kNaN);
            }
            for (int i = 0; i < n; ++i) feed[i] = z[i * ncell + c];
            Max3Result r;
            if (!std::isfinite(t[c]) || !(t[c] > 0) || !make_temp_cache(m, t[c], wk.tc))
                r.status = -1;
            else
                r = solve_max3(m, wk, p[c], t[c], feed, init, fin, three, vo);
            if (o->max3_status) o->max3_status[c] = r.status;
            if (o->attempts) o->attempts[c] = r.attempts;
            int pub = -1;
            const SplitState* pair = nullptr;
            switch (r.status) {
            case kM3Single: pub = 0; break;
            case kM3Two:
                pub = 1;
                pair = r.has_neighbor ? &r.neighbor.candidate : &r.base.candidate;
                break;
            case kM3Three: pub = 4; break;
            case kM3Higher:
                pub = 2;
                pair = &r.base.candidate;
                break;
            case kM3Boundary:
            case kM3Indeterminate: pub = 3; break;
            default: pub = -1; break;
            }
            if (o->published) o->published[c] = pub;
            if (pair) {
                put(o->beta, 0, pair->rr.beta);
                for (int i = 0; i < n; ++i) {
                    put(o->x, i, pair->rr.x[i]);
                    put(o->y, i, pair->rr.y[i]);
                }
            }
            if (r.has_three) {
                for (int k = 0; k < 3; ++k) {
                    put(o->beta3, k, r.three.fraction[k]);
                    put(o->z3, k, r.three.zf[k]);
                    for (int i = 0; i < n; ++i) {
                        put(o->x3, k * n + i, r.three.x[k][i]);
                        put(o->lnphi3, k * n + i, r.three.ln_phi[k][i]);
                    }
                }
            }
        }
    };
    if (threads < 1) threads = 1;
    if (threads > ncell) threads = static_cast<int>(std::max<int64_t>(ncell, 1));
    std::vector<std::thread> pool;
    const int64_t chunk = (ncell + threads - 1) / threads;
    for (int k = 0; k < threads; ++k) {
        const int64_t lo = k * chunk, hi = std::min<int64_t>(ncell, lo + chunk);
        if (lo < hi) pool.emplace_back(run, lo, hi);
    }
    for (auto& th : pool) th.join();
    return 0;
}

int oracle_max3_batch(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                      int64_t ncell, const double* p, const double* t, const double* z, int threads,
                      const Max3Outputs* o) {
    return max3_batch(n, tc, pc, omega, kij, ncell, p, t, z, threads, o, nullptr);
}

// oracle_max3_batch with caller starts and options (StartHints).
int oracle_max3_hinted_batch(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                             int64_t ncell, const double* p, const double* t, const double* z,
                             const StartHints* hints, int threads, const Max3Outputs* o) {
    if (!hints) return -1;
    return max3_batch(n, tc, pc, omega, kij, ncell, p, t, z, threads, o, hints);
}

// Ordered-path continuation of npath feeds z [n * npath], each along its own
// npoint states (p, t [npath * npoint], path-major): per point the max3 status
// (codes of oracle_max3_batch; -1 on every point of an invalid path).
int oracle_continuation_batch(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                              int64_t npath, int64_t npoint, const double* p, const double* t, const double* z,
                              int threads, int32_t* max3_status) {
    if (n < 1 || n > 256 || npath < 0 || npoint < 1 || !p || !t || !z || !max3_status) return -1;
    const oracle::Model m = oracle::make_model(n, tc, pc, omega, kij);
    auto run = [&](int64_t lo, int64_t hi) {
        oracle::Work wk;
        wk.init(n);
        std::vector<double> feed(n);
        std::vector<int> st(static_cast<size_t>(npoint));
        for (int64_t path = lo; path < hi; ++path) {
            for (int i = 0; i < n; ++i) feed[i] = z[i * npath + path];
            const bool ok = oracle::solve_continuation(m, wk, p + path * npoint, t + path * npoint,
                                                       static_cast<int>(npoint), feed, st.data());
            for (int64_t k = 0; k < npoint; ++k) max3_status[path * npoint + k] = ok ? st[k] : -1;
        }
    };
    if (threads < 1) threads = 1;
    std::vector<std::thread> pool;
    const int64_t chunk = (npath + threads - 1) / threads;
    for (int k = 0; k < threads; ++k) {
        const int64_t lo = k * chunk, hi = std::min<int64_t>(npath, lo + chunk);
        if (lo < hi) pool.emplace_back(run, lo, hi);
    }
    for (auto& th : pool) th.join();
    return 0;
}

// One phase property evaluation at a fixed composition (stability provider:
// minimum-Gibbs admissible branch).  Returns the issue code (0 = ok).
int oracle_stability_phase(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                           double p, double t, const double* x, double* ln_phi, double* z_out, int* branch,
                           int* smooth) {
    const oracle::Model m = oracle::make_model(n, tc, pc, omega, kij);
    oracle::Work wk;
    wk.init(n);
    if (!oracle::make_temp_cache(m, t, wk.tc)) return oracle::kRootRange;
    oracle::StabilityPhase ph;
    const oracle::Issue is = oracle::stability_provider(m, wk, p, t, x, ph);
    if (is != oracle::kOk) return is;
    for (int i = 0; i < n; ++i) ln_phi[i] = ph.ln_phi[i];
    *z_out = ph.z;
    *branch = ph.branch;
    *smooth = ph.smooth ? 1 : 0;
    return 0;
}

// Newton-polish two-phase states (see oracle::polish) of `ncell` cells given
// their ln K (layout [i*ncell + c]); cells with ok[c] == 0 are skipped.
// Writes polished ln K, beta, x, y, the final max |F| and ||(dF/dlnK)^-1||_inf
// (NaN where the polish failed).
int oracle_polish_batch(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                        int64_t ncell, const double* p, const double* t, const double* z, const int32_t* ok,
                        const double* lnk_in, int threads, double* lnk_out, double* beta_out, double* x_out,
                        double* y_out, double* res_out, double* ainv_out) {
    using namespace oracle;
    const Model m = make_model(n, tc, pc, omega, kij);
    auto run = [&](int64_t lo, int64_t hi) {
        Work wk;
        wk.init(n);
        for (int64_t c = lo; c < hi; ++c) {
            for (int i = 0; i < n; ++i) lnk_out[i * ncell + c] = x_out[i * ncell + c] = y_out[i * ncell + c] = kNaN;
            beta_out[c] = res_out[c] = ainv_out[c] = kNaN;
            if (!ok[c]) continue;
            std::vector<double> zz(n), lk(n), x, y;
            double sum = 0, cs = 0;
            for (int i = 0; i < n; ++i) kahan_add(z[i * ncell + c], sum, cs);
            for (int i = 0; i < n; ++i) {
                zz[i] = z[i * ncell + c] / sum;
                lk[i] = zz[i] > 0 ? lnk_in[i * ncell + c] : 0.0;
            }
            if (!make_temp_cache(m, t[c], wk.tc)) continue;
            double beta, res, ainv;
            if (!polish(m, wk, p[c], t[c], zz, lk, beta, x, y, res, ainv)) continue;
            for (int i = 0; i < n; ++i) {
                lnk_out[i * ncell + c] = lk[i];
                x_out[i * ncell + c] = x[i];
                y_out[i * ncell + c] = y[i];
            }
            beta_out[c] = beta;
            res_out[c] = res;
            ainv_out[c] = ainv;
        }
    };
    if (threads < 1) threads = 1;
    std::vector<std::thread> pool;
    const int64_t chunk = (ncell + threads - 1) / threads;
    for (int k = 0; k < threads; ++k) {
        const int64_t lo = k * chunk, hi = std::min<int64_t>(ncell, lo + chunk);
        if (lo < hi) pool.emplace_back(run, lo, hi);
    }
    for (auto& th : pool) th.join();
    return 0;
}

// Sensitivities (differentiate_pr76_pt_vle + closure + per-phase Jacobians) at
// GIVEN accepted two-phase states (x, y, ln K, beta per cell), so that a
// device implementation can be compared at identical base points.  Only
// cells with ok[c] != 0 are processed; `out` uses the OracleOutputs layout
// (sensitivity fields only).
void oracle_set_manifold_identity(int on) { oracle::g_manifold_identity.store(on ? 1 : 0); }

int oracle_sensitivity_at(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                          int64_t ncell, const double* p, const double* t, const double* z, const int32_t* ok,
                          const double* x, const double* y, const double* lnk, const double* beta, int threads,
                          const OracleOutputs* o) {
    using namespace oracle;
    const Model m = make_model(n, tc, pc, omega, kij);
    auto run = [&](int64_t lo, int64_t hi) {
        Work wk;
        wk.init(n);
        for (int64_t c = lo; c < hi; ++c) {
            auto put = [&](double* arr, int k, double v) {
                if (arr) arr[k * ncell + c] = v;
            };
            Sensitivity s;
            s.status = 1;
            if (ok[c] && make_temp_cache(m, t[c], wk.tc)) {
                FlashResult fr;
                fr.status = kTwoPhase;
                fr.has_candidate = true;
                std::vector<double> feed(n);
                double sum = 0, cs = 0;
                for (int i = 0; i < n; ++i) kahan_add(z[i * ncell + c], sum, cs);
                for (int i = 0; i < n; ++i) feed[i] = z[i * ncell + c] / sum;
                fr.initial.feed = feed;
                SplitState& st = fr.candidate;
                st.rr.x.resize(n);
                st.rr.y.resize(n);
                st.log_k.resize(n);
                for (int i = 0; i < n; ++i) {
                    st.rr.x[i] = x[i * ncell + c];
                    st.rr.y[i] = y[i * ncell + c];
                    st.log_k[i] = lnk[i * ncell + c];
                }
                st.rr.beta = beta[c];
                Issue a = role_provider(m, wk, p[c], t[c], st.rr.x.data(), false, st.liquid);
                Issue b = role_provider(m, wk, p[c], t[c], st.rr.y.data(), true, st.vapor);
                if (a == kOk && b == kOk) {
                    st.fug_norm = 0;
                    for (int i = 0; i < n; ++i)
                        st.fug_norm = std::max(st.fug_norm, std::abs(std::log(st.rr.x[i]) - std::log(st.rr.y[i]) +
                                                                     st.liquid.ln_phi[i] - st.vapor.ln_phi[i]));
                    differentiate(m, fr, p[c], t[c], s);
                } else {
                    s.status = 4;
                }
            }
            const double nan = kNaN;
            if (o->sens_status) o->sens_status[c] = s.status;
            if (o->rcond) o->rcond[c] = s.rcond > 0.0 ? s.rcond : nan;
            const int q = n + 1;
            const bool good = s.status == 0;
            for (int k = 0; k < n * q; ++k) {
                put(o->dlnk, k, good ? s.dlnk[k] : nan);
                put(o->dx, k, good ? s.dx[k] : nan);
                put(o->dy, k, good ? s.dy[k] : nan);
            }
            for (int k = 0; k < q; ++k) {
                put(o->dbeta, k, good ? s.dbeta[k] : nan);
                put(o->dzl, k, good ? s.dzl[k] : nan);
                put(o->dzv, k, good ? s.dzv[k] : nan);
                put(o->drhol, k, good ? s.drhol[k] : nan);
                put(o->drhov, k, good ? s.drhov[k] : nan);
            }
            for (int k = 0; k < (n + 1) * (n + 2); ++k) {
                put(o->jl, k, good ? s.jl[k] : nan);
                put(o->jv, k, good ? s.jv[k] : nan);
            }
        }
    };
    if (threads < 1) threads = 1;
    std::vector<std::thread> pool;
    const int64_t chunk = (ncell + threads - 1) / threads;
    for (int k = 0; k < threads; ++k) {
        const int64_t lo = k * chunk, hi = std::min<int64_t>(ncell, lo + chunk);
        if (lo < hi) pool.emplace_back(run, lo, hi);
    }
    for (auto& th : pool) th.join();
    return 0;
}

// Rachford-Rice at fixed ln K.  Returns the RR status code.
int oracle_rachford_rice(int n, const double* z, const double* ln_k, double* beta, double* x, double* y) {
    std::vector<double> zz(z, z + n), lk(ln_k, ln_k + n);
    oracle::Work wk;
    const oracle::RrResult r = oracle::solve_rr(zz, lk, wk);
    *beta = r.beta;
    if (r.status == oracle::kRrInterior)
        for (int i = 0; i < n; ++i) {
            x[i] = r.x[i];
            y[i] = r.y[i];
        }
    return r.status;
}

}  // extern "C"
