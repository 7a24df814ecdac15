// Reference-side binding of the hint-seeded ordered-path continuation on the
// GPU: the reference's solve_pr76_pt_continuation
// (modules/flash/include/mpmc/flash/pr76_pt_continuation.hpp:194-308, default
// options) for many paths at once, one device call per path point through
// mpmc_gpu_flash_solve_hinted.
//
// Every path point is a max-3-phase solve seeded as the reference seeds it
// (:216-300): the previous accepted point's phase compositions as extra
// starts of the feed stability test and the final review, and its
// three-phase set as a three-phase start; the hints reset after an
// unresolved point.  Results keep the reference's point fields that the C
// ABI returns -- state, max3 status, accepted phase count, the incoming hint
// kind and the carried starts -- and its transition brackets and diagnostics
// (:266-290, :304-306).  Not carried: the per-point solve internals
// (Pr76PtMax3Result attempts and trials) and whether a carried three-phase
// start was the one consumed.
//
// Paths are solved in lockstep, so all paths of one call have the same
// number of points.  Errors follow the reference: an empty path or an
// invalid feed throws std::invalid_argument, a non-positive or non-finite
// state std::domain_error, more than max_points points std::length_error.
#pragma once

#include <mpmc/flash/pr76_pt_continuation.hpp>

#include <cmath>
#include <cstdint>
#include <limits>
#include <optional>
#include <span>
#include <stdexcept>
#include <string>
#include <vector>

#include "gpu_pr76_pt_flash_backend.hpp"
#include "mpmc_gb300_flash.h"

namespace mpmc::flash {

struct GpuPr76PtContinuationPoint {
    Pr76PtPathState state;
    Pr76PtMax3Status status{Pr76PtMax3Status::indeterminate};
    std::optional<std::size_t> accepted_phase_count;
    Pr76PtContinuationHintKind incoming_hint{Pr76PtContinuationHintKind::none};
    std::size_t carried_stability_start_count{};
    bool carried_three_phase_start{false};
};

struct GpuPr76PtContinuationResult {
    std::vector<double> feed;
    std::vector<GpuPr76PtContinuationPoint> points;
    std::vector<Pr76PtTransitionBracket> transition_brackets;
    bool all_points_accepted{true};
    std::string diagnostic;
};

// One handle (mpmc_gpu_flash_create) for the mixture; paths[k] with feeds[k]
// (component order of the handle's mixture).
[[nodiscard]] inline std::vector<GpuPr76PtContinuationResult> solve_gpu_pr76_pt_continuation(
    mpmc_gpu_flash* handle, std::span<const std::vector<Pr76PtPathState>> paths,
    std::span<const std::vector<double>> feeds, std::size_t max_points = 4096) {
    if (handle == nullptr) throw std::invalid_argument("GPU PR76 continuation: null handle");
    const std::size_t npath = paths.size();
    if (feeds.size() != npath) throw std::invalid_argument("GPU PR76 continuation: one feed per path");
    const std::size_t n = static_cast<std::size_t>(mpmc_gpu_flash_components(handle));
    const std::size_t npoint = npath ? paths[0].size() : 0U;
    std::vector<GpuPr76PtContinuationResult> results(npath);
    for (std::size_t k = 0; k < npath; ++k) {
        const auto& path = paths[k];
        if (path.empty()) throw std::invalid_argument("PR76 PT continuation: ordered path is empty");
        if (path.size() > max_points || max_points == 0U)
            throw std::length_error("PR76 PT continuation: point quota exceeded");
        if (path.size() != npoint)
            throw std::invalid_argument("GPU PR76 continuation: paths of one call have the same length");
        if (feeds[k].size() != n)
            throw std::invalid_argument("PR76 PT continuation: feed does not match ordered parameter snapshot");
        for (const auto& st : path)
            if (!std::isfinite(st.pressure_pa) || !(st.pressure_pa > 0.0) || !std::isfinite(st.temperature_k) ||
                !(st.temperature_k > 0.0))
                throw std::domain_error("PR76 PT continuation: every path state requires finite p>0 Pa and T>0 K");
        // the feed normalised once with the compensated sum (:206-207)
        double sum = 0.0, carry = 0.0;
        for (double v : feeds[k]) {
            if (!std::isfinite(v) || v < 0.0 || v > 1.0)
                throw std::invalid_argument("PR76 PT continuation: feed entries must be finite and in [0,1]");
            const double inc = v - carry;
            const double next = sum + inc;
            carry = (next - sum) - inc;
            sum = next;
        }
        if (std::abs(sum - 1.0) > 64.0 * std::numeric_limits<double>::epsilon())
            throw std::invalid_argument("PR76 PT continuation: feed is not normalized");
        results[k].feed.resize(n);
        for (std::size_t i = 0; i < n; ++i) results[k].feed[i] = feeds[k][i] / sum;
    }
    const std::size_t cells = npath;
    std::vector<double> p(cells), t(cells), z(n * cells);
    for (std::size_t c = 0; c < cells; ++c)
        for (std::size_t i = 0; i < n; ++i) z[i * cells + c] = results[c].feed[i];
    std::vector<int32_t> count(cells, 0), three(cells, 0);
    std::vector<double> hx(3 * n * cells, 0.0), frac(2 * cells, 0.0);
    std::vector<int32_t> status(cells), max3(cells);
    std::vector<double> x(n * cells), y(n * cells), lnk(n * cells), f3(3 * cells), x3(3 * n * cells),
        phi3(3 * n * cells), z3(3 * cells);
    std::vector<std::optional<std::size_t>> previous(cells);
    for (std::size_t k = 0; k < npoint; ++k) {
        for (std::size_t c = 0; c < cells; ++c) {
            p[c] = paths[c][k].pressure_pa;
            t[c] = paths[c][k].temperature_k;
        }
        mpmc_flash_outputs out{};
        out.status = status.data();
        out.liquid = x.data();
        out.vapor = y.data();
        out.ln_k = lnk.data();
        mpmc_three_phase_outputs out3{max3.data(), f3.data(), x3.data(), phi3.data(), z3.data()};
        const mpmc_start_hints hints{count.data(), hx.data(), three.data(), frac.data()};
        const int rc = cells ? mpmc_gpu_flash_solve_hinted(handle, static_cast<int64_t>(cells), p.data(), t.data(),
                                                           z.data(), &hints, &out, &out3)
                             : MPMC_OK;
        if (rc != MPMC_OK) throw std::runtime_error(mpmc_gpu_flash_last_error());
        for (std::size_t c = 0; c < cells; ++c) {
            GpuPr76PtContinuationResult& res = results[c];
            GpuPr76PtContinuationPoint point;
            point.state = paths[c][k];
            if (max3[c] < 0) throw std::invalid_argument("PR76 PT continuation: a path point rejected its request");
            point.status = static_cast<Pr76PtMax3Status>(max3[c]);
            if (max3[c] == MPMC_MAX3_SINGLE_PHASE) point.accepted_phase_count = 1U;
            if (max3[c] == MPMC_MAX3_TWO_PHASE) point.accepted_phase_count = 2U;
            if (max3[c] == MPMC_MAX3_THREE_PHASE) point.accepted_phase_count = 3U;
            if (previous[c]) {
                point.incoming_hint = *previous[c] == 1U   ? Pr76PtContinuationHintKind::one_phase
                                      : *previous[c] == 2U ? Pr76PtContinuationHintKind::two_phase
                                                           : Pr76PtContinuationHintKind::three_phase;
                point.carried_stability_start_count = static_cast<std::size_t>(count[c]);
                point.carried_three_phase_start = three[c] != 0;
            }
            if (!point.accepted_phase_count) res.all_points_accepted = false;
            // transition bracket against the previous point (:266-290)
            if (k > 0 && res.points.back().accepted_phase_count && point.accepted_phase_count &&
                *res.points.back().accepted_phase_count != *point.accepted_phase_count) {
                Pr76PtTransitionBracket b;
                b.left_index = k - 1;
                b.right_index = k;
                b.left_phase_count = *res.points.back().accepted_phase_count;
                b.right_phase_count = *point.accepted_phase_count;
                b.left = res.points.back().state;
                b.right = point.state;
                const std::size_t d = b.left_phase_count > b.right_phase_count
                                          ? b.left_phase_count - b.right_phase_count
                                          : b.right_phase_count - b.left_phase_count;
                b.adjacent_phase_count_step = d == 1U;
                b.exact_boundary_resolved = false;
                b.diagnostic = b.adjacent_phase_count_step
                                   ? "PR76 PT continuation: adjacent accepted path points bracket a phase-count "
                                     "change; the exact boundary is not resolved by the discrete scan"
                                   : "PR76 PT continuation: accepted path points skip one or more phase counts; "
                                     "path refinement is required before interpreting the transition sequence";
                res.transition_brackets.push_back(std::move(b));
            }
            // the next point's hints: the accepted phases; none after an unresolved point
            count[c] = 0;
            three[c] = 0;
            previous[c] = point.accepted_phase_count;
            auto put = [&](int slot, const std::vector<double>& src, std::size_t row0) {
                for (std::size_t i = 0; i < n; ++i) hx[(slot * n + i) * cells + c] = src[(row0 + i) * cells + c];
            };
            if (max3[c] == MPMC_MAX3_SINGLE_PHASE) {
                put(0, x, 0);
                count[c] = 1;
            } else if (max3[c] == MPMC_MAX3_TWO_PHASE && std::isfinite(x[c]) && std::isfinite(y[c])) {
                put(0, x, 0);
                put(1, y, 0);
                bool same = true;
                for (std::size_t i = 0; i < n; ++i) same = same && x[i * cells + c] == y[i * cells + c];
                count[c] = same ? 1 : 2;  // unique starts only (:103-118)
            } else if (max3[c] == MPMC_MAX3_THREE_PHASE) {
                for (int q = 0; q < 3; ++q) put(q, x3, static_cast<std::size_t>(q) * n);
                count[c] = 3;
                three[c] = 1;
                frac[c] = f3[1 * cells + c];
                frac[cells + c] = f3[2 * cells + c];
            }
            res.points.push_back(point);
        }
    }
    for (auto& res : results)
        res.diagnostic = res.all_points_accepted
                             ? "PR76 PT continuation: every ordered path point completed a fresh accepted max3 "
                               "solve; transition brackets are discrete only"
                             : "PR76 PT continuation: one or more path points remained unresolved; continuation "
                               "hints were reset after each unresolved point";
    return results;
}

}  // namespace mpmc::flash
