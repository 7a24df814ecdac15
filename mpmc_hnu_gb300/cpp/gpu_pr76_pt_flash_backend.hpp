// Reference-side binding of the GB300 flash: a PtFlashBackend whose solve
// calls the C ABI of include/mpmc_gb300_flash.h.
//
// A maintainer adds this header to a build of MPMC_HNU's flash module and
// constructs it where a Pr76PtFlashBackend is constructed today
// (modules/flash/include/mpmc/flash/pr76_pt_flash_backend.hpp:177-237; callers
// pt_service.hpp:335, pr76_executable_model.hpp:219).  It keeps the interface
// of modules/flash/include/mpmc/flash/pt_flash_backend.hpp:187-195 unchanged
// and adds solve_batch() for the cell loops that own many requests.
//
// Contract: the PR76 max3 backend's (pr76_pt_flash_backend.hpp:190-237) with
// its default options, under a distinct backend id.  Every request runs the
// two-phase flash and, where the pair fails its final review, the
// max-3-phase continuation (mpmc_gpu_flash_solve_max3), so phase counts
// {1, 2, 3} are published as project_max3_solution does
// (pt_phase_set.hpp:91-150).  The transition report carries the evidence
// project_pr76_pt_max3_transition_report (pr76_pt_flash_backend.hpp:94-175)
// gives every accepted, phase-set-unstable and boundary-unresolved result,
// which is what the flow module's transition candidates need
// (phase_set_transition_flash_adapter.hpp:130-248); an indeterminate result
// from an unresolved two-phase or three-phase search carries none, since the
// C ABI does not return the attempts behind it.  Caller starts are carried in
// the form the C ABI takes (GpuPr76BackendStarts, below): the continuation's
// form (the same compositions as initial, final and three-phase starts) or
// the general one, which gpu_starts_from() fills from the reference's own
// Pr76PtFlashBackendOptions (initial_starts, final_starts, one three-phase
// start, split.initial_stability.automatic_starts, split.max_split_attempts;
// every other field at its default, as the device code implements it); not
// carried: the phase metadata.
//
// Errors follow the reference's classes: an invalid request (feed size,
// non-finite or non-positive p and T, a feed outside the simplex) throws
// std::invalid_argument; invalid mixture data at construction throws
// std::domain_error; a device failure throws std::runtime_error.  Numerical
// failure is the indeterminate status, never an exception.
//
// Not reentrant, like the reference backend (pr76_split.hpp:16-18): one
// instance per simultaneous caller.
#pragma once

#include <mpmc/flash/pt_flash_backend.hpp>

#include <array>
#include <cmath>
#include <cstdint>
#include <optional>
#include <span>
#include <stdexcept>
#include <string>
#include <vector>

#include "mpmc_gb300_flash.h"

namespace mpmc::flash {

inline constexpr std::string_view gpu_pr76_pt_flash_backend_id = "GB300/PR76/PT/max3/phase-set-backend/v1";
inline constexpr std::string_view gpu_pr76_pt_result_convention = "GB300/PR76/PT/max3/phase-set/v1";
inline constexpr std::string_view gpu_pr76_pt_transition_evidence_profile =
    "GB300/PR76/PT/max3/phase-transition-evidence/v1";

struct GpuPr76Mixture {
    std::vector<std::string> component_ids;
    std::vector<double> critical_temperature_k;
    std::vector<double> critical_pressure_pa;
    std::vector<double> acentric_factor;
    std::vector<double> kij;  // row-major n x n, symmetric, zero diagonal
    std::string dataset_id;
    std::string revision;
};

// Caller starts of the backend, the part of Pr76PtFlashBackendOptions
// (pr76_pt_flash_backend.hpp:26-40) that the C ABI carries: up to three
// compositions used as both initial_starts and final_starts and, when
// `three_phase_fraction_seed` is set, one three-phase start made of the same
// three compositions with that phase_fraction_seed (Pr76PtThreePhaseStart,
// pr76_three_phase.hpp:114-117).  Every request of the backend gets them.
struct GpuPr76BackendStarts {
    // the continuation's form: these compositions are the initial and the
    // final starts and, with a fraction seed, the three-phase start
    std::vector<std::vector<double>> stability_starts;
    std::optional<std::array<double, 2>> three_phase_fraction_seed;
    // the general form (mpmc_gpu_flash_solve_hinted_ex), used when `general`
    bool general = false;
    std::vector<std::vector<double>> initial_starts, final_starts;
    std::optional<std::array<std::vector<double>, 3>> three_phase_start;
    std::array<double, 2> three_phase_seed{1.0 / 3.0, 1.0 / 3.0};
    bool initial_automatic_starts = true;
    int max_split_attempts = 16;
};

#if __has_include(<mpmc/flash/pr76_pt_flash_backend.hpp>)
}  // namespace mpmc::flash
#include <mpmc/flash/pr76_pt_flash_backend.hpp>
namespace mpmc::flash {

// The caller inputs of a Pr76PtFlashBackendOptions (pr76_pt_flash_backend.hpp:
// 26-40) in the binding's general form.  The device code takes at most three
// initial and three final starts and one three-phase start per cell, and the
// two split options; more starts throw std::invalid_argument.
inline GpuPr76BackendStarts gpu_starts_from(const Pr76PtFlashBackendOptions& o) {
    if (o.initial_starts.size() > 3 || o.final_starts.size() > 3 || o.three_phase_starts.size() > 1)
        throw std::invalid_argument("GPU PR76 backend: at most three initial and three final starts and one "
                                    "three-phase start");
    if (o.split.max_split_attempts > 65536)
        throw std::invalid_argument("GPU PR76 backend: max_split_attempts above 65536");
    GpuPr76BackendStarts s;
    s.general = true;
    s.initial_starts = o.initial_starts;
    s.final_starts = o.final_starts;
    if (!o.three_phase_starts.empty()) {
        s.three_phase_start = o.three_phase_starts.front().compositions;
        s.three_phase_seed = o.three_phase_starts.front().phase_fraction_seed;
    }
    s.initial_automatic_starts = o.split.initial_stability.automatic_starts;
    s.max_split_attempts = static_cast<int>(o.split.max_split_attempts);
    return s;
}
#endif

class GpuPr76PtFlashBackend final : public PtFlashBackend {
public:
    explicit GpuPr76PtFlashBackend(const GpuPr76Mixture& mixture, int form = MPMC_FORM_MIXED, int device = 0,
                                   GpuPr76BackendStarts starts = {})
        : n_(mixture.component_ids.size()), starts_(std::move(starts)) {
        if (starts_.stability_starts.size() > 3 ||
            (starts_.three_phase_fraction_seed && starts_.stability_starts.size() != 3))
            throw std::invalid_argument("GPU PR76 backend: at most three stability starts, exactly three with a "
                                        "three-phase start");
        if (starts_.general && (starts_.initial_starts.size() > 3 || starts_.final_starts.size() > 3 ||
                                starts_.max_split_attempts < 0))
            throw std::invalid_argument("GPU PR76 backend: at most three initial and three final starts");
        auto sized = [&](const std::vector<double>& st) {
            if (st.size() != n_) throw std::invalid_argument("GPU PR76 backend: start size does not match the mixture");
        };
        for (const auto& st : starts_.stability_starts) sized(st);
        for (const auto& st : starts_.initial_starts) sized(st);
        for (const auto& st : starts_.final_starts) sized(st);
        if (starts_.three_phase_start)
            for (const auto& st : *starts_.three_phase_start) sized(st);
        if (n_ == 0 || mixture.critical_temperature_k.size() != n_ || mixture.critical_pressure_pa.size() != n_ ||
            mixture.acentric_factor.size() != n_ || mixture.kij.size() != n_ * n_)
            throw std::invalid_argument("GPU PR76 backend: mixture arrays do not match the component list");
        mpmc_pr76_mixture m{static_cast<int32_t>(n_), mixture.critical_temperature_k.data(),
                            mixture.critical_pressure_pa.data(), mixture.acentric_factor.data(), mixture.kij.data()};
        mpmc_flash_options o{form, 0, device, 0};
        check(mpmc_gpu_flash_create(&m, &o, &handle_));
        capability_.backend_id = std::string(gpu_pr76_pt_flash_backend_id);
        capability_.model_profile = "PR76";
        capability_.algorithm_profile = "GB300/PR76/PT/max3/v1";
        capability_.publication_profile = std::string(gpu_pr76_pt_result_convention);
        capability_.configuration_profile =
            form == MPMC_FORM_MIXED ? "mixed-precision" : (form == MPMC_FORM_BATCHED ? "fp64-work-queue" : "plain-fp64");
        capability_.dataset_id = mixture.dataset_id;
        capability_.revision = mixture.revision;
        capability_.component_ids = mixture.component_ids;
        capability_.supported_phase_counts = {1U, 2U, 3U};
        capability_.transition_capability.edges = {
            {1U, 2U, PtPhaseTransitionSupport::fresh_target_resolve, true},
            {2U, 1U, PtPhaseTransitionSupport::detection_only, true},
            {2U, 3U, PtPhaseTransitionSupport::fresh_target_resolve, true},
            {3U, 2U, PtPhaseTransitionSupport::fresh_target_resolve, true}};
        capability_.performs_initial_stability_search = true;
        capability_.performs_final_phase_set_review = true;
        capability_.performs_boundary_neighbor_resolve = true;
        capability_.global_stability_proven = false;
    }

    GpuPr76PtFlashBackend(const GpuPr76PtFlashBackend&) = delete;
    GpuPr76PtFlashBackend& operator=(const GpuPr76PtFlashBackend&) = delete;
    ~GpuPr76PtFlashBackend() override { mpmc_gpu_flash_destroy(handle_); }

    [[nodiscard]] const PtFlashBackendCapability& capability() const noexcept override { return capability_; }

    [[nodiscard]] PtFlashBackendResult solve(const PtFlashRequest& request) override {
        return std::move(solve_batch(std::span<const PtFlashRequest>(&request, 1)).front());
    }

    // One device call for every request; results in request order.  Throws
    // std::invalid_argument for the first request outside the flash domain.
    [[nodiscard]] std::vector<PtFlashBackendResult> solve_batch(std::span<const PtFlashRequest> requests) {
        auto cells = solve_cells(requests);
        std::vector<PtFlashBackendResult> results;
        results.reserve(cells.size());
        for (std::size_t c = 0; c < cells.size(); ++c) {
            if (!cells[c])
                throw std::invalid_argument("GPU PR76 backend: request " + std::to_string(c) +
                                            " is outside the flash domain (p, T, feed)");
            results.push_back(std::move(*cells[c]));
        }
        return results;
    }

    // One device call for every request; an empty entry marks a request
    // outside the flash domain, where the reference's solve throws
    // std::invalid_argument for that request alone.  Feed-size mismatches
    // still throw for the whole batch.
    [[nodiscard]] std::vector<std::optional<PtFlashBackendResult>> solve_cells(
        std::span<const PtFlashRequest> requests) {
        const std::size_t cells = requests.size();
        std::vector<double> p(cells), t(cells), z(n_ * cells);
        for (std::size_t c = 0; c < cells; ++c) {
            const PtFlashRequest& r = requests[c];
            if (r.feed.size() != n_)
                throw std::invalid_argument("GPU PR76 backend: feed size does not match the capability");
            p[c] = r.pressure_pa;
            t[c] = r.temperature_k;
            for (std::size_t i = 0; i < n_; ++i) z[i * cells + c] = r.feed[i];
        }
        std::vector<int32_t> status(cells), counters(MPMC_COUNTER_COUNT * cells);
        std::vector<double> beta(cells), x(n_ * cells), y(n_ * cells), lnk(n_ * cells), phil(n_ * cells),
            phiv(n_ * cells), zl(cells), zv(cells);
        mpmc_flash_outputs out{};
        out.status = status.data();
        out.vapor_fraction = beta.data();
        out.liquid = x.data();
        out.vapor = y.data();
        out.ln_k = lnk.data();
        out.ln_phi_liquid = phil.data();
        out.ln_phi_vapor = phiv.data();
        out.z_liquid = zl.data();
        out.z_vapor = zv.data();
        out.counters = counters.data();
        std::vector<int32_t> max3(cells);
        std::vector<double> frac3(3 * cells), comp3(3 * n_ * cells), phi3(3 * n_ * cells), z3(3 * cells);
        mpmc_three_phase_outputs out3{max3.data(), frac3.data(), comp3.data(), phi3.data(), z3.data()};
        if (cells > 0 && starts_.general) {
            // the general caller inputs, the same for every request
            auto set = [&](const std::vector<std::vector<double>>& starts, std::vector<int32_t>& count,
                           std::vector<double>& comp) {
                count.assign(cells, static_cast<int32_t>(starts.size()));
                comp.assign(3 * n_ * cells, 0.0);
                for (std::size_t c = 0; c < cells; ++c)
                    for (std::size_t q = 0; q < starts.size(); ++q)
                        for (std::size_t i = 0; i < n_; ++i) comp[(q * n_ + i) * cells + c] = starts[q][i];
            };
            std::vector<int32_t> icount, fcount, three(cells, starts_.three_phase_start ? 1 : 0);
            std::vector<double> icomp, fcomp, tcomp(3 * n_ * cells, 0.0), frac(2 * cells, 0.0);
            set(starts_.initial_starts, icount, icomp);
            set(starts_.final_starts, fcount, fcomp);
            for (std::size_t c = 0; c < cells; ++c) {
                frac[c] = starts_.three_phase_seed[0];
                frac[cells + c] = starts_.three_phase_seed[1];
                if (starts_.three_phase_start)
                    for (std::size_t q = 0; q < 3; ++q)
                        for (std::size_t i = 0; i < n_; ++i)
                            tcomp[(q * n_ + i) * cells + c] = (*starts_.three_phase_start)[q][i];
            }
            const mpmc_start_hints_ex hints{icount.data(), icomp.data(), fcount.data(), fcomp.data(), three.data(),
                                            tcomp.data(),  frac.data(),  starts_.initial_automatic_starts ? 1 : 0,
                                            starts_.max_split_attempts};
            check(mpmc_gpu_flash_solve_hinted_ex(handle_, static_cast<int64_t>(cells), p.data(), t.data(), z.data(),
                                                 &hints, &out, &out3));
        } else if (cells > 0 && starts_.stability_starts.empty()) {
            check(mpmc_gpu_flash_solve_max3(handle_, static_cast<int64_t>(cells), p.data(), t.data(), z.data(), &out,
                                            &out3));
        } else if (cells > 0) {
            // the backend's caller starts, the same for every request
            const std::size_t k = starts_.stability_starts.size();
            std::vector<int32_t> count(cells, static_cast<int32_t>(k)), three(cells, 0);
            std::vector<double> comp(3 * n_ * cells, 0.0), frac(2 * cells, 0.0);
            for (std::size_t c = 0; c < cells; ++c) {
                for (std::size_t q = 0; q < k; ++q)
                    for (std::size_t i = 0; i < n_; ++i) comp[(q * n_ + i) * cells + c] = starts_.stability_starts[q][i];
                if (starts_.three_phase_fraction_seed) {
                    three[c] = 1;
                    frac[c] = (*starts_.three_phase_fraction_seed)[0];
                    frac[cells + c] = (*starts_.three_phase_fraction_seed)[1];
                }
            }
            const mpmc_start_hints hints{count.data(), comp.data(), three.data(), frac.data()};
            check(mpmc_gpu_flash_solve_hinted(handle_, static_cast<int64_t>(cells), p.data(), t.data(), z.data(),
                                              &hints, &out, &out3));
        }

        std::vector<std::optional<PtFlashBackendResult>> results(cells);
        for (std::size_t c = 0; c < cells; ++c) {
            if (status[c] == MPMC_FLASH_INVALID_REQUEST) continue;
            results[c].emplace();
            auto column = [&](const std::vector<double>& a) {
                std::vector<double> v(n_);
                for (std::size_t i = 0; i < n_; ++i) v[i] = a[i * cells + c];
                return v;
            };
            PtFlashBackendResult& r = *results[c];
            r.capability = capability_;
            r.transition_report = transition_report(status[c], max3[c]);
            r.provider_result_convention = std::string(gpu_pr76_pt_result_convention);
            PtPhaseSetResult& s = r.solution;
            s.capability.maximum_phase_count = 3U;
            s.pressure_pa = requests[c].pressure_pa;
            s.temperature_k = requests[c].temperature_k;
            s.feed = requests[c].feed;
            auto phase = [&](double fraction, std::vector<double> comp, std::vector<double> lnphi, double zf) {
                PtCandidatePhase ph;
                ph.mole_phase_fraction = fraction;
                ph.composition = std::move(comp);
                ph.activity.ln_phi = std::move(lnphi);
                ph.activity.smooth = true;  // accepted roots are smooth by construction
                ph.compressibility_factor = zf;
                return ph;
            };
            switch (status[c]) {
            case MPMC_FLASH_SINGLE_PHASE: {
                PtCandidatePhaseSet set;
                set.phases.push_back(phase(1.0, column(x), column(phil), zl[c]));
                s.candidate_phase_set = std::move(set);
                s.status = PtPhaseSetStatus::accepted;
                break;
            }
            case MPMC_FLASH_TWO_PHASE:
            case MPMC_FLASH_PHASE_SET_UNSTABLE: {
                PtCandidatePhaseSet set;
                set.phases.push_back(phase(1.0 - beta[c], column(x), column(phil), zl[c]));
                set.phases.push_back(phase(beta[c], column(y), column(phiv), zv[c]));
                s.candidate_phase_set = std::move(set);
                s.status = status[c] == MPMC_FLASH_TWO_PHASE ? PtPhaseSetStatus::accepted
                                                             : PtPhaseSetStatus::phase_set_unstable;
                if (status[c] == MPMC_FLASH_PHASE_SET_UNSTABLE)
                    s.diagnostic = "three-phase candidate final review found additional lower-Gibbs evidence";
                break;
            }
            case MPMC_FLASH_THREE_PHASE: {
                PtCandidatePhaseSet set;
                for (std::size_t q = 0; q < 3; ++q) {
                    std::vector<double> comp(n_), lnphi(n_);
                    for (std::size_t i = 0; i < n_; ++i) {
                        comp[i] = comp3[(q * n_ + i) * cells + c];
                        lnphi[i] = phi3[(q * n_ + i) * cells + c];
                    }
                    set.phases.push_back(phase(frac3[q * cells + c], std::move(comp), std::move(lnphi), z3[q * cells + c]));
                }
                s.candidate_phase_set = std::move(set);
                s.status = PtPhaseSetStatus::accepted;
                break;
            }
            default:
                s.status = PtPhaseSetStatus::indeterminate;
                s.diagnostic = "GB300 flash: no accepted phase set within the reference's iteration budgets";
                break;
            }
        }
        return results;
    }

    // The evidence of project_pr76_pt_max3_transition_report
    // (pr76_pt_flash_backend.hpp:94-175) for a published status and its max3
    // status, with the backend's default options (no caller hints, so a
    // max3 two-phase answer is always the base pair).
    [[nodiscard]] static PtPhaseTransitionReport transition_report(int32_t status, int32_t max3_status) {
        PtPhaseTransitionReport report;
        auto add = [&report](std::size_t from, std::optional<std::size_t> to, PtPhaseTransitionTrigger trigger,
                             PtPhaseTransitionResolution resolution, bool fresh, bool closed, const char* why) {
            report.evidence.push_back({from, to, trigger, resolution, fresh, closed,
                                       std::string(gpu_pr76_pt_transition_evidence_profile), why});
        };
        using Trigger = PtPhaseTransitionTrigger;
        using Resolution = PtPhaseTransitionResolution;
        const auto unstable_pair = [&] {
            add(1U, 2U, Trigger::initial_stability_witness, Resolution::candidate_not_accepted, true, false,
                "the first two-phase candidate failed its final common-tangent review");
        };
        switch (status) {
        case MPMC_FLASH_TWO_PHASE:
            add(1U, 2U, Trigger::initial_stability_witness, Resolution::accepted_target, true, true,
                "negative feed-stability evidence was followed by a fresh two-phase solve and final review");
            break;
        case MPMC_FLASH_THREE_PHASE:
            unstable_pair();
            add(2U, 3U, Trigger::final_phase_set_instability, Resolution::accepted_target, true, true,
                "negative final-stability evidence triggered a fresh three-phase solve that passed its final review");
            break;
        case MPMC_FLASH_PHASE_SET_UNSTABLE:
            unstable_pair();
            add(3U, std::nullopt, Trigger::final_phase_set_instability, Resolution::broader_topology_required, true,
                false, "the three-phase candidate failed its final review");
            break;
        case MPMC_FLASH_INDETERMINATE:
            if (max3_status == MPMC_MAX3_BOUNDARY_UNRESOLVED) {
                unstable_pair();
                add(2U, 3U, Trigger::final_phase_set_instability, Resolution::candidate_not_accepted, true, false,
                    "additional-phase evidence reached a three-phase disappearance boundary");
                add(3U, 2U, Trigger::phase_disappearance, Resolution::target_resolve_failed, true, false,
                    "no fresh two-phase neighbor closed");
            }
            break;
        default:
            break;
        }
        return report;
    }

private:
    static void check(int rc) {
        if (rc == MPMC_OK) return;
        const std::string what = mpmc_gpu_flash_last_error();
        if (rc == MPMC_ERR_DOMAIN) throw std::domain_error(what);
        if (rc == MPMC_ERR_INVALID_ARGUMENT || rc == MPMC_ERR_UNSUPPORTED) throw std::invalid_argument(what);
        throw std::runtime_error(what);
    }

    std::size_t n_;
    GpuPr76BackendStarts starts_;
    mpmc_gpu_flash* handle_ = nullptr;
    PtFlashBackendCapability capability_;
};

}  // namespace mpmc::flash
