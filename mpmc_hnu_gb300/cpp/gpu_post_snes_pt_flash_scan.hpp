// Batched post-SNES PT-flash phase-transition scan for the flow cell loop.
//
// The reference scans the owned cells of a converged SNES state one at a
// time: scan_post_snes_pt_flash_phase_transitions_3d
// (modules/flow/discretization/petsc/include/mpmc/flow_discretization_petsc/
// post_snes_pt_flash_phase_transition_scanner.hpp:303-421) builds each
// cell's source snapshot and calls scan_post_snes_pt_flash_source_cell_3d
// (:207-301), whose PtFlashBackend::solve is one flash.  Here the flashes of
// every source cell go to the device in one call (GpuPr76PtFlashBackend::
// solve_cells), and each cell is then judged by the reference's own rules in
// the reference's order:
//   * a malformed snapshot or a backend that does not match the cell's
//     components or phase count            -> incompatible (PETSC_ERR_ARG_INCOMP);
//   * a request the flash rejects          -> incompatible (the reference's
//                                             std::invalid_argument);
//   * a result whose provenance, p, T or feed differ from the request, or
//     without an accepted phase set         -> indeterminate;
//   * the source's phase count accepted    -> complete, no proposal;
//   * otherwise the caller's density resolver and
//     make_phase_set_transition_candidate_from_flash
//     (phase_set_transition_flash_adapter.hpp:130-248) give the proposal, or
//     indeterminate, or the resolver's error; the candidate's
//     std::invalid_argument -> incompatible, std::out_of_range ->
//     out_of_range (PETSC_ERR_ARG_OUTOFRANGE), any other exception ->
//     indeterminate.
// summarize() then applies the loop's rule (:397-418): the first cell, in
// order, that is not complete decides -- an error code is returned, an
// indeterminate cell makes the whole scan indeterminate with no proposals --
// and otherwise every proposal is kept in cell order.
//
// A source cell here is the per-cell function's input: a malformed one is
// incompatible, as there.  The loop builds its snapshots from the converged
// state first (make_source_snapshot, :160-203) and reports a snapshot it
// cannot build as an indeterminate scan; a caller that builds its own
// snapshots reports that case itself before calling.
//
// This header needs no PETSc: the status enum maps one to one onto the
// scanner's PetscErrorCode / PostSnesPhaseTransitionScanStatus3D, and
// ScanSourceCell carries the fields of PostSnesPtFlashSourceCellSnapshot3D
// (:30-38).  The density resolver is called for every cell whose accepted
// phase count changed, including cells after the first indeterminate one,
// so it must not have side effects that the reference's early return would
// have skipped.
#pragma once

#include <mpmc/flow/detail/validation.hpp>
#include <mpmc/flow/phase_set_transition_flash_adapter.hpp>

#include <cmath>
#include <cstdint>
#include <exception>
#include <optional>
#include <span>
#include <stdexcept>
#include <string>
#include <vector>

#include "gpu_pr76_pt_flash_backend.hpp"

namespace mpmc::flow {

struct ScanSourceCell {
    std::uint64_t cell_global{};
    std::size_t source_phase_count{};
    double pressure_pa{};
    double temperature_k{};
    std::vector<std::string> component_ids;
    std::vector<double> overall_composition;
};

enum class ScanCellStatus {
    complete,       // PETSC_SUCCESS, scan status complete (with or without a proposal)
    indeterminate,  // PETSC_SUCCESS, scan status indeterminate
    incompatible,   // PETSC_ERR_ARG_INCOMP
    out_of_range,   // PETSC_ERR_ARG_OUTOFRANGE
    resolver_error  // the density resolver's own nonzero error code
};

struct ScanCellResult {
    ScanCellStatus status{ScanCellStatus::complete};
    int resolver_error{0};
    std::optional<PhaseSetTransitionCandidate> candidate;
};

namespace gpu_scan_detail {

[[nodiscard]] inline bool near_roundoff(double a, double b) {
    return validation_detail::near_roundoff<8192>(a, b);
}

// validate_source_snapshot (:76-114): a status, never an exception.
[[nodiscard]] inline bool valid_source(const ScanSourceCell& s) {
    if (s.source_phase_count == 0U || s.source_phase_count > fixed_three_phase_count ||
        !std::isfinite(s.pressure_pa) || !(s.pressure_pa > 0.0) || !std::isfinite(s.temperature_k) ||
        !(s.temperature_k > 0.0) || s.component_ids.size() < 2U ||
        s.overall_composition.size() != s.component_ids.size())
        return false;
    long double sum = 0.0L;
    for (std::size_t i = 0; i < s.component_ids.size(); ++i) {
        if (s.component_ids[i].empty() || !std::isfinite(s.overall_composition[i]) ||
            !(s.overall_composition[i] > 0.0))
            return false;
        for (std::size_t j = 0; j < i; ++j)
            if (s.component_ids[j] == s.component_ids[i]) return false;
        sum += static_cast<long double>(s.overall_composition[i]);
    }
    const long double tolerance = 4096.0L * static_cast<long double>(std::numeric_limits<double>::epsilon()) *
                                  static_cast<long double>(s.component_ids.size());
    return std::isfinite(static_cast<double>(sum)) && std::abs(sum - 1.0L) <= tolerance;
}

}  // namespace gpu_scan_detail

// Backend: flash::GpuPr76PtFlashBackend, or any type with capability() and
// solve_cells(std::span<const PtFlashRequest>) ->
// std::vector<std::optional<PtFlashBackendResult>> (empty = the request was
// rejected).  Resolver: int(const flash::PtFlashBackendResult&,
// std::optional<std::vector<double>>*), returning 0 on success (the
// PostSnesPtFlashTargetPhaseMolarDensityResolver3D contract, :40-49, without
// the user context).
template <class Backend, class DensityResolver>
[[nodiscard]] std::vector<ScanCellResult> scan_pt_flash_source_cells_batched(
    std::span<const ScanSourceCell> sources, Backend& backend, DensityResolver&& resolver) {
    using namespace gpu_scan_detail;
    const std::size_t cells = sources.size();
    std::vector<ScanCellResult> out(cells);
    const auto& capability = backend.capability();
    std::vector<flash::PtFlashRequest> requests;
    std::vector<std::size_t> solved;
    for (std::size_t c = 0; c < cells; ++c) {
        const ScanSourceCell& s = sources[c];
        if (!valid_source(s) || !capability.structurally_valid() || capability.component_ids != s.component_ids ||
            !capability.supports_phase_count(s.source_phase_count)) {
            out[c].status = ScanCellStatus::incompatible;
            continue;
        }
        requests.push_back({s.pressure_pa, s.temperature_k, s.overall_composition});
        solved.push_back(c);
    }
    auto results = backend.solve_cells(requests);
    for (std::size_t k = 0; k < solved.size(); ++k) {
        const std::size_t c = solved[k];
        const ScanSourceCell& s = sources[c];
        ScanCellResult& cell = out[c];
        if (!results[k]) {
            cell.status = ScanCellStatus::incompatible;
            continue;
        }
        const flash::PtFlashBackendResult& r = *results[k];
        const flash::PtFlashRequest& q = requests[k];
        bool same_feed = r.solution.feed.size() == q.feed.size();
        for (std::size_t i = 0; same_feed && i < q.feed.size(); ++i)
            same_feed = near_roundoff(r.solution.feed[i], q.feed[i]);
        if (!r.structurally_valid() || r.capability.backend_id != capability.backend_id ||
            r.capability.model_profile != capability.model_profile ||
            r.capability.configuration_profile != capability.configuration_profile ||
            r.capability.dataset_id != capability.dataset_id || r.capability.revision != capability.revision ||
            r.capability.component_ids != capability.component_ids ||
            !near_roundoff(r.solution.pressure_pa, q.pressure_pa) ||
            !near_roundoff(r.solution.temperature_k, q.temperature_k) || !same_feed) {
            cell.status = ScanCellStatus::indeterminate;
            continue;
        }
        const auto* accepted = r.accepted_phase_set();
        if (accepted == nullptr) {
            cell.status = ScanCellStatus::indeterminate;
            continue;
        }
        if (accepted->phases.size() == s.source_phase_count) continue;  // complete, no proposal
        try {
            std::optional<std::vector<double>> densities;
            const int err = resolver(r, &densities);
            if (err != 0) {
                cell.status = ScanCellStatus::resolver_error;
                cell.resolver_error = err;
                continue;
            }
            if (!densities) {
                cell.status = ScanCellStatus::indeterminate;
                continue;
            }
            cell.candidate = make_phase_set_transition_candidate_from_flash(s.source_phase_count, r, *densities);
            if (!cell.candidate) cell.status = ScanCellStatus::indeterminate;
        } catch (const std::invalid_argument&) {
            cell.status = ScanCellStatus::incompatible;
        } catch (const std::out_of_range&) {
            cell.status = ScanCellStatus::out_of_range;
        } catch (const std::exception&) {
            cell.status = ScanCellStatus::indeterminate;
        }
    }
    return out;
}

// The loop's verdict over the cells in order (:397-418).
struct ScanSummary {
    ScanCellStatus status{ScanCellStatus::complete};  // complete, indeterminate, or the first error
    int resolver_error{0};
    std::size_t deciding_cell{0};                        // the first cell that was not complete
    std::vector<std::pair<std::uint64_t, PhaseSetTransitionCandidate>> proposals;
};

[[nodiscard]] inline ScanSummary summarize(std::span<const ScanSourceCell> sources,
                                           std::span<const ScanCellResult> cells) {
    ScanSummary summary;
    for (std::size_t c = 0; c < cells.size(); ++c) {
        if (cells[c].status != ScanCellStatus::complete) {
            summary.status = cells[c].status;
            summary.resolver_error = cells[c].resolver_error;
            summary.deciding_cell = c;
            summary.proposals.clear();
            return summary;
        }
        if (cells[c].candidate) summary.proposals.emplace_back(sources[c].cell_global, *cells[c].candidate);
    }
    summary.deciding_cell = cells.size();
    return summary;
}

}  // namespace mpmc::flow
