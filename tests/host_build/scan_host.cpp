// The batched post-SNES scan (mpmc_hnu_gb300/cpp/gpu_post_snes_pt_flash_scan.hpp)
// run on the CPU over the reference's own Pr76PtFlashBackend (test
// infrastructure only).  Prints one line per scenario: the cell statuses, the
// target phase counts of the proposals and the summary, for
// tests/test_adapter.py to check against the reference's scan rules.
#include "gpu_post_snes_pt_flash_scan.hpp"

#include <mpmc/flash/pr76_pt_flash_backend.hpp>

#include <cstdio>

namespace fl = mpmc::flash;
namespace fw = mpmc::flow;
namespace th = mpmc::thermodynamics;

namespace {

th::Provenance source() {
    th::Provenance p;
    p.kind = th::SourceKind::synthetic_test;
    p.reference = "scan-check";
    p.revision = "v1";
    p.locator = "fixture";
    p.note = "binary fixture for the scan check";
    p.acquisition = "generated";
    p.usage_terms = "test data";
    return p;
}

// CPU stand-in of the GPU backend: the reference backend, one request at a
// time, a rejected request as an empty entry.
struct ReferenceCells {
    fl::Pr76PtFlashBackend& backend;
    const fl::PtFlashBackendCapability& capability() const { return backend.capability(); }
    std::vector<std::optional<fl::PtFlashBackendResult>> solve_cells(std::span<const fl::PtFlashRequest> rs) {
        std::vector<std::optional<fl::PtFlashBackendResult>> out(rs.size());
        for (std::size_t k = 0; k < rs.size(); ++k) {
            try {
                out[k] = backend.solve(rs[k]);
            } catch (const std::invalid_argument&) {
            }
        }
        return out;
    }
};

const char* name(fw::ScanCellStatus s) {
    switch (s) {
    case fw::ScanCellStatus::complete: return "complete";
    case fw::ScanCellStatus::indeterminate: return "indeterminate";
    case fw::ScanCellStatus::incompatible: return "incompatible";
    case fw::ScanCellStatus::out_of_range: return "out_of_range";
    case fw::ScanCellStatus::resolver_error: return "resolver_error";
    }
    return "?";
}

}  // namespace

int main() {
    // methane / n-butane (PR76 critical data of the two components)
    const auto src = source();
    std::vector<th::Component> catalog;
    th::PrParameterInput input;
    input.model_id = std::string(th::pr76_profile);
    input.dataset_id = "scan-check";
    input.revision = "v1";
    input.applicability = {std::nullopt, std::nullopt, src};
    const std::vector<std::string> ids{"c1", "c4"};
    const double tc[2] = {190.6, 425.1}, pc[2] = {4.599e6, 3.796e6}, om[2] = {0.012, 0.200};
    for (int i = 0; i < 2; ++i) {
        catalog.push_back({ids[i], ids[i], th::ComponentKind::pure, src, {}});
        input.pure.push_back({ids[i], th::SourcedScalar{tc[i], th::Unit::kelvin, src, "K", "identity"},
                              th::SourcedScalar{pc[i], th::Unit::pascal, src, "Pa", "identity"},
                              th::SourcedScalar{om[i], th::Unit::dimensionless, src, "1", "identity"}});
    }
    input.binary.push_back({ids[0], ids[1], th::SourcedScalar{0.0, th::Unit::dimensionless, src, "1", "identity"}});
    const auto params = th::PrParameterSet::create(catalog, ids, input, th::DataPolicy::allow_synthetic_tests);
    const auto model = th::Pr76Phase<double>::from_parameters(params);
    fl::Pr76VleEvaluator evaluator(model);
    fl::Pr76PtFlashBackend backend(evaluator);
    ReferenceCells cells{backend};

    // two-phase: 3 MPa, 300 K, z = (0.5, 0.5); single-phase gas: 1 MPa, 350 K, z = (0.9, 0.1)
    auto cell = [&](std::uint64_t id, std::size_t count, double p, double t, double z0) {
        return fw::ScanSourceCell{id, count, p, t, ids, {z0, 1.0 - z0}};
    };
    const auto two = [&](std::uint64_t id, std::size_t count) { return cell(id, count, 3.0e6, 300.0, 0.5); };
    const auto one = [&](std::uint64_t id, std::size_t count) { return cell(id, count, 1.0e6, 350.0, 0.9); };
    auto densities = [](const fl::PtFlashBackendResult& r, std::optional<std::vector<double>>* d) {
        std::vector<double> rho;
        for (const auto& ph : r.accepted_phase_set()->phases)
            rho.push_back(r.solution.pressure_pa /
                          (ph.compressibility_factor.value_or(1.0) * 8.31446261815324 * r.solution.temperature_k));
        *d = std::move(rho);
        return 0;
    };
    auto none = [](const fl::PtFlashBackendResult&, std::optional<std::vector<double>>*) { return 0; };
    auto fails = [](const fl::PtFlashBackendResult&, std::optional<std::vector<double>>*) { return 42; };

    auto report = [&](const char* scenario, std::vector<fw::ScanSourceCell> sources, auto resolver) {
        const auto res = fw::scan_pt_flash_source_cells_batched(std::span<const fw::ScanSourceCell>(sources), cells,
                                                               resolver);
        const auto sum = fw::summarize(sources, res);
        std::printf("%s cells", scenario);
        for (const auto& r : res)
            std::printf(" %s:%zu", name(r.status), r.candidate ? r.candidate->target_phase_count : 0);
        std::printf(" summary %s %zu %d", name(sum.status), sum.deciding_cell, sum.resolver_error);
        for (const auto& [id, cand] : sum.proposals)
            std::printf(" proposal %llu %zu->%zu", static_cast<unsigned long long>(id), cand.source_phase_count,
                        cand.target_phase_count);
        std::printf("\n");
    };
    auto bad = two(9, 1);
    bad.overall_composition = {0.5, 0.49};
    report("steady", {two(1, 2), one(2, 1)}, densities);
    report("appear", {one(1, 1), two(2, 1), two(3, 2)}, densities);
    report("vanish", {two(1, 2), one(2, 2)}, densities);
    report("malformed", {two(1, 1), bad}, densities);
    report("no_density", {two(1, 1)}, none);
    report("resolver", {one(1, 1), two(2, 1)}, fails);
    report("indeterminate_first", {two(1, 1), bad, one(3, 1)}, none);
    return 0;
}
