// The backend binding with caller starts (GpuPr76PtFlashBackend with
// GpuPr76BackendStarts, mpmc_hnu_gb300/cpp/gpu_pr76_pt_flash_backend.hpp) run
// on the CPU beside the reference's own seeded Pr76PtFlashBackend (test
// infrastructure only).  The C-ABI calls of the binding are provided here by
// the host build of the device code (flash_host.cpp, linked beside this
// file).  The scenario is the reference's seeded-backend test
// (tests/flash/pt_flash_backend/pr76_max3_seeded_backend_test.cpp): the
// synthetic three-phase fixture at 1 MPa, 250 K with its structural starts
// as initial, final and three-phase starts.  Prints the statuses, phase
// counts, the largest composition difference and the 2 -> 3 evidence.
#include "gpu_pr76_pt_flash_backend.hpp"

#include <mpmc/flash/pr76_pt_flash_backend.hpp>

#include <cmath>
#include <cstdio>
#include <limits>

#include "synthetic_fixture.hpp"  // the reference tests' fixture (tests/flash/pr76_three_phase)

extern "C" int host_hinted_batch(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                                 int64_t ncell, const double* p, const double* t, const double* z,
                                 const int32_t* hint_count, const double* hint_x, const int32_t* three,
                                 const double* fraction, int32_t* published, int32_t* max3, double* x, double* y,
                                 double* x3, double* f3);

struct mpmc_gpu_flash {
    int n;
    std::vector<double> tc, pc, omega, kij;
};

extern "C" {
int mpmc_gpu_flash_create(const mpmc_pr76_mixture* m, const mpmc_flash_options*, mpmc_gpu_flash** out) {
    const int n = m->n_components;
    *out = new mpmc_gpu_flash{n, {m->critical_temperature_k, m->critical_temperature_k + n},
                              {m->critical_pressure_pa, m->critical_pressure_pa + n},
                              {m->acentric_factor, m->acentric_factor + n}, {m->kij, m->kij + n * n}};
    return MPMC_OK;
}
int mpmc_gpu_flash_destroy(mpmc_gpu_flash* h) {
    delete h;
    return MPMC_OK;
}
const char* mpmc_gpu_flash_last_error(void) { return "host build"; }
int mpmc_gpu_flash_solve_max3(mpmc_gpu_flash*, int64_t, const double*, const double*, const double*,
                              const mpmc_flash_outputs*, const mpmc_three_phase_outputs*) {
    return MPMC_ERR_UNSUPPORTED;  // not used: this scenario has caller starts
}
int mpmc_gpu_flash_solve_hinted_ex(mpmc_gpu_flash*, int64_t, const double*, const double*, const double*,
                                   const mpmc_start_hints_ex*, const mpmc_flash_outputs*,
                                   const mpmc_three_phase_outputs*) {
    return MPMC_ERR_UNSUPPORTED;  // not used: this scenario has the continuation's starts
}
int mpmc_gpu_flash_solve_hinted(mpmc_gpu_flash* h, int64_t ncell, const double* p, const double* t, const double* z,
                                const mpmc_start_hints* hints, const mpmc_flash_outputs* out,
                                const mpmc_three_phase_outputs* out3) {
    const double nan = std::numeric_limits<double>::quiet_NaN();
    const int64_t n = h->n;
    for (int64_t k = 0; k < n * ncell; ++k) out->ln_phi_liquid[k] = out->ln_phi_vapor[k] = out->ln_k[k] = nan;
    for (int64_t k = 0; k < ncell; ++k) out->vapor_fraction[k] = out->z_liquid[k] = out->z_vapor[k] = nan;
    for (int64_t k = 0; k < 3 * n * ncell; ++k) out3->ln_phi[k] = nan;
    for (int64_t k = 0; k < 3 * ncell; ++k) out3->z_factor[k] = nan;
    return host_hinted_batch(h->n, h->tc.data(), h->pc.data(), h->omega.data(), h->kij.data(), ncell, p, t, z,
                             hints->count, hints->composition, hints->three_phase, hints->fraction, out->status,
                             out3->max3_status, out->liquid, out->vapor, out3->composition, out3->phase_fraction);
}
}

namespace fl = mpmc::flash;

int main() {
    const auto model = pr76_max3_test::model();
    fl::Pr76VleEvaluator evaluator(model);
    const auto feed = pr76_max3_test::equal_feed();
    const auto starts = pr76_max3_test::starts();
    // the reference's seeded backend
    fl::Pr76PtFlashBackendOptions options;
    options.initial_starts = starts;
    options.final_starts = starts;
    fl::Pr76PtThreePhaseStart three;
    three.compositions = {starts[0], starts[1], starts[2]};
    options.three_phase_starts.push_back(three);
    fl::Pr76PtFlashBackend reference(evaluator, options);
    const auto ref = reference.solve({1.0e6, 250.0, feed});
    // the binding with the same starts
    fl::GpuPr76Mixture mix;
    mix.component_ids = {"c0", "c1", "c2"};  // the fixture's PR76 data (synthetic_fixture.hpp:33-57)
    mix.critical_temperature_k = {190.6, 500.0, 500.0};
    mix.critical_pressure_pa = {4.6e6, 5.0e6, 5.0e6};
    mix.acentric_factor = {0.01, 0.10, 0.10};
    mix.kij = {0.0, 0.05, 0.05, 0.05, 0.0, 0.20, 0.05, 0.20, 0.0};
    mix.dataset_id = "synthetic";
    mix.revision = "v1";
    fl::GpuPr76BackendStarts gs;
    gs.stability_starts = starts;
    gs.three_phase_fraction_seed = three.phase_fraction_seed;
    fl::GpuPr76PtFlashBackend gpu(mix, MPMC_FORM_PLAIN_FP64, 0, gs);
    const auto got = gpu.solve({1.0e6, 250.0, feed});
    const auto* a = ref.solution.accepted_phase_set();
    const auto* b = got.solution.accepted_phase_set();
    double worst = -1.0;
    if (a && b && a->phases.size() == b->phases.size()) {
        worst = 0.0;
        for (std::size_t q = 0; q < a->phases.size(); ++q)
            for (std::size_t i = 0; i < feed.size(); ++i)
                worst = std::max(worst, std::abs(a->phases[q].composition[i] - b->phases[q].composition[i]));
    }
    auto has_2_to_3 = [](const fl::PtFlashBackendResult& r) {
        for (const auto& e : r.transition_report.evidence)
            if (e.source_phase_count == 2U && e.target_phase_count == 3U &&
                e.resolution == fl::PtPhaseTransitionResolution::accepted_target && e.fresh_target_solve_attempted &&
                e.target_topology_closed)
                return 1;
        return 0;
    };
    std::printf("%d %d %zu %zu %.3g %d %d\n", static_cast<int>(ref.solution.status),
                static_cast<int>(got.solution.status), a ? a->phases.size() : 0, b ? b->phases.size() : 0, worst,
                has_2_to_3(ref), has_2_to_3(got));
    return 0;
}
