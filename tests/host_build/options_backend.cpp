// The backend binding with the reference's own Pr76PtFlashBackendOptions
// (GpuPr76PtFlashBackend with gpu_starts_from(options),
// mpmc_hnu_gb300/cpp/gpu_pr76_pt_flash_backend.hpp) run on the CPU beside the
// reference's Pr76PtFlashBackend built with the same options (test
// infrastructure only).  The binding's C-ABI calls are provided by the host
// build of the device code (flash_host.cpp, linked beside this file); the
// reference model is built by the oracle's harness (included below).
//
// Input (binary, from the test): n; tc, pc, omega [n]; kij [n n]; p, T;
// feed [n]; initial starts (count, then count x n); final starts (likewise);
// a three-phase start flag, its 3 x n compositions and 2 fraction seeds;
// automatic initial starts (0/1); max split attempts.  Prints the reference's
// and the binding's statuses and phase counts and the largest difference of
// their published compositions.
#include "gpu_pr76_pt_flash_backend.hpp"

#include "../../oracle/ref_harness.cpp"

#include <cstdio>
#include <fstream>
#include <limits>

extern "C" int host_hinted_batch(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                                 int64_t ncell, const double* p, const double* t, const double* z,
                                 const int32_t* hint_count, const double* hint_x, const int32_t* three,
                                 const double* fraction, int32_t* published, int32_t* max3, double* x, double* y,
                                 double* x3, double* f3);
extern "C" int host_hinted_ex_batch(int n, const double* tc, const double* pc, const double* omega,
                                    const double* kij, int64_t ncell, const double* p, const double* t,
                                    const double* z, const int32_t* initial_count, const double* initial_x,
                                    const int32_t* final_count, const double* final_x, const int32_t* three,
                                    const double* three_x, const double* fraction, int32_t initial_automatic_starts,
                                    int32_t max_split_attempts, int32_t* published, int32_t* max3, double* x,
                                    double* y, double* x3, double* f3);

struct mpmc_gpu_flash {
    int n;
    std::vector<double> tc, pc, omega, kij;
};

namespace {
void fill_unused(int64_t n, int64_t ncell, const mpmc_flash_outputs* out, const mpmc_three_phase_outputs* out3) {
    const double nan = std::numeric_limits<double>::quiet_NaN();
    for (int64_t k = 0; k < n * ncell; ++k) out->ln_phi_liquid[k] = out->ln_phi_vapor[k] = out->ln_k[k] = nan;
    for (int64_t k = 0; k < ncell; ++k) out->vapor_fraction[k] = out->z_liquid[k] = out->z_vapor[k] = nan;
    for (int64_t k = 0; k < 3 * n * ncell; ++k) out3->ln_phi[k] = nan;
    for (int64_t k = 0; k < 3 * ncell; ++k) out3->z_factor[k] = nan;
}
}  // namespace

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
    return MPMC_ERR_UNSUPPORTED;  // not used: these scenarios carry options
}
int mpmc_gpu_flash_solve_hinted(mpmc_gpu_flash* h, int64_t ncell, const double* p, const double* t, const double* z,
                                const mpmc_start_hints* hints, const mpmc_flash_outputs* out,
                                const mpmc_three_phase_outputs* out3) {
    fill_unused(h->n, ncell, out, out3);
    return host_hinted_batch(h->n, h->tc.data(), h->pc.data(), h->omega.data(), h->kij.data(), ncell, p, t, z,
                             hints->count, hints->composition, hints->three_phase, hints->fraction, out->status,
                             out3->max3_status, out->liquid, out->vapor, out3->composition, out3->phase_fraction);
}
int mpmc_gpu_flash_solve_hinted_ex(mpmc_gpu_flash* h, int64_t ncell, const double* p, const double* t,
                                   const double* z, const mpmc_start_hints_ex* hints, const mpmc_flash_outputs* out,
                                   const mpmc_three_phase_outputs* out3) {
    fill_unused(h->n, ncell, out, out3);
    return host_hinted_ex_batch(h->n, h->tc.data(), h->pc.data(), h->omega.data(), h->kij.data(), ncell, p, t, z,
                                hints->initial_count, hints->initial_composition, hints->final_count,
                                hints->final_composition, hints->three_phase, hints->three_phase_composition,
                                hints->fraction, hints->initial_automatic_starts, hints->max_split_attempts,
                                out->status, out3->max3_status, out->liquid, out->vapor, out3->composition,
                                out3->phase_fraction);
}
}

int main(int argc, char** argv) {
    if (argc != 2) return 2;
    std::ifstream in(argv[1], std::ios::binary);
    auto rd = [&](double* v, std::size_t k) { in.read(reinterpret_cast<char*>(v), static_cast<std::streamsize>(8 * k)); };
    auto rd1 = [&]() {
        double v;
        rd(&v, 1);
        return v;
    };
    const int n = static_cast<int>(rd1());
    std::vector<double> tc(n), pc(n), om(n), kij(n * n), feed(n);
    rd(tc.data(), n);
    rd(pc.data(), n);
    rd(om.data(), n);
    rd(kij.data(), n * n);
    const double p = rd1(), t = rd1();
    rd(feed.data(), n);
    auto starts = [&]() {
        std::vector<std::vector<double>> s(static_cast<std::size_t>(rd1()), std::vector<double>(n));
        for (auto& w : s) rd(w.data(), n);
        return s;
    };
    fl::Pr76PtFlashBackendOptions options;
    options.initial_starts = starts();
    options.final_starts = starts();
    if (rd1() != 0.0) {
        fl::Pr76PtThreePhaseStart st;
        for (auto& w : st.compositions) {
            w.resize(n);
            rd(w.data(), n);
        }
        rd(st.phase_fraction_seed.data(), 2);
        options.three_phase_starts.push_back(st);
    }
    options.split.initial_stability.automatic_starts = rd1() != 0.0;
    options.split.max_split_attempts = static_cast<std::size_t>(rd1());
    // the reference's backend
    std::vector<std::string> order;
    const auto model = th::Pr76Phase<double>::from_parameters(
        make_parameters(n, tc.data(), pc.data(), om.data(), kij.data(), order));
    fl::Pr76VleEvaluator evaluator(model);
    fl::Pr76PtFlashBackend reference(evaluator, options);
    const auto ref = reference.solve({p, t, feed});
    // the binding with the same options
    fl::GpuPr76Mixture mix;
    mix.component_ids = order;
    mix.critical_temperature_k = tc;
    mix.critical_pressure_pa = pc;
    mix.acentric_factor = om;
    mix.kij = kij;
    mix.dataset_id = "synthetic";
    mix.revision = "v1";
    fl::GpuPr76PtFlashBackend gpu(mix, MPMC_FORM_PLAIN_FP64, 0, fl::gpu_starts_from(options));
    const auto got = gpu.solve({p, t, feed});
    const auto* a = ref.solution.accepted_phase_set();
    const auto* b = got.solution.accepted_phase_set();
    double worst = -1.0;
    if (a && b && a->phases.size() == b->phases.size()) {
        worst = 0.0;
        for (std::size_t q = 0; q < a->phases.size(); ++q)
            for (int i = 0; i < n; ++i)
                worst = std::max(worst, std::abs(a->phases[q].composition[i] - b->phases[q].composition[i]));
    }
    std::printf("%d %d %zu %zu %.3g\n", static_cast<int>(ref.solution.status), static_cast<int>(got.solution.status),
                a ? a->phases.size() : 0, b ? b->phases.size() : 0, worst);
    return 0;
}
