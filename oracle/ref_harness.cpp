// Harness around the UNMODIFIED MPMC_HNU reference headers (test
// infrastructure).  oracle/Makefile compiles this file against the reference
// include directories where they lie and writes oracle/_ref/libpr76_ref.so.
// It exposes the same C interface as oracle/pr76_flash_oracle.cpp
// (ref_flash_batch <-> oracle_flash_batch) so that tests can compare the CPU
// restatement with the reference on identical inputs, and so that
// tests/golden/make_golden.py can record reference outputs as fixtures.
//
// Reference entry points used:
//   mpmc::flash::solve_pr76_pt_vle                 modules/flash/include/mpmc/flash/pr76_split.hpp:99
//   mpmc::flash::differentiate_pr76_pt_vle         modules/flash/include/mpmc/flash/pr76_sensitivity.hpp:51
//   mpmc::physics::build_pr76_pt_vle_closure       modules/physics/include/mpmc/physics/pr76_thermodynamic_closure.hpp:148
//   mpmc::thermodynamics::Pr76PhaseAdWorkspace     modules/thermodynamics/include/mpmc/thermodynamics/pr76_phase_ad.hpp:43
//   mpmc::flash::Pr76PtFlashBackend::solve         modules/flash/include/mpmc/flash/pr76_pt_flash_backend.hpp:190
//   mpmc::flash::solve_pr76_pt_max3                modules/flash/include/mpmc/flash/pr76_three_phase.hpp:328
//   mpmc::flash::solve_pr76_pt_continuation        modules/flash/include/mpmc/flash/pr76_pt_continuation.hpp:183
//   mpmc::flow::evaluate_pr76_selected_phase_property_chart
//                                                  modules/flow/include/mpmc/flow/pr76_selected_phase_property_closure.hpp:533

#include <mpmc/flash/pr76_pt_flash_backend.hpp>
#include <mpmc/flash/pr76_three_phase.hpp>
#include <mpmc/flash/pr76_max3_phase_set.hpp>
#include <mpmc/flash/pr76_pt_continuation.hpp>
#include <mpmc/flash/pr76_sensitivity.hpp>
#include <mpmc/flow/pr76_selected_phase_property_closure.hpp>
#include <mpmc/physics/pr76_thermodynamic_closure.hpp>
#include <mpmc/thermodynamics/pr76_phase_ad.hpp>

#include <cmath>
#include <cstdint>
#include <limits>
#include <string>
#include <thread>
#include <vector>

namespace {
namespace fl = mpmc::flash;
namespace th = mpmc::thermodynamics;
namespace ph = mpmc::physics;

th::Provenance synthetic_source() {
    th::Provenance p;
    p.kind = th::SourceKind::synthetic_test;
    p.reference = "mpmc-gb300-synthetic";
    p.revision = "v1";
    p.locator = "seeded generator";
    p.note = "synthetic mixture for GPU parity tests";
    p.acquisition = "generated";
    p.usage_terms = "test data";
    return p;
}

th::PrParameterSet make_parameters(int n, const double* tc, const double* pc, const double* omega,
                                   const double* kij, std::vector<std::string>& order,
                                   const double* molar_mass = nullptr) {
    const auto src = synthetic_source();
    std::vector<th::Component> catalog;
    th::PrParameterInput input;
    input.model_id = std::string(th::pr76_profile);
    input.dataset_id = "synthetic";
    input.revision = "v1";
    input.applicability = {std::nullopt, std::nullopt, src};
    order.clear();
    for (int i = 0; i < n; ++i) {
        const std::string id = "c" + std::to_string(i);
        order.push_back(id);
        std::optional<th::SourcedScalar> mw;
        if (molar_mass) mw = th::SourcedScalar{molar_mass[i], th::Unit::kilogram_per_mole, src, "kg/mol", "identity"};
        catalog.push_back({id, id, th::ComponentKind::pure, src, std::move(mw)});
        input.pure.push_back({id, th::SourcedScalar{tc[i], th::Unit::kelvin, src, "K", "identity"},
                              th::SourcedScalar{pc[i], th::Unit::pascal, src, "Pa", "identity"},
                              th::SourcedScalar{omega[i], th::Unit::dimensionless, src, "1", "identity"}});
    }
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j)
            input.binary.push_back({order[i], order[j],
                                    th::SourcedScalar{kij[i * n + j], th::Unit::dimensionless, src, "1",
                                                      "identity"}});
    return th::PrParameterSet::create(catalog, order, input, th::DataPolicy::allow_synthetic_tests);
}

int status_code(fl::PtSplitStatus s) {
    switch (s) {
    case fl::PtSplitStatus::single_phase_no_instability_found: return 0;
    case fl::PtSplitStatus::two_phase_no_instability_found: return 1;
    case fl::PtSplitStatus::phase_set_unstable: return 2;
    case fl::PtSplitStatus::indeterminate: return 3;
    }
    return 3;
}
}  // namespace

extern "C" {

struct OracleOutputs {
    int32_t* status;
    double* beta;
    double* x;
    double* y;
    double* ln_k;
    double* ln_phi_l;
    double* ln_phi_v;
    double* z_l;
    double* z_v;
    int64_t* counters;
    int32_t* sens_status;
    double* dlnk;
    double* dbeta;
    double* dx;
    double* dy;
    double* dzl;
    double* dzv;
    double* drhol;
    double* drhov;
    double* jl;
    double* jv;
};

int ref_flash_batch(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                    int64_t ncell, const double* p, const double* t, const double* z, int threads,
                    int want_sensitivity, const OracleOutputs* o) {
    std::vector<std::string> order;
    const th::PrParameterSet params = make_parameters(n, tc, pc, omega, kij, order);
    const auto model = th::Pr76Phase<double>::from_parameters(params);
    const double nan = std::numeric_limits<double>::quiet_NaN();
    auto run = [&](int64_t lo, int64_t hi) {
        fl::Pr76VleEvaluator evaluator(model);
        for (int64_t c = lo; c < hi; ++c) {
            auto put = [&](double* arr, int k, double v) {
                if (arr) arr[k * ncell + c] = v;
            };
            std::vector<double> feed(n);
            for (int i = 0; i < n; ++i) feed[i] = z[i * ncell + c];
            fl::Pr76PtSplitResult split;
            bool invalid = false;
            try {
                split = fl::solve_pr76_pt_vle(p[c], t[c], feed, evaluator);
            } catch (const std::exception&) {
                invalid = true;
            }
            const int st = invalid ? -1 : status_code(split.solution.status);
            if (o->status) o->status[c] = st;
            const fl::PtSplitState* cand = invalid ? nullptr : split.solution.candidate();
            const bool pair = cand != nullptr && st != 0;
            put(o->beta, 0, pair ? cand->fractions.vapor_fraction : nan);
            double zl = nan;
            if (!invalid && st == 0) {
                // Z of the minimum-Gibbs feed branch (the reference's generic
                // stability phase carries only its branch index).
                th::Pr76PhaseWorkspace<double> ws;
                const auto& ref = *split.solution.initial_stability.reference;
                zl = model.evaluate_full(p[c], t[c], std::span<const double>{split.solution.initial_stability.feed},
                                         ref.branch, ws)
                         .z;
            }
            for (int i = 0; i < n; ++i) {
                if (pair) {
                    put(o->x, i, cand->fractions.liquid[i]);
                    put(o->y, i, cand->fractions.vapor[i]);
                    put(o->ln_k, i, cand->log_k[i]);
                    put(o->ln_phi_l, i, cand->liquid.activity.ln_phi[i]);
                    put(o->ln_phi_v, i, cand->vapor.activity.ln_phi[i]);
                } else if (st == 0) {
                    put(o->x, i, split.solution.initial_stability.feed[i]);
                    put(o->y, i, nan);
                    put(o->ln_k, i, nan);
                    put(o->ln_phi_l, i, split.solution.initial_stability.reference->ln_phi[i]);
                    put(o->ln_phi_v, i, nan);
                } else {
                    for (double* arr : {o->x, o->y, o->ln_k, o->ln_phi_l, o->ln_phi_v}) put(arr, i, nan);
                }
            }
            put(o->z_l, 0, pair ? cand->liquid.z : zl);
            put(o->z_v, 0, pair ? cand->vapor.z : nan);
            if (o->counters) {
                int64_t cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                if (!invalid) {
                    cnt[0] = static_cast<int64_t>(split.solution.initial_stability.evaluations);
                    cnt[1] = static_cast<int64_t>(split.solution.split_evaluations);
                    cnt[2] = split.solution.final_stability
                                 ? static_cast<int64_t>(split.solution.final_stability->evaluations)
                                 : 0;
                    for (const auto& a : split.solution.attempts) cnt[3] += a.iterations;
                    cnt[6] = static_cast<int64_t>(split.solution.attempts.size());
                    for (const auto& tr : split.solution.initial_stability.trials) cnt[7] += tr.iterations;
                    if (split.solution.final_stability)
                        for (const auto& tr : split.solution.final_stability->trials) cnt[7] += tr.iterations;
                }
                for (int k = 0; k < 8; ++k) o->counters[k * ncell + c] = cnt[k];
            }
            if (!want_sensitivity) continue;
            const int q = n + 1;
            int sstat = 1;
            std::vector<double> dlnk, dx, dy, dbeta, dzl, dzv, drl, drv, jl, jv;
            if (!invalid && st == 1) {
                const auto sens = fl::differentiate_pr76_pt_vle(split, evaluator);
                sstat = static_cast<int>(sens.sensitivity.status);
                if (sstat == 0) {
                    dlnk = sens.sensitivity.log_k_jacobian;
                    dx = sens.sensitivity.liquid_jacobian;
                    dy = sens.sensitivity.vapor_jacobian;
                    dbeta = sens.sensitivity.vapor_fraction_gradient;
                    const auto closure = ph::build_pr76_pt_vle_closure(split, evaluator);
                    if (closure.linearization) {
                        dzl = closure.linearization->liquid_compressibility_gradient;
                        dzv = closure.linearization->vapor_compressibility_gradient;
                        drl = closure.linearization->liquid_molar_density_gradient;
                        drv = closure.linearization->vapor_molar_density_gradient;
                    }
                    th::Pr76PhaseAdWorkspace<double, 4> ad;
                    const auto lj = ad.value_and_jacobian_full(model, p[c], t[c], cand->fractions.liquid,
                                                               cand->liquid.activity.branch);
                    const auto vj = ad.value_and_jacobian_full(model, p[c], t[c], cand->fractions.vapor,
                                                               cand->vapor.activity.branch);
                    jl = lj.jacobian;
                    jv = vj.jacobian;
                }
            }
            if (o->sens_status) o->sens_status[c] = sstat;
            auto copy = [&](double* arr, const std::vector<double>& v, int count) {
                for (int k = 0; k < count; ++k) put(arr, k, k < static_cast<int>(v.size()) ? v[k] : nan);
            };
            copy(o->dlnk, dlnk, n * q);
            copy(o->dx, dx, n * q);
            copy(o->dy, dy, n * q);
            copy(o->dbeta, dbeta, q);
            copy(o->dzl, dzl, q);
            copy(o->dzv, dzv, q);
            copy(o->drhol, drl, q);
            copy(o->drhov, drv, q);
            copy(o->jl, jl, (n + 1) * (n + 2));
            copy(o->jv, jv, (n + 1) * (n + 2));
        }
    };
    if (threads < 1) threads = 1;
    if (threads > ncell) threads = static_cast<int>(ncell > 0 ? ncell : 1);
    std::vector<std::thread> pool;
    const int64_t chunk = (ncell + threads - 1) / threads;
    for (int k = 0; k < threads; ++k) {
        const int64_t lo = k * chunk, hi = std::min<int64_t>(ncell, lo + chunk);
        if (lo < hi) pool.emplace_back(run, lo, hi);
    }
    for (auto& th : pool) th.join();
    return 0;
}

// The reference's unified backend entry point (max-3-phase orchestration),
// returning only the published status and phase count per cell; used for
// timing and to count cells that leave the two-phase path.
int ref_backend_batch(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                      int64_t ncell, const double* p, const double* t, const double* z, int threads,
                      int32_t* status, int32_t* phase_count) {
    std::vector<std::string> order;
    const th::PrParameterSet params = make_parameters(n, tc, pc, omega, kij, order);
    const auto model = th::Pr76Phase<double>::from_parameters(params);
    auto run = [&](int64_t lo, int64_t hi) {
        fl::Pr76VleEvaluator evaluator(model);
        fl::Pr76PtFlashBackend backend(evaluator);
        for (int64_t c = lo; c < hi; ++c) {
            fl::PtFlashRequest req;
            req.pressure_pa = p[c];
            req.temperature_k = t[c];
            req.feed.resize(n);
            for (int i = 0; i < n; ++i) req.feed[i] = z[i * ncell + c];
            try {
                const auto r = backend.solve(req);
                status[c] = static_cast<int32_t>(r.solution.status);
                phase_count[c] = static_cast<int32_t>(r.solution.accepted_phase_count());
            } catch (const std::exception&) {
                status[c] = -1;
                phase_count[c] = 0;
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

// Outputs of the max-3-phase orchestration per cell (layouts a[k * ncell + c];
// phase-major for the three-phase fields: phase q, component i at
// (q * n + i) * ncell + c).
struct Max3Outputs {
    int32_t* max3_status;  // Pr76PtMax3Status: 0 single, 1 two, 2 three, 3 boundary unresolved,
                           // 4 higher phase count or wrong candidate, 5 indeterminate
    int32_t* published;    // 0 single, 1 two, 2 phase set unstable, 3 indeterminate, 4 three, -1 invalid
    double* beta3;         // [3] phase fractions of the accepted three-phase set
    double* x3;            // [3 * n] compositions
    double* lnphi3;        // [3 * n]
    double* z3;            // [3]
    double* beta;          // two-phase pair published for status two / higher (vapor fraction)
    double* x;             // [n]
    double* y;             // [n]
    int32_t* attempts;     // three-phase attempts run
};

// Caller starts and options of solve_pr76_pt_max3 (the oracle's StartHints):
// compositions cell-fastest, composition k of cell c, component i at
// (k * n + i) * ncell + c.
struct StartHints {
    const int32_t* initial_count;
    const double* initial_x;
    const int32_t* final_count;
    const double* final_x;
    const int32_t* three_phase;
    const double* three_x;
    const double* fraction;
    int32_t initial_automatic_starts;
    int32_t max_split_attempts;
};

static std::vector<std::vector<double>> hint_set(const int32_t* count, const double* x, int n, int64_t ncell,
                                                 int64_t c) {
    std::vector<std::vector<double>> out;
    if (!count || !x) return out;
    const int k = std::min(3, std::max(0, static_cast<int>(count[c])));
    for (int q = 0; q < k; ++q) {
        std::vector<double> w(n);
        for (int i = 0; i < n; ++i) w[i] = x[(static_cast<int64_t>(q) * n + i) * ncell + c];
        out.push_back(std::move(w));
    }
    return out;
}

static int max3_batch(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                      int64_t ncell, const double* p, const double* t, const double* z, int threads,
                      const Max3Outputs* o, const StartHints* h) {
    std::vector<std::string> order;
    const th::PrParameterSet params = make_parameters(n, tc, pc, omega, kij, order);
    const auto model = th::Pr76Phase<double>::from_parameters(params);
    const double nan = std::numeric_limits<double>::quiet_NaN();
    auto run = [&](int64_t lo, int64_t hi) {
        fl::Pr76VleEvaluator evaluator(model);
        for (int64_t c = lo; c < hi; ++c) {
            fl::Pr76PtMax3Options options;
            std::vector<std::vector<double>> init, fin;
            if (h) {
                options.two_phase.initial_stability.automatic_starts = h->initial_automatic_starts != 0;
                options.two_phase.max_split_attempts = static_cast<std::size_t>(h->max_split_attempts);
                init = hint_set(h->initial_count, h->initial_x, n, ncell, c);
                fin = hint_set(h->final_count, h->final_x, n, ncell, c);
                if (h->three_phase && h->three_x && h->fraction && h->three_phase[c]) {
                    fl::Pr76PtThreePhaseStart st;
                    for (int q = 0; q < 3; ++q) {
                        st.compositions[q].resize(n);
                        for (int i = 0; i < n; ++i)
                            st.compositions[q][i] = h->three_x[(static_cast<int64_t>(q) * n + i) * ncell + c];
                    }
                    st.phase_fraction_seed = {h->fraction[c], h->fraction[ncell + c]};
                    options.three_phase_starts.push_back(std::move(st));
                }
            }
            auto put = [&](double* arr, int k, double v) {
                if (arr) arr[k * ncell + c] = v;
            };
            for (int k = 0; k < 3; ++k) {
                put(o->beta3, k, nan);
                put(o->z3, k, nan);
                for (int i = 0; i < n; ++i) {
                    put(o->x3, k * n + i, nan);
                    put(o->lnphi3, k * n + i, nan);
                }
            }
            put(o->beta, 0, nan);
            for (int i = 0; i < n; ++i) {
                put(o->x, i, nan);
                put(o->y, i, nan);
            }
            std::vector<double> feed(n);
            for (int i = 0; i < n; ++i) feed[i] = z[i * ncell + c];
            fl::Pr76PtMax3Result r;
            try {
                r = fl::solve_pr76_pt_max3(p[c], t[c], feed, evaluator, options, init, fin);
            } catch (const std::exception&) {
                if (o->max3_status) o->max3_status[c] = -1;
                if (o->published) o->published[c] = -1;
                if (o->attempts) o->attempts[c] = 0;
                continue;
            }
            const int ms = static_cast<int>(r.status);
            if (o->max3_status) o->max3_status[c] = ms;
            if (o->attempts) o->attempts[c] = static_cast<int32_t>(r.attempts.size());
            const fl::PtSplitState* pair = nullptr;
            int pub = 3;
            switch (r.status) {
            case fl::Pr76PtMax3Status::single_phase: pub = 0; break;
            case fl::Pr76PtMax3Status::two_phase: {
                const auto* nb = r.two_phase_neighbor();
                pair = nb ? nb->solution.candidate() : r.base.solution.candidate();
                pub = 1;
                break;
            }
            case fl::Pr76PtMax3Status::three_phase: pub = 4; break;
            case fl::Pr76PtMax3Status::higher_phase_count_or_wrong_candidate:
                pair = r.base.solution.candidate();
                pub = 2;
                break;
            default: pub = 3; break;
            }
            if (o->published) o->published[c] = pub;
            if (pair) {
                put(o->beta, 0, pair->fractions.vapor_fraction);
                for (int i = 0; i < n; ++i) {
                    put(o->x, i, pair->fractions.liquid[i]);
                    put(o->y, i, pair->fractions.vapor[i]);
                }
            }
            if (const auto* cand = r.three_phase_candidate()) {
                for (int k = 0; k < 3; ++k) {
                    const auto& ph = cand->phases[k];
                    put(o->beta3, k, ph.mole_phase_fraction);
                    put(o->z3, k, ph.z);
                    for (int i = 0; i < n; ++i) {
                        put(o->x3, k * n + i, ph.composition[i]);
                        put(o->lnphi3, k * n + i, ph.activity.ln_phi[i]);
                    }
                }
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

int ref_max3_batch(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                   int64_t ncell, const double* p, const double* t, const double* z, int threads,
                   const Max3Outputs* o) {
    return max3_batch(n, tc, pc, omega, kij, ncell, p, t, z, threads, o, nullptr);
}

// ref_max3_batch with caller starts and options (StartHints).
int ref_max3_hinted_batch(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                          int64_t ncell, const double* p, const double* t, const double* z, const StartHints* hints,
                          int threads, const Max3Outputs* o) {
    if (!hints) return -1;
    return max3_batch(n, tc, pc, omega, kij, ncell, p, t, z, threads, o, hints);
}

// The reference's ordered-path continuation (default options: previous phase
// compositions and three-phase state carried as hints) of npath feeds, each
// along its own npoint states; per point the max3 status and the published
// status (codes of ref_max3_batch).  p, t are [npath * npoint] path-major,
// z is [n * npath].
int ref_continuation_batch(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                           int64_t npath, int64_t npoint, const double* p, const double* t, const double* z,
                           int threads, int32_t* max3_status, int32_t* published) {
    std::vector<std::string> order;
    const th::PrParameterSet params = make_parameters(n, tc, pc, omega, kij, order);
    const auto model = th::Pr76Phase<double>::from_parameters(params);
    auto run = [&](int64_t lo, int64_t hi) {
        fl::Pr76VleEvaluator evaluator(model);
        for (int64_t path = lo; path < hi; ++path) {
            std::vector<fl::Pr76PtPathState> states(static_cast<size_t>(npoint));
            for (int64_t k = 0; k < npoint; ++k) states[k] = {p[path * npoint + k], t[path * npoint + k]};
            std::vector<double> feed(n);
            for (int i = 0; i < n; ++i) feed[i] = z[i * npath + path];
            try {
                const auto r = fl::solve_pr76_pt_continuation(states, feed, evaluator);
                for (int64_t k = 0; k < npoint; ++k) {
                    const auto& pt = r.points[static_cast<size_t>(k)];
                    const int ms = static_cast<int>(pt.solve.status);
                    int pub = 3;
                    switch (pt.solve.status) {
                    case fl::Pr76PtMax3Status::single_phase: pub = 0; break;
                    case fl::Pr76PtMax3Status::two_phase: pub = 1; break;
                    case fl::Pr76PtMax3Status::three_phase: pub = 4; break;
                    case fl::Pr76PtMax3Status::higher_phase_count_or_wrong_candidate: pub = 2; break;
                    default: pub = 3; break;
                    }
                    max3_status[path * npoint + k] = ms;
                    published[path * npoint + k] = pub;
                }
            } catch (const std::exception&) {
                for (int64_t k = 0; k < npoint; ++k) {
                    max3_status[path * npoint + k] = -1;
                    published[path * npoint + k] = -1;
                }
            }
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

// The reference backend's transition report (project_pr76_pt_max3_transition_report,
// modules/flash/include/mpmc/flash/pr76_pt_flash_backend.hpp:94-175) of each
// cell, with its published status (0 single, 1 two, 2 unstable, 3
// indeterminate, 4 three) and max3 status.  Evidence k of cell c occupies
// evidence[(c * 8 + k) * 6 ..]: source, target (0 = none), trigger,
// resolution, fresh target solve attempted, target topology closed; count[c]
// evidence entries (at most 8).
int ref_transition_reports(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                           int64_t ncell, const double* p, const double* t, const double* z, int32_t* published,
                           int32_t* max3_status, int32_t* count, int32_t* evidence) {
    std::vector<std::string> order;
    const th::PrParameterSet params = make_parameters(n, tc, pc, omega, kij, order);
    const auto model = th::Pr76Phase<double>::from_parameters(params);
    fl::Pr76VleEvaluator evaluator(model);
    for (int64_t c = 0; c < ncell; ++c) {
        std::vector<double> feed(n);
        for (int i = 0; i < n; ++i) feed[i] = z[i * ncell + c];
        count[c] = -1;
        try {
            const auto source = fl::solve_pr76_pt_max3(p[c], t[c], feed, evaluator);
            const auto set = fl::project_pr76_pt_max3_phase_set(source);
            const auto report = fl::project_pr76_pt_max3_transition_report(source);
            int pub = 3;
            if (set.solution.status == fl::PtPhaseSetStatus::accepted && set.solution.candidate_phase_set) {
                const auto k = set.solution.candidate_phase_set->phases.size();
                pub = k == 1 ? 0 : (k == 2 ? 1 : 4);
            } else if (set.solution.status == fl::PtPhaseSetStatus::phase_set_unstable) {
                pub = 2;
            }
            published[c] = pub;
            max3_status[c] = static_cast<int32_t>(source.status);
            count[c] = static_cast<int32_t>(std::min<std::size_t>(report.evidence.size(), 8));
            for (int k = 0; k < count[c]; ++k) {
                const auto& e = report.evidence[k];
                int32_t* row = evidence + (c * 8 + k) * 6;
                row[0] = static_cast<int32_t>(e.source_phase_count);
                row[1] = e.target_phase_count ? static_cast<int32_t>(*e.target_phase_count) : 0;
                row[2] = static_cast<int32_t>(e.trigger);
                row[3] = static_cast<int32_t>(e.resolution);
                row[4] = e.fresh_target_solve_attempted ? 1 : 0;
                row[5] = e.target_topology_closed ? 1 : 0;
            }
        } catch (const std::exception&) {
            published[c] = -1;
            max3_status[c] = -1;
        }
    }
    return 0;
}

// The reference's selected-phase property chart of `ncell` cells with the
// affine transport/caloric provider of the C ABI (the same arithmetic order as
// oracle::affine_model).  Layouts and status codes as
// oracle_property_chart_batch; 7 = an unexpected exception.
int ref_property_chart_batch(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                             int phases, const int* root_index, const double* molar_mass, const double* visc,
                             const double* enth, int64_t ncell, const double* q, const int* dep, int threads,
                             int* status, double* values, double* jac) {
    namespace fw = mpmc::flow;
    std::vector<std::string> order;
    const th::PrParameterSet params = make_parameters(n, tc, pc, omega, kij, order, molar_mass);
    const auto model = th::Pr76Phase<double>::from_parameters(params);
    const std::vector<double> cv(visc, visc + 7 + n), ce(enth, enth + 7 + n);
    const auto provider = [cv, ce](const th::Pr76SelectedPhase& selection, const auto& p, const auto& t,
                                   auto x, const auto& mm, const auto& rho, const auto& rhom) {
        using Number = std::decay_t<decltype(p)>;
        auto affine = [&](const std::vector<double>& c) {
            Number f = Number{c[0]} + p * c[1] + t * c[2];
            for (size_t i = 0; i < x.size(); ++i) f += x[i] * c[7 + i];
            return f + rho * c[3] + mm * c[4] + rhom * c[5] + Number{c[6] * static_cast<double>(selection.root_index)};
        };
        return fw::SelectedPhaseTransportCaloricValues<Number>{affine(cv), affine(ce)};
    };
    std::vector<th::Pr76SelectedPhase> selections;
    for (int k = 0; k < phases; ++k) selections.push_back({static_cast<std::size_t>(root_index[k]), {}});
    const fw::SelectedPhasePropertyProvenance provenance{{"affine test model", "mpmc-gb300-synthetic", "v1"},
                                                         {"affine test model", "mpmc-gb300-synthetic", "v1"},
                                                         {"affine test model", "mpmc-gb300-synthetic", "v1"},
                                                         {"u = h - p/rho_mass", "mpmc-gb300-synthetic", "v1"}};
    const auto closure = fw::make_pr76_selected_phase_property_closure(model, selections, provider, provenance);
    const int cols = phases * n + 1;
    const int rows = phases * (5 + n) + (phases - 1) * n;
    const double nan = std::numeric_limits<double>::quiet_NaN();
    auto classify = [](const std::exception& e) {
        const std::string what = e.what();
        auto has = [&](const char* s) { return what.find(s) != std::string::npos; };
        if (has("mpmc::ad::runtime: nonfinite input")) return 1;
        if (has("mpmc::ad::runtime:")) return 6;
        if (has("mpmc::flow: PR76 selected-phase")) {
            if (has("composition") || has("pressure [Pa]") || has("temperature [K]") || has("molar mass"))
                return 1;
            return 6;
        }
        return 2;
    };
    auto run = [&](int64_t lo, int64_t hi) {
        mpmc::ad::RuntimeJacobianWorkspace<double, 4U> workspace;
        std::vector<double> qc(cols);
        for (int64_t c = lo; c < hi; ++c) {
            for (int k = 0; k < cols; ++k) qc[k] = q[k * ncell + c];
            std::vector<std::size_t> pivots(phases);
            for (int k = 0; k < phases; ++k) pivots[k] = dep ? static_cast<std::size_t>(dep[k * ncell + c]) : n - 1;
            int st = 0;
            try {
                const fw::NaturalVariableLayoutDescriptor layout(static_cast<std::size_t>(n),
                                                                 static_cast<std::size_t>(phases), pivots);
                const auto r = fw::evaluate_pr76_selected_phase_property_chart(layout, closure.component_ids(), qc,
                                                                               closure, workspace);
                for (int ph = 0; ph < phases; ++ph) {
                    const int base = ph * (5 + n);
                    const auto& pp = r.phase_properties[ph];
                    const double v5[5] = {pp.molar_density_mol_per_m3, pp.mass_density_kg_per_m3,
                                          pp.dynamic_viscosity_pa_s, pp.specific_enthalpy_j_per_kg,
                                          pp.specific_internal_energy_j_per_kg};
                    const std::vector<double>* g5[5] = {&r.molar_density_gradient[ph], &r.mass_density_gradient[ph],
                                                        &r.viscosity_gradient[ph], &r.enthalpy_gradient[ph],
                                                        &r.internal_energy_gradient[ph]};
                    for (int k = 0; k < 5; ++k) {
                        if (values) values[(base + k) * ncell + c] = v5[k];
                        if (jac)
                            for (int col = 0; col < cols; ++col)
                                jac[(static_cast<int64_t>(base + k) * cols + col) * ncell + c] = (*g5[k])[col];
                    }
                    for (int i = 0; i < n; ++i) {
                        if (values) values[(base + 5 + i) * ncell + c] = r.ln_phi[ph][i];
                        if (jac)
                            for (int col = 0; col < cols; ++col)
                                jac[(static_cast<int64_t>(base + 5 + i) * cols + col) * ncell + c] =
                                    r.ln_phi_jacobian[ph][static_cast<size_t>(i) * cols + col];
                    }
                }
                const int prop = phases * (5 + n);
                for (int e = 0; e < (phases - 1) * n; ++e) {
                    if (values) values[(prop + e) * ncell + c] = r.equilibrium_residual[e];
                    if (jac)
                        for (int col = 0; col < cols; ++col)
                            jac[(static_cast<int64_t>(prop + e) * cols + col) * ncell + c] =
                                r.equilibrium_jacobian[static_cast<size_t>(e) * cols + col];
                }
            } catch (const th::Pr76PhaseError& e) {
                st = e.code() == th::Pr76PhaseErrorCode::ill_conditioned_derivative ? 5 : 3;
            } catch (const std::out_of_range&) {
                st = 4;
            } catch (const std::range_error& e) {
                st = classify(e);
            } catch (const std::domain_error& e) {
                st = classify(e);
            } catch (const std::invalid_argument& e) {
                st = classify(e);
            } catch (const std::exception&) {
                st = 7;
            }
            if (status) status[c] = st;
            if (st != 0)
                for (int r = 0; r < rows; ++r) {
                    if (values) values[r * ncell + c] = nan;
                    if (jac)
                        for (int col = 0; col < cols; ++col) jac[(static_cast<int64_t>(r) * cols + col) * ncell + c] = nan;
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

}  // extern "C"
