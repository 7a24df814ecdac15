// Reference-side binding of the GB300 selected-phase property chart: the
// flow module's evaluate_pr76_selected_phase_property_chart
// (modules/flow/include/mpmc/flow/pr76_selected_phase_property_closure.hpp:533-822)
// on many cells per device call, through the C ABI of include/mpmc_gb300_flash.h
// (mpmc_gpu_flash_property_chart).
//
// A maintainer adds this header to a build of MPMC_HNU's flow module and
// evaluates the cells of a frozen closure in one call where the production
// cell evaluators call the chart once per cell
// (Pr76ProductionCellEvaluatorTraits::evaluate_property_chart,
// modules/flow/discretization/petsc/include/mpmc/flow_discretization_petsc/
// pr76_production_cell_evaluator.hpp:88-101).  evaluate() keeps the per-cell
// signature and exception classes of the reference function, so it also
// drops into those traits unchanged.
//
// The closure is the reference's Pr76SelectedPhasePropertyClosure with an
// AffineTransportCaloricProvider (below) as its viscosity/enthalpy provider:
// the device evaluates that model.  The same provider object builds the
// reference's own CPU closure, so a caller can compare the two on its states.
//
// Status -> exception (the classes the reference throws, which the
// production traits map to domain_error or PETSC_ERR_PLIB,
// pr76_production_cell_evaluator.hpp:42-86):
//   MPMC_CHART_INPUT_DOMAIN, MPMC_CHART_PROPERTY_DOMAIN -> std::range_error
//   MPMC_CHART_EOS_DOMAIN                               -> std::domain_error
//   MPMC_CHART_ROOT_UNRESOLVED                          -> Pr76PhaseError (unrepresentable_root)
//   MPMC_CHART_ROOT_INDEX                               -> std::out_of_range
//   MPMC_CHART_ILL_CONDITIONED                          -> Pr76PhaseError (ill_conditioned_derivative)
// A device failure throws std::runtime_error.  Not reentrant: one instance
// per simultaneous caller.
#pragma once

#include <mpmc/flow/pr76_selected_phase_property_closure.hpp>

#include <cstdint>
#include <span>
#include <stdexcept>
#include <string>
#include <vector>

#include "gpu_pr76_pt_flash_backend.hpp"
#include "mpmc_gb300_flash.h"

namespace mpmc::flow {

// f = c[0] + c[1] p + c[2] T + sum_i c[7+i] x_i + c[3] rho + c[4] M + c[5] rho_mass
//     + c[6] root_index, for the viscosity and for the enthalpy: the
// provider slot of Pr76SelectedPhasePropertyClosure (:258-270) in the form
// the device evaluates.
struct AffineTransportCaloricProvider {
    std::vector<double> viscosity;  // [7 + n]
    std::vector<double> enthalpy;   // [7 + n]

    template <typename Number>
    [[nodiscard]] SelectedPhaseTransportCaloricValues<Number> operator()(
        const thermodynamics::Pr76SelectedPhase& selection, const Number& pressure_pa, const Number& temperature_k,
        std::span<const Number> composition, const Number& mixture_molar_mass, const Number& molar_density,
        const Number& mass_density) const {
        auto affine = [&](const std::vector<double>& c) {
            Number f = Number{c[0]} + pressure_pa * c[1] + temperature_k * c[2];
            for (std::size_t i = 0; i < composition.size(); ++i) f += composition[i] * c[7 + i];
            return f + molar_density * c[3] + mixture_molar_mass * c[4] + mass_density * c[5] +
                   Number{c[6] * static_cast<double>(selection.root_index)};
        };
        return {affine(viscosity), affine(enthalpy)};
    }
};

class GpuPr76SelectedPhasePropertyChart {
public:
    GpuPr76SelectedPhasePropertyChart(const flash::GpuPr76Mixture& mixture,
                                      std::vector<thermodynamics::Pr76SelectedPhase> selections,
                                      std::vector<double> molar_mass, AffineTransportCaloricProvider provider,
                                      SelectedPhasePropertyProvenance provenance, int device = 0)
        : n_(mixture.component_ids.size()),
          component_ids_(mixture.component_ids),
          selections_(std::move(selections)),
          molar_mass_(std::move(molar_mass)),
          provider_(std::move(provider)),
          provenance_(std::move(provenance)) {
        if (selections_.empty() || selections_.size() > fixed_three_phase_count)
            throw std::invalid_argument("GPU PR76 property chart: 1..3 frozen selections required");
        if (n_ < 2) throw std::invalid_argument("GPU PR76 property chart: at least two components required");
        if (molar_mass_.size() != n_ || provider_.viscosity.size() != 7 + n_ || provider_.enthalpy.size() != 7 + n_)
            throw std::invalid_argument("GPU PR76 property chart: molar masses or model coefficients mis-sized");
        pr76_selected_phase_property_detail::validate_provenance(provenance_);
        if (mixture.critical_temperature_k.size() != n_ || mixture.critical_pressure_pa.size() != n_ ||
            mixture.acentric_factor.size() != n_ || mixture.kij.size() != n_ * n_)
            throw std::invalid_argument("GPU PR76 property chart: mixture arrays do not match the component list");
        mpmc_pr76_mixture m{static_cast<int32_t>(n_), mixture.critical_temperature_k.data(),
                            mixture.critical_pressure_pa.data(), mixture.acentric_factor.data(), mixture.kij.data()};
        mpmc_flash_options o{MPMC_FORM_PLAIN_FP64, 0, device, 0};
        check(mpmc_gpu_flash_create(&m, &o, &handle_));
        spec_.phase_count = static_cast<int32_t>(selections_.size());
        for (std::size_t k = 0; k < selections_.size(); ++k)
            spec_.root_index[k] = static_cast<int32_t>(selections_[k].root_index);
        spec_.molar_mass = molar_mass_.data();
        spec_.viscosity = provider_.viscosity.data();
        spec_.enthalpy = provider_.enthalpy.data();
    }

    GpuPr76SelectedPhasePropertyChart(const GpuPr76SelectedPhasePropertyChart&) = delete;
    GpuPr76SelectedPhasePropertyChart& operator=(const GpuPr76SelectedPhasePropertyChart&) = delete;
    ~GpuPr76SelectedPhasePropertyChart() { mpmc_gpu_flash_destroy(handle_); }

    [[nodiscard]] std::size_t phase_count() const noexcept { return selections_.size(); }
    [[nodiscard]] std::span<const std::string> component_ids() const noexcept { return component_ids_; }
    [[nodiscard]] const SelectedPhasePropertyProvenance& provenance() const noexcept { return provenance_; }
    [[nodiscard]] const AffineTransportCaloricProvider& provider() const noexcept { return provider_; }

    // The reference function's per-cell contract: the linearization, or the
    // reference's exception for the cell's status.
    [[nodiscard]] Pr76SelectedPhasePropertyChartLinearization evaluate(
        const NaturalVariableLayoutDescriptor& layout, std::span<const std::string> component_ids,
        std::span<const double> natural_variables) const {
        if (layout.phase_count() != phase_count() || component_ids.size() != n_ ||
            natural_variables.size() != layout.unknown_count())
            throw std::invalid_argument("mpmc::flow: PR76 selected-phase chart shape/cardinality mismatch");
        pr76_selected_phase_property_detail::validate_component_ids(component_ids_, component_ids);
        std::vector<Pr76SelectedPhasePropertyChartLinearization> out;
        const auto status = evaluate_batch(std::span<const NaturalVariableLayoutDescriptor>(&layout, 1),
                                           std::span<const std::span<const double>>(&natural_variables, 1), out);
        raise(status.front());
        return std::move(out.front());
    }

    // Every cell in one device call.  Returns the mpmc_chart_status of each
    // cell; results[c] is filled where it is MPMC_CHART_OK (default-constructed
    // otherwise).
    std::vector<int32_t> evaluate_batch(std::span<const NaturalVariableLayoutDescriptor> layouts,
                                        std::span<const std::span<const double>> natural_variables,
                                        std::vector<Pr76SelectedPhasePropertyChartLinearization>& results) const {
        const std::size_t cells = layouts.size();
        if (natural_variables.size() != cells)
            throw std::invalid_argument("GPU PR76 property chart: one natural-variable vector per layout");
        const std::size_t phases = phase_count();
        const std::size_t q = phases * n_ + 1;
        const std::size_t rows = phases * (5 + n_) + (phases - 1) * n_;
        std::vector<double> qv(q * cells);
        std::vector<int32_t> dep(phases * cells);
        for (std::size_t c = 0; c < cells; ++c) {
            if (layouts[c].phase_count() != phases || layouts[c].component_count() != n_ ||
                natural_variables[c].size() != q)
                throw std::invalid_argument("mpmc::flow: PR76 selected-phase chart shape/cardinality mismatch");
            for (std::size_t k = 0; k < q; ++k) qv[k * cells + c] = natural_variables[c][k];
            for (std::size_t ph = 0; ph < phases; ++ph)
                dep[ph * cells + c] =
                    static_cast<int32_t>(layouts[c].dependent_composition_component(static_cast<PhaseSlot3>(ph)));
        }
        std::vector<int32_t> status(cells);
        std::vector<double> values(rows * cells), jac(rows * q * cells);
        mpmc_property_chart_outputs out{status.data(), values.data(), jac.data()};
        if (cells > 0)
            check(mpmc_gpu_flash_property_chart(handle_, static_cast<int64_t>(cells), &spec_, qv.data(), dep.data(),
                                                &out));
        results.assign(cells, Pr76SelectedPhasePropertyChartLinearization{});
        for (std::size_t c = 0; c < cells; ++c) {
            if (status[c] != MPMC_CHART_OK) continue;
            auto& r = results[c];
            r.layout = layouts[c];
            r.component_ids = component_ids_;
            r.provenance = provenance_;
            auto value = [&](std::size_t row) { return values[row * cells + c]; };
            auto gradient = [&](std::size_t row) {
                std::vector<double> g(q);
                for (std::size_t k = 0; k < q; ++k) g[k] = jac[(row * q + k) * cells + c];
                return g;
            };
            for (std::size_t ph = 0; ph < phases; ++ph) {
                const std::size_t base = ph * (5 + n_);
                r.phase_properties.push_back(
                    PhasePropertyPayload{value(base), value(base + 1), value(base + 2), value(base + 3), value(base + 4)});
                r.phase_compositions.push_back(pr76_selected_phase_property_detail::reconstruct_composition<double>(
                    layouts[c], ph, natural_variables[c]));
                r.molar_density_gradient.push_back(gradient(base));
                r.mass_density_gradient.push_back(gradient(base + 1));
                r.viscosity_gradient.push_back(gradient(base + 2));
                r.enthalpy_gradient.push_back(gradient(base + 3));
                r.internal_energy_gradient.push_back(gradient(base + 4));
                std::vector<double> lnphi(n_), lnphi_jac(n_ * q);
                for (std::size_t i = 0; i < n_; ++i) {
                    lnphi[i] = value(base + 5 + i);
                    const auto g = gradient(base + 5 + i);
                    std::copy(g.begin(), g.end(), lnphi_jac.begin() + static_cast<std::ptrdiff_t>(i * q));
                }
                r.ln_phi.push_back(std::move(lnphi));
                r.ln_phi_jacobian.push_back(std::move(lnphi_jac));
            }
            const std::size_t prop = phases * (5 + n_);
            for (std::size_t e = 0; e < (phases - 1) * n_; ++e) {
                r.equilibrium_residual.push_back(value(prop + e));
                const auto g = gradient(prop + e);
                r.equilibrium_jacobian.insert(r.equilibrium_jacobian.end(), g.begin(), g.end());
            }
        }
        return status;
    }

    // The reference's exception for a cell status (no-op for MPMC_CHART_OK).
    static void raise(int32_t status) {
        using thermodynamics::Pr76PhaseError;
        using thermodynamics::Pr76PhaseErrorCode;
        switch (status) {
        case MPMC_CHART_OK: return;
        case MPMC_CHART_INPUT_DOMAIN:
            throw std::range_error("mpmc::flow: PR76 selected-phase chart input must be finite and strictly positive");
        case MPMC_CHART_EOS_DOMAIN: throw std::domain_error("Pr76Phase: state outside the PR76 domain");
        case MPMC_CHART_ROOT_UNRESOLVED:
            throw Pr76PhaseError(Pr76PhaseErrorCode::unrepresentable_root, "Pr76Phase: unresolved root set");
        case MPMC_CHART_ROOT_INDEX: throw std::out_of_range("Pr76Phase: invalid root index");
        case MPMC_CHART_ILL_CONDITIONED:
            throw Pr76PhaseError(Pr76PhaseErrorCode::ill_conditioned_derivative,
                                 "Pr76Phase: selected root has no reliable local derivative");
        default:
            throw std::range_error("mpmc::flow: PR76 selected-phase property is non-finite or non-positive");
        }
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
    std::vector<std::string> component_ids_;
    std::vector<thermodynamics::Pr76SelectedPhase> selections_;
    std::vector<double> molar_mass_;
    AffineTransportCaloricProvider provider_;
    SelectedPhasePropertyProvenance provenance_;
    mpmc_gpu_flash* handle_ = nullptr;
    mpmc_property_chart_spec spec_{};
};

}  // namespace mpmc::flow
