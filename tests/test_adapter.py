"""The reference-side C++ bindings compile against the reference's own
interfaces: mpmc_hnu_gb300/cpp/gpu_pr76_pt_flash_backend.hpp as a
PtFlashBackend, and mpmc_hnu_gb300/cpp/gpu_pr76_selected_phase_property_chart.hpp
beside the reference's flow property closure (its affine provider also
instantiates the reference's own CPU closure and chart).

Needs the reference's headers (present where the oracle's reference harness is
built); skipped elsewhere.  Compile only: no GPU is touched.
"""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REFERENCE = os.environ.get("MPMC_REFERENCE_ROOT", "/root/reference")
MODULES = ("ad", "thermodynamics", "flash", "physics", "flow", "mesh")

SOURCE = r"""
#include "gpu_pr76_pt_flash_backend.hpp"
#include <memory>
#include <type_traits>
static_assert(std::is_base_of_v<mpmc::flash::PtFlashBackend, mpmc::flash::GpuPr76PtFlashBackend>);
std::unique_ptr<mpmc::flash::PtFlashBackend> make(const mpmc::flash::GpuPr76Mixture& m) {
    return std::make_unique<mpmc::flash::GpuPr76PtFlashBackend>(m);
}
"""


CHART_SOURCE = r"""
#include "gpu_pr76_selected_phase_property_chart.hpp"
#include <memory>
namespace fw = mpmc::flow;
std::unique_ptr<fw::GpuPr76SelectedPhasePropertyChart> make(const mpmc::flash::GpuPr76Mixture& m,
                                                             std::vector<double> mm,
                                                             fw::AffineTransportCaloricProvider p,
                                                             fw::SelectedPhasePropertyProvenance prov) {
    return std::make_unique<fw::GpuPr76SelectedPhasePropertyChart>(
        m, std::vector<mpmc::thermodynamics::Pr76SelectedPhase>{{0U, {}}, {2U, {}}}, std::move(mm), std::move(p),
        std::move(prov));
}
fw::Pr76SelectedPhasePropertyChartLinearization one(const fw::GpuPr76SelectedPhasePropertyChart& g,
                                                    const fw::NaturalVariableLayoutDescriptor& layout,
                                                    std::span<const double> q) {
    return g.evaluate(layout, g.component_ids(), q);
}
void cpu(const mpmc::thermodynamics::Pr76Phase<double>& model, fw::AffineTransportCaloricProvider p,
         fw::SelectedPhasePropertyProvenance prov, const fw::NaturalVariableLayoutDescriptor& layout,
         std::span<const double> q) {
    auto c = fw::make_pr76_selected_phase_property_closure(
        model, std::vector<mpmc::thermodynamics::Pr76SelectedPhase>{{0U, {}}}, std::move(p), std::move(prov));
    mpmc::ad::RuntimeJacobianWorkspace<double, 4U> w;
    (void)fw::evaluate_pr76_selected_phase_property_chart(layout, c.component_ids(), q, c, w);
}
"""


@pytest.mark.skipif(not os.path.isdir(os.path.join(REFERENCE, "modules", "flow", "include")),
                    reason="reference headers not present")
@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_chart_binding_compiles_against_reference_flow_module(tmp_path):
    src = tmp_path / "chart_binding_check.cpp"
    src.write_text(CHART_SOURCE)
    cmd = ["g++", "-std=c++20", "-fsyntax-only", "-Wall", "-Wextra", "-Werror",
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "mpmc_hnu_gb300", "cpp")]
    cmd += ["-I" + os.path.join(REFERENCE, "modules", m, "include") for m in MODULES]
    res = subprocess.run(cmd + [str(src)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr


@pytest.mark.skipif(not os.path.isdir(os.path.join(REFERENCE, "modules", "flash", "include")),
                    reason="reference headers not present")
@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_adapter_compiles_against_reference_interface(tmp_path):
    src = tmp_path / "adapter_check.cpp"
    src.write_text(SOURCE)
    cmd = ["g++", "-std=c++20", "-fsyntax-only", "-Wall", "-Wextra", "-Werror",
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "mpmc_hnu_gb300", "cpp")]
    cmd += ["-I" + os.path.join(REFERENCE, "modules", m, "include") for m in MODULES]
    res = subprocess.run(cmd + [str(src)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
