"""The reference-side C++ bindings compile against the reference's own
interfaces: mpmc_hnu_gb300/cpp/gpu_pr76_pt_flash_backend.hpp as a
PtFlashBackend, mpmc_hnu_gb300/cpp/gpu_pr76_pt_continuation.hpp with the
reference's continuation types, and mpmc_hnu_gb300/cpp/gpu_pr76_selected_phase_property_chart.hpp
beside the reference's flow property closure (its affine provider also
instantiates the reference's own CPU closure and chart).

Needs the reference's headers (present where the oracle's reference harness is
built); skipped elsewhere.  Compile only: no GPU is touched.
"""

import os
import shutil
import subprocess

import pytest

from oracle import pyoracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REFERENCE = pyoracle.REFERENCE_ROOT
MODULES = ("ad", "thermodynamics", "flash", "physics", "flow", "mesh")

SOURCE = r"""
#include "gpu_pr76_pt_flash_backend.hpp"
#include "gpu_pr76_pt_continuation.hpp"
std::vector<mpmc::flash::GpuPr76PtContinuationResult> scan(
    mpmc_gpu_flash* h, std::span<const std::vector<mpmc::flash::Pr76PtPathState>> paths,
    std::span<const std::vector<double>> feeds) {
    return mpmc::flash::solve_gpu_pr76_pt_continuation(h, paths, feeds);
}
#include <memory>
#include <type_traits>
static_assert(std::is_base_of_v<mpmc::flash::PtFlashBackend, mpmc::flash::GpuPr76PtFlashBackend>);
std::unique_ptr<mpmc::flash::PtFlashBackend> make(const mpmc::flash::GpuPr76Mixture& m) {
    return std::make_unique<mpmc::flash::GpuPr76PtFlashBackend>(m);
}
"""


CHART_SOURCE = r"""
#include "gpu_pr76_selected_phase_property_chart.hpp"
#include "gpu_post_snes_pt_flash_scan.hpp"
#include <memory>
mpmc::flow::ScanSummary scan(std::span<const mpmc::flow::ScanSourceCell> cells,
                             mpmc::flash::GpuPr76PtFlashBackend& gpu) {
    auto r = mpmc::flow::scan_pt_flash_source_cells_batched(
        cells, gpu, [](const mpmc::flash::PtFlashBackendResult&, std::optional<std::vector<double>>*) { return 0; });
    return mpmc::flow::summarize(cells, r);
}
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
def test_flow_bindings_compile_against_reference_flow_module(tmp_path):
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


@pytest.mark.skipif(not os.path.isdir(os.path.join(REFERENCE, "modules", "flash", "include")),
                    reason="reference headers not present")
@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_transition_report_matches_reference(tmp_path, oracle_lib):
    """The binding's transition report for each published status equals the
    reference backend's project_pr76_pt_max3_transition_report on the same
    cells (source, target, trigger, resolution, fresh solve, closed), except
    for indeterminate results, which the binding leaves without evidence."""
    import ctypes

    import numpy as np

    from mpmc_hnu_gb300 import synth

    if not oracle_lib.reference_available():
        pytest.skip("reference harness not built")
    so = str(tmp_path / "libreport_host.so")
    cmd = ["g++", "-std=c++20", "-O1", "-fPIC", "-shared", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "mpmc_hnu_gb300", "cpp")]
    cmd += ["-I" + os.path.join(REFERENCE, "modules", m, "include") for m in MODULES]
    subprocess.check_call(cmd + [os.path.join(ROOT, "tests", "host_build", "report_host.cpp"), "-o", so])
    ours = ctypes.CDLL(so)
    ref = ctypes.CDLL(oracle_lib.REF_SO)
    d = np.load(os.path.join(ROOT, "tests", "golden", "max3_reference.npz"))
    cases = [(synth.three_phase_fixture_mixture(), d["p"][::2], d["t"][::2], d["z"][:, ::2])]
    mix10 = synth.make_mixture(10, 1001)
    p10, t10, z10 = synth.make_cells(10, 300, 2001)
    cases.append((mix10, p10, t10, z10))
    seen = set()
    for mix, p, t, z in cases:
        tc, pc, om, kij = (np.ascontiguousarray(a, dtype=np.float64) for a in mix.as_tuple())
        p, t, z = (np.ascontiguousarray(a, dtype=np.float64) for a in (p, t, z))
        n, ncell = z.shape
        pub = np.empty(ncell, np.int32)
        m3 = np.empty(ncell, np.int32)
        cnt = np.empty(ncell, np.int32)
        ev = np.zeros((ncell, 8, 6), np.int32)
        ref.ref_transition_reports(ctypes.c_int(n), *[ctypes.c_void_p(a.ctypes.data) for a in (tc, pc, om, kij)],
                                   ctypes.c_int64(ncell), *[ctypes.c_void_p(a.ctypes.data) for a in (p, t, z)],
                                   *[ctypes.c_void_p(a.ctypes.data) for a in (pub, m3, cnt, ev)])
        for c in range(ncell):
            assert cnt[c] >= 0
            mine = np.zeros((8, 6), np.int32)
            k = ours.our_transition_report(ctypes.c_int32(int(pub[c])), ctypes.c_int32(int(m3[c])),
                                           ctypes.c_void_p(mine.ctypes.data))
            seen.add((int(pub[c]), int(m3[c])))
            if pub[c] == 3 and m3[c] == 5:
                assert k == 0
                continue
            assert k == cnt[c] and np.array_equal(mine[:k], ev[c, :k]), (c, int(pub[c]), int(m3[c]))
    assert {(0, 0), (1, 1), (4, 2), (2, 4)} <= seen


SCAN_EXPECTED = {
    # a cell already in its accepted phase count proposes nothing
    "steady": "cells complete:0 complete:0 summary complete 2 0",
    # a one-phase source cell that flashes to two phases proposes 1 -> 2
    "appear": "cells complete:0 complete:2 complete:0 summary complete 3 0 proposal 2 1->2",
    # the PR76 backend publishes no disappearance evidence for 2 -> 1, so the
    # reference's candidate adapter rejects it (std::invalid_argument)
    "vanish": "cells complete:0 incompatible:0 summary incompatible 1 0",
    "malformed": "cells complete:2 incompatible:0 summary incompatible 1 0",
    "no_density": "cells indeterminate:0 summary indeterminate 0 0",
    "resolver": "cells complete:0 resolver_error:0 summary resolver_error 1 42",
    # the first cell that is not complete decides, as the loop's early return does
    "indeterminate_first": "cells indeterminate:0 incompatible:0 complete:0 summary indeterminate 0 0",
}


@pytest.mark.skipif(not os.path.isdir(os.path.join(REFERENCE, "modules", "flow", "include")),
                    reason="reference headers not present")
@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_batched_scan_follows_the_reference_rules(tmp_path):
    """mpmc_hnu_gb300/cpp/gpu_post_snes_pt_flash_scan.hpp over the reference's
    own Pr76PtFlashBackend (tests/host_build/scan_host.cpp) on a methane /
    n-butane mixture: per-cell statuses, proposals and the loop verdict of the
    reference scanner (post_snes_pt_flash_phase_transition_scanner.hpp:207-421)
    in each scenario."""
    exe = str(tmp_path / "scan_host")
    cmd = ["g++", "-std=c++20", "-O1", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "mpmc_hnu_gb300", "cpp")]
    cmd += ["-I" + os.path.join(REFERENCE, "modules", m, "include") for m in MODULES]
    subprocess.check_call(cmd + [os.path.join(ROOT, "tests", "host_build", "scan_host.cpp"), "-o", exe])
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.splitlines()
    got = {line.split(" ", 1)[0]: line.split(" ", 1)[1] for line in out}
    assert got == SCAN_EXPECTED


@pytest.mark.skipif(not os.path.isdir(os.path.join(REFERENCE, "tests", "flash", "pr76_three_phase")),
                    reason="reference tests not present")
@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_seeded_backend_binding_matches_reference(tmp_path):
    """GpuPr76PtFlashBackend with caller starts (GpuPr76BackendStarts) over the
    host build of the device code, beside the reference's seeded
    Pr76PtFlashBackend in the reference's own seeded-backend scenario
    (pr76_max3_seeded_backend_test.cpp): both accept three phases with the
    same compositions and publish the 2 -> 3 evidence."""
    exe = str(tmp_path / "seeded_backend")
    cmd = ["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-Wno-attributes", "-I/usr/local/cuda/include",
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "mpmc_hnu_gb300", "csrc"),
           "-I" + os.path.join(ROOT, "mpmc_hnu_gb300", "cpp"),
           "-I" + os.path.join(REFERENCE, "tests", "flash", "pr76_three_phase")]
    cmd += ["-I" + os.path.join(REFERENCE, "modules", m, "include") for m in ("ad", "thermodynamics", "flash",
                                                                               "physics")]
    subprocess.check_call(cmd + [os.path.join(ROOT, "tests", "host_build", "seeded_backend.cpp"),
                                 os.path.join(ROOT, "tests", "host_build", "flash_host.cpp"), "-o", exe])
    ref_status, got_status, ref_phases, got_phases, worst, ref_23, got_23 = \
        subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    assert ref_status == got_status == "0" and ref_phases == got_phases == "3"
    assert float(worst) <= 1e-12
    assert ref_23 == got_23 == "1"


@pytest.mark.skipif(not os.path.isdir(os.path.join(REFERENCE, "modules", "flash", "include")),
                    reason="reference headers not present")
@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_backend_binding_takes_the_reference_options(tmp_path):
    """GpuPr76PtFlashBackend built from the reference's own
    Pr76PtFlashBackendOptions (gpu_starts_from) over the host build of the
    device code, beside the reference's Pr76PtFlashBackend with the same
    options, on the recorded hinted cases (tests/golden/max3_hinted_reference.npz):
    the 3 -> 2 recovery through a phase disappearance (initial starts without
    the automatic ones, 2 split attempts, separate final and three-phase
    starts) and the zero split-attempt quota.  Same status, same phase count,
    compositions within 1e-12."""
    import numpy as np

    from tests.test_oracle_max3 import hinted_cases

    exe = str(tmp_path / "options_backend")
    cmd = ["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-Wno-attributes", "-I/usr/local/cuda/include",
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "mpmc_hnu_gb300", "csrc"),
           "-I" + os.path.join(ROOT, "mpmc_hnu_gb300", "cpp")]
    cmd += ["-I" + os.path.join(REFERENCE, "modules", m, "include") for m in ("ad", "thermodynamics", "flash",
                                                                               "physics", "flow", "mesh")]
    subprocess.check_call(cmd + [os.path.join(ROOT, "tests", "host_build", "options_backend.cpp"),
                                 os.path.join(ROOT, "tests", "host_build", "flash_host.cpp"), "-o", exe,
                                 "-lpthread"])
    cases = hinted_cases()
    for name in ("recovery", "budget", "three"):
        mix, z, h, ref = cases[name]
        n = z.shape[0]

        def comps(count_key, comp_key):
            k = int(np.ravel(h[count_key])[0])
            return [np.asarray(h[comp_key])[q * n:(q + 1) * n, 0] for q in range(k)]

        vals = [n, *mix.tc, *mix.pc, *mix.omega, *np.asarray(mix.kij).ravel(), 1e6, 250.0, *z[:, 0]]
        for key in (("initial_count", "initial_composition"), ("final_count", "final_composition")):
            sts = comps(*key)
            vals += [len(sts)] + [v for w in sts for v in w]
        three = int(np.ravel(h["three_phase"])[0])
        vals.append(three)
        if three:
            vals += list(np.asarray(h["three_phase_composition"])[:, 0]) + list(np.asarray(h["fraction"])[:, 0])
        vals += [1.0 if h["initial_automatic_starts"] else 0.0, float(h["max_split_attempts"])]
        inp = tmp_path / f"{name}.bin"
        inp.write_bytes(np.asarray(vals, dtype=np.float64).tobytes())
        out = subprocess.run([exe, str(inp)], capture_output=True, text=True, check=True).stdout.split()
        ref_status, got_status, ref_phases, got_phases, worst = out
        assert ref_status == got_status, (name, out)
        assert ref_phases == got_phases, (name, out)
        if int(ref_phases) > 0:
            assert float(worst) <= 1e-12, (name, out)
        if name == "recovery":
            assert ref_phases == "2"
