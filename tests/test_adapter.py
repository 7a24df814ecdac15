"""The reference-side C++ binding (mpmc_hnu_gb300/cpp/gpu_pr76_pt_flash_backend.hpp)
compiles against the reference's own PtFlashBackend interface.

Needs the reference's headers (present where the oracle's reference harness is
built); skipped elsewhere.  Compile only: no GPU is touched.
"""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REFERENCE = os.environ.get("MPMC_REFERENCE_ROOT", "/root/reference")
MODULES = ("ad", "thermodynamics", "flash", "physics")

SOURCE = r"""
#include "gpu_pr76_pt_flash_backend.hpp"
#include <memory>
#include <type_traits>
static_assert(std::is_base_of_v<mpmc::flash::PtFlashBackend, mpmc::flash::GpuPr76PtFlashBackend>);
std::unique_ptr<mpmc::flash::PtFlashBackend> make(const mpmc::flash::GpuPr76Mixture& m) {
    return std::make_unique<mpmc::flash::GpuPr76PtFlashBackend>(m);
}
"""


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
