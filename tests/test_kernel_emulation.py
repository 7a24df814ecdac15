"""The plain flash kernel and the max-3-phase kernel as launched, on the CPU
under the host launch emulation (tests/host_build/cuda_emu.h,
tests/host_build/kernels_host.cpp): launch shapes, grid-stride loops, the
max3 kernel's warp per cell with lane 0 writing, the publication rules.

1. The plain kernel then the max3 kernel reproduce every recorded max3 and
   published status of the reference's solve_pr76_pt_max3 on the
   three-phase fixture's 1,649 cells and the six-component fixture's 429,
   with three-phase sets within 1e-9 of the recorded ones; also with the
   opt-in bracketed-Newton roots (MPMC_FLAG_MAX3_NEWTON_ROOTS).
2. The plain kernel's statuses equal the oracle's on synthetic cells.
"""

import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from mpmc_hnu_gb300 import synth

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "mpmc_hnu_gb300", "csrc")


@pytest.fixture(scope="module")
def kernels(tmp_path_factory):
    cxx = shutil.which("g++")
    cuda_inc = "/usr/local/cuda/include"
    if not cxx or not os.path.exists(os.path.join(cuda_inc, "cuda_runtime.h")):
        pytest.skip("host compiler or CUDA headers missing")
    from tests.host_build import emulate_launches
    tmp = tmp_path_factory.mktemp("kernels_emu")
    plain, max3 = str(tmp / "flash_plain_emulated.cpp"), str(tmp / "flash_max3_emulated.cpp")
    emulate_launches.rewrite(os.path.join(CSRC, "flash_plain.cu"), plain)
    emulate_launches.rewrite(os.path.join(CSRC, "flash_max3.cu"), max3)
    libs = {}
    for nm in (4, 8, 12):
        so = str(tmp / f"libkernels_nm{nm}.so")
        subprocess.check_call([cxx, "-std=c++20", "-O2", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
                               "-Wno-attributes", "-Wno-unknown-pragmas", "-Wl,-Bsymbolic", f"-DMPMC_NM={nm}",
                               f'-DMPMC_PLAIN_SOURCE="{plain}"', f'-DMPMC_MAX3_SOURCE="{max3}"', "-I" + cuda_inc,
                               "-I" + os.path.join(ROOT, "include"), "-I" + CSRC,
                               "-I" + os.path.join(HERE, "host_build"),
                               os.path.join(HERE, "host_build", "kernels_host.cpp"), "-o", so])
        libs[nm] = ctypes.CDLL(so)
    return libs


def run(libs, mix, p, t, z, max3=True, newton_roots=False):
    n = mix.n
    lib = libs[4 if n <= 4 else (8 if n <= 8 else 12)]
    tc, pc, om, kij = (np.ascontiguousarray(a, dtype=np.float64) for a in mix.as_tuple())
    z = np.ascontiguousarray(z, dtype=np.float64)
    nc = z.shape[1]
    o = {"status": np.empty(nc, np.int32), "beta": np.empty(nc), "x": np.empty((n, nc)), "y": np.empty((n, nc)),
         "lnk": np.empty((n, nc)), "lnphi_l": np.empty((n, nc)), "lnphi_v": np.empty((n, nc)), "z_l": np.empty(nc),
         "z_v": np.empty(nc), "counters": np.zeros((8, nc), np.int32), "max3_status": np.full(nc, -9, np.int32),
         "fraction": np.empty((3, nc)), "x3": np.empty((3 * n, nc)), "lnphi3": np.empty((3 * n, nc)),
         "z3": np.empty((3, nc))}
    keys = ("status", "beta", "x", "y", "lnk", "lnphi_l", "lnphi_v", "z_l", "z_v", "counters", "max3_status",
            "fraction", "x3", "lnphi3", "z3")
    ins = [np.ascontiguousarray(a, dtype=np.float64) for a in (p, t)] + [z]
    rc = lib.host_plain_max3(ctypes.c_int(n), *[ctypes.c_void_p(a.ctypes.data) for a in (tc, pc, om, kij)],
                             ctypes.c_int64(nc), *[ctypes.c_void_p(a.ctypes.data) for a in ins],
                             ctypes.c_int(int(max3)), ctypes.c_int(int(newton_roots)),
                             *[ctypes.c_void_p(o[k].ctypes.data) for k in keys])
    assert rc != -1, "emulated lanes diverged"
    assert rc == 0
    return o


@pytest.mark.parametrize("newton_roots", [False, True])
def test_max3_kernel_reproduces_the_recorded_statuses(kernels, newton_roots):
    d = np.load(os.path.join(HERE, "golden", "max3_reference.npz"))
    out = run(kernels, synth.three_phase_fixture_mixture(), d["p"], d["t"], d["z"], newton_roots=newton_roots)
    assert np.array_equal(out["max3_status"], d["ref_max3_status"])
    assert np.array_equal(out["status"], d["ref_published"])
    three = out["max3_status"] == 2
    assert three.sum() > 600
    assert np.abs(out["x3"][:, three] - d["ref_x3"][:, three]).max() <= 1e-9
    assert np.abs(out["fraction"][:, three] - d["ref_beta3"][:, three]).max() <= 1e-9


def test_max3_kernel_on_six_components(kernels):
    h = np.load(os.path.join(HERE, "golden", "max3_heringer_reference.npz"))
    mix = synth.Mixture(h["tc"], h["pc"], h["omega"], h["kij"])
    out = run(kernels, mix, h["p"], h["t"], h["z"])
    assert np.array_equal(out["max3_status"], h["ref_max3_status"])
    assert np.array_equal(out["status"], h["ref_published"])


@pytest.mark.parametrize("n,ncell,seed", [(3, 256, 5), (10, 128, 2)])
def test_plain_kernel_matches_the_oracle(kernels, oracle_lib, n, ncell, seed):
    mix = synth.make_mixture(n, seed)
    p, t, z = synth.make_cells(n, ncell, seed)
    out = run(kernels, mix, p, t, z, max3=False)
    ref = oracle_lib.flash(mix, p, t, z, threads=8)
    assert np.array_equal(out["status"], ref["status"])
    two = ref["status"] == 1
    assert two.sum() > 0
    assert np.abs(out["lnk"][:, two] - ref["ln_k"][:, two]).max() <= 1e-9 * max(1.0, np.abs(ref["ln_k"][:, two]).max())
