"""The batched flash pipeline -- the headline mixed-precision form and the FP64
work-queue form, every kernel of flash_batched.cu -- run on the CPU under the
host launch emulation, against the oracle.

tests/host_build/emulate_launches.py rewrites the kernel launches of
flash_batched.cu into calls of tests/host_build/cuda_emu.h, which runs each
launch's blocks as host threads with the warp intrinsics as rendezvous of the
named lanes; tests/host_build/batched_host.cpp calls the unchanged
orchestration (launch_batched_nm) on host memory.  So the device code of the
pipeline -- FP32 screening, FP64 lane-group items, the polish, the queues, the
exact sub-solve -- is checked here without a GPU, at small sizes and with the
host compiler's arithmetic:

1. the mixed form's statuses equal the oracle's on every cell, and its
   outputs meet the GPU parity bar of tests/test_gpu_parity.py
   (parity.assert_flash_parity: polished ln K within 1e-10, raw values in the
   reference's stopping band), at N = 3, 6, 10 and 20 and on near-critical
   cells;
2. the same for the FP64 work-queue form;
3. from ln K warm starts (a second solve started at the first one's ln K,
   perturbed), the statuses are the cold ones;
4. the opt-in state-machine polish (MPMC_FLAG_POLISH_STREAM) gives the
   default polish's outputs bit for bit;
5. no emulated lane ever waits at an intrinsic that another lane of its mask
   does not reach.
"""

import concurrent.futures as cf
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from mpmc_hnu_gb300 import synth
from tests import parity
from tests.host_build import emulate_launches

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "mpmc_hnu_gb300", "csrc")
CAPACITIES = (4, 8, 12, 20)


@pytest.fixture(scope="module")
def pipeline(tmp_path_factory):
    cxx = shutil.which("g++")
    cuda_inc = "/usr/local/cuda/include"
    if not cxx or not os.path.exists(os.path.join(cuda_inc, "cuda_runtime.h")):
        pytest.skip("host compiler or CUDA headers missing")
    tmp = tmp_path_factory.mktemp("batched_emu")
    source = str(tmp / "flash_batched_emulated.cpp")
    emulate_launches.rewrite(os.path.join(CSRC, "flash_batched.cu"), source)

    def build(nm):
        so = str(tmp / f"libbatched_emu_nm{nm}.so")
        subprocess.check_call([cxx, "-std=c++20", "-O2", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
                               "-Wno-attributes", "-Wno-unknown-pragmas", "-Wl,-Bsymbolic", f"-DMPMC_NM={nm}",
                               f'-DMPMC_BATCHED_SOURCE="{source}"', "-I" + cuda_inc,
                               "-I" + os.path.join(ROOT, "include"), "-I" + CSRC,
                               "-I" + os.path.join(HERE, "host_build"),
                               os.path.join(HERE, "host_build", "batched_host.cpp"), "-o", so])
        return nm, ctypes.CDLL(so)

    with cf.ThreadPoolExecutor(max_workers=len(CAPACITIES)) as ex:
        return dict(ex.map(build, CAPACITIES))


def _capacity(n):
    return next(c for c in CAPACITIES if n <= c)


STATS = 48  # batched::qSlots


def solve(libs, mix, p, t, z, fp64=False, warm=None, polish_stream=False, stats=None):
    n = mix.n
    lib = libs[_capacity(n)]
    tc, pc, om, kij = (np.ascontiguousarray(a, dtype=np.float64) for a in mix.as_tuple())
    z = np.ascontiguousarray(z, dtype=np.float64)
    nc = z.shape[1]
    o = {"status": np.full(nc, -7, np.int32), "vapor_fraction": np.empty(nc), "liquid": np.empty((n, nc)),
         "vapor": np.empty((n, nc)), "ln_k": np.empty((n, nc)), "ln_phi_liquid": np.empty((n, nc)),
         "ln_phi_vapor": np.empty((n, nc)), "z_liquid": np.empty(nc), "z_vapor": np.empty(nc),
         "counters": np.zeros((8, nc), np.int32)}
    ins = [np.ascontiguousarray(a, dtype=np.float64) for a in (p, t)] + [z]
    w = np.ascontiguousarray(warm, dtype=np.float64) if warm is not None else None
    rc = lib.host_batched_solve(ctypes.c_int(n), *[ctypes.c_void_p(a.ctypes.data) for a in (tc, pc, om, kij)],
                                ctypes.c_int64(nc), *[ctypes.c_void_p(a.ctypes.data) for a in ins],
                                ctypes.c_void_p(w.ctypes.data if w is not None else None), ctypes.c_int(int(fp64)),
                                ctypes.c_int(int(polish_stream)),
                                *[ctypes.c_void_p(o[k].ctypes.data) for k in
                                  ("status", "vapor_fraction", "liquid", "vapor", "ln_k", "ln_phi_liquid",
                                   "ln_phi_vapor", "z_liquid", "z_vapor", "counters")],
                                ctypes.c_void_p(stats.ctypes.data if stats is not None else None))
    assert rc != -1, "emulated lanes diverged at an intrinsic"
    assert rc == 0, f"orchestration error {rc}"
    return o


@pytest.mark.parametrize("n,ncell,seed", [(3, 512, 5), (6, 256, 1), (10, 256, 2), (20, 64, 4)])
def test_mixed_form_matches_the_oracle(pipeline, oracle_lib, n, ncell, seed):
    mix = synth.make_mixture(n, seed)
    p, t, z = synth.make_cells(n, ncell, seed)
    out = solve(pipeline, mix, p, t, z)
    ref = oracle_lib.flash(mix, p, t, z, threads=8)
    rep = parity.flash_report(out, ref, mix, p, t, z)
    parity.assert_flash_parity(rep)
    assert rep["two_phase"] > 0


@pytest.mark.parametrize("n,ncell,seed", [(10, 128, 12), (20, 48, 13)])
def test_mixed_form_near_critical(pipeline, oracle_lib, n, ncell, seed):
    mix = synth.make_mixture(n, seed)
    p, t, z = synth.make_near_critical_cells(mix, ncell, seed, fraction=0.5)
    out = solve(pipeline, mix, p, t, z)
    ref = oracle_lib.flash(mix, p, t, z, threads=8)
    parity.assert_flash_parity(parity.flash_report(out, ref, mix, p, t, z))


@pytest.mark.parametrize("n,ncell,seed", [(3, 256, 5), (4, 64, 6)])
def test_fp64_form_matches_the_oracle(pipeline, oracle_lib, n, ncell, seed):
    mix = synth.make_mixture(n, seed)
    p, t, z = synth.make_cells(n, ncell, seed)
    out = solve(pipeline, mix, p, t, z, fp64=True)
    ref = oracle_lib.flash(mix, p, t, z, threads=8)
    parity.assert_flash_parity(parity.flash_report(out, ref, mix, p, t, z))


def test_warm_starts_keep_the_cold_statuses(pipeline, oracle_lib):
    n, ncell, seed = 6, 256, 3
    mix = synth.make_mixture(n, seed)
    p, t, z = synth.make_cells(n, ncell, seed)
    cold = solve(pipeline, mix, p, t, z)
    rng = np.random.default_rng(seed)
    warm = cold["ln_k"] + 0.1 * rng.standard_normal(cold["ln_k"].shape)
    warm[:, cold["status"] != 1] = np.nan
    out = solve(pipeline, mix, p, t, z, warm=warm)
    ref = oracle_lib.flash(mix, p, t, z, threads=8)
    assert np.array_equal(out["status"], ref["status"])
    assert np.array_equal(out["status"], cold["status"])


@pytest.mark.parametrize("n,ncell,seed", [(3, 512, 5), (6, 256, 1), (10, 256, 2), (20, 64, 4)])
def test_state_machine_polish_equals_the_default(pipeline, oracle_lib, n, ncell, seed):
    """MPMC_FLAG_POLISH_STREAM: the state-machine polish makes the same
    evaluations per cell as the default polish, so every output is the same
    bit for bit (at N = 20 both run the lane-group polish)."""
    mix = synth.make_mixture(n, seed)
    p, t, z = synth.make_cells(n, ncell, seed)
    a = solve(pipeline, mix, p, t, z)
    b = solve(pipeline, mix, p, t, z, polish_stream=True)
    for k in a:
        assert a[k].tobytes() == b[k].tobytes(), k
    ref = oracle_lib.flash(mix, p, t, z, threads=8)
    parity.assert_flash_parity(parity.flash_report(b, ref, mix, p, t, z))


def test_exact_sub_solve_matches_the_oracle(pipeline, oracle_lib):
    """Hard cells (N = 10 at 10-12 MPa and 365-375 K) on which FP32 cannot
    screen one cell: it is marked for the exact sub-solve (the FP64
    work-queue form on that cell alone, gathered and scattered back), and
    every status and value still meets the parity bar."""
    n, seed, ncell = 10, 7, 128
    rng = np.random.default_rng(1000 + seed)
    mix = synth.make_mixture(n, seed)
    p = rng.uniform(10e6, 12e6, ncell)
    t = rng.uniform(365.0, 375.0, ncell)
    z = rng.exponential(size=(n, ncell))
    z /= z.sum(axis=0)
    stats = np.zeros(STATS, np.int32)
    out = solve(pipeline, mix, p, t, z, stats=stats)
    assert stats[46] >= 1  # batched::sExactCells
    ref = oracle_lib.flash(mix, p, t, z, threads=8)
    parity.assert_flash_parity(parity.flash_report(out, ref, mix, p, t, z))


def _near_boundary_cells(oracle_lib, mix, ncell, seed):
    """Cells placed within 2 % of a pressure where the oracle's phase count
    changes (bisection in ln p on [0.5, 40] MPa), as the bench places 30 % of
    its cells; cells with no change in range are dropped."""
    n = mix.n
    p, t, z = synth.make_cells(n, 4 * ncell, seed)
    lo, hi = np.full(p.shape, np.log(0.5e6)), np.full(p.shape, np.log(40e6))
    s_lo = oracle_lib.flash(mix, np.exp(lo), t, z, threads=8)["status"]
    s_hi = oracle_lib.flash(mix, np.exp(hi), t, z, threads=8)["status"]
    keep = s_lo != s_hi
    lo, hi, t, z, s_lo = lo[keep], hi[keep], t[keep], z[:, keep], s_lo[keep]
    for _ in range(30):
        mid = 0.5 * (lo + hi)
        s_mid = oracle_lib.flash(mix, np.exp(mid), t, z, threads=8)["status"]
        same = s_mid == s_lo
        lo = np.where(same, mid, lo)
        hi = np.where(same, hi, mid)
    rng = np.random.default_rng(seed)
    pb = np.exp(0.5 * (lo + hi)) * (1.0 + rng.uniform(-0.02, 0.02, lo.shape))
    return pb[:ncell], t[:ncell], np.ascontiguousarray(z[:, :ncell])


@pytest.mark.parametrize("n,ncell,seed", [(4, 256, 21), (10, 128, 22)])
def test_mixed_form_near_the_phase_boundary(pipeline, oracle_lib, n, ncell, seed):
    """The bench's hard regime: every cell within 2 % of its own phase-count
    change pressure."""
    mix = synth.make_mixture(n, seed)
    p, t, z = _near_boundary_cells(oracle_lib, mix, ncell, seed)
    assert p.size >= ncell // 2
    out = solve(pipeline, mix, p, t, z)
    ref = oracle_lib.flash(mix, p, t, z, threads=8)
    rep = parity.flash_report(out, ref, mix, p, t, z)
    parity.assert_flash_parity(rep)
    assert rep["two_phase"] > 0
