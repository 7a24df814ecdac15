"""The max-3-phase kernel's warp form, run on the CPU under a warp emulation.

max3_kernel runs each phase_set_unstable cell on the 32 lanes of a warp:
every lane holds its own copy of the same state, and the three-phase
attempts' line searches evaluate their 32 backtracking trials at once, one
per lane, then walk the outcomes in order (iterate_three, pr76_max3.cuh).
tests/host_build/flash_host.cpp built with -DMPMC_WARP_EMULATION runs that
code on 32 host threads (tests/host_build/warp_emu.h), every shuffle a
rendezvous of all 32.  On the CPU:

1. the lanes never diverge (a lane missing at a shuffle would leave the GPU's
   full-mask shuffle waiting; here it times out and marks the cell -99), and
   all 32 end with the same answer;
2. every output equals the sequential host build bit for bit -- the walk
   picks the trial, and spends the evaluation budget, the sequential line
   search would -- on the 1,649 recorded cells of the three-phase fixture
   (tests/golden/max3_reference.npz, whose statuses it also reproduces) and
   on the 32 cells of the smoke set, one of which runs two attempts to the
   30,000-evaluation limit.
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


def _build(tmp, emulate):
    cxx = shutil.which("g++")
    cuda_inc = "/usr/local/cuda/include"
    if not cxx or not os.path.exists(os.path.join(cuda_inc, "cuda_runtime.h")):
        pytest.skip("host compiler or CUDA headers missing")
    so = str(tmp / ("libflash_host_warp.so" if emulate else "libflash_host_seq.so"))
    cmd = [cxx, "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-Wno-attributes", "-pthread",
           "-I" + cuda_inc, "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "mpmc_hnu_gb300", "csrc"),
           os.path.join(HERE, "host_build", "flash_host.cpp"), "-o", so]
    if emulate:
        cmd.insert(1, "-DMPMC_WARP_EMULATION")
    subprocess.check_call(cmd)
    return ctypes.CDLL(so)


@pytest.fixture(scope="module")
def libs(tmp_path_factory):
    tmp = tmp_path_factory.mktemp("max3_warp")
    return _build(tmp, False), _build(tmp, True)


def _solve(lib, mix, p, t, z):
    tc, pc, om, kij = (np.ascontiguousarray(a, dtype=np.float64) for a in mix.as_tuple())
    z = np.ascontiguousarray(z, dtype=np.float64)
    n, ncell = z.shape
    ins = [np.ascontiguousarray(p, dtype=np.float64), np.ascontiguousarray(t, dtype=np.float64), z,
           np.zeros(ncell, np.int32), np.zeros((3 * n, ncell)), np.zeros(ncell, np.int32), np.zeros((2, ncell))]
    outs = {"published": np.empty(ncell, np.int32), "max3": np.empty(ncell, np.int32), "x": np.empty((n, ncell)),
            "y": np.empty((n, ncell)), "x3": np.empty((3 * n, ncell)), "f3": np.empty((3, ncell))}
    rc = lib.host_hinted_batch(ctypes.c_int(n), *[ctypes.c_void_p(a.ctypes.data) for a in (tc, pc, om, kij)],
                               ctypes.c_int64(ncell), *[ctypes.c_void_p(a.ctypes.data) for a in ins],
                               *[ctypes.c_void_p(outs[k].ctypes.data)
                                 for k in ("published", "max3", "x", "y", "x3", "f3")])
    assert rc == 0
    return outs


def _assert_bitwise_equal(a, b):
    for k in a:
        assert a[k].tobytes() == b[k].tobytes(), k


def test_warp_form_equals_sequential_on_the_smoke_set(libs):
    seq, warp = libs
    mix = synth.three_phase_fixture_mixture()
    p, t, z = synth.make_three_phase_cells(32, seed=5, anchor_fraction=0.5)
    a, b = _solve(seq, mix, p, t, z), _solve(warp, mix, p, t, z)
    assert not (b["max3"] == -99).any(), "lanes diverged or disagreed"
    assert (a["max3"] == 2).sum() == 14
    _assert_bitwise_equal(a, b)


def test_warp_form_equals_sequential_on_recorded_cells(libs):
    seq, warp = libs
    d = np.load(os.path.join(HERE, "golden", "max3_reference.npz"))
    mix = synth.three_phase_fixture_mixture()
    a, b = _solve(seq, mix, d["p"], d["t"], d["z"]), _solve(warp, mix, d["p"], d["t"], d["z"])
    assert not (b["max3"] == -99).any(), "lanes diverged or disagreed"
    assert np.array_equal(b["max3"], d["ref_max3_status"])
    assert np.array_equal(b["published"], d["ref_published"])
    _assert_bitwise_equal(a, b)


def test_warp_form_with_newton_roots_equals_sequential(libs):
    """The same with bracketed-Newton roots (MPMC_FLAG_MAX3_NEWTON_ROOTS)."""
    seq, warp = libs
    mix = synth.three_phase_fixture_mixture()
    p, t, z = synth.make_three_phase_cells(32, seed=5, anchor_fraction=0.5)
    for lib in libs:
        lib.host_set_max3_newton(1)
    try:
        a, b = _solve(seq, mix, p, t, z), _solve(warp, mix, p, t, z)
    finally:
        for lib in libs:
            lib.host_set_max3_newton(0)
    assert not (b["max3"] == -99).any(), "lanes diverged or disagreed"
    assert (a["max3"] == 2).sum() == 14
    _assert_bitwise_equal(a, b)
