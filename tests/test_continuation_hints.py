"""The device code of the hinted max-3-phase solve, built for the host, and
the hint-seeded scan of mpmc_hnu_gb300/continuation.py over it.

tests/host_build/flash_host.cpp compiles the per-cell functions of the plain
and max3 kernels (fp64::solve_cell, fp64::max3_cell, fp64::load_hints) with
the host compiler and applies the kernels' per-cell sequence.  On the CPU:

1. without hints it reproduces every max3 status of the reference's
   solve_pr76_pt_max3 on the recorded fixture cells
   (tests/golden/max3_reference.npz);
2. continuation.scan_with_hints over it reproduces the reference's
   hint-seeded solve_pr76_pt_continuation on every recorded point
   (tests/golden/continuation_reference.npz), including the 63 points where
   the hints change the answer;
3. a three-phase start outside the simplex makes the cell an invalid
   request, as the reference's start check throws.
"""

import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from mpmc_hnu_gb300 import continuation, synth
from oracle import pyoracle

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def host_flash(tmp_path_factory):
    cxx = shutil.which("g++")
    cuda_inc = "/usr/local/cuda/include"
    if not cxx or not os.path.exists(os.path.join(cuda_inc, "cuda_runtime.h")):
        pytest.skip("host compiler or CUDA headers missing")
    so = str(tmp_path_factory.mktemp("flash_host") / "libflash_host.so")
    subprocess.check_call([cxx, "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-Wno-attributes",
                           "-I" + cuda_inc, "-I" + os.path.join(ROOT, "include"),
                           "-I" + os.path.join(ROOT, "mpmc_hnu_gb300", "csrc"),
                           os.path.join(HERE, "host_build", "flash_host.cpp"), "-o", so])
    lib = ctypes.CDLL(so)

    def make_step(mix):
        tc, pc, om, kij = (np.ascontiguousarray(a, dtype=np.float64) for a in mix.as_tuple())

        def step(p, t, z, count, hx, three, frac):
            n, ncell = z.shape
            outs = {"published": np.empty(ncell, np.int32), "max3": np.empty(ncell, np.int32),
                    "x": np.empty((n, ncell)), "y": np.empty((n, ncell)), "x3": np.empty((3 * n, ncell)),
                    "f3": np.empty((3, ncell))}
            args = [np.ascontiguousarray(a, dtype=dt) for a, dt in
                    ((p, np.float64), (t, np.float64), (z, np.float64), (count, np.int32), (hx, np.float64),
                     (three, np.int32), (frac, np.float64))]
            rc = lib.host_hinted_batch(ctypes.c_int(n), *[ctypes.c_void_p(a.ctypes.data) for a in (tc, pc, om, kij)],
                                       ctypes.c_int64(ncell), *[ctypes.c_void_p(a.ctypes.data) for a in args],
                                       *[ctypes.c_void_p(outs[k].ctypes.data)
                                         for k in ("published", "max3", "x", "y", "x3", "f3")])
            assert rc == 0
            return outs

        return step

    make_step.lib = lib
    return make_step


def _no_hints(n, ncell):
    return (np.zeros(ncell, np.int32), np.zeros((3 * n, ncell)), np.zeros(ncell, np.int32), np.zeros((2, ncell)))


def test_device_max3_without_hints_matches_reference(host_flash):
    d = np.load(os.path.join(HERE, "golden", "max3_reference.npz"))
    mix = synth.three_phase_fixture_mixture()
    z = np.ascontiguousarray(d["z"])
    out = host_flash(mix)(d["p"], d["t"], z, *_no_hints(3, z.shape[1]))
    assert np.array_equal(out["max3"], d["ref_max3_status"])
    assert np.array_equal(out["published"], d["ref_published"])


def test_hinted_scan_matches_reference_continuation(host_flash):
    d = np.load(os.path.join(HERE, "golden", "continuation_reference.npz"))
    mix = synth.three_phase_fixture_mixture()
    res = continuation.scan_with_hints(host_flash(mix), d["z"], d["p"], d["t"])
    assert np.array_equal(res["max3_status"], d["ref_max3_status"])
    assert np.array_equal(res["status"], d["ref_published"])
    settled = (d["ref_max3_status"] != d["ref_cold_max3_status"]) & (res["max3_status"] == 2)
    assert settled.sum() == 63


def test_invalid_three_phase_start_is_an_invalid_request(host_flash):
    mix = synth.three_phase_fixture_mixture()
    z = np.ascontiguousarray(synth.THREE_PHASE_ANCHOR.mean(axis=0)[:, None])
    count, hx, three, frac = _no_hints(3, 1)
    count[0] = 3
    hx[:, 0] = synth.THREE_PHASE_ANCHOR.ravel()
    three[0] = 1
    frac[:, 0] = [0.7, 0.6]  # outside the simplex
    out = host_flash(mix)(np.array([1e6]), np.array([250.0]), z, count, hx, three, frac)
    assert out["published"][0] == -1 and out["max3"][0] == -1
    frac[:, 0] = [0.3, 0.3]
    out = host_flash(mix)(np.array([1e6]), np.array([250.0]), z, count, hx, three, frac)
    assert out["published"][0] == 4 and out["max3"][0] == 2


def test_device_max3_with_starts_and_options_matches_reference(host_flash, tmp_path):
    """The general caller inputs (mpmc_start_hints_ex): every recorded case of
    tests/golden/max3_hinted_reference.npz -- the reference test's 3 -> 2
    recovery through a phase disappearance and its fresh two-phase neighbour,
    the 3 -> 3 base, a zero split-attempt quota, an empty feed test and a
    final start off the support -- gives the reference's max3 and published
    statuses, and the recovery's pair equals the reference's to 1e-12."""
    from tests.test_oracle_max3 import hinted_cases

    so = str(tmp_path / "libflash_host_ex.so")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-Wno-attributes",
                           "-I/usr/local/cuda/include", "-I" + os.path.join(ROOT, "include"),
                           "-I" + os.path.join(ROOT, "mpmc_hnu_gb300", "csrc"),
                           os.path.join(HERE, "host_build", "flash_host.cpp"), "-o", so])
    lib = ctypes.CDLL(so)
    for name, (mix, z, h, ref) in hinted_cases().items():
        n = z.shape[0]
        outs = {"published": np.empty(1, np.int32), "max3": np.empty(1, np.int32), "x": np.empty((n, 1)),
                "y": np.empty((n, 1)), "x3": np.empty((3 * n, 1)), "f3": np.empty((3, 1))}
        arrays = [np.ascontiguousarray(a) for a in (np.array([1e6]), np.array([250.0]), z)]
        hints = [np.ascontiguousarray(h[k]) for k in ("initial_count", "initial_composition", "final_count",
                                                       "final_composition", "three_phase",
                                                       "three_phase_composition", "fraction")]
        tc, pc, om, kij = (np.ascontiguousarray(a, dtype=np.float64) for a in mix.as_tuple())
        rc = lib.host_hinted_ex_batch(ctypes.c_int(n), *[ctypes.c_void_p(a.ctypes.data) for a in (tc, pc, om, kij)],
                                      ctypes.c_int64(1), *[ctypes.c_void_p(a.ctypes.data) for a in arrays + hints],
                                      ctypes.c_int32(int(h["initial_automatic_starts"])),
                                      ctypes.c_int32(int(h["max_split_attempts"])),
                                      *[ctypes.c_void_p(outs[k].ctypes.data)
                                        for k in ("published", "max3", "x", "y", "x3", "f3")])
        assert rc == 0
        assert outs["max3"][0] == np.ravel(ref["max3_status"])[0], name
        assert outs["published"][0] == np.ravel(ref["published"])[0], name
        if name == "recovery":
            assert np.allclose(outs["x"][:, 0], np.ravel(ref["x"]), rtol=0, atol=1e-12)
            assert np.allclose(outs["y"][:, 0], np.ravel(ref["y"]), rtol=0, atol=1e-12)


@pytest.mark.skipif(not os.path.isdir(os.path.join(pyoracle.REFERENCE_ROOT,
                                                   "modules", "flash", "include")),
                    reason="reference headers not present")
def test_cpp_continuation_binding_matches_reference(tmp_path):
    """mpmc_hnu_gb300/cpp/gpu_pr76_pt_continuation.hpp over the host build of
    the device code (its three C-ABI calls provided by
    tests/host_build/continuation_binding.cpp): every recorded point's max3
    status and every path's brackets as the reference's continuation has them."""
    ref_root = pyoracle.REFERENCE_ROOT
    d = np.load(os.path.join(HERE, "golden", "continuation_reference.npz"))
    exe = str(tmp_path / "continuation_binding")
    cmd = ["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-Wno-attributes", "-I/usr/local/cuda/include",
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "mpmc_hnu_gb300", "csrc"),
           "-I" + os.path.join(ROOT, "mpmc_hnu_gb300", "cpp")]
    cmd += ["-I" + os.path.join(ref_root, "modules", m, "include") for m in ("ad", "thermodynamics", "flash",
                                                                               "physics")]
    subprocess.check_call(cmd + [os.path.join(HERE, "host_build", "continuation_binding.cpp"),
                                 os.path.join(HERE, "host_build", "flash_host.cpp"), "-o", exe])
    inp = tmp_path / "paths.bin"
    npath, npoint = d["p"].shape
    with open(inp, "wb") as f:
        f.write(np.array([npath, npoint], np.int64).tobytes())
        for a in (d["p"], d["t"], d["z"]):
            f.write(np.ascontiguousarray(a, np.float64).tobytes())
    lines = subprocess.run([exe, str(inp)], capture_output=True, text=True, check=True).stdout.splitlines()
    assert len(lines) == npath
    ref = d["ref_max3_status"]
    counts = continuation.phase_counts(d["ref_published"])
    for k, line in enumerate(lines):
        statuses, brackets = line.split("|")
        assert [int(v) for v in statuses.split()] == list(ref[k])
        expect = [(b[1], b[2]) for b in continuation.transition_brackets(counts[k:k + 1])]
        got = [tuple(int(v) for v in b.split("-")) for b in brackets.split()[1:]]
        assert got == expect


def test_device_max3_on_six_components_matches_reference(host_flash):
    """The six-component sour-gas fixture of the reference's tests
    (tests/golden/max3_heringer_reference.npz): the host build of the device
    code reproduces every max3 and published status."""
    d = np.load(os.path.join(HERE, "golden", "max3_heringer_reference.npz"))
    mix = synth.Mixture(d["tc"], d["pc"], d["omega"], d["kij"])
    z = np.ascontiguousarray(d["z"])
    out = host_flash(mix)(d["p"], d["t"], z, *_no_hints(6, z.shape[1]))
    assert np.array_equal(out["max3"], d["ref_max3_status"])
    assert np.array_equal(out["published"], d["ref_published"])


def test_newton_roots_keep_every_recorded_status(host_flash):
    """MPMC_FLAG_MAX3_NEWTON_ROOTS: the continuation with bracketed-Newton
    roots and Rachford-Rice (the flash's FP64 items' solvers, the reference's
    stopping width) instead of bisection reproduces every recorded max3 and
    published status -- the three-phase fixture's 1,649 cells, the
    six-component fixture's 429 and the hint-seeded scan's 960 points -- and
    its three-phase sets equal the bisection ones to 1e-9."""
    lib = host_flash.lib
    d = np.load(os.path.join(HERE, "golden", "max3_reference.npz"))
    mix3 = synth.three_phase_fixture_mixture()
    z3 = np.ascontiguousarray(d["z"])
    bisection = host_flash(mix3)(d["p"], d["t"], z3, *_no_hints(3, z3.shape[1]))
    lib.host_set_max3_newton(1)
    try:
        out = host_flash(mix3)(d["p"], d["t"], z3, *_no_hints(3, z3.shape[1]))
        assert np.array_equal(out["max3"], d["ref_max3_status"])
        assert np.array_equal(out["published"], d["ref_published"])
        three = out["max3"] == 2
        assert three.sum() > 600
        assert np.abs(out["x3"][:, three] - bisection["x3"][:, three]).max() <= 1e-9
        assert np.abs(out["f3"][:, three] - bisection["f3"][:, three]).max() <= 1e-9
        h = np.load(os.path.join(HERE, "golden", "max3_heringer_reference.npz"))
        mix6 = synth.Mixture(h["tc"], h["pc"], h["omega"], h["kij"])
        z6 = np.ascontiguousarray(h["z"])
        out6 = host_flash(mix6)(h["p"], h["t"], z6, *_no_hints(6, z6.shape[1]))
        assert np.array_equal(out6["max3"], h["ref_max3_status"])
        assert np.array_equal(out6["published"], h["ref_published"])
        c = np.load(os.path.join(HERE, "golden", "continuation_reference.npz"))
        res = continuation.scan_with_hints(host_flash(mix3), c["z"], c["p"], c["t"])
        assert np.array_equal(res["max3_status"], c["ref_max3_status"])
        assert np.array_equal(res["status"], c["ref_published"])
    finally:
        lib.host_set_max3_newton(0)
