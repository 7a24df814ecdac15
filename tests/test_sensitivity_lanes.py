"""The lane-group sensitivity kernel (pr76_sensw.cuh), run on the CPU under a
warp emulation, against the per-thread device function and the oracle.

tests/host_build/sens_host.cpp solves cells with the plain flash's device
function and differentiates each accepted pair with either ad::sensitivity_cell
(one thread per cell) or sensw::cell on an emulated group of S lanes
(tests/host_build/warp_emu.h: every shuffle a rendezvous of the group's lanes,
a missing lane a reported divergence).  On the CPU:

1. on solved cells (N = 3..20) the two forms give the same statuses and NaN
   patterns, bit-identical phase Jacobians, and derivatives within 1e-13
   normwise per column (the LU back substitution subtracts in the other
   order); the lanes never diverge;
2. the lane form meets the GPU sensitivity test's bar against the oracle's
   differentiate_pr76_pt_vle restatement at the same accepted states
   (parity.sensitivity_report: 1e-8 normwise, widened by cond(dF/dln K) eps);
3. on given pairs made to fail (beta at the guard, ln K without contrast,
   equal phases, a NaN or negative fraction, perturbed pairs) both forms end
   with the same status: phase boundary, ill-conditioned or arithmetic.
"""

import collections
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from mpmc_hnu_gb300 import synth
from tests import parity

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
DERIVS = ("d_ln_k", "d_vapor_fraction", "d_liquid", "d_vapor", "d_z_liquid", "d_z_vapor", "d_rho_liquid",
          "d_rho_vapor")
KEYS = ("status", "beta", "x", "y", "lnk", "z_l", "z_v", "sens_status") + DERIVS + ("jac_liquid", "jac_vapor")


@pytest.fixture(scope="module")
def host(tmp_path_factory):
    cxx = shutil.which("g++")
    cuda_inc = "/usr/local/cuda/include"
    if not cxx or not os.path.exists(os.path.join(cuda_inc, "cuda_runtime.h")):
        pytest.skip("host compiler or CUDA headers missing")
    so = str(tmp_path_factory.mktemp("sens_host") / "libsens_host.so")
    subprocess.check_call([cxx, "-std=c++17", "-O2", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
                           "-Wno-attributes", "-DMPMC_WARP_EMULATION", "-I" + cuda_inc,
                           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "mpmc_hnu_gb300", "csrc"),
                           os.path.join(HERE, "host_build", "sens_host.cpp"), "-o", so])
    return ctypes.CDLL(so)


def _outputs(n, nc):
    q = n + 1
    shapes = {"status": (nc,), "beta": (nc,), "x": (n, nc), "y": (n, nc), "lnk": (n, nc), "z_l": (nc,),
              "z_v": (nc,), "sens_status": (nc,), "d_ln_k": (n * q, nc), "d_vapor_fraction": (q, nc),
              "d_liquid": (n * q, nc), "d_vapor": (n * q, nc), "d_z_liquid": (q, nc), "d_z_vapor": (q, nc),
              "d_rho_liquid": (q, nc), "d_rho_vapor": (q, nc), "jac_liquid": ((n + 1) * (n + 2), nc),
              "jac_vapor": ((n + 1) * (n + 2), nc)}
    return {k: np.empty(v, np.int32 if k in ("status", "sens_status") else np.float64) for k, v in shapes.items()}


def run(lib, mix, p, t, z, lanes, given=None):
    """mode bit 0: the lane form; with `given` (a previous run's flash
    fields), differentiate those pairs instead of solving the cells."""
    tc, pc, om, kij = (np.ascontiguousarray(a, dtype=np.float64) for a in mix.as_tuple())
    z = np.ascontiguousarray(z, dtype=np.float64)
    n, nc = z.shape
    o = _outputs(n, nc)
    if given is not None:
        for k in ("status", "beta", "x", "y", "lnk", "z_l", "z_v"):
            o[k][...] = given[k]
    ins = [np.ascontiguousarray(a, dtype=np.float64) for a in (p, t)] + [z]
    mode = (1 if lanes else 0) | (2 if given is not None else 0)
    rc = lib.host_sensitivity_batch(ctypes.c_int(n), *[ctypes.c_void_p(a.ctypes.data) for a in (tc, pc, om, kij)],
                                    ctypes.c_int64(nc), *[ctypes.c_void_p(a.ctypes.data) for a in ins],
                                    ctypes.c_int(mode), *[ctypes.c_void_p(o[k].ctypes.data) for k in KEYS])
    assert rc == 0
    return o


def _normwise(a, b, ok):
    worst = 0.0
    for k in DERIVS:
        x, y = a[k][:, ok], b[k][:, ok]
        if x.size:
            scale = np.maximum(np.abs(x).max(axis=0, keepdims=True), 1e-300)
            worst = max(worst, float((np.abs(x - y) / scale).max()))
    return worst


@pytest.mark.parametrize("n,ncell,seed", [(3, 600, 5), (4, 300, 6), (6, 200, 1), (10, 96, 2), (16, 32, 3),
                                          (20, 32, 4)])
def test_lane_form_equals_per_thread(host, n, ncell, seed):
    mix = synth.make_mixture(n, seed)
    p, t, z = synth.make_cells(n, ncell, seed)
    a, b = run(host, mix, p, t, z, False), run(host, mix, p, t, z, True)
    assert not (b["sens_status"] == -99).any(), "lanes diverged or disagreed"
    assert np.array_equal(a["sens_status"], b["sens_status"])
    ok = a["sens_status"] == 0
    assert ok.sum() > 0
    for k in DERIVS + ("jac_liquid", "jac_vapor"):
        assert np.array_equal(np.isnan(a[k]), np.isnan(b[k])), k
    for k in ("jac_liquid", "jac_vapor"):
        assert np.array_equal(a[k][:, ok], b[k][:, ok]), k
    assert _normwise(a, b, ok) <= 1e-13


@pytest.mark.parametrize("n,ncell,seed", [(3, 128, 5), (6, 192, 1), (10, 128, 2), (20, 48, 4)])
def test_lane_form_matches_the_oracle(host, n, ncell, seed):
    from oracle import pyoracle
    pyoracle.build()
    mix = synth.make_mixture(n, seed)
    p, t, z = synth.make_cells(n, ncell, seed)
    b = run(host, mix, p, t, z, True)
    two = b["status"] == 1
    ref = pyoracle.sensitivity_at(mix, p, t, z, two, b["x"], b["y"], b["lnk"], b["beta"], manifold_identity=True)
    ref["sens_status"] = np.where(two, ref["sens_status"], 1)
    got = dict(b)
    got["sensitivity_status"] = b["sens_status"]
    rep = parity.sensitivity_report(got, ref, rcond=ref["rcond"])
    assert rep["status_match"] == 1.0, rep
    assert rep["both_ok"] > 0
    for f, v in rep["bound_ratio"].items():
        assert v <= 1.0, (f, rep)


def test_failure_statuses_agree(host):
    n, seed = 6, 31
    mix = synth.make_mixture(n, seed)
    p, t, z = synth.make_cells(n, 400, seed)
    base = run(host, mix, p, t, z, False)
    two = np.flatnonzero(base["status"] == 1)[:40]
    assert two.size >= 20
    p, t, z = p[two], t[two], np.ascontiguousarray(z[:, two])
    given = {k: np.array(v[..., two]) for k, v in base.items() if k in ("status", "beta", "x", "y", "lnk", "z_l",
                                                                         "z_v")}
    rng = np.random.default_rng(7)
    variants = []
    g = {k: v.copy() for k, v in given.items()}
    g["beta"][:] = 1e-9
    variants.append(g)
    g = {k: v.copy() for k, v in given.items()}
    g["lnk"] *= 1e-9
    variants.append(g)
    g = {k: v.copy() for k, v in given.items()}
    g["z_v"] = g["z_l"].copy()
    variants.append(g)
    g = {k: v.copy() for k, v in given.items()}
    g["y"] = g["x"].copy()
    variants.append(g)
    g = {k: v.copy() for k, v in given.items()}
    g["x"][0] = np.nan
    variants.append(g)
    g = {k: v.copy() for k, v in given.items()}
    g["x"][0] = -0.01
    variants.append(g)
    for scale in (1e-6, 1e-3, 1e-1):
        g = {k: v.copy() for k, v in given.items()}
        g["x"] *= 1.0 + scale * rng.standard_normal(g["x"].shape)
        g["y"] *= 1.0 + scale * rng.standard_normal(g["y"].shape)
        g["lnk"] *= 1.0 + scale * rng.standard_normal(g["lnk"].shape)
        variants.append(g)
    seen = collections.Counter()
    for g in variants:
        a, b = run(host, mix, p, t, z, False, given=g), run(host, mix, p, t, z, True, given=g)
        assert not (b["sens_status"] == -99).any()
        assert np.array_equal(a["sens_status"], b["sens_status"])
        ok = a["sens_status"] == 0
        if ok.any():
            assert _normwise(a, b, ok) <= 1e-12
        seen.update(a["sens_status"].tolist())
    # the phase-boundary, ill-conditioned and arithmetic statuses are all reached
    assert seen[2] > 0 and seen[5] > 0 and seen[6] > 0, seen


@pytest.fixture(scope="module")
def kernels(tmp_path_factory):
    """sensitivity.cu itself under the host launch emulation (cuda_emu.h):
    both kernels with their launch shapes, grid-stride loops and fills."""
    cxx = shutil.which("g++")
    cuda_inc = "/usr/local/cuda/include"
    if not cxx or not os.path.exists(os.path.join(cuda_inc, "cuda_runtime.h")):
        pytest.skip("host compiler or CUDA headers missing")
    from tests.host_build import emulate_launches
    tmp = tmp_path_factory.mktemp("sens_kernels")
    source = str(tmp / "sensitivity_emulated.cpp")
    emulate_launches.rewrite(os.path.join(ROOT, "mpmc_hnu_gb300", "csrc", "sensitivity.cu"), source)
    libs = {}
    for nm in (4, 12, 20):
        so = str(tmp / f"libsens_kernels_nm{nm}.so")
        subprocess.check_call([cxx, "-std=c++20", "-O2", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
                               "-Wno-attributes", "-Wno-unknown-pragmas", "-Wl,-Bsymbolic", f"-DMPMC_NM={nm}",
                               f'-DMPMC_SENS_SOURCE="{source}"', "-I" + cuda_inc,
                               "-I" + os.path.join(ROOT, "include"),
                               "-I" + os.path.join(ROOT, "mpmc_hnu_gb300", "csrc"),
                               "-I" + os.path.join(HERE, "host_build"),
                               os.path.join(HERE, "host_build", "sens_kernels_host.cpp"), "-o", so])
        libs[nm] = ctypes.CDLL(so)
    return libs


def run_kernel(libs, mix, p, t, z, lanes):
    n = mix.n
    lib = libs[4 if n <= 4 else (12 if n <= 12 else 20)]
    tc, pc, om, kij = (np.ascontiguousarray(a, dtype=np.float64) for a in mix.as_tuple())
    z = np.ascontiguousarray(z, dtype=np.float64)
    nc = z.shape[1]
    o = _outputs(n, nc)
    for k, v in o.items():
        v.fill(-5 if v.dtype == np.int32 else 7.0)  # a value no kernel writes
    ins = [np.ascontiguousarray(a, dtype=np.float64) for a in (p, t)] + [z]
    rc = lib.host_sensitivity_kernel(ctypes.c_int(n), *[ctypes.c_void_p(a.ctypes.data) for a in (tc, pc, om, kij)],
                                     ctypes.c_int64(nc), *[ctypes.c_void_p(a.ctypes.data) for a in ins],
                                     ctypes.c_int(int(lanes)), *[ctypes.c_void_p(o[k].ctypes.data) for k in KEYS])
    assert rc != -1, "emulated lanes diverged"
    assert rc == 0
    return o


@pytest.mark.parametrize("n,ncell,seed", [(3, 200, 5), (9, 150, 7), (12, 100, 3), (20, 40, 4)])
def test_lane_kernel_equals_per_thread_kernel(kernels, n, ncell, seed):
    """The kernels as launched: every cell gets a status and every output a
    value (NaN where the status is not success), the same in both."""
    mix = synth.make_mixture(n, seed)
    p, t, z = synth.make_cells(n, ncell, seed)
    a, b = run_kernel(kernels, mix, p, t, z, False), run_kernel(kernels, mix, p, t, z, True)
    assert np.array_equal(a["sens_status"], b["sens_status"])
    ok = a["sens_status"] == 0
    assert 0 < ok.sum() < ncell
    for k in DERIVS + ("jac_liquid", "jac_vapor"):
        assert not (a[k] == 7.0).any() and not (b[k] == 7.0).any(), k
        assert np.array_equal(np.isnan(a[k]), np.isnan(b[k])), k
        assert np.isnan(b[k][:, ~ok]).all(), k
    assert _normwise(a, b, ok) <= 1e-13
