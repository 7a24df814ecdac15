"""GPU checks of the opt-in paths, run with MPMC_TEST_OPT_IN=1:

* MPMC_FLAG_SENSITIVITY_LANES, the lane-group sensitivity kernel
  (pr76_sensw.cuh): the same statuses and flash fields as the per-thread
  kernel, derivatives within 1e-12 of it normwise, and the oracle's bar of
  tests/test_gpu_sensitivity.py;
* MPMC_FLAG_MAX3_NEWTON_ROOTS, bracketed-Newton roots in the max-3-phase
  continuation: the recorded statuses of tests/test_gpu_max3.py, and
  three-phase sets within 1e-9 of the recorded ones;
* MPMC_FLAG_POLISH_STREAM, the state-machine FP64 polish: the default
  polish's statuses and the oracle's parity bar.

All three are checked on the CPU (tests/test_sensitivity_lanes.py,
tests/test_continuation_hints.py, tests/test_max3_warp_emulation.py,
tests/test_batched_emulation.py); these tests are their first GPU runs, kept
out of the default suite until a GPU has run them.
"""

import os

import numpy as np
import pytest

from mpmc_hnu_gb300 import synth
from tests import parity

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(os.environ.get("MPMC_TEST_OPT_IN") != "1",
                                 reason="opt-in paths: run with MPMC_TEST_OPT_IN=1")]

DERIVS = ("d_ln_k", "d_vapor_fraction", "d_liquid", "d_vapor", "d_z_liquid", "d_z_vapor", "d_rho_liquid",
          "d_rho_vapor")
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "max3_reference.npz")


@pytest.mark.parametrize("form", ["plain", "mixed"])
@pytest.mark.parametrize("n,ncell,seed", [(3, 128, 5), (6, 192, 1), (10, 128, 2), (16, 64, 3), (20, 48, 4)])
def test_lane_sensitivity_matches_per_thread_and_oracle(gpu_lib, oracle_lib, n, ncell, seed, form):
    mix = synth.make_mixture(n, seed)
    p, t, z = synth.make_cells(n, ncell, seed)
    outs = []
    for lanes in (False, True):
        g = gpu_lib.GpuFlash(mix, form=form, sensitivity=True, sensitivity_lanes=lanes)
        outs.append(g.solve(p, t, z))
        g.close()
    a, b = outs
    for f in ("status", "vapor_fraction", "liquid", "vapor", "ln_k", "sensitivity_status"):
        assert np.array_equal(a[f], b[f], equal_nan=True), f
    ok = a["sensitivity_status"] == 0
    assert ok.sum() > 0
    worst = 0.0
    for f in DERIVS + ("jac_liquid", "jac_vapor"):
        assert np.array_equal(np.isnan(a[f]), np.isnan(b[f])), f
        x, y = a[f][:, ok], b[f][:, ok]
        scale = np.maximum(np.abs(x).max(axis=0, keepdims=True), 1e-300)
        worst = max(worst, float((np.abs(x - y) / scale).max()))
    print(form, n, "lane vs per-thread", worst)
    assert worst <= 1e-12
    two = b["status"] == 1
    ref = oracle_lib.sensitivity_at(mix, p, t, z, two, b["liquid"], b["vapor"], b["ln_k"], b["vapor_fraction"],
                                    manifold_identity=True)
    ref["sens_status"] = np.where(two, ref["sens_status"], 1)
    rep = parity.sensitivity_report(b, ref, rcond=ref["rcond"])
    assert rep["status_match"] == 1.0, rep
    for f, v in rep["bound_ratio"].items():
        assert v <= 1.0, (f, rep)


@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_max3_newton_roots_keep_the_recorded_statuses(gpu_lib, form):
    d = np.load(GOLDEN)
    mix = synth.three_phase_fixture_mixture()
    g = gpu_lib.GpuFlash(mix, form=form, max3_newton_roots=True)
    out, out3 = g.solve_max3(d["p"], d["t"], d["z"])
    g.close()
    ms, rs = out3["max3_status"], d["ref_max3_status"]
    mismatch = np.nonzero(ms != rs)[0]
    assert mismatch.size <= (0 if form == "plain" else len(ms) // 500)
    same = ms == rs
    assert np.array_equal(out["status"][same], d["ref_published"][same])
    three = same & (rs == 2)
    assert three.sum() > 100
    for f_gpu, f_ref in (("phase_fraction", "ref_beta3"), ("composition", "ref_x3"), ("z_factor", "ref_z3")):
        assert np.abs(out3[f_gpu][:, three] - d[f_ref][:, three]).max() <= 1e-9, f_gpu


@pytest.mark.parametrize("n,ncell,seed", [(3, 2048, 5), (6, 2048, 1), (10, 2048, 2)])
def test_state_machine_polish_matches_the_default_and_the_oracle(gpu_lib, oracle_lib, n, ncell, seed):
    """MPMC_FLAG_POLISH_STREAM: the same statuses as the default polish, and
    the parity bar of tests/test_gpu_parity.py against the oracle."""
    from tests import parity
    mix = synth.make_mixture(n, seed)
    p, t, z = synth.make_cells(n, ncell, seed)
    outs = []
    for stream in (False, True):
        g = gpu_lib.GpuFlash(mix, form="mixed", polish_stream=stream)
        outs.append(g.solve(p, t, z))
        g.close()
    assert np.array_equal(outs[0]["status"], outs[1]["status"])
    ref = oracle_lib.flash(mix, p, t, z, threads=8)
    parity.assert_flash_parity(parity.flash_report(outs[1], ref, mix, p, t, z))
