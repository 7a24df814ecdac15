"""Ordered-path continuation on the GPU: 96 feeds of the three-phase fixture
mixture stepped along p = 0.2 .. 5 MPa at 250 K with ln K warm starts.  Every
point's published status equals a fresh cold max-3-phase solve of that point,
so the transition brackets are the cold scan's."""

import numpy as np
import pytest

from mpmc_hnu_gb300 import continuation, synth


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["mixed", "batched"])
def test_continuation_equals_fresh_solves(gpu_lib, form):
    mix = synth.three_phase_fixture_mixture()
    _, _, z = synth.make_three_phase_cells(96, seed=51, anchor_fraction=0.5)
    npoint = 10
    p = np.tile(np.exp(np.linspace(np.log(2e5), np.log(5e6), npoint)), (96, 1))
    t = np.full_like(p, 250.0)
    res = continuation.solve_paths(mix, z, p, t, form=form)
    g = gpu_lib.GpuFlash(mix, form=form)
    cold = np.empty_like(res["status"])
    for k in range(npoint):
        out, _ = g.solve_max3(np.ascontiguousarray(p[:, k]), np.ascontiguousarray(t[:, k]), z)
        cold[:, k] = out["status"]
    g.close()
    print(form, "phase counts", np.bincount(res["phase_count"].ravel(), minlength=4), "brackets",
          len(res["brackets"]))
    assert np.array_equal(res["status"], cold)
    assert res["brackets"] == continuation.transition_brackets(continuation.phase_counts(cold))
    assert (res["phase_count"] == 3).any() and len(res["brackets"]) > 0


@pytest.mark.gpu
def test_hinted_continuation_matches_reference(gpu_lib):
    """The reference's hint-seeded scan (mpmc_gpu_flash_solve_hinted) on the
    recorded fixture paths: every max3 and published status equals the
    reference's solve_pr76_pt_continuation, including the 63 points that the
    hints settle as three-phase where a fresh solve ends indeterminate."""
    import os

    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "continuation_reference.npz"))
    mix = synth.three_phase_fixture_mixture()
    res = continuation.solve_paths(mix, d["z"], d["p"], d["t"], hints=True)
    assert np.array_equal(res["max3_status"], d["ref_max3_status"])
    assert np.array_equal(res["status"], d["ref_published"])
    assert ((d["ref_max3_status"] != d["ref_cold_max3_status"]) & (res["max3_status"] == 2)).sum() == 63
