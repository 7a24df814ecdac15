"""Max-3-phase continuation on the GPU (mpmc_gpu_flash_solve_max3) against the
recorded outputs of the reference's solve_pr76_pt_max3
(tests/golden/max3_reference.npz, fixture mixture of the reference's own
three-phase tests) and the fixture's independent three-phase anchor.

The continuation runs the reference's FP64 arithmetic for every form; its
two-phase input is the form's own answer.  The plain form, which follows the
reference step for step, must reproduce every max3 status; the work-queue
forms may differ on a cell where their two-phase answer differs (at most 1 in
500 here).  Three-phase sets agree to 1e-9.
"""

import os

import numpy as np
import pytest

from mpmc_hnu_gb300 import synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "max3_reference.npz")


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["plain", "batched", "mixed"])
def test_max3_matches_reference(gpu_lib, form):
    d = np.load(GOLDEN)
    mix = synth.three_phase_fixture_mixture()
    p, t, z = d["p"], d["t"], d["z"]
    g = gpu_lib.GpuFlash(mix, form=form)
    out, out3 = g.solve_max3(p, t, z)
    base = g.solve(p, t, z)
    g.close()
    ms, rs = out3["max3_status"], d["ref_max3_status"]
    mismatch = np.nonzero(ms != rs)[0]
    print(form, "max3 status counts", np.bincount(ms + 1, minlength=7), "mismatches", mismatch.size,
          [(int(c), int(rs[c]), int(ms[c])) for c in mismatch[:6]])
    assert mismatch.size <= (0 if form == "plain" else len(ms) // 500)
    same = ms == rs
    assert np.array_equal(out["status"][same], d["ref_published"][same])
    three = same & (rs == 2)
    assert three.sum() > 100
    for f_gpu, f_ref in (("phase_fraction", "ref_beta3"), ("composition", "ref_x3"), ("z_factor", "ref_z3")):
        err = np.abs(out3[f_gpu][:, three] - d[f_ref][:, three]).max()
        assert err <= 1e-9, (f_gpu, err)
    err = np.abs(out3["ln_phi"][:, three] - d["ref_lnphi3"][:, three]).max()
    assert err <= 1e-8, ("ln_phi", err)
    # the published pair of a failed three-phase review is the two-phase answer
    higher = same & (rs == 4)
    if higher.any():
        assert np.abs(out["liquid"][:, higher] - d["ref_x"][:, higher]).max() <= 1e-7
    # cells that were not phase_set_unstable are untouched by the continuation
    other = base["status"] != 2
    for f in ("status", "vapor_fraction", "liquid", "vapor", "ln_k"):
        assert np.array_equal(out[f][..., other], base[f][..., other], equal_nan=True), f
    assert np.all(np.isnan(out3["phase_fraction"][:, ms != 2]))


@pytest.mark.gpu
def test_max3_three_phase_sets_match_the_anchor(gpu_lib):
    mix = synth.three_phase_fixture_mixture()
    p, t, z = synth.make_three_phase_cells(512, seed=21, anchor_fraction=1.0)
    g = gpu_lib.GpuFlash(mix, form="mixed")
    out, out3 = g.solve_max3(p, t, z)
    g.close()
    three = np.nonzero(out3["max3_status"] == 2)[0]
    assert three.size > 100
    assert np.all(out["status"][three] == gpu_lib.FLASH_THREE_PHASE)
    x3 = out3["composition"].reshape(3, 3, -1)
    worst = 0.0
    for c in three:
        for k in range(3):
            worst = max(worst, np.abs(synth.THREE_PHASE_ANCHOR - x3[k, :, c]).max(axis=1).min())
    assert worst <= 1e-9, worst
    assert np.allclose(out3["phase_fraction"][:, three].sum(axis=0), 1.0, atol=1e-13)


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["plain", "batched", "mixed"])
def test_max3_matches_reference_on_six_components(gpu_lib, form):
    """The reference tests' six-component Heringer-2026 sour-gas fixture along
    its P-Z path (tests/golden/max3_heringer_reference.npz).  The path
    crosses phase boundaries on purpose, and 26 of its 429 cells end
    indeterminate.  The plain form may differ on at most one cell, where the
    device's fused multiply-adds move a decision of the finite search (its
    host build, without them, reproduces every status); the work-queue forms
    may differ where their two-phase answer does (at most 1 in 100);
    three-phase sets agree to 1e-9."""
    d = np.load(os.path.join(os.path.dirname(GOLDEN), "max3_heringer_reference.npz"))
    mix = synth.Mixture(d["tc"], d["pc"], d["omega"], d["kij"])
    g = gpu_lib.GpuFlash(mix, form=form)
    out, out3 = g.solve_max3(d["p"], d["t"], d["z"])
    g.close()
    ms, rs = out3["max3_status"], d["ref_max3_status"]
    mismatch = np.nonzero(ms != rs)[0]
    assert mismatch.size <= (1 if form == "plain" else len(ms) // 100)
    same = ms == rs
    assert np.array_equal(out["status"][same], d["ref_published"][same])
    three = same & (rs == 2)
    assert three.sum() > 50
    err = np.abs(out3["composition"][:, three] - d["ref_x3"][:, three]).max()
    assert err <= 1e-9, err


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_max3_with_starts_and_options_matches_reference(gpu_lib, form):
    """mpmc_gpu_flash_solve_hinted_ex on every recorded case of
    tests/golden/max3_hinted_reference.npz (the reference's solve_pr76_pt_max3
    with caller starts and split options): the reference test's 3 -> 2
    recovery, whose first three-phase attempt ends in a phase disappearance
    that a fresh two-phase solve resolves (pr76_max3_robustness_test.cpp:275-356;
    pr76_three_phase.hpp:408-428), the 3 -> 3 base, a zero split-attempt
    quota, an empty feed test and a final start off the feed's support.
    Statuses equal the reference's; the recovery's pair to 1e-12."""
    from tests.test_oracle_max3 import hinted_cases

    for name, (mix, z, h, ref) in hinted_cases().items():
        g = gpu_lib.GpuFlash(mix, form=form)
        out, out3 = g.solve_hinted_ex(np.array([1e6]), np.array([250.0]), z, h)
        g.close()
        assert int(np.ravel(out3["max3_status"])[0]) == int(np.ravel(ref["max3_status"])[0]), name
        published = int(np.ravel(out["status"])[0])
        assert published == int(np.ravel(ref["published"])[0]), name
        if name == "recovery":
            assert np.allclose(np.ravel(out["liquid"]), np.ravel(ref["x"]), rtol=0, atol=1e-12)
            assert np.allclose(np.ravel(out["vapor"]), np.ravel(ref["y"]), rtol=0, atol=1e-12)
        if name == "three":
            assert np.allclose(np.ravel(out3["phase_fraction"]), np.ravel(ref["beta3"]), rtol=0, atol=1e-9)
