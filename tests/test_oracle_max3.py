"""The oracle's max-3-phase restatement against the reference.

1. Against the recorded outputs of the reference's solve_pr76_pt_max3
   (tests/golden/max3_reference.npz, written by make_max3_golden.py from the
   unmodified reference headers): statuses, attempt counts and every phase
   field bit-identical.
2. Against the independent anchor of the reference's own tests: at 1 MPa and
   250 K every three-phase answer of a feed inside the fixture's tie triangle
   has the anchor's three phase compositions (synthetic_fixture.hpp:63-72),
   within 1e-10.
3. Where the reference harness is built here, against the live reference on
   freshly drawn cells.
"""

import os

import numpy as np
import pytest

from mpmc_hnu_gb300 import synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "max3_reference.npz")


def _same(a, b):
    return np.array_equal(np.asarray(a), np.asarray(b), equal_nan=True)


def test_oracle_max3_matches_recorded_reference(oracle_lib):
    d = np.load(GOLDEN)
    mix = synth.three_phase_fixture_mixture()
    out = oracle_lib.max3(mix, d["p"], d["t"], d["z"], threads=8)
    counts = np.bincount(d["ref_max3_status"] + 1, minlength=7)
    assert counts[3] > 100 and counts[5] > 0  # three-phase cells and failed reviews are covered
    for k, v in out.items():
        assert _same(v, d[f"ref_{k}"]), k


def test_three_phase_answers_match_the_anchor(oracle_lib):
    mix = synth.three_phase_fixture_mixture()
    p, t, z = synth.make_three_phase_cells(400, seed=21, anchor_fraction=1.0)
    out = oracle_lib.max3(mix, p, t, z, threads=8)
    three = np.nonzero(out["max3_status"] == 2)[0]
    assert three.size > 100
    x3 = out["x3"].reshape(3, 3, -1)
    worst = 0.0
    for c in three:
        for k in range(3):
            worst = max(worst, np.abs(synth.THREE_PHASE_ANCHOR - x3[k, :, c]).max(axis=1).min())
    assert worst <= 1e-10, worst
    # published three-phase sets are material-balanced and sum to one
    b = out["beta3"][:, three]
    assert np.allclose(b.sum(axis=0), 1.0, atol=1e-14)
    assert np.all(out["published"][three] == 4)


def test_oracle_max3_matches_live_reference(oracle_lib):
    if not oracle_lib.reference_available():
        pytest.skip("reference harness not built here")
    mix = synth.three_phase_fixture_mixture()
    p, t, z = synth.make_three_phase_cells(600, seed=31)
    a = oracle_lib.max3(mix, p, t, z, threads=8)
    b = oracle_lib.reference_max3(mix, p, t, z, threads=8)
    for k in a:
        assert _same(a[k], b[k]), k


def test_oracle_max3_matches_recorded_reference_on_six_components(oracle_lib):
    """The reference tests' six-component Heringer-2026 sour-gas fixture along
    its own P-Z path (tests/golden/max3_heringer_reference.npz, written by
    make_heringer_golden.py): every field bit-identical."""
    d = np.load(os.path.join(os.path.dirname(GOLDEN), "max3_heringer_reference.npz"))
    mix = synth.Mixture(d["tc"], d["pc"], d["omega"], d["kij"])
    out = oracle_lib.max3(mix, d["p"], d["t"], d["z"], threads=8)
    counts = np.bincount(d["ref_max3_status"] + 1, minlength=7)
    assert counts[1] > 50 and counts[2] > 100 and counts[3] > 50
    for k, v in out.items():
        assert _same(v, d[f"ref_{k}"]), k
