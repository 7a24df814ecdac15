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


HINTED = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "max3_hinted_reference.npz")


def hinted_cases():
    """The recorded hinted max-3-phase cases (make_max3_hinted_golden.py):
    name -> (mixture, z [n, 1], start hints, reference outputs)."""
    d = np.load(HINTED)
    cases = {}
    for name in d["cases"]:
        name = str(name)
        model = str(d[f"{name}_model"])
        n = len(d[f"{model}_tc"])
        mix = synth.Mixture(d[f"{model}_tc"], d[f"{model}_pc"], d[f"{model}_omega"],
                            d[f"{model}_kij"].reshape(n, n))
        pre = f"{name}_hint_"
        h = {k[len(pre):]: d[k] for k in d.files if k.startswith(pre)}
        h["initial_automatic_starts"] = bool(h["initial_automatic_starts"])
        h["max_split_attempts"] = int(h["max_split_attempts"])
        pre = f"{name}_ref_"
        ref = {k[len(pre):]: d[k] for k in d.files if k.startswith(pre)}
        cases[name] = (mix, d[f"{name}_z"], h, ref)
    return cases


def test_oracle_max3_with_starts_and_options_matches_recorded_reference(oracle_lib):
    """Caller starts and split options: the reference test's 3 -> 2 recovery
    through a phase disappearance and a fresh two-phase neighbour
    (pr76_max3_robustness_test.cpp:275-356), the 3 -> 3 continuation base, a
    zero split-attempt quota, an empty search and a final start off the
    feed's support, bit-identical to the recorded reference."""
    cases = hinted_cases()
    mix, z, h, ref = cases["recovery"]
    # the recovery publishes the fresh two-phase neighbour of its first attempt
    first = {name: {k: int(np.ravel(c[3][k])[0]) for k in ("max3_status", "published", "attempts")}
             for name, c in cases.items()}
    assert first["recovery"] == {"max3_status": 1, "published": 1, "attempts": 1}
    assert first["three"]["max3_status"] == 2 and first["budget"]["max3_status"] == 5
    assert first["no_starts"]["max3_status"] == -1 and first["support"]["max3_status"] == -1
    for name, (mix, z, h, ref) in cases.items():
        out = oracle_lib.max3_hinted(mix, np.array([1e6]), np.array([250.0]), z, h, threads=1)
        for k, v in out.items():
            assert _same(v, ref[k]), (name, k)


def test_oracle_max3_with_starts_matches_live_reference(oracle_lib):
    if not oracle_lib.reference_available():
        pytest.skip("reference harness not built here")
    for name, (mix, z, h, ref) in hinted_cases().items():
        live = oracle_lib.reference_max3_hinted(mix, np.array([1e6]), np.array([250.0]), z, h, threads=1)
        out = oracle_lib.max3_hinted(mix, np.array([1e6]), np.array([250.0]), z, h, threads=1)
        for k, v in out.items():
            assert _same(v, live[k]), (name, k)
