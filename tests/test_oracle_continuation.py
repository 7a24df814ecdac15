"""The oracle's restatement of the reference's ordered-path continuation
(solve_pr76_pt_continuation, pr76_pt_continuation.hpp:183-306, default
options: the previous accepted point's phase compositions and three-phase set
carried as start hints) against the reference's recorded scan
(tests/golden/continuation_reference.npz) and, where the harness is built,
the live reference.

The recorded scan also shows what the hints change: on these fixture paths
the hint-seeded scan settles some points as three-phase that a fresh solve
leaves indeterminate.  mpmc_hnu_gb300/continuation.py runs the same
hint-seeded scan through mpmc_gpu_flash_solve_hinted
(tests/test_continuation_hints.py, tests/test_gpu_continuation.py)."""

import os

import numpy as np
import pytest

from mpmc_hnu_gb300 import synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "continuation_reference.npz")


def test_oracle_continuation_matches_recorded_reference(oracle_lib):
    d = np.load(GOLDEN)
    mix = synth.three_phase_fixture_mixture()
    ms = oracle_lib.continuation(mix, d["p"], d["t"], d["z"], threads=8)
    assert np.array_equal(ms, d["ref_max3_status"])
    differ = d["ref_max3_status"] != d["ref_cold_max3_status"]
    # the hints only ever settle more points (indeterminate -> three phases)
    assert np.all(d["ref_cold_max3_status"][differ] == 5) and np.all(d["ref_max3_status"][differ] == 2)


def test_oracle_continuation_matches_live_reference(oracle_lib):
    if not oracle_lib.reference_available():
        pytest.skip("reference harness not built here")
    mix = synth.three_phase_fixture_mixture()
    _, _, z = synth.make_three_phase_cells(48, seed=61, anchor_fraction=0.5)
    p = np.tile(np.exp(np.linspace(np.log(3e5), np.log(3e6), 8)), (48, 1))
    t = np.full_like(p, 245.0)
    ms_ref, _ = oracle_lib.reference_continuation(mix, p, t, z, threads=8)
    assert np.array_equal(oracle_lib.continuation(mix, p, t, z, threads=8), ms_ref)
