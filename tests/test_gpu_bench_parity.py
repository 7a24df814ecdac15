"""The mixed form against the oracle on the bench's own distribution at
65,536 cells (N = 10): the bench generator's cells with 30 % of them placed
within 2 % of a phase-count change pressure of theirs, as the bench places
them.  Every status must match, and the raw ln K, beta, x and y lie within the
band the reference's stopping rule leaves (tests/parity.py)."""

import os
import sys

import numpy as np
import pytest

from mpmc_hnu_gb300 import synth
from tests import parity

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


@pytest.mark.gpu
def test_mixed_form_matches_the_oracle_on_the_bench_distribution(gpu_lib, oracle_lib):
    import bench

    n, ncell, near = 10, 65536, 19661
    mix = synth.make_mixture(n, bench.MIXTURE_SEED)
    p, t, z = synth.make_cells(n, ncell, bench.CELL_SEED)
    g = gpu_lib.GpuFlash(mix, form="mixed")
    p, t, z, placed, _ = bench.place_workload(n, p, t, z, 0, near,
                                              lambda a, b, c: g.solve(a, b, c, fields=["status"])["status"], synth)
    assert placed.mean() > 0.99
    out = g.solve(p, t, z)
    g.close()
    ref = oracle_lib.flash(mix, p, t, z, threads=os.cpu_count() or 8)
    rep = parity.flash_report(out, ref, mix, p, t, z)
    print({k: rep[k] for k in ("n_mismatch", "two_phase", "max", "p99", "polished_max",
                               "polished_band_ratio_max", "lnk_bound_ratio_max", "rr_bound_ratio_max")})
    assert rep["two_phase"] > 10000
    parity.assert_flash_parity(rep, 0)
