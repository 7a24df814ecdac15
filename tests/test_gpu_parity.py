"""GPU flash vs the CPU oracle on seeded synthetic cells (through the C ABI)."""

import numpy as np
import pytest

from mpmc_hnu_gb300 import synth
from tests import parity

CASES = [(3, 256, 5), (4, 256, 6), (6, 512, 1), (10, 384, 2), (12, 192, 3), (20, 96, 4)]


@pytest.mark.gpu
@pytest.mark.parametrize("n,ncell,seed", CASES)
@pytest.mark.parametrize("form", ["plain", "batched", "mixed"])
def test_flash_matches_oracle(gpu_lib, oracle_lib, n, ncell, seed, form):
    mix = synth.make_mixture(n, seed)
    p, t, z = synth.make_cells(n, ncell, seed)
    ref = oracle_lib.flash(mix, p, t, z, threads=8)
    g = gpu_lib.GpuFlash(mix, form=form)
    out = g.solve(p, t, z)
    rep = parity.flash_report(out, ref, mix, p, t, z)
    print(form, n, rep)
    parity.assert_flash_parity(rep)
