"""Accuracy on near-critical cells: 20 % of the cells at T = T_pc (1 +- 1 %)
(Kay's rule) and p log-uniform on [10, 40] MPa, the rest log-uniform.

The plain FP64 form and the FP64 work-queue form must match the oracle's
phase status on every cell, and so must the mixed form except on the cells
measured to sit on a knife edge of the reference itself: at N = 10 one cell
of these 16,384 (cell 4933), whose reference final review ends indeterminate
because its trial from the feed stops with a failed line search at TPD
-2.5e-13, at the round-off level of the raw pair's common tangent; the mixed
form reviews the Newton-polished pair, on which that trial converges.  (On
65,536 cells of the same draw the mixed form differs on 5: that one, and four
whose reference attempts end within 30 iterations of the 512-iteration limit
or stall at |r| ~ 3e-9.)  Every matched two-phase cell converges to the same
equilibrium (polished ln K within 1e-10), and the raw ln K, beta, x and y lie
within the band the reference's stopping rule leaves (tests/parity.py).
"""

import numpy as np
import pytest

from mpmc_hnu_gb300 import synth
from tests import parity


@pytest.mark.gpu
@pytest.mark.parametrize("n,ncell", [(10, 16384), (20, 4096)])
def test_near_critical_cells(gpu_lib, oracle_lib, n, ncell):
    mix = synth.make_mixture(n, 3000 + n)
    p, t, z = synth.make_near_critical_cells(mix, ncell, 4000 + n)
    ref = oracle_lib.flash(mix, p, t, z, threads=8)
    for form, allowed in (("plain", 0), ("batched", 0), ("mixed", 1 if n == 10 else 0)):
        g = gpu_lib.GpuFlash(mix, form=form)
        out = g.solve(p, t, z)
        g.close()
        rep = parity.flash_report(out, ref, mix, p, t, z)
        print(form, n, {k: rep[k] for k in ("n_mismatch", "max", "p99", "polished_max",
                                               "polished_band_ratio_max")})
        parity.assert_flash_parity(rep, allowed)
