"""Every form against the oracle on the edge cells of the request contract:
absent components (z_i = 0), pure feeds, two-component subsets, invalid
requests (p or T not finite and positive, a negative or above-one fraction,
a feed sum off by 1e-2; a sum within 64 eps is accepted), extreme pressures
and temperatures, at N = 3, 10 and 20; and an empty batch."""

import numpy as np
import pytest

from mpmc_hnu_gb300 import synth
from tests import parity
from tests.edge_cells import edge_cells


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["plain", "batched", "mixed"])
@pytest.mark.parametrize("n", [3, 10, 20])
def test_edge_cells_match_oracle(gpu_lib, oracle_lib, form, n):
    mix = synth.make_mixture(n, 70 + n)
    p, t, z, kinds = edge_cells(n, 80 + n)
    ref = oracle_lib.flash(mix, p, t, z, threads=8)
    g = gpu_lib.GpuFlash(mix, form=form)
    out = g.solve(p, t, z)
    g.close()
    bad = np.nonzero(out["status"] != ref["status"])[0]
    assert bad.size == 0, [(int(c), kinds[c], int(ref["status"][c]), int(out["status"][c])) for c in bad]
    invalid = ref["status"] == -1
    assert np.all(np.isnan(out["vapor_fraction"][invalid]))
    rep = parity.flash_report(out, ref, mix, p, t, z)
    print(form, n, {k: rep[k] for k in ("two_phase", "single_phase", "max")})
    parity.assert_flash_parity(rep)


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["plain", "batched", "mixed"])
def test_empty_batch(gpu_lib, form):
    mix = synth.make_mixture(4, 5)
    g = gpu_lib.GpuFlash(mix, form=form, sensitivity=True)
    out = g.solve(np.zeros(0), np.zeros(0), np.zeros((4, 0)))
    g.close()
    assert all(v.shape[-1] == 0 for v in out.values())
