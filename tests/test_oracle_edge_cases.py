"""The oracle against the reference on the edge cells of the request contract
(absent components, pure feeds, invalid requests, extreme states).  Runs where
the reference harness is built; the GPU tests then check the device forms
against the oracle on the same cells."""

import numpy as np
import pytest

from mpmc_hnu_gb300 import synth
from tests.edge_cells import edge_cells

# counter rows the harness records (it leaves the RR and root iteration rows 4-5 at zero)
ROWS = [0, 1, 2, 3, 6, 7]


@pytest.mark.parametrize("n", [3, 10, 20])
def test_oracle_matches_reference_on_edge_cells(oracle_lib, n):
    if not oracle_lib.reference_available():
        pytest.skip("reference harness not built here")
    mix = synth.make_mixture(n, 70 + n)
    p, t, z, kinds = edge_cells(n, 80 + n)
    a = oracle_lib.flash(mix, p, t, z, threads=8)
    b = oracle_lib.reference_flash(mix, p, t, z, threads=8)
    for k in a:
        if k not in b:
            continue
        if k == "counters":
            assert np.array_equal(a[k][ROWS], b[k][ROWS]), k
        else:
            assert np.array_equal(a[k], b[k], equal_nan=True), k
    assert (a["status"] == -1).sum() >= 8  # the invalid requests are rejected as such
