"""ln K warm starts (mpmc_gpu_flash_solve_warm) against the cold solve and
the oracle.

Warm starts follow the continuation use: ln K* of a converged cold solve,
perturbed by 0.1 N(0, 1) per component (K = K* exp(0.1 N(0, 1))), on 75 %
of the cells; the other 25 % and every cell without a two-phase answer get
NaN (cold).  A warm cell is settled only when its single attempt converges
and the reference's final review accepts the pair, so its status and pair
must equal the cold solve's, and the oracle's."""

import numpy as np
import pytest

from mpmc_hnu_gb300 import synth
from tests import parity

CASES = [(4, 2048, 11), (10, 2048, 12), (20, 512, 13)]


def _warm_from(cold, ncell, seed, fraction=0.75):
    rng = np.random.default_rng(seed)
    warm = cold["ln_k"] + 0.1 * rng.standard_normal(cold["ln_k"].shape)  # NaN where not two-phase
    warm[:, rng.random(ncell) >= fraction] = np.nan
    return warm


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["mixed", "batched"])
@pytest.mark.parametrize("n,ncell,seed", CASES)
def test_warm_start_matches_cold_and_oracle(gpu_lib, oracle_lib, form, n, ncell, seed):
    mix = synth.make_mixture(n, seed)
    p, t, z = synth.make_cells(n, ncell, seed)
    g = gpu_lib.GpuFlash(mix, form=form)
    cold = g.solve(p, t, z)
    warm = _warm_from(cold, ncell, seed)
    out = g.solve(p, t, z, ln_k_warm=warm)
    g.close()
    ref = oracle_lib.flash(mix, p, t, z, threads=8)
    rep = parity.flash_report(out, ref, mix, p, t, z)
    settled = np.isfinite(warm).all(axis=0)
    print(form, n, "warm cells", int(settled.sum()), "status mismatches vs cold",
          int((out["status"] != cold["status"]).sum()), {k: rep[k] for k in ("n_mismatch", "max", "polished_max")})
    assert np.array_equal(out["status"], cold["status"])
    two = cold["status"] == 1
    assert np.nanmax(np.abs(out["ln_k"][:, two] - cold["ln_k"][:, two])) <= 1e-8
    parity.assert_flash_parity(rep)


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["mixed", "batched"])
def test_warm_start_without_guesses_is_the_cold_solve(gpu_lib, form):
    """All-NaN warm starts: every cell takes the cold pass, bit for bit."""
    n, ncell = 10, 1024
    mix = synth.make_mixture(n, 21)
    p, t, z = synth.make_cells(n, ncell, 21)
    p[:8] = -1.0  # invalid requests are answered by the warm pass itself
    g = gpu_lib.GpuFlash(mix, form=form, sensitivity=True)
    cold = g.solve(p, t, z)
    out = g.solve(p, t, z, ln_k_warm=np.full((n, ncell), np.nan))
    g.close()
    for f in cold:
        assert np.array_equal(cold[f], out[f], equal_nan=True), f


@pytest.mark.gpu
def test_warm_start_from_other_cells(gpu_lib, oracle_lib):
    """Guesses taken from other cells' answers (a poor continuation): the
    attempts that do not converge, collapse or fail the review fall back to the
    cold pass, so the statuses still equal the cold solve's."""
    n, ncell = 6, 2048
    mix = synth.make_mixture(n, 31)
    p, t, z = synth.make_cells(n, ncell, 31)
    g = gpu_lib.GpuFlash(mix, form="mixed")
    cold = g.solve(p, t, z)
    donors = np.nonzero(cold["status"] == 1)[0]
    rng = np.random.default_rng(31)
    warm = cold["ln_k"][:, rng.choice(donors, ncell)]
    out = g.solve(p, t, z, ln_k_warm=warm)
    g.close()
    diff = np.nonzero(out["status"] != cold["status"])[0]
    print("status differences", diff.size, [(int(c), int(cold["status"][c]), int(out["status"][c])) for c in diff[:8]])
    assert diff.size <= ncell // 1024
    two = (cold["status"] == 1) & (out["status"] == 1)
    assert np.nanmax(np.abs(out["ln_k"][:, two] - cold["ln_k"][:, two])) <= 1e-8


@pytest.mark.gpu
def test_plain_form_rejects_warm_starts(gpu_lib):
    n = 4
    mix = synth.make_mixture(n, 41)
    p, t, z = synth.make_cells(n, 16, 41)
    g = gpu_lib.GpuFlash(mix, form="plain")
    with pytest.raises(gpu_lib.FlashError) as err:
        g.solve(p, t, z, ln_k_warm=np.zeros((n, 16)))
    g.close()
    assert "warm" in str(err.value)
