"""Comparison helpers between the GPU flash (C ABI) and the CPU oracle.

Parity bar, per cell:

1. Phase-set status identical (single / two-phase / phase-set unstable /
   indeterminate / invalid).
2. Two-phase cells converge to the SAME equilibrium: the GPU's and the
   oracle's ln K, each Newton-polished by the oracle to |F| ~ 1e-15, agree
   within POLISHED_TOL relative (ln K floor LNK_FLOOR) -- typically ~1e-12.
   The polished beta, x and y agree within POLISHED_TOL relative (beta floor
   BETA_FLOOR) plus that ln K tolerance carried through the Rachford-Rice
   solution (`rr_band`): near a critical point d beta / d ln K grows large,
   and two ln K that agree to 2e-11 give betas 1.5e-10 apart.
3. The raw (unpolished) ln K agree within
       FLASH_TOL * max(|ln K|, LNK_FLOOR) + 4 * 1e-11 * ||(dF/dlnK)^-1||_inf,
   i.e. 1e-10 relative plus the band that the reference's own stopping rule
   |F|_inf <= 1e-11 (pt_split.hpp:31, :351) leaves around the exact root for
   two independent runs.  The reference compiled with and without FMA
   contraction differs from itself by the same amount.
4. Raw beta, x and y within the same band carried through the
   Rachford-Rice solution: |x_gpu - x_ref|_i <= sum_j |dx_i / d ln K_j| b_j
   + FLASH_TOL |x_i| with b_j the ln K band of 3. (likewise y and beta), the
   derivatives taken by differences of the Rachford-Rice solution at the
   oracle's ln K (`rr_band`).  Raw ln phi and Z: max <= RAW_MAX (ln phi
   relative to max(|ln phi|, 1)); the p99 is reported.

Sensitivities are compared at the same accepted state (the oracle
differentiates the GPU's state): see `sensitivity_report`.
"""

from __future__ import annotations

import numpy as np

# GPU output name -> oracle output name
FLASH_MAP = {"vapor_fraction": "beta", "liquid": "x", "vapor": "y", "ln_k": "ln_k",
             "ln_phi_liquid": "ln_phi_l", "ln_phi_vapor": "ln_phi_v", "z_liquid": "z_l", "z_vapor": "z_v"}
SENS_MAP = {"d_ln_k": "dlnk", "d_vapor_fraction": "dbeta", "d_liquid": "dx", "d_vapor": "dy",
            "d_z_liquid": "dzl", "d_z_vapor": "dzv", "d_rho_liquid": "drhol", "d_rho_vapor": "drhov",
            "jac_liquid": "jl", "jac_vapor": "jv"}

FLASH_TOL = 1e-10
# Polished beta is compared relative to max(beta, BETA_FLOOR): a cell within a
# hair of its phase boundary has beta -> 0, and there d beta / d ln K * beta^-1
# grows without bound, so two ln K that agree to 1e-12 still give betas whose
# relative difference is large while the absolute one stays ~1e-13.
BETA_FLOOR = 1e-3
# ln phi_i = 0 at the ideal-gas limit, so a component with ln phi_i near zero
# carries the same absolute error from the stopping band as any other: ln phi
# is compared relative to max(|ln phi|, 1).
LNPHI_FLOOR = 1.0
POLISHED_TOL = 1e-10
LNK_FLOOR = 1e-3
STOP_TOL = 1e-11
RAW_MAX = 1e-7
# Derivatives: 1e-8 normwise relative per derivative column, widened by the
# forward-error bound of the linear solve with dF/dln K: a cell passes when
# its error is below SENS_TOL + SENS_COND_FACTOR * eps / rcond(dF/dln K).
SENS_TOL = 1e-8
SENS_COND_FACTOR = 64.0
EPS = float(np.finfo(np.float64).eps)


def rel_err(a, b, floor):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


def _rows(a):
    a = np.asarray(a, dtype=np.float64)
    return a[None] if a.ndim == 1 else a


def rr_solution(z, lnk):
    """Rachford-Rice solution (beta, x, y) of each cell (columns) at ln K, by
    bisection on the feasible interval of beta (test arithmetic, FP64)."""
    k = np.exp(lnk)
    lo = np.full(z.shape[1], -1e300)
    hi = np.full(z.shape[1], 1e300)
    km = k - 1.0
    with np.errstate(divide="ignore"):
        # 1 + beta (K - 1) > 0 for every component present
        lo = np.max(np.where((km > 0) & (z > 0), -1.0 / np.where(km > 0, km, 1.0), -np.inf), axis=0)
        hi = np.min(np.where((km < 0) & (z > 0), -1.0 / np.where(km < 0, km, -1.0), np.inf), axis=0)
    a, b = lo + 1e-15 * np.maximum(1, np.abs(lo)), hi - 1e-15 * np.maximum(1, np.abs(hi))
    for _ in range(200):
        m = 0.5 * (a + b)
        f = np.sum(z * km / (1.0 + m * km), axis=0)
        a = np.where(f > 0, m, a)
        b = np.where(f > 0, b, m)
    beta = 0.5 * (a + b)
    x = z / (1.0 + beta * km)
    y = k * x
    return beta, x / x.sum(axis=0), y / y.sum(axis=0)


def rr_band(z, lnk, band):
    """First-order bounds on beta, x and y from ln K errors up to `band`
    (per component and cell): sum_j |d(.)/d ln K_j| band_j, by central
    differences of the Rachford-Rice solution."""
    n = lnk.shape[0]
    bb = np.zeros(lnk.shape[1])
    bx = np.zeros_like(lnk)
    by = np.zeros_like(lnk)
    for j in range(n):
        h = 1e-6 * np.maximum(1.0, np.abs(lnk[j]))
        up, dn = lnk.copy(), lnk.copy()
        up[j] += h
        dn[j] -= h
        b1, x1, y1 = rr_solution(z, up)
        b0, x0, y0 = rr_solution(z, dn)
        bb += np.abs((b1 - b0) / (2 * h)) * band[j]
        bx += np.abs((x1 - x0) / (2 * h)) * band[j]
        by += np.abs((y1 - y0) / (2 * h)) * band[j]
    return bb, bx, by


def flash_report(gpu: dict, ref: dict, mix=None, p=None, t=None, z=None):
    """Status agreement and per-field errors; with (mix, p, t, z) also the
    polished comparison and the conditioning-aware ln K bound."""
    gs = np.asarray(gpu["status"])
    rs = np.asarray(ref["status"])
    same = gs == rs
    two = same & (rs == 1)
    one = same & (rs == 0)
    out = {"cells": int(len(rs)), "status_match": float(same.mean()), "n_mismatch": int((~same).sum()),
           "mismatch_cells": np.nonzero(~same)[0][:20].tolist(), "two_phase": int(two.sum()),
           "single_phase": int(one.sum()), "max": {}, "p99": {}}
    for g, r in FLASH_MAP.items():
        a, b = _rows(gpu[g]), _rows(ref[r])
        floor = LNK_FLOOR if g == "ln_k" else (LNPHI_FLOOR if g.startswith("ln_phi") else 1e-12)
        per_cell = np.zeros(len(rs))
        if two.any():
            per_cell[two] = rel_err(a[:, two], b[:, two], floor).max(axis=0)
        if g in ("liquid", "ln_phi_liquid", "z_liquid") and one.any():
            per_cell[one] = rel_err(a[:, one], b[:, one], floor).max(axis=0)
        sel = two | (one if g in ("liquid", "ln_phi_liquid", "z_liquid") else False)
        vals = per_cell[sel]
        out["max"][g] = float(vals.max()) if vals.size else 0.0
        out["p99"][g] = float(np.percentile(vals, 99)) if vals.size else 0.0
    if mix is not None and two.any():
        from oracle import pyoracle

        pg = pyoracle.polish(mix, p, t, z, gpu["ln_k"], two)
        pr = pyoracle.polish(mix, p, t, z, ref["ln_k"], two)
        ok = two & np.isfinite(pg["beta"]) & np.isfinite(pr["beta"])
        out["polish_failed"] = int((two & ~ok).sum())
        out["polished_max"] = {
            "ln_k": float(rel_err(pg["ln_k"][:, ok], pr["ln_k"][:, ok], LNK_FLOOR).max()) if ok.any() else 0.0,
            "beta": float(rel_err(pg["beta"][ok], pr["beta"][ok], BETA_FLOOR).max()) if ok.any() else 0.0,
            "x": float(rel_err(pg["x"][:, ok], pr["x"][:, ok], 1e-300).max()) if ok.any() else 0.0,
            "y": float(rel_err(pg["y"][:, ok], pr["y"][:, ok], 1e-300).max()) if ok.any() else 0.0,
        }
        if ok.any():
            zp = np.asarray(z, dtype=np.float64)[:, ok]
            zp = zp / zp.sum(axis=0)
            lk = pr["ln_k"][:, ok]
            pb, px, py = rr_band(zp, lk, POLISHED_TOL * np.maximum(np.abs(lk), LNK_FLOOR))
            floors = {"beta": BETA_FLOOR, "x": 1e-300, "y": 1e-300}
            band = {"beta": pb, "x": px, "y": py}
            out["polished_band_ratio_max"] = {
                k: float((np.abs(pg[k][..., ok] - pr[k][..., ok]) /
                          (band[k] + POLISHED_TOL * np.maximum(np.abs(pr[k][..., ok]), floors[k]))).max())
                for k in ("beta", "x", "y")}
        a, b = _rows(gpu["ln_k"]), _rows(ref["ln_k"])
        bound = FLASH_TOL * np.maximum(np.abs(b), LNK_FLOOR) + 4 * STOP_TOL * np.nan_to_num(pr["ainv"], nan=0.0)
        ratio = np.abs(a - b) / bound
        out["lnk_bound_ratio_max"] = float(ratio[:, ok].max()) if ok.any() else 0.0
        if ok.any():
            # beta, x and y: the same band through the Rachford-Rice solution
            zz = np.asarray(z, dtype=np.float64)[:, ok]
            zz = zz / zz.sum(axis=0)
            bb, bx, by = rr_band(zz, b[:, ok], bound[:, ok])
            ratios = {}
            for g, r, bd in (("vapor_fraction", "beta", bb), ("liquid", "x", bx), ("vapor", "y", by)):
                ga, ra = _rows(gpu[g])[:, ok], _rows(ref[r])[:, ok]
                ratios[r] = float((np.abs(ga - ra) / (bd + FLASH_TOL * np.abs(ra) + 1e-300)).max())
            out["rr_bound_ratio_max"] = ratios
    return out


def assert_flash_parity(rep: dict, allowed: int = 0) -> None:
    assert rep["n_mismatch"] <= allowed, rep
    for g in ("ln_phi_liquid", "ln_phi_vapor", "z_liquid", "z_vapor"):
        assert rep["max"][g] <= RAW_MAX, (g, rep)
    if "polished_max" in rep:
        assert rep["polish_failed"] == 0, rep
        assert rep["polished_max"]["ln_k"] <= POLISHED_TOL, rep
        for k, v in rep.get("polished_band_ratio_max", {}).items():
            assert v <= 1.0, (k, rep)
        assert rep["lnk_bound_ratio_max"] <= 1.0, rep
        for k, v in rep.get("rr_bound_ratio_max", {}).items():
            assert v <= 1.0, (k, rep)


def sensitivity_report(gpu: dict, ref: dict, rcond=None):
    """Normwise relative error of every derivative direction: per cell and per
    column j (one chart variable q_j), max_i |got_ij - ref_ij| / max_i |ref_ij|.

    Derivatives of ln K come from a linear solve with A = dF/dln K, so every
    entry of a column carries an absolute error of order cond(A) * eps times
    the column's norm; entries far below the norm have no relative accuracy of
    their own in either implementation.  `elementwise` reports the entrywise
    relative error as well (with a floor of 1e-8 of the column scale).  With
    `rcond` (the oracle's reciprocal condition estimate of A per cell),
    `bound_ratio` is the error over SENS_TOL + SENS_COND_FACTOR * eps / rcond."""
    gs = np.asarray(gpu["sensitivity_status"])
    rs = np.asarray(ref["sens_status"])
    ok = (gs == 0) & (rs == 0)
    out = {"status_match": float((gs == rs).mean()), "both_ok": int(ok.sum()), "max": {}}
    for g, r in SENS_MAP.items():
        a = np.asarray(gpu[g], dtype=np.float64)[:, ok]
        b = np.asarray(ref[r], dtype=np.float64)[:, ok]
        if b.size == 0:
            out["max"][g] = 0.0
            continue
        rows_total = b.shape[0]
        n = int(np.asarray(gpu["d_vapor_fraction"]).shape[0]) - 1  # q = n + 1
        cols = n + 2 if g.startswith("jac") else n + 1
        a = a.reshape(rows_total // cols, cols, -1)
        b = b.reshape(rows_total // cols, cols, -1)
        scale = np.abs(b).max(axis=0, keepdims=True)
        err = np.abs(a - b) / np.maximum(scale, 1e-300)
        out["max"][g] = float(err.max())
        if rcond is not None:
            # a linear solve with dF/dln K loses cond(A) * eps of forward accuracy
            bound = SENS_TOL + SENS_COND_FACTOR * EPS / rcond[ok]
            out.setdefault("bound_ratio", {})[g] = float((err.max(axis=(0, 1)) / bound).max())
        out.setdefault("elementwise", {})[g] = float(
            (np.abs(a - b) / np.maximum(np.abs(b), 1e-8 * scale + 1e-300)).max())
        w = np.unravel_index(int(np.argmax(err)), err.shape)
        out.setdefault("worst", {})[g] = {"row": int(w[0]), "col": int(w[1]), "got": float(a[w]),
                                          "ref": float(b[w]), "col_scale": float(scale[(0, w[1], w[2])])}
    return out
