"""Comparison helpers between the GPU flash (C ABI) and the CPU oracle."""

from __future__ import annotations

import numpy as np

# GPU output name -> oracle output name
FLASH_MAP = {"vapor_fraction": "beta", "liquid": "x", "vapor": "y", "ln_k": "ln_k",
             "ln_phi_liquid": "ln_phi_l", "ln_phi_vapor": "ln_phi_v", "z_liquid": "z_l", "z_vapor": "z_v"}
SENS_MAP = {"d_ln_k": "dlnk", "d_vapor_fraction": "dbeta", "d_liquid": "dx", "d_vapor": "dy",
            "d_z_liquid": "dzl", "d_z_vapor": "dzv", "d_rho_liquid": "drhol", "d_rho_vapor": "drhov",
            "jac_liquid": "jl", "jac_vapor": "jv"}

# Parity bar for converged two-phase values: relative error
#   |gpu - ref| / max(|ref|, floor)
# with floor = 1e-3 for ln K (relative error is ill-posed as ln K -> 0 near a
# critical point) and 1e-12 elsewhere.
FLASH_TOL = 1e-10
LNK_FLOOR = 1e-3
# Derivatives: 1e-8 relative to max(|ref|, 1e-8 * row scale).
SENS_TOL = 1e-8


def rel_err(a, b, floor):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


def flash_report(gpu: dict, ref: dict, cells=None):
    """Per-field max relative error over cells whose status matches and is
    two-phase (pair fields) or single-phase (feed fields)."""
    gs = np.asarray(gpu["status"])
    rs = np.asarray(ref["status"])
    same = gs == rs
    two = same & (rs == 1)
    one = same & (rs == 0)
    out = {"status_match": float(same.mean()), "n_mismatch": int((~same).sum()),
           "mismatch_cells": np.nonzero(~same)[0][:20].tolist(), "two_phase": int(two.sum()),
           "single_phase": int(one.sum())}
    for g, r in FLASH_MAP.items():
        a = np.asarray(gpu[g], dtype=np.float64)
        b = np.asarray(ref[r], dtype=np.float64)
        if a.ndim == 1:
            a = a[None]
            b = b[None]
        floor = LNK_FLOOR if g == "ln_k" else 1e-12
        errs = []
        if two.any():
            errs.append(rel_err(a[:, two], b[:, two], floor).max())
        if g in ("liquid", "ln_phi_liquid", "z_liquid") and one.any():
            errs.append(rel_err(a[:, one], b[:, one], floor).max())
        out[g] = float(max(errs)) if errs else 0.0
    return out


def sensitivity_report(gpu: dict, ref: dict):
    gs = np.asarray(gpu["sensitivity_status"])
    rs = np.asarray(ref["sens_status"])
    ok = (gs == 0) & (rs == 0)
    out = {"status_match": float((gs == rs).mean()), "both_ok": int(ok.sum())}
    for g, r in SENS_MAP.items():
        a = np.asarray(gpu[g], dtype=np.float64)[:, ok]
        b = np.asarray(ref[r], dtype=np.float64)[:, ok]
        if b.size == 0:
            out[g] = 0.0
            continue
        scale = np.maximum(np.abs(b).max(axis=0, keepdims=True), 1.0)
        out[g] = float((np.abs(a - b) / np.maximum(np.abs(b), 1e-8 * scale)).max())
    return out
