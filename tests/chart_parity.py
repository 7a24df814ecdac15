"""Comparison rules of the selected-phase property chart tests.

Values compare relative to max(1, |reference|).  A Jacobian entry compares
in units of its row: with s_c = |q_c| the scale of chart column c, the error
|dJ_rc| s_c is divided by the row's largest |J_rc'| s_c', so that a
derivative by pressure (in Pa) and one by a mole fraction are judged on the
same footing.  The reference's forward-mode derivatives and the closed form
of the CUDA path agree to rounding of the root's implicit derivative, far
inside these bounds.
"""

from __future__ import annotations

import numpy as np

VALUE_TOL = 1e-10     # relative to max(1, |value|)
JACOBIAN_TOL = 1e-9   # relative to the row's largest column-scaled derivative


def value_error(got, ref) -> float:
    ok = np.isfinite(ref)
    if not ok.any():
        return 0.0
    return float(np.max(np.abs(got[ok] - ref[ok]) / np.maximum(1.0, np.abs(ref[ok]))))


def jacobian_error(got, ref, q) -> float:
    """got, ref [rows, cols, ncell]; q [cols, ncell]."""
    cells = np.isfinite(ref).all(axis=(0, 1))
    if not cells.any():
        return 0.0
    s = np.abs(q[:, cells])[None, :, :]
    g = got[:, :, cells] * s
    r = ref[:, :, cells] * s
    row_scale = np.max(np.abs(r), axis=1, keepdims=True)
    return float(np.max(np.abs(g - r) / np.maximum(row_scale, 1e-300)))


def check_chart(got: dict, ref: dict, q, label: str = "") -> None:
    """Statuses equal, failed cells NaN everywhere, values and Jacobians of the
    others within the tolerances and finite."""
    st_g, st_r = np.asarray(got["status"]), np.asarray(ref["status"])
    assert np.array_equal(st_g, st_r), f"{label}: statuses {st_g} vs {st_r}"
    ok = st_r == 0
    assert np.isnan(got["values"][:, ~ok]).all(), f"{label}: failed cells not NaN-filled"
    assert np.isfinite(got["values"][:, ok]).all(), f"{label}: non-finite values"
    ev = value_error(got["values"][:, ok], ref["values"][:, ok])
    assert ev <= VALUE_TOL, f"{label}: value error {ev:.3e}"
    if "jacobian" in got and got["jacobian"] is not None:
        assert np.isnan(got["jacobian"][:, :, ~ok]).all(), f"{label}: failed cells not NaN-filled"
        assert np.isfinite(got["jacobian"][:, :, ok]).all(), f"{label}: non-finite derivatives"
        ej = jacobian_error(got["jacobian"][:, :, ok], ref["jacobian"][:, :, ok], np.asarray(q)[:, ok])
        assert ej <= JACOBIAN_TOL, f"{label}: Jacobian error {ej:.3e}"
