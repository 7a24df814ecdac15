"""ctypes loader for the CPU oracle (test infrastructure).

Only tests, the smoke check and the benchmark's CPU-baseline leg use this
module.  `flash()` runs oracle/_build/libpr76_oracle.so (the C++ restatement of
the reference algorithm); `reference_flash()` runs oracle/_ref/libpr76_ref.so
(the reference headers themselves), which exists only where the reference
sources were available at build time.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libpr76_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libpr76_ref.so")

FIELDS = [
    ("status", ctypes.c_void_p), ("beta", ctypes.c_void_p), ("x", ctypes.c_void_p),
    ("y", ctypes.c_void_p), ("ln_k", ctypes.c_void_p), ("ln_phi_l", ctypes.c_void_p),
    ("ln_phi_v", ctypes.c_void_p), ("z_l", ctypes.c_void_p), ("z_v", ctypes.c_void_p),
    ("counters", ctypes.c_void_p), ("sens_status", ctypes.c_void_p), ("dlnk", ctypes.c_void_p),
    ("dbeta", ctypes.c_void_p), ("dx", ctypes.c_void_p), ("dy", ctypes.c_void_p),
    ("dzl", ctypes.c_void_p), ("dzv", ctypes.c_void_p), ("drhol", ctypes.c_void_p),
    ("drhov", ctypes.c_void_p), ("jl", ctypes.c_void_p), ("jv", ctypes.c_void_p),
    ("rcond", ctypes.c_void_p),  # oracle only: the reference harness leaves it unset
]

COUNTER_NAMES = ["init_evals", "split_evals", "final_evals", "split_iters", "rr_iters",
                 "root_bisections", "attempts", "trial_iters"]


class _Out(ctypes.Structure):
    _fields_ = FIELDS


_built = False
# Where the reference sources lie, if at all: MPMC_REFERENCE_ROOT, else the
# checkout this recipe was written against.  The tests and the golden-vector
# scripts take it from here; oracle/Makefile has the same default.
REFERENCE_ROOT = os.environ.get("MPMC_REFERENCE_ROOT", "/root/reference")


def build(force: bool = False) -> None:
    """Compile the oracle (always) and the reference harness (if sources
    exist); make rebuilds whatever is older than its source."""
    global _built
    if _built and not force:
        return
    subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    if os.path.isdir(os.path.join(REFERENCE_ROOT, "modules")):
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", f"REFERENCE_ROOT={REFERENCE_ROOT}"])
    _built = True


_libs: dict[str, ctypes.CDLL] = {}


def _lib(path: str) -> ctypes.CDLL:
    if path not in _libs:
        _libs[path] = ctypes.CDLL(path)
    return _libs[path]


def reference_available() -> bool:
    build()
    return os.path.exists(REF_SO)


def _alloc(n: int, ncell: int, sens: bool):
    q = n + 1
    out = {
        "status": np.full(ncell, -9, np.int32), "beta": np.empty(ncell),
        "x": np.empty((n, ncell)), "y": np.empty((n, ncell)), "ln_k": np.empty((n, ncell)),
        "ln_phi_l": np.empty((n, ncell)), "ln_phi_v": np.empty((n, ncell)),
        "z_l": np.empty(ncell), "z_v": np.empty(ncell), "counters": np.zeros((8, ncell), np.int64),
    }
    if sens:
        out.update({
            "sens_status": np.full(ncell, -9, np.int32), "dlnk": np.empty((n * q, ncell)),
            "dbeta": np.empty((q, ncell)), "dx": np.empty((n * q, ncell)), "dy": np.empty((n * q, ncell)),
            "dzl": np.empty((q, ncell)), "dzv": np.empty((q, ncell)), "drhol": np.empty((q, ncell)),
            "drhov": np.empty((q, ncell)), "jl": np.empty(((n + 1) * (n + 2), ncell)),
            "jv": np.empty(((n + 1) * (n + 2), ncell)), "rcond": np.full(ncell, np.nan),
        })
    s = _Out()
    for name, _ in FIELDS:
        setattr(s, name, out[name].ctypes.data if name in out else None)
    return out, s


def _run(fn_name: str, so: str, mix, p, t, z, threads: int, sens: bool):
    tc, pc, omega, kij = (np.ascontiguousarray(a, dtype=np.float64) for a in mix.as_tuple())
    p = np.ascontiguousarray(p, dtype=np.float64)
    t = np.ascontiguousarray(t, dtype=np.float64)
    z = np.ascontiguousarray(z, dtype=np.float64)
    n, ncell = z.shape
    out, s = _alloc(n, ncell, sens)
    fn = getattr(_lib(so), fn_name)
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 4 + [ctypes.c_int64] + [ctypes.c_void_p] * 3 + \
        [ctypes.c_int, ctypes.c_int, ctypes.POINTER(_Out)]
    rc = fn(n, tc.ctypes.data, pc.ctypes.data, omega.ctypes.data, kij.ctypes.data, ncell,
            p.ctypes.data, t.ctypes.data, z.ctypes.data, threads, int(sens), ctypes.byref(s))
    if rc != 0:
        raise RuntimeError(f"{fn_name} returned {rc}")
    return out


def flash(mix, p, t, z, threads: int = 1, sens: bool = False):
    """CPU restatement of the reference flash; see oracle/pr76_flash_oracle.cpp."""
    build()
    return _run("oracle_flash_batch", ORACLE_SO, mix, p, t, z, threads, sens)


def reference_flash(mix, p, t, z, threads: int = 1, sens: bool = False):
    """The reference headers themselves (only where they were compiled)."""
    if not reference_available():
        raise FileNotFoundError(REF_SO)
    return _run("ref_flash_batch", REF_SO, mix, p, t, z, threads, sens)


def reference_backend(mix, p, t, z, threads: int = 1):
    """Pr76PtFlashBackend::solve per cell: (PtPhaseSetStatus, accepted phase count)."""
    tc, pc, omega, kij = (np.ascontiguousarray(a, dtype=np.float64) for a in mix.as_tuple())
    z = np.ascontiguousarray(z, dtype=np.float64)
    n, ncell = z.shape
    status = np.empty(ncell, np.int32)
    count = np.empty(ncell, np.int32)
    fn = _lib(REF_SO).ref_backend_batch
    fn.restype = ctypes.c_int
    p = np.ascontiguousarray(p, dtype=np.float64)
    t = np.ascontiguousarray(t, dtype=np.float64)
    fn(ctypes.c_int(n), *(ctypes.c_void_p(a.ctypes.data) for a in (tc, pc, omega, kij)), ctypes.c_int64(ncell),
       *(ctypes.c_void_p(a.ctypes.data) for a in (p, t, z)), ctypes.c_int(threads),
       ctypes.c_void_p(status.ctypes.data), ctypes.c_void_p(count.ctypes.data))
    return status, count


def polish(mix, p, t, z, ln_k, ok, threads: int = 8):
    """Newton-polish two-phase states (test instrument, see oracle::polish).

    Returns dict with polished ln_k, beta, x, y, residual (max |F|) and
    ainv (||(dF/dlnK)^-1||_inf); NaN where skipped or failed."""
    build()
    tc, pc, omega, kij = (np.ascontiguousarray(a, dtype=np.float64) for a in mix.as_tuple())
    z = np.ascontiguousarray(z, dtype=np.float64)
    n, ncell = z.shape
    lk = np.ascontiguousarray(np.nan_to_num(np.asarray(ln_k, dtype=np.float64)))
    okv = np.ascontiguousarray(np.asarray(ok, dtype=np.int32))
    p = np.ascontiguousarray(p, dtype=np.float64)
    t = np.ascontiguousarray(t, dtype=np.float64)
    out = {"ln_k": np.empty((n, ncell)), "beta": np.empty(ncell), "x": np.empty((n, ncell)),
           "y": np.empty((n, ncell)), "residual": np.empty(ncell), "ainv": np.empty(ncell)}
    fn = _lib(ORACLE_SO).oracle_polish_batch
    fn.restype = ctypes.c_int
    args = [ctypes.c_int(n)] + [ctypes.c_void_p(a.ctypes.data) for a in (tc, pc, omega, kij)] + \
        [ctypes.c_int64(ncell)] + [ctypes.c_void_p(a.ctypes.data) for a in (p, t, z, okv, lk)] + \
        [ctypes.c_int(threads)] + [ctypes.c_void_p(out[k].ctypes.data) for k in
                                   ("ln_k", "beta", "x", "y", "residual", "ainv")]
    fn(*args)
    return out


def sensitivity_at(mix, p, t, z, ok, x, y, ln_k, beta, threads: int = 8, manifold_identity: bool = False):
    """Oracle sensitivities at GIVEN accepted two-phase states (see
    oracle_sensitivity_at): isolates the derivative computation from the
    convergence noise of the flash that produced the state.

    manifold_identity: take d(ln x_i - ln y_i) = -d ln K_i exactly instead of
    through the reference's dependent last fractions (a diagnostic that
    removes the reference's own cancellation noise in the last row)."""
    build()
    _lib(ORACLE_SO).oracle_set_manifold_identity(ctypes.c_int(1 if manifold_identity else 0))
    tc, pc, omega, kij = (np.ascontiguousarray(a, dtype=np.float64) for a in mix.as_tuple())
    z = np.ascontiguousarray(z, dtype=np.float64)
    n, ncell = z.shape
    out, s = _alloc(n, ncell, True)
    arrays = [np.ascontiguousarray(np.nan_to_num(np.asarray(a, dtype=np.float64), nan=0.5)) for a in (x, y, ln_k)]
    b = np.ascontiguousarray(np.nan_to_num(np.asarray(beta, dtype=np.float64), nan=0.5))
    okv = np.ascontiguousarray(np.asarray(ok, dtype=np.int32))
    p = np.ascontiguousarray(p, dtype=np.float64)
    t = np.ascontiguousarray(t, dtype=np.float64)
    fn = _lib(ORACLE_SO).oracle_sensitivity_at
    fn.restype = ctypes.c_int
    fn(ctypes.c_int(n), *(ctypes.c_void_p(a.ctypes.data) for a in (tc, pc, omega, kij)), ctypes.c_int64(ncell),
       *(ctypes.c_void_p(a.ctypes.data) for a in (p, t, z, okv)), *(ctypes.c_void_p(a.ctypes.data) for a in arrays),
       ctypes.c_void_p(b.ctypes.data), ctypes.c_int(threads), ctypes.byref(s))
    _lib(ORACLE_SO).oracle_set_manifold_identity(ctypes.c_int(0))
    return out

MAX3_FIELDS = [("max3_status", np.int32, 1), ("published", np.int32, 1), ("beta3", np.float64, 3),
               ("x3", np.float64, -3), ("lnphi3", np.float64, -3), ("z3", np.float64, 3),
               ("beta", np.float64, 1), ("x", np.float64, -1), ("y", np.float64, -1), ("attempts", np.int32, 1)]


class _Max3(ctypes.Structure):
    _fields_ = [(f, ctypes.c_void_p) for f, _, _ in MAX3_FIELDS]


def _max3(fn_name: str, so: str, mix, p, t, z, threads: int):
    tc, pc, omega, kij = (np.ascontiguousarray(a, dtype=np.float64) for a in mix.as_tuple())
    z = np.ascontiguousarray(z, dtype=np.float64)
    p = np.ascontiguousarray(p, dtype=np.float64)
    t = np.ascontiguousarray(t, dtype=np.float64)
    n, ncell = z.shape
    out = {f: np.empty(((-r) * n if r < 0 else r, ncell), d) for f, d, r in MAX3_FIELDS}
    o = _Max3(**{f: v.ctypes.data for f, v in out.items()})
    fn = getattr(_lib(so), fn_name)
    fn.restype = ctypes.c_int
    fn(ctypes.c_int(n), *[ctypes.c_void_p(a.ctypes.data) for a in (tc, pc, omega, kij)], ctypes.c_int64(ncell),
       *[ctypes.c_void_p(a.ctypes.data) for a in (p, t, z)], ctypes.c_int(threads), ctypes.byref(o))
    return {f: (v[0] if v.shape[0] == 1 else v) for f, v in out.items()}


def max3(mix, p, t, z, threads: int = 8):
    """Max-3-phase orchestration (solve_pr76_pt_max3 restated, backend
    defaults).  Statuses: max3_status 0 single, 1 two, 2 three, 3 boundary
    unresolved, 4 higher phase count, 5 indeterminate, -1 invalid; published
    0 single, 1 two, 2 phase set unstable, 3 indeterminate, 4 three."""
    build()
    return _max3("oracle_max3_batch", ORACLE_SO, mix, p, t, z, threads)


def reference_max3(mix, p, t, z, threads: int = 8):
    """The reference's solve_pr76_pt_max3 through oracle/_ref (only where the
    reference sources were present to build it)."""
    if not reference_available():
        raise FileNotFoundError(REF_SO)
    return _max3("ref_max3_batch", REF_SO, mix, p, t, z, threads)


class _StartHints(ctypes.Structure):
    _fields_ = [("initial_count", ctypes.c_void_p), ("initial_x", ctypes.c_void_p),
                ("final_count", ctypes.c_void_p), ("final_x", ctypes.c_void_p),
                ("three_phase", ctypes.c_void_p), ("three_x", ctypes.c_void_p), ("fraction", ctypes.c_void_p),
                ("initial_automatic_starts", ctypes.c_int32), ("max_split_attempts", ctypes.c_int32)]


def start_hints(n: int, ncell: int, initial=None, final=None, three_phase=None, fraction=None,
                initial_automatic_starts: bool = True, max_split_attempts: int = 16):
    """Arrays of a hinted max-3-phase solve.  `initial` / `final`: per cell a
    list of up to 3 compositions (solve_pr76_pt_max3's initial_starts /
    final_starts); `three_phase`: per cell None or 3 compositions (one
    three-phase start) with `fraction` per cell (phase_fraction_seed of
    phases 1 and 2).  Returns a dict of contiguous arrays in the C layout
    (composition k of cell c, component i at (k * n + i) * ncell + c)."""
    def pack(sets):
        cnt = np.zeros(ncell, np.int32)
        x = np.zeros((3 * n, ncell))
        for c, comps in enumerate(sets if sets is not None else [[]] * ncell):
            comps = list(comps or [])[:3]
            cnt[c] = len(comps)
            for k, w in enumerate(comps):
                x[k * n:(k + 1) * n, c] = w
        return cnt, x
    ic, ix = pack(initial)
    fc, fx = pack(final)
    tf = np.zeros(ncell, np.int32)
    tx = np.zeros((3 * n, ncell))
    fr = np.full((2, ncell), 1.0 / 3.0)
    if three_phase is not None:
        for c, comps in enumerate(three_phase):
            if comps is None:
                continue
            tf[c] = 1
            for k in range(3):
                tx[k * n:(k + 1) * n, c] = comps[k]
            if fraction is not None and fraction[c] is not None:
                fr[:, c] = fraction[c]
    return {"initial_count": ic, "initial_composition": ix, "final_count": fc, "final_composition": fx,
            "three_phase": tf, "three_phase_composition": tx, "fraction": fr,
            "initial_automatic_starts": bool(initial_automatic_starts), "max_split_attempts": int(max_split_attempts)}


def _max3_hinted(fn_name: str, so: str, mix, p, t, z, hints: dict, threads: int):
    tc, pc, omega, kij = (np.ascontiguousarray(a, dtype=np.float64) for a in mix.as_tuple())
    z = np.ascontiguousarray(z, dtype=np.float64)
    p = np.ascontiguousarray(p, dtype=np.float64)
    t = np.ascontiguousarray(t, dtype=np.float64)
    n, ncell = z.shape
    arr = {k: np.ascontiguousarray(hints[k]) for k in ("initial_count", "initial_composition", "final_count",
                                                         "final_composition", "three_phase",
                                                         "three_phase_composition", "fraction")}
    h = _StartHints(*(arr[k].ctypes.data for k in ("initial_count", "initial_composition", "final_count",
                                                   "final_composition", "three_phase", "three_phase_composition",
                                                   "fraction")),
                    int(bool(hints["initial_automatic_starts"])), int(hints["max_split_attempts"]))
    out = {f: np.empty(((-r) * n if r < 0 else r, ncell), d) for f, d, r in MAX3_FIELDS}
    o = _Max3(**{f: v.ctypes.data for f, v in out.items()})
    fn = getattr(_lib(so), fn_name)
    fn.restype = ctypes.c_int
    fn(ctypes.c_int(n), *[ctypes.c_void_p(a.ctypes.data) for a in (tc, pc, omega, kij)], ctypes.c_int64(ncell),
       *[ctypes.c_void_p(a.ctypes.data) for a in (p, t, z)], ctypes.byref(h), ctypes.c_int(threads),
       ctypes.byref(o))
    return {f: (v[0] if v.shape[0] == 1 else v) for f, v in out.items()}


def max3_hinted(mix, p, t, z, hints: dict, threads: int = 8):
    """`max3` with caller starts and the two split options (`start_hints`)."""
    build()
    return _max3_hinted("oracle_max3_hinted_batch", ORACLE_SO, mix, p, t, z, hints, threads)


def reference_max3_hinted(mix, p, t, z, hints: dict, threads: int = 8):
    """The reference's solve_pr76_pt_max3 with the same starts and options
    through oracle/_ref."""
    if not reference_available():
        raise FileNotFoundError(REF_SO)
    return _max3_hinted("ref_max3_hinted_batch", REF_SO, mix, p, t, z, hints, threads)


def reference_continuation(mix, pressures, temperatures, z, threads: int = 8):
    """The reference's solve_pr76_pt_continuation (default options) of feeds
    z [n, npath] along paths pressures / temperatures [npath, npoint]; returns
    (max3_status, published) [npath, npoint] with ref_max3_batch's codes."""
    if not reference_available():
        raise FileNotFoundError(REF_SO)
    tc, pc, omega, kij = (np.ascontiguousarray(a, dtype=np.float64) for a in mix.as_tuple())
    z = np.ascontiguousarray(z, dtype=np.float64)
    p = np.ascontiguousarray(pressures, dtype=np.float64)
    t = np.ascontiguousarray(temperatures, dtype=np.float64)
    n, npath = z.shape
    npoint = p.shape[1]
    ms = np.empty((npath, npoint), np.int32)
    pub = np.empty((npath, npoint), np.int32)
    fn = _lib(REF_SO).ref_continuation_batch
    fn.restype = ctypes.c_int
    fn(ctypes.c_int(n), *[ctypes.c_void_p(a.ctypes.data) for a in (tc, pc, omega, kij)], ctypes.c_int64(npath),
       ctypes.c_int64(npoint), *[ctypes.c_void_p(a.ctypes.data) for a in (p, t, z)], ctypes.c_int(threads),
       ctypes.c_void_p(ms.ctypes.data), ctypes.c_void_p(pub.ctypes.data))
    return ms, pub


def continuation(mix, pressures, temperatures, z, threads: int = 8):
    """The oracle's restatement of solve_pr76_pt_continuation (default
    options): max3 status [npath, npoint] of feeds z [n, npath] along paths
    pressures / temperatures [npath, npoint]."""
    build()
    tc, pc, omega, kij = (np.ascontiguousarray(a, dtype=np.float64) for a in mix.as_tuple())
    z = np.ascontiguousarray(z, dtype=np.float64)
    p = np.ascontiguousarray(pressures, dtype=np.float64)
    t = np.ascontiguousarray(temperatures, dtype=np.float64)
    n, npath = z.shape
    npoint = p.shape[1]
    ms = np.empty((npath, npoint), np.int32)
    fn = _lib(ORACLE_SO).oracle_continuation_batch
    fn.restype = ctypes.c_int
    fn(ctypes.c_int(n), *[ctypes.c_void_p(a.ctypes.data) for a in (tc, pc, omega, kij)], ctypes.c_int64(npath),
       ctypes.c_int64(npoint), *[ctypes.c_void_p(a.ctypes.data) for a in (p, t, z)], ctypes.c_int(threads),
       ctypes.c_void_p(ms.ctypes.data))
    return ms


def _property_chart(fn_name: str, so: str, mix, phases: int, root_index, molar_mass, viscosity, enthalpy, q,
                    dependent=None, threads: int = 8):
    tc, pc, omega, kij = (np.ascontiguousarray(a, dtype=np.float64) for a in mix.as_tuple())
    n = len(tc)
    q = np.ascontiguousarray(q, dtype=np.float64)
    cols, ncell = q.shape
    if cols != phases * n + 1:
        raise ValueError(f"expected {phases * n + 1} chart rows, got {cols}")
    rows = phases * (5 + n) + (phases - 1) * n
    ri = np.zeros(3, np.int32)
    ri[:phases] = root_index
    mm = np.ascontiguousarray(molar_mass, dtype=np.float64)
    cv = np.ascontiguousarray(viscosity, dtype=np.float64)
    ce = np.ascontiguousarray(enthalpy, dtype=np.float64)
    dep = None if dependent is None else np.ascontiguousarray(dependent, dtype=np.int32)
    status = np.full(ncell, -9, np.int32)
    values = np.empty((rows, ncell))
    jac = np.empty((rows * cols, ncell))
    fn = getattr(_lib(so), fn_name)
    fn.restype = ctypes.c_int
    fn(ctypes.c_int(n), *[ctypes.c_void_p(a.ctypes.data) for a in (tc, pc, omega, kij)], ctypes.c_int(phases),
       ctypes.c_void_p(ri.ctypes.data), *[ctypes.c_void_p(a.ctypes.data) for a in (mm, cv, ce)],
       ctypes.c_int64(ncell), ctypes.c_void_p(q.ctypes.data),
       ctypes.c_void_p(dep.ctypes.data) if dep is not None else ctypes.c_void_p(None), ctypes.c_int(threads),
       *[ctypes.c_void_p(a.ctypes.data) for a in (status, values, jac)])
    return {"status": status, "values": values, "jacobian": jac.reshape(rows, cols, ncell)}


def property_chart(mix, phases: int, root_index, molar_mass, viscosity, enthalpy, q, dependent=None,
                   threads: int = 8):
    """The oracle's restatement of evaluate_pr76_selected_phase_property_chart
    with the affine transport/caloric model: q [(P n + 1), ncell] chart
    values, dependent [P, ncell] or None (last component).  Returns status
    [ncell] (mpmc_chart_status codes), values [rows, ncell] and jacobian
    [rows, q, ncell]."""
    build()
    return _property_chart("oracle_property_chart_batch", ORACLE_SO, mix, phases, root_index, molar_mass,
                           viscosity, enthalpy, q, dependent, threads)


def reference_property_chart(mix, phases: int, root_index, molar_mass, viscosity, enthalpy, q, dependent=None,
                             threads: int = 8):
    """The reference's evaluate_pr76_selected_phase_property_chart through
    oracle/_ref (status 7 = an unexpected exception)."""
    if not reference_available():
        raise FileNotFoundError(REF_SO)
    return _property_chart("ref_property_chart_batch", REF_SO, mix, phases, root_index, molar_mass, viscosity,
                           enthalpy, q, dependent, threads)
