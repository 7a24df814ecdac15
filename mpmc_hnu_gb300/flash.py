"""Python binding of the C ABI in include/mpmc_gb300_flash.h (ctypes).

`GpuFlash` mirrors the reference's per-mixture backend object
(mpmc::flash::Pr76PtFlashBackend, modules/flash/include/mpmc/flash/
pr76_pt_flash_backend.hpp:177-282) for a batch of cells: construct it once per
mixture, then call `solve()` with host arrays (copies in and out inside the
call) or `solve_device()` with device pointers on a CUDA stream.  The compiled
library must exist: there is no CPU fallback, and a missing library raises.
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_lib", "libmpmc_gb300_flash.so")

FORM_PLAIN_FP64 = 0
FORM_BATCHED = 1
FORM_MIXED = 2
FORMS = {"plain": FORM_PLAIN_FP64, "batched": FORM_BATCHED, "mixed": FORM_MIXED}

SINGLE_PHASE, TWO_PHASE, PHASE_SET_UNSTABLE, INDETERMINATE, INVALID_REQUEST = 0, 1, 2, 3, -1
COUNTER_NAMES = ["init_evals", "split_evals", "final_evals", "split_iters", "rr_iters", "root_iters",
                 "attempts", "trial_iters"]
MAX_COMPONENTS = 20


class _Mixture(ctypes.Structure):
    _fields_ = [("n_components", ctypes.c_int32), ("critical_temperature_k", ctypes.c_void_p),
                ("critical_pressure_pa", ctypes.c_void_p), ("acentric_factor", ctypes.c_void_p),
                ("kij", ctypes.c_void_p)]


class _Options(ctypes.Structure):
    _fields_ = [("form", ctypes.c_int32), ("want_sensitivity", ctypes.c_int32), ("device", ctypes.c_int32),
                ("flags", ctypes.c_int32)]


# (field, dtype, rows(n)) in mpmc_flash_outputs order
OUTPUT_FIELDS = [
    ("status", np.int32, lambda n: 1), ("vapor_fraction", np.float64, lambda n: 1),
    ("liquid", np.float64, lambda n: n), ("vapor", np.float64, lambda n: n),
    ("ln_k", np.float64, lambda n: n), ("ln_phi_liquid", np.float64, lambda n: n),
    ("ln_phi_vapor", np.float64, lambda n: n), ("z_liquid", np.float64, lambda n: 1),
    ("z_vapor", np.float64, lambda n: 1), ("counters", np.int32, lambda n: 8),
    ("sensitivity_status", np.int32, lambda n: 1), ("d_ln_k", np.float64, lambda n: n * (n + 1)),
    ("d_vapor_fraction", np.float64, lambda n: n + 1), ("d_liquid", np.float64, lambda n: n * (n + 1)),
    ("d_vapor", np.float64, lambda n: n * (n + 1)), ("d_z_liquid", np.float64, lambda n: n + 1),
    ("d_z_vapor", np.float64, lambda n: n + 1), ("d_rho_liquid", np.float64, lambda n: n + 1),
    ("d_rho_vapor", np.float64, lambda n: n + 1), ("jac_liquid", np.float64, lambda n: (n + 1) * (n + 2)),
    ("jac_vapor", np.float64, lambda n: (n + 1) * (n + 2)),
]
FLASH_FIELDS = [f for f, _, _ in OUTPUT_FIELDS[:10]]
SENSITIVITY_FIELDS = [f for f, _, _ in OUTPUT_FIELDS[10:]]


class _Outputs(ctypes.Structure):
    _fields_ = [(f, ctypes.c_void_p) for f, _, _ in OUTPUT_FIELDS]


# three-phase outputs of the max-3-phase entry points (mpmc_three_phase_outputs)
THREE_PHASE_FIELDS = [("max3_status", np.int32, lambda n: 1), ("phase_fraction", np.float64, lambda n: 3),
                      ("composition", np.float64, lambda n: 3 * n), ("ln_phi", np.float64, lambda n: 3 * n),
                      ("z_factor", np.float64, lambda n: 3)]
MAX3_STATUS = {0: "single_phase", 1: "two_phase", 2: "three_phase", 3: "phase_boundary_unresolved",
               4: "higher_phase_count_or_wrong_candidate", 5: "indeterminate", -1: "invalid"}
FLASH_THREE_PHASE = 4


class _ThreePhaseOutputs(ctypes.Structure):
    _fields_ = [(f, ctypes.c_void_p) for f, _, _ in THREE_PHASE_FIELDS]


# caller start hints of the hinted max-3-phase solve (mpmc_start_hints)
class _StartHints(ctypes.Structure):
    _fields_ = [("count", ctypes.c_void_p), ("composition", ctypes.c_void_p), ("three_phase", ctypes.c_void_p),
                ("fraction", ctypes.c_void_p)]


class _StartHintsEx(ctypes.Structure):
    _fields_ = [("initial_count", ctypes.c_void_p), ("initial_composition", ctypes.c_void_p),
                ("final_count", ctypes.c_void_p), ("final_composition", ctypes.c_void_p),
                ("three_phase", ctypes.c_void_p), ("three_phase_composition", ctypes.c_void_p),
                ("fraction", ctypes.c_void_p), ("initial_automatic_starts", ctypes.c_int32),
                ("max_split_attempts", ctypes.c_int32)]


# selected-phase property chart (mpmc_property_chart_spec / _outputs)
class _ChartSpec(ctypes.Structure):
    _fields_ = [("phase_count", ctypes.c_int32), ("root_index", ctypes.c_int32 * 3),
                ("molar_mass", ctypes.c_void_p), ("viscosity", ctypes.c_void_p), ("enthalpy", ctypes.c_void_p)]


class _ChartOutputs(ctypes.Structure):
    _fields_ = [("status", ctypes.c_void_p), ("values", ctypes.c_void_p), ("jacobian", ctypes.c_void_p)]


CHART_STATUS = {0: "ok", 1: "input_domain", 2: "eos_domain", 3: "root_unresolved", 4: "root_index",
                5: "ill_conditioned_root", 6: "property_domain"}
CHART_PROPERTIES = ["molar_density", "mass_density", "viscosity", "enthalpy", "internal_energy"]


def chart_shape(n: int, phases: int) -> tuple[int, int]:
    """(rows, columns) of a property chart: P (5 + n) + (P - 1) n output rows
    and P n + 1 natural variables."""
    return phases * (5 + n) + (phases - 1) * n, phases * n + 1


class PropertyChartSpec:
    """Closure of a selected-phase property chart (mpmc_property_chart_spec):
    phase count, selected root index per phase, molar masses [n] in kg/mol and
    the affine viscosity and enthalpy models [7 + n] each (constant, p, T,
    molar density, molar mass, mass density, root index, then x_i)."""

    def __init__(self, phases: int, root_index, molar_mass, viscosity, enthalpy):
        self.phases = int(phases)
        self.root_index = [int(r) for r in root_index]
        self.molar_mass = np.ascontiguousarray(molar_mass, dtype=np.float64)
        self.viscosity = np.ascontiguousarray(viscosity, dtype=np.float64)
        self.enthalpy = np.ascontiguousarray(enthalpy, dtype=np.float64)
        if len(self.root_index) != self.phases:
            raise ValueError("one root index per phase")

    def _struct(self) -> _ChartSpec:
        s = _ChartSpec()
        s.phase_count = self.phases
        for k, r in enumerate(self.root_index):
            s.root_index[k] = r
        s.molar_mass = self.molar_mass.ctypes.data
        s.viscosity = self.viscosity.ctypes.data
        s.enthalpy = self.enthalpy.ctypes.data
        return s


class _ServerOptions(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("slots", ctypes.c_int32), ("max_batch_cells", ctypes.c_int64),
                ("memory_budget_bytes", ctypes.c_int64), ("form", ctypes.c_int32), ("flags", ctypes.c_int32)]


class _ServerPolicy(ctypes.Structure):
    _fields_ = [("small_request_cells", ctypes.c_int64), ("latency_slots", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("latency_batch_cells", ctypes.c_int64), ("chunk_cells", ctypes.c_int64),
                ("max_request_cells", ctypes.c_int64), ("max_in_flight", ctypes.c_int64),
                ("max_deadline_us", ctypes.c_int64)]


SERVER_WARM_CACHE = 1
ERR_TIMEOUT, ERR_BUSY, ERR_DEADLINE = 5, 6, 7


EXPORTED_SYMBOLS = ["mpmc_gpu_flash_create", "mpmc_gpu_flash_destroy", "mpmc_gpu_flash_solve",
                    "mpmc_gpu_flash_solve_device", "mpmc_gpu_flash_components", "mpmc_gpu_flash_last_error",
                    "mpmc_gpu_flash_abi_version", "mpmc_gpu_flash_stage_timings", "mpmc_gpu_flash_batch_stats",
                    "mpmc_gpu_flash_solve_device_noalloc", "mpmc_flash_server_create", "mpmc_flash_server_add_mixture",
                    "mpmc_flash_server_submit", "mpmc_flash_server_wait", "mpmc_flash_server_stats",
                    "mpmc_flash_server_destroy", "mpmc_gpu_flash_set_launch_shape", "mpmc_gpu_flash_solve_warm",
                    "mpmc_gpu_flash_solve_device_warm", "mpmc_gpu_flash_solve_max3", "mpmc_gpu_flash_solve_device_max3",
                    "mpmc_gpu_flash_property_chart", "mpmc_gpu_flash_property_chart_device",
                    "mpmc_gpu_flash_solve_hinted", "mpmc_gpu_flash_solve_device_hinted",
                    "mpmc_flash_server_set_policy", "mpmc_flash_server_submit_deadline",
                    "mpmc_gpu_flash_solve_hinted_ex", "mpmc_gpu_flash_solve_device_hinted_ex"]
FLAG_CUDA_GRAPH = 2
FLAG_SENSITIVITY_LANES = 4  # the lane-group sensitivity kernel (opt-in)
FLAG_MAX3_NEWTON_ROOTS = 8  # Newton roots in the max-3-phase continuation (opt-in)
FLAG_POLISH_STREAM = 16  # the state-machine FP64 polish (opt-in)
NOALLOC_SCRATCH_BYTES = 48 << 20
BATCH_STATS = ["feed_continued", "feed_rerun", "review_continued", "review_rerun", "fallback_nonsmooth",
               "fp64_attempts_no_fp32", "fp64_attempts_polish_failed", "fp64_attempts_rejected", "fallback_load",
               "two_candidates", "fp64_trial_items", "fp64_attempt_items", "polished_cells", "select64_cells",
               "slow_trials_skipped", "limit_attempts", "warm_cells", "warm_redo",
               "warm_redo_no_pair", "warm_redo_unstable", "competing_cells", "competing_cells_fp64", "replay_risk_cells",
               "fp64_evals_setup", "fp64_evals_feed_trials", "fp64_evals_review_trials", "fp64_evals_polish",
               "fp64_evals_split64", "polish_jacobians", "polish_solves", "fallback_cells", "exact_cells"]
FLAG_STAGE_TIMING = 1
_QUEUE_STAGES = ["setup", "feed_trials", "feed_classify", "feed_trials64", "decide", "split", "polish",
                 "open32", "compete", "split64", "select64", "relist", "review_trials", "review_classify", "review_trials64",
                 "finish", "fallback", "sensitivity"]
# the FP64 work-queue form runs on the same stage slots; its FP32 stages
# (feed_trials, split, review_trials) only queue items or are empty
STAGES = {FORM_PLAIN_FP64: ["flash", "sensitivity"], FORM_MIXED: _QUEUE_STAGES, FORM_BATCHED: _QUEUE_STAGES}

_LIB = None


def library() -> ctypes.CDLL:
    """Load the compiled library (raises if it was not built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} missing: run `python -m mpmc_hnu_gb300.build` (no CPU fallback)")
        lib = ctypes.CDLL(LIB_PATH)
        lib.mpmc_gpu_flash_create.argtypes = [ctypes.POINTER(_Mixture), ctypes.POINTER(_Options),
                                              ctypes.POINTER(ctypes.c_void_p)]
        lib.mpmc_gpu_flash_destroy.argtypes = [ctypes.c_void_p]
        lib.mpmc_gpu_flash_solve.argtypes = [ctypes.c_void_p, ctypes.c_int64] + [ctypes.c_void_p] * 3 + \
            [ctypes.POINTER(_Outputs)]
        lib.mpmc_gpu_flash_solve_device.argtypes = [ctypes.c_void_p, ctypes.c_int64] + [ctypes.c_void_p] * 3 + \
            [ctypes.POINTER(_Outputs), ctypes.c_void_p]
        lib.mpmc_gpu_flash_solve_device_noalloc.argtypes = lib.mpmc_gpu_flash_solve_device.argtypes
        lib.mpmc_gpu_flash_solve_warm.argtypes = [ctypes.c_void_p, ctypes.c_int64] + [ctypes.c_void_p] * 4 + \
            [ctypes.POINTER(_Outputs)]
        lib.mpmc_gpu_flash_solve_device_warm.argtypes = [ctypes.c_void_p, ctypes.c_int64] + [ctypes.c_void_p] * 4 + \
            [ctypes.POINTER(_Outputs), ctypes.c_void_p]
        lib.mpmc_gpu_flash_solve_max3.argtypes = [ctypes.c_void_p, ctypes.c_int64] + [ctypes.c_void_p] * 3 + \
            [ctypes.POINTER(_Outputs), ctypes.POINTER(_ThreePhaseOutputs)]
        lib.mpmc_gpu_flash_solve_device_max3.argtypes = [ctypes.c_void_p, ctypes.c_int64] + [ctypes.c_void_p] * 3 + \
            [ctypes.POINTER(_Outputs), ctypes.POINTER(_ThreePhaseOutputs), ctypes.c_void_p]
        lib.mpmc_gpu_flash_solve_hinted.argtypes = [ctypes.c_void_p, ctypes.c_int64] + [ctypes.c_void_p] * 3 + \
            [ctypes.POINTER(_StartHints), ctypes.POINTER(_Outputs), ctypes.POINTER(_ThreePhaseOutputs)]
        lib.mpmc_gpu_flash_solve_device_hinted.argtypes = lib.mpmc_gpu_flash_solve_hinted.argtypes + \
            [ctypes.c_void_p]
        lib.mpmc_gpu_flash_property_chart.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(_ChartSpec),
                                                      ctypes.c_void_p, ctypes.c_void_p,
                                                      ctypes.POINTER(_ChartOutputs)]
        lib.mpmc_gpu_flash_property_chart_device.argtypes = lib.mpmc_gpu_flash_property_chart.argtypes + \
            [ctypes.c_void_p]
        lib.mpmc_gpu_flash_components.argtypes = [ctypes.c_void_p]
        lib.mpmc_gpu_flash_stage_timings.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        lib.mpmc_gpu_flash_batch_stats.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        lib.mpmc_flash_server_create.argtypes = [ctypes.POINTER(_ServerOptions), ctypes.POINTER(ctypes.c_void_p)]
        lib.mpmc_flash_server_add_mixture.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Mixture),
                                                      ctypes.POINTER(ctypes.c_int32)]
        lib.mpmc_flash_server_submit.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64] + \
            [ctypes.c_void_p] * 3 + [ctypes.POINTER(_Outputs), ctypes.POINTER(ctypes.c_uint64)]
        lib.mpmc_flash_server_wait.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int64,
                                               ctypes.POINTER(ctypes.c_double)]
        lib.mpmc_flash_server_set_policy.argtypes = [ctypes.c_void_p, ctypes.POINTER(_ServerPolicy)]
        lib.mpmc_flash_server_submit_deadline.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64] + \
            [ctypes.c_void_p] * 3 + [ctypes.POINTER(_Outputs), ctypes.c_int64, ctypes.POINTER(ctypes.c_uint64)]
        lib.mpmc_flash_server_stats.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        lib.mpmc_flash_server_destroy.argtypes = [ctypes.c_void_p]
        lib.mpmc_gpu_flash_set_launch_shape.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        for name in EXPORTED_SYMBOLS:
            getattr(lib, name).restype = ctypes.c_int
        lib.mpmc_gpu_flash_last_error.restype = ctypes.c_char_p
        _LIB = lib
    return _LIB


class FlashError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"mpmc_gpu_flash error {code}: {message}")
        self.code = code


def _check(rc: int) -> None:
    if rc != 0:
        raise FlashError(rc, library().mpmc_gpu_flash_last_error().decode())


def output_rows(n: int) -> dict[str, int]:
    return {f: rows(n) for f, _, rows in OUTPUT_FIELDS}


class GpuFlash:
    """One mixture on one GPU; batches of cells per call."""

    def __init__(self, mixture, form: str | int = "plain", sensitivity: bool = False, device: int = 0,
                 stage_timing: bool = False, graphs: bool = False, sensitivity_lanes: bool = False,
                 max3_newton_roots: bool = False, polish_stream: bool = False):
        self.mixture = mixture
        self.n = int(mixture.n)
        self.form = FORMS[form] if isinstance(form, str) else int(form)
        self.sensitivity = bool(sensitivity)
        self._keep = [np.ascontiguousarray(a, dtype=np.float64) for a in
                      (mixture.tc, mixture.pc, mixture.omega, np.asarray(mixture.kij).reshape(-1))]
        m = _Mixture(self.n, *(a.ctypes.data for a in self._keep))
        flags = ((FLAG_STAGE_TIMING if stage_timing else 0) | (FLAG_CUDA_GRAPH if graphs else 0)
                 | (FLAG_SENSITIVITY_LANES if sensitivity_lanes else 0)
                 | (FLAG_MAX3_NEWTON_ROOTS if max3_newton_roots else 0)
                 | (FLAG_POLISH_STREAM if polish_stream else 0))
        o = _Options(self.form, int(self.sensitivity), device, flags)
        h = ctypes.c_void_p()
        _check(library().mpmc_gpu_flash_create(ctypes.byref(m), ctypes.byref(o), ctypes.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            library().mpmc_gpu_flash_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def fields(self, want_sensitivity: bool | None = None) -> list[str]:
        sens = self.sensitivity if want_sensitivity is None else want_sensitivity
        return FLASH_FIELDS + (SENSITIVITY_FIELDS if sens else [])

    def solve(self, p, t, z, fields: list[str] | None = None, ln_k_warm=None) -> dict[str, np.ndarray]:
        """Host arrays in, host arrays out (the copies happen inside the call).
        `ln_k_warm` [n, ncell] (optional): ln K warm starts, NaN columns cold
        (mpmc_gpu_flash_solve_warm)."""
        p = np.ascontiguousarray(p, dtype=np.float64)
        t = np.ascontiguousarray(t, dtype=np.float64)
        z = np.ascontiguousarray(z, dtype=np.float64)
        if z.shape != (self.n, p.shape[0]) or t.shape != p.shape:
            raise ValueError("expected p[ncell], t[ncell], z[n, ncell]")
        warm = None
        if ln_k_warm is not None:
            warm = np.ascontiguousarray(ln_k_warm, dtype=np.float64)
            if warm.shape != z.shape:
                raise ValueError("expected ln_k_warm[n, ncell]")
        ncell = p.shape[0]
        fields = fields or self.fields()
        rows = output_rows(self.n)
        dtypes = {f: d for f, d, _ in OUTPUT_FIELDS}
        out = {f: np.empty((rows[f], ncell), dtypes[f]) for f in fields}
        s = _Outputs(**{f: out[f].ctypes.data for f in fields})
        _check(library().mpmc_gpu_flash_solve_warm(self._h, ncell, p.ctypes.data, t.ctypes.data, z.ctypes.data,
                                                   None if warm is None else warm.ctypes.data, ctypes.byref(s)))
        return {f: (v[0] if rows[f] == 1 else v) for f, v in out.items()}

    def solve_max3(self, p, t, z, fields: list[str] | None = None):
        """`solve` followed by the max-3-phase continuation of phase-set-unstable
        cells (mpmc_gpu_flash_solve_max3).  Returns (flash outputs, three-phase
        outputs); `status` is the published one (4 = three phases)."""
        p = np.ascontiguousarray(p, dtype=np.float64)
        t = np.ascontiguousarray(t, dtype=np.float64)
        z = np.ascontiguousarray(z, dtype=np.float64)
        if z.shape != (self.n, p.shape[0]) or t.shape != p.shape:
            raise ValueError("expected p[ncell], t[ncell], z[n, ncell]")
        ncell = p.shape[0]
        fields = fields or self.fields()
        rows = output_rows(self.n)
        dtypes = {f: d for f, d, _ in OUTPUT_FIELDS}
        out = {f: np.empty((rows[f], ncell), dtypes[f]) for f in fields}
        out3 = {f: np.empty((r(self.n), ncell), d) for f, d, r in THREE_PHASE_FIELDS}
        s = _Outputs(**{f: out[f].ctypes.data for f in fields})
        s3 = _ThreePhaseOutputs(**{f: v.ctypes.data for f, v in out3.items()})
        _check(library().mpmc_gpu_flash_solve_max3(self._h, ncell, p.ctypes.data, t.ctypes.data, z.ctypes.data,
                                                   ctypes.byref(s), ctypes.byref(s3)))
        return ({f: (v[0] if rows[f] == 1 else v) for f, v in out.items()},
                {f: (v[0] if v.shape[0] == 1 else v) for f, v in out3.items()})

    def solve_hinted(self, p, t, z, count, composition, three_phase=None, fraction=None,
                     fields: list[str] | None = None):
        """`solve_max3` with caller start hints (mpmc_gpu_flash_solve_hinted):
        count [ncell] (0..3) compositions composition [3 n, ncell] per cell as
        extra stability starts; three_phase [ncell] (nonzero: a three-phase
        start, count 3) with its phase-1 and phase-2 fractions fraction
        [2, ncell].  Runs the reference algorithm in FP64 for every form.
        Returns (flash outputs, three-phase outputs)."""
        p = np.ascontiguousarray(p, dtype=np.float64)
        t = np.ascontiguousarray(t, dtype=np.float64)
        z = np.ascontiguousarray(z, dtype=np.float64)
        if z.shape != (self.n, p.shape[0]) or t.shape != p.shape:
            raise ValueError("expected p[ncell], t[ncell], z[n, ncell]")
        ncell = p.shape[0]
        cnt = np.ascontiguousarray(count, dtype=np.int32)
        comp = np.ascontiguousarray(composition, dtype=np.float64)
        if cnt.shape != (ncell,) or comp.shape != (3 * self.n, ncell):
            raise ValueError("expected count[ncell] and composition[3 n, ncell]")
        three = frac = None
        if three_phase is not None:
            three = np.ascontiguousarray(three_phase, dtype=np.int32)
            frac = np.ascontiguousarray(fraction, dtype=np.float64)
            if three.shape != (ncell,) or frac.shape != (2, ncell):
                raise ValueError("expected three_phase[ncell] and fraction[2, ncell]")
        hints = _StartHints(cnt.ctypes.data, comp.ctypes.data, three.ctypes.data if three is not None else None,
                            frac.ctypes.data if frac is not None else None)
        fields = fields or self.fields()
        for need in ("status", "ln_k"):
            if need not in fields:
                fields = fields + [need]
        rows = output_rows(self.n)
        dtypes = {f: d for f, d, _ in OUTPUT_FIELDS}
        out = {f: np.empty((rows[f], ncell), dtypes[f]) for f in fields}
        out3 = {f: np.empty((r(self.n), ncell), d) for f, d, r in THREE_PHASE_FIELDS}
        s = _Outputs(**{f: out[f].ctypes.data for f in fields})
        s3 = _ThreePhaseOutputs(**{f: v.ctypes.data for f, v in out3.items()})
        _check(library().mpmc_gpu_flash_solve_hinted(self._h, ncell, p.ctypes.data, t.ctypes.data, z.ctypes.data,
                                                     ctypes.byref(hints), ctypes.byref(s), ctypes.byref(s3)))
        return ({f: (v[0] if rows[f] == 1 else v) for f, v in out.items()},
                {f: (v[0] if v.shape[0] == 1 else v) for f, v in out3.items()})

    def solve_hinted_ex(self, p, t, z, hints: dict, fields: list[str] | None = None):
        """`solve_max3` with the general caller inputs of solve_pr76_pt_max3
        (mpmc_gpu_flash_solve_hinted_ex).  `hints` holds initial_count [ncell]
        and initial_composition [3 n, ncell] (initial starts), final_count /
        final_composition (final starts), three_phase [ncell] /
        three_phase_composition [3 n, ncell] / fraction [2, ncell] (one
        three-phase start), initial_automatic_starts and max_split_attempts;
        a missing start class is no starts of that class.  Returns (flash
        outputs, three-phase outputs)."""
        p = np.ascontiguousarray(p, dtype=np.float64)
        t = np.ascontiguousarray(t, dtype=np.float64)
        z = np.ascontiguousarray(z, dtype=np.float64)
        if z.shape != (self.n, p.shape[0]) or t.shape != p.shape:
            raise ValueError("expected p[ncell], t[ncell], z[n, ncell]")
        ncell = p.shape[0]
        keep = {}

        def arr(name, dtype, shape):
            v = hints.get(name)
            if v is None:
                return None
            a = np.ascontiguousarray(v, dtype=dtype)
            if a.shape != shape:
                raise ValueError(f"expected {name} of shape {shape}")
            keep[name] = a
            return a.ctypes.data

        h = _StartHintsEx(arr("initial_count", np.int32, (ncell,)),
                          arr("initial_composition", np.float64, (3 * self.n, ncell)),
                          arr("final_count", np.int32, (ncell,)),
                          arr("final_composition", np.float64, (3 * self.n, ncell)),
                          arr("three_phase", np.int32, (ncell,)),
                          arr("three_phase_composition", np.float64, (3 * self.n, ncell)),
                          arr("fraction", np.float64, (2, ncell)),
                          int(bool(hints.get("initial_automatic_starts", True))),
                          int(hints.get("max_split_attempts", 16)))
        fields = fields or self.fields()
        for need in ("status", "ln_k"):
            if need not in fields:
                fields = fields + [need]
        rows = output_rows(self.n)
        dtypes = {f: d for f, d, _ in OUTPUT_FIELDS}
        out = {f: np.empty((rows[f], ncell), dtypes[f]) for f in fields}
        out3 = {f: np.empty((r(self.n), ncell), d) for f, d, r in THREE_PHASE_FIELDS}
        s = _Outputs(**{f: out[f].ctypes.data for f in fields})
        s3 = _ThreePhaseOutputs(**{f: v.ctypes.data for f, v in out3.items()})
        _check(library().mpmc_gpu_flash_solve_hinted_ex(self._h, ncell, p.ctypes.data, t.ctypes.data, z.ctypes.data,
                                                        ctypes.byref(h), ctypes.byref(s), ctypes.byref(s3)))
        return ({f: (v[0] if rows[f] == 1 else v) for f, v in out.items()},
                {f: (v[0] if v.shape[0] == 1 else v) for f, v in out3.items()})

    def property_chart(self, spec: PropertyChartSpec, q, dependent=None, jacobian: bool = True) -> dict:
        """Selected-phase property chart of every cell (mpmc_gpu_flash_property_chart):
        q [(P n + 1), ncell] natural variables, dependent [P, ncell] pivot
        components or None (the last component).  Returns status [ncell],
        values [rows, ncell] and jacobian [rows, q, ncell]."""
        q = np.ascontiguousarray(q, dtype=np.float64)
        rows, cols = chart_shape(self.n, spec.phases)
        if q.ndim != 2 or q.shape[0] != cols:
            raise ValueError(f"expected q of shape [{cols}, ncell]")
        ncell = q.shape[1]
        dep = None
        if dependent is not None:
            dep = np.ascontiguousarray(dependent, dtype=np.int32)
            if dep.shape != (spec.phases, ncell):
                raise ValueError(f"expected dependent of shape [{spec.phases}, ncell]")
        out = {"status": np.empty(ncell, np.int32), "values": np.empty((rows, ncell))}
        if jacobian:
            out["jacobian"] = np.empty((rows, cols, ncell))
        o = _ChartOutputs(**{k: v.ctypes.data for k, v in out.items()})
        st = spec._struct()
        _check(library().mpmc_gpu_flash_property_chart(self._h, ncell, ctypes.byref(st), q.ctypes.data,
                                                       dep.ctypes.data if dep is not None else None,
                                                       ctypes.byref(o)))
        return out

    def property_chart_device(self, spec: PropertyChartSpec, ncell: int, q_ptr: int, dep_ptr: int,
                              out_ptrs: dict[str, int], stream: int = 0) -> None:
        """Device pointers in and out (keys status, values, jacobian; 0 skips);
        enqueued on `stream` without synchronisation."""
        o = _ChartOutputs(**out_ptrs)
        st = spec._struct()
        _check(library().mpmc_gpu_flash_property_chart_device(self._h, ncell, ctypes.byref(st), q_ptr,
                                                              dep_ptr or None, ctypes.byref(o), stream))

    def solve_host_ptrs(self, ncell: int, p_ptr: int, t_ptr: int, z_ptr: int, out_ptrs: dict[str, int]) -> None:
        """Host-buffer entry with caller-owned (e.g. pinned) host pointers."""
        s = _Outputs(**out_ptrs)
        _check(library().mpmc_gpu_flash_solve(self._h, ncell, p_ptr, t_ptr, z_ptr, ctypes.byref(s)))

    def set_launch_shape(self, values) -> None:
        """Mixed-form launch shape (see mpmc_gpu_flash_set_launch_shape)."""
        v = np.ascontiguousarray(values, dtype=np.int32)
        _check(library().mpmc_gpu_flash_set_launch_shape(self._h, v.ctypes.data, int(v.size)))

    def batch_stats(self) -> dict[str, int]:
        """Work statistics of the last mixed-form solve."""
        out = np.zeros(64, np.int64)
        k = library().mpmc_gpu_flash_batch_stats(self._h, out.ctypes.data, 64)
        return {BATCH_STATS[i]: int(out[i]) for i in range(min(k, len(BATCH_STATS)))}

    def stage_timings(self) -> dict[str, float]:
        """Per-stage device milliseconds of the last solve (stage_timing=True)."""
        ms = np.zeros(24, np.float32)
        k = library().mpmc_gpu_flash_stage_timings(self._h, ms.ctypes.data, 24)
        names = STAGES.get(self.form, [])
        return {names[i] if i < len(names) else f"stage{i}": float(ms[i]) for i in range(max(k, 0))}

    def solve_device(self, ncell: int, p_ptr: int, t_ptr: int, z_ptr: int, out_ptrs: dict[str, int],
                     stream: int = 0, warm_ptr: int = 0) -> None:
        """Device pointers in and out; enqueued on `stream` (no synchronisation).
        `warm_ptr`: device ln K warm starts [n, ncell] (0 = cold solve)."""
        s = _Outputs(**out_ptrs)
        if warm_ptr:
            _check(library().mpmc_gpu_flash_solve_device_warm(self._h, ncell, p_ptr, t_ptr, z_ptr, warm_ptr,
                                                              ctypes.byref(s), stream))
        else:
            _check(library().mpmc_gpu_flash_solve_device(self._h, ncell, p_ptr, t_ptr, z_ptr, ctypes.byref(s),
                                                         stream))

    def solve_device_noalloc(self, ncell: int, p_ptr: int, t_ptr: int, z_ptr: int, out_ptrs: dict[str, int],
                             stream: int = 0) -> None:
        """`solve_device` through the entry point that allocates no device memory
        (fixed library scratch shared by every handle on the device: calls must
        not overlap on the device)."""
        s = _Outputs(**out_ptrs)
        _check(library().mpmc_gpu_flash_solve_device_noalloc(self._h, ncell, p_ptr, t_ptr, z_ptr, ctypes.byref(s),
                                                             stream))


SERVER_STATS = ["submitted", "completed", "batches", "cells", "slots", "slot_bytes", "most_requests_in_batch",
                "most_slots_busy", "refused_busy", "expired", "in_flight", "warm_cells"]
# mpmc_server_policy fields, in order
SERVER_POLICY = ["small_request_cells", "latency_slots", "latency_batch_cells", "chunk_cells", "max_request_cells",
                 "max_in_flight", "max_deadline_us"]


class FlashServer:
    """Continuous-batching flash server (C ABI "Flash server").

    `submit()` queues host arrays and returns a ticket at once; the arrays and
    the output arrays it allocates are kept alive here until `wait()`."""

    def __init__(self, device: int = 0, slots: int = 4, max_batch_cells: int = 65536,
                 memory_budget_bytes: int = 40 << 30, form: str = "mixed", warm_cache: bool = False,
                 policy: dict | None = None):
        o = _ServerOptions(device, slots, max_batch_cells, memory_budget_bytes, FORMS[form],
                           SERVER_WARM_CACHE if warm_cache else 0)
        h = ctypes.c_void_p()
        _check(library().mpmc_flash_server_create(ctypes.byref(o), ctypes.byref(h)))
        self._h = h
        if policy:
            unknown = set(policy) - set(SERVER_POLICY)
            if unknown:
                raise ValueError(f"unknown policy fields {sorted(unknown)}")
            pol = _ServerPolicy(**{k: int(policy.get(k, 0)) for k in SERVER_POLICY})
            _check(library().mpmc_flash_server_set_policy(self._h, ctypes.byref(pol)))
        self._n = {}
        self._keep = {}
        self._mix_keep = []

    def add_mixture(self, mixture) -> int:
        arrays = [np.ascontiguousarray(a, dtype=np.float64) for a in
                  (mixture.tc, mixture.pc, mixture.omega, np.asarray(mixture.kij).reshape(-1))]
        self._mix_keep.append(arrays)
        m = _Mixture(int(mixture.n), *(a.ctypes.data for a in arrays))
        mid = ctypes.c_int32()
        _check(library().mpmc_flash_server_add_mixture(self._h, ctypes.byref(m), ctypes.byref(mid)))
        self._n[mid.value] = int(mixture.n)
        return mid.value

    def submit(self, mixture_id: int, p, t, z, fields: list[str] | None = None,
               deadline_s: float | None = None) -> int:
        n = self._n[mixture_id]
        p = np.ascontiguousarray(p, dtype=np.float64)
        t = np.ascontiguousarray(t, dtype=np.float64)
        z = np.ascontiguousarray(z, dtype=np.float64)
        ncell = p.shape[0]
        rows = output_rows(n)
        dtypes = {f: d for f, d, _ in OUTPUT_FIELDS}
        out = {f: np.empty((rows[f], ncell), dtypes[f]) for f in (fields or FLASH_FIELDS)}
        s = _Outputs(**{f: v.ctypes.data for f, v in out.items()})
        ticket = ctypes.c_uint64()
        if deadline_s is None:
            _check(library().mpmc_flash_server_submit(self._h, mixture_id, ncell, p.ctypes.data, t.ctypes.data,
                                                      z.ctypes.data, ctypes.byref(s), ctypes.byref(ticket)))
        else:
            us = int(round(deadline_s * 1e6))
            if deadline_s > 0:
                us = max(us, 1)
            _check(library().mpmc_flash_server_submit_deadline(self._h, mixture_id, ncell, p.ctypes.data,
                                                               t.ctypes.data, z.ctypes.data, ctypes.byref(s), us,
                                                               ctypes.byref(ticket)))
        self._keep[ticket.value] = (p, t, z, out)
        return ticket.value

    def wait(self, ticket: int, timeout_s: float | None = None) -> tuple[dict[str, np.ndarray], float]:
        """Outputs of the request and its submit-to-completion latency (s)."""
        lat = ctypes.c_double()
        tmo = -1 if timeout_s is None else int(timeout_s * 1e6)
        rc = library().mpmc_flash_server_wait(self._h, ticket, tmo, ctypes.byref(lat))
        # the ticket is spent unless the wait timed out (the request stays queued)
        kept = self._keep.pop(ticket, None) if rc != ERR_TIMEOUT else None
        _check(rc)
        out = kept[3]
        return {f: (v[0] if v.shape[0] == 1 else v) for f, v in out.items()}, lat.value

    def stats(self) -> dict[str, int]:
        out = np.zeros(len(SERVER_STATS), np.int64)
        k = library().mpmc_flash_server_stats(self._h, out.ctypes.data, len(SERVER_STATS))
        return {SERVER_STATS[i]: int(out[i]) for i in range(k)}

    def close(self) -> None:
        if getattr(self, "_h", None):
            library().mpmc_flash_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
