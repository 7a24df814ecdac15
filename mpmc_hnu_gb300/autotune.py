"""Launch-shape autotuner of the mixed-precision flash.

Picks, per component capacity and batch-size class, the knobs of
`mpmc_gpu_flash_set_launch_shape`: residency (blocks per SM) of the FP32
trial and attempt kernels, of the FP64 trial items, of the FP64 attempt items
and the polish, and of the per-cell kernels; whether the polish runs one cell
per thread or one per lane group; and the successive-substitution -> Newton
switch (the FP32 |r| at which the FP32 ln K iteration hands the attempt to the
FP64 polish).  It measures on the caller's own cells (device time of one
solve, CUDA events) and walks the knobs one at a time from the defaults,
keeping a change only when it is faster (coordinate descent) and leaves every
phase status of the calibration cells unchanged, so a tuning run costs about
a dozen solves.  Results are cached per GPU model, capacity and
size class in a JSON file.

    from mpmc_hnu_gb300 import autotune, flash
    g = flash.GpuFlash(mixture, "mixed")
    best = autotune.tune(g, p, t, z)      # measures, applies, caches
    autotune.apply(g, ncell)              # later: apply a cached result
"""

from __future__ import annotations

import json
import math
import os
import time

import numpy as np

from . import flash

# knob index -> candidate values tried after the default (0 = library default)
KNOBS = [
    ("trial_blocks_per_sm", 0, [2, 4]),
    ("split_blocks_per_sm", 1, [2, 4]),
    ("fp64_trial_blocks_per_sm", 2, [1, 4]),
    ("fp64_attempt_and_polish_blocks_per_sm", 3, [1, 4]),
    ("cell_blocks_per_sm", 4, [4, 8]),
    ("item_form", 5, [8, 16]),      # polish one cell per thread (8) or per lane group (16)
    ("ss_switch_1e6", 6, [10, 50]),  # FP32 |r| handover at 1e-5 or 5e-5 (default 2e-5)
]

CACHE = os.path.join(os.path.expanduser("~"), ".cache", "mpmc_gb300", "launch_shapes.json")


def capacity(n: int) -> int:
    for c in (4, 8, 12, 16, 20):
        if n <= c:
            return c
    raise ValueError("at most 20 components")


def size_class(ncell: int) -> int:
    """log4 bucket of the batch size (1, 4, 16, ... cells)."""
    return int(math.log(max(ncell, 1), 4))


def _gpu_name() -> str:
    try:
        import torch

        return torch.cuda.get_device_name(torch.cuda.current_device())
    except Exception:
        return "unknown"


def _key(n: int, ncell: int) -> str:
    return f"{_gpu_name()}|cap{capacity(n)}|size{size_class(ncell)}"


def _load() -> dict:
    try:
        with open(CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(table: dict) -> None:
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    tmp = CACHE + f".{os.getpid()}"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, CACHE)


def _measure(mixture, sensitivity: bool, device: int, shape, p, t, z, repeats: int):
    g = flash.GpuFlash(mixture, "mixed", sensitivity=sensitivity, device=device, stage_timing=True)
    try:
        g.set_launch_shape(shape)
        best = math.inf
        status = None
        for _ in range(repeats):
            status = g.solve(p, t, z, fields=["status"])["status"]
            best = min(best, sum(g.stage_timings().values()))
        return best, status
    finally:
        g.close()


def tune(handle: "flash.GpuFlash", p, t, z, repeats: int = 1, use_cache: bool = True, log=None) -> dict:
    """Tune the launch shape for `handle`'s mixture on the cells (p, t, z),
    apply it to the handle and cache it.  Returns {'shape', 'ms', 'default_ms',
    'steps'}."""
    if handle.form != flash.FORM_MIXED:
        raise ValueError("the autotuner tunes the mixed form")
    ncell = int(np.asarray(p).shape[0])
    key = _key(handle.n, ncell)
    table = _load() if use_cache else {}
    if use_cache and key in table:
        handle.set_launch_shape(table[key]["shape"])
        return table[key]
    device = 0
    shape = [0] * 7
    t0 = time.perf_counter()
    measure = lambda s: _measure(handle.mixture, handle.sensitivity, device, s, p, t, z, repeats)  # noqa: E731
    measure(shape)  # warm-up (workspace allocation, module load)
    best_ms, status0 = measure(shape)
    default_ms = best_ms
    steps = [{"shape": list(shape), "ms": default_ms}]
    for name, k, values in KNOBS:
        for v in values:
            trial = list(shape)
            trial[k] = v
            ms, status = measure(trial)
            # residency cannot change a result; the item forms round
            # differently and the SS -> Newton switch moves where FP32 stops,
            # so a candidate that changes any phase status of the calibration
            # cells is rejected outright
            same = bool(np.array_equal(status, status0))
            steps.append({"shape": trial, "ms": ms, "same_statuses": same})
            if log:
                log(f"autotune {name}={v}: {ms:.1f} ms (best {best_ms:.1f}){'' if same else ' statuses differ: rejected'}")
            if same and ms < 0.98 * best_ms:  # keep a change only for a clear gain
                best_ms, shape = ms, trial
    result = {"shape": shape, "ms": best_ms, "default_ms": default_ms, "steps": steps,
              "cells": ncell, "seconds": time.perf_counter() - t0}
    handle.set_launch_shape(shape)
    if use_cache:
        table = _load()
        table[key] = result
        _store(table)
    return result


def apply(handle: "flash.GpuFlash", ncell: int) -> bool:
    """Apply a cached shape for this handle's capacity and size class."""
    entry = _load().get(_key(handle.n, ncell))
    if not entry:
        return False
    handle.set_launch_shape(entry["shape"])
    return True
