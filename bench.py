"""Benchmark of the GB300 PR76 PT flash (one JSON line on rank 0).

Workload (default): 1,048,576 cells of one seeded Nc = 10 mixture, FP64 outputs
plus the forward-AD implicit derivatives (d ln K, d beta, d x, d y over
q = (p, T, z_0..z_8), the closure dZ/d rho and the per-phase full-chart
d[Z, ln phi]/d[p, T, x]).  70 % of the cells have p log-uniform on
[0.5, 40] MPa; 30 % sit within +-2 % of their own phase-count change pressure
(found by bisection with the flash itself on the GPU before timing).  Mixture
and cell distributions: Tc ~ U[190, 620] K, Pc ~ U[2.5, 4.6] MPa,
omega ~ U[0.01, 0.35], kij ~ U[0, 0.12], z ~ Dirichlet(1), T ~ U[280, 450] K.

A step is one pass of the chosen form (batched mixed precision) over all
cells, flash + derivatives, inputs already resident in HBM.  `e2e` times the
same step through the host-buffer C ABI entry (pinned host inputs, every
output copied back).  Inputs (96 MB) and outputs (~5 GB) exceed the 126 MB L2,
so no extra flush is needed between steps.  The plain FP64 form and the FP64
work-queue form are timed on bounded samples of the same cells; the ln K
warm-start path is timed on the full workload (warm starts from the timed
solve's own answers); the CPU oracle (the reference algorithm restated in
C++) is timed on a bounded sample with every host thread.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
# the flash server overlaps batches on up to 16 streams: give the device as
# many hardware work queues (read when the CUDA context is created)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
sys.path.insert(0, ROOT)

MIXTURE_SEED = 1001
CELL_SEED = 2001
METRIC = "PT flashes/s (Nc=10, 1M cells) mixed vs plain FP64"


# ---------------------------------------------------------------------------
# workload
def f_eval(n: int) -> float:
    """Algorithmic flops of one property evaluation (mixing with row sums,
    cubic set-up, ln phi, TPD bookkeeping)."""
    return 12 * n * (n - 1) / 2 + 6 * n + 10 * n + 40 + 14 * n + 30


def f_ad(n: int) -> float:
    return (2 / 3) * n ** 3 + 2 * n * n * (n + 1) + 2 * n * (2 * n + 1) * (n + 1) + 2 * (n + 2) * f_eval(n)


def f_jacobian(n: int) -> float:
    """One closed-form Jacobian of the Newton polish: d ln phi / d x of both
    phases (6 n^2 + 40 n + 60 each) and its LU factorisation (2/3 n^3)."""
    return 2 * (6 * n * n + 40 * n + 60) + (2 / 3) * n ** 3


def stage_flops(n: int, stats: dict, counters_sum: dict, sens_cells: int) -> dict:
    """Algorithmic flops of each stage of one mixed-form solve (the flop
    conventions of f_eval and f_ad): property evaluations x f_eval, the polish's Rachford-
    Rice iterations x 6 n, Jacobians x f_jacobian and chord solves x 2 n^2,
    the sensitivities x f_ad.  FP32 evaluations come from the per-cell work
    counters, FP64 ones from the per-stage totals."""
    fe = f_eval(n)
    return {
        "setup": ("fp64", stats["fp64_evals_setup"] * fe),
        "feed_trials": ("fp32", counters_sum["init"] * fe),
        "feed_trials64": ("fp64", stats["fp64_evals_feed_trials"] * fe),
        "split+open32": ("fp32", counters_sum["split"] * (fe + 6 * n)),
        "polish": ("fp64", stats["fp64_evals_polish"] * fe + counters_sum["rr"] * 6 * n
                   + stats["polish_jacobians"] * f_jacobian(n) + stats["polish_solves"] * 2 * n * n),
        "split64": ("fp64", stats["fp64_evals_split64"] * fe),
        "review_trials": ("fp32", counters_sum["final"] * fe),
        "review_trials64": ("fp64", stats["fp64_evals_review_trials"] * fe),
        "sensitivity": ("fp64", sens_cells * f_ad(n)),
    }


def roofline_of(n: int, stages: dict, stats: dict, counters: np.ndarray, sens_cells: int, fp64_tf: float,
                fp32_tf: float, step_ms: float, traffic_of) -> dict:
    """The dominant stage's own algorithmic flops over its CUDA-event time,
    against the measured peak of the pipe it runs on; beside it the FP32
    screening stages together and the whole step's FP64 work."""
    csum = {"init": float(counters[0].sum()), "split": float(counters[1].sum()), "final": float(counters[2].sum()),
            "rr": float(counters[4].sum())}
    fl = stage_flops(n, stats, csum, sens_cells)
    ms = dict(stages)
    ms["split+open32"] = ms.get("split", 0.0) + ms.get("open32", 0.0)
    per = {}
    for k, (pipe, flops) in fl.items():
        t = ms.get(k, 0.0)
        peak = fp64_tf if pipe == "fp64" else fp32_tf
        ach = flops / (t * 1e-3) / 1e12 if t > 0 else 0.0
        per[k] = {"pipe": pipe, "ms": round(t, 2), "flops": flops, "tflops": ach, "frac": ach / peak}
    dom = max(per, key=lambda k: per[k]["ms"])
    d = per[dom]
    fp32_keys = [k for k in per if per[k]["pipe"] == "fp32"]
    fp32_ms = sum(per[k]["ms"] for k in fp32_keys)
    fp32_fl = sum(per[k]["flops"] for k in fp32_keys)
    fp64_fl = sum(per[k]["flops"] for k in per if per[k]["pipe"] == "fp64")
    return {"bound": d["pipe"], "achieved": d["tflops"], "peak": fp64_tf if d["pipe"] == "fp64" else fp32_tf,
            "unit": "TFLOP/s", "frac": d["frac"], "traffic": traffic_of(dom), "kernel": dom, "kernel_ms": d["ms"],
            "flops_per_launch": d["flops"],
            "peak_source": "FP64/FP32 FMA-chain rates measured in this run (mpmc_hnu_gb300/csrc/peak_probe.cu)",
            "fp32_screening": {"stages": fp32_keys, "ms": round(fp32_ms, 1),
                               "tflops": fp32_fl / (fp32_ms * 1e-3) / 1e12 if fp32_ms else 0.0,
                               "frac": fp32_fl / (fp32_ms * 1e-3) / 1e12 / fp32_tf if fp32_ms else 0.0},
            "fp64_step": {"flops": fp64_fl, "tflops": fp64_fl / (step_ms * 1e-3) / 1e12,
                          "frac": fp64_fl / (step_ms * 1e-3) / 1e12 / fp64_tf},
            "stages": {k: {"ms": v["ms"], "frac": round(v["frac"], 5)} for k, v in per.items()}}


def error_report(n: int, gpu: dict, ref: dict, sens: bool) -> dict:
    """Status agreement and raw errors of a GPU solve against the oracle on
    the same cells: ln K, beta, x, y relative to max(|ref|, 1e-3) over the
    two-phase cells both call two-phase; with sensitivities, the normwise
    relative error per derivative column over cells both differentiated."""
    st, rs = np.asarray(gpu["status"]).reshape(-1), np.asarray(ref["status"]).reshape(-1)
    rep = {"cells": int(st.size), "status_mismatches": int((st != rs).sum())}
    two = (st == 1) & (rs == 1)
    rep["two_phase"] = int(two.sum())
    errs = {}
    for gname, rname in (("ln_k", "ln_k"), ("vapor_fraction", "beta"), ("liquid", "x"), ("vapor", "y")):
        a = np.atleast_2d(np.asarray(gpu[gname], dtype=float))[:, two]
        b = np.atleast_2d(np.asarray(ref[rname], dtype=float))[:, two]
        if a.size:
            e = (np.abs(a - b) / np.maximum(np.abs(b), 1e-3)).max(axis=0)
            errs[rname] = {"max": float(e.max()), "p99": float(np.percentile(e, 99))}
    if sens and "d_ln_k" in gpu:
        ok = two & (np.asarray(gpu["sensitivity_status"]).reshape(-1) == 0) & (ref["sens_status"] == 0)
        q = n + 1
        for gname, rname, rows in (("d_ln_k", "dlnk", n), ("d_vapor_fraction", "dbeta", 1), ("d_liquid", "dx", n),
                                   ("d_vapor", "dy", n)):
            a = np.asarray(gpu[gname], dtype=float)[:, ok].reshape(rows, q, -1)
            b = np.asarray(ref[rname], dtype=float)[:, ok].reshape(rows, q, -1)
            if a.size:
                num = np.abs(a - b).max(axis=0)
                den = np.maximum(np.abs(b).max(axis=0), 1e-12)
                e = (num / den).max(axis=0)
                errs[rname] = {"max": float(e.max()), "p99": float(np.percentile(e, 99))}
        rep["differentiated"] = int(ok.sum())
    rep["errors"] = {k: {kk: float(f"{vv:.3g}") for kk, vv in v.items()} for k, v in errs.items()}
    return rep


def f_chart(n: int, phases: int) -> float:
    """Algorithmic flops of one selected-phase property chart: per phase one
    property evaluation, its closed-form d[Z, ln phi]/d[p, T, x]
    (6 n^2 + 40 n + 60) and the chain rule of the five properties
    (5 (n + 2) x 8), plus 3 n per equilibrium row."""
    per_phase = f_eval(n) + 6 * n * n + 40 * n + 60 + 40 * (n + 2)
    return phases * per_phase + 3 * n * (phases - 1)


# ---------------------------------------------------------------------------
# replicas (one process per GPU; cells are independent, so no data exchange)
def cell_offset(rank: int, ncell: int) -> int:
    """First index of rank's cell stream: ranks draw disjoint cells."""
    return rank * (4 * ncell)


def max_over_ranks(value: float, world: int, device: str) -> float:
    """The job's time is its slowest rank's (a MAX all-reduce; no-op at N=1)."""
    if world <= 1:
        return value
    import torch

    tt = torch.tensor([value], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
    return float(tt.item())


def place_near(t, z, idx, noise_index, status_fn):
    """Phase-count change pressure of cells `idx` by a 9-point log-p grid and 7
    bisection steps in ln p (bracket width 0.55 * 2**-7 < 0.5 %) with
    `status_fn(p, t, z) -> status`; returns (p of the placed cells, mask, the
    final brackets [lo, hi] in ln p).  The +-2 % placement noise is drawn at
    the cells' global indices."""
    from mpmc_hnu_gb300.synth import uniform, S_NEAR

    grid = np.exp(np.linspace(np.log(0.5e6), np.log(40e6), 9))
    tt = np.repeat(t[idx], len(grid))
    zz = np.repeat(z[:, idx], len(grid), axis=1)
    pp = np.tile(grid, len(idx))
    st = status_fn(pp, tt, zz).reshape(len(idx), len(grid))
    two = st == 1
    lo = np.full(len(idx), np.nan)
    hi = np.full(len(idx), np.nan)
    lo_two = np.zeros(len(idx), bool)
    for j in range(len(grid) - 1):
        change = (two[:, j] != two[:, j + 1]) & ((st[:, j] <= 1) & (st[:, j + 1] <= 1)) & np.isnan(lo)
        lo[change] = np.log(grid[j])
        hi[change] = np.log(grid[j + 1])
        lo_two[change] = two[change, j]
    ok = np.isfinite(lo)
    sel = np.nonzero(ok)[0]
    for _ in range(7):
        mid = 0.5 * (lo[sel] + hi[sel])
        s = status_fn(np.exp(mid), t[idx[sel]], z[:, idx[sel]])
        same_as_lo = (s == 1) == lo_two[sel]
        lo[sel] = np.where(same_as_lo, mid, lo[sel])
        hi[sel] = np.where(same_as_lo, hi[sel], mid)
    u = uniform(CELL_SEED, S_NEAR, np.asarray(noise_index))
    return np.exp(0.5 * (lo + hi)) * (1.0 + 0.04 * (u - 0.5)), ok, np.stack([lo, hi])


RESAMPLE_ROUNDS = 8


def place_workload(n, p, t, z, offset, n_near, status_fn, synth):
    """The first n_near cells go within 2 % of a phase-count change pressure
    of theirs on [0.5, 40] MPa; a cell with no change there draws a new
    (T, z) at its own index from the next seed stream (up to RESAMPLE_ROUNDS
    rounds), so that the share of near-boundary cells is the requested one.
    Returns p, t, z, the placed mask over the first n_near cells and the
    brackets [2, n_near] in ln p."""
    return _place_at(n, p, t, z, offset + np.arange(p.shape[0]), n_near, status_fn, synth)


def base_cells(n: int, ncell: int, near_fraction: float, rank: int, synth):
    mix = synth.make_mixture(n, MIXTURE_SEED)
    offset = cell_offset(rank, ncell)
    p, t, z = synth.make_cells(n, ncell, CELL_SEED, offset=offset)
    n_near = int(round(near_fraction * ncell))  # the first n_near cells go near their boundary
    return mix, offset, p, t, z, n_near


def stratified(ncell: int, sample: int) -> np.ndarray:
    """Every (ncell / sample)-th cell: keeps the near/far mix of the workload."""
    return np.unique(np.linspace(0, ncell - 1, min(sample, ncell)).astype(np.int64))


def make_workload(n: int, ncell: int, near_fraction: float, rank: int, torch, flash, synth, log):
    """Seeded cells; the near-boundary subset is placed by bisection with the
    mixed form's phase status on the GPU.  Both ends of every bracket are then
    solved with the FP64 work-queue form (whose statuses equal the oracle's):
    a cell whose bracket that form does not confirm is placed again by
    bisection with the FP64 form itself.  Finally 1 % of the brackets are
    checked with the CPU oracle."""
    mix, offset, p, t, z, n_near = base_cells(n, ncell, near_fraction, rank, synth)
    info = {"near_target": n_near}
    if n_near == 0:
        return mix, p, t, z, info
    cache_dir = os.path.join(os.path.expanduser("~"), ".cache", "mpmc_gb300")
    key = f"near4_n{n}_c{ncell}_f{near_fraction}_r{rank}_m{MIXTURE_SEED}_s{CELL_SEED}.npz"
    path = os.path.join(cache_dir, key)
    if os.path.exists(path):
        d = np.load(path)
        return mix, d["p"], d["t"], d["z"], json.loads(str(d["info"]))
    t0 = time.time()
    g = flash.GpuFlash(mix, "mixed")
    p, t, z, placed, brackets = place_workload(n, p, t, z, offset, n_near,
                                               lambda a, b, c: g.solve(a, b, c, fields=["status"])["status"], synth)
    g.close()
    # every bracket confirmed by the FP64 work-queue form
    g64 = flash.GpuFlash(mix, "batched")
    status64 = lambda a, b, c: g64.solve(a, b, c, fields=["status"])["status"]  # noqa: E731
    idx = np.nonzero(placed)[0]
    ends = [status64(np.exp(brackets[k, idx]), t[idx], np.ascontiguousarray(z[:, idx])) for k in (0, 1)]
    bad = idx[(ends[0] == 1) == (ends[1] == 1)]
    if bad.size:
        p2, t2, z2, placed2, br2 = _place_at(n, p[bad], t[bad], np.ascontiguousarray(z[:, bad]), offset + bad,
                                             bad.size, status64, synth)
        p[bad], t[bad], z[:, bad] = p2, t2, z2
        placed[bad] = placed2
        brackets[:, bad] = br2
    g64.close()
    info.update({"near_placed": int(placed.sum()), "placement_s": round(time.time() - t0, 1),
                 "fp64_confirmation": {"brackets": int(idx.size), "confirmed": int(idx.size - bad.size),
                                       "placed_again_with_fp64": int(bad.size)}})
    # spot check: the oracle's statuses at both ends of 1 % of the brackets
    from oracle import pyoracle

    chk = np.nonzero(placed)[0][::100]
    ends = np.exp(brackets[:, chk])
    st = [pyoracle.flash(mix, ends[k], t[chk], z[:, chk], threads=os.cpu_count() or 1)["status"] for k in (0, 1)]
    straddle = (st[0] == 1) != (st[1] == 1)
    info["placement_check"] = {"cells": int(chk.size), "brackets_confirmed_by_oracle": int(straddle.sum())}
    log(f"near-boundary placement: {info['near_placed']}/{n_near} cells ({info['placement_s']} s); FP64 form "
        f"confirms {idx.size - bad.size}/{idx.size} brackets ({bad.size} placed again with it); oracle confirms "
        f"{int(straddle.sum())}/{chk.size} checked brackets")
    os.makedirs(cache_dir, exist_ok=True)
    np.savez(path, p=p, t=t, z=z, info=json.dumps(info))
    return mix, p, t, z, info


def cpu_workload_sample(n: int, ncell: int, near_fraction: float, sample: int, threads: int, synth):
    """The stratified sample of the workload placed by the CPU oracle alone
    (same grid, bisection, resampling and noise as the GPU placement)."""
    from oracle import pyoracle

    mix, offset, p, t, z, n_near = base_cells(n, ncell, near_fraction, 0, synth)
    idx = stratified(ncell, sample)
    p, t, z = p[idx].copy(), t[idx].copy(), np.ascontiguousarray(z[:, idx])
    near = np.nonzero(idx < n_near)[0]
    if near.size:
        # place the sampled near cells at their own global indices
        order = np.concatenate([near, np.setdiff1d(np.arange(idx.size), near)])
        pp, tt, zz = p[order], t[order], z[:, order]
        status_fn = lambda a, b, c: pyoracle.flash(mix, a, b, c, threads=threads)["status"]  # noqa: E731
        pp2, tt2, zz2, _, _ = _place_at(n, pp, tt, zz, offset + idx[order], near.size, status_fn, synth)
        inv = np.argsort(order)
        p, t, z = pp2[inv], tt2[inv], np.ascontiguousarray(zz2[:, inv])
    return mix, p, t, z


def _place_at(n, p, t, z, gidx, n_near, status_fn, synth):
    """place_workload for cells whose global indices are gidx: the first
    n_near of them are placed."""
    p, t, z = p.copy(), t.copy(), z.copy()
    placed = np.zeros(n_near, bool)
    brackets = np.full((2, n_near), np.nan)
    todo = np.arange(n_near)
    for rnd in range(RESAMPLE_ROUNDS + 1):
        if rnd > 0:
            _, t_new, z_new = synth.make_cells_at(n, gidx[todo], CELL_SEED + 7919 * rnd)
            t[todo], z[:, todo] = t_new, z_new
        pb, ok, br = place_near(t, z, todo, gidx[todo], status_fn)
        p[todo[ok]] = pb[ok]
        placed[todo[ok]] = True
        brackets[:, todo[ok]] = br[:, ok]
        todo = todo[~ok]
        if todo.size == 0:
            break
    return p, t, np.ascontiguousarray(z), placed, brackets


# ---------------------------------------------------------------------------
class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, device: int):
        self.samples = []
        self.proc = None
        self.device = device

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        reasons = set()
        for s in self.samples:
            for name, v in zip(["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"],
                               s[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def measured_peaks(flash_pkg):
    lib = ctypes.CDLL(os.path.join(os.path.dirname(flash_pkg.__file__), "_lib", "libmpmc_gb300_probe.so"))
    lib.mpmc_probe_fp64_flops.restype = ctypes.c_double
    lib.mpmc_probe_fp32_flops.restype = ctypes.c_double
    return lib.mpmc_probe_fp64_flops(200) / 1e12, lib.mpmc_probe_fp32_flops(2000) / 1e12


def cpu_flash_rate(mix, p, t, z, threads: int, sens: bool):
    """The CPU oracle (reference algorithm in C++) over the given cells."""
    from oracle import pyoracle

    pyoracle.build()
    t0 = time.perf_counter()
    pyoracle.flash(mix, p, t, z, threads=threads, sens=sens)
    dt = time.perf_counter() - t0
    return p.shape[0] / dt, dt


# ---------------------------------------------------------------------------
# config 2: 4 mixtures x cells at N = 4, 8, 12, 20, warm-started as in a time step
CONFIG2_COMPONENTS = (4, 8, 12, 20)


def wilson_ln_k(mix, p, t):
    """Wilson's K: ln K_i = ln(Pc_i / p) + 5.373 (1 + omega_i)(1 - Tc_i / T)."""
    tc, pc, om = (np.asarray(a)[:, None] for a in (mix.tc, mix.pc, mix.omega))
    return np.log(pc / p[None, :]) + 5.373 * (1.0 + om) * (1.0 - tc / t[None, :])


def kernels_per_solve(form: str, sens: bool) -> int:
    """Kernels one cold device-resident solve launches (counted in the ncu
    launch list of one solve): the mixed form's pass has 17 (setup, feed
    trials32 / classify / trials64, decide, split32, polish, open32, compete,
    split64, select64, relist, review trials32 / classify / trials64, finish,
    fallback); the FP64 work-queue form's 15 (no FP32 ln K iterations, its
    trials queued by rerun_all); the mixed form adds the exact sub-solve
    (gather, the FP64 form's 15, scatter); the plain form is one kernel; plus
    the sensitivity kernel."""
    per = {"plain": 1, "batched": 15, "mixed": 34}[form]
    return per + (1 if sens else 0)


def _timed(fn, stream, torch):
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def config2_leg(flash, synth, torch, device: int, stream, ncell: int, fp64_sample: int, plain_sample: int,
                warm_fraction: float, log):
    """Per mixture (N = 4, 8, 12, 20; the bench generator): a cold solve gives
    the converged ln K* of the two-phase cells; then `warm_fraction` of all
    cells start from ln K* + 0.1 N(0, 1) where they have one, and every other
    cell starts cold.  A cold start is the reference's own (the feed's TPD
    stability test): a Wilson-K start through the warm entry would only add a
    collapsing attempt to every single-phase cell.  Timed, flash without
    sensitivities:
      mixed      the mixed form's warm solve of all `ncell` cells (CUDA graph);
      fp64_queue the FP64 work-queue form's warm solve of a stratified sample;
      plain      the plain FP64 one-thread-per-cell kernel (the reference
                 algorithm, cold: it has no ln K start) on a stratified sample.
    Whole-job flashes/s per arm, per-mixture figures and the mixed form's
    slowest stages."""
    dev = torch.device(f"cuda:{device}")
    per, tot = {}, {"mixed": [0, 0.0], "fp64_queue": [0, 0.0], "plain": [0, 0.0]}
    fields = ["status", "vapor_fraction", "liquid", "vapor", "ln_k", "z_liquid", "z_vapor"]
    for n in CONFIG2_COMPONENTS:
        mix = synth.make_mixture(n, 1100 + n)
        p, t, z = synth.make_cells(n, ncell, 2100 + n)
        dp, dt, dz = (torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (p, t, z))
        rows = flash.output_rows(n)

        def buffers(count):
            o = {f: torch.empty((rows[f], count), dtype=torch.int32 if f == "status" else torch.float64, device=dev)
                 for f in fields}
            return o, {f: v.data_ptr() for f, v in o.items()}

        outs, ptrs = buffers(ncell)
        g = flash.GpuFlash(mix, "mixed", device=device, graphs=True)
        stream.wait_stream(torch.cuda.current_stream(dev))
        g.solve_device(ncell, dp.data_ptr(), dt.data_ptr(), dz.data_ptr(), ptrs, stream.cuda_stream)
        torch.cuda.synchronize()
        rng = np.random.default_rng(17 + n)
        st = outs["status"][0].cpu().numpy()
        lnk = outs["ln_k"].cpu().numpy()
        pick = (st == 1) & (rng.random(ncell) < warm_fraction)
        warm = np.where(pick[None, :], lnk + 0.1 * rng.standard_normal(lnk.shape), np.nan)
        dwarm = torch.from_numpy(np.ascontiguousarray(warm)).to(dev)
        cold_status = st.copy()
        call = lambda: g.solve_device(ncell, dp.data_ptr(), dt.data_ptr(), dz.data_ptr(), ptrs,  # noqa: E731
                                      stream.cuda_stream, warm_ptr=dwarm.data_ptr())
        _timed(call, stream, torch)
        ms = _timed(call, stream, torch)
        agree = float((outs["status"][0].cpu().numpy() == cold_status).mean())
        g.close()
        # the slowest stages of the warm solve (a separate instrumented call)
        gt = flash.GpuFlash(mix, "mixed", device=device, stage_timing=True)
        gt.solve_device(ncell, dp.data_ptr(), dt.data_ptr(), dz.data_ptr(), ptrs, stream.cuda_stream,
                        warm_ptr=dwarm.data_ptr())
        stg = gt.stage_timings()
        bs = gt.batch_stats()
        gt.close()
        top = sorted(stg.items(), key=lambda kv: -kv[1])[:3]
        entry = {"mixed": {"value": ncell / (ms * 1e-3), "ms": round(ms, 1), "status_agreement_with_cold": agree,
                           "warm_cells": bs.get("warm_cells"), "sent_to_cold_pass": bs.get("warm_redo"),
                           "top_stages_ms": {k: round(v, 1) for k, v in top}}}
        for arm, form, size, use_warm in (("fp64_queue", "batched", fp64_sample, True),
                                          ("plain", "plain", plain_sample, False)):
            if size <= 0:
                continue
            sel = stratified(ncell, size)
            isel = torch.from_numpy(sel).to(dev)
            sp, stt, sz = dp[isel].contiguous(), dt[isel].contiguous(), dz[:, isel].contiguous()
            sw = dwarm[:, isel].contiguous()
            so, sptr = buffers(sel.size)
            gs = flash.GpuFlash(mix, form, device=device)
            kw = {"warm_ptr": sw.data_ptr()} if use_warm else {}
            call_s = lambda: gs.solve_device(sel.size, sp.data_ptr(), stt.data_ptr(), sz.data_ptr(), sptr,  # noqa: E731
                                             stream.cuda_stream, **kw)
            sms = _timed(call_s, stream, torch)
            agree_s = float((so["status"][0].cpu().numpy() == outs["status"][0][isel].cpu().numpy()).mean())
            gs.close()
            entry[arm] = {"value": sel.size / (sms * 1e-3), "cells": int(sel.size), "ms": round(sms, 1),
                          "status_agreement_with_mixed": agree_s}
            tot[arm][0] += sel.size
            tot[arm][1] += sms
        tot["mixed"][0] += ncell
        tot["mixed"][1] += ms
        per[f"n{n}"] = entry
        log(f"config 2, N={n}: mixed {entry['mixed']['value']:.0f}/s" +
            "".join(f", {a} {entry[a]['value']:.0f}/s" for a in ("fp64_queue", "plain") if a in entry))
        del outs, dp, dt, dz, dwarm
    res = {arm: {"value": c / (m * 1e-3) if m else None, "unit": "flashes/s", "cells": c} for arm, (c, m) in tot.items()}
    return {"whole_job": res, "per_mixture": per,
            "setup": f"4 mixtures x {ncell} cells (N = 4, 8, 12, 20); {warm_fraction:.0%} of all cells warm from "
                     "ln K* + 0.1 N(0,1) where the cold solve converged, every other cell cold (the reference's "
                     "TPD test); the FP64 arms on stratified samples (the plain kernel cold); no sensitivities"}


# ---------------------------------------------------------------------------
# config 3: near-critical cells, mixed form with AD, errors against the oracle
def config3_leg(flash, synth, torch, device: int, stream, n: int, ncell: int, sample: int, threads: int, log):
    """1M cells, 20 % near-critical (T within 1 % of the Kay pseudo-critical
    temperature, p log-uniform on [10, 40] MPa), the mixed form with implicit
    sensitivities: flashes/s over one timed solve, and error_report against
    the oracle (flash + AD) on a stratified sample."""
    from oracle import pyoracle

    dev = torch.device(f"cuda:{device}")
    mix = synth.make_mixture(n, 3100 + n)
    p, t, z = synth.make_near_critical_cells(mix, ncell, 4100 + n)
    dp, dt, dz = (torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (p, t, z))
    g = flash.GpuFlash(mix, "mixed", sensitivity=True, device=device, graphs=True)
    rows = flash.output_rows(n)
    dtypes = {f: d for f, d, _ in flash.OUTPUT_FIELDS}
    outs = {f: torch.empty((rows[f], ncell), dtype=torch.int32 if dtypes[f] == np.int32 else torch.float64,
                           device=dev) for f in g.fields()}
    ptrs = {f: v.data_ptr() for f, v in outs.items()}
    stream.wait_stream(torch.cuda.current_stream(dev))
    call = lambda: g.solve_device(ncell, dp.data_ptr(), dt.data_ptr(), dz.data_ptr(), ptrs,  # noqa: E731
                                  stream.cuda_stream)
    _timed(call, stream, torch)
    ms = _timed(call, stream, torch)
    g.close()
    sel = stratified(ncell, sample)
    isel = torch.from_numpy(sel).to(dev)
    gpu = {f: (v[:, isel].cpu().numpy()) for f, v in outs.items()}
    gpu = {f: (a[0] if a.shape[0] == 1 else a) for f, a in gpu.items()}
    t0 = time.perf_counter()
    ref = pyoracle.flash(mix, p[sel], t[sel], z[:, sel], threads=threads, sens=True)
    rep = error_report(n, gpu, ref, True)
    log(f"config 3, N={n}: {ncell / (ms * 1e-3):.0f} flashes/s; {rep['status_mismatches']} status mismatches "
        f"in {sel.size} (oracle {time.perf_counter() - t0:.1f} s)")
    del outs, dp, dt, dz
    return {"value": ncell / (ms * 1e-3), "unit": "flashes/s", "ms": round(ms, 1), "cells": ncell, "components": n,
            "vs_oracle": rep, "sample": f"{sel.size} stratified cells, oracle flash + AD"}


# ---------------------------------------------------------------------------
# config 0: the reference's CPU-runnable case, 4,096 cells at N = 6
def config0_leg(flash, synth, threads: int):
    """The CPU oracle (the reference algorithm) on 4,096 cells of one N = 6
    mixture on every host core, and the mixed form on the same cells (host
    buffers in and out, one call)."""
    from oracle import pyoracle

    mix = synth.make_mixture(6, 600)
    p, t, z = synth.make_cells(6, 4096, 601)
    pyoracle.build()
    t0 = time.perf_counter()
    ref = pyoracle.flash(mix, p, t, z, threads=threads)
    cpu_s = time.perf_counter() - t0
    g = flash.GpuFlash(mix, "mixed")
    g.solve(p, t, z, fields=["status"])
    t0 = time.perf_counter()
    out = g.solve(p, t, z, fields=["status"])
    gpu_s = time.perf_counter() - t0
    g.close()
    return {"cpu": {"value": p.size / cpu_s, "unit": "flashes/s", "cores": threads, "kind": "port"},
            "gpu_mixed_host_buffers": {"value": p.size / gpu_s, "unit": "flashes/s"},
            "status_mismatches": int((out["status"] != ref["status"]).sum()), "cells": int(p.size)}


# ---------------------------------------------------------------------------
# selected-phase property chart (the flow module's per-cell property and
# Jacobian publication, mpmc_gpu_flash_property_chart)
CHART_N, CHART_PHASES = 10, 2


def chart_states(n: int, phases: int, ncell: int, seed: int):
    """Two-phase chart states: p log-uniform on [0.5, 40] MPa, T ~ U[280, 450] K,
    a saturation ~ U[0.05, 0.95], each phase's composition ~ Dirichlet(1) with
    the last component as the pivot (rows [P n + 1, ncell])."""
    rng = np.random.default_rng(seed)
    p = np.exp(rng.uniform(np.log(5.0e5), np.log(4.0e7), ncell))
    t = rng.uniform(280.0, 450.0, ncell)
    sat = rng.uniform(0.05, 0.95, (phases - 1, ncell))
    blocks = [rng.dirichlet(np.ones(n), ncell).T[:n - 1] for _ in range(phases)]
    return np.ascontiguousarray(np.vstack([p[None], t[None], sat] + blocks))


def chart_leg(flash, synth, torch, device: int, stream, ncell: int, threads: int, cpu_sample: int, hbm_gbs,
              fp64_tf):
    """Device-resident chart of `ncell` two-phase cells at 10 components (roots
    0 and 0, affine viscosity/enthalpy model): cells/s over 5 launches timed
    with CUDA events on the launching stream; its algorithmic FP64 flops
    (f_chart) against the measured FP64 peak, its algorithmic bytes (chart
    read, status, values and Jacobian written) against the measured copy
    bandwidth; and the CPU oracle on a sample of the same cells."""
    n, phases = CHART_N, CHART_PHASES
    rows, cols = flash.chart_shape(n, phases)
    mix = synth.make_mixture(n, 1001)
    rng = np.random.default_rng(33)
    visc = np.concatenate([[8.0e-6, 1.0e-12, 1.0e-8, 1.0e-12, 1.0e-4, 1.0e-9, 1.0e-7], rng.uniform(0, 1e-6, n)])
    enth = np.concatenate([[0.0, 2.0e-4, 1200.0, 0.5, 1.0e4, 0.1, 10.0], rng.uniform(0, 2000.0, n)])
    spec = flash.PropertyChartSpec(phases, [0, 0], rng.uniform(0.016, 0.2, n), visc, enth)
    q = chart_states(n, phases, ncell, 34)
    dev = torch.device(f"cuda:{device}")
    dq = torch.from_numpy(q).to(dev)
    st = torch.empty(ncell, dtype=torch.int32, device=dev)
    vals = torch.empty((rows, ncell), dtype=torch.float64, device=dev)
    jac = torch.empty((rows, cols, ncell), dtype=torch.float64, device=dev)
    ptrs = {"status": st.data_ptr(), "values": vals.data_ptr(), "jacobian": jac.data_ptr()}
    g = flash.GpuFlash(mix, "plain", device=device)
    stream.wait_stream(torch.cuda.current_stream(dev))
    for _ in range(2):
        g.property_chart_device(spec, ncell, dq.data_ptr(), 0, ptrs, stream.cuda_stream)
    torch.cuda.synchronize()
    launches = 5
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(launches):
        g.property_chart_device(spec, ncell, dq.data_ptr(), 0, ptrs, stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    g.close()
    ms = e0.elapsed_time(e1) / launches
    status = st.cpu().numpy()
    bytes_per_cell = cols * 8 + 4 + rows * 8 + rows * cols * 8
    gbs = bytes_per_cell * ncell / (ms * 1e-3) / 1e9
    flops = f_chart(n, phases) * ncell
    tfs = flops / (ms * 1e-3) / 1e12
    leg = {"value": ncell / (ms * 1e-3), "unit": "cells/s", "cells": ncell, "ms_per_launch": ms,
           "components": n, "phases": phases,
           "statuses": {str(k): int(v) for k, v in enumerate(np.bincount(status, minlength=7)) if v},
           "roofline": {"bound": "fp64", "achieved": tfs, "peak": fp64_tf, "unit": "TFLOP/s",
                        "frac": tfs / fp64_tf if fp64_tf else None, "flops_per_cell": f_chart(n, phases),
                        "peak_source": "measured in this run by mpmc_hnu_gb300/csrc/peak_probe.cu (FMA chains)",
                        "hbm": {"achieved": gbs, "peak": hbm_gbs, "unit": "GB/s",
                                "frac": gbs / hbm_gbs if hbm_gbs else None, "bytes_per_cell": bytes_per_cell,
                                "peak_source": "hbm_gbs of MEASURED_PEAKS.json"}},
           "dtype": "f64", "l2_flush": f"outputs {bytes_per_cell * ncell / 1e9:.1f} GB per launch, far above L2"}
    if cpu_sample > 0:
        from oracle import pyoracle

        cols_sel = np.arange(0, ncell, max(1, ncell // cpu_sample))[:cpu_sample]
        sel = np.ascontiguousarray(q[:, cols_sel])
        pyoracle.build()
        t0 = time.perf_counter()
        ref = pyoracle.property_chart(mix, phases, [0, 0], spec.molar_mass, visc, enth, sel, None, threads=threads)
        dt = time.perf_counter() - t0
        leg["cpu_baseline"] = {"value": sel.shape[1] / dt, "unit": "cells/s", "cores": threads, "kind": "port",
                               "sample": f"{sel.shape[1]} of the same cells (every {ncell // sel.shape[1]}th), "
                                         f"{dt:.1f} s wall; the oracle is bit-identical to the reference's chart"}
        # parity of the timed launch's outputs on those cells
        isel = torch.from_numpy(cols_sel).to(dev)
        gv, gj = vals[:, isel].cpu().numpy(), jac[:, :, isel].cpu().numpy()
        ok = (status[cols_sel] == 0) & (ref["status"] == 0)
        rv, rj = ref["values"][:, ok], ref["jacobian"][:, :, ok]
        verr = float((np.abs(gv[:, ok] - rv) / np.maximum(np.abs(rv), 1.0)).max()) if ok.any() else None
        scale = np.maximum(np.abs(rj).max(axis=1, keepdims=True), 1e-300)
        jerr = float((np.abs(gj[:, :, ok] - rj) / scale).max()) if ok.any() else None
        leg["vs_oracle"] = {"cells": int(cols_sel.size),
                            "status_mismatches": int((status[cols_sel] != ref["status"]).sum()),
                            "values_max_rel": verr, "jacobian_max_of_row_scale": jerr}
    del dq, vals, jac
    return leg


# ---------------------------------------------------------------------------
# ---------------------------------------------------------------------------
# serving (continuous batching through the flash server)
SERVING_MIXTURES = [(3, 501), (3, 502), (6, 503), (6, 504), (10, 505), (10, 506), (20, 507), (20, 508)]


def serving_pool(synth, count: int, seed: int = 77):
    """Seeded requests: mixture among 8 (N in {3, 6, 10, 20}), cells per request
    floor(exp(U ln 65536)), cells from the base distributions.  Half re-query
    an earlier fresh request (drawn uniformly): its mixture and cells (drawn
    with replacement) at p * exp(N(0, 0.02)), T + N(0, 1 K).  A re-query
    perturbs a fresh request's states, never another re-query's, so repeated
    re-queries do not random-walk the states into one small (p, T) region."""
    rng = np.random.default_rng(seed)
    pool, fresh = [], []
    for k in range(count):
        ncell = max(1, int(np.exp(rng.uniform(0.0, np.log(65536.0)))))
        if fresh and rng.uniform() < 0.5:
            j, p0, t0, z0 = pool[fresh[int(rng.integers(0, len(fresh)))]]
            src = rng.integers(0, p0.shape[0], ncell)
            p = p0[src] * np.exp(rng.normal(0.0, 0.02, ncell))
            t = t0[src] + rng.normal(0.0, 1.0, ncell)
            z = np.ascontiguousarray(z0[:, src])
        else:
            j = int(rng.integers(0, len(SERVING_MIXTURES)))
            n = SERVING_MIXTURES[j][0]
            p, t, z = synth.make_cells(n, ncell, 9000 + k)
            fresh.append(k)
        pool.append((j, np.ascontiguousarray(p), np.ascontiguousarray(t), z))
    return pool


def serving_closed(server, ids, pool, outstanding, seconds):
    """Closed loop: keep `outstanding` requests queued for `seconds`, then drain.
    Its throughput is the server's saturated rate at that queue depth."""
    done = []
    queue = []
    k = 0
    t0 = time.perf_counter()

    def submit():
        nonlocal k
        j, p, t, z = pool[k % len(pool)]
        k += 1
        queue.append((server.submit(ids[j], p, t, z, fields=["status", "vapor_fraction"]), p.shape[0]))

    for _ in range(outstanding):
        submit()
    while queue:
        tk, ncell = queue.pop(0)
        _, lat = server.wait(tk)
        done.append((ncell, lat))
        if time.perf_counter() - t0 < seconds:
            submit()
    return done, time.perf_counter() - t0


def serving_run(server, ids, pool, rate, seconds):
    """Open-loop Poisson arrivals at `rate` requests/s for `seconds` (rate None:
    submit the whole pool at once, i.e. saturation).  Returns per-request
    (cells, latency s) and the wall time to drain."""
    rng = np.random.default_rng(4242)
    done = []
    tickets = []
    lock = threading.Lock()
    finished = threading.Event()

    def waiter():
        k = 0
        while True:
            with lock:
                if k < len(tickets):
                    tk, ncell = tickets[k]
                else:
                    tk = None
            if tk is None:
                if finished.is_set():
                    with lock:
                        if k >= len(tickets):
                            return
                    continue
                time.sleep(0.0002)
                continue
            _, lat = server.wait(tk)
            done.append((ncell, lat))
            k += 1

    th = threading.Thread(target=waiter)
    th.start()
    t0 = time.perf_counter()
    k = 0
    if rate is None:
        for j, p, t, z in pool:
            tk = server.submit(ids[j], p, t, z, fields=["status", "vapor_fraction"])
            with lock:
                tickets.append((tk, p.shape[0]))
    else:
        next_t = t0
        while True:
            next_t += rng.exponential(1.0 / rate)
            if next_t - t0 > seconds:
                break
            delay = next_t - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            j, p, t, z = pool[k % len(pool)]
            k += 1
            tk = server.submit(ids[j], p, t, z, fields=["status", "vapor_fraction"])
            with lock:
                tickets.append((tk, p.shape[0]))
    finished.set()
    th.join()
    return done, time.perf_counter() - t0


def serving_summary(done, wall, offered=None):
    cells = np.array([c for c, _ in done], dtype=np.float64)
    lat = np.array([l for _, l in done]) * 1e3
    small = cells <= 4096
    out = {"requests": int(len(done)), "flashes_per_s": float(cells.sum() / wall),
           "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99))}
    if small.any():
        out["p50_ms_le4096"] = float(np.percentile(lat[small], 50))
        out["p99_ms_le4096"] = float(np.percentile(lat[small], 99))
    if offered is not None:
        out["offered_req_per_s"] = float(offered)
    return out


# scheduling of the serving leg: requests of at most 4,096 cells on 4 latency
# slots of the highest stream priority, larger ones cut into 16,384-cell
# chunks on the other 12; each mixture's recent ln K cached on the device
SERVING_SLOTS = 16
SERVING_BATCH = 16384
SERVING_POLICY = {"small_request_cells": 4096, "latency_slots": 4, "latency_batch_cells": SERVING_BATCH,
                  "chunk_cells": SERVING_BATCH, "max_request_cells": 65536}


def serving_probe(flash, synth, device, seconds, fractions, log):
    """Saturated throughput (closed loop), then open-loop Poisson load at each
    fraction of the saturated request rate, `seconds` each, every run on its
    own freshly drawn requests."""
    server = flash.FlashServer(device=device, slots=SERVING_SLOTS, max_batch_cells=SERVING_BATCH,
                               memory_budget_bytes=40 << 30, warm_cache=True, policy=SERVING_POLICY)
    ids = [server.add_mixture(synth.make_mixture(n, s)) for n, s in SERVING_MIXTURES]
    serving_run(server, ids, serving_pool(synth, 16, seed=70), None, 0)  # warm-up
    sat_s = min(seconds, 20.0)
    done, wall = serving_closed(server, ids, serving_pool(synth, 1024, seed=71), 2 * SERVING_SLOTS, sat_s)
    sat = serving_summary(done, wall)
    sat_req = len(done) / wall
    log(f"serving: saturated {sat['flashes_per_s']:.0f} flashes/s, {sat_req:.1f} requests/s "
        f"({2 * SERVING_SLOTS} requests outstanding)")
    rates = []
    for k, f in enumerate(fractions):
        count = int(f * sat_req * seconds * 1.3) + 16
        d, w = serving_run(server, ids, serving_pool(synth, count, seed=80 + k), f * sat_req, seconds)
        r = serving_summary(d, w, f * sat_req)
        r["fraction_of_saturated_requests"] = f
        r["fraction_of_saturated_flashes"] = r["flashes_per_s"] / sat["flashes_per_s"]
        rates.append(r)
        log(f"serving at {f:.0%}: {r}")
    st = server.stats()
    server.close()
    return {"saturated_flashes_per_s": sat["flashes_per_s"], "saturated_req_per_s": sat_req,
            "saturation": f"closed loop, {2 * SERVING_SLOTS} requests outstanding, {sat_s:.0f} s",
            "saturated_latency": sat, "rates": rates, "slots": st.get("slots"), "max_batch_cells": SERVING_BATCH,
            "policy": SERVING_POLICY, "warm_cache_cells": st.get("warm_cells"),
            "workload": "8 seeded mixtures (N 3, 6, 10, 20), cells/request log-uniform 1-65536, "
                        "half re-query the previous mixture with perturbed p, T; open-loop Poisson arrivals",
            "seconds_per_rate": seconds}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="mixed", choices=["mixed", "batched", "plain"])
    ap.add_argument("--n", type=int, default=10)
    ap.add_argument("--cells", type=int, default=1 << 20)
    ap.add_argument("--near-fraction", type=float, default=0.3)
    ap.add_argument("--no-ad", action="store_true")
    ap.add_argument("--sensitivity-lanes", action="store_true",
                    help="take the sensitivities with the opt-in lane-group kernel (MPMC_FLAG_SENSITIVITY_LANES)")
    ap.add_argument("--polish-stream", action="store_true",
                    help="run the opt-in state-machine FP64 polish (MPMC_FLAG_POLISH_STREAM)")
    ap.add_argument("--plain-sample", type=int, default=65536)
    ap.add_argument("--batched-sample", type=int, default=131072)
    ap.add_argument("--warm-fraction", type=float, default=0.75,
                    help="share of cells given a perturbed converged ln K in the warm-start legs (0 = skip)")
    ap.add_argument("--cpu-sample", type=int, default=65536)
    ap.add_argument("--profile", action="store_true", help="one untimed solve of the workload (for ncu)")
    ap.add_argument("--serving-seconds", type=float, default=60.0,
                    help="seconds per arrival rate of the serving sweep (0 = skip)")
    ap.add_argument("--serving-fractions", default="0.5,0.7,0.9",
                    help="arrival rates of the serving sweep, as fractions of the saturated request rate")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shape")
    ap.add_argument("--launch-shape", default="",
                    help="comma-separated mixed-form launch shape to use instead of autotuning")
    ap.add_argument("--config2-cells", type=int, default=1 << 20,
                    help="cells per mixture of the 4-mixture warm-start workload (0 = skip)")
    ap.add_argument("--config3-cells", type=int, default=1 << 20,
                    help="cells of each near-critical workload, N = 10 and N = 20 (0 = skip)")
    ap.add_argument("--chart-cells", type=int, default=1 << 20,
                    help="cells of the selected-phase property chart leg (0 = skip)")
    ap.add_argument("--serving-sweep", action="store_true",
                    help="only the serving sweep: 10%%..100%% of saturation, --serving-seconds per rate")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    log = (lambda m: print(f"[bench] {m}", file=sys.stderr, flush=True)) if rank == 0 else (lambda m: None)
    sens = not args.no_ad
    threads = os.cpu_count() or 1

    from mpmc_hnu_gb300 import synth

    # the workload: identical in both arms
    workload = {"workload": f"PR76 two-phase PT flash + implicit AD, Nc={args.n}, {args.cells} cells per GPU, "
                            f"{int(args.near_fraction * 100)}% within 2% of the phase-boundary pressure",
                "cells_per_gpu": args.cells, "components": args.n, "sensitivity": sens,
                "l2_flush": "inputs+outputs larger than L2", "parallelism": f"replicas{world}"}
    if args.sensitivity_lanes:
        workload["sensitivity_kernel"] = "lane groups (MPMC_FLAG_SENSITIVITY_LANES)"
    if args.polish_stream:
        workload["polish_kernel"] = "state machine (MPMC_FLAG_POLISH_STREAM)"

    if args.impl == "reference":
        # the reference's CPU flash (C++ restatement; the reference sources are
        # not present on the GPU host) on every host core; rank 0 only
        if rank != 0:
            return
        t0 = time.time()
        mix, p, t, z = cpu_workload_sample(args.n, args.cells, args.near_fraction, args.cpu_sample, threads, synth)
        log(f"reference arm: {p.shape[0]} stratified cells placed in {time.time() - t0:.1f} s")
        rates = []
        for k in range(args.warmup + args.steps):
            r, _ = cpu_flash_rate(mix, p, t, z, threads, sens)
            if k >= args.warmup:
                rates.append(r)
        v = statistics.median(rates)
        sample = (f"{p.shape[0]} stratified cells (every {args.cells // p.shape[0]}th) of the workload per step, "
                  f"near-boundary cells placed by the same bisection and resampling with the CPU flash; flash"
                  f"{' + AD' if sens else ''}")
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "flashes/s",
                "n_gpus": 0, "steps": args.steps, "warmup": args.warmup, "ms_per_step": p.shape[0] / v * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded generator, stratified sample)", "config": workload,
                "cpu_baseline": {"value": v, "unit": "flashes/s", "cores": threads, "kind": "port",
                                 "sample": sample},
                "e2e": {"value": v, "unit": "flashes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import torch

    from mpmc_hnu_gb300 import build, flash

    build.build()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
        torch.cuda.set_device(local_rank)
    device = torch.cuda.current_device()
    torch.zeros(1, device="cuda")

    if args.serving_sweep:
        if rank == 0:
            sv = serving_probe(flash, synth, device, args.serving_seconds or 60.0,
                               [0.1, 0.3, 0.5, 0.7, 0.9, 1.0], log)
            print(json.dumps({"metric": "serving p50/p99 latency and flashes/s per arrival rate",
                              "unit": "ms", "n_gpus": 1, "data": "synthetic (seeded generator)",
                              "serving": sv}), flush=True)
        return

    mix, p, t, z, place_info = make_workload(args.n, args.cells, args.near_fraction, rank, torch, flash, synth, log)
    n, ncell = args.n, args.cells
    # the timed handle replays its launch sequence as a CUDA graph (same cells
    # and buffers every step)
    lanes, pstream = bool(args.sensitivity_lanes), bool(args.polish_stream)
    g = flash.GpuFlash(mix, args.form, sensitivity=sens, device=device, graphs=True, sensitivity_lanes=lanes,
                       polish_stream=pstream)
    tuning = None
    if args.form == "mixed" and args.launch_shape:
        tuning = {"shape": [int(v) for v in args.launch_shape.split(",")]}
        g.set_launch_shape(tuning["shape"])
    elif args.form == "mixed" and not args.no_autotune and not args.profile:
        from mpmc_hnu_gb300 import autotune

        tuned = autotune.tune(g, p, t, z, log=log)
        log(f"autotuned launch shape {tuned['shape']}: {tuned['ms']:.1f} ms vs default {tuned['default_ms']:.1f} ms")
        tuning = {"shape": tuned["shape"], "ms": round(tuned["ms"], 1), "default_ms": round(tuned["default_ms"], 1)}
    fields = g.fields()
    rows = flash.output_rows(n)
    dtypes = {f: d for f, d, _ in flash.OUTPUT_FIELDS}
    dp = torch.tensor(p, device="cuda")
    dt = torch.tensor(t, device="cuda")
    dz = torch.tensor(z, device="cuda")
    outs = {f: torch.empty((rows[f], ncell), device="cuda",
                           dtype=torch.int32 if dtypes[f] == np.int32 else torch.float64) for f in fields}
    ptrs = {f: v.data_ptr() for f, v in outs.items()}
    stream = torch.cuda.current_stream()

    def step():
        g.solve_device(ncell, dp.data_ptr(), dt.data_ptr(), dz.data_ptr(), ptrs, stream.cuda_stream)

    if args.profile:
        step()
        torch.cuda.synchronize()
        log("profile solve done")
        return

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with Clocks(device) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, world, "cuda")
    value = world * ncell / (ms * 1e-3)
    status = outs["status"][0].cpu().numpy()

    # end-to-end: pinned host inputs -> C ABI host entry -> every output back on the host
    hp = torch.tensor(p).pin_memory()
    ht = torch.tensor(t).pin_memory()
    hz = torch.tensor(z).pin_memory()
    houts = {f: torch.empty((rows[f], ncell), dtype=torch.int32 if dtypes[f] == np.int32 else torch.float64)
             .pin_memory() for f in fields}
    hptrs = {f: v.data_ptr() for f, v in houts.items()}
    h2d = (2 + n) * 8 * ncell
    d2h = sum(v.numel() * v.element_size() for v in houts.values())
    g.solve_host_ptrs(ncell, hp.data_ptr(), ht.data_ptr(), hz.data_ptr(), hptrs)  # warm-up
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        g.solve_host_ptrs(ncell, hp.data_ptr(), ht.data_ptr(), hz.data_ptr(), hptrs)
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps, world, "cuda")
    e2e = {"value": world * ncell / e2e_s, "unit": "flashes/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
           "host_buffers": "pinned (cudaHostAlloc through torch), one per array"}
    del houts, hp, ht, hz

    # per-stage device times and work totals (separate instrumented call) for the roofline
    gt = flash.GpuFlash(mix, args.form, sensitivity=sens, device=device, stage_timing=True,
                        sensitivity_lanes=lanes, polish_stream=pstream)
    if tuning is not None:
        gt.set_launch_shape(tuning["shape"])
    gt.solve_device(ncell, dp.data_ptr(), dt.data_ptr(), dz.data_ptr(), ptrs, stream.cuda_stream)
    stages = gt.stage_timings()
    stats = gt.batch_stats() if args.form != "plain" else {}
    counters = outs["counters"].cpu().numpy().astype(np.float64)
    sens_cells = int(((outs["sensitivity_status"][0] == 0) & (outs["status"][0] == 1)).sum().item()) if sens else 0
    gt.close()
    fp64_tf, fp32_tf = measured_peaks(flash)
    tr = {}
    tpath = os.path.join(ROOT, "profiles", "dram_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            tr = json.load(f)

    def traffic_of(stage):
        e = tr.get(f"{args.form}:{stage}:n{n}")
        return e["bytes_per_cell"] * ncell if e else None

    if args.form == "mixed":
        roofline = roofline_of(n, stages, stats, counters, sens_cells, fp64_tf, fp32_tf, ms, traffic_of)
    else:
        flops = float(counters[0].sum() + counters[1].sum() + counters[2].sum()) * f_eval(n)
        k = max(stages, key=stages.get)
        ach = flops / (stages[k] * 1e-3) / 1e12
        roofline = {"bound": "fp64", "achieved": ach, "peak": fp64_tf, "unit": "TFLOP/s", "frac": ach / fp64_tf,
                    "traffic": None, "kernel": k, "kernel_ms": stages[k], "flops_per_launch": flops}

    # the all-FP64 forms on a stratified sample, beside the mixed form on the same cells
    def sample_leg(form, size):
        sel = stratified(ncell, size)
        ns = int(sel.size)
        isel = torch.from_numpy(sel).to(dp.device)
        sub = {f: torch.empty((v.shape[0], ns), dtype=v.dtype, device=v.device) for f, v in outs.items()}
        sp = {f: v.data_ptr() for f, v in sub.items()}
        dps, dts, dzs = dp[isel].contiguous(), dt[isel].contiguous(), dz[:, isel].contiguous()
        res = {}
        for f_ in (form, "mixed"):
            gp = flash.GpuFlash(mix, f_, sensitivity=sens, device=device)
            gp.solve_device(min(ns, 4096), dps.data_ptr(), dts.data_ptr(), dzs.data_ptr(), sp, stream.cuda_stream)
            torch.cuda.synchronize()
            pms = _timed(lambda: gp.solve_device(ns, dps.data_ptr(), dts.data_ptr(), dzs.data_ptr(), sp,
                                                 stream.cuda_stream), stream, torch)
            if f_ == form:
                ps = sub["status"][0].cpu().numpy()
            gp.close()
            res[f_] = ns / (pms * 1e-3)
        return {"value": res[form], "unit": "flashes/s", "cells": ns, "mixed_same_cells": res["mixed"],
                "sample": f"{ns} stratified cells (every {ncell // ns}th) of the workload, one launch each",
                "status_agreement_with_mixed": float((ps == status[sel]).mean())}

    plain = batched = None
    if args.form == "mixed" and rank == 0:
        if args.plain_sample > 0:
            plain = sample_leg("plain", args.plain_sample)
            log(f"plain FP64 kernel: {plain['value']:.0f} flashes/s; mixed on the same cells "
                f"{plain['mixed_same_cells']:.0f}")
        if args.batched_sample > 0:
            batched = sample_leg("batched", args.batched_sample)

    # ln K warm starts (continuation use): the timed solve's own ln K, perturbed
    # by 0.1 N(0, 1) per component, on 75 % of the two-phase cells; the rest cold
    warm_leg = None
    if args.form in ("mixed", "batched") and args.warm_fraction > 0 and rank == 0:
        gen = torch.Generator(device="cuda").manual_seed(7)
        lnk = outs["ln_k"]
        two = outs["status"][0] == 1
        pick = two & (torch.rand(ncell, device="cuda", generator=gen) < args.warm_fraction)
        warm = lnk + 0.1 * torch.randn(lnk.shape, device="cuda", dtype=lnk.dtype, generator=gen)
        warm[:, ~pick] = float("nan")
        warm = warm.contiguous()
        cold_status = outs["status"][0].clone()
        gw = flash.GpuFlash(mix, args.form, sensitivity=sens, device=device, graphs=True)
        if tuning is not None:
            gw.set_launch_shape(tuning["shape"])
        wouts = {f: torch.empty_like(v) for f, v in outs.items()}
        wptrs = {f: v.data_ptr() for f, v in wouts.items()}
        call = lambda: gw.solve_device(ncell, dp.data_ptr(), dt.data_ptr(), dz.data_ptr(), wptrs,  # noqa: E731
                                       stream.cuda_stream, warm_ptr=warm.data_ptr())
        _timed(call, stream, torch)  # capture
        wms = _timed(call, stream, torch)
        wstats = gw.batch_stats()
        gw.close()
        warm_leg = {"value": ncell / (wms * 1e-3), "unit": "flashes/s", "ms": round(wms, 1),
                    "warm_cells": wstats["warm_cells"], "sent_to_cold_pass": wstats["warm_redo"],
                    "status_agreement_with_cold": float((wouts["status"][0] == cold_status).float().mean().item())}
        del wouts, warm

    # CPU baseline (the oracle on every host core) on a stratified sample, and
    # the timed solve's parity against it on the same cells
    cpu = parity = None
    if rank == 0:
        from oracle import pyoracle

        sel = stratified(ncell, args.cpu_sample)
        pyoracle.build()
        t0 = time.perf_counter()
        ref = pyoracle.flash(mix, p[sel], t[sel], z[:, sel], threads=threads, sens=sens)
        secs = time.perf_counter() - t0
        cpu = {"value": sel.size / secs, "unit": "flashes/s", "cores": threads, "kind": "port",
               "sample": f"{sel.size} stratified cells (every {ncell // sel.size}th) of this workload, flash"
                         f"{' + AD' if sens else ''}, {secs:.1f} s wall on {threads} threads"}
        isel = torch.from_numpy(sel).to(dp.device)
        gpu = {f: v[:, isel].cpu().numpy() for f, v in outs.items()}
        gpu = {f: (a[0] if a.shape[0] == 1 else a) for f, a in gpu.items()}
        parity = error_report(n, gpu, ref, sens)
        log(f"parity on {sel.size} cells: {parity['status_mismatches']} status mismatches")
    del outs
    g.close()

    legs = {}
    if rank == 0:
        # the secondary legs: a failure there is recorded in the line
        def guarded(name, fn):
            t0 = time.time()
            try:
                legs[name] = fn()
            except Exception as e:  # noqa: BLE001 - reported in the line
                legs[name] = {"error": f"{type(e).__name__}: {e}"}
            log(f"{name}: {time.time() - t0:.0f} s")

        guarded("config0", lambda: config0_leg(flash, synth, threads))
        if args.config3_cells > 0:
            guarded("config3_n10", lambda: config3_leg(flash, synth, torch, device, stream, 10, args.config3_cells,
                                                        65536, threads, log))
            guarded("config3_n20", lambda: config3_leg(flash, synth, torch, device, stream, 20, args.config3_cells,
                                                        32768, threads, log))
        if args.config2_cells > 0:
            guarded("config2", lambda: config2_leg(flash, synth, torch, device, stream, args.config2_cells, 65536,
                                                   16384, args.warm_fraction, log))
        if args.chart_cells > 0:
            peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
            hbm = json.load(open(peaks_path)).get("hbm_gbs") if os.path.exists(peaks_path) else None
            guarded("property_chart", lambda: chart_leg(flash, synth, torch, device, stream, args.chart_cells, threads,
                                                        min(args.cpu_sample, 65536), hbm, fp64_tf))
        if args.serving_seconds > 0:
            fr = [float(v) for v in args.serving_fractions.split(",") if v]
            guarded("serving", lambda: serving_probe(flash, synth, device, args.serving_seconds, fr, log))

    if rank == 0:
        line = {"metric": METRIC, "value": value,
                "unit": "flashes/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 iterations + f64 decisions/polish/AD" if args.form == "mixed" else "f64",
                "data": f"synthetic (seeded generator; {place_info.get('near_placed', 0)} of "
                        f"{place_info.get('near_target', 0)} near-boundary cells placed by GPU bisection)",
                "config": workload, "e2e": e2e, "gpu_launches": kernels_per_solve(args.form, sens) * args.steps,
                "roofline": roofline, "cpu_baseline": cpu, "clocks": clk.summary(),
                "form": args.form, "tuning": tuning, "placement": place_info, "work": stats,
                "phase_counts": {"single": int((status == 0).sum()), "two": int((status == 1).sum()),
                                 "unstable": int((status == 2).sum()), "indeterminate": int((status == 3).sum()),
                                 "invalid": int((status == -1).sum())},
                "warm_start": warm_leg, "property_chart": legs.get("property_chart"),
                "config0": legs.get("config0"), "config2": legs.get("config2"),
                "batched_fp64": batched, "plain_fp64": plain, "parity": parity,
                "config3_n10": legs.get("config3_n10"), "config3_n20": legs.get("config3_n20"),
                "serving": legs.get("serving")}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
