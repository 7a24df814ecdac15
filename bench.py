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
    `status_fn(p, t, z) -> status`; returns (p of the placed cells, mask).
    The +-2 % placement noise is drawn at the cells' global indices."""
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
    return np.exp(0.5 * (lo + hi)) * (1.0 + 0.04 * (u - 0.5)), ok


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
    """Seeded cells; the near-saturation subset is placed by GPU bisection."""
    mix, offset, p, t, z, n_near = base_cells(n, ncell, near_fraction, rank, synth)
    if n_near == 0:
        return mix, p, t, z, 0
    cache_dir = os.path.join(os.path.expanduser("~"), ".cache", "mpmc_gb300")
    key = f"near2_n{n}_c{ncell}_f{near_fraction}_r{rank}_m{MIXTURE_SEED}_s{CELL_SEED}.npz"
    path = os.path.join(cache_dir, key)
    if os.path.exists(path):
        d = np.load(path)
        return mix, d["p"], d["t"], d["z"], int(d["placed"])
    t0 = time.time()
    g = flash.GpuFlash(mix, "mixed")
    idx = np.arange(n_near)
    pb, placed = place_near(t, z, idx, offset + idx,
                            lambda a, b, c: g.solve(a, b, c, fields=["status"])["status"])
    g.close()
    p = p.copy()
    p[idx[placed]] = pb[placed]
    log(f"near-saturation placement: {int(placed.sum())}/{n_near} cells bracketed "
        f"({time.time() - t0:.1f} s); the rest keep log-uniform p")
    os.makedirs(cache_dir, exist_ok=True)
    np.savez(path, p=p, t=t, z=z, placed=int(placed.sum()))
    return mix, p, t, z, int(placed.sum())


def cpu_workload_sample(n: int, ncell: int, near_fraction: float, sample: int, threads: int, synth):
    """The stratified sample of the workload placed by the CPU oracle alone
    (same grid, bisection and noise as the GPU placement)."""
    from oracle import pyoracle

    mix, offset, p, t, z, n_near = base_cells(n, ncell, near_fraction, 0, synth)
    idx = stratified(ncell, sample)
    p, t, z = p[idx].copy(), t[idx], z[:, idx]
    near = np.nonzero(idx < n_near)[0]
    if near.size:
        pb, placed = place_near(t, z, near, offset + idx[near],
                                lambda a, b, c: pyoracle.flash(mix, a, b, c, threads=threads)["status"])
        p[near[placed]] = pb[placed]
    return mix, p, t, z


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
# multi-mixture warm-start workload: 4 mixtures x cells at N = 4, 8, 12, 20
CONFIG2_COMPONENTS = (4, 8, 12, 20)


def multi_mixture_leg(flash, synth, torch, device: int, stream, ncell: int, form: str, warm_fraction: float):
    """Per mixture (N = 4, 8, 12, 20; seeds 1104.., cells of the bench
    generator): a cold solve gives each two-phase cell its converged ln K*;
    then `warm_fraction` of ALL cells get ln K* + 0.1 N(0, 1) where they have
    one (the rest start cold, Wilson K) and that warm solve is timed with CUDA
    events on the launching stream, after one untimed warm-up of the same
    call.  Flash without sensitivities.  Returns per-mixture and whole-job
    flashes/s."""
    rows_of = flash.output_rows
    per, total_ms, total_cells = {}, 0.0, 0
    dev = torch.device(f"cuda:{device}")
    for n in CONFIG2_COMPONENTS:
        mix = synth.make_mixture(n, 1100 + n)
        p, t, z = synth.make_cells(n, ncell, 2100 + n)
        dp, dt, dz = (torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (p, t, z))
        rows = rows_of(n)
        fields = ["status", "vapor_fraction", "liquid", "vapor", "ln_k", "z_liquid", "z_vapor"]
        outs = {f: torch.empty((rows[f], ncell), dtype=torch.int32 if f == "status" else torch.float64, device=dev)
                for f in fields}
        ptrs = {f: v.data_ptr() for f, v in outs.items()}
        g = flash.GpuFlash(mix, form, sensitivity=False, device=device)
        stream.wait_stream(torch.cuda.current_stream(dev))
        g.solve_device(ncell, dp.data_ptr(), dt.data_ptr(), dz.data_ptr(), ptrs, stream.cuda_stream)
        torch.cuda.synchronize()
        gen = torch.Generator(device=dev).manual_seed(17 + n)
        two = outs["status"][0] == 1
        pick = two & (torch.rand(ncell, device=dev, generator=gen) < warm_fraction)
        warm = outs["ln_k"] + 0.1 * torch.randn(outs["ln_k"].shape, device=dev, dtype=torch.float64, generator=gen)
        warm[:, ~pick] = float("nan")
        warm = warm.contiguous()
        cold_status = outs["status"][0].clone()
        times = []
        for _ in range(2):  # warm-up, then the timed call
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            g.solve_device(ncell, dp.data_ptr(), dt.data_ptr(), dz.data_ptr(), ptrs, stream.cuda_stream,
                           warm_ptr=warm.data_ptr())
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        g.close()
        ms = times[-1]
        per[f"n{n}"] = {"value": ncell / (ms * 1e-3), "unit": "flashes/s", "ms": ms,
                        "warm_cells": int(pick.sum().item()), "two_phase_cells": int(two.sum().item()),
                        "status_agreement_with_cold": float((outs["status"][0] == cold_status).float().mean().item())}
        total_ms += ms
        total_cells += ncell
        del outs, warm, dp, dt, dz
    return {"value": total_cells / (total_ms * 1e-3), "unit": "flashes/s", "cells": total_cells, "form": form,
            "per_mixture": per,
            "setup": f"4 mixtures x {ncell} cells (N = 4, 8, 12, 20), ln K* of a cold solve + 0.1 N(0,1) on "
                     f"{warm_fraction:.0%} of all cells where a pair converged, the rest cold; no sensitivities"}


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
    del dq, vals, jac
    if cpu_sample > 0:
        from oracle import pyoracle

        sel = q[:, :: max(1, ncell // cpu_sample)][:, :cpu_sample]
        sel = np.ascontiguousarray(sel)
        pyoracle.build()
        t0 = time.perf_counter()
        pyoracle.property_chart(mix, phases, [0, 0], spec.molar_mass, visc, enth, sel, None, threads=threads)
        dt = time.perf_counter() - t0
        leg["cpu_baseline"] = {"value": sel.shape[1] / dt, "unit": "cells/s", "cores": threads, "kind": "port",
                               "sample": f"{sel.shape[1]} of the same cells (every {ncell // sel.shape[1]}th), "
                                         f"{dt:.1f} s wall; the oracle is bit-identical to the reference's chart"}
    return leg


# ---------------------------------------------------------------------------
# ---------------------------------------------------------------------------
# serving (continuous batching through the flash server)
SERVING_MIXTURES = [(3, 501), (3, 502), (6, 503), (6, 504), (10, 505), (10, 506), (20, 507), (20, 508)]


def serving_pool(synth, count: int, seed: int = 77):
    """Seeded requests: mixture among 8 (N in {3, 6, 10, 20}), cells per request
    floor(exp(U ln 65536)), cells from the base distributions; half re-query
    the previous request's mixture with p * exp(N(0, 0.02)), T + N(0, 1 K)."""
    rng = np.random.default_rng(seed)
    pool = []
    for k in range(count):
        ncell = max(1, int(np.exp(rng.uniform(0.0, np.log(65536.0)))))
        if pool and rng.uniform() < 0.5:
            j, p0, t0, z0 = pool[-1]
            n = SERVING_MIXTURES[j][0]
            src = rng.integers(0, p0.shape[0], ncell)
            p = p0[src] * np.exp(rng.normal(0.0, 0.02, ncell))
            t = t0[src] + rng.normal(0.0, 1.0, ncell)
            z = np.ascontiguousarray(z0[:, src])
        else:
            j = int(rng.integers(0, len(SERVING_MIXTURES)))
            n = SERVING_MIXTURES[j][0]
            p, t, z = synth.make_cells(n, ncell, 9000 + k)
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


def serving_probe(flash, synth, device, seconds, fractions, log):
    """Saturated throughput, then open-loop Poisson load at each fraction of it."""
    slots = 16
    server = flash.FlashServer(device=device, slots=slots, max_batch_cells=65536, memory_budget_bytes=40 << 30)
    ids = [server.add_mixture(synth.make_mixture(n, s)) for n, s in SERVING_MIXTURES]
    pool = serving_pool(synth, 256)
    serving_run(server, ids, pool[:16], None, 0)  # warm-up
    done, wall = serving_closed(server, ids, pool, 2 * slots, seconds)
    sat = serving_summary(done, wall)
    sat_req = len(done) / wall
    log(f"serving: saturated {sat['flashes_per_s']:.0f} flashes/s, {sat_req:.1f} requests/s "
        f"({2 * slots} requests outstanding)")
    rates = []
    for f in fractions:
        d, w = serving_run(server, ids, pool, f * sat_req, seconds)
        r = serving_summary(d, w, f * sat_req)
        r["fraction_of_saturation"] = f
        rates.append(r)
        log(f"serving at {f:.0%}: {r}")
    st = server.stats()
    server.close()
    return {"saturated_flashes_per_s": sat["flashes_per_s"], "saturated_req_per_s": sat_req,
            "saturation": f"closed loop, {2 * slots} requests outstanding", "saturated_latency": sat,
            "rates": rates, "slots": st.get("slots"), "max_batch_cells": 65536,
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
    ap.add_argument("--plain-sample", type=int, default=32768)
    ap.add_argument("--batched-sample", type=int, default=131072)
    ap.add_argument("--warm-fraction", type=float, default=0.75,
                    help="share of the two-phase cells given a ln K warm start in the warm-start leg (0 = skip)")
    ap.add_argument("--cpu-sample", type=int, default=65536)
    ap.add_argument("--profile", action="store_true", help="one untimed solve of the workload (for ncu)")
    ap.add_argument("--serving-seconds", type=float, default=8.0,
                    help="open-loop serving probe at 70%% of saturation (0 = skip)")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shape")
    ap.add_argument("--launch-shape", default="",
                    help="comma-separated mixed-form launch shape to use instead of autotuning")
    ap.add_argument("--multi-mixture-cells", type=int, default=1 << 20,
                    help="cells per mixture of the 4-mixture warm-start leg (0 = skip)")
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

    workload = {"workload": f"PR76 two-phase PT flash + implicit AD, Nc={args.n}, {args.cells} cells per GPU, "
                            f"{int(args.near_fraction * 100)}% within 2% of the phase-boundary pressure",
                "cells_per_gpu": args.cells, "components": args.n, "sensitivity": sens,
                "form": args.form, "l2_flush": "inputs+outputs larger than L2", "parallelism": f"replicas{world}"}

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
                  f"near-boundary cells placed by the same bisection with the CPU flash; flash"
                  f"{' + AD' if sens else ''}")
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "flashes/s",
                "n_gpus": 0, "steps": args.steps, "warmup": args.warmup, "ms_per_step": p.shape[0] / v * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded generator, stratified sample)",
                "config": {**workload, "cells_per_step": int(p.shape[0])},
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

    mix, p, t, z, placed = make_workload(args.n, args.cells, args.near_fraction, rank, torch, flash, synth, log)
    n, ncell = args.n, args.cells
    # the timed handle replays its launch sequence as a CUDA graph (same cells
    # and buffers every step)
    g = flash.GpuFlash(mix, args.form, sensitivity=sens, device=device, graphs=True)
    tuned = None
    if args.form == "mixed" and args.launch_shape:
        tuned = {"shape": [int(v) for v in args.launch_shape.split(",")], "ms": float("nan"),
                 "default_ms": float("nan")}
        g.set_launch_shape(tuned["shape"])
        workload = {**workload, "launch_shape": tuned["shape"]}
    elif args.form == "mixed" and not args.no_autotune and not args.profile:
        from mpmc_hnu_gb300 import autotune

        tuned = autotune.tune(g, p, t, z, log=log)
        log(f"autotuned launch shape {tuned['shape']}: {tuned['ms']:.1f} ms vs default {tuned['default_ms']:.1f} ms")
        workload = {**workload, "launch_shape": tuned["shape"], "autotune_ms": round(tuned["ms"], 1),
                    "default_shape_ms": round(tuned["default_ms"], 1)}
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
    counters = outs["counters"].cpu().numpy().astype(np.float64)

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

    # per-stage device times (separate instrumented pass) for the roofline
    gt = flash.GpuFlash(mix, args.form, sensitivity=sens, device=device, stage_timing=True)
    if tuned is not None:
        gt.set_launch_shape(tuned["shape"])
    gt.solve_device(ncell, dp.data_ptr(), dt.data_ptr(), dz.data_ptr(), ptrs, stream.cuda_stream)
    stages = gt.stage_timings()
    counters_t = outs["counters"].cpu().numpy().astype(np.float64)
    gt.close()

    # the all-FP64 forms on bounded samples of the same cells
    def sample_leg(form, size):
        sel = stratified(ncell, size)
        ns = int(sel.size)
        isel = torch.from_numpy(sel).to(dp.device)
        gp = flash.GpuFlash(mix, form, sensitivity=sens, device=device)
        sub = {f: torch.empty((v.shape[0], ns), dtype=v.dtype, device=v.device) for f, v in outs.items()}
        sp = {f: v.data_ptr() for f, v in sub.items()}
        dps, dts, dzs = dp[isel].contiguous(), dt[isel].contiguous(), dz[:, isel].contiguous()
        gp.solve_device(min(ns, 4096), dps.data_ptr(), dts.data_ptr(), dzs.data_ptr(), sp, stream.cuda_stream)
        torch.cuda.synchronize()
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        gp.solve_device(ns, dps.data_ptr(), dts.data_ptr(), dzs.data_ptr(), sp, stream.cuda_stream)
        a1.record(stream)
        torch.cuda.synchronize()
        pms = a0.elapsed_time(a1)
        ps = sub["status"][0].cpu().numpy()
        gp.close()
        return {"value": ns / (pms * 1e-3), "unit": "flashes/s", "cells": ns,
                "sample": f"{ns} stratified cells (every {ncell // ns}th) of the workload, one launch",
                "status_agreement_with_chosen": float((ps == status[sel]).mean())}

    plain = batched = None
    if args.form == "mixed" and rank == 0:
        if args.plain_sample > 0:
            plain = sample_leg("plain", args.plain_sample)
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
        if tuned is not None:
            gw.set_launch_shape(tuned["shape"])
        wouts = {f: torch.empty_like(v) for f, v in outs.items()}
        wptrs = {f: v.data_ptr() for f, v in wouts.items()}
        wtimes = []
        for k in range(2):  # capture, then replay
            w0 = torch.cuda.Event(enable_timing=True)
            w1 = torch.cuda.Event(enable_timing=True)
            w0.record(stream)
            gw.solve_device(ncell, dp.data_ptr(), dt.data_ptr(), dz.data_ptr(), wptrs, stream.cuda_stream,
                            warm_ptr=warm.data_ptr())
            w1.record(stream)
            torch.cuda.synchronize()
            wtimes.append(w0.elapsed_time(w1))
        stats = gw.batch_stats()
        gw.close()
        wms = wtimes[-1]
        warm_leg = {"value": ncell / (wms * 1e-3), "unit": "flashes/s", "ms": wms, "cold_ms": ms,
                    "warm_cells": stats["warm_cells"], "sent_to_cold_pass": stats["warm_redo"],
                    "status_agreement_with_cold": float((wouts["status"][0] == cold_status).float().mean().item()),
                    "setup": f"ln K of the timed solve + 0.1 N(0,1) on {args.warm_fraction:.0%} of the two-phase "
                             "cells, the rest cold; same cells and handle settings, one replayed graph"}
        del wouts, warm

    fp64_tf, fp32_tf = measured_peaks(flash)
    # roofline of the dominant stage: FP32 screening kernels on the FP32 pipe
    ev32 = counters_t[0] + counters_t[1] + counters_t[2]
    ev64 = counters_t[5]
    fe = f_eval(n)
    if args.form in ("mixed", "batched"):
        dominant = max((k for k in stages if k != "sensitivity"), key=lambda k: stages[k])
        fp32_stage = {"feed_trials": counters_t[0], "split": counters_t[1], "review_trials": counters_t[2]}
        if dominant in fp32_stage:
            flops = float(fp32_stage[dominant].sum()) * (fe + (6 * n if dominant == "split" else 0))
            bound, peak = "fp32", fp32_tf
        else:
            flops = float(ev64.sum()) * fe
            bound, peak = "fp64", fp64_tf
    else:
        dominant = "flash"
        flops = float(ev32.sum()) * fe + float(counters_t[4].sum()) * 6 * n + float(counters_t[5].sum()) * 8
        bound, peak = "fp64", fp64_tf
    dom_ms = stages.get(dominant, ms)
    achieved = flops / (dom_ms * 1e-3) / 1e12
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "dram_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            tr = json.load(f)
        key = f"{args.form}:{dominant}:n{n}"
        if key in tr:
            traffic = tr[key]["bytes_per_cell"] * ncell
    roofline = {"bound": bound, "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": dominant, "kernel_ms": dom_ms,
                "peak_source": "measured in this run by mpmc_hnu_gb300/csrc/peak_probe.cu (FMA chains)",
                "flops_per_launch": flops, "stage_ms": stages,
                "fp64_evals_per_cell": float(ev64.mean()), "fp32_evals_per_cell": float(ev32.mean())}

    cpu = None
    if rank == 0:
        sel = stratified(ncell, args.cpu_sample)
        rate, secs = cpu_flash_rate(mix, p[sel], t[sel], z[:, sel], threads, sens)
        cpu = {"value": rate, "unit": "flashes/s", "cores": threads, "kind": "port",
               "sample": f"{sel.size} stratified cells (every {ncell // sel.size}th) of this workload, flash"
                         f"{' + AD' if sens else ''}, {secs:.1f} s wall on {threads} threads"}

    serving = None
    if rank == 0 and args.serving_seconds > 0:
        g.close()
        serving = serving_probe(flash, synth, device, args.serving_seconds, [0.7], log)

    # the secondary legs run last: a failure there leaves the flash line intact
    multi = None
    if rank == 0 and args.multi_mixture_cells > 0 and args.form in ("mixed", "batched"):
        try:
            multi = multi_mixture_leg(flash, synth, torch, device, stream, args.multi_mixture_cells, args.form,
                                      args.warm_fraction)
        except Exception as e:  # noqa: BLE001 - reported in the line
            multi = {"error": f"{type(e).__name__}: {e}"}
    chart = None
    if rank == 0 and args.chart_cells > 0:
        try:
            peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
            hbm = json.load(open(peaks_path)).get("hbm_gbs") if os.path.exists(peaks_path) else None
            chart = chart_leg(flash, synth, torch, device, stream, args.chart_cells, threads,
                              min(args.cpu_sample, 65536), hbm, fp64_tf)
        except Exception as e:  # noqa: BLE001 - reported in the line
            chart = {"error": f"{type(e).__name__}: {e}"}

    if rank == 0:
        line = {"metric": METRIC, "value": value,
                "unit": "flashes/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 iterations + f64 decisions/polish/AD" if args.form == "mixed" else "f64",
                "data": f"synthetic (seeded generator; {placed} near-boundary cells placed by GPU bisection)",
                "config": workload, "e2e": e2e, "gpu_launches": len(stages) * args.steps,
                "roofline": roofline, "cpu_baseline": cpu, "plain_fp64": plain, "batched_fp64": batched,
                "warm_start": warm_leg, "multi_mixture_warm": multi, "property_chart": chart,
                "phase_counts": {"single": int((status == 0).sum()), "two": int((status == 1).sum()),
                                 "unstable": int((status == 2).sum()), "indeterminate": int((status == 3).sum()),
                                 "invalid": int((status == -1).sum())},
                "clocks": clk.summary(), "serving": serving}
        print(json.dumps(line), flush=True)
    g.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
