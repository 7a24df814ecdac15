"""Ordered-path PT continuation of many feeds at once.

The reference scans one feed along an ordered path of (p, T) states
(modules/flash/include/mpmc/flash/pr76_pt_continuation.hpp:183-306): every
point is a fresh max-3-phase solve, seeded with the previous accepted point's
phase compositions (hints reset after an unresolved point).  Between
consecutive accepted points whose phase counts differ it records a transition
bracket; the exact boundary is not resolved.

Here every path advances one point per step; a step is one batched solve of
all paths' current points through the C ABI.  Two seedings:

* `solve_paths(..., hints=True)` carries the reference's own hints
  (pr76_pt_continuation.hpp:216-300): the previous accepted point's phase
  compositions as extra starts of the feed test and the final review, and its
  three-phase set as a three-phase start, through
  mpmc_gpu_flash_solve_hinted (the reference algorithm in FP64, then the
  max-3-phase continuation).  This is the reference's scan point for point.
* `solve_paths(..., hints=False)` warm-starts each point from the previous
  ln K (mpmc_gpu_flash_solve_warm, the fast forms), then runs the
  max-3-phase continuation on the phase_set_unstable points
  (mpmc_gpu_flash_solve_max3).  Each point equals a fresh solve.

Hints reset after an unresolved point in both, as in the reference.

    from mpmc_hnu_gb300 import continuation, synth
    res = continuation.solve_paths(mix, z, p_path, t_path, hints=True)
    res["phase_count"]      # [npath, npoint]: 1, 2, 3 or 0 (unresolved)
    res["brackets"]         # list of (path, left, right, left_count, right_count, adjacent)
"""

from __future__ import annotations

import numpy as np

from . import flash


def phase_counts(status: np.ndarray) -> np.ndarray:
    """Accepted phase count per published status (pr76_pt_continuation.hpp:77-90):
    single 1, two 2, three 3; unstable, indeterminate and invalid 0."""
    s = np.asarray(status)
    return np.where(s == 0, 1, np.where(s == 1, 2, np.where(s == 4, 3, 0))).astype(np.int32)


def transition_brackets(counts: np.ndarray) -> list[tuple[int, int, int, int, int, bool]]:
    """Brackets between consecutive accepted points with different phase
    counts (pr76_pt_continuation.hpp:263-290): (path, left index, right index,
    left count, right count, adjacent count step).  `counts` is [npath, npoint]
    with 0 for unresolved points, which bracket nothing."""
    c = np.asarray(counts)
    out = []
    for path in range(c.shape[0]):
        for k in range(1, c.shape[1]):
            a, b = int(c[path, k - 1]), int(c[path, k])
            if a and b and a != b:
                out.append((path, k - 1, k, a, b, abs(a - b) == 1))
    return out


def normalise_feeds(z: np.ndarray) -> np.ndarray:
    """z / sum(z) per column with the reference's compensated sum
    (stability_check_composition, pt_stability.hpp:110-122), component by
    component in order, so the normalised feeds round as the reference's do."""
    z = np.asarray(z, dtype=np.float64)
    total = np.zeros(z.shape[1])
    carry = np.zeros(z.shape[1])
    for i in range(z.shape[0]):
        inc = z[i] - carry
        nxt = total + inc
        carry = (nxt - total) - inc
        total = nxt
    return np.ascontiguousarray(z / total)


def scan_with_hints(step, feeds, pressures, temperatures) -> dict:
    """The reference's hint-seeded ordered-path scan (pr76_pt_continuation.hpp:
    183-306, default options) over all paths at once.  `step(p, t, z, count,
    x, three, fraction)` solves one point of every path with its hints (the
    mpmc_start_hints arrays) and returns published [npath], max3 [npath],
    x, y [n, npath] (the published pair, or the feed for one phase),
    x3 [3 n, npath] and f3 [3, npath] (the three-phase set).  The feeds are
    normalised once, as the reference does before the scan."""
    z = normalise_feeds(feeds)
    p = np.asarray(pressures, dtype=np.float64)
    t = np.asarray(temperatures, dtype=np.float64)
    n, npath = z.shape
    npoint = p.shape[1]
    count = np.zeros(npath, np.int32)
    hx = np.zeros((3 * n, npath))
    three = np.zeros(npath, np.int32)
    frac = np.zeros((2, npath))
    published = np.empty((npath, npoint), np.int32)
    max3_status = np.empty((npath, npoint), np.int32)
    for k in range(npoint):
        out = step(np.ascontiguousarray(p[:, k]), np.ascontiguousarray(t[:, k]), z, count, hx, three, frac)
        m3 = np.asarray(out["max3"])
        published[:, k] = out["published"]
        max3_status[:, k] = m3
        # the next point's hints: the accepted phases (:262-300); an
        # unresolved point resets them
        count = np.zeros(npath, np.int32)
        hx = np.zeros((3 * n, npath))
        three = np.zeros(npath, np.int32)
        frac = np.zeros((2, npath))
        single = m3 == 0
        count[single] = 1
        hx[:n, single] = out["x"][:, single]
        two = (m3 == 1) & np.isfinite(out["x"][0]) & np.isfinite(out["y"][0])
        hx[:n, two] = out["x"][:, two]
        hx[n:2 * n, two] = out["y"][:, two]
        # unique starts only (pr76_pt_continuation_append_unique, :103-118)
        count[two] = np.where((out["x"][:, two] == out["y"][:, two]).all(axis=0), 1, 2)
        tri = m3 == 2
        count[tri] = 3
        hx[:, tri] = out["x3"][:, tri]
        three[tri] = 1
        frac[:, tri] = out["f3"][1:3, tri]
    counts = phase_counts(published)
    return {"status": published, "max3_status": max3_status, "phase_count": counts,
            "brackets": transition_brackets(counts), "all_points_accepted": bool((counts > 0).all())}


def solve_paths(mixture, feeds, pressures, temperatures, form: str = "mixed", warm: bool = True,
                max3: bool = True, device: int = 0, hints: bool = False) -> dict:
    """Continuation of npath feeds z [n, npath] along their own paths
    pressures / temperatures [npath, npoint].  Returns per point the published
    status, accepted phase count, vapor fraction and ln K ([npath, npoint] and
    [n, npath, npoint]), the max3 status where the continuation ran, and the
    transition brackets.  With hints=True the scan is the reference's
    hint-seeded one (`scan_with_hints` through mpmc_gpu_flash_solve_hinted;
    `form`, `warm` and `max3` do not apply) and returns its statuses and
    brackets."""
    if hints:
        g = flash.GpuFlash(mixture, form="plain", device=device)
        try:
            def step(pk, tk, zk, count, hx, three, frac):
                out, out3 = g.solve_hinted(pk, tk, zk, count, hx, three, frac)
                return {"published": out["status"], "max3": out3["max3_status"], "x": out["liquid"],
                        "y": out["vapor"], "x3": out3["composition"], "f3": out3["phase_fraction"]}
            return scan_with_hints(step, feeds, pressures, temperatures)
        finally:
            g.close()
    z = np.ascontiguousarray(feeds, dtype=np.float64)
    p = np.asarray(pressures, dtype=np.float64)
    t = np.asarray(temperatures, dtype=np.float64)
    n, npath = z.shape
    if p.shape != t.shape or p.shape[0] != npath:
        raise ValueError("expected pressures and temperatures of shape [npath, npoint]")
    npoint = p.shape[1]
    g = flash.GpuFlash(mixture, form=form, device=device)
    status = np.empty((npath, npoint), np.int32)
    beta = np.full((npath, npoint), np.nan)
    ln_k = np.full((n, npath, npoint), np.nan)
    max3_status = np.full((npath, npoint), -2, np.int32)  # -2: not run (the point was not unstable)
    fields = ["status", "vapor_fraction", "liquid", "vapor", "ln_k", "ln_phi_liquid", "ln_phi_vapor",
              "z_liquid", "z_vapor"]
    guess = None
    try:
        for k in range(npoint):
            pk = np.ascontiguousarray(p[:, k])
            tk = np.ascontiguousarray(t[:, k])
            out = g.solve(pk, tk, z, fields=fields, ln_k_warm=guess if warm else None)
            st = out["status"].copy()
            unstable = np.nonzero(st == 2)[0]
            if max3 and unstable.size:
                sub_out, sub3 = g.solve_max3(pk[unstable], tk[unstable], np.ascontiguousarray(z[:, unstable]),
                                             fields=fields)
                st[unstable] = sub_out["status"]
                max3_status[unstable, k] = sub3["max3_status"]
                for f in ("vapor_fraction", "ln_k"):
                    out[f][..., unstable] = sub_out[f]
            status[:, k] = st
            beta[:, k] = out["vapor_fraction"]
            ln_k[:, :, k] = out["ln_k"]
            # the next point starts from this point's accepted two-phase pairs;
            # every other path is solved cold (hints reset, :291-300)
            guess = np.where((st == 1)[None, :], out["ln_k"], np.nan)
    finally:
        g.close()
    counts = phase_counts(status)
    return {"status": status, "phase_count": counts, "vapor_fraction": beta, "ln_k": ln_k,
            "max3_status": max3_status, "brackets": transition_brackets(counts),
            "all_points_accepted": bool((counts > 0).all())}
