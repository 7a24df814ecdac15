"""Ordered-path PT continuation of many feeds at once.

The reference scans one feed along an ordered path of (p, T) states
(modules/flash/include/mpmc/flash/pr76_pt_continuation.hpp:183-306): every
point is a fresh max-3-phase solve, seeded with the previous accepted point's
phase compositions (hints reset after an unresolved point).  Between
consecutive accepted points whose phase counts differ it records a transition
bracket; the exact boundary is not resolved.

Here every path advances one point per step.  A step is one batched solve of
all paths' current points through the C ABI, warm-started with each path's
previous ln K: mpmc_gpu_flash_solve_warm, with the feed test skipped only
where the reference's own review accepts the warm pair.  The phase_set_unstable
points then get the max-3-phase continuation (mpmc_gpu_flash_solve_max3).
Hints reset after an unresolved point as in the reference.  Each point's
answer is therefore a solve whose acceptance is the reference's.  The seeding
is the warm start, not the reference's start compositions, which the C ABI
does not take.

    from mpmc_hnu_gb300 import continuation, synth
    res = continuation.solve_paths(mix, z, p_path, t_path, form="mixed")
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


def solve_paths(mixture, feeds, pressures, temperatures, form: str = "mixed", warm: bool = True,
                max3: bool = True, device: int = 0) -> dict:
    """Continuation of npath feeds z [n, npath] along their own paths
    pressures / temperatures [npath, npoint].  Returns per point the published
    status, accepted phase count, vapor fraction and ln K ([npath, npoint] and
    [n, npath, npoint]), the max3 status where the continuation ran, and the
    transition brackets."""
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
