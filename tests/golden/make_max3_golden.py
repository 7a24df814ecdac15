"""Record the reference's max-3-phase orchestration on fixture cells.

Runs only where the MPMC_HNU reference sources were present to build
oracle/_ref/libpr76_ref.so (`make -C oracle ref`).  Writes
tests/golden/max3_reference.npz: the inputs and the outputs of
solve_pr76_pt_max3 (modules/flash/include/mpmc/flash/pr76_three_phase.hpp:328)
with the PR76 backend's default options, through the harness's
ref_max3_batch, on cells of the three-phase fixture mixture of the
reference's own tests (tests/flash/pr76_three_phase/synthetic_fixture.hpp):
a quarter at the fixture's anchor state (1 MPa, 250 K, feeds inside the tie
triangle), the rest spread over p in [0.2, 5] MPa and T in [200, 300] K;
feeds on and near the triangle's edges; and the cells of a wide scan whose
three-phase candidate failed its final review, with a sample of the others.
Also writes tests/golden/continuation_reference.npz: the reference's
ordered-path continuation (solve_pr76_pt_continuation, default options) of
96 fixture feeds along p = 0.2 .. 5 MPa at 250 K, with the fresh (cold)
max3 status of every point beside it.
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from mpmc_hnu_gb300 import synth  # noqa: E402
from oracle import pyoracle  # noqa: E402


def main() -> None:
    pyoracle.build()
    if not pyoracle.reference_available():
        raise SystemExit("reference harness not built (make -C oracle ref)")
    mix = synth.three_phase_fixture_mixture()
    p, t, z = synth.make_three_phase_cells(1200, seed=11)
    # feeds on and near the edges of the anchor tie triangle (a phase fraction
    # at or close to zero)
    rng = np.random.default_rng(3)
    anchor = synth.THREE_PHASE_ANCHOR
    edge = []
    for a, b in ((0, 1), (0, 2), (1, 2)):
        c = 3 - a - b
        for beta in rng.uniform(0.02, 0.98, 20):
            for eps in (0.0, 1e-6, 1e-3, -1e-3):
                f = (1 - beta) * anchor[a] + beta * anchor[b] + eps * (anchor[c] - 0.5 * (anchor[a] + anchor[b]))
                edge.append(f / f.sum())
    ze = np.array(edge).T
    # a wide scan (p 0.05-20 MPa, T 150-350 K), keeping every cell whose
    # three-phase candidate failed its final review plus a sample of the rest
    rng = np.random.default_rng(5)
    nw = 40000
    zw = rng.dirichlet(np.ones(3) * 0.5, nw).T
    tw = rng.uniform(150.0, 350.0, nw)
    pw = np.exp(rng.uniform(np.log(5e4), np.log(2e7), nw))
    scan = pyoracle.reference_max3(mix, pw, tw, zw, threads=16)
    keep = np.nonzero(scan["max3_status"] == 4)[0]
    keep = np.concatenate([keep, np.arange(0, nw, 200)])
    p = np.concatenate([p, np.full(ze.shape[1], 1e6), pw[keep]])
    t = np.concatenate([t, np.full(ze.shape[1], 250.0), tw[keep]])
    z = np.ascontiguousarray(np.concatenate([z, ze, zw[:, keep]], axis=1))
    ref = pyoracle.reference_max3(mix, p, t, z, threads=16)
    np.savez_compressed(os.path.join(HERE, "max3_reference.npz"), p=p, t=t, z=z,
                        **{f"ref_{k}": v for k, v in ref.items()})
    counts = np.bincount(ref["max3_status"] + 1, minlength=7)
    print("max3 status counts (invalid, single, two, three, boundary, higher, indeterminate):", counts)
    # the reference's ordered-path continuation (pr76_pt_continuation.hpp:183-306,
    # default options) of 96 fixture feeds along p = 0.2 .. 5 MPa at 250 K
    _, _, zc = synth.make_three_phase_cells(96, seed=51, anchor_fraction=0.5)
    pc = np.tile(np.exp(np.linspace(np.log(2e5), np.log(5e6), 10)), (96, 1))
    tc = np.full_like(pc, 250.0)
    ms, pub = pyoracle.reference_continuation(mix, pc, tc, zc, threads=16)
    cold = np.stack([pyoracle.reference_max3(mix, np.ascontiguousarray(pc[:, k]), np.ascontiguousarray(tc[:, k]),
                                             zc, threads=16)["max3_status"] for k in range(pc.shape[1])], axis=1)
    np.savez_compressed(os.path.join(HERE, "continuation_reference.npz"), p=pc, t=tc, z=zc, ref_max3_status=ms,
                        ref_published=pub, ref_cold_max3_status=cold)
    print("continuation: points whose hint-seeded status differs from a fresh solve:", int((ms != cold).sum()))


if __name__ == "__main__":
    main()
