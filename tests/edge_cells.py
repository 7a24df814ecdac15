"""Edge-case cells of the PT flash request contract (pt_split.hpp:184-188,
pt_stability.hpp:110-122, 263-285): absent components, pure feeds, invalid
requests and extreme states, for the parity tests."""

import numpy as np

from mpmc_hnu_gb300 import synth


def edge_cells(n: int, seed: int):
    """(p, t, z, kinds): a list of seeded edge cases of n components."""
    rng = np.random.default_rng(seed)
    base_p, base_t, base_z = synth.make_cells(n, 64, seed)
    cells, kinds = [], []

    def add(p, t, z, kind):
        cells.append((float(p), float(t), np.asarray(z, dtype=np.float64)))
        kinds.append(kind)

    for c in range(16):  # absent components: a random subset set to zero, renormalised
        z = base_z[:, c].copy()
        z[rng.random(n) < 0.4] = 0.0
        if not (z > 0).any():
            z[0] = 1.0
        add(base_p[c], base_t[c], z / z.sum(), "absent components")
    for c in range(min(n, 6)):  # a pure component
        z = np.zeros(n)
        z[c] = 1.0
        add(base_p[16 + c], base_t[16 + c], z, "pure feed")
    for c in range(4):  # two active components only
        z = np.zeros(n)
        i, j = rng.choice(n, 2, replace=False)
        z[i], z[j] = 0.3, 0.7
        add(base_p[24 + c], base_t[24 + c], z, "binary subset")
    z0 = base_z[:, 30].copy()
    for p, t, kind in ((0.0, 300.0, "p = 0"), (-1e6, 300.0, "p < 0"), (np.nan, 300.0, "p NaN"),
                       (1e6, 0.0, "T = 0"), (1e6, np.inf, "T inf"), (1e6, np.nan, "T NaN")):
        add(p, t, z0, kind)
    z = z0.copy()
    z[0] = -1e-3
    add(1e6, 300.0, z, "negative fraction")
    add(1e6, 300.0, z0 * 1.01, "feed sum 1.01")
    add(1e6, 300.0, z0 * (1.0 + 1e-15), "feed sum within 64 eps")
    z = z0.copy()
    z[0] = 1.5
    add(1e6, 300.0, z, "fraction above one")
    for c, p in enumerate((1e3, 1e4, 5e7, 1e8)):  # extreme pressures
        add(p, base_t[40 + c], base_z[:, 40 + c], "extreme pressure")
    for c, t in enumerate((150.0, 900.0)):  # extreme temperatures
        add(base_p[44 + c], t, base_z[:, 44 + c], "extreme temperature")
    p = np.array([c[0] for c in cells])
    t = np.array([c[1] for c in cells])
    z = np.ascontiguousarray(np.array([c[2] for c in cells]).T)
    return p, t, z, kinds
