"""Seeded synthetic PR76 mixtures and cell states.

Counter-based SplitMix64 streams with uniform = (u64 >> 11) * 2**-53, so every
value is a pure function of (seed, stream, index) and is identical on every
host.  Distributions follow the benchmark workloads of the PR76 PT flash:

* mixture: Tc ~ U[190, 620] K, Pc ~ U[2.5, 4.6] MPa, omega ~ U[0.01, 0.35],
  symmetric kij ~ U[0, 0.12] with a zero diagonal, no volume shift;
* cell: z ~ Dirichlet(1) (normalised Exp(1)), T ~ U[280, 450] K,
  p log-uniform on [0.5, 40] MPa.

Layouts are component-major with the cell index fastest (z[i, c]), which is
the structure-of-arrays layout the device kernels read.
"""

from __future__ import annotations

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)

# stream identifiers
S_TC, S_PC, S_OMEGA, S_KIJ = 1, 2, 3, 4
S_Z, S_T, S_P, S_PICK, S_NEAR = 11, 12, 13, 14, 15
S_CRIT_PICK, S_CRIT_T, S_CRIT_P = 16, 17, 18


def _mix(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = x + _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, stream: int, index) -> np.ndarray:
    """U[0,1) doubles for counter positions `index` of (seed, stream)."""
    idx = np.asarray(index, dtype=np.uint64)
    with np.errstate(over="ignore"):
        key = _mix(np.uint64(seed) * np.uint64(0x100000001B3) + np.uint64(stream))
        u = _mix(key ^ _mix(idx + np.uint64(stream) * _GOLDEN))
    return (u >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


class Mixture:
    """PR76 parameters of one mixture, in component order."""

    def __init__(self, tc, pc, omega, kij):
        self.tc = np.ascontiguousarray(tc, dtype=np.float64)
        self.pc = np.ascontiguousarray(pc, dtype=np.float64)
        self.omega = np.ascontiguousarray(omega, dtype=np.float64)
        self.kij = np.ascontiguousarray(kij, dtype=np.float64).reshape(len(self.tc), len(self.tc))
        self.n = len(self.tc)

    def as_tuple(self):
        return self.tc, self.pc, self.omega, self.kij


def make_mixture(n: int, seed: int) -> Mixture:
    i = np.arange(n)
    tc = 190.0 + 430.0 * uniform(seed, S_TC, i)
    pc = (2.5 + 2.1 * uniform(seed, S_PC, i)) * 1e6
    omega = 0.01 + 0.34 * uniform(seed, S_OMEGA, i)
    kij = np.zeros((n, n))
    for a in range(n):
        for b in range(a + 1, n):
            kij[a, b] = kij[b, a] = 0.12 * uniform(seed, S_KIJ, a * n + b)[()]
    return Mixture(tc, pc, omega, kij)


def make_cells(n: int, ncell: int, seed: int, offset: int = 0):
    """(p [Pa], T [K], z [n, ncell]) for cells offset .. offset+ncell-1."""
    return make_cells_at(n, np.arange(offset, offset + ncell, dtype=np.uint64), seed)


def make_cells_at(n: int, index, seed: int):
    """(p [Pa], T [K], z [n, len(index)]) for the cells at counter positions
    `index` (make_cells draws a contiguous range of them)."""
    c = np.asarray(index, dtype=np.uint64)
    ncell = c.size
    e = np.empty((n, ncell))
    for i in range(n):
        u = uniform(seed, S_Z, c * np.uint64(n) + np.uint64(i))
        e[i] = -np.log1p(-u)
    # guard the measure-zero all-zero draw
    e = np.maximum(e, 1e-300)
    z = e / e.sum(axis=0)
    t = 280.0 + 170.0 * uniform(seed, S_T, c)
    p = np.exp(np.log(0.5e6) + (np.log(40e6) - np.log(0.5e6)) * uniform(seed, S_P, c))
    return np.ascontiguousarray(p), np.ascontiguousarray(t), np.ascontiguousarray(z)


def make_near_critical_cells(mixture, ncell: int, seed: int, fraction: float = 0.2, offset: int = 0):
    """Cells with `fraction` of them near-critical: T = T_pc (1 + U[-0.01, 0.01])
    with the pseudo-critical T_pc = sum_i z_i Tc_i (Kay's rule) and p
    log-uniform on [10, 40] MPa; the rest as in make_cells."""
    n = int(mixture.n)
    p, t, z = make_cells(n, ncell, seed, offset)
    c = np.arange(offset, offset + ncell, dtype=np.uint64)
    pick = uniform(seed, S_CRIT_PICK, c) < fraction
    tpc = np.asarray(mixture.tc) @ z
    t = np.where(pick, tpc * (1.0 + 0.02 * (uniform(seed, S_CRIT_T, c) - 0.5)), t)
    p = np.where(pick, np.exp(np.log(10e6) + (np.log(40e6) - np.log(10e6)) * uniform(seed, S_CRIT_P, c)), p)
    return np.ascontiguousarray(p), np.ascontiguousarray(t), z


def three_phase_fixture_mixture():
    """The three-component PR76 mixture of the reference's max3 tests
    (tests/flash/pr76_three_phase/synthetic_fixture.hpp:33-57): a light
    component and two symmetric heavy ones with k_12 = 0.20, which split into
    three phases at 1 MPa and 250 K."""
    return Mixture(np.array([190.6, 500.0, 500.0]), np.array([4.6e6, 5.0e6, 5.0e6]), np.array([0.01, 0.10, 0.10]),
                   np.array([[0.0, 0.05, 0.05], [0.05, 0.0, 0.20], [0.05, 0.20, 0.0]]))


# the three phases of that fixture at 1 MPa, 250 K (synthetic_fixture.hpp:63-72,
# an independent root/equality solve recorded by the reference's tests)
THREE_PHASE_ANCHOR = np.array([[0.04844395156186141, 0.9076712804842868, 0.0438847679538518],
                               [0.9696550397025219, 0.015172480148739028, 0.015172480148739028],
                               [0.048443951561861175, 0.04388476795385164, 0.9076712804842871]])


def make_three_phase_cells(ncell: int, seed: int, anchor_fraction: float = 0.25):
    """Cells for the max-3-phase path on the fixture mixture: a share at the
    anchor state (1 MPa, 250 K, feeds inside the tie triangle: barycentric
    weights ~ Dirichlet(1) over the anchor phases), the rest with p
    log-uniform on [0.2, 5] MPa, T ~ U[200, 300] K, z ~ Dirichlet(1)."""
    rng = np.random.default_rng(seed)
    na = int(round(anchor_fraction * ncell))
    z = rng.dirichlet(np.ones(3), ncell).T.copy()
    t = rng.uniform(200.0, 300.0, ncell)
    p = np.exp(rng.uniform(np.log(2e5), np.log(5e6), ncell))
    w = rng.dirichlet(np.ones(3), na)
    z[:, :na] = (w @ THREE_PHASE_ANCHOR).T
    z[:, :na] /= z[:, :na].sum(axis=0)
    p[:na] = 1e6
    t[:na] = 250.0
    return p, t, z
