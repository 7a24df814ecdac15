"""Selected-phase property chart cases shared by the oracle, host-build and
GPU tests and by tests/golden/make_property_chart_golden.py.

A case is (mixture, PropertyChartSpec, q [P n + 1, ncell], dependent
[P, ncell] or None).  `fixture_cases()` holds the states of the reference's
own closure test (tests/flow/core/pr76_selected_phase_property_closure_test.cpp:
the manufactured three-component mixture at :92-158, its synthetic
viscosity/enthalpy provider at :191-231 written as affine coefficients, the
chart states of :309-359 and the selections of :438-470).  `random_cases()`
draws seeded synthetic states with random pivot components on the bench
mixture generator; `edge_case()` appends the failure classes the chart
reports.
"""

from __future__ import annotations

import numpy as np

from mpmc_hnu_gb300 import synth
from mpmc_hnu_gb300.flash import PropertyChartSpec


def fixture_mixture():
    """Manufactured mixture of the reference's closure test (:92-158)."""
    return synth.Mixture(np.array([400.0, 500.0, 600.0]), np.array([4.0e6, 3.0e6, 5.0e6]),
                         np.array([-0.125, 0.25, 0.5]),
                         np.array([[0.0, 0.125, -0.0625], [0.125, 0.0, 0.0625], [-0.0625, 0.0625, 0.0]]))


def fixture_models(n: int = 3):
    """The test provider (:191-231) as affine coefficients: viscosity
    8e-6 + 1e-12 p + 1e-8 T + 1e-6 sum (i+1) x_i + 1e-12 rho + 1e-7 root,
    enthalpy 1200 T + 2e-4 p + 2000 sum (i+1) x_i + 1e4 M + 0.1 rho_mass."""
    visc = np.zeros(7 + n)
    visc[[0, 1, 2, 3, 6]] = [8.0e-6, 1.0e-12, 1.0e-8, 1.0e-12, 1.0e-7]
    visc[7:] = (np.arange(n) + 1) * 1.0e-6
    enth = np.zeros(7 + n)
    enth[[1, 2, 4, 5]] = [2.0e-4, 1200.0, 1.0e4, 0.1]
    enth[7:] = (np.arange(n) + 1) * 2000.0
    return visc, enth


FIXTURE_MOLAR_MASS = np.array([0.016, 0.030, 0.044])


def fixture_cases():
    """The closure test's three charts (P = 1, 2, 3 at 1 MPa, 450 K, every
    phase at x = (0.25, 0.5, 0.25), saturations 0.4 or 0.2 / 0.3) with its
    selections: root 2; roots 0, 2; roots 0, 1, 2."""
    mix = fixture_mixture()
    visc, enth = fixture_models()
    out = []
    for phases, roots, sat in ((1, [2], []), (2, [0, 2], [0.4]), (3, [0, 1, 2], [0.2, 0.3])):
        q = np.array([1.0e6, 450.0] + sat + [0.25, 0.5] * phases)[:, None]
        out.append((f"fixture_p{phases}", mix, PropertyChartSpec(phases, roots, FIXTURE_MOLAR_MASS, visc, enth), q,
                    None))
    return out


def random_states(n: int, phases: int, ncell: int, seed: int):
    """q [P n + 1, ncell] and dependent [P, ncell]: p log-uniform on
    [0.5, 40] MPa, T ~ U[200, 450] K, saturations ~ U[0.05, 0.4], each
    phase's composition ~ Dirichlet(1) with a random pivot component."""
    rng = np.random.default_rng(seed)
    p = np.exp(rng.uniform(np.log(5.0e5), np.log(4.0e7), ncell))
    t = rng.uniform(200.0, 450.0, ncell)
    sat = rng.uniform(0.05, 0.4, (phases - 1, ncell))
    dep = rng.integers(0, n, (phases, ncell)).astype(np.int32)
    blocks = []
    for ph in range(phases):
        x = rng.dirichlet(np.ones(n), ncell).T
        keep = np.ones((n, ncell), bool)
        keep[dep[ph], np.arange(ncell)] = False
        blocks.append(x.T[keep.T].reshape(ncell, n - 1).T)
    # C order: vstack keeps its inputs' (Fortran) layout, and device copies of
    # the array must be row-major [q, ncell] like the C ABI's chart layout
    q = np.ascontiguousarray(np.vstack([p[None], t[None], sat] + blocks))
    return q, dep


def random_spec(n: int, phases: int, roots, seed: int) -> PropertyChartSpec:
    rng = np.random.default_rng(seed + 1)
    mm = rng.uniform(0.01, 0.2, n)
    visc = np.concatenate([[1.0e-5, 1.0e-12, 1.0e-8, 1.0e-12, 1.0e-4, 1.0e-9, 1.0e-7], rng.uniform(0, 1.0e-6, n)])
    enth = np.concatenate([[1.0e3, 2.0e-4, 1200.0, 0.5, 1.0e4, 0.1, 10.0], rng.uniform(0, 2000.0, n)])
    return PropertyChartSpec(phases, roots, mm, visc, enth)


def random_case(name: str, n: int, phases: int, roots, ncell: int, seed: int):
    mix = synth.make_mixture(n, 1001 + n)
    q, dep = random_states(n, phases, ncell, seed)
    return (name, mix, random_spec(n, phases, roots, seed), q, dep)


def edge_case(n: int = 6, seed: int = 7):
    """Two-phase cells whose chart fails in each class the chart reports:
    a NaN entry (1), a zero and a negative independent fraction (1), fractions
    whose dependent one is negative (1); then the first three states again with
    a second phase selecting a third root that does not exist (4) and with a
    viscosity model that is negative there (6).  Cells 0-2 and 7 succeed."""
    name, mix, spec, q, dep = random_case("edge", n, 2, [0, 0], 8, seed)
    q = q.copy()
    first = 3  # first independent fraction of phase 0
    q[0, 3] = np.nan
    q[first, 4] = 0.0
    q[first, 5] = -0.1
    q[first:first + n - 1, 6] = 0.9 / (n - 2)
    spec_bad_root = PropertyChartSpec(2, [0, 2], spec.molar_mass, spec.viscosity, spec.enthalpy)
    visc_neg = spec.viscosity.copy()
    visc_neg[0] = -1.0
    spec_neg = PropertyChartSpec(2, [0, 0], spec.molar_mass, visc_neg, spec.enthalpy)
    return [(name, mix, spec, q, dep), ("edge_root", mix, spec_bad_root, q[:, :3].copy(), dep[:, :3].copy()),
            ("edge_visc", mix, spec_neg, q[:, :3].copy(), dep[:, :3].copy())]


def golden_cases():
    """Every case recorded in tests/golden/property_chart_reference.npz."""
    return (fixture_cases() +
            [random_case("n10_p2", 10, 2, [0, 0], 32, 21), random_case("n10_p3", 10, 3, [0, 1, 2], 32, 22),
             random_case("n4_p2", 4, 2, [0, 0], 24, 23), random_case("n20_p1", 20, 1, [0], 12, 24),
             random_case("n2_p2", 2, 2, [0, 0], 24, 25)] + edge_case())
