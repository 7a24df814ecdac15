"""Host helpers of bench.py: the stratified sample, the near-boundary
placement by bisection (against a synthetic status function with a known
boundary), rank cell offsets and the max-over-ranks reduction."""

import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_stratified_sample_spans_the_workload():
    idx = bench.stratified(1000, 100)
    assert idx.size == 100 and idx[0] == 0 and idx[-1] == 999
    assert np.all(np.diff(idx) > 0)
    assert bench.stratified(50, 100).size == 50


def test_placement_brackets_a_known_boundary():
    rng = np.random.default_rng(3)
    ncell = 400
    t = rng.uniform(280.0, 450.0, ncell)
    z = rng.dirichlet(np.ones(3), ncell).T
    boundary = 1e6 * (1.0 + (t - 280.0) / 20.0)  # two-phase below, single-phase above
    idx = np.arange(ncell)

    def status(p, tt, zz):
        pb = 1e6 * (1.0 + (tt - 280.0) / 20.0)
        return np.where(p < pb, 1, 0)

    p, ok, br = bench.place_near(t, z, idx, idx, status)
    assert ok.all()
    assert np.all(np.exp(br[0]) < boundary) and np.all(np.exp(br[1]) >= boundary)
    # 7 bisections of a 9-point log grid leave a 0.43 % bracket; the placement
    # noise is +-2 % of the bracket midpoint
    rel = p / boundary - 1.0
    assert np.all(np.abs(rel) <= 0.0205 + 0.0025), np.abs(rel).max()
    assert rel.min() < -0.01 and rel.max() > 0.01  # the noise spreads both ways


def test_rank_offsets_are_disjoint_and_reduction_is_identity_on_one_rank():
    ncell = 1 << 20
    spans = [(bench.cell_offset(r, ncell), bench.cell_offset(r, ncell) + ncell) for r in range(8)]
    for a, b in zip(spans, spans[1:]):
        assert a[1] <= b[0]
    assert bench.max_over_ranks(3.5, 1, "cpu") == 3.5


def test_chart_states_are_valid_two_phase_charts(oracle_lib):
    """The chart leg's states: [P n + 1, ncell], positive fractions whose
    dependent (last) one stays positive; the oracle evaluates them."""
    import numpy as np

    import bench
    from mpmc_hnu_gb300 import synth

    n, phases = bench.CHART_N, bench.CHART_PHASES
    q = bench.chart_states(n, phases, 500, 34)
    assert q.shape == (phases * n + 1, 500)
    for ph in range(phases):
        block = q[phases + 1 + ph * (n - 1):phases + 1 + (ph + 1) * (n - 1)]
        assert (block > 0).all() and (block.sum(axis=0) < 1).all()
    visc = np.concatenate([[8.0e-6, 1e-12, 1e-8, 1e-12, 1e-4, 1e-9, 1e-7], np.full(n, 1e-7)])
    enth = np.concatenate([[0.0, 2e-4, 1200.0, 0.5, 1e4, 0.1, 10.0], np.full(n, 100.0)])
    out = oracle_lib.property_chart(synth.make_mixture(n, 1001), phases, [0, 0], np.full(n, 0.05), visc, enth, q)
    assert (out["status"] == 0).mean() > 0.99


def test_resampling_places_every_cell_that_a_redraw_brackets():
    """A cell whose draw has no phase-count change on [0.5, 40] MPa draws a
    new (T, z) at its own index until one brackets; here only T < 400 K has a
    boundary, so every cell ends placed after a few rounds."""
    from mpmc_hnu_gb300 import synth

    n, ncell = 3, 300
    p, t, z = synth.make_cells(n, ncell, bench.CELL_SEED)

    def status(pp, tt, zz):
        return np.where((tt < 400.0) & (pp < 2e6 + 1e5 * (tt - 280.0)), 1, 0)

    p2, t2, z2, placed, br = bench.place_workload(n, p, t, z, 0, 200, status, synth)
    assert placed.all()
    assert np.all(t2[:200] < 400.0)
    assert np.array_equal(t2[200:], t[200:]) and np.array_equal(p2[200:], p[200:])
    first = t[:200] < 400.0  # cells that bracketed on their first draw keep it
    assert np.array_equal(t2[:200][first], t[:200][first])
    assert np.isfinite(br).all()


def test_wilson_k_matches_its_formula():
    from mpmc_hnu_gb300 import synth

    mix = synth.make_mixture(4, 5)
    p, t = np.array([2e6, 8e6]), np.array([300.0, 420.0])
    lk = bench.wilson_ln_k(mix, p, t)
    i, c = 2, 1
    want = np.log(mix.pc[i] / p[c]) + 5.373 * (1 + mix.omega[i]) * (1 - mix.tc[i] / t[c])
    assert abs(lk[i, c] - want) < 1e-12


def test_stage_roofline_uses_each_stage_own_work():
    n = 10
    stats = {"fp64_evals_setup": 100, "fp64_evals_feed_trials": 2000, "fp64_evals_review_trials": 300,
             "fp64_evals_polish": 500, "fp64_evals_split64": 700, "polish_jacobians": 50, "polish_solves": 90}
    counters = np.zeros((8, 4))
    counters[0] = 10.0
    counters[1] = 20.0
    counters[2] = 5.0
    counters[4] = 3.0
    stages = {"setup": 1.0, "feed_trials": 2.0, "feed_trials64": 3.0, "split": 1.0, "open32": 0.5, "polish": 9.0,
              "split64": 4.0, "review_trials": 1.0, "review_trials64": 1.0, "sensitivity": 2.0}
    r = bench.roofline_of(n, stages, stats, counters, 7, 1.0, 50.0, 30.0, lambda k: None)
    assert r["kernel"] == "polish" and r["bound"] == "fp64"
    want = 500 * bench.f_eval(n) + 12 * 6 * n + 50 * bench.f_jacobian(n) + 90 * 2 * n * n
    assert r["flops_per_launch"] == want
    assert abs(r["achieved"] - want / 9e-3 / 1e12) < 1e-15
    assert abs(r["frac"] - r["achieved"] / 1.0) < 1e-15
    assert r["fp32_screening"]["ms"] == 4.5


def test_error_report_counts_statuses_and_relative_errors():
    n = 2
    ref = {"status": np.array([1, 1, 0]), "ln_k": np.array([[1.0, 2.0, np.nan], [-1.0, -2.0, np.nan]]),
           "beta": np.array([0.5, 0.25, np.nan]), "x": np.full((2, 3), 0.5), "y": np.full((2, 3), 0.5)}
    gpu = {"status": np.array([1, 1, 1]), "ln_k": ref["ln_k"] * (1 + 1e-9), "vapor_fraction": ref["beta"],
           "liquid": ref["x"], "vapor": ref["y"]}
    rep = bench.error_report(n, gpu, ref, False)
    assert rep["status_mismatches"] == 1 and rep["two_phase"] == 2
    assert abs(rep["errors"]["ln_k"]["max"] - 1e-9) < 1e-12
    assert rep["errors"]["beta"]["max"] == 0.0
