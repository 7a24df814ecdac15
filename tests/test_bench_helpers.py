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

    p, ok = bench.place_near(t, z, idx, idx, status)
    assert ok.all()
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
