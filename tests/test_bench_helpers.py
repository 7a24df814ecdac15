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
