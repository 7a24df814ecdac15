"""Host logic of the ordered-path continuation (mpmc_hnu_gb300/continuation.py):
phase counts of the published statuses and transition brackets, as in
pr76_pt_continuation.hpp:77-90 and :263-300."""

import numpy as np

from mpmc_hnu_gb300 import continuation


def test_phase_counts_follow_the_published_status():
    st = np.array([0, 1, 4, 2, 3, -1])
    assert continuation.phase_counts(st).tolist() == [1, 2, 3, 0, 0, 0]


def test_brackets_between_accepted_points_only():
    counts = np.array([[1, 1, 2, 2, 0, 2, 3],
                       [3, 1, 1, 1, 1, 1, 1],
                       [2, 2, 2, 2, 2, 2, 2]])
    br = continuation.transition_brackets(counts)
    assert br == [(0, 1, 2, 1, 2, True), (0, 5, 6, 2, 3, True), (1, 0, 1, 3, 1, False)]


def test_scan_with_hints_carries_the_accepted_phases():
    """The hints of the next point (pr76_pt_continuation.hpp:262-300): the feed
    after one phase, the pair after two (one start if x equals y), the set and
    its phase-1/phase-2 fractions after three, nothing after an unresolved
    point; the feed is normalised once."""
    n, npath = 2, 5
    feeds = np.array([[0.2, 0.4, 0.5, 0.6, 0.7], [0.8, 0.6, 0.5, 0.4, 0.30000000000000004]])
    p = np.full((npath, 3), 1e6)
    t = np.full((npath, 3), 300.0)
    seen = []
    # per path: single, two, two with x == y, three, unresolved (max3 5)
    m3 = np.array([0, 1, 1, 2, 5])

    def step(pk, tk, z, count, hx, three, frac):
        seen.append((count.copy(), hx.copy(), three.copy(), frac.copy(), z.copy()))
        x = np.vstack([z[0], z[1]])
        y = x.copy()
        y[:, 1] = [0.9, 0.1]
        x3 = np.tile(np.array([[0.1], [0.9], [0.5], [0.5], [0.9], [0.1]]), (1, npath))
        f3 = np.tile(np.array([[0.2], [0.3], [0.5]]), (1, npath))
        return {"published": np.array([0, 1, 1, 4, 3]), "max3": m3, "x": x, "y": y, "x3": x3, "f3": f3}

    res = continuation.scan_with_hints(step, feeds, p, t)
    assert len(seen) == 3
    count, hx, three, frac, z = seen[0]
    assert (count == 0).all() and (three == 0).all()
    assert np.allclose(z.sum(axis=0), 1.0)
    count, hx, three, frac, z = seen[1]
    assert list(count) == [1, 2, 1, 3, 0]
    assert np.array_equal(hx[:n, 0], z[:, 0])
    assert np.array_equal(hx[n:2 * n, 1], [0.9, 0.1])
    assert list(three) == [0, 0, 0, 1, 0]
    assert np.allclose(frac[:, 3], [0.3, 0.5]) and np.all(frac[:, [0, 1, 2, 4]] == 0)
    assert np.array_equal(res["phase_count"][:, 0], [1, 2, 2, 3, 0])
