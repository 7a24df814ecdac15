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
