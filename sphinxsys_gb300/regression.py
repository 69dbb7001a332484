"""Dynamic-time-warping regression comparator.

Restates RegressionTestDynamicTimeWarping (src/shared/regression_test/
dynamic_time_warping_method.hpp:17-55 for the distance, :162-186 for the pass rule):
a run passes against a stored run when its DTW distance is at most 1.01 times the
stored maximum distance.  Reproduced quirks: the local-distance table starts at zero,
cells outside the +/- window keep that zero, and the window widens to the length
difference of the two series.
"""
from __future__ import annotations

from typing import Sequence

import numpy as np


def dtw_distance(a: Sequence[float], b: Sequence[float], window: int = 5) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    la, lb = len(a), len(b)
    if lb > 1.2 * la or lb < 0.8 * la:
        raise ValueError("series lengths differ by more than 20%")
    d = np.zeros((la, lb))
    d[0, 0] = abs(a[0] - b[0])
    for i in range(1, la):
        d[i, 0] = d[i - 1, 0] + abs(a[i] - b[0])
    for j in range(1, lb):
        d[0, j] = d[0, j - 1] + abs(a[0] - b[j])
    window = max(window, abs(la - lb))
    for i in range(1, la):
        for j in range(max(1, i - window), min(lb, i + window)):
            d[i, j] = abs(a[i] - b[j]) + min(d[i - 1, j], d[i, j - 1], d[i - 1, j - 1])
    return float(d[la - 1, lb - 1])


def passes(stored_runs, current, stored_dtw, both_orders: bool = False) -> tuple:
    """Returns (ok, distances) for a (observations x snapshots) series against stored runs.

    The reference measures dtw(stored, current).  When the current series is longer than a
    stored one by the window or more, the last cell of that table lies outside the band
    and keeps its zero, so the distance is zero whatever the data; ``both_orders`` also
    requires dtw(current, stored), whose last cell is inside the band, to pass."""
    current = np.atleast_2d(np.asarray(current, dtype=np.float64))
    dists = []
    ok = True
    for run in stored_runs:
        run = np.atleast_2d(run)
        row = []
        for k in range(current.shape[0]):
            ref = run[k][~np.isnan(run[k])]
            dk = dtw_distance(ref, current[k])
            if both_orders:
                dk = max(dk, dtw_distance(current[k], ref))
            row.append(dk)
            if dk > 1.01 * stored_dtw[k]:
                ok = False
        dists.append(row)
    return ok, np.array(dists)
