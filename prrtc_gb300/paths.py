"""Path utilities around the planner's output.

pRRTC returns a path goal first (pRRTC.cu:568-602); the smoothing entry
points take fixed-size paths start first.  `resample` turns one planner path
into `waypoints` rows on the same polyline: every planner vertex is kept and
the remaining rows are spread over the segments in proportion to their
length, so the resampled path passes through exactly the configurations the
planner connected.
"""
from __future__ import annotations

import numpy as np


def start_first(path: np.ndarray) -> np.ndarray:
    """Planner path (goal first) -> start-first rows."""
    return np.ascontiguousarray(np.asarray(path, np.float32)[::-1])


def resample(path: np.ndarray, waypoints: int = 64) -> np.ndarray | None:
    """[k, dof] start-first path -> [waypoints, dof] float32 on the same
    polyline, or None when the path has more than `waypoints` vertices."""
    p = np.asarray(path, np.float64)
    # drop repeated vertices (zero-length segments)
    keep = np.concatenate([[True], np.linalg.norm(np.diff(p, axis=0), axis=1) > 0])
    p = p[keep]
    k = len(p)
    if k > waypoints:
        return None
    if k == 1:
        return np.repeat(p.astype(np.float32), waypoints, axis=0)
    seg = np.linalg.norm(np.diff(p, axis=0), axis=1)
    extra = waypoints - k
    # largest-remainder split of the extra rows over the segments by length
    share = seg / seg.sum() * extra
    n = np.floor(share).astype(int)
    rest = extra - n.sum()
    if rest:
        n[np.argsort(-(share - n), kind="stable")[:rest]] += 1
    rows = [p[0]]
    for i in range(k - 1):
        a, b = p[i], p[i + 1]
        for j in range(1, n[i] + 1):
            rows.append(a + (b - a) * (j / (n[i] + 1)))
        rows.append(b)
    out = np.asarray(rows, np.float32)
    assert out.shape[0] == waypoints
    return out


def length(path: np.ndarray) -> np.ndarray:
    """Joint-space length of [..., W, dof] paths."""
    p = np.asarray(path, np.float64)
    return np.linalg.norm(np.diff(p, axis=-2), axis=-1).sum(-1)
