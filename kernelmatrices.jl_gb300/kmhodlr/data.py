"""Input helpers: seeded synthetic points and a k-d ordering of 2-D points.

The reference sorts points with ``NearestNeighbors.KDTree(pts).data`` (maxlikdata,
src/HODLR/src/constructor.jl:171-181) so that consecutive indices are spatially close.  This
module provides its own deterministic k-d ordering (median split on the wider coordinate,
recursively); the ordering is an input of the engine, so the engine and the oracle are always
fed the same ordered points.
"""
from __future__ import annotations

import numpy as np


def kd_order(pts: np.ndarray, leaf: int = 32) -> np.ndarray:
    """Permutation that orders (n, 2) points by recursive median splits."""
    pts = np.asarray(pts, dtype=np.float64)
    out = np.empty(len(pts), dtype=np.int64)
    pos = 0
    stack = [np.arange(len(pts))]
    while stack:
        idx = stack.pop()
        if len(idx) <= leaf:
            out[pos:pos + len(idx)] = idx
            pos += len(idx)
            continue
        sub = pts[idx]
        ax = 0 if np.ptp(sub[:, 0]) >= np.ptp(sub[:, 1]) else 1
        o = idx[np.argsort(sub[:, ax], kind="stable")]
        h = len(o) // 2
        stack.append(o[h:])
        stack.append(o[:h])
    return out


def uniform_points(n: int, seed: int, kd: bool = True) -> np.ndarray:
    """n points uniform on [0, 1]^2 from ``default_rng(seed)``, k-d ordered when ``kd``."""
    pts = np.random.default_rng(seed).uniform(size=(n, 2))
    return np.ascontiguousarray(pts[kd_order(pts)] if kd else pts)


def normal_points(n: int, seed: int) -> np.ndarray:
    """n points with iid N(0, 1) coordinates (README.md:34), unsorted as in the README."""
    return np.ascontiguousarray(np.random.default_rng(seed).standard_normal((n, 2)))


def rademacher(n: int, count: int, seed: int) -> np.ndarray:
    """(n, count) Rademacher probe matrix (the role of givesaa, src/HODLR/src/utils.jl:22-27)."""
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.choice(np.array([-1.0, 1.0]), size=(n, count)))
