"""Seeded synthetic point-cloud generators for the benchmark workloads.

The reference ships no dataset; its own benches draw uniform clouds
(``tests/bench_knn.py:11``: 1M points in [0, 200)^3; ``tests/helpers.py:7``).
The outdoor-scene generator below stands in for LiDAR-like data: a noisy
ground plane, vertical wall rectangles, vertical cylinders (poles, trunks) and
uniform scatter (vegetation / noise). Everything is float32 and reproducible
from the seed.
"""

from __future__ import annotations

import numpy as np

__all__ = ["uniform_cube", "outdoor_scene", "scaled_scene", "log_uniform_sizes"]


def uniform_cube(n: int, seed: int = 0, side: float = 1.0) -> np.ndarray:
    """``n`` points uniform in ``[0, side)^3`` as a C-contiguous float32 (n, 3) array."""
    rng = np.random.default_rng(seed)
    return np.ascontiguousarray(rng.random((n, 3), dtype=np.float32) * np.float32(side))


def _split_counts(n: int, fractions) -> list[int]:
    counts = [int(n * f) for f in fractions]
    counts[0] += n - sum(counts)
    return counts


def outdoor_scene(
    n: int,
    seed: int = 1,
    box=(100.0, 100.0, 20.0),
    n_walls: int = 40,
    n_cylinders: int = 200,
) -> np.ndarray:
    """Outdoor scene of ``n`` points in a ``box`` (metres), float32 (n, 3).

    Composition: 50% ground plane z ~ N(0, 0.01); 25% on ``n_walls`` random
    vertical rectangles; 15% on ``n_cylinders`` vertical cylinders with radius
    U(0.1, 0.5) and height U(2, 10); 10% uniform scatter in the box. Points are
    shuffled so that memory order carries no spatial locality.
    """
    rng = np.random.default_rng(seed)
    bx, by, bz = (float(v) for v in box)
    n_ground, n_wall, n_cyl, n_scatter = _split_counts(n, (0.50, 0.25, 0.15, 0.10))
    parts = []

    g = np.empty((n_ground, 3), dtype=np.float64)
    g[:, 0] = rng.uniform(0.0, bx, n_ground)
    g[:, 1] = rng.uniform(0.0, by, n_ground)
    g[:, 2] = rng.normal(0.0, 0.01, n_ground)
    parts.append(g)

    if n_wall:
        length = rng.uniform(0.05, 0.3, n_walls) * min(bx, by)
        height = rng.uniform(0.15, 0.75, n_walls) * bz
        angle = rng.uniform(0.0, np.pi, n_walls)
        # keep every wall inside the box: |cos|, |sin| <= 1
        cx = rng.uniform(0.0, 1.0, n_walls) * (bx - length) + 0.5 * length
        cy = rng.uniform(0.0, 1.0, n_walls) * (by - length) + 0.5 * length
        area = length * height
        wid = rng.choice(n_walls, size=n_wall, p=area / area.sum())
        u = rng.uniform(-0.5, 0.5, n_wall) * length[wid]
        w = np.empty((n_wall, 3), dtype=np.float64)
        w[:, 0] = cx[wid] + u * np.cos(angle[wid])
        w[:, 1] = cy[wid] + u * np.sin(angle[wid])
        w[:, 2] = rng.uniform(0.0, 1.0, n_wall) * height[wid]
        # small thickness noise along the wall normal
        t = rng.normal(0.0, 0.005, n_wall)
        w[:, 0] += -t * np.sin(angle[wid])
        w[:, 1] += t * np.cos(angle[wid])
        parts.append(w)

    if n_cyl:
        radius = rng.uniform(0.1, 0.5, n_cylinders)
        height = rng.uniform(2.0, 10.0, n_cylinders) * (bz / 20.0)
        cx = rng.uniform(0.0, 1.0, n_cylinders) * (bx - 2 * radius) + radius
        cy = rng.uniform(0.0, 1.0, n_cylinders) * (by - 2 * radius) + radius
        area = radius * height
        cid = rng.choice(n_cylinders, size=n_cyl, p=area / area.sum())
        theta = rng.uniform(0.0, 2.0 * np.pi, n_cyl)
        c = np.empty((n_cyl, 3), dtype=np.float64)
        c[:, 0] = cx[cid] + radius[cid] * np.cos(theta)
        c[:, 1] = cy[cid] + radius[cid] * np.sin(theta)
        c[:, 2] = rng.uniform(0.0, 1.0, n_cyl) * height[cid]
        parts.append(c)

    if n_scatter:
        s = np.empty((n_scatter, 3), dtype=np.float64)
        s[:, 0] = rng.uniform(0.0, bx, n_scatter)
        s[:, 1] = rng.uniform(0.0, by, n_scatter)
        s[:, 2] = rng.uniform(0.0, bz, n_scatter)
        parts.append(s)

    xyz = np.concatenate(parts, axis=0)
    xyz = xyz[rng.permutation(len(xyz))]
    return np.ascontiguousarray(xyz.astype(np.float32))


def scaled_scene(n: int, seed: int, side: float) -> np.ndarray:
    """The outdoor-scene generator scaled into a cube-ish box of ``side`` metres."""
    return outdoor_scene(
        n, seed=seed, box=(side, side, side * 0.2),
        n_walls=max(1, int(round(40 * (side / 100.0) ** 2))) if side >= 10 else 2,
        n_cylinders=max(2, int(round(200 * (side / 100.0) ** 2))),
    )


def log_uniform_sizes(count: int, lo: int, hi: int, seed: int) -> np.ndarray:
    """``count`` integer sizes log-uniform in ``[lo, hi]``."""
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(lo), np.log(hi), count)).astype(np.int64)
