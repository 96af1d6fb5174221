"""Signed distance grids for the marching-cubes tests, and the per-cube comparison they share."""
from __future__ import annotations

from types import SimpleNamespace

import numpy as np


def grid(origin, cell: float, dims) -> SimpleNamespace:
    return SimpleNamespace(origin=[float(origin[0]), float(origin[1]), float(origin[2]), 0.0], cell_size=float(cell),
                           num_cells_x=int(dims[0]), num_cells_y=int(dims[1]), num_cells_z=int(dims[2]))


def sphere_plane(dims=(24, 20, 28), origin=(-0.3, 0.1, 0.2), cell=0.05) -> tuple[SimpleNamespace, np.ndarray]:
    """min(|p - c| - r, p.y - h) on the grid points, float32 arithmetic only (+ - * sqrt)."""
    X, Y, Z = dims
    f = np.float32
    z, y, x = np.meshgrid(np.arange(Z, dtype=f), np.arange(Y, dtype=f), np.arange(X, dtype=f), indexing="ij")
    px = x * f(cell) + f(origin[0])
    py = y * f(cell) + f(origin[1])
    pz = z * f(cell) + f(origin[2])
    dx, dy, dz = px - f(0.31), py - f(0.52), pz - f(0.83)
    sphere = np.sqrt(dx * dx + dy * dy + dz * dz) - f(0.37)
    plane = py - f(0.33)
    return grid(origin, cell, dims), np.minimum(sphere, plane).astype(np.float32)


def noise(dims=(12, 11, 13), seed=5) -> tuple[SimpleNamespace, np.ndarray]:
    """Gaussian noise: every cube configuration, ambiguous faces included, appears."""
    rng = np.random.default_rng(seed)
    X, Y, Z = dims
    return grid((0.5, -0.25, 0.125), 0.1, dims), rng.standard_normal((Z, Y, X)).astype(np.float32)


def configs(g, sdf: np.ndarray, iso: float) -> np.ndarray:
    """cubeIndex of every cube (x < X-1, y < Y-1, z < Z-1) in cell-index order, -1 elsewhere."""
    s = np.asarray(sdf, np.float32).reshape(g.num_cells_z, g.num_cells_y, g.num_cells_x)
    iso = np.float32(iso)
    c = np.full(s.shape, -1, np.int32)
    corner = [(0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1), (0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1)]
    inner = np.zeros(s[:-1, :-1, :-1].shape, np.int32)
    Z, Y, X = s.shape
    for k, (ox, oy, oz) in enumerate(corner):
        inner |= (s[oz:Z - 1 + oz, oy:Y - 1 + oy, ox:X - 1 + ox] < iso).astype(np.int32) << k
    c[:-1, :-1, :-1] = inner
    return c.reshape(-1)


def vertex_counts(tri_table: np.ndarray, edge_table: np.ndarray) -> np.ndarray:
    t = np.asarray(tri_table).reshape(256, 16)
    n = np.array([int(np.argmax(np.append(r, -1) == -1)) for r in t])
    return np.where(np.asarray(edge_table) != 0, n, 0)


def cube_vertex_sets(cfg: np.ndarray, counts: np.ndarray, positions: np.ndarray, written: int) -> np.ndarray:
    """Rows (cube index, x, y, z bit patterns), unique and sorted, of the first `written` vertices,
    cut into cubes in cell order by their vertex counts."""
    nv = np.where(cfg >= 0, counts[np.maximum(cfg, 0)], 0)
    ends = np.cumsum(nv)
    cells = np.nonzero(nv)[0]
    owner = np.repeat(cells, nv[cells])[:written]
    bits = np.ascontiguousarray(positions[:written, :3], np.float32).view(np.uint32).astype(np.int64)
    rows = np.column_stack([owner.astype(np.int64), bits])
    assert ends[-1] >= written
    return np.unique(rows, axis=0)


def written_vertices(cfg: np.ndarray, counts: np.ndarray, max_vertices: int) -> int:
    """Vertices the cubes that fit occupy: cubes in cell order while offset + count < max."""
    nv = np.where(cfg >= 0, counts[np.maximum(cfg, 0)], 0)
    ends = np.cumsum(nv)
    ok = (ends < max_vertices) & (nv > 0)
    return int(ends[ok].max()) if ok.any() else 0
