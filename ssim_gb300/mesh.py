"""Tet mesh generators and the seeded PRNG used by every synthetic workload.

``unit_box`` follows ssim::mesh::unit_box (ssim/include/ssim/mesh/common_shapes.hpp:67-132):
vertex *counts* per axis, vertex id (i*ny + j)*nz + k, five tets per cell with
parity-dependent mirroring.  ``kuhn_box`` cuts every hex cell into the six tets
around its main diagonal (the Kuhn / Freudenthal subdivision), which is
conforming across cells.  Both return X [V,3] float64 and cells [T,4] int32.
"""
from __future__ import annotations

import numpy as np

# ---------------------------------------------------------------- SplitMix64
_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def _mix(z: np.ndarray) -> np.ndarray:
    z = (z ^ (z >> np.uint64(30))) * _M1
    z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def splitmix64(seed: int, n: int, offset: int = 0) -> np.ndarray:
    """Outputs offset .. offset+n-1 of SplitMix64 (Steele, Lea & Flood, OOPSLA 2014) seeded with ``seed``:
    x_k = mix(seed + (k+1) * 0x9E3779B97F4A7C15)."""
    k = np.arange(offset + 1, offset + n + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        return _mix(np.uint64(seed) + k * _GAMMA)


def uniform(seed: int, n: int, lo: float = 0.0, hi: float = 1.0, offset: int = 0) -> np.ndarray:
    """n doubles in [lo, hi) from the top 53 bits of SplitMix64."""
    u = (splitmix64(seed, n, offset) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return lo + (hi - lo) * u


def normal(seed: int, n: int, offset: int = 0) -> np.ndarray:
    """n standard normals by Box-Muller over pairs of ``uniform`` draws."""
    m = (n + 1) // 2
    u1 = uniform(seed, m, offset=offset)
    u2 = uniform(seed, m, offset=offset + m)
    r = np.sqrt(-2.0 * np.log1p(-u1))
    z = np.concatenate([r * np.cos(2 * np.pi * u2), r * np.sin(2 * np.pi * u2)])
    return z[:n]


# ---------------------------------------------------------------- meshes
def unit_box(nx: int = 2, ny: int = 2, nz: int = 2):
    """ssim::mesh::unit_box: [0,1]^3 with nx*ny*nz vertices, 5 tets per cell."""
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    X = np.stack([i / (nx - 1), j / (ny - 1), k / (nz - 1)], axis=-1).reshape(-1, 3).astype(np.float64)
    ci, cj, ck = [a.reshape(-1) for a in np.meshgrid(np.arange(nx - 1), np.arange(ny - 1), np.arange(nz - 1), indexing="ij")]

    def vid(a, b, c):
        return (a * ny + b) * nz + c

    # corner (dx, dy, dz) of every cell, mirrored per axis on odd cells (common_shapes.hpp:101-126)
    fx, fy, fz = ci % 2, cj % 2, ck % 2

    def corner(dx, dy, dz):
        return vid(ci + (dx ^ fx), cj + (dy ^ fy), ck + (dz ^ fz))

    c000, c100, c010, c001 = corner(0, 0, 0), corner(1, 0, 0), corner(0, 1, 0), corner(0, 0, 1)
    c110, c101, c011, c111 = corner(1, 1, 0), corner(1, 0, 1), corner(0, 1, 1), corner(1, 1, 1)
    tets = np.stack(
        [
            np.stack([c000, c100, c010, c001], -1),
            np.stack([c010, c100, c110, c111], -1),
            np.stack([c100, c010, c001, c111], -1),
            np.stack([c100, c001, c101, c111], -1),
            np.stack([c011, c001, c010, c111], -1),
        ],
        axis=1,
    )
    return X, tets.reshape(-1, 4).astype(np.int32)


def unit_square(nx: int = 2, ny: int = 2):
    """Triangles of the unit square: an nx x ny vertex grid (vertex (i, j) = i * ny + j at (i/(nx-1),
    j/(ny-1))), each cell cut along its (i, j)-(i+1, j+1) diagonal into two counter-clockwise triangles."""
    xs = np.linspace(0.0, 1.0, nx)
    ys = np.linspace(0.0, 1.0, ny)
    X = np.stack(np.meshgrid(xs, ys, indexing="ij"), axis=-1).reshape(-1, 2)
    idx = np.arange(nx * ny, dtype=np.int32).reshape(nx, ny)
    a, b, c, d = idx[:-1, :-1], idx[1:, :-1], idx[1:, 1:], idx[:-1, 1:]
    T = np.concatenate([np.stack([a, b, c], -1).reshape(-1, 3), np.stack([a, c, d], -1).reshape(-1, 3)])
    return X, T.astype(np.int32)


def tetra():
    """ssim::mesh::tetra (common_shapes.hpp:134-145)."""
    X = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=np.float64)
    return X, np.array([[0, 1, 2, 3]], dtype=np.int32)


_KUHN_PATHS = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]


def kuhn_box(cells=(10, 10, 10), size=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0)):
    """Box of nx*ny*nz hex cells, 6 positively oriented tets per cell (Kuhn subdivision).
    Vertex (i, j, k) has id (i*(ny+1) + j)*(nz+1) + k."""
    nx, ny, nz = cells
    vx, vy, vz = nx + 1, ny + 1, nz + 1
    i, j, k = np.meshgrid(np.arange(vx), np.arange(vy), np.arange(vz), indexing="ij")
    X = np.stack(
        [origin[0] + size[0] * i / nx, origin[1] + size[1] * j / ny, origin[2] + size[2] * k / nz], axis=-1
    ).reshape(-1, 3)
    ci, cj, ck = [a.reshape(-1) for a in np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")]
    tets = []
    for a, b, c in _KUHN_PATHS:
        step = np.zeros((4, 3), dtype=np.int64)
        e = np.eye(3, dtype=np.int64)
        step[1] = e[a]
        step[2] = e[a] + e[b]
        step[3] = e[a] + e[b] + e[c]
        # orientation of [e_a, e_b, e_c] is the sign of the axis permutation: swap two vertices if odd
        order = [0, 1, 2, 3] if np.linalg.det(np.stack([e[a], e[b], e[c]], 1).astype(float)) > 0 else [0, 2, 1, 3]
        ids = [((ci + step[o, 0]) * vy + (cj + step[o, 1])) * vz + (ck + step[o, 2]) for o in order]
        tets.append(np.stack(ids, -1))
    T = np.stack(tets, axis=1).reshape(-1, 4).astype(np.int32)
    return X.astype(np.float64), T


def boundary_vertices(X: np.ndarray, tol: float = 1e-12) -> np.ndarray:
    """Mask of vertices on the bounding box's surface."""
    lo, hi = X.min(0), X.max(0)
    return np.any((np.abs(X - lo) <= tol) | (np.abs(X - hi) <= tol), axis=1)


def jitter_interior(X: np.ndarray, amplitude: float, seed: int) -> np.ndarray:
    """Interior vertices moved by U(-amplitude, amplitude) per coordinate (SplitMix64 stream ``seed``)."""
    Y = X.copy()
    inner = np.where(~boundary_vertices(X))[0]
    d = uniform(seed, 3 * inner.size, -amplitude, amplitude).reshape(-1, 3)
    Y[inner] += d
    return Y


def volumes(X: np.ndarray, cells: np.ndarray) -> np.ndarray:
    x = X[cells]
    D = np.stack([x[:, 1] - x[:, 0], x[:, 2] - x[:, 0], x[:, 3] - x[:, 0]], axis=-1)
    return np.linalg.det(D) / 6.0
