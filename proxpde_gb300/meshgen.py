"""Synthetic inputs: structured unit-cube meshes and seeded random fields.

- ``cube_hex(n)`` and ``cube_tet5(n)`` build the same meshes as proxpde's
  ``buildCube`` for hexahedra and for 5-tetrahedra cubes (src/mesh.cpp:355-534): node
  id ``i + (n+1) j + (n+1)^2 k`` at ``(i, j, k) h``, elements in k, j, i order.
- ``cube_tet6(n)`` splits every cube in 6 tetrahedra (Kuhn split, not in proxpde):
  for each axis permutation (a, b, c) in lexicographic order the tetrahedron
  ``{v0, v0 + e_a, v0 + e_a + e_b, v0 + e_a + e_b + e_c}``.
- ``perturb`` moves interior nodes by a seeded uniform offset in [-alpha h, alpha h]
  per coordinate (boundary nodes stay on the cube faces).
- ``lognormal`` gives ``exp(sigma N(0,1))`` per element.

Random numbers come from SplitMix64 keyed by (seed, entity id), so every input is a
pure function of its seed and identical on every machine that runs numpy.
"""
from __future__ import annotations

import numpy as np

_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_G = np.uint64(0x9E3779B97F4A7C15)


def splitmix64(seed: int, idx: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = (np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + (idx.astype(np.uint64) + np.uint64(1)) * _G)
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform01(seed: int, idx: np.ndarray) -> np.ndarray:
    """Uniform in [0, 1) with 53 random bits."""
    return (splitmix64(seed, idx) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def _grid(n):
    np1 = n + 1
    h = 1.0 / n
    k, j, i = np.meshgrid(np.arange(np1), np.arange(np1), np.arange(np1), indexing="ij")
    xyz = np.stack([i.reshape(-1) * h, j.reshape(-1) * h, k.reshape(-1) * h], axis=1)
    return np.ascontiguousarray(xyz)


def _bases(n):
    np1 = n + 1
    k, j, i = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    return (i + j * np1 + k * np1 * np1).reshape(-1).astype(np.int64), (i + j + k).reshape(-1)


def cube_hex(n: int):
    np1 = n + 1
    dx, dy, dz = 1, np1, np1 * np1
    b, _ = _bases(n)
    conn = np.stack([b, b + dx, b + dx + dy, b + dy, b + dz, b + dx + dz, b + dx + dy + dz, b + dy + dz], axis=1)
    return _grid(n), conn.astype(np.uint32)


def cube_tet5(n: int):
    np1 = n + 1
    dx, dy, dz = 1, np1, np1 * np1
    b, par = _bases(n)
    odd = np.array([[dx, dy, dz, dx + dy + dz], [0, dx, dy, dz], [dx, dx + dy, dy, dx + dy + dz],
                    [dx, dz, dx + dz, dx + dy + dz], [dy, dz, dx + dy + dz, dy + dz]], dtype=np.int64)
    even = np.array([[0, dx + dy, dx + dz, dy + dz], [0, dx, dx + dy, dx + dz], [0, dx + dy, dy, dy + dz],
                     [0, dz, dx + dz, dy + dz], [dx + dy, dx + dz, dx + dy + dz, dy + dz]], dtype=np.int64)
    off = np.where((par % 2 == 1)[:, None, None], odd[None], even[None])
    conn = (b[:, None, None] + off).reshape(-1, 4)
    return _grid(n), conn.astype(np.uint32)


def cube_tet6(n: int):
    np1 = n + 1
    e = [1, np1, np1 * np1]
    b, _ = _bases(n)
    perms = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    off = np.array([[0, e[a], e[a] + e[bb], e[a] + e[bb] + e[c]] for a, bb, c in perms], dtype=np.int64)
    conn = (b[:, None, None] + off[None]).reshape(-1, 4)
    return _grid(n), conn.astype(np.uint32)


def perturb(xyz: np.ndarray, n: int, alpha: float, seed: int) -> np.ndarray:
    """Interior nodes move by U(-alpha h, alpha h) per coordinate."""
    np1 = n + 1
    h = 1.0 / n
    ids = np.arange(xyz.shape[0], dtype=np.int64)
    i, j, k = ids % np1, (ids // np1) % np1, ids // (np1 * np1)
    interior = (i > 0) & (i < n) & (j > 0) & (j < n) & (k > 0) & (k < n)
    out = xyz.copy()
    for d in range(3):
        u = uniform01(seed, ids * 3 + d)
        out[:, d] += np.where(interior, (2.0 * u - 1.0) * (alpha * h), 0.0)
    return out


def normal(seed: int, count: int) -> np.ndarray:
    idx = np.arange(count, dtype=np.int64)
    u1 = ((splitmix64(seed, 2 * idx) >> np.uint64(11)).astype(np.float64) + 1.0) * (1.0 / 9007199254740992.0)
    u2 = uniform01(seed, 2 * idx + 1)
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def lognormal(seed: int, count: int, sigma: float = 1.0) -> np.ndarray:
    return np.exp(sigma * normal(seed, count))


def boundary_nodes(n: int, planes=("x0", "x1", "y0", "y1", "z0", "z1")) -> np.ndarray:
    """Node ids of the structured cube on the given faces."""
    np1 = n + 1
    ids = np.arange(np1 ** 3, dtype=np.int64)
    i, j, k = ids % np1, (ids // np1) % np1, ids // (np1 * np1)
    m = np.zeros(ids.size, dtype=bool)
    for p in planes:
        a = {"x": i, "y": j, "z": k}[p[0]]
        m |= a == (0 if p[1] == "0" else n)
    return ids[m]
