"""Seeded synthetic tetrahedral meshes and scalar fields.

The reference measures on VTK datasets that are not available here, so every
workload is a seeded synthetic stand-in with the shapes the workloads name:

* Kuhn (Freudenthal) tetrahedralisation of an ``n x n x n`` cube grid: six
  tets per cube, all sharing the cube's main diagonal.  Vertex ``(i, j, k)``
  has id ``i + (n+1) * (j + (n+1) * k)``; cells are emitted cube by cube in
  the same x-fastest order, so the cell order is spatially coherent the way
  meshes written by mesh generators are.
* Centre coning: a seeded fraction of cubes is replaced by a centre vertex
  joined to the cube's 12 boundary triangles.  Each cube face is split along
  the diagonal from its lowest to its highest corner, which is the split the
  neighbouring Kuhn cubes use, so the mesh stays conforming.
* Vertex ids randomly permuted (destroys id locality) and the 4 slots of
  every tet shuffled.
* Fields: a sum of isotropic Gaussians plus noise, or a product of sines
  plus noise, evaluated on the vertex coordinates in the unit cube.

Everything is numpy and deterministic in its 64-bit seed.
"""
from __future__ import annotations

import dataclasses
import itertools

import numpy as np

__all__ = [
    "Mesh",
    "kuhn_mesh",
    "gaussian_mixture_field",
    "sine_field",
    "workload_small",
    "workload_irregular",
    "workload_large",
    "workload_batch",
    "tiny_meshes",
]

_PERMS = list(itertools.permutations(range(3)))


@dataclasses.dataclass
class Mesh:
    tv: np.ndarray        # int32 [n_cells, 4]
    n_verts: int
    coords: np.ndarray    # float32 [n_verts, 3]
    field: np.ndarray | None = None   # float32 [n_verts]
    name: str = ""

    @property
    def n_cells(self) -> int:
        return int(self.tv.shape[0])


def _corner_offsets(n1: int) -> dict:
    return {(dx, dy, dz): dx + n1 * (dy + n1 * dz)
            for dx in (0, 1) for dy in (0, 1) for dz in (0, 1)}


def _kuhn_local() -> np.ndarray:
    """The 6 Kuhn tets of a unit cube as corner triples (6, 4, 3)."""
    out = []
    for p in _PERMS:
        v = [0, 0, 0]
        path = [tuple(v)]
        for a in p:
            v[a] = 1
            path.append(tuple(v))
        out.append(path)
    return np.array(out, dtype=np.int64)


def _cone_local() -> np.ndarray:
    """The 12 boundary triangles of a unit cube, split lowest-to-highest
    corner on every face, as corner triples (12, 3, 3)."""
    tris = []
    for a in range(3):
        b, c = [x for x in range(3) if x != a]
        for t in (0, 1):
            base = [0, 0, 0]
            base[a] = t
            eb = list(base); eb[b] = 1
            ec = list(base); ec[c] = 1
            top = list(base); top[b] = 1; top[c] = 1
            tris.append([tuple(base), tuple(eb), tuple(top)])
            tris.append([tuple(base), tuple(ec), tuple(top)])
    return np.array(tris, dtype=np.int64)


def kuhn_mesh(n, cone_fraction: float = 0.0, seed: int = 0,
              permute: bool = True, shuffle_slots: bool = True,
              jitter: float = 0.0) -> Mesh:
    """Kuhn tetrahedralisation of an ``nx x ny x nz`` cube grid (``n`` an int
    or a 3-tuple), with a seeded fraction of cubes centre-coned."""
    if np.isscalar(n):
        nx = ny = nz = int(n)
    else:
        nx, ny, nz = (int(x) for x in n)
    rng = np.random.default_rng(seed)
    gx, gy, gz = nx + 1, ny + 1, nz + 1
    n_grid = gx * gy * gz
    n_cubes = nx * ny * nz
    n_coned = int(round(cone_fraction * n_cubes))
    coned = np.zeros(n_cubes, dtype=bool)
    if n_coned:
        coned[rng.choice(n_cubes, size=n_coned, replace=False)] = True

    q = np.arange(n_cubes, dtype=np.int64)
    ci, cj, ck = q % nx, (q // nx) % ny, q // (nx * ny)
    base = ci + gx * (cj + gy * ck)

    def corner_id(loc):  # loc (..., 3) of 0/1 offsets
        return loc[..., 0] + gx * (loc[..., 1] + gy * loc[..., 2])

    kl = corner_id(_kuhn_local())            # (6, 4)
    cl = corner_id(_cone_local())            # (12, 3)
    per_cube = np.where(coned, 12, 6)
    start = np.zeros(n_cubes + 1, dtype=np.int64)
    np.cumsum(per_cube, out=start[1:])
    n_cells = int(start[-1])
    tv = np.empty((n_cells, 4), dtype=np.int64)

    plain = ~coned
    pb = base[plain]
    pos = start[:-1][plain][:, None] + np.arange(6)[None, :]
    tv[pos.reshape(-1)] = (pb[:, None, None] + kl[None, :, :]).reshape(-1, 4)
    if n_coned:
        cb = base[coned]
        centre = n_grid + np.arange(n_coned, dtype=np.int64)
        pos = start[:-1][coned][:, None] + np.arange(12)[None, :]
        tri = cb[:, None, None] + cl[None, :, :]                    # (m, 12, 3)
        cells = np.concatenate([np.broadcast_to(centre[:, None, None], (n_coned, 12, 1)), tri], axis=2)
        tv[pos.reshape(-1)] = cells.reshape(-1, 4)

    n_verts = n_grid + n_coned
    coords = np.empty((n_verts, 3), dtype=np.float64)
    g = np.arange(n_grid, dtype=np.int64)
    coords[:n_grid, 0] = (g % gx) / nx
    coords[:n_grid, 1] = ((g // gx) % gy) / ny
    coords[:n_grid, 2] = (g // (gx * gy)) / nz
    if jitter:
        coords[:n_grid] += rng.uniform(-jitter, jitter, size=(n_grid, 3)) / np.array([nx, ny, nz])
    if n_coned:
        cq = q[coned]
        coords[n_grid:, 0] = (ci[cq] + 0.5) / nx
        coords[n_grid:, 1] = (cj[cq] + 0.5) / ny
        coords[n_grid:, 2] = (ck[cq] + 0.5) / nz

    if permute:
        perm = rng.permutation(n_verts)
        tv = perm[tv]
        c2 = np.empty_like(coords)
        c2[perm] = coords
        coords = c2
    if shuffle_slots:
        order = np.argsort(rng.random((n_cells, 4)), axis=1)
        tv = np.take_along_axis(tv, order, axis=1)
    return Mesh(tv=np.ascontiguousarray(tv, dtype=np.int32), n_verts=int(n_verts),
                coords=coords.astype(np.float32))


def gaussian_mixture_field(coords: np.ndarray, n_gauss: int = 32, seed: int = 0,
                           sigma=(0.02, 0.2), noise: float = 1e-3) -> np.ndarray:
    """Sum of isotropic Gaussians (centres uniform in the unit cube, widths
    uniform in ``sigma``, amplitudes uniform in +-[0.5, 1.5]) plus N(0, noise)."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.0, 1.0, size=(n_gauss, 3))
    s = rng.uniform(sigma[0], sigma[1], size=n_gauss)
    a = rng.uniform(0.5, 1.5, size=n_gauss) * rng.choice([-1.0, 1.0], size=n_gauss)
    x = coords.astype(np.float64)
    out = np.zeros(x.shape[0], dtype=np.float64)
    for lo in range(0, x.shape[0], 1 << 20):
        xs = x[lo:lo + (1 << 20)]
        d2 = ((xs[:, None, :] - c[None, :, :]) ** 2).sum(-1)
        out[lo:lo + xs.shape[0]] = (a[None, :] * np.exp(-d2 / (2.0 * s[None, :] ** 2))).sum(-1)
    out += rng.normal(0.0, noise, size=out.shape)
    return out.astype(np.float32)


def sine_field(coords: np.ndarray, seed: int = 0, noise: float = 1e-4) -> np.ndarray:
    """sin(a x) sin(b y) sin(c z) with a, b, c uniform in [4 pi, 12 pi], plus
    N(0, noise)."""
    rng = np.random.default_rng(seed)
    a, b, c = rng.uniform(4 * np.pi, 12 * np.pi, size=3)
    x = coords.astype(np.float64)
    out = np.sin(a * x[:, 0]) * np.sin(b * x[:, 1]) * np.sin(c * x[:, 2])
    out += rng.normal(0.0, noise, size=out.shape)
    return out.astype(np.float32)


# --------------------------------------------------------------------------
# The named workloads (seeds are fixed and recorded with the measurements).
# --------------------------------------------------------------------------

SEEDS = {"small": 1234, "irregular": 2025, "large": 4242, "batch": 777}


def workload_small(seed: int = SEEDS["small"]) -> Mesh:
    """Kuhn 16^3 (4,913 vertices, 24,576 tets), ids permuted, slots shuffled,
    +-0.1-cell coordinate jitter."""
    m = kuhn_mesh(16, 0.0, seed=seed, jitter=0.1)
    m.field = gaussian_mixture_field(m.coords, seed=seed + 1)
    m.name = "kuhn16"
    return m


def workload_irregular(seed: int = SEEDS["irregular"]) -> Mesh:
    """Kuhn 64^3 with 20% of cubes centre-coned (1,887,438 tets, 327,054
    vertices), ids permuted; field = 32 Gaussians + N(0, 1e-3)."""
    m = kuhn_mesh(64, 0.2, seed=seed)
    m.field = gaussian_mixture_field(m.coords, n_gauss=32, seed=seed + 1, noise=1e-3)
    m.name = "kuhn64_coned20"
    return m


def workload_large(seed: int = SEEDS["large"]) -> Mesh:
    """Kuhn 128^3 (2,146,689 vertices, 12,582,912 tets), ids permuted; field =
    sin(ax) sin(by) sin(cz) + N(0, 1e-4)."""
    m = kuhn_mesh(128, 0.0, seed=seed)
    m.field = sine_field(m.coords, seed=seed + 1, noise=1e-4)
    m.name = "kuhn128"
    return m


def _dims_for(target_tets: int, rng) -> tuple:
    """Grid dims whose Kuhn tet count 6*nx*ny*nz is near the target."""
    n = max(1, round((target_tets / 6.0) ** (1.0 / 3.0)))
    dims = [n, n, n]
    # nudge one axis to land closer to the target
    best = dims
    for d in range(3):
        for delta in (-1, 0, 1):
            cand = list(dims)
            cand[d] = max(1, cand[d] + delta)
            if abs(6 * np.prod(cand) - target_tets) < abs(6 * np.prod(best) - target_tets):
                best = cand
    return tuple(int(x) for x in best)


def workload_batch(n_meshes: int = 512, lo: int = 2000, hi: int = 400000,
                   seed: int = SEEDS["batch"]) -> list:
    """Meshes of uneven size: tet counts log-uniform in [lo, hi], each a Kuhn
    grid of matching dims with a seeded 0-30% of cubes coned, ids permuted,
    each with its own Gaussian-mixture field."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_meshes):
        target = float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        dims = _dims_for(target, rng)
        frac = float(rng.uniform(0.0, 0.3))
        s = int(rng.integers(0, 2**62))
        m = kuhn_mesh(dims, frac, seed=s)
        m.field = gaussian_mixture_field(m.coords, n_gauss=32, seed=s + 1, noise=1e-3)
        m.name = f"batch{i}"
        out.append(m)
    return out


def tiny_meshes() -> dict:
    """Hand-checkable meshes with their known counts (V, E, F, T)."""
    two = Mesh(tv=np.array([[0, 1, 2, 3], [1, 2, 3, 4]], dtype=np.int32), n_verts=5,
               coords=np.zeros((5, 3), np.float32), name="two_tets")
    one_cube = kuhn_mesh(1, 0.0, seed=0, permute=False, shuffle_slots=False)
    one_cube.name = "kuhn_cube"
    coned_cube = kuhn_mesh(1, 1.0, seed=0, permute=False, shuffle_slots=False)
    coned_cube.name = "coned_cube"
    return {
        "two_tets": (two, (5, 9, 7, 2)),
        "kuhn_cube": (one_cube, (8, 19, 18, 6)),
        "coned_cube": (coned_cube, (9, 26, 30, 12)),
    }
