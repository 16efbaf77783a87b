"""Ray-set generators shared by the tests (numpy, float32)."""
from __future__ import annotations

import numpy as np

from kiraray_gb300.scenes import bounce_rays, pinhole_rays  # noqa: F401  (ray sets)


def random_soup(n: int, seed: int, size: float = 0.2) -> np.ndarray:
    rng = np.random.default_rng(seed)
    c = rng.random((n, 1, 3)) * 2 - 1
    return (c + (rng.random((n, 3, 3)) - 0.5) * size).reshape(n, 9).astype(np.float32)


def random_rays(n: int, seed: int, box: float = 1.5) -> np.ndarray:
    rng = np.random.default_rng(seed)
    o = (rng.random((n, 3)) * 2 - 1) * box
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    out = np.zeros((n, 8), np.float32)
    out[:, :3] = o
    out[:, 4:7] = d
    out[:, 7] = np.inf
    return out


def grid_mesh(n: int) -> np.ndarray:
    """n x n unit quads in the z=0 plane as 2n^2 triangles (shared edges)."""
    tris = []
    for j in range(n):
        for i in range(n):
            a, b, c, d = (i, j, 0), (i + 1, j, 0), (i + 1, j + 1, 0), (i, j + 1, 0)
            tris.append([*a, *b, *c])
            tris.append([*a, *c, *d])
    return (np.array(tris, np.float32) / n).astype(np.float32)


def vertex_edge_rays(n: int, seed: int) -> np.ndarray:
    """Rays through the shared vertices and edge midpoints of grid_mesh(n),
    from random origins above the plane."""
    rng = np.random.default_rng(seed)
    pts = []
    for j in range(n + 1):
        for i in range(n + 1):
            pts.append((i / n, j / n))
            if i < n:
                pts.append(((i + 0.5) / n, j / n))
            if j < n:
                pts.append((i / n, (j + 0.5) / n))
            if i < n and j < n:
                pts.append(((i + 0.5) / n, (j + 0.5) / n))   # on the diagonal
    pts = np.array(pts, np.float64)
    # keep strictly interior targets so that every ray must hit
    inner = (pts[:, 0] > 0) & (pts[:, 0] < 1) & (pts[:, 1] > 0) & (pts[:, 1] < 1)
    pts = pts[inner]
    o = np.concatenate([rng.random((pts.shape[0], 2)) * 2 - 0.5,
                        rng.random((pts.shape[0], 1)) * 2 + 0.5], 1)
    tgt = np.concatenate([pts, np.zeros((pts.shape[0], 1))], 1)
    d = tgt - o
    out = np.zeros((pts.shape[0], 8), np.float32)
    out[:, :3] = o
    out[:, 4:7] = d
    out[:, 7] = np.inf
    return out


def furnace_sphere(le=(1.0, 2.0, 0.5), albedo: float = 0.5, max_depth: int = 40, size: int = 24):
    """A closed icosphere seen from its centre, emitting `le` and reflecting
    with Lambertian `albedo` on its inside (flat normals pointing inward):
    its radiance is le (1 - albedo^(max_depth+1)) / (1 - albedo) everywhere."""
    from kiraray_gb300 import _lib as L
    from kiraray_gb300 import scenes

    sph = scenes.icosphere(2)
    tri = sph.positions[sph.indices[:, [0, 2, 1]]]          # reversed winding: normals point inward
    n = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    pos = tri.reshape(-1, 3).astype(np.float32)
    nrm = np.repeat(n, 3, axis=0).astype(np.float32)
    idx = np.arange(pos.shape[0], dtype=np.uint32).reshape(-1, 3)
    mesh = scenes.Mesh(pos, nrm, idx, material=0, emission=tuple(float(x) for x in le))
    mats = [scenes.Material(type=L.MATERIAL_DIFFUSE, diffuse=(albedo, albedo, albedo))]
    cam = scenes._camera((0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 60.0, size, size)
    sc = scenes.Scene([mesh], [(0, scenes.IDENTITY)], mats, cam, size, size, max_depth=max_depth,
                      name="furnace")
    want = np.asarray(le, np.float64) * (1 - albedo ** (max_depth + 1)) / (1 - albedo)
    return sc, want

