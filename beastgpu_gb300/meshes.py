"""Seeded synthetic triangle meshes for the assembly workloads.

A mesh is a pair (vertices float64[nv, 3], triangles int32[nt, 3]) with 0-based vertex
indices.  Triangle vertex order is the chart order used by BEAST / CompScienceMeshes:
tangents are v1 - v3 and v2 - v3 and the outward normal is (v1 - v3) x (v2 - v3).

Workloads:
  * icosphere(level)        -- midpoint subdivision of a regular icosahedron, projected
                               to the sphere; 20 * 4**level triangles.  Children of a
                               triangle are stored contiguously, so triangle and edge
                               numbering is spatially coherent (like a quadtree order).
  * ellipsoid(level, axes)  -- an icosphere scaled per axis.
  * plate(n, jitter, seed)  -- unit square, n x n cells split into 2 n^2 triangles, with
                               interior vertices jittered in-plane by U(-jitter*h, jitter*h).
  * two_plates(...)         -- the plate plus a coplanar copy shifted along x so the gap
                               between them is `gap`.
  * meshcuboid(a, b, c, h)  -- the closed surface of the box [0, a] x [0, b] x [0, c] as a
                               structured grid of step h on each face, 2 triangles per cell:
                               the mesh of the reference's only test and benchmark
                               (CompScienceMeshes' meshcuboid(1.0, 1.0, 1.0, 0.5/d),
                               test/correctness.jl:22, data/graph_data.jl:2-4).
"""
from __future__ import annotations

import numpy as np


class Mesh:
    __slots__ = ("vertices", "triangles")

    def __init__(self, vertices, triangles):
        self.vertices = np.ascontiguousarray(vertices, dtype=np.float64)
        self.triangles = np.ascontiguousarray(triangles, dtype=np.int32)
        if self.vertices.ndim != 2 or self.vertices.shape[1] != 3:
            raise ValueError("vertices must be [nv, 3]")
        if self.triangles.ndim != 2 or self.triangles.shape[1] != 3:
            raise ValueError("triangles must be [nt, 3]")

    @property
    def nv(self) -> int:
        return self.vertices.shape[0]

    @property
    def nt(self) -> int:
        return self.triangles.shape[0]

    def areas(self) -> np.ndarray:
        v = self.vertices[self.triangles]
        t1 = v[:, 0] - v[:, 2]
        t2 = v[:, 1] - v[:, 2]
        return 0.5 * np.linalg.norm(np.cross(t1, t2), axis=1)

    def __repr__(self):
        return f"Mesh(nv={self.nv}, nt={self.nt})"


def _icosahedron():
    p = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, p, 0], [1, p, 0], [-1, -p, 0], [1, -p, 0],
                  [0, -1, p], [0, 1, p], [0, -1, -p], [0, 1, -p],
                  [p, 0, -1], [p, 0, 1], [-p, 0, -1], [-p, 0, 1]], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    # chart order (v1, v2, v3) with outward normal (v1-v3) x (v2-v3)
    out = []
    for a, b, c in f:
        n = np.cross(v[a] - v[c], v[b] - v[c])
        if np.dot(n, v[a] + v[b] + v[c]) < 0:
            a, b = b, a
        out.append((a, b, c))
    return v, np.array(out, dtype=np.int64)


def icosphere(level: int, radius: float = 1.0) -> Mesh:
    """Regular icosahedron refined `level` times by midpoint subdivision, on a sphere."""
    if level < 0:
        raise ValueError("level must be >= 0")
    verts, faces = _icosahedron()
    verts = list(map(tuple, verts))
    for _ in range(level):
        cache = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            idx = cache.get(key)
            if idx is None:
                m = np.add(verts[a], verts[b]) * 0.5
                m = m / np.linalg.norm(m)
                idx = len(verts)
                verts.append(tuple(m))
                cache[key] = idx
            return idx

        nf = np.empty((faces.shape[0] * 4, 3), dtype=np.int64)
        for t, (a, b, c) in enumerate(faces):
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf[4 * t + 0] = (a, ab, ca)
            nf[4 * t + 1] = (ab, b, bc)
            nf[4 * t + 2] = (ca, bc, c)
            nf[4 * t + 3] = (ab, bc, ca)
        faces = nf
    v = np.array(verts, dtype=np.float64) * radius
    return Mesh(v, faces.astype(np.int32))


def ellipsoid(level: int, axes) -> Mesh:
    """Icosphere of the given level scaled by `axes` = (a, b, c)."""
    m = icosphere(level)
    return Mesh(m.vertices * np.asarray(axes, dtype=np.float64)[None, :], m.triangles)


def plate(n: int = 96, jitter: float = 0.3, seed: int = 1, size: float = 1.0) -> Mesh:
    """Flat square plate in z=0 meshed as an n x n grid, 2 triangles per cell.

    Interior vertices are moved in-plane by independent U(-jitter*h, jitter*h) offsets
    drawn from numpy's default_rng(seed); boundary vertices stay on the square.
    """
    h = size / n
    xs = np.arange(n + 1, dtype=np.float64) * h
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    v = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], axis=1)
    if jitter:
        rng = np.random.default_rng(seed)
        d = rng.uniform(-jitter * h, jitter * h, size=(v.shape[0], 2))
        ij = np.stack(np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij"), axis=-1).reshape(-1, 2)
        interior = (ij[:, 0] > 0) & (ij[:, 0] < n) & (ij[:, 1] > 0) & (ij[:, 1] < n)
        v[interior, :2] += d[interior]
    tris = []
    idx = lambda i, j: i * (n + 1) + j  # noqa: E731
    for i in range(n):
        for j in range(n):
            a, b, c, d_ = idx(i, j), idx(i + 1, j), idx(i + 1, j + 1), idx(i, j + 1)
            # both triangles oriented with normal +z: (v1 - v3) x (v2 - v3) . z > 0
            tris.append((b, c, a))
            tris.append((c, d_, a))
    t = np.array(tris, dtype=np.int32)
    return Mesh(v, t)


def two_plates(n: int = 96, jitter: float = 0.3, seed: int = 1, gap: float = 0.01) -> Mesh:
    """Jittered plate plus a coplanar copy shifted along x so that the gap is `gap`."""
    p = plate(n, jitter, seed)
    q_v = p.vertices.copy()
    q_v[:, 0] += 1.0 + gap
    v = np.concatenate([p.vertices, q_v])
    t = np.concatenate([p.triangles, p.triangles + p.nv])
    return Mesh(v, t)


def merge(meshes) -> Mesh:
    vs, ts, off = [], [], 0
    for m in meshes:
        vs.append(m.vertices)
        ts.append(m.triangles + off)
        off += m.nv
    return Mesh(np.concatenate(vs), np.concatenate(ts))


def ellipsoid_batch(count: int = 64, seed: int = 2, levels=(1, 4), axis_range=(0.5, 2.0), k_range=(1.0, 10.0)):
    """Seeded batch of ellipsoids: level ~ U{levels}, axes ~ U[axis_range]^3, k ~ U[k_range].

    Returns a list of (mesh, wavenumber).
    """
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        lvl = int(rng.integers(levels[0], levels[1] + 1))
        axes = rng.uniform(axis_range[0], axis_range[1], size=3)
        k = float(rng.uniform(k_range[0], k_range[1]))
        out.append((ellipsoid(lvl, axes), k))
    return out


def meshcuboid(width: float, height: float, length: float, delta: float) -> Mesh:
    """Closed surface of the box [0, width] x [0, height] x [0, length], each face a structured
    grid of step `delta` (the face extents must be multiples of it), each cell split into two
    triangles along the same diagonal, normals outward.

    The counts are those of CompScienceMeshes' meshcuboid that the reference tests and times
    (test/correctness.jl:22; data/graph_data.jl:2-4): for the unit cube and delta = 0.5/d,
    12 (2d)^2 triangles and 6 (2d)^2 + 2 vertices.  Vertex and face numbering are this
    generator's: faces are taken in the order z = 0, z = length, y = 0, y = height, x = 0,
    x = width; a face's vertices are numbered row by row, each lattice point once (the first
    face that reaches it), and a face's cells in the same order, two triangles per cell.
    """
    dims = (float(width), float(height), float(length))
    h = float(delta)
    if h <= 0 or min(dims) <= 0:
        raise ValueError("extents and delta must be positive")
    n = [int(round(d / h)) for d in dims]
    for d, k in zip(dims, n):
        if k < 1 or abs(k * h - d) > 1e-9 * max(1.0, d):
            raise ValueError("each extent must be a positive multiple of delta")
    nx, ny, nz = n
    # (fixed axis, its lattice value, u axis, v axis): u x v is the outward normal
    faces = [(2, 0, 1, 0), (2, nz, 0, 1), (1, 0, 0, 2), (1, ny, 2, 0), (0, 0, 2, 1), (0, nx, 1, 2)]
    index = {}
    verts = []
    tris = []
    for fixed, value, ua, va in faces:
        nu, nv = n[ua], n[va]
        ids = np.empty((nu + 1, nv + 1), dtype=np.int64)
        for i in range(nu + 1):
            for j in range(nv + 1):
                key = [0, 0, 0]
                key[fixed], key[ua], key[va] = value, i, j
                key = tuple(key)
                k = index.get(key)
                if k is None:
                    k = len(verts)
                    index[key] = k
                    verts.append(key)
                ids[i, j] = k
        for i in range(nu):
            for j in range(nv):
                p00, p10, p11, p01 = ids[i, j], ids[i + 1, j], ids[i + 1, j + 1], ids[i, j + 1]
                tris.append((p00, p10, p11))  # counter-clockwise about u x v: chart normal outward
                tris.append((p00, p11, p01))
    lat = np.array(verts, dtype=np.float64)
    v = lat * np.array([dims[0] / nx, dims[1] / ny, dims[2] / nz])[None, :]
    return Mesh(v, np.array(tris, dtype=np.int32))
