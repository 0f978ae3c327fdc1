"""Function spaces on triangle meshes, expressed as per-triangle assembly tables.

A space is what BEAST's `assemblydata` hands the reference's GPU path
(load_parameters.jl:50-54 packs it into index/coefficient matrices [3, nt]): for every
triangle t and local shape function i in {0, 1, 2} the global function it belongs to
(`fn_index[t, i]`, -1 when the local shape carries no global function) and the
coefficient (`fn_coef[t, i]`).  As in the reference, each local shape maps to at most
one global function.

Local shapes follow BEAST's reference spaces on the chart (v1, v2, v3), with the chart
parameters (u, v) of the point u*v1 + v*v2 + (1-u-v)*v3:
  * lagrangec0d1 ("LAGRANGE"): shape i is the barycentric hat of vertex i: (u, v, 1-u-v).
  * raviartthomas ("RT", RWG): shape i is (x - v_i) / (2 A), divergence 1 / A, i.e. the
    unit-flux Raviart-Thomas function through the edge opposite vertex i.  A global RWG
    function on an interior edge is +shape on its first triangle and -shape on its second.
"""
from __future__ import annotations

import numpy as np

from .curves import CurveMesh, curve_lagrangec0d1, curve_lagrangecxd0
from .meshes import Mesh

REFSPACE_LAGRANGE_C0D1 = 0
REFSPACE_RT = 1


class Space:
    __slots__ = ("mesh", "refspace", "fn_index", "fn_coef", "nfun", "name")

    def __init__(self, mesh: Mesh, refspace: int, fn_index, fn_coef, nfun: int, name: str = ""):
        self.mesh = mesh
        self.refspace = int(refspace)
        self.fn_index = np.ascontiguousarray(fn_index, dtype=np.int32)
        self.fn_coef = np.ascontiguousarray(fn_coef, dtype=np.float64)
        self.nfun = int(nfun)
        self.name = name
        if self.fn_index.shape != (mesh.nt, 3) or self.fn_coef.shape != (mesh.nt, 3):
            raise ValueError("fn_index / fn_coef must be [nt, 3]")

    def supports(self):
        """CSR of function supports: (offsets[nfun+1], tri[], local[], coef[]) sorted by triangle."""
        t, i = np.nonzero(self.fn_index >= 0)
        f = self.fn_index[t, i]
        order = np.lexsort((t, f))
        f, t, i = f[order], t[order], i[order]
        off = np.zeros(self.nfun + 1, dtype=np.int64)
        np.add.at(off, f + 1, 1)
        off = np.cumsum(off)
        return off, t.astype(np.int32), i.astype(np.int32), self.fn_coef[t, i]

    def __repr__(self):
        kind = {0: "lagrangec0d1", 1: "raviartthomas"}[self.refspace]
        return f"Space({kind}, nfun={self.nfun}, nt={self.mesh.nt})"


def _edges(mesh: Mesh):
    """Edges numbered by first appearance (triangles in order, local edge opposite vertex i).

    Returns (edge_of[nt, 3], cells[nedges, 2], local[nedges, 2]) where edge_of[t, i] is the
    edge opposite vertex i of triangle t and cells/local list the (up to two) incident
    triangles in order of appearance (-1 when absent).
    """
    tri = mesh.triangles.astype(np.int64)
    nt = tri.shape[0]
    a = np.stack([tri[:, 1], tri[:, 2], tri[:, 0]], axis=1)  # edge opposite vertex i: (i+1, i+2)
    b = np.stack([tri[:, 2], tri[:, 0], tri[:, 1]], axis=1)
    lo = np.minimum(a, b).ravel()
    hi = np.maximum(a, b).ravel()
    key = lo * (mesh.nv + 1) + hi
    uniq, first, inv = np.unique(key, return_index=True, return_inverse=True)
    # renumber edges by first appearance
    order = np.argsort(first, kind="stable")
    rank = np.empty_like(order)
    rank[order] = np.arange(order.size)
    eid = rank[inv].reshape(nt, 3)
    ne = uniq.size
    cells = -np.ones((ne, 2), dtype=np.int64)
    local = -np.ones((ne, 2), dtype=np.int64)
    cnt = np.zeros(ne, dtype=np.int64)
    for t in range(nt):
        for i in range(3):
            e = eid[t, i]
            c = cnt[e]
            if c >= 2:
                raise ValueError("non-manifold edge shared by more than two triangles")
            cells[e, c] = t
            local[e, c] = i
            cnt[e] = c + 1
    return eid, cells, local


def raviartthomas(mesh: Mesh) -> Space:
    """RWG space: one function per interior edge (two incident triangles), +1 / -1 halves."""
    eid, cells, local = _edges(mesh)
    interior = cells[:, 1] >= 0
    fnum = -np.ones(cells.shape[0], dtype=np.int64)
    fnum[interior] = np.arange(int(interior.sum()))
    fn_index = -np.ones((mesh.nt, 3), dtype=np.int32)
    fn_coef = np.zeros((mesh.nt, 3), dtype=np.float64)
    e = np.nonzero(interior)[0]
    fn_index[cells[e, 0], local[e, 0]] = fnum[e]
    fn_coef[cells[e, 0], local[e, 0]] = 1.0
    fn_index[cells[e, 1], local[e, 1]] = fnum[e]
    fn_coef[cells[e, 1], local[e, 1]] = -1.0
    return Space(mesh, REFSPACE_RT, fn_index, fn_coef, int(interior.sum()), "raviartthomas")


def boundary_vertices(mesh: Mesh) -> np.ndarray:
    _eid, cells, _local = _edges(mesh)
    tri = mesh.triangles
    bnd = np.zeros(mesh.nv, dtype=bool)
    ebnd = np.nonzero(cells[:, 1] < 0)[0]
    for e in ebnd:
        t, i = cells[e, 0], _local[e, 0]
        bnd[tri[t, (i + 1) % 3]] = True
        bnd[tri[t, (i + 2) % 3]] = True
    return bnd


def lagrangec0d1(mesh, dirichlet: bool = True):
    """Continuous piecewise-linear Lagrange space: one function per vertex.

    With dirichlet=True (BEAST's default) vertices on the mesh boundary carry no function;
    on closed surfaces every vertex does.  On a curve mesh this is the curve space of hats.
    """
    if isinstance(mesh, CurveMesh):
        return curve_lagrangec0d1(mesh, dirichlet)
    keep = np.ones(mesh.nv, dtype=bool)
    if dirichlet:
        keep &= ~boundary_vertices(mesh)
    used = np.zeros(mesh.nv, dtype=bool)
    used[mesh.triangles.ravel()] = True
    keep &= used
    fnum = -np.ones(mesh.nv, dtype=np.int64)
    fnum[keep] = np.arange(int(keep.sum()))
    fn_index = fnum[mesh.triangles].astype(np.int32)
    fn_coef = np.where(fn_index >= 0, 1.0, 0.0)
    return Space(mesh, REFSPACE_LAGRANGE_C0D1, fn_index, fn_coef, int(keep.sum()), "lagrangec0d1")


def lagrangecxd0(mesh):
    """Piecewise constants; implemented on curve meshes (one function per segment)."""
    if isinstance(mesh, CurveMesh):
        return curve_lagrangecxd0(mesh)
    raise NotImplementedError("piecewise-constant spaces are implemented on curve meshes only")
