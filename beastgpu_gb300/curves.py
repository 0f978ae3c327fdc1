"""Curves in the plane: segment meshes, function spaces on them and BEAST's Helmholtz2D operators.

The 2-D path of the library (bgb_assemble_curve) assembles the Galerkin matrices of the
Helmholtz operators on polygonal curves, the family of the reference's 2-D hypersingular
prototype (old_code/doubleQuadRule_2d_gpu.jl).

Mesh: vertices float64[nv, 2], segments int32[ns, 2] = (v0, v1); the chart of a segment is
x(s) = (1 - s) v0 + s v1, its normal n = (d_y, -d_x) / |d| with d = v1 - v0 (outward on a
counter-clockwise closed curve).

Spaces (per-segment assembly tables fn_index / fn_coef of shape [ns, 2], as for triangles):
  * lagrangec0d1: one hat per vertex (local shapes 1 - s at v0 and s at v1); on an open curve
    the two end vertices carry no function when dirichlet=True.
  * lagrangecxd0: one constant per segment (local shape 1; column 1 of the tables unused).

Operators (kernel G(R) = -(i/4) H0^(2)(kR), or -(1/2 pi) ln R for k = 0):
  single layer alpha <f, G g>; double layer alpha <f, dG/dn_y g>; its transpose alpha
  <f, dG/dn_x g>; hypersingular <G, alpha (n_x.n_y) f g + beta f' g'> with BEAST's alpha =
  -k^2, beta = 1 (the prototype's integrand, doubleQuadRule_2d_gpu.jl:88-97).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

REFSPACE2D_LAGRANGE_C0D1 = 0
REFSPACE2D_LAGRANGE_CXD0 = 1

OP2D_SL, OP2D_DL, OP2D_DLT, OP2D_HS = 0, 1, 2, 3
_NAMES = {OP2D_SL: "Helmholtz2D.singlelayer", OP2D_DL: "Helmholtz2D.doublelayer",
          OP2D_DLT: "Helmholtz2D.doublelayer_transposed", OP2D_HS: "Helmholtz2D.hypersingular"}

CLASS2D_FAR, CLASS2D_CV, CLASS2D_CF, CLASS2D_NEAR = 0, 1, 3, 4


class CurveMesh:
    __slots__ = ("vertices", "segments")

    def __init__(self, vertices, segments):
        self.vertices = np.ascontiguousarray(vertices, dtype=np.float64)
        self.segments = np.ascontiguousarray(segments, dtype=np.int32)
        if self.vertices.ndim != 2 or self.vertices.shape[1] != 2:
            raise ValueError("vertices must be [nv, 2]")
        if self.segments.ndim != 2 or self.segments.shape[1] != 2:
            raise ValueError("segments must be [ns, 2]")

    @property
    def nv(self) -> int:
        return self.vertices.shape[0]

    @property
    def ns(self) -> int:
        return self.segments.shape[0]

    def lengths(self) -> np.ndarray:
        d = self.vertices[self.segments[:, 1]] - self.vertices[self.segments[:, 0]]
        return np.linalg.norm(d, axis=1)

    def __repr__(self):
        return f"CurveMesh(nv={self.nv}, ns={self.ns})"


def circle(n: int, radius: float = 1.0, center=(0.0, 0.0)) -> CurveMesh:
    """Regular n-gon inscribed in a circle, counter-clockwise (BEAST meshcircle)."""
    return ellipse(n, radius, radius, center)


def ellipse(n: int, a: float = 1.0, b: float = 0.5, center=(0.0, 0.0), jitter: float = 0.0, seed: int = 0) -> CurveMesh:
    """Closed polygon with n vertices on an ellipse (semi-axes a, b), counter-clockwise; the
    vertex angles are jittered by U(-jitter, jitter) times the angular step (seeded)."""
    t = 2 * np.pi * np.arange(n) / n
    if jitter:
        t = t + np.random.default_rng(seed).uniform(-jitter, jitter, n) * (2 * np.pi / n)
    v = np.stack([center[0] + a * np.cos(t), center[1] + b * np.sin(t)], axis=1)
    seg = np.stack([np.arange(n), (np.arange(n) + 1) % n], axis=1)
    return CurveMesh(v, seg)


def arc(n: int, radius: float = 1.0, angle: float = np.pi, center=(0.0, 0.0)) -> CurveMesh:
    """Open circular arc of `angle` radians with n segments (n + 1 vertices)."""
    t = angle * np.arange(n + 1) / n
    v = np.stack([center[0] + radius * np.cos(t), center[1] + radius * np.sin(t)], axis=1)
    seg = np.stack([np.arange(n), np.arange(n) + 1], axis=1)
    return CurveMesh(v, seg)


def union(*meshes: CurveMesh) -> CurveMesh:
    """Disjoint union (vertex indices of later meshes shifted)."""
    vs, ss, off = [], [], 0
    for m in meshes:
        vs.append(m.vertices)
        ss.append(m.segments + off)
        off += m.nv
    return CurveMesh(np.concatenate(vs), np.concatenate(ss))


class CurveSpace:
    __slots__ = ("mesh", "refspace", "fn_index", "fn_coef", "nfun", "name")

    def __init__(self, mesh: CurveMesh, refspace: int, fn_index, fn_coef, nfun: int, name: str = ""):
        self.mesh = mesh
        self.refspace = int(refspace)
        self.fn_index = np.ascontiguousarray(fn_index, dtype=np.int32)
        self.fn_coef = np.ascontiguousarray(fn_coef, dtype=np.float64)
        self.nfun = int(nfun)
        self.name = name
        if self.fn_index.shape != (mesh.ns, 2) or self.fn_coef.shape != (mesh.ns, 2):
            raise ValueError("fn_index / fn_coef must be [ns, 2]")

    def __repr__(self):
        return f"CurveSpace({self.name}, nfun={self.nfun}, ns={self.mesh.ns})"


def curve_lagrangec0d1(mesh: CurveMesh, dirichlet: bool = True) -> CurveSpace:
    """Continuous piecewise-linear hats, one per vertex; vertices used by one segment only (the
    ends of an open curve) carry no function when dirichlet=True."""
    count = np.bincount(mesh.segments.ravel(), minlength=mesh.nv)
    keep = count > 0
    if dirichlet:
        keep &= count != 1
    fnum = -np.ones(mesh.nv, dtype=np.int64)
    fnum[keep] = np.arange(int(keep.sum()))
    fn_index = fnum[mesh.segments].astype(np.int32)
    fn_coef = np.where(fn_index >= 0, 1.0, 0.0)
    return CurveSpace(mesh, REFSPACE2D_LAGRANGE_C0D1, fn_index, fn_coef, int(keep.sum()), "lagrangec0d1")


def curve_lagrangecxd0(mesh: CurveMesh) -> CurveSpace:
    """Piecewise constants, one per segment."""
    fn_index = -np.ones((mesh.ns, 2), dtype=np.int32)
    fn_index[:, 0] = np.arange(mesh.ns)
    fn_coef = np.zeros((mesh.ns, 2))
    fn_coef[:, 0] = 1.0
    return CurveSpace(mesh, REFSPACE2D_LAGRANGE_CXD0, fn_index, fn_coef, mesh.ns, "lagrangecxd0")


@dataclass(frozen=True)
class Operator2D:
    kind: int
    wavenumber: float
    alpha: complex = 1.0
    beta: complex = 0.0

    def __repr__(self):
        return f"{_NAMES[self.kind]}(wavenumber={self.wavenumber}, alpha={self.alpha}, beta={self.beta})"


class Helmholtz2D:
    """Constructors of BEAST's Helmholtz2D operators (real wave number k >= 0)."""

    @staticmethod
    def singlelayer(*, wavenumber, alpha=None) -> Operator2D:
        return Operator2D(OP2D_SL, float(wavenumber), complex(1.0 if alpha is None else alpha))

    @staticmethod
    def doublelayer(*, wavenumber, alpha=None) -> Operator2D:
        return Operator2D(OP2D_DL, float(wavenumber), complex(1.0 if alpha is None else alpha))

    @staticmethod
    def doublelayer_transposed(*, wavenumber, alpha=None) -> Operator2D:
        return Operator2D(OP2D_DLT, float(wavenumber), complex(1.0 if alpha is None else alpha))

    @staticmethod
    def hypersingular(*, wavenumber, alpha=None, beta=None) -> Operator2D:
        """<G, alpha (n_x.n_y) f g + beta f' g'>; alpha defaults to -k^2, beta to 1."""
        k = float(wavenumber)
        return Operator2D(OP2D_HS, k, complex(-k * k if alpha is None else alpha),
                          complex(1.0 if beta is None else beta))


@dataclass(frozen=True)
class QuadStrat2D:
    """Rules of the 2-D path: Gauss-Legendre points per segment for far pairs (test, trial) and
    near pairs, and the order of the graded rules for pairs that share vertices."""
    far_test: int = 4
    far_trial: int = 4
    near: int = 12
    singular: int = 10


def defaultquadstrat2d(op=None, test=None, trial=None) -> QuadStrat2D:
    return QuadStrat2D()
