"""ctypes front end of the FP64 CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use this module,
and only as the checker or the timed CPU restatement; the product path never calls it.
Parity against BEAST itself is unpinned (see bem_oracle.h).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "libbem_oracle.so")

OP_HELMHOLTZ3D_SL = 0
OP_MAXWELL3D_SL = 1
OP_MAXWELL3D_DL = 2
CLASS_FAR, CLASS_CV, CLASS_CE, CLASS_CF, CLASS_NEAR = range(5)


class _Op(C.Structure):
    _fields_ = [("kind", C.c_int32), ("alpha", C.c_double * 2), ("beta", C.c_double * 2), ("gamma", C.c_double * 2)]


class _Space(C.Structure):
    _fields_ = [("refspace", C.c_int32), ("nv", C.c_int32), ("nt", C.c_int32), ("nfun", C.c_int32),
                ("vertices", C.c_void_p), ("triangles", C.c_void_p), ("fn_index", C.c_void_p),
                ("fn_coef", C.c_void_p)]


class _QS(C.Structure):
    _fields_ = [("far_test", C.c_int32), ("far_trial", C.c_int32), ("near_test", C.c_int32),
                ("near_trial", C.c_int32), ("ss_cf", C.c_int32), ("ss_ce", C.c_int32), ("ss_cv", C.c_int32)]


class _Op2(C.Structure):
    _fields_ = [("kind", C.c_int32), ("wavenumber", C.c_double), ("alpha", C.c_double * 2), ("beta", C.c_double * 2)]


class _Space2(C.Structure):
    _fields_ = [("refspace", C.c_int32), ("nv", C.c_int32), ("ns", C.c_int32), ("nfun", C.c_int32),
                ("vertices", C.c_void_p), ("segments", C.c_void_p), ("fn_index", C.c_void_p),
                ("fn_coef", C.c_void_p)]


class _QS2(C.Structure):
    _fields_ = [("far_test", C.c_int32), ("far_trial", C.c_int32), ("near", C.c_int32), ("singular", C.c_int32)]


def build(force: bool = False) -> str:
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < max(
            os.path.getmtime(os.path.join(_HERE, f))
            for f in ("bem_oracle.c", "bem_oracle.h", "trirules.h", "bem2d_oracle.c", "bem2d_oracle.h", "Makefile")):
        subprocess.check_call(["make", "-s", "-C", _HERE], stdout=subprocess.DEVNULL)
    return _LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB)
        L.orc_classify_block.argtypes = [C.POINTER(_Space), C.POINTER(_Space), C.c_double, C.c_int32, C.c_int32,
                                         C.c_int32, C.c_int32, C.c_void_p]
        L.orc_local_matrices.argtypes = [C.POINTER(_Op), C.POINTER(_Space), C.POINTER(_Space), C.POINTER(_QS),
                                         C.c_int64, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]
        L.orc_assemble_rows.argtypes = [C.POINTER(_Op), C.POINTER(_Space), C.POINTER(_Space), C.POINTER(_QS),
                                        C.c_int64, C.c_void_p, C.c_void_p, C.c_int32]
        L.orc_gauss_legendre01.argtypes = [C.c_int32, C.c_void_p, C.c_void_p]
        L.orc_triangle_area.argtypes = [C.POINTER(_Space), C.c_int32]
        L.orc_triangle_area.restype = C.c_double
        L.orc_max_threads.restype = C.c_int
        L.orc2_green.argtypes = [C.c_double, C.c_double, C.c_void_p]
        L.orc2_graded01.argtypes = [C.c_int32, C.c_void_p, C.c_void_p]
        L.orc2_classify_block.argtypes = [C.POINTER(_Space2), C.POINTER(_Space2), C.c_double, C.c_int32, C.c_int32,
                                          C.c_int32, C.c_int32, C.c_void_p]
        L.orc2_local_matrices.argtypes = [C.POINTER(_Op2), C.POINTER(_Space2), C.POINTER(_Space2), C.POINTER(_QS2),
                                          C.c_int64, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]
        L.orc2_assemble_rows.argtypes = [C.POINTER(_Op2), C.POINTER(_Space2), C.POINTER(_Space2), C.POINTER(_QS2),
                                         C.c_int64, C.c_void_p, C.c_void_p, C.c_int32]
        _lib = L
    return _lib


class _Keep:
    """Holds the numpy buffers a ctypes struct points into."""

    def __init__(self):
        self.refs = []

    def arr(self, a, dtype):
        a = np.ascontiguousarray(a, dtype=dtype)
        self.refs.append(a)
        return a.ctypes.data


def _space(space, keep):
    m = space.mesh
    return _Space(space.refspace, m.nv, m.nt, space.nfun, keep.arr(m.vertices, np.float64),
                  keep.arr(m.triangles, np.int32), keep.arr(space.fn_index, np.int32),
                  keep.arr(space.fn_coef, np.float64))


def _op(op):
    a, b, g = complex(op.alpha), complex(op.beta), complex(op.gamma)
    return _Op(op.kind, (C.c_double * 2)(a.real, a.imag), (C.c_double * 2)(b.real, b.imag),
               (C.c_double * 2)(g.real, g.imag))


def _qs(qs):
    return _QS(qs.far_test, qs.far_trial, qs.near_test, qs.near_trial, qs.ss_cf, qs.ss_ce, qs.ss_cv)


def classify_block(test, trial, k2, t0=0, t1=None, s0=0, s1=None):
    t1 = test.mesh.nt if t1 is None else t1
    s1 = trial.mesh.nt if s1 is None else s1
    keep = _Keep()
    out = np.empty((t1 - t0, s1 - s0), dtype=np.int8)
    rc = lib().orc_classify_block(C.byref(_space(test, keep)), C.byref(_space(trial, keep)), float(k2),
                                  t0, t1, s0, s1, out.ctypes.data)
    if rc:
        raise RuntimeError(f"orc_classify_block failed ({rc})")
    return out


def local_matrices(op, test, trial, qs, tau, sigma, force_class=-1):
    keep = _Keep()
    tau = np.ascontiguousarray(tau, dtype=np.int32)
    sigma = np.ascontiguousarray(sigma, dtype=np.int32)
    out = np.empty((tau.size, 3, 3, 2), dtype=np.float64)
    cls = np.empty(tau.size, dtype=np.int8)
    rc = lib().orc_local_matrices(C.byref(_op(op)), C.byref(_space(test, keep)), C.byref(_space(trial, keep)),
                                  C.byref(_qs(qs)), tau.size, tau.ctypes.data, sigma.ctypes.data,
                                  int(force_class), out.ctypes.data, cls.ctypes.data)
    if rc:
        raise RuntimeError(f"orc_local_matrices failed ({rc})")
    return out[..., 0] + 1j * out[..., 1], cls


def assemble_rows(op, test, trial, qs, rows, nthreads=0):
    keep = _Keep()
    rows = np.ascontiguousarray(rows, dtype=np.int32)
    out = np.empty((rows.size, trial.nfun, 2), dtype=np.float64)
    rc = lib().orc_assemble_rows(C.byref(_op(op)), C.byref(_space(test, keep)), C.byref(_space(trial, keep)),
                                 C.byref(_qs(qs)), rows.size, rows.ctypes.data, out.ctypes.data, int(nthreads))
    if rc:
        raise RuntimeError(f"orc_assemble_rows failed ({rc})")
    return out[..., 0] + 1j * out[..., 1]


def assemble(op, test, trial, qs, nthreads=0):
    return assemble_rows(op, test, trial, qs, np.arange(test.nfun), nthreads)


def gauss_legendre01(n):
    x = np.empty(n)
    w = np.empty(n)
    if lib().orc_gauss_legendre01(n, x.ctypes.data, w.ctypes.data):
        raise ValueError("n out of range")
    return x, w


def max_threads():
    return lib().orc_max_threads()


# ---- curves (bem2d_oracle.h) -----------------------------------------------------------------


def _space2(space, keep):
    m = space.mesh
    return _Space2(space.refspace, m.nv, m.ns, space.nfun, keep.arr(m.vertices, np.float64),
                   keep.arr(m.segments, np.int32), keep.arr(space.fn_index, np.int32),
                   keep.arr(space.fn_coef, np.float64))


def _op2(op):
    a, b = complex(op.alpha), complex(op.beta)
    return _Op2(op.kind, float(op.wavenumber), (C.c_double * 2)(a.real, a.imag), (C.c_double * 2)(b.real, b.imag))


def _qs2(qs):
    return _QS2(qs.far_test, qs.far_trial, qs.near, qs.singular)


def green2d(k, R):
    """(G, g1) of the 2-D kernel at distance R: G = -(i/4) H0^(2)(kR), grad_x G = (x - y) g1."""
    out = np.empty(4)
    if lib().orc2_green(float(k), float(R), out.ctypes.data):
        raise ValueError("R must be > 0 and k >= 0")
    return out[0] + 1j * out[1], out[2] + 1j * out[3]


def graded01(n):
    x = np.empty((3 * n + 1) * n)
    w = np.empty((3 * n + 1) * n)
    if lib().orc2_graded01(n, x.ctypes.data, w.ctypes.data):
        raise ValueError("n out of range")
    return x, w


def classify_block_curve(test, trial, k2, t0=0, t1=None, s0=0, s1=None):
    t1 = test.mesh.ns if t1 is None else t1
    s1 = trial.mesh.ns if s1 is None else s1
    keep = _Keep()
    out = np.empty((t1 - t0, s1 - s0), dtype=np.int8)
    rc = lib().orc2_classify_block(C.byref(_space2(test, keep)), C.byref(_space2(trial, keep)), float(k2),
                                   t0, t1, s0, s1, out.ctypes.data)
    if rc:
        raise RuntimeError(f"orc2_classify_block failed ({rc})")
    return out


def local_matrices_curve(op, test, trial, qs, tau, sigma, force_class=-1):
    keep = _Keep()
    tau = np.ascontiguousarray(tau, dtype=np.int32)
    sigma = np.ascontiguousarray(sigma, dtype=np.int32)
    out = np.empty((tau.size, 2, 2, 2), dtype=np.float64)
    cls = np.empty(tau.size, dtype=np.int8)
    rc = lib().orc2_local_matrices(C.byref(_op2(op)), C.byref(_space2(test, keep)), C.byref(_space2(trial, keep)),
                                   C.byref(_qs2(qs)), tau.size, tau.ctypes.data, sigma.ctypes.data,
                                   int(force_class), out.ctypes.data, cls.ctypes.data)
    if rc:
        raise RuntimeError(f"orc2_local_matrices failed ({rc})")
    return out[..., 0] + 1j * out[..., 1], cls


def assemble_rows_curve(op, test, trial, qs, rows, nthreads=0):
    keep = _Keep()
    rows = np.ascontiguousarray(rows, dtype=np.int32)
    out = np.empty((rows.size, trial.nfun, 2), dtype=np.float64)
    rc = lib().orc2_assemble_rows(C.byref(_op2(op)), C.byref(_space2(test, keep)), C.byref(_space2(trial, keep)),
                                  C.byref(_qs2(qs)), rows.size, rows.ctypes.data, out.ctypes.data, int(nthreads))
    if rc:
        raise RuntimeError(f"orc2_assemble_rows failed ({rc})")
    return out[..., 0] + 1j * out[..., 1]


def assemble_curve(op, test, trial, qs, nthreads=0):
    return assemble_rows_curve(op, test, trial, qs, np.arange(test.nfun), nthreads)
