"""Host-side mirror of BEASTGPU's `assemble_gpu` interface over the C ABI.

    Z = assemble_gpu(op, X, Y, config, GpuWriteBackTrueInstance(); quadstrat=...)

follows assemble_gpu(operator, test_functions, trial_functions, config, writeBackStrategy;
storage_policy, threading, quadstrat) (assamble_gpu.jl:8,25): it returns the dense complex
Galerkin matrix with test functions as rows and trial functions as columns.  `assemble`
mirrors BEAST.assemble(op, X, Y; quadstrat).  Both write-back strategies of the reference give
the same matrix here: the gather write is always done on the GPU (no FP64 atomics), and the
matrix is copied to the host (column-major, Julia's layout) unless `out="device"`.

Everything runs through libbeastgb.so; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import threading
from dataclasses import dataclass

import numpy as np

from . import _lib
from .curves import CurveSpace, Operator2D, QuadStrat2D, defaultquadstrat2d
from .operators import Operator, QuadStrat, defaultquadstrat
from .spaces import Space

# ---- write-back strategies (CustomDataStructs/GpuWriteBack.jl) -----------------------------


class GpuWriteBack:
    pass


class GpuWriteBackTrue(GpuWriteBack):
    """Matrix assembled in device memory, then copied to the host (reference default)."""


class GpuWriteBackFalse(GpuWriteBack):
    """Reference: per-pair blocks copied to the host and scattered there.  Here the scatter is
    a deterministic gather on the GPU for both strategies, so the result is identical."""


def GpuWriteBackTrueInstance():
    return GpuWriteBackTrue()


def GpuWriteBackFalseInstance():
    return GpuWriteBackFalse()


@dataclass
class GPUConfiguration:
    """The fields of the reference's GPUConfiguration (utils/configuration.jl:11-26) that mean
    something on one GB300, plus the precision mode and tile choice.

    floatType: the reference's field; np.float64 (or float) selects the plain FP64 kernels and
    np.float32 the mixed ones, overriding `precision` when given.
    amount_of_gpus: the reference's chunk count (assamble_chunk_gpu.jl:123-130): the matrix is
    assembled in that many row windows, one after the other; the result is the same.
    precision: "fp64" (plain all-FP64 kernels, the drop-in) or "mixed" (FP32 far pairs with
    double-float phase base, FP64-accurate singular and near pairs).
    total_GPU_budget: HBM bytes the call may use for the output staging (0 = 90% of free);
    host outputs are produced in blocks of columns of at most a quarter of it (two device
    staging buffers), and large outputs in about 16 blocks so that copies overlap the fill.
    pinned_ring_bytes: size of each half of the pinned host ring that pageable host outputs
    are copied through when the device cannot write pageable memory directly (0 = 512 MiB).
    pageable_via_ring: use the ring even where the device writes pageable memory directly.
    """
    writeBackStrategy: GpuWriteBack = None
    precision: str = "fp64"
    device: int = 0
    total_GPU_budget: int = 0
    tile_config: int = -1
    makeCompexWithGPU: bool = True
    pinned_ring_bytes: int = 0
    pageable_via_ring: bool = False
    floatType: type = None
    amount_of_gpus: int = 1

    def __post_init__(self):
        if self.writeBackStrategy is None:
            self.writeBackStrategy = GpuWriteBackTrueInstance()
        if self.floatType is not None:
            ft = np.dtype(self.floatType)
            if ft not in (np.float64, np.float32):
                raise ValueError("floatType must be Float64 or Float32")
            self.precision = "fp64" if ft == np.float64 else "mixed"
        if self.precision not in ("fp64", "mixed"):
            raise ValueError("precision must be 'fp64' or 'mixed'")
        if self.amount_of_gpus < 1:
            raise ValueError("amount_of_gpus must be at least 1")


_handles = {}
_hlock = threading.Lock()


class Handle:
    """Owns one bgb_handle (device scratch, streams)."""

    def __init__(self, device: int = 0, hbm_budget: int = 0, tile_config: int = -1, pinned_ring: int = 0,
                 flags: int = 0):
        lib = _lib.load()
        self.ptr = C.c_void_p()
        cfg = _lib.Config(device, int(hbm_budget), int(pinned_ring), int(tile_config), int(flags))
        _lib.check(lib.bgb_create(C.byref(self.ptr), C.byref(cfg)))
        self.device = device

    def close(self):
        if self.ptr:
            _lib.load().bgb_destroy(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def get_handle(device: int = 0, hbm_budget: int = 0, tile_config: int = -1, pinned_ring: int = 0,
               flags: int = 0) -> Handle:
    key = (device, int(hbm_budget), int(tile_config), int(pinned_ring), int(flags))
    with _hlock:
        h = _handles.get(key)
        if h is None:
            h = Handle(device, hbm_budget, tile_config, pinned_ring, flags)
            _handles[key] = h
        return h


class _Keep:
    def __init__(self):
        self.refs = []

    def ptr(self, a, dtype):
        a = np.ascontiguousarray(a, dtype=dtype)
        self.refs.append(a)
        return a.ctypes.data


def c_space(space: Space, keep: _Keep) -> _lib.Space:
    m = space.mesh
    return _lib.Space(space.refspace, m.nv, m.nt, space.nfun, keep.ptr(m.vertices, np.float64),
                      keep.ptr(m.triangles, np.int32), keep.ptr(space.fn_index, np.int32),
                      keep.ptr(space.fn_coef, np.float64))


def c_operator(op: Operator) -> _lib.Operator:
    a, b, g = complex(op.alpha), complex(op.beta), complex(op.gamma)
    return _lib.Operator(op.kind, (C.c_double * 2)(a.real, a.imag), (C.c_double * 2)(b.real, b.imag),
                         (C.c_double * 2)(g.real, g.imag))


def c_curve_space(space: CurveSpace, keep: _Keep) -> _lib.CurveSpace:
    m = space.mesh
    return _lib.CurveSpace(space.refspace, m.nv, m.ns, space.nfun, keep.ptr(m.vertices, np.float64),
                           keep.ptr(m.segments, np.int32), keep.ptr(space.fn_index, np.int32),
                           keep.ptr(space.fn_coef, np.float64))


def c_operator2d(op: Operator2D) -> _lib.Operator2D:
    a, b = complex(op.alpha), complex(op.beta)
    return _lib.Operator2D(op.kind, float(op.wavenumber), (C.c_double * 2)(a.real, a.imag),
                           (C.c_double * 2)(b.real, b.imag))


def c_quadstrat2d(qs: QuadStrat2D) -> _lib.QuadStrat2D:
    return _lib.QuadStrat2D(qs.far_test, qs.far_trial, qs.near, qs.singular)


def c_quadstrat(qs: QuadStrat) -> _lib.QuadStrat:
    return _lib.QuadStrat(qs.far_test, qs.far_trial, qs.near_test, qs.near_trial, qs.ss_cf, qs.ss_ce, qs.ss_cv)


def _precision(p):
    if isinstance(p, int):
        return p
    return {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED}[p]


def _out_ptr(buf, dtype, nelem: int, on_device: bool, device: int) -> int:
    """Address of a caller-provided output buffer, after the checks that keep every write of the
    library inside it: the element type of the output, contiguous storage of at least `nelem`
    elements, and host memory for a host output / a tensor on `device` for a device output."""
    if hasattr(buf, "data_ptr"):  # torch tensor
        import torch
        want = torch.complex128 if dtype == np.complex128 else torch.complex64
        if buf.dtype != want:
            raise ValueError(f"out_buffer has dtype {buf.dtype}; this output is {want}")
        if not buf.is_contiguous():
            raise ValueError("out_buffer must be contiguous")
        if buf.is_cuda != on_device or (on_device and buf.device.index != device):
            raise ValueError(f"out_buffer is on {buf.device}; this output goes to "
                             f"{'cuda:%d' % device if on_device else 'host memory'}")
        n, ptr = buf.numel(), buf.data_ptr()
    else:
        if on_device:
            raise ValueError("a device output needs a torch CUDA tensor as out_buffer")
        if not isinstance(buf, np.ndarray) or buf.dtype != dtype:
            raise ValueError(f"out_buffer must be a numpy array of {np.dtype(dtype)}")
        if not (buf.flags.f_contiguous or buf.flags.c_contiguous) or not buf.flags.writeable:
            raise ValueError("out_buffer must be contiguous and writeable")
        n, ptr = buf.size, buf.ctypes.data
    if n < nelem:
        raise ValueError(f"out_buffer holds {n} elements; the output needs {nelem}")
    return ptr


def assemble_gpu(operator: Operator, test_functions: Space, trial_functions: Space, config: GPUConfiguration = None,
                 writeBackStrategy: GpuWriteBack = None, *, storage_policy=None, threading=None,
                 quadstrat: QuadStrat = None, out: str = "host", dtype=None, rows=None, out_buffer=None, stream=None,
                 return_stats: bool = False):
    """Dense Galerkin matrix Z[m, n] = <f_m, op g_n> (test rows, trial columns).

    The reference's signature, assemble_gpu(operator, test_functions, trial_functions, config,
    writeBackStrategy; storage_policy, threading, quadstrat) (assamble_gpu.jl:8,25): both
    write-back strategies give the same matrix; storage_policy and threading are accepted and
    ignored (the matrix is dense, the threads are the library's); quadstrat defaults to
    defaultquadstrat(operator, test_functions, trial_functions).  The keywords after it are this
    binding's: out="host": numpy array in Fortran (column-major) order, complex128 for precision
    "fp64" and complex64 for "mixed" unless `dtype` says otherwise.  out="device": a torch CUDA
    tensor view of shape (rows, cols) with column-major strides.  rows=(row0, nrows) assembles
    a row window.  out_buffer: a preallocated host (numpy or pinned torch) or device (torch)
    buffer of the right shape/dtype to write into; its element type, contiguous size and side
    (host or device) are checked before any device work (ValueError otherwise).
    """
    config = config or GPUConfiguration()
    if config.amount_of_gpus > 1 and rows is None and out == "host" and out_buffer is None \
            and not isinstance(test_functions, CurveSpace):
        return _assemble_chunks(operator, test_functions, trial_functions, config, quadstrat, dtype, return_stats)
    if isinstance(test_functions, CurveSpace):
        return _assemble_curve(operator, test_functions, trial_functions, config, quadstrat, out, dtype, rows,
                               out_buffer, stream, return_stats)
    quadstrat = quadstrat or defaultquadstrat(operator, test_functions, trial_functions)
    prec = _precision(config.precision)
    if dtype is None:
        dtype = np.complex128 if prec == _lib.PREC_FP64 else np.complex64
    dtype = np.dtype(dtype)
    if dtype not in (np.complex128, np.complex64):
        raise ValueError("dtype must be complex128 or complex64")
    c64 = dtype == np.complex128
    row0, nrows = (0, test_functions.nfun) if rows is None else (int(rows[0]), int(rows[1]))
    ncols = trial_functions.nfun
    if out not in ("host", "device"):
        raise ValueError("out must be 'host' or 'device'")
    buf_ptr = None if out_buffer is None else _out_ptr(out_buffer, dtype, max(1, nrows) * ncols, out == "device",
                                                           config.device)
    h = get_handle(config.device, config.total_GPU_budget, config.tile_config, config.pinned_ring_bytes,
                   _lib.CFG_PAGEABLE_VIA_RING if config.pageable_via_ring else 0)
    keep = _Keep()
    cop, ct, cb, cq = c_operator(operator), c_space(test_functions, keep), c_space(trial_functions, keep), \
        c_quadstrat(quadstrat)
    stats = _lib.Stats()
    lib = _lib.load()
    if out == "host":
        if out_buffer is None:
            Z = np.empty((nrows, ncols), dtype=dtype, order="F")
            ptr = Z.ctypes.data
        else:
            Z, ptr = out_buffer, buf_ptr
        kind = _lib.OUT_HOST_C64 if c64 else _lib.OUT_HOST_C32
        _lib.check(lib.bgb_assemble(h.ptr, C.byref(cop), C.byref(ct), C.byref(cb), C.byref(cq), prec, C.c_void_p(ptr),
                                    kind, max(1, nrows), row0, nrows, None, C.byref(stats)))
    elif out == "device":
        import torch
        tdt = torch.complex128 if c64 else torch.complex64
        if out_buffer is None:
            Zt = torch.empty((ncols, max(1, nrows)), dtype=tdt, device=f"cuda:{config.device}")
        else:
            Zt = out_buffer
        st = stream if stream is not None else torch.cuda.current_stream(config.device).cuda_stream
        kind = _lib.OUT_DEVICE_C64 if c64 else _lib.OUT_DEVICE_C32
        _lib.check(lib.bgb_assemble(h.ptr, C.byref(cop), C.byref(ct), C.byref(cb), C.byref(cq), prec,
                                    C.c_void_p(Zt.data_ptr()), kind, max(1, nrows), row0, nrows, C.c_void_p(st),
                                    C.byref(stats)))
        Z = Zt.T
    else:
        raise ValueError("out must be 'host' or 'device'")
    return (Z, stats.as_dict()) if return_stats else Z


def _assemble_chunks(operator, X, Y, config, quadstrat, dtype, return_stats):
    """config.amount_of_gpus row windows of one host matrix, assembled one after the other (the
    reference's chunks, assamble_chunk_gpu.jl:123-130)."""
    prec = _precision(config.precision)
    dtype = np.dtype(dtype or (np.complex128 if prec == _lib.PREC_FP64 else np.complex64))
    Z = np.empty((X.nfun, Y.nfun), dtype=dtype, order="F")
    one = GPUConfiguration(writeBackStrategy=config.writeBackStrategy, precision=config.precision,
                           device=config.device, total_GPU_budget=config.total_GPU_budget,
                           tile_config=config.tile_config, pinned_ring_bytes=config.pinned_ring_bytes,
                           pageable_via_ring=config.pageable_via_ring)
    stats = []
    for c in range(config.amount_of_gpus):
        r0, n = row_shard(X.nfun, c, config.amount_of_gpus)
        if n == 0:
            continue
        part, st = assemble_gpu(operator, X, Y, one, quadstrat=quadstrat, dtype=dtype, rows=(r0, n),
                                return_stats=True)
        Z[r0:r0 + n, :] = part
        stats.append(st)
    return (Z, stats) if return_stats else Z


def _assemble_curve(operator, X, Y, config, quadstrat, out, dtype, rows, out_buffer, stream, return_stats):
    """The curve (2-D) path: precision "fp64" (complex128 output by default) or "mixed" (FP32 far
    pairs, complex64 output by default)."""
    if not isinstance(Y, CurveSpace) or not isinstance(operator, Operator2D):
        raise TypeError("curve spaces need a Helmholtz2D operator and a curve trial space")
    quadstrat = quadstrat or defaultquadstrat2d(operator, X, Y)
    prec = _precision(config.precision)
    if dtype is None:
        dtype = np.complex128 if prec == _lib.PREC_FP64 else np.complex64
    dtype = np.dtype(dtype)
    if dtype not in (np.complex128, np.complex64):
        raise ValueError("dtype must be complex128 or complex64")
    c64 = dtype == np.complex128
    row0, nrows = (0, X.nfun) if rows is None else (int(rows[0]), int(rows[1]))
    ncols = Y.nfun
    if out not in ("host", "device"):
        raise ValueError("out must be 'host' or 'device'")
    buf_ptr = None if out_buffer is None else _out_ptr(out_buffer, dtype, max(1, nrows) * ncols, out == "device",
                                                           config.device)
    h = get_handle(config.device, config.total_GPU_budget, config.tile_config, config.pinned_ring_bytes, 0)
    keep = _Keep()
    cop, ct, cb, cq = c_operator2d(operator), c_curve_space(X, keep), c_curve_space(Y, keep), c_quadstrat2d(quadstrat)
    stats = _lib.Stats()
    lib = _lib.load()
    if out == "host":
        Z = np.empty((nrows, ncols), dtype=dtype, order="F") if out_buffer is None else out_buffer
        ptr = Z.ctypes.data if out_buffer is None else buf_ptr
        kind = _lib.OUT_HOST_C64 if c64 else _lib.OUT_HOST_C32
        _lib.check(lib.bgb_assemble_curve(h.ptr, C.byref(cop), C.byref(ct), C.byref(cb), C.byref(cq), prec,
                                          C.c_void_p(ptr), kind, max(1, nrows), row0, nrows, None, C.byref(stats)))
    elif out == "device":
        import torch
        tdt = torch.complex128 if c64 else torch.complex64
        Zt = torch.empty((ncols, max(1, nrows)), dtype=tdt, device=f"cuda:{config.device}") if out_buffer is None \
            else out_buffer
        st = stream if stream is not None else torch.cuda.current_stream(config.device).cuda_stream
        kind = _lib.OUT_DEVICE_C64 if c64 else _lib.OUT_DEVICE_C32
        _lib.check(lib.bgb_assemble_curve(h.ptr, C.byref(cop), C.byref(ct), C.byref(cb), C.byref(cq), prec,
                                          C.c_void_p(Zt.data_ptr()), kind, max(1, nrows), row0, nrows, C.c_void_p(st),
                                          C.byref(stats)))
        Z = Zt.T
    else:
        raise ValueError("out must be 'host' or 'device'")
    return (Z, stats.as_dict()) if return_stats else Z


def local_matrices_curve(operator: Operator2D, test_functions: CurveSpace, trial_functions: CurveSpace, tau, sigma, *,
                         quadstrat: QuadStrat2D = None, precision: str = "fp64", force_class: int = -1,
                         device: int = 0):
    """2x2 local matrices L[p, i, j] of explicit segment pairs and their classes (curve path)."""
    quadstrat = quadstrat or defaultquadstrat2d()
    tau = np.ascontiguousarray(tau, dtype=np.int32)
    sigma = np.ascontiguousarray(sigma, dtype=np.int32)
    h = get_handle(device)
    keep = _Keep()
    out = np.empty((tau.size, 2, 2, 2), dtype=np.float64)
    cls = np.empty(tau.size, dtype=np.int8)
    _lib.check(_lib.load().bgb_local_matrices_curve(
        h.ptr, C.byref(c_operator2d(operator)), C.byref(c_curve_space(test_functions, keep)),
        C.byref(c_curve_space(trial_functions, keep)), C.byref(c_quadstrat2d(quadstrat)), _precision(precision),
        tau.size, tau.ctypes.data,
        sigma.ctypes.data, int(force_class), out.ctypes.data, cls.ctypes.data))
    return out[..., 0] + 1j * out[..., 1], cls


def row_shard(nrows: int, rank: int, world: int):
    """Row window (row0, nrows) of `rank` among `world` processes: contiguous, balanced to one
    row, covering [0, nrows) exactly once (the multi-GPU split of one matrix; the reference
    splits the same way, assamble_chunk_gpu.jl:123-130).  No data exchange is needed: each rank
    assembles its rows against all trial functions."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    r0 = nrows * rank // world
    return r0, nrows * (rank + 1) // world - r0


def assemble(operator: Operator, test_functions: Space, trial_functions: Space, *, quadstrat: QuadStrat = None,
             precision: str = "fp64", **kw):
    """BEAST.assemble(op, X, Y; quadstrat) on the GPU (host complex matrix)."""
    return assemble_gpu(operator, test_functions, trial_functions, GPUConfiguration(precision=precision),
                        quadstrat=quadstrat, **kw)


def tile_order(space: Space, width: int = 64, functions=None):
    """The far kernel's tiling of one side, computed on the host (no GPU): the order in which tiles
    of `width` functions take the functions [f0, f1) (`functions`, default all) and the number of
    (tile, support triangle) slots those tiles stage (the triangles per side the far kernel
    evaluates, halo included)."""
    f0, f1 = (0, space.nfun) if functions is None else (int(functions[0]), int(functions[1]))
    keep = _Keep()
    order = np.empty(max(0, f1 - f0), dtype=np.int32)
    slots = C.c_int64(0)
    _lib.check(_lib.load().bgb_plan_order(C.byref(c_space(space, keep)), f0, f1, int(width), order.ctypes.data,
                                          C.byref(slots)))
    return order, int(slots.value)


def classify(test_functions: Space, trial_functions: Space, k2: float, block=None, device: int = 0):
    """Pair classes (0 far, 1 CV, 2 CE, 3 CF, 4 near) of a block of triangle pairs on the GPU."""
    t0, t1, s0, s1 = block or (0, test_functions.mesh.nt, 0, trial_functions.mesh.nt)
    h = get_handle(device)
    keep = _Keep()
    out = np.empty((t1 - t0, s1 - s0), dtype=np.int8)
    _lib.check(_lib.load().bgb_classify_block(h.ptr, C.byref(c_space(test_functions, keep)),
                                              C.byref(c_space(trial_functions, keep)), float(k2), t0, t1, s0, s1,
                                              out.ctypes.data))
    return out


def local_matrices(operator: Operator, test_functions: Space, trial_functions: Space, tau, sigma, *,
                   quadstrat: QuadStrat = None, precision: str = "fp64", force_class: int = -1, device: int = 0):
    """3x3 local matrices L[p, i, j] of explicit triangle pairs and their classes."""
    quadstrat = quadstrat or defaultquadstrat()
    tau = np.ascontiguousarray(tau, dtype=np.int32)
    sigma = np.ascontiguousarray(sigma, dtype=np.int32)
    h = get_handle(device)
    keep = _Keep()
    out = np.empty((tau.size, 3, 3, 2), dtype=np.float64)
    cls = np.empty(tau.size, dtype=np.int8)
    _lib.check(_lib.load().bgb_local_matrices(
        h.ptr, C.byref(c_operator(operator)), C.byref(c_space(test_functions, keep)),
        C.byref(c_space(trial_functions, keep)), C.byref(c_quadstrat(quadstrat)), _precision(precision), tau.size,
        tau.ctypes.data, sigma.ctypes.data, int(force_class), out.ctypes.data, cls.ctypes.data))
    return out[..., 0] + 1j * out[..., 1], cls


def measure_issue_peaks(device: int = 0):
    """(FP32 TFLOP/s, FP64 TFLOP/s, MUFU Tops/s) measured on the device."""
    h = get_handle(device)
    a, b, c = C.c_double(), C.c_double(), C.c_double()
    _lib.check(_lib.load().bgb_measure_issue_peaks(h.ptr, C.byref(a), C.byref(b), C.byref(c)))
    return a.value, b.value, c.value


class Batch:
    """Plan / execute form of a batch of independent problems (bgb_batch_create / _run).

    problems: list of (operator, test space, trial space).  All share the operator kind, the
    space kind and the quadrature strategy.  On construction every problem is assembled once
    (one classification launch, one singular-pair launch and ONE persistent far-pair launch
    over a work queue of tiles of all problems), the tile shape and work-queue schedule are
    autotuned (autotune=True), and the device sequence is captured in a CUDA graph that
    run() replays.  `outputs` are the matrices (torch CUDA tensors for out="device", numpy
    column-major arrays for out="host").
    """

    def __init__(self, problems, config: GPUConfiguration = None, *, quadstrat: QuadStrat = None, out="device",
                 dtype=None, autotune=True):
        config = config or GPUConfiguration()
        self.config = config
        prec = _precision(config.precision)
        if dtype is None:
            dtype = np.complex128 if prec == _lib.PREC_FP64 else np.complex64
        dtype = np.dtype(dtype)
        c64 = dtype == np.complex128
        self.h = get_handle(config.device, config.total_GPU_budget, config.tile_config, config.pinned_ring_bytes,
                   _lib.CFG_PAGEABLE_VIA_RING if config.pageable_via_ring else 0)
        self._keep = _Keep()
        arr = (_lib.Problem * len(problems))()
        self.outputs = []
        self._bufs = []
        for i, (op, X, Y) in enumerate(problems):
            qs = quadstrat or defaultquadstrat(op, X, Y)
            arr[i].op = c_operator(op)
            arr[i].test = c_space(X, self._keep)
            arr[i].trial = c_space(Y, self._keep)
            arr[i].qs = c_quadstrat(qs)
            arr[i].ld = max(1, X.nfun)
            if out == "device":
                import torch
                t = torch.empty((Y.nfun, max(1, X.nfun)), dtype=torch.complex128 if c64 else torch.complex64,
                                device=f"cuda:{config.device}")
                self._bufs.append(t)
                arr[i].out = t.data_ptr()
                self.outputs.append(t.T)
            elif out == "host":
                Z = np.empty((X.nfun, Y.nfun), dtype=dtype, order="F")
                self._bufs.append(Z)
                arr[i].out = Z.ctypes.data
                self.outputs.append(Z)
            else:
                raise ValueError("out must be 'host' or 'device'")
        self._arr = arr
        kind = (_lib.OUT_DEVICE_C64 if c64 else _lib.OUT_DEVICE_C32) if out == "device" else \
            (_lib.OUT_HOST_C64 if c64 else _lib.OUT_HOST_C32)
        self.ptr = C.c_void_p()
        st = _lib.Stats()
        _lib.check(_lib.load().bgb_batch_create(self.h.ptr, len(problems), arr, prec, kind, 1 if autotune else 0,
                                                C.byref(self.ptr), C.byref(st)))
        self.create_stats = st.as_dict()

    def run(self, stream=None):
        """Replay the captured graph (re-assembles every problem); returns the stats."""
        st = _lib.Stats()
        _lib.check(_lib.load().bgb_batch_run(self.ptr, C.c_void_p(stream) if stream else None, C.byref(st)))
        return st.as_dict()

    def close(self):
        if self.ptr:
            _lib.load().bgb_batch_destroy(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def assemble_batch(problems, config: GPUConfiguration = None, *, quadstrat: QuadStrat = None, out="device", dtype=None,
                   autotune=False):
    """Assemble independent problems [(op, X, Y), ...] with one persistent far-pair launch."""
    b = Batch(problems, config, quadstrat=quadstrat, out=out, dtype=dtype, autotune=autotune)
    outs = b.outputs
    b.close()
    return outs
