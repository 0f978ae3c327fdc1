"""ctypes binding of libbeastgb.so (include/beastgb.h).

The library is loaded from the package directory; there is no fallback: if the shared
object is missing or no CUDA device is present, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libbeastgb.so")

BGB_OK = 0
STATUS = {0: "OK", -1: "INVALID", -2: "OOM", -3: "CUDA", -4: "TIMEOUT", -5: "ABORTED", -6: "CAPACITY",
          -7: "NOT_SUPPORTED"}
PREC_FP64, PREC_MIXED = 0, 1
OUT_HOST_C64, OUT_HOST_C32, OUT_DEVICE_C64, OUT_DEVICE_C32 = 0, 1, 2, 3
CFG_PAGEABLE_VIA_RING = 1
ABI_VERSION = 3  # BGB_ABI_VERSION of include/beastgb.h


class BGBError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"libbeastgb error {code} ({STATUS.get(code, '?')}): {msg}")
        self.code = code


class Operator(C.Structure):
    _fields_ = [("kind", C.c_int32), ("alpha", C.c_double * 2), ("beta", C.c_double * 2), ("gamma", C.c_double * 2)]


class Space(C.Structure):
    _fields_ = [("refspace", C.c_int32), ("nv", C.c_int32), ("nt", C.c_int32), ("nfun", C.c_int32),
                ("vertices", C.c_void_p), ("triangles", C.c_void_p), ("fn_index", C.c_void_p),
                ("fn_coef", C.c_void_p)]


class QuadStrat(C.Structure):
    _fields_ = [("far_test", C.c_int32), ("far_trial", C.c_int32), ("near_test", C.c_int32),
                ("near_trial", C.c_int32), ("ss_cf", C.c_int32), ("ss_ce", C.c_int32), ("ss_cv", C.c_int32)]


class Config(C.Structure):
    _fields_ = [("device", C.c_int32), ("hbm_budget_bytes", C.c_int64), ("pinned_ring_bytes", C.c_int64),
                ("tile_config", C.c_int32), ("flags", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("pairs_total", C.c_int64), ("pairs_class", C.c_int64 * 5), ("pairs_computed", C.c_int64),
                ("ms_classify", C.c_double), ("ms_singular", C.c_double), ("ms_far", C.c_double),
                ("ms_copy", C.c_double), ("ms_total", C.c_double), ("ms_pipeline", C.c_double),
                ("ms_plan", C.c_double), ("out_blocks", C.c_int32), ("tile_config", C.c_int32),
                ("kernel_launches", C.c_int32), ("schedule", C.c_int32)]

    def as_dict(self):
        return {"pairs_total": self.pairs_total, "pairs_class": list(self.pairs_class),
                "pairs_computed": self.pairs_computed, "ms_classify": self.ms_classify,
                "ms_singular": self.ms_singular, "ms_far": self.ms_far, "ms_copy": self.ms_copy,
                "ms_total": self.ms_total, "ms_pipeline": self.ms_pipeline, "ms_plan": self.ms_plan,
                "out_blocks": self.out_blocks, "tile_config": self.tile_config,
                "kernel_launches": self.kernel_launches, "schedule": self.schedule}


class Problem(C.Structure):
    _fields_ = [("op", Operator), ("test", Space), ("trial", Space), ("qs", QuadStrat), ("out", C.c_void_p),
                ("ld", C.c_int64)]


class Operator2D(C.Structure):
    _fields_ = [("kind", C.c_int32), ("wavenumber", C.c_double), ("alpha", C.c_double * 2), ("beta", C.c_double * 2)]


class CurveSpace(C.Structure):
    _fields_ = [("refspace", C.c_int32), ("nv", C.c_int32), ("ns", C.c_int32), ("nfun", C.c_int32),
                ("vertices", C.c_void_p), ("segments", C.c_void_p), ("fn_index", C.c_void_p),
                ("fn_coef", C.c_void_p)]


class QuadStrat2D(C.Structure):
    _fields_ = [("far_test", C.c_int32), ("far_trial", C.c_int32), ("near", C.c_int32), ("singular", C.c_int32)]


# every exported symbol of include/beastgb.h with its ctypes signature
SIGNATURES = {
    "bgb_abi_version": ([], C.c_int),
    "bgb_last_error": ([], C.c_char_p),
    "bgb_create": ([C.POINTER(C.c_void_p), C.POINTER(Config)], C.c_int),
    "bgb_destroy": ([C.c_void_p], C.c_int),
    "bgb_abort": ([C.c_void_p], C.c_int),
    "bgb_tile_info": ([C.c_void_p, C.c_int32], C.c_int),
    "bgb_measure_issue_peaks": ([C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                 C.POINTER(C.c_double)], C.c_int),
    "bgb_classify_block": ([C.c_void_p, C.POINTER(Space), C.POINTER(Space), C.c_double, C.c_int32, C.c_int32,
                            C.c_int32, C.c_int32, C.c_void_p], C.c_int),
    "bgb_local_matrices": ([C.c_void_p, C.POINTER(Operator), C.POINTER(Space), C.POINTER(Space),
                            C.POINTER(QuadStrat), C.c_int32, C.c_int64, C.c_void_p, C.c_void_p, C.c_int32,
                            C.c_void_p, C.c_void_p], C.c_int),
    "bgb_assemble": ([C.c_void_p, C.POINTER(Operator), C.POINTER(Space), C.POINTER(Space), C.POINTER(QuadStrat),
                      C.c_int32, C.c_void_p, C.c_int32, C.c_int64, C.c_int64, C.c_int64, C.c_void_p,
                      C.POINTER(Stats)], C.c_int),
    "bgb_assemble_batch": ([C.c_void_p, C.c_int32, C.POINTER(Problem), C.c_int32, C.c_int32, C.c_void_p,
                            C.POINTER(Stats)], C.c_int),
    "bgb_batch_create": ([C.c_void_p, C.c_int32, C.POINTER(Problem), C.c_int32, C.c_int32, C.c_int32,
                          C.POINTER(C.c_void_p), C.POINTER(Stats)], C.c_int),
    "bgb_batch_run": ([C.c_void_p, C.c_void_p, C.POINTER(Stats)], C.c_int),
    "bgb_batch_destroy": ([C.c_void_p], C.c_int),
    "bgb_classify_csr_noalloc": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32,
                                  C.c_int32, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                  C.POINTER(C.c_int64), C.c_void_p], C.c_int),
    "bgb_assemble_curve": ([C.c_void_p, C.POINTER(Operator2D), C.POINTER(CurveSpace), C.POINTER(CurveSpace),
                            C.POINTER(QuadStrat2D), C.c_int32, C.c_void_p, C.c_int32, C.c_int64, C.c_int64, C.c_int64,
                            C.c_void_p, C.POINTER(Stats)], C.c_int),
    "bgb_plan_order": ([C.POINTER(Space), C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.POINTER(C.c_int64)],
                       C.c_int),
    "bgb_local_matrices_curve": ([C.c_void_p, C.POINTER(Operator2D), C.POINTER(CurveSpace), C.POINTER(CurveSpace),
                                  C.POINTER(QuadStrat2D), C.c_int32, C.c_int64, C.c_void_p, C.c_void_p, C.c_int32,
                                  C.c_void_p, C.c_void_p], C.c_int),
}

_lib = None


def load():
    """Load libbeastgb.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m beastgpu_gb300.csrc.build` "
                               "(or __graft_entry__.build())")
        lib = C.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        if lib.bgb_abi_version() != ABI_VERSION:
            raise RuntimeError(f"{LIB_PATH} has ABI {lib.bgb_abi_version()}, the bindings expect {ABI_VERSION}: rebuild it")
        _lib = lib
    return _lib


def check(rc):
    if rc != BGB_OK:
        raise BGBError(rc, load().bgb_last_error().decode(errors="replace"))
    return rc
