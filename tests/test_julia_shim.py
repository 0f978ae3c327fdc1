"""The Julia shim (beastgpu_gb300/julia/BEASTGB.jl) against the C ABI (include/beastgb.h), on the CPU.

No Julia toolchain is available here, so the shim cannot run; what can be checked is that every
struct it passes has the header's field order and types, that every ccall's argument and return
types are the header prototype's, that it keeps the reference's assemble_gpu signature
(assamble_gpu.jl:8,25) with one method per write-back strategy and the reference's
GPUConfiguration fields (utils/configuration.jl:11-26), and that the Python ctypes bindings
(beastgpu_gb300/_lib.py) have the same layouts.
"""
import ctypes as C
import os
import re

import pytest

from beastgpu_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = open(os.path.join(ROOT, "include", "beastgb.h")).read()
SHIM = open(os.path.join(ROOT, "beastgpu_gb300", "julia", "BEASTGB.jl")).read()
HDR = re.sub(r"/\*.*?\*/", "", HEADER, flags=re.S)

C2JL = {"int32_t": "Int32", "int64_t": "Int64", "double": "Float64", "int": "Cint", "void": "Cvoid"}
STRUCTS = {"bgb_operator": "BgbOperator", "bgb_space": "BgbSpace", "bgb_quadstrat": "BgbQuadStrat",
           "bgb_config": "BgbConfig", "bgb_stats": "BgbStats"}


def c_struct(name):
    body = re.search(r"typedef struct \{([^{}]*)\}\s*" + name + r";", HDR).group(1)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        m = re.match(r"(const\s+)?(\w+)\s*(\*?)\s*(.+)", decl)
        base, ptr, names = m.group(2), m.group(3), m.group(4)
        for nm in names.split(","):
            nm = nm.strip()
            arr = re.match(r"(\w+)\[(\d+)\]", nm)
            if arr:
                fields.append((arr.group(1), f"NTuple{{{arr.group(2)},{C2JL[base]}}}"))
            elif ptr:
                fields.append((nm, f"Ptr{{{C2JL[base]}}}"))
            else:
                fields.append((nm, C2JL[base]))
    return fields


def jl_struct(name):
    body = re.search(r"struct " + name + r"\n(.*?)\nend", SHIM, flags=re.S).group(1)
    return [tuple(x.strip() for x in line.strip().split("::")) for line in body.splitlines() if "::" in line]


@pytest.mark.parametrize("cname", list(STRUCTS))
def test_shim_structs_match_the_header(cname):
    assert jl_struct(STRUCTS[cname]) == c_struct(cname)


def c_param_to_jl(p):
    p = p.strip()
    m = re.match(r"(const\s+)?(\w+)\s*(\**)\s*\w*$", p)
    base, stars = m.group(2), m.group(3)
    if base == "bgb_handle":
        return {"*": "Ptr{Cvoid}", "**": "Ptr{Ptr{Cvoid}}"}[stars]
    if base in STRUCTS:
        assert stars == "*"
        return f"Ptr{{{STRUCTS[base]}}}"
    if stars:
        return "Ptr{Cvoid}" if base == "void" else f"Ptr{{{C2JL[base]}}}"
    return C2JL[base]


def c_prototype(fn):
    m = re.search(r"(const char\*|int)\s+" + fn + r"\(([^)]*)\);", HDR, flags=re.S)
    ret = "Cstring" if m.group(1) == "const char*" else "Cint"
    params = [p for p in m.group(2).split(",") if p.strip() and p.strip() != "void"]
    return ret, [c_param_to_jl(p) for p in params]


def shim_ccalls():
    calls = []
    for m in re.finditer(r"ccall\(\(:(\w+), libbeastgb\), (\w+),\s*\(([^()]*)\)", SHIM):
        types = [t.strip() for t in m.group(3).replace("\n", " ").split(",") if t.strip()]
        calls.append((m.group(1), m.group(2), types))
    return calls


def test_shim_ccalls_match_the_prototypes():
    calls = shim_ccalls()
    assert {c[0] for c in calls} >= {"bgb_create", "bgb_destroy", "bgb_assemble", "bgb_last_error"}
    for fn, ret, types in calls:
        cret, cparams = c_prototype(fn)
        assert ret == cret, fn
        assert types == cparams, (fn, types, cparams)


def test_shim_keeps_the_reference_signature():
    # assemble_gpu(operator, test_functions, trial_functions, config, writeBackStrategy; storage_policy,
    # threading, quadstrat), one method per strategy (assamble_gpu.jl:8,25)
    for strat in ("GpuWriteBackFalseInstance", "GpuWriteBackTrueInstance"):
        pat = (r"function assemble_gpu\(operator::BEAST\.AbstractOperator, test_functions, trial_functions, config,\s*"
               r"writeBackStrategy::" + strat + r";\s*storage_policy = Val\{:bandedstorage\}, "
               r"threading = BEAST\.Threading\{:single\},\s*"
               r"quadstrat = BEAST\.defaultquadstrat\(operator, test_functions, trial_functions\)\)")
        assert re.search(pat, SHIM), strat
    # GPUConfiguration: the reference's 14 fields in order (utils/configuration.jl:11-26)
    fields = [f[0] for f in jl_struct("GPUConfiguration")]
    assert fields == ["writeBackStrategy", "amount_of_gpus", "total_GPU_budget",
                      "InstancedoubleQuadRuleGpuStrategyShouldCalculate", "ShouldCalcInstance",
                      "GPU_budget_pipeline_result", "amount_of_producers", "makeCompexWithGPU", "backend",
                      "timeLogger", "floatType", "sortOnCPU", "filename_benchmark", "gpu_schedular_print_filename"]
    # floatType selects the precision; quadstrat fields are translated, not hard-coded
    assert "config.floatType === Float32 ? BGB_PREC_MIXED : BGB_PREC_FP64" in SHIM
    for f in ("outer_rule_far", "inner_rule_far", "outer_rule_near", "inner_rule_near", "sauter_schwab_common_face",
              "sauter_schwab_common_edge", "sauter_schwab_common_vert"):
        assert "qs." + f in SHIM


CT = {C.c_int32: "Int32", C.c_int64: "Int64", C.c_double: "Float64", C.c_void_p: "Ptr"}


@pytest.mark.parametrize("cname,pyname", [("bgb_operator", "Operator"), ("bgb_space", "Space"),
                                          ("bgb_quadstrat", "QuadStrat"), ("bgb_config", "Config"),
                                          ("bgb_stats", "Stats")])
def test_ctypes_structs_match_the_header(cname, pyname):
    got = []
    for name, t in getattr(_lib, pyname)._fields_:
        if hasattr(t, "_length_"):
            got.append((name, f"NTuple{{{t._length_},{CT[t._type_]}}}"))
        else:
            got.append((name, CT[t]))
    want = [(n, "Ptr" if t.startswith("Ptr") else t) for n, t in c_struct(cname)]
    assert got == want
