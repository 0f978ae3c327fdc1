# BEASTGB.jl -- the Julia side of libbeastgb: BEASTGPU's assemble_gpu surface over the C ABI.
#
# A BEASTGPU caller switches by loading this module instead of the reference's files; its calls
#     assemble_gpu(op, X, Y, config, GpuWriteBackTrueInstance())              (run.jl:52)
#     assemble_gpu(S, X, X, config, config.writeBackStrategy)                (test/correctness.jl:36)
# bind unchanged: the signature is the reference's
#     assemble_gpu(operator, test_functions, trial_functions, config, writeBackStrategy;
#                  storage_policy, threading, quadstrat)                     (assamble_gpu.jl:8,25)
# with one method per write-back strategy, and GPUConfiguration keeps the reference's fields and
# positional constructor (utils/configuration.jl:11-50).  The reference's own GPUConfiguration
# objects work too: only their fields are read.
#
# What the fields mean here:
#   floatType           Float64 -> BGB_PREC_FP64 (the drop-in); Float32 -> BGB_PREC_MIXED (FP32 far
#                       pairs, FP64-accurate singular and near pairs)
#   total_GPU_budget    bgb_config.hbm_budget_bytes (device staging of the host output)
#   amount_of_gpus      the matrix is assembled in that many row windows (the reference's chunks,
#                       assamble_chunk_gpu.jl:123-130); the result is the same
#   writeBackStrategy   both strategies give the same matrix (a deterministic gather on the GPU)
#   the other fields    (producers, pipeline budgets, backend, loggers) have no counterpart
# storage_policy and threading are accepted and ignored (the matrix is dense; threads are the
# library's).  quadstrat is BEAST's DoubleNumWiltonSauterQStrat, translated field by field.
#
# The struct layouts below must match include/beastgb.h exactly (tests/test_julia_shim.py parses
# both).  Written for BEAST 2.6 / CompScienceMeshes 0.9; it needs no CUDA.jl.
module BEASTGB

using BEAST

export assemble_gpu, GPUConfiguration, GpuWriteBackTrueInstance, GpuWriteBackFalseInstance

const libbeastgb = get(ENV, "LIBBEASTGB", joinpath(@__DIR__, "..", "libbeastgb.so"))

# ---- C structs of include/beastgb.h -------------------------------------------------------
struct BgbOperator
    kind::Int32
    alpha::NTuple{2,Float64}
    beta::NTuple{2,Float64}
    gamma::NTuple{2,Float64}
end

struct BgbSpace
    refspace::Int32
    nv::Int32
    nt::Int32
    nfun::Int32
    vertices::Ptr{Float64}
    triangles::Ptr{Int32}
    fn_index::Ptr{Int32}
    fn_coef::Ptr{Float64}
end

struct BgbQuadStrat
    far_test::Int32
    far_trial::Int32
    near_test::Int32
    near_trial::Int32
    ss_cf::Int32
    ss_ce::Int32
    ss_cv::Int32
end

struct BgbConfig
    device::Int32
    hbm_budget_bytes::Int64
    pinned_ring_bytes::Int64
    tile_config::Int32
    flags::Int32
end

struct BgbStats
    pairs_total::Int64
    pairs_class::NTuple{5,Int64}
    pairs_computed::Int64
    ms_classify::Float64
    ms_singular::Float64
    ms_far::Float64
    ms_copy::Float64
    ms_total::Float64
    ms_pipeline::Float64
    ms_plan::Float64
    out_blocks::Int32
    tile_config::Int32
    kernel_launches::Int32
    schedule::Int32
end

const BGB_PREC_FP64 = Int32(0)
const BGB_PREC_MIXED = Int32(1)
const BGB_OUT_HOST_C64 = Int32(0)
const BGB_OUT_HOST_C32 = Int32(1)
const BGB_REFSPACE_LAGRANGE_C0D1 = Int32(0)
const BGB_REFSPACE_RT = Int32(1)

# ---- the reference's configuration and write-back types ------------------------------------
abstract type GpuWriteBack end
abstract type GpuWriteBackTrue <: GpuWriteBack end
abstract type GpuWriteBackFalse <: GpuWriteBack end
struct GpuWriteBackTrueInstance <: GpuWriteBackTrue end
struct GpuWriteBackFalseInstance <: GpuWriteBackFalse end

struct GPUConfiguration
    writeBackStrategy::Any
    amount_of_gpus::Int
    total_GPU_budget::Int
    InstancedoubleQuadRuleGpuStrategyShouldCalculate::Any
    ShouldCalcInstance::Any
    GPU_budget_pipeline_result::Int
    amount_of_producers::Int
    makeCompexWithGPU::Bool
    backend::Any
    timeLogger::Any
    floatType::Type
    sortOnCPU::Bool
    filename_benchmark::String
    gpu_schedular_print_filename::Union{Nothing,String}
end

# the reference's zero-argument helper (utils/configuration.jl:29-50): 3 GiB budget, FP64
GPUConfiguration() = GPUConfiguration(GpuWriteBackTrueInstance(), 1, 3 * 2^30, nothing, nothing, 24 * 2^30, 16, true,
                                      nothing, nothing, Float64, false, "", nothing)

# ---- marshaling ------------------------------------------------------------------------------
cplx(z) = (Float64(real(z)), Float64(imag(z)))

function field(op, names, default)
    for n in names
        hasproperty(op, n) && return getproperty(op, n)
    end
    return default
end

function bgb_operator(op)
    kind = op isa BEAST.HH3DSingleLayerFDBIO ? 0 :
           op isa BEAST.MWSingleLayer3D ? 1 :
           op isa BEAST.MWDoubleLayer3D ? 2 :
           op isa BEAST.HH3DDoubleLayerFDBIO ? 3 :
           op isa BEAST.HH3DDoubleLayerTransposedFDBIO ? 4 :
           op isa BEAST.HH3DHyperSingularFDBIO ? 5 :
           error("libbeastgb has no kernel for $(typeof(op))")
    gamma = field(op, (:gamma,), 0.0)
    alpha = field(op, (:alpha, :α), 1.0)
    beta = field(op, (:beta, :β), 0.0)
    return BgbOperator(Int32(kind), cplx(alpha), cplx(beta), cplx(gamma))
end

# points of the symmetric triangle rule of each degree BEAST's quadrature strategies name; the
# reference reads 3 and 4 points from BEAST's default far rules (GPU_scheduler.jl:94-95)
const TRIANGLE_RULE_POINTS = Dict(1 => 1, 2 => 3, 3 => 4, 4 => 6, 5 => 7, 6 => 12, 7 => 13)

rule_points(degree) = Int32(get(TRIANGLE_RULE_POINTS, Int(degree)) do
    error("libbeastgb has triangle rules of degree 1..7 only (got $degree)")
end)

function bgb_quadstrat(qs)
    qs isa BgbQuadStrat && return qs
    hasproperty(qs, :outer_rule_far) || error("quadrature strategy $(typeof(qs)) has no counterpart in libbeastgb")
    return BgbQuadStrat(rule_points(qs.outer_rule_far), rule_points(qs.inner_rule_far),
                        rule_points(qs.outer_rule_near), rule_points(qs.inner_rule_near),
                        Int32(qs.sauter_schwab_common_face), Int32(qs.sauter_schwab_common_edge),
                        Int32(qs.sauter_schwab_common_vert))
end

# Per-element tables as the reference packs them (load_parameters.jl:25-54): the chart vertices of
# each element of assemblydata (vertex i of element p is vertex 3(p-1)+i: pairs are classified by
# coordinates, so shared vertices need no common index) and, per local shape, the (function,
# coefficient) pair; one function per local shape.
function pack(X)
    elements, ad, _cells = BEAST.assemblydata(X)
    nt = length(elements)
    V = Matrix{Float64}(undef, 3, 3nt)
    for (p, el) in enumerate(elements), i in 1:3
        V[:, 3(p - 1) + i] = el.vertices[i]
    end
    T = reshape(Int32.(0:(3nt - 1)), 3, nt)
    size(ad.data, 1) == 1 || error("one function per local shape expected (load_parameters.jl:50-54)")
    I = fill(Int32(-1), 3, nt)
    C = zeros(Float64, 3, nt)
    for p in 1:nt, i in 1:size(ad.data, 2)
        m, a = ad.data[1, i, p]
        if m > 0 && a != 0
            I[i, p] = Int32(m - 1)
            C[i, p] = Float64(a)
        end
    end
    rs = BEAST.refspace(X) isa BEAST.RTRefSpace ? BGB_REFSPACE_RT : BGB_REFSPACE_LAGRANGE_C0D1
    return V, T, I, C, rs, Int32(BEAST.numfunctions(X))
end

last_error() = unsafe_string(ccall((:bgb_last_error, libbeastgb), Cstring, ()))
check(rc) = rc == 0 || error("libbeastgb: $(last_error()) (status $rc)")

# ---- the drop-in ------------------------------------------------------------------------------
function assemble_gpu(operator::BEAST.AbstractOperator, test_functions, trial_functions, config,
                      writeBackStrategy::GpuWriteBackFalseInstance;
                      storage_policy = Val{:bandedstorage}, threading = BEAST.Threading{:single},
                      quadstrat = BEAST.defaultquadstrat(operator, test_functions, trial_functions))
    return assemble_bgb(operator, test_functions, trial_functions, config, quadstrat)
end

function assemble_gpu(operator::BEAST.AbstractOperator, test_functions, trial_functions, config,
                      writeBackStrategy::GpuWriteBackTrueInstance;
                      storage_policy = Val{:bandedstorage}, threading = BEAST.Threading{:single},
                      quadstrat = BEAST.defaultquadstrat(operator, test_functions, trial_functions))
    return assemble_bgb(operator, test_functions, trial_functions, config, quadstrat)
end

function assemble_bgb(operator, X, Y, config, quadstrat; device::Integer = 0)
    precision = config.floatType === Float32 ? BGB_PREC_MIXED : BGB_PREC_FP64
    budget = Int64(hasproperty(config, :total_GPU_budget) ? config.total_GPU_budget : 0)
    chunks = max(1, hasproperty(config, :amount_of_gpus) ? Int(config.amount_of_gpus) : 1)
    Vx, Tx, Ix, Cx, rx, nx = pack(X)
    Vy, Ty, Iy, Cy, ry, ny = pack(Y)
    Z = Matrix{ComplexF64}(undef, nx, ny)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    cfg = Ref(BgbConfig(Int32(device), budget, Int64(0), Int32(-1), Int32(0)))
    check(ccall((:bgb_create, libbeastgb), Cint, (Ptr{Ptr{Cvoid}}, Ptr{BgbConfig}), h, cfg))
    try
        GC.@preserve Vx Tx Ix Cx Vy Ty Iy Cy Z begin
            sx = Ref(BgbSpace(rx, Int32(size(Vx, 2)), Int32(size(Tx, 2)), nx, pointer(Vx), pointer(Tx), pointer(Ix),
                              pointer(Cx)))
            sy = Ref(BgbSpace(ry, Int32(size(Vy, 2)), Int32(size(Ty, 2)), ny, pointer(Vy), pointer(Ty), pointer(Iy),
                              pointer(Cy)))
            op = Ref(bgb_operator(operator))
            qs = Ref(bgb_quadstrat(quadstrat))
            stats = Ref{BgbStats}()
            for c in 0:(chunks - 1)                       # row windows, as the reference's chunks
                row0 = div(nx * c, chunks)
                nrows = div(nx * (c + 1), chunks) - row0
                nrows == 0 && continue
                out = pointer(Z) + row0 * sizeof(ComplexF64)  # column-major window, leading dimension nx
                check(ccall((:bgb_assemble, libbeastgb), Cint,
                            (Ptr{Cvoid}, Ptr{BgbOperator}, Ptr{BgbSpace}, Ptr{BgbSpace}, Ptr{BgbQuadStrat}, Int32,
                             Ptr{Cvoid}, Int32, Int64, Int64, Int64, Ptr{Cvoid}, Ptr{BgbStats}),
                            h[], op, sx, sy, qs, precision, out, BGB_OUT_HOST_C64, Int64(nx), Int64(row0),
                            Int64(nrows), C_NULL, stats))
            end
        end
    finally
        ccall((:bgb_destroy, libbeastgb), Cint, (Ptr{Cvoid},), h[])
    end
    return Z
end

end # module
