"""
    BEASTGPU

Julia side of the GB300 assembly/solve library: `ccall` bindings of `libbeastgpu.so`
(include/beastgpu.h) and the methods that route BEAST's `assemble` through it.

    using BEAST, BEASTGPU
    T = assemble(Maxwell3D.singlelayer(wavenumber=2.0), X, X;
                 quadstrat=BEASTGPU.GPUQStrat(BEAST.defaultquadstrat))
    u = BEASTGPU.solve(T, e)                       # LU on the device

The matrix layout is BEAST's own (`Matrix{ComplexF64}`, rows = test dofs in `tfs.fns`
order), so the result drops into `T \\ e`, GMRES or any later BEAST code unchanged.
"""
module BEASTGPU

using BEAST
using LinearAlgebra

const libbeastgpu = get(ENV, "BEASTGPU_LIB", joinpath(@__DIR__, "..", "beastgpu", "libbeastgpu.so"))

# ---- enums (include/beastgpu.h)
const MW_SL, MW_DL, MW_NXDL, HH_SL, HH_DL, HH_DLT = 1, 2, 3, 4, 5, 6
const P0, P1, RT = 0, 1, 2
const QS_WILTON_SAUTER, QS_SAUTER, QS_DOUBLENUM = 1, 2, 3
const FP64, MIXED, MIXED_ACCURATE = 0, 1, 2
const C128, C64 = 0, 1
const HOST, DEVICE = 0, 1

struct OpDesc
    kind::Cint
    gamma_re::Cdouble; gamma_im::Cdouble
    alpha_re::Cdouble; alpha_im::Cdouble
    beta_re::Cdouble;  beta_im::Cdouble
end

struct QsDesc
    kind::Cint
    outer_far::Cint; inner_far::Cint; outer_near::Cint; inner_near::Cint
    ss_tetr::Cint; ss_face::Cint; ss_edge::Cint; ss_vert::Cint
end

function check(ctx, rc)
    rc == 0 && return nothing
    buf = Vector{UInt8}(undef, 1024)
    ccall((:beast_last_error, libbeastgpu), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t), ctx, buf, length(buf))
    error("beastgpu error $rc: " * unsafe_string(pointer(buf)))
end

mutable struct Context
    ptr::Ptr{Cvoid}
    function Context(device::Integer=0)
        r = Ref{Ptr{Cvoid}}(C_NULL)
        rc = ccall((:beast_ctx_create, libbeastgpu), Cint, (Cint, Ptr{Ptr{Cvoid}}), device, r)
        rc == 0 || error("beastgpu: cannot create a context on device $device (code $rc)")
        c = new(r[])
        finalizer(c -> ccall((:beast_ctx_destroy, libbeastgpu), Cint, (Ptr{Cvoid},), c.ptr), c)
        return c
    end
end

const CTX = Ref{Union{Nothing,Context}}(nothing)
context() = (CTX[] === nothing && (CTX[] = Context(0)); CTX[])

"""
    GPUQStrat(inner; precision=FP64)

Quadrature strategy wrapper: the rule orders come from `inner` (the reference's strategy
object or function); the work runs on the GPU.
"""
struct GPUQStrat{Q}
    inner::Q
    precision::Int
end
GPUQStrat(inner; precision=FP64) = GPUQStrat(inner, precision)

qsdesc(qs::BEAST.DoubleNumWiltonSauterQStrat) = QsDesc(QS_WILTON_SAUTER,
    qs.outer_rule_far, qs.inner_rule_far, qs.outer_rule_near, qs.inner_rule_near,
    qs.sauter_schwab_common_tetr, qs.sauter_schwab_common_face,
    qs.sauter_schwab_common_edge, qs.sauter_schwab_common_vert)
qsdesc(qs::BEAST.DoubleNumSauterQstrat) = QsDesc(QS_SAUTER,
    qs.outer_rule, qs.inner_rule, qs.outer_rule, qs.inner_rule,
    qs.sauter_schwab_common_tetr, qs.sauter_schwab_common_face,
    qs.sauter_schwab_common_edge, qs.sauter_schwab_common_vert)
qsdesc(qs::BEAST.DoubleNumQStrat) = QsDesc(QS_DOUBLENUM, qs.outer_rule, qs.inner_rule, 0, 0, 0, 0, 0, 0)

_c(x) = ComplexF64(x)
opdesc(op::BEAST.MWSingleLayer3D) = (g = _c(BEAST.gamma(op)); a = _c(op.α); b = _c(op.β);
    OpDesc(MW_SL, real(g), imag(g), real(a), imag(a), real(b), imag(b)))
opdesc(op::BEAST.MWDoubleLayer3D) = (g = _c(BEAST.gamma(op)); OpDesc(MW_DL, real(g), imag(g), 1, 0, 0, 0))
opdesc(op::BEAST.DoubleLayerRotatedMW3D) = (g = _c(BEAST.gamma(op)); OpDesc(MW_NXDL, real(g), imag(g), 1, 0, 0, 0))
opdesc(op::BEAST.HH3DSingleLayerFDBIO) = (g = _c(BEAST.gamma(op)); a = _c(op.alpha);
    OpDesc(HH_SL, real(g), imag(g), real(a), imag(a), 0, 0))
opdesc(op::BEAST.HH3DDoubleLayerFDBIO) = (g = _c(BEAST.gamma(op)); a = _c(op.alpha);
    OpDesc(HH_DL, real(g), imag(g), real(a), imag(a), 0, 0))
opdesc(op::BEAST.HH3DDoubleLayerTransposedFDBIO) = (g = _c(BEAST.gamma(op)); a = _c(op.alpha);
    OpDesc(HH_DLT, real(g), imag(g), real(a), imag(a), 0, 0))

spacekind(::BEAST.RTRefSpace) = RT
spacekind(::BEAST.LagrangeRefSpace{T,0,3}) where {T} = P0
spacekind(::BEAST.LagrangeRefSpace{T,1,3}) where {T} = P1

# resident copies of meshes and spaces, keyed by object identity
const SPACES = IdDict{Any,Ptr{Cvoid}}()
const MESHES = IdDict{Any,Ptr{Cvoid}}()

function mesh_handle(ctx, mesh)
    get!(MESHES, mesh) do
        V = reduce(hcat, mesh.vertices)                       # 3 x nv Float64
        F = Int32.(reduce(hcat, [collect(c) for c in mesh.faces]))  # 3 x nc, 1-based
        r = Ref{Ptr{Cvoid}}(C_NULL)
        check(ctx.ptr, ccall((:beast_mesh_upload, libbeastgpu), Cint,
            (Ptr{Cvoid}, Ptr{Float64}, Int64, Ptr{Int32}, Int64, Cint, Ptr{Ptr{Cvoid}}),
            ctx.ptr, V, size(V, 2), F, size(F, 2), 1, r))
        r[]
    end
end

function space_handle(ctx, X)
    get!(SPACES, X) do
        charts, ad, a2g = BEAST.assemblydata(X)
        data = ad.data                                        # (maxfn, nshapes, ncells) of (Int, T)
        dof = Int64[d[1] for d in data]                       # Julia memory order == [c][r][k]
        coeff = Float64[d[2] for d in data]
        mh = mesh_handle(ctx, BEAST.geometry(X))
        r = Ref{Ptr{Cvoid}}(C_NULL)
        check(ctx.ptr, ccall((:beast_space_upload, libbeastgpu), Cint,
            (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Int64, Ptr{Int64}, Cint, Cint, Ptr{Int64}, Ptr{Float64},
             Int64, Cint, Ptr{Ptr{Cvoid}}),
            ctx.ptr, mh, spacekind(BEAST.refspace(X)), length(a2g), Int64.(a2g), size(data, 1),
            size(data, 2), dof, coeff, BEAST.numfunctions(X), 1, r))
        r[]
    end
end

"""
Dense store lowered to arguments: `Z[row_off + m, col_off + n] += coeff * a(m, n)`.
"""
struct DenseStore
    Z::Matrix{ComplexF64}
    row_off::Int
    col_off::Int
    coeff::ComplexF64
end

function assemble_into!(store::DenseStore, op, tfs, bfs, qs::GPUQStrat; accumulate=true)
    ctx = context()
    inner = qs.inner isa Function ? qs.inner(op, tfs, bfs) : qs.inner
    od = Ref(opdesc(op)); qd = Ref(qsdesc(inner))
    Z = store.Z
    GC.@preserve Z begin
        check(ctx.ptr, ccall((:beast_assemble, libbeastgpu), Cint,
            (Ptr{Cvoid}, Ref{OpDesc}, Ref{QsDesc}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{ComplexF64},
             Int64, Cint, Cint, Int64, Int64, Cdouble, Cdouble, Cint),
            ctx.ptr, od, qd, space_handle(ctx, tfs), space_handle(ctx, bfs), qs.precision, Z,
            size(Z, 1), C128, HOST, store.row_off, store.col_off, real(store.coeff),
            imag(store.coeff), accumulate ? 1 : 0))
    end
    return Z
end

# `assemble(op, X, Y; quadstrat=GPUQStrat(...))` for the supported integral operators
const GPUOps = Union{BEAST.MWSingleLayer3D, BEAST.MWDoubleLayer3D, BEAST.DoubleLayerRotatedMW3D,
                     BEAST.HH3DSingleLayerFDBIO, BEAST.HH3DDoubleLayerFDBIO,
                     BEAST.HH3DDoubleLayerTransposedFDBIO}

function BEAST.assemble(op::GPUOps, tfs::BEAST.Space, bfs::BEAST.Space; quadstrat::GPUQStrat, kwargs...)
    Z = zeros(ComplexF64, BEAST.numfunctions(tfs), BEAST.numfunctions(bfs))
    assemble_into!(DenseStore(Z, 0, 0, one(ComplexF64)), op, tfs, bfs, quadstrat; accumulate=false)
end

"""
    blockassembler(op, tfs, bfs, qs::GPUQStrat) -> (test_ids, trial_ids, store) -> nothing

`BEAST.blockassembler` on the device: the block a(test_ids[i], trial_ids[j]) is assembled
into a block-local buffer by `beast_assemble_block` and handed to `store(v, i, j)` entry by
entry, like the reference's functor (block-local 1-based indices).
"""
function blockassembler(op::GPUOps, tfs::BEAST.Space, bfs::BEAST.Space, qs::GPUQStrat)
    ctx = context()
    inner = qs.inner isa Function ? qs.inner(op, tfs, bfs) : qs.inner
    od = Ref(opdesc(op)); qd = Ref(qsdesc(inner))
    return function (test_ids, trial_ids, store)
        I = collect(Int64, test_ids); J = collect(Int64, trial_ids)
        B = zeros(ComplexF64, length(I), length(J))
        GC.@preserve I J B begin
            check(ctx.ptr, ccall((:beast_assemble_block, libbeastgpu), Cint,
                (Ptr{Cvoid}, Ref{OpDesc}, Ref{QsDesc}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Int64}, Int64,
                 Ptr{Int64}, Int64, Cint, Cint, Ptr{ComplexF64}, Int64, Cint, Cint, Cdouble, Cdouble,
                 Cint),
                ctx.ptr, od, qd, space_handle(ctx, tfs), space_handle(ctx, bfs), I, length(I), J,
                length(J), 1, qs.precision, B, length(I), C128, HOST, 1.0, 0.0, 0))
        end
        for j in axes(B, 2), i in axes(B, 1)
            store(B[i, j], i, j)
        end
        return nothing
    end
end

"""
    solve(Z, b; precision=FP64, tol=1e-12) -> x

`Z \\ b` on the device: FP64 LU, or (MIXED, or MIXED_ACCURATE -- the same here) FP32 LU
with tensor-core updates and FP64 iterative refinement to `tol` against `Z` as given (an FP64
assembly, `GPUQStrat(inner; precision=FP64)`, then gives the FP64 solution to the tolerance).
"""
function solve(Z::Matrix{ComplexF64}, b::Vector{ComplexF64}; precision=FP64, tol=1e-12, maxiter=30)
    ctx = context()
    n = size(Z, 1)
    x = similar(b)
    it = Ref{Cint}(0); res = Ref{Cdouble}(0)
    dZ = device_copy(Z)
    try
        GC.@preserve b x begin
            check(ctx.ptr, ccall((:beast_solve_dense, libbeastgpu), Cint,
                (Ptr{Cvoid}, Int64, Ptr{Cvoid}, Int64, Cint, Cint, Ptr{ComplexF64}, Ptr{ComplexF64},
                 Int64, Cint, Cdouble, Cint, Ref{Cint}, Ref{Cdouble}),
                ctx.ptr, n, dZ, n, C128, precision, b, x, 1, HOST, tol, maxiter, it, res))
        end
    finally
        ccall((:cudaFree, "libcudart"), Cint, (Ptr{Cvoid},), dZ)
    end
    return x
end

"""
    last_factor_mode()

Factorisation behind the last `solve`: 0 LU with partial pivoting, 1 unpivoted LU (mixed),
2 symmetric LDL^T-type (mixed, near complex-symmetric matrix such as the Galerkin EFIE).
"""
function last_factor_mode()
    ctx = context()
    m = Ref{Cint}(-1)
    check(ctx.ptr, ccall((:beast_last_factor_mode, libbeastgpu), Cint, (Ptr{Cvoid}, Ref{Cint}), ctx.ptr, m))
    return Int(m[])
end

# device copy of a host matrix through the CUDA runtime (no CUDA.jl dependency)
function device_copy(Z)
    p = Ref{Ptr{Cvoid}}(C_NULL)
    bytes = sizeof(Z)
    ccall((:cudaMalloc, "libcudart"), Cint, (Ptr{Ptr{Cvoid}}, Csize_t), p, bytes) == 0 ||
        error("cudaMalloc of $bytes bytes failed")
    ccall((:cudaMemcpy, "libcudart"), Cint, (Ptr{Cvoid}, Ptr{ComplexF64}, Csize_t, Cint),
          p[], Z, bytes, 1) == 0 || error("cudaMemcpy failed")
    return p[]
end

end # module
