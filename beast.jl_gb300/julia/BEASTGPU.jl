"""
    BEASTGPU

Julia side of the GB300 assembly/solve library: `ccall` bindings of `libbeastgpu.so`
(include/beastgpu.h) and the methods that route BEAST's own assembly through it.

The GPU is asked for through BEAST's storage trait, so nothing changes for calls that do
not ask for it:

    using BEAST, BEASTGPU
    T = assemble(Maxwell3D.singlelayer(wavenumber=2.0), X, X; storage_policy=Val{:gpu})
    Z = assemble(nxK - 0.5Id, X, X; storage_policy=Val{:gpu})   # linear combinations too
    u = BEASTGPU.solve(T, e)                                     # dense solve on the device
    u = BEASTGPU.solve(mfie)                                     # `solve(eq)` of @discretise

`assemble` (src/operator.jl:100-116) calls `allocatestorage(op, X, Y, storage_policy)`
(src/operator.jl:168-183); for the policies `Val{:gpu}` (FP64), `Val{:gpu_mixed_accurate}`,
`Val{:gpu_mixed_balanced}` and `Val{:gpu_mixed}` this returns a `DenseStore` instead of the `store(v,m,n) = (Z[m,n] += v)`
closure.  `assemble!` (src/operator.jl:207-357) then dispatches on the store's type:

  * integral operators of the supported kinds on RT / P0 / P1 spaces with a supported
    strategy -> `beast_assemble` (the store's offsets and coefficient become its arguments);
  * Identity / NCross on RT x RT of one mesh -> `beast_assemble_local`;
  * linear combinations -> each term with its coefficient folded into the store;
  * transposed operators -> the operator on the swapped spaces, added transposed;
  * direct-product spaces -> each factor with its row / column offset;
  * anything else -> the reference's own method, which calls the store like its closure
    (`DenseStore` is callable: `store(v, m, n)` adds `coeff * v` at the offset entry).

The matrix layout is BEAST's own (`Matrix{ComplexF64}`, rows = test dofs in `tfs.fns`
order), so the result drops into `T \\ e`, GMRES or any later BEAST code unchanged.
"""
module BEASTGPU

using BEAST
using CompScienceMeshes
using LinearAlgebra

const libbeastgpu = get(ENV, "BEASTGPU_LIB", joinpath(@__DIR__, "..", "beastgpu", "libbeastgpu.so"))

# ---- enums (include/beastgpu.h)
const MW_SL, MW_DL, MW_NXDL, HH_SL, HH_DL, HH_DLT = 1, 2, 3, 4, 5, 6
const P0, P1, RT = 0, 1, 2
const QS_WILTON_SAUTER, QS_SAUTER, QS_DOUBLENUM = 1, 2, 3
const QS_TEST_REFINES_TRIAL, QS_TRIAL_REFINES_TEST = 4, 5
const FP64, MIXED, MIXED_ACCURATE, MIXED_BALANCED = 0, 1, 2, 3
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

# ---- what the device path covers
const GPUOps = Union{BEAST.MWSingleLayer3D, BEAST.MWDoubleLayer3D, BEAST.DoubleLayerRotatedMW3D,
                     BEAST.HH3DSingleLayerFDBIO, BEAST.HH3DDoubleLayerFDBIO,
                     BEAST.HH3DDoubleLayerTransposedFDBIO}

qsdesc(qs::BEAST.DoubleNumWiltonSauterQStrat) = QsDesc(QS_WILTON_SAUTER,
    qs.outer_rule_far, qs.inner_rule_far, qs.outer_rule_near, qs.inner_rule_near,
    qs.sauter_schwab_common_tetr, qs.sauter_schwab_common_face,
    qs.sauter_schwab_common_edge, qs.sauter_schwab_common_vert)
qsdesc(qs::BEAST.DoubleNumSauterQstrat) = QsDesc(QS_SAUTER,
    qs.outer_rule, qs.inner_rule, qs.outer_rule, qs.inner_rule,
    qs.sauter_schwab_common_tetr, qs.sauter_schwab_common_face,
    qs.sauter_schwab_common_edge, qs.sauter_schwab_common_vert)
qsdesc(qs::BEAST.DoubleNumQStrat) = QsDesc(QS_DOUBLENUM, qs.outer_rule, qs.inner_rule, 0, 0, 0, 0, 0, 0)
qsdesc(qs) = nothing   # any other strategy: the reference's own assembly

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
spacekind(::Any) = nothing

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
    DenseStore(Z, row_off, col_off, coeff, precision)

The dense store of `allocatestorage` (src/operator.jl:168-183) lowered to arguments: entry
(m, n) of a block goes to `Z[row_off + m, col_off + n] += coeff * v`.  The device path passes
the four fields to the C ABI; every other method calls it like the reference's closure.
"""
struct DenseStore
    Z::Matrix{ComplexF64}
    row_off::Int
    col_off::Int
    coeff::ComplexF64
    precision::Int
end
(s::DenseStore)(v, m, n) = (s.Z[s.row_off + m, s.col_off + n] += s.coeff * v; nothing)
scaled(s::DenseStore, a) = DenseStore(s.Z, s.row_off, s.col_off, s.coeff * a, s.precision)
shifted(s::DenseStore, dm, dn) = DenseStore(s.Z, s.row_off + dm, s.col_off + dn, s.coeff, s.precision)

const GPUPolicy = Union{Type{Val{:gpu}}, Type{Val{:gpu_mixed_accurate}}, Type{Val{:gpu_mixed_balanced}},
                        Type{Val{:gpu_mixed}}}
policy_precision(::Type{Val{:gpu}}) = FP64
policy_precision(::Type{Val{:gpu_mixed_accurate}}) = MIXED_ACCURATE
policy_precision(::Type{Val{:gpu_mixed_balanced}}) = MIXED_BALANCED
policy_precision(::Type{Val{:gpu_mixed}}) = MIXED

function BEAST.allocatestorage(op::BEAST.AbstractOperator, tfs, bfs, policy::GPUPolicy,
                               longdelays_trait=nothing)
    Z = zeros(ComplexF64, BEAST.numfunctions(tfs), BEAST.numfunctions(bfs))
    return () -> Z, DenseStore(Z, 0, 0, one(ComplexF64), policy_precision(policy))
end

function gpu_assemble!(store::DenseStore, op, tfs, bfs, qd::QsDesc)
    ctx = context()
    od = Ref(opdesc(op)); qr = Ref(qd)
    Z = store.Z
    GC.@preserve Z begin
        check(ctx.ptr, ccall((:beast_assemble, libbeastgpu), Cint,
            (Ptr{Cvoid}, Ref{OpDesc}, Ref{QsDesc}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{ComplexF64},
             Int64, Cint, Cint, Int64, Int64, Cdouble, Cdouble, Cint),
            ctx.ptr, od, qr, space_handle(ctx, tfs), space_handle(ctx, bfs), store.precision, Z,
            size(Z, 1), C128, HOST, store.row_off, store.col_off, real(store.coeff),
            imag(store.coeff), 1))
    end
    return nothing
end

on_device(tfs, bfs) = spacekind(BEAST.refspace(tfs)) !== nothing &&
    spacekind(BEAST.refspace(bfs)) !== nothing && BEAST.geometry(tfs) === BEAST.geometry(bfs)

# the children of every cell of `coarse` in its refinement `fine` (CompScienceMeshes.parent /
# children, as rules/testrefinestrialqrule.jl:23-24 reads them), registered once per mesh
const CHILDREN = IdDict{Any,Bool}()
function register_children!(ctx, coarse, fine)
    get!(CHILDREN, coarse) do
        pm = CompScienceMeshes.parent(fine)
        kids = [collect(CompScienceMeshes.children(pm, c)) for c in 1:length(coarse)]
        nchild = length(kids[1])
        all(length(k) == nchild for k in kids) || error("refinement with a varying number of children")
        CV = Float64[]
        for k in kids, p in k, v in CompScienceMeshes.chart(fine, p).vertices
            append!(CV, v)
        end
        check(ctx.ptr, ccall((:beast_mesh_set_children, libbeastgpu), Cint,
            (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Float64}), ctx.ptr, mesh_handle(ctx, coarse), nchild, CV))
        true
    end
end

# RT x RT across a barycentric refinement with the Wilton-Sauter strategy: the strategy the
# reference's assemble! wraps it in (src/operator.jl:256-262), children registered; else nothing
function refines_qsdesc(ctx, tfs, bfs, qs)
    qs isa BEAST.DoubleNumWiltonSauterQStrat || return nothing
    (spacekind(BEAST.refspace(tfs)) == RT && spacekind(BEAST.refspace(bfs)) == RT) || return nothing
    tg, bg = BEAST.geometry(tfs), BEAST.geometry(bfs)
    kind = CompScienceMeshes.refines(tg, bg) ? QS_TEST_REFINES_TRIAL :
           CompScienceMeshes.refines(bg, tg) ? QS_TRIAL_REFINES_TEST : 0
    kind == 0 && return nothing
    kind == QS_TEST_REFINES_TRIAL ? register_children!(ctx, bg, tg) : register_children!(ctx, tg, bg)
    d = qsdesc(qs)
    return QsDesc(kind, d.outer_far, d.inner_far, d.outer_near, d.inner_near, d.ss_tetr, d.ss_face,
                  d.ss_edge, d.ss_vert)
end

# integral operators (src/operator.jl:207-281, one method per threading trait so that each
# is at least as specific as the reference's in every argument)
for T in (:multi, :single, :cellcoloring)
    @eval function BEAST.assemble!(op::GPUOps, tfs::BEAST.Space, bfs::BEAST.Space, store::DenseStore,
                                   threading::Type{BEAST.Threading{$(QuoteNode(T))}};
                                   quadstrat=BEAST.defaultquadstrat, kwargs...)
        qs = quadstrat(op, tfs, bfs)
        qd = qsdesc(qs)
        if qd !== nothing && on_device(tfs, bfs)
            return gpu_assemble!(store, op, tfs, bfs, qd)
        end
        qr = BEAST.geometry(tfs) === BEAST.geometry(bfs) ? nothing : refines_qsdesc(context(), tfs, bfs, qs)
        qr !== nothing && return gpu_assemble!(store, op, tfs, bfs, qr)
        return invoke(BEAST.assemble!, Tuple{BEAST.Operator, BEAST.Space, BEAST.Space, Any,
                                             Type{BEAST.Threading{$(QuoteNode(T))}}},
                      op, tfs, bfs, store, threading; quadstrat=(a...) -> qs, kwargs...)
    end
end

# Identity / NCross on RT x RT of one mesh (src/identityop.jl:7-24, src/localop.jl:60-110)
for T in (:multi, :single)
    @eval function BEAST.assemble!(op::Union{BEAST.Identity, BEAST.NCross}, tfs::BEAST.RTBasis,
                                   bfs::BEAST.RTBasis, store::DenseStore,
                                   threading::Type{BEAST.Threading{$(QuoteNode(T))}};
                                   quadstrat=BEAST.defaultquadstrat, kwargs...)
        if BEAST.geometry(tfs) !== BEAST.geometry(bfs)
            return invoke(BEAST.assemble!, Tuple{BEAST.LocalOperator, BEAST.Space, BEAST.Space, Any,
                                                 Type{BEAST.Threading{$(QuoteNode(T))}}},
                          op, tfs, bfs, store, threading; quadstrat, kwargs...)
        end
        ctx = context()
        Z = store.Z
        GC.@preserve Z begin
            check(ctx.ptr, ccall((:beast_assemble_local, libbeastgpu), Cint,
                (Ptr{Cvoid}, Cint, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{ComplexF64}, Int64, Cint, Cint,
                 Int64, Int64, Cdouble, Cdouble),
                ctx.ptr, op isa BEAST.Identity ? 0 : 1, space_handle(ctx, tfs), space_handle(ctx, bfs), 6,
                Z, size(Z, 1), C128, HOST, store.row_off, store.col_off, real(store.coeff),
                imag(store.coeff)))
        end
        return nothing
    end
end

# linear combinations (src/operator.jl:294-304): the coefficient folds into the store
function BEAST.assemble!(op::BEAST.LinearCombinationOfOperators, tfs::BEAST.Space, bfs::BEAST.Space,
                         store::DenseStore, threading=BEAST.Threading{:multi};
                         quadstrat=BEAST.defaultquadstrat, kwargs...)
    for (a, A) in zip(op.coeffs, op.ops)
        BEAST.assemble!(A, tfs, bfs, scaled(store, a), threading; quadstrat, kwargs...)
    end
end

# transposed operators (src/operator.jl:284-291): the operator on the swapped spaces, added
# transposed into the store's block
function BEAST.assemble!(op::BEAST.TransposedOperator, tfs::BEAST.Space, bfs::BEAST.Space,
                         store::DenseStore,
                         threading::Type{BEAST.Threading{:multi}}=BEAST.Threading{:multi};
                         quadstrat=BEAST.defaultquadstrat(op, tfs, bfs), kwargs...)
    nt, nb = BEAST.numfunctions(tfs), BEAST.numfunctions(bfs)
    W = zeros(ComplexF64, nb, nt)
    BEAST.assemble!(op.op, bfs, tfs, DenseStore(W, 0, 0, one(ComplexF64), store.precision), threading;
                    quadstrat, kwargs...)
    rows = store.row_off .+ (1:nt)
    cols = store.col_off .+ (1:nb)
    store.Z[rows, cols] .+= store.coeff .* transpose(W)
    return nothing
end

# direct-product spaces (src/operator.jl:319-357): each factor at its offset
function BEAST.assemble!(op::BEAST.AbstractOperator, tfs::BEAST.DirectProductSpace, bfs::BEAST.Space,
                         store::DenseStore, threading=BEAST.Threading{:multi};
                         quadstrat=BEAST.defaultquadstrat(op, tfs[1], bfs), kwargs...)
    m = 0
    for s in tfs.factors
        BEAST.assemble!(op, s, bfs, shifted(store, m, 0), threading; quadstrat, kwargs...)
        m += BEAST.numfunctions(s)
    end
end

function BEAST.assemble!(op::BEAST.AbstractOperator, tfs::BEAST.Space, bfs::BEAST.DirectProductSpace,
                         store::DenseStore, threading=BEAST.Threading{:multi};
                         quadstrat=BEAST.defaultquadstrat(op, tfs, bfs[1]), kwargs...)
    n = 0
    for s in bfs.factors
        BEAST.assemble!(op, tfs, s, shifted(store, 0, n), threading; quadstrat, kwargs...)
        n += BEAST.numfunctions(s)
    end
end

function BEAST.assemble!(op::BEAST.AbstractOperator, tfs::BEAST.DirectProductSpace,
                         bfs::BEAST.DirectProductSpace, store::DenseStore, threading=BEAST.Threading{:multi};
                         quadstrat=BEAST.defaultquadstrat(op, tfs[1], bfs[1]), kwargs...)
    m = 0
    for s in tfs.factors
        BEAST.assemble!(op, s, bfs, shifted(store, m, 0), threading; quadstrat, kwargs...)
        m += BEAST.numfunctions(s)
    end
end

"""
    blockassembler(op, tfs, bfs; precision=FP64, quadstrat=BEAST.defaultquadstrat)
        -> (test_ids, trial_ids, store) -> nothing

`BEAST.blockassembler` on the device: the block a(test_ids[i], trial_ids[j]) is assembled
into a block-local buffer by `beast_assemble_block` and handed to `store(v, i, j)` entry by
entry, like the reference's functor (block-local 1-based indices).
"""
function blockassembler(op::GPUOps, tfs::BEAST.Space, bfs::BEAST.Space; precision=FP64,
                        quadstrat=BEAST.defaultquadstrat)
    ctx = context()
    qd = qsdesc(quadstrat(op, tfs, bfs))
    qd === nothing && error("blockassembler: quadrature strategy not available on the device")
    od = Ref(opdesc(op)); qr = Ref(qd)
    return function (test_ids, trial_ids, store)
        I = collect(Int64, test_ids); J = collect(Int64, trial_ids)
        B = zeros(ComplexF64, length(I), length(J))
        GC.@preserve I J B begin
            check(ctx.ptr, ccall((:beast_assemble_block, libbeastgpu), Cint,
                (Ptr{Cvoid}, Ref{OpDesc}, Ref{QsDesc}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Int64}, Int64,
                 Ptr{Int64}, Int64, Cint, Cint, Ptr{ComplexF64}, Int64, Cint, Cint, Cdouble, Cdouble,
                 Cint),
                ctx.ptr, od, qr, space_handle(ctx, tfs), space_handle(ctx, bfs), I, length(I), J,
                length(J), 1, precision, B, length(I), C128, HOST, 1.0, 0.0, 0))
        end
        for j in axes(B, 2), i in axes(B, 1)
            store(B[i, j], i, j)
        end
        return nothing
    end
end

"""
    solve(Z, b; precision=MIXED_ACCURATE, tol=1e-10) -> x

`Z \\ b` on the device: FP64 LU (`FP64`), or a complex FP32 factorisation with tensor-core
updates and FP64 iterative refinement to `tol` against `Z` as given (`MIXED`,
`MIXED_ACCURATE`, `MIXED_BALANCED`: for an FP64 `Z` the FP64 solution to the tolerance).
"""
function solve(Z::Matrix{ComplexF64}, b::Vector{ComplexF64}; precision=MIXED_ACCURATE, tol=1e-10,
               maxiter=30)
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
    solve(eq; precision=MIXED_ACCURATE, tol=1e-10)

`solve(eq)` of src/solvers/lusolver.jl:9-39 for an equation from `@discretise`: the right-hand
side as in the reference, every operator term of the left-hand side assembled on the device
(`materialize` of src/solvers/solver.jl:226), the dense solve on the device.
"""
function solve(eq; precision=MIXED_ACCURATE, tol=1e-10)
    X = BEAST._spacedict_to_directproductspace(eq.test_space_dict)
    Y = BEAST._spacedict_to_directproductspace(eq.trial_space_dict)
    b = BEAST.assemble(eq.equation.rhs, X)
    policy = precision == FP64 ? Val{:gpu} : precision == MIXED ? Val{:gpu_mixed} :
             precision == MIXED_BALANCED ? Val{:gpu_mixed_balanced} : Val{:gpu_mixed_accurate}
    materialize = (a, x, y; kw...) -> BEAST.assemble(a, x, y; storage_policy=policy, kw...)
    Z = BEAST.assemble(eq.equation.lhs, X, Y; materialize)
    u = solve(Matrix{ComplexF64}(Matrix(Z)), Vector{ComplexF64}(Vector(b)); precision, tol)
    ax = BEAST.nestedrange(Y, 1, BEAST.numfunctions)
    return BEAST.BlockedVector(u, (ax,))
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
