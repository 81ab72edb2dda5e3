# TenetGB300.jl — Julia binding of libtenetgb.so (C ABI: include/tenet_gb300.h).
#
# Tenet.jl never computes itself: every contraction, QR, SVD and simple update goes
# through Muscle.jl on `Tangles.Tensor{T,N,A}` values, dispatched on the array type `A`.
# This module adds a device array type `GB300Array` and, for `Tensor`s backed by it, the
# Muscle methods Tenet calls — `binary_einsum` (also as the Hadamard product of a real Λ
# and a site), `tensor_qr_thin`, `tensor_svd_thin`, `simple_update`, `hadamard`, `fuse` —
# plus `conj` and `norm`, so Tenet's call sites (src/Operations/canonize.jl:41-100,
# simple_update.jl:34,53-64, overlap.jl:26-46, evolve.jl:35-39) reach the sm_103a kernels
# unchanged once the sites' arrays are `GB300Array`s (`Tensor(GB300Array(a), inds)`).
#
# It also exposes the device-resident MPS (`GB300MPS`), which keeps whole sweeps on the
# GPU (canonize!, compress!, simple_update!, evolve!, overlap, norm) — the fast path.
#
# No Julia toolchain exists in the build container, so this file is shipped unexecuted;
# the same entry points are exercised from Python (tenet.jl_gb300/tenetgb) by the tests.
module TenetGB300

using LinearAlgebra
import Muscle
using Tangles: Tensor, Index, inds

const libtenetgb = get(ENV, "TENETGB_LIB", joinpath(@__DIR__, "..", "tenetgb", "_lib", "libtenetgb.so"))

const TN_OK = Int32(0)
const TN_C64 = Int32(3)
const TN_C32 = Int32(2)
const TN_F64 = Int32(1)
const TN_F32 = Int32(0)
const TN_PREC_NATIVE = Int32(0)
const TN_PREC_MIXED = Int32(1)

dtype(::Type{ComplexF64}) = TN_C64
dtype(::Type{ComplexF32}) = TN_C32
dtype(::Type{Float64}) = TN_F64
dtype(::Type{Float32}) = TN_F32

# ---- context ---------------------------------------------------------------------------
mutable struct Context
    h::Ptr{Cvoid}
end

function check(st::Int32, ctx::Ptr{Cvoid})
    st == TN_OK && return nothing
    msg = unsafe_string(ccall((:tn_last_error_string, libtenetgb), Cstring, (Ptr{Cvoid},), ctx))
    st == 1 && throw(ArgumentError(msg))          # TN_EINVAL ↔ Tenet's @argcheck
    st == 2 && throw(OutOfMemoryError())           # TN_ENOMEM
    throw(ErrorException("libtenetgb status $st: $msg"))
end

function Context(device::Integer=0)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:tn_create, libtenetgb), Int32, (Ref{Ptr{Cvoid}}, Cint), r, device), C_NULL)
    ctx = Context(r[])
    finalizer(c -> ccall((:tn_destroy, libtenetgb), Int32, (Ptr{Cvoid},), c.h), ctx)
    return ctx
end

const DEFAULT = Ref{Union{Nothing,Context}}(nothing)
default_context() = something(DEFAULT[], (DEFAULT[] = Context(0)))

# ---- device array ----------------------------------------------------------------------
"""
    GB300Array{T,N}

Dense column-major device array owned by a libtenetgb context (tn_alloc / tn_free).
"""
mutable struct GB300Array{T,N} <: AbstractArray{T,N}
    ptr::Ptr{Cvoid}
    dims::NTuple{N,Int}
    ctx::Context
end

Base.size(a::GB300Array) = a.dims
Base.getindex(::GB300Array, ::Int...) = error("GB300Array: scalar indexing is disabled; use Array(a)")
# the scalar a full contraction ends in (overlap.jl:36-50 returns a 0-dimensional tensor)
Base.getindex(a::GB300Array{T,0}) where {T} = only(Array(a))

function GB300Array{T}(::UndefInitializer, dims::NTuple{N,Int}; ctx=default_context()) where {T,N}
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:tn_alloc, libtenetgb), Int32, (Ptr{Cvoid}, Csize_t, Ref{Ptr{Cvoid}}), ctx.h, max(1, prod(dims) * sizeof(T)), r), ctx.h)
    a = GB300Array{T,N}(r[], dims, ctx)
    finalizer(x -> ccall((:tn_free, libtenetgb), Int32, (Ptr{Cvoid}, Ptr{Cvoid}), x.ctx.h, x.ptr), a)
    return a
end

function GB300Array(x::Array{T,N}; ctx=default_context()) where {T,N}
    a = GB300Array{T}(undef, size(x); ctx)
    GC.@preserve x check(ccall((:tn_memcpy_h2d, libtenetgb), Int32, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Csize_t), ctx.h, a.ptr, pointer(x), sizeof(x)), ctx.h)
    return a
end

function Base.Array(a::GB300Array{T,N}) where {T,N}
    x = Array{T,N}(undef, a.dims)
    GC.@preserve x check(ccall((:tn_memcpy_d2h, libtenetgb), Int32, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Csize_t), a.ctx.h, pointer(x), a.ptr, sizeof(x)), a.ctx.h)
    return x
end

# ---- Muscle-level entry points ---------------------------------------------------------
# tn_tensor {int32 rank; int64 dims[16]; int32 modes[16]; void* data}
struct TnTensor
    rank::Int32
    dims::NTuple{16,Int64}
    modes::NTuple{16,Int32}
    data::Ptr{Cvoid}
end

pad16(v, fill) = ntuple(i -> i <= length(v) ? v[i] : fill, 16)

"""
    binary_einsum(a, a_inds, b, b_inds, c_inds; precision=TN_PREC_NATIVE)

`Muscle.binary_einsum` on GB300 arrays: labels are integers; labels shared by `a` and `b`
and present in `c_inds` are kept (Hadamard modes), shared labels absent from `c_inds`
are contracted (src/Operations/canonize.jl:44,61).
"""
function binary_einsum(a::GB300Array{T}, ai::Vector{<:Integer}, b::GB300Array{T}, bi::Vector{<:Integer},
                       ci::Vector{<:Integer};
                       precision=TN_PREC_NATIVE) where {T}
    cdims = [i in ai ? size(a, findfirst(==(i), ai)) : size(b, findfirst(==(i), bi)) for i in ci]
    c = GB300Array{T}(undef, Tuple(cdims); ctx=a.ctx)
    ta = Ref(TnTensor(length(ai), pad16(collect(size(a)), 0), pad16(Int32.(ai), Int32(0)), a.ptr))
    tb = Ref(TnTensor(length(bi), pad16(collect(size(b)), 0), pad16(Int32.(bi), Int32(0)), b.ptr))
    tc = Ref(TnTensor(length(ci), pad16(cdims, 0), pad16(Int32.(ci), Int32(0)), c.ptr))
    check(ccall((:tn_contract, libtenetgb), Int32, (Ptr{Cvoid}, Int32, Int32, Ref{TnTensor}, Ref{TnTensor}, Ref{TnTensor}),
                a.ctx.h, dtype(T), precision, ta, tb, tc), a.ctx.h)
    return c
end

"""
    permutedims(a::GB300Array, perm; conj=false)

Index permutation on the device (tn_permute; the copy Muscle makes inside binary_einsum
and fuse), optionally conjugating.
"""
function permutedims_gb(a::GB300Array{T,N}, perm; conj::Bool=false) where {T,N}
    out = GB300Array{T}(undef, ntuple(i -> size(a, perm[i]), N); ctx=a.ctx)
    dims = Int64[size(a)...]
    p = Int32[perm...] .- Int32(1)
    check(ccall((:tn_permute, libtenetgb), Int32,
                (Ptr{Cvoid}, Int32, Int32, Ptr{Int64}, Ptr{Int64}, Ptr{Int32}, Ptr{Cvoid}, Ptr{Cvoid}, Int32),
                a.ctx.h, dtype(T), N, dims, C_NULL, p, a.ptr, out.ptr, conj ? 1 : 0), a.ctx.h)
    return out
end
Base.permutedims(a::GB300Array, perm) = permutedims_gb(a, perm)
Base.conj(a::GB300Array{T,N}) where {T<:Complex,N} = permutedims_gb(a, ntuple(identity, N); conj=true)
Base.conj(a::GB300Array{T}) where {T<:Real} = a

"""
    hadamard(t::GB300Array, s::GB300Array{Float64,1}, axis) -> t .* s along `axis`

`Muscle.hadamard` (src/Operations/canonize.jl:198,209) with a real FP64 vector (tn_hadamard).
"""
function hadamard(t::GB300Array{T,N}, s::GB300Array{Float64,1}, axis::Integer) where {T,N}
    out = GB300Array{T}(undef, size(t); ctx=t.ctx)
    dims = Int64[size(t)...]
    check(ccall((:tn_hadamard, libtenetgb), Int32, (Ptr{Cvoid}, Int32, Int32, Ptr{Int64}, Int32, Ptr{Cvoid}, Ptr{Cvoid},
                                                    Ptr{Cvoid}),
                t.ctx.h, dtype(T), N, dims, axis - 1, t.ptr, s.ptr, out.ptr), t.ctx.h)
    return out
end

"""
    tensor_qr_thin(A::GB300Array{ComplexF64,2}) -> (Q, R)

Thin QR of a matrix (the caller permutes `inds_q` first, as Muscle does):
src/Operations/canonize.jl:58.
"""
function tensor_qr_thin(A::GB300Array{T,2}; precision=TN_PREC_NATIVE) where {T}
    m, n = size(A)
    k = min(m, n)
    Q = GB300Array{T}(undef, (m, k); ctx=A.ctx)
    R = GB300Array{T}(undef, (k, n); ctx=A.ctx)
    check(ccall((:tn_qr_thin, libtenetgb), Int32,
                (Ptr{Cvoid}, Int32, Int32, Int64, Int64, Ptr{Cvoid}, Int64, Int64, Ptr{Cvoid}, Int64, Ptr{Cvoid}, Int64, Int64),
                A.ctx.h, dtype(T), precision, m, n, A.ptr, max(m, 1), 0, Q.ptr, 0, R.ptr, 0, 1), A.ctx.h)
    return Q, R
end

"""
    tensor_svd_thin(A::GB300Array{ComplexF64,2}) -> (U, s, V)

Thin SVD A = U diag(s) V with s real descending (src/Operations/canonize.jl:41,97).
"""
function tensor_svd_thin(A::GB300Array{T,2}; precision=TN_PREC_NATIVE) where {T}
    m, n = size(A)
    k = min(m, n)
    U = GB300Array{T}(undef, (m, k); ctx=A.ctx)
    s = GB300Array{Float64}(undef, (k,); ctx=A.ctx)
    V = GB300Array{T}(undef, (k, n); ctx=A.ctx)
    check(ccall((:tn_svd_thin, libtenetgb), Int32,
                (Ptr{Cvoid}, Int32, Int32, Int64, Int64, Ptr{Cvoid}, Int64, Int64, Ptr{Cvoid}, Int64, Ptr{Cvoid}, Int64,
                 Ptr{Cvoid}, Int64, Int64),
                A.ctx.h, dtype(T), precision, m, n, A.ptr, max(m, 1), 0, U.ptr, 0, s.ptr, 0, V.ptr, 0, 1), A.ctx.h)
    return U, s, V
end

"""
    simple_update(A, B, G; maxdim=-1, threshold=-1.0) -> (A′, B′)

`Muscle.simple_update(...; absorb=AbsorbEqually())` (src/Operations/simple_update.jl:53-64)
for A (χl, d1, χm), B (χm, d2, χr), G (d1, d2, d1, d2) with index order
[out_a, out_b, in_a, in_b].
"""
function simple_update(A::GB300Array{ComplexF64,3}, B::GB300Array{ComplexF64,3}, G::GB300Array{ComplexF64,4};
                       maxdim=-1, threshold=-1.0, precision=TN_PREC_NATIVE)
    chl, d1, chm = size(A)
    _, d2, chr = size(B)
    kmax = min(chl * d1, d2 * chr)
    An = GB300Array{ComplexF64}(undef, (chl, d1, kmax); ctx=A.ctx)
    Bn = GB300Array{ComplexF64}(undef, (kmax, d2, chr); ctx=A.ctx)
    r = Ref{Int64}(0)
    check(ccall((:tn_simple_update, libtenetgb), Int32,
                (Ptr{Cvoid}, Int32, Int32, Int64, Int64, Int64, Int64, Int64, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Int64,
                 Float64, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ref{Int64}),
                A.ctx.h, TN_C64, precision, chl, d1, chm, d2, chr, A.ptr, B.ptr, G.ptr, maxdim, threshold, An.ptr, Bn.ptr,
                C_NULL, r), A.ctx.h)
    An.dims = (chl, d1, Int(r[]))  # the kept columns are a column-major prefix
    Bn.dims = (Int(r[]), d2, chr)  # compacted by the library to leading dimension r
    return An, Bn
end

# ---- Muscle methods on Tangles.Tensor backed by GB300Array ---------------------------
# Index values are mapped to the integer mode labels of the C ABI per call; outputs are
# wrapped in new Tensors whose indices follow Muscle's conventions (new virtual / singular
# indices where Tenet passes them, `ind_virtual`, `ind_s`).

const GB300Tensor{T,N} = Tensor{T,N,<:GB300Array{T,N}}

# one Int32 label per distinct Index of a call
struct Labels
    d::Dict{Index,Int32}
end
Labels() = Labels(Dict{Index,Int32}())
(l::Labels)(i::Index) = get!(l.d, i, Int32(length(l.d)))

tntensor(a::GB300Array, lab::Vector{Int32}) =
    TnTensor(length(lab), pad16(Int64[size(a)...], 0), pad16(lab, Int32(0)), a.ptr)

# a GB300 tensor with its indices put in the order `order` (a device permutation when needed)
function arranged(t::Tensor, order)
    ti = collect(inds(t))
    ti == collect(order) && return parent(t)
    return permutedims_gb(parent(t), Tuple(findfirst(==(i), ti) for i in order))
end

"""
    Muscle.binary_einsum(a, b; dims) on GB300 tensors (tn_contract)

Indices in `dims` are contracted (default: every shared index); shared indices not in
`dims` are kept (Hadamard / batch modes, `dims=Index[]` at src/Operations/canonize.jl:44).
Output indices: a's kept indices, then b's indices not in a.
"""
function Muscle.binary_einsum(a::Tensor{T,Na,<:GB300Array}, b::Tensor{T,Nb,<:GB300Array};
                              dims=intersect(inds(a), inds(b)), out=nothing) where {T,Na,Nb}
    ia, ib = collect(inds(a)), collect(inds(b))
    all(in(ib), dims) && all(in(ia), dims) || throw(ArgumentError("contracted indices must be shared"))
    oi = out === nothing ? vcat(filter(!in(dims), ia), filter(i -> !(i in dims) && !(i in ia), ib)) : collect(out)
    lab = Labels()
    c = binary_einsum(parent(a), lab.(ia), parent(b), lab.(ib), lab.(oi))
    return Tensor(c, oi)
end

# Λ (a real FP64 vector) absorbed into a complex site: the `binary_einsum(s, V;
# dims=Index[])` of src/Operations/canonize.jl:44, as a device Hadamard product
function Muscle.binary_einsum(s::Tensor{Float64,1,<:GB300Array}, t::Tensor{T,N,<:GB300Array};
                              dims=intersect(inds(s), inds(t)), out=nothing) where {T<:Complex,N}
    i = only(inds(s))
    (isempty(dims) && i in inds(t)) ||
        throw(ArgumentError("a real GB300 vector meets a complex tensor only as a Hadamard factor"))
    o = Tensor(hadamard(parent(t), parent(s), findfirst(==(i), collect(inds(t)))), collect(inds(t)))
    return out === nothing ? o : Tensor(arranged(o, out), collect(out))
end
Muscle.binary_einsum(t::Tensor{T,N,<:GB300Array}, s::Tensor{Float64,1,<:GB300Array}; kwargs...) where {T<:Complex,N} =
    Muscle.binary_einsum(s, t; kwargs...)
Muscle.hadamard(t::Tensor{T,N,<:GB300Array}, s::Tensor{Float64,1,<:GB300Array}) where {T<:Complex,N} =
    Muscle.binary_einsum(s, t; dims=Index[])

function _factor_shapes(A::Tensor, left)
    ia = collect(inds(A))
    all(in(ia), left) || throw(ArgumentError("factorisation indices must be indices of the tensor"))
    rest = filter(!in(left), ia)
    ldims = [size(parent(A), findfirst(==(i), ia)) for i in left]
    rdims = [size(parent(A), findfirst(==(i), ia)) for i in rest]
    return ia, rest, ldims, rdims, prod(ldims; init=1), prod(rdims; init=1)
end

"""
    Muscle.tensor_qr_thin(A; inds_q, inds_r, ind_virtual) on a GB300 tensor (tn_tensor_qr_thin)

Q carries (inds_q…, ind_virtual), R (ind_virtual, inds_r…): src/Operations/canonize.jl:58.
"""
function Muscle.tensor_qr_thin(A::Tensor{T,N,<:GB300Array}; inds_q, inds_r=nothing,
                               ind_virtual=Index(gensym(:qr)), precision=TN_PREC_NATIVE) where {T,N}
    ia, rest, qd, rd, m, n = _factor_shapes(A, collect(inds_q))
    k = min(m, n)
    ctx = parent(A).ctx
    Q = GB300Array{T}(undef, (qd..., k); ctx)
    R = GB300Array{T}(undef, (k, rd...); ctx)
    lab = Labels()
    la = lab.(ia)
    tA = Ref(tntensor(parent(A), la))
    tQ, tR = Ref(tntensor(Q, Int32[])), Ref(tntensor(R, Int32[]))
    qm = Int32[lab(i) for i in inds_q]
    check(ccall((:tn_tensor_qr_thin, libtenetgb), Int32,
                (Ptr{Cvoid}, Int32, Int32, Ref{TnTensor}, Int32, Ptr{Int32}, Int32, Ref{TnTensor}, Ref{TnTensor}),
                ctx.h, dtype(T), precision, tA, length(qm), qm, lab(ind_virtual), tQ, tR), ctx.h)
    Qt = Tensor(Q, [collect(inds_q)..., ind_virtual])
    Rt = Tensor(R, [ind_virtual, rest...])
    if inds_r !== nothing && collect(inds_r) != rest
        Rt = Tensor(arranged(Rt, [ind_virtual, inds_r...]), [ind_virtual, inds_r...])
    end
    return Qt, Rt
end

"""
    Muscle.tensor_svd_thin(A; inds_u, inds_v, ind_s, maxdim, threshold) on a GB300 tensor
    (tn_tensor_svd_thin)

U (inds_u…, ind_s), s (ind_s) real FP64 descending, V (ind_s, inds_v…), A = U·diag(s)·V
(src/Operations/canonize.jl:41,97).  `maxdim` / `threshold` truncate like compress!
(src/Operations/compress.jl:47-59) inside the same call.
"""
function Muscle.tensor_svd_thin(A::Tensor{T,N,<:GB300Array}; inds_u, inds_v=nothing, ind_s=Index(gensym(:svd)),
                                maxdim=nothing, threshold=nothing, precision=TN_PREC_NATIVE) where {T,N}
    ia, rest, ud, vd, m, n = _factor_shapes(A, collect(inds_u))
    k = min(m, n)
    ctx = parent(A).ctx
    U = GB300Array{T}(undef, (ud..., k); ctx)
    s = GB300Array{Float64}(undef, (k,); ctx)
    V = GB300Array{T}(undef, (k, vd...); ctx)
    lab = Labels()
    la = lab.(ia)
    tA = Ref(tntensor(parent(A), la))
    tU, tV = Ref(tntensor(U, Int32[])), Ref(tntensor(V, Int32[]))
    um = Int32[lab(i) for i in inds_u]
    r = Ref{Int64}(0)
    check(ccall((:tn_tensor_svd_thin, libtenetgb), Int32,
                (Ptr{Cvoid}, Int32, Int32, Ref{TnTensor}, Int32, Ptr{Int32}, Int32, Int64, Float64, Ref{TnTensor},
                 Ptr{Cvoid}, Ref{TnTensor}, Ref{Int64}),
                ctx.h, dtype(T), precision, tA, length(um), um, lab(ind_s), maxdim === nothing ? -1 : maxdim,
                threshold === nothing ? -1.0 : Float64(threshold), tU, s.ptr, tV, r), ctx.h)
    kr = Int(r[])  # the kept rank: U's columns are a prefix, V's rows were compacted
    U.dims = (ud..., kr)
    s.dims = (kr,)
    V.dims = (kr, vd...)
    Vt = Tensor(V, [ind_s, rest...])
    if inds_v !== nothing && collect(inds_v) != rest
        Vt = Tensor(arranged(Vt, [ind_s, inds_v...]), [ind_s, inds_v...])
    end
    return Tensor(U, [collect(inds_u)..., ind_s]), Tensor(s, [ind_s]), Vt
end

"""
    Muscle.simple_update(A, ia, B, ib, bond, op, oa, ob; maxdim, absorb=AbsorbEqually())
    on GB300 tensors (tn_simple_update_absorb; src/Operations/simple_update.jl:53-64)

θ = op·A·B over the bond and the physical indices ia/ib (op's input indices), thin SVD
over (A's side)|(B's side), at most `maxdim` values kept, S split by `absorb`
(AbsorbEqually: √S into both sides; AbsorbU: into A'; AbsorbV: into B').  A'
carries (A's other indices…, ia, bond), B' (bond, ib, B's other indices…): the
physical indices keep A's and B's labels, which Tenet renames back afterwards.
"""
function Muscle.simple_update(A::Tensor{ComplexF64,Na,<:GB300Array}, ia::Index, B::Tensor{ComplexF64,Nb,<:GB300Array},
                              ib::Index, bond::Index, op::Tensor{ComplexF64,4,<:GB300Array}, oa::Index, ob::Index;
                              maxdim=nothing, threshold=nothing, absorb=Muscle.AbsorbEqually(),
                              precision=TN_PREC_NATIVE) where {Na,Nb}
    # Muscle's absorb behaviours (AbsorbEqually, AbsorbU, AbsorbV) → TN_ABSORB_*
    mode = absorb isa Muscle.AbsorbEqually ? Int32(0) : absorb isa Muscle.AbsorbV ? Int32(1) :
           absorb isa Muscle.AbsorbU ? Int32(2) :
           throw(ArgumentError("GB300 simple_update: absorb must be AbsorbEqually, AbsorbU or AbsorbV"))
    la = filter(i -> i != ia && i != bond, collect(inds(A)))
    lb = filter(i -> i != ib && i != bond, collect(inds(B)))
    Am = arranged(A, [la..., ia, bond])
    Bm = arranged(B, [bond, ib, lb...])
    G = arranged(op, [oa, ob, ia, ib])
    chl = prod(size(Am)[1:length(la)]; init=1)
    d1, chm = size(Am, length(la) + 1), size(Am, length(la) + 2)
    d2 = size(Bm, 2)
    chr = prod(size(Bm)[3:end]; init=1)
    kmax = min(chl * d1, d2 * chr)
    ctx = Am.ctx
    An = GB300Array{ComplexF64}(undef, (size(Am)[1:length(la)]..., d1, kmax); ctx)
    Bn = GB300Array{ComplexF64}(undef, (kmax, d2, size(Bm)[3:end]...); ctx)
    r = Ref{Int64}(0)
    check(ccall((:tn_simple_update_absorb, libtenetgb), Int32,
                (Ptr{Cvoid}, Int32, Int32, Int64, Int64, Int64, Int64, Int64, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Int64,
                 Float64, Int32, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ref{Int64}),
                ctx.h, TN_C64, precision, chl, d1, chm, d2, chr, Am.ptr, Bm.ptr, G.ptr,
                maxdim === nothing ? -1 : maxdim, threshold === nothing ? -1.0 : Float64(threshold), mode, An.ptr,
                Bn.ptr, C_NULL, r), ctx.h)
    An.dims = (size(Am)[1:length(la)]..., d1, Int(r[]))
    Bn.dims = (Int(r[]), d2, size(Bm)[3:end]...)
    return Tensor(An, [la..., ia, bond]), Tensor(Bn, [bond, ib, lb...])
end

"""
    Muscle.fuse(t, fused; ind) on a GB300 tensor (src/Operations/evolve.jl:35,39)

The indices `fused` (first fastest) become one index `ind` of their product dimension,
placed last; the others keep their order.
"""
function Muscle.fuse(t::Tensor{T,N,<:GB300Array}, fused; ind=Index(gensym(:fuse))) where {T,N}
    ti = collect(inds(t))
    others = filter(!in(fused), ti)
    a = arranged(t, [others..., fused...])
    od = size(a)[1:length(others)]
    f = GB300Array{T,length(others) + 1}(a.ptr, (od..., prod(size(a)[length(others)+1:end])), a.ctx)
    # `f` views `a`'s buffer: keep `a` alive as long as `f` (a device array is freed by its finalizer)
    finalizer(_ -> (a; nothing), f)
    return Tensor(f, [others..., ind])
end

Base.conj(t::Tensor{T,N,<:GB300Array}) where {T<:Complex,N} = Tensor(conj(parent(t)), collect(inds(t)))

function LinearAlgebra.norm(t::Tensor{T,N,<:GB300Array}) where {T,N}
    a = parent(t)
    out = Ref{Float64}(0.0)
    check(ccall((:tn_norm2, libtenetgb), Int32, (Ptr{Cvoid}, Int32, Int64, Ptr{Cvoid}, Ref{Float64}), a.ctx.h, dtype(T),
                length(a), a.ptr, out), a.ctx.h)
    return out[]
end

# ---- device-resident MPS ---------------------------------------------------------------
mutable struct GB300MPS
    h::Ptr{Cvoid}
    ctx::Context
    L::Int
    d::Int
end

"""
    GB300MPS(arrays; max_bond=0) where arrays are (χl, d, χr) Complex{Float64} site arrays

(Tenet's (:l, :o, :r) order, src/Components/MPS.jl:50-94, with the boundary tensors
lifted to 3-D.)
"""
function GB300MPS(arrays::Vector{Array{ComplexF64,3}}; max_bond=0, precision=TN_PREC_NATIVE, ctx=default_context())
    L = length(arrays)
    L >= 2 || throw(ArgumentError("an MPS needs at least two sites"))
    d = size(arrays[1], 2)
    # the library reads χl·d·χr entries of every site with one d for all of them
    all(a -> size(a, 2) == d, arrays) || throw(ArgumentError("every site must have the same physical dimension"))
    bonds = Int64[size(a, 3) for a in arrays[1:(end - 1)]]
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:tn_mps_create, libtenetgb), Int32, (Ptr{Cvoid}, Int32, Int32, Ptr{Int64}, Int64, Int32, Ref{Ptr{Cvoid}}),
                ctx.h, L, d, bonds, max_bond, precision, r), ctx.h)
    mps = GB300MPS(r[], ctx, L, d)
    finalizer(m -> ccall((:tn_mps_destroy, libtenetgb), Int32, (Ptr{Cvoid},), m.h), mps)
    for (i, a) in enumerate(arrays)
        check(ccall((:tn_mps_set_site, libtenetgb), Int32, (Ptr{Cvoid}, Int32, Int64, Int64, Ptr{Cvoid}),
                    mps.h, i, size(a, 1), size(a, 3), a), ctx.h)
    end
    return mps
end

canonize!(ψ::GB300MPS, lo::Integer, hi::Integer=lo) =
    (check(ccall((:tn_mps_canonize_mixed, libtenetgb), Int32, (Ptr{Cvoid}, Int32, Int32), ψ.h, lo, hi), ψ.ctx.h); ψ)
canonize_bond!(ψ::GB300MPS, a::Integer) =
    (check(ccall((:tn_mps_canonize_bond, libtenetgb), Int32, (Ptr{Cvoid}, Int32), ψ.h, a), ψ.ctx.h); ψ)
compress!(ψ::GB300MPS; bond=0, maxdim=-1, threshold=-1.0) =
    (check(ccall((:tn_mps_compress, libtenetgb), Int32, (Ptr{Cvoid}, Int32, Int64, Float64), ψ.h, bond, maxdim, threshold), ψ.ctx.h); ψ)

function simple_update!(ψ::GB300MPS, G::Array{ComplexF64}, site::Integer; maxdim=-1, threshold=-1.0)
    nsites = ndims(G) == 2 ? 1 : 2
    # the library reads d^(2·nsites) entries from G
    length(G) == ψ.d^(2 * nsites) ||
        throw(ArgumentError("a $nsites-site operator on sites of dimension $(ψ.d) has $(ψ.d^(2 * nsites)) entries"))
    check(ccall((:tn_mps_simple_update, libtenetgb), Int32, (Ptr{Cvoid}, Int32, Int32, Ptr{ComplexF64}, Int64, Float64),
                ψ.h, nsites, site, G, maxdim, threshold), ψ.ctx.h)
    return ψ
end
evolve!(ψ::GB300MPS, G::Array{ComplexF64}, site::Integer) = simple_update!(ψ, G, site)  # evolve.jl:140-143

function overlap(a::GB300MPS, b::GB300MPS)
    out = zeros(Float64, 2)
    check(ccall((:tn_mps_overlap, libtenetgb), Int32, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}), a.h, b.h, out), a.ctx.h)
    return complex(out[1], out[2])
end

function LinearAlgebra.norm(ψ::GB300MPS)
    out = Ref{Float64}(0.0)
    check(ccall((:tn_mps_norm, libtenetgb), Int32, (Ptr{Cvoid}, Ref{Float64}), ψ.h, out), ψ.ctx.h)
    return out[]
end

LinearAlgebra.normalize!(ψ::GB300MPS) = (check(ccall((:tn_mps_normalize, libtenetgb), Int32, (Ptr{Cvoid},), ψ.h), ψ.ctx.h); ψ)

# the library reads w_{i-1}·d·d·w_i entries of MPO site i (w_0 = w_L = 1): the sizes must chain
function check_mpo(ψ, H)
    length(H) == ψ.L || throw(ArgumentError("the MPO must have one site per MPS site"))
    for (i, W) in enumerate(H)
        (size(W, 2) == ψ.d && size(W, 3) == ψ.d) ||
            throw(ArgumentError("MPO site $i: physical dimensions must be $(ψ.d)"))
        size(W, 1) == (i == 1 ? 1 : size(H[i - 1], 4)) ||
            throw(ArgumentError("MPO site $i: left virtual dimension does not match its neighbour"))
    end
    size(H[end], 4) == 1 || throw(ArgumentError("the last MPO site must have a right virtual dimension of 1"))
    return nothing
end

# evolve!(ψ, op::MPO) — src/Operations/evolve.jl:19-137 (algorithm :direct or :zipup); the
# MPO as its (w_l, d_out, d_in, w_r) site arrays
function evolve!(ψ::GB300MPS, H::Vector{Array{ComplexF64,4}}; algorithm::Symbol=:direct, maxdim::Integer=0,
                 threshold::Real=0.0)
    check_mpo(ψ, H)
    ptrs = Ptr{ComplexF64}[pointer(W) for W in H]
    bonds = Int64[size(W, 4) for W in H[1:end-1]]
    GC.@preserve H begin
        check(ccall((:tn_mps_evolve_mpo, libtenetgb), Int32,
                    (Ptr{Cvoid}, Ptr{Ptr{ComplexF64}}, Ptr{Int64}, Int32, Int64, Float64),
                    ψ.h, ptrs, bonds, algorithm === :zipup ? 1 : 0, maxdim, threshold), ψ.ctx.h)
    end
    return ψ
end

# sample(ψ, nshots) — src/Operations/sample.jl:20-72; the caller's uniforms (an L × nshots
# matrix in [0, 1), one column per shot) make the draw reproducible; outcomes are 1-based
# like the reference's, one row per shot.  ψ itself is left as it is: the sampler moves
# the orthogonality centre of a device copy (the reference samples canonize(ψ, …)).
function sample(ψ::GB300MPS, nshots::Integer; uniforms::Matrix{Float64}=rand(ψ.L, nshots))
    size(uniforms) == (ψ.L, nshots) || throw(ArgumentError("uniforms must be an L × nshots matrix"))
    out = Matrix{Int32}(undef, ψ.L, nshots)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:tn_mps_copy, libtenetgb), Int32, (Ptr{Cvoid}, Ref{Ptr{Cvoid}}), ψ.h, r), ψ.ctx.h)
    try
        check(ccall((:tn_mps_sample, libtenetgb), Int32, (Ptr{Cvoid}, Int32, Int64, Ptr{Float64}, Ptr{Int32}),
                    r[], 0, nshots, uniforms, out), ψ.ctx.h)
    finally
        ccall((:tn_mps_destroy, libtenetgb), Int32, (Ptr{Cvoid},), r[])
    end
    return permutedims(out)
end

# device MPS dump / load (raw column-major format, warm restarts)
save(ψ::GB300MPS, path::AbstractString) =
    check(ccall((:tn_mps_save, libtenetgb), Int32, (Ptr{Cvoid}, Cstring), ψ.h, path), ψ.ctx.h)

function load(path::AbstractString; max_bond::Integer=0, ctx=default_context())
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:tn_mps_load, libtenetgb), Int32, (Ptr{Cvoid}, Cstring, Int64, Ref{Ptr{Cvoid}}), ctx.h, path, max_bond,
                r), ctx.h)
    L, d, B = Ref{Int32}(0), Ref{Int32}(0), Ref{Int32}(0)
    check(ccall((:tn_mps_shape, libtenetgb), Int32, (Ptr{Cvoid}, Ref{Int32}, Ref{Int32}, Ref{Int32}), r[], L, d, B),
          ctx.h)
    mps = GB300MPS(r[], ctx, L[], d[])
    finalizer(m -> ccall((:tn_mps_destroy, libtenetgb), Int32, (Ptr{Cvoid},), m.h), mps)
    return mps
end

# dmrg!(ψ, H, nsweeps; method) — src/Algorithms/DMRG.jl:45-459.  H: the MPO's site arrays,
# column-major (w_l, d_out, d_in, w_r) with w_0 = w_L = 1 (`MPO(arrays; order=(:l, :o, :i, :r))`).
function dmrg!(ψ::GB300MPS, H::Vector{Array{ComplexF64,4}}, nsweeps::Integer=4; method::Symbol=:dmrg1,
               maxdim::Integer=128, krylovdim::Integer=3, maxiter::Integer=2, tol::Real=1e-12)
    check_mpo(ψ, H)
    ptrs = Ptr{ComplexF64}[pointer(W) for W in H]
    bonds = Int64[size(W, 4) for W in H[1:end-1]]
    energy = Ref{Float64}(0.0)
    GC.@preserve H begin
        check(ccall((:tn_mps_dmrg, libtenetgb), Int32,
                    (Ptr{Cvoid}, Ptr{Ptr{ComplexF64}}, Ptr{Int64}, Int32, Int32, Int32, Int64, Int32, Int32, Float64,
                     Ref{Float64}, Ptr{Float64}),
                    ψ.h, ptrs, bonds, 1, method === :dmrg2 ? 2 : 1, nsweeps, maxdim, krylovdim, maxiter, tol, energy,
                    C_NULL), ψ.ctx.h)
    end
    return ψ, energy[]
end

end # module
