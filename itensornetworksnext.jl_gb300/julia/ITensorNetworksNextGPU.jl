# ITensorNetworksNextGPU.jl -- Julia side of the drop-in: GPU strategies for
# ITensorNetworksNext.jl that call libitn_gpu.so through `ccall`.
#
# Plug-in points used (paths inside ITensorNetworksNext.jl):
#   * MessageUpdateAlgorithm + message_update!(alg, cache, factors, edge)
#       src/beliefpropagation/beliefpropagation.jl:214-235 (strategy interface)
#   * AI.solve specialised on BeliefPropagationAlgorithm whose sweep uses GPUMessageUpdate,
#     so `beliefpropagation(factors, messages; ...)` (beliefpropagation.jl:69-92) keeps its
#     signature and returns a MessageCache
#   * bethe_free_energy(factors, messages) (src/beliefpropagation/messagecache.jl:185-201)
#   * ChainRulesCore.rrule for the converged BP log-norm (no reference counterpart)
#
# Not exercised in this repository: no Julia toolchain is available where it was built.
module ITensorNetworksNextGPU

using ITensorNetworksNext: ITensorNetworksNext, MessageUpdateAlgorithm, MessageCache,
    NormNetwork, messagecache, linknames, sitenames, kettensor, braname
using ITensorNetworksNext.AlgorithmsInterfaceExtensions: StopWhenConverged
using AlgorithmsInterface: AlgorithmsInterface as AI
using Graphs: vertices, edges, src, dst, neighbors
using ITensorBase: dimnames, unnamed
using ChainRulesCore: ChainRulesCore, NoTangent

const libitn = get(ENV, "ITN_GPU_LIB",
    joinpath(@__DIR__, "..", "lib", "libitn_gpu.so"))

# ---- status handling (include/itn_gpu.h) --------------------------------------------------
const ITN_OK = Int32(0)
const ITN_ERR_ARG = Int32(1)

function check(ctx::Ptr{Cvoid}, st::Int32)
    st == ITN_OK && return nothing
    msg = unsafe_string(ccall((:itn_last_error, libitn), Cstring, (Ptr{Cvoid},), ctx))
    st == ITN_ERR_ARG && throw(ArgumentError(msg))
    return error("libitn_gpu status $st: $msg")
end

eltype_code(::Type{Float32}) = Int32(0)
eltype_code(::Type{Float64}) = Int32(1)
eltype_code(::Type{ComplexF32}) = Int32(2)
eltype_code(::Type{ComplexF64}) = Int32(3)

struct ItnBpOpts
    schedule::Int32
    maxiter::Int32
    tol::Float64
    normalize::Int32
    precision::Int32
    split_sweeps::Int32
    reserved0::Int32
    edges::Ptr{Int64}
    n_edges::Int64
end

struct ItnBpResult
    iterations::Int32
    at_iteration::Int32
    delta::Float64
    device_ms::Float64
    kernel_launches::Int32
    reserved0::Int32
end

struct ItnGradOpts
    adjoint::Int32
    maxiter::Int32
    tol::Float64
    normalized::Int32
    reserved0::Int32
end

struct ItnGradResult
    adjoint_iterations::Int32
    reserved0::Int32
    adjoint_residual::Float64
    device_ms::Float64
end

# ---- the strategy -----------------------------------------------------------------------
"""
    GPUMessageUpdate(; precision = :native, split_sweeps = 0, device = 0, schedule = :parallel)

Message-update strategy that runs the whole BP solve on the GPU. `precision = :bf16`
uses the tcgen05 tensor-core sweep (Float32 networks, 4 legs of dimension 8) with
`split_sweeps` final hi/lo sweeps.
"""
Base.@kwdef struct GPUMessageUpdate <: MessageUpdateAlgorithm
    precision::Symbol = :native
    split_sweeps::Int = 0
    device::Int = 0
    schedule::Symbol = :parallel
end

# A flattened norm network on the device.
mutable struct DeviceNetwork{V}
    ctx::Ptr{Cvoid}
    verts::Vector{V}
    slot::Dict{Pair{V, V}, Int}   # directed edge -> CSR slot
    off::Vector{Int64}
    bond::Vector{Int32}
    moff::Vector{Int64}
    elt::DataType
end

function destroy!(d::DeviceNetwork)
    d.ctx == C_NULL || ccall((:itn_destroy, libitn), Int32, (Ptr{Cvoid},), d.ctx)
    d.ctx = C_NULL
    return nothing
end

# Build the CSR description (one leg per neighbour; all shared link names of a pair
# fuse into that leg, abstracttensornetwork.jl:52-73) and upload the ket tensors with
# their own strides (permuted to [site, legs...] on the device).
function DeviceNetwork(nn::NormNetwork; device::Integer = 0)
    ctxr = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:itn_create, libitn), Int32, (Ptr{Ptr{Cvoid}}, Int32, Int32), ctxr, device, 0)
    st == ITN_OK || error("itn_create failed with status $st")
    ctx = ctxr[]
    verts = collect(vertices(nn))
    vidx = Dict(v => i - 1 for (i, v) in enumerate(verts))
    off = Int64[0]; nbr = Int64[]; bond = Int32[]; phys = Int32[]
    slot = Dict{Pair{eltype(verts), eltype(verts)}, Int}()
    ptrs = Ptr{Cvoid}[]; strides = Int64[]
    elt = eltype(unnamed(kettensor(nn, first(verts))))
    keep = Any[]
    for v in verts
        A = kettensor(nn, v)
        names = dimnames(A)
        data = unnamed(A)                       # Julia array, column-major
        st_of = Dict(n => stride(data, i) for (i, n) in enumerate(names))
        sz_of = Dict(n => size(data, i) for (i, n) in enumerate(names))
        sites = sitenames(nn.ket, v)
        # fused site axis: a single site name is required for a strided upload
        length(sites) <= 1 || throw(ArgumentError("vertex $v has several site indices"))
        push!(phys, isempty(sites) ? 1 : sz_of[only(sites)])
        push!(strides, isempty(sites) ? 0 : st_of[only(sites)])
        for w in neighbors(nn, v)
            ln = collect(linknames(nn.ket, v => w))
            length(ln) == 1 || throw(ArgumentError("edge $v => $w carries $(length(ln)) links; fuse them first"))
            slot[v => w] = length(nbr)
            push!(nbr, vidx[w]); push!(bond, sz_of[only(ln)]); push!(strides, st_of[only(ln)])
        end
        push!(off, length(nbr))
        push!(ptrs, pointer(data)); push!(keep, data)
    end
    GC.@preserve keep off nbr bond phys begin
        check(ctx, ccall((:itn_graph_upload, libitn), Int32,
            (Ptr{Cvoid}, Int64, Ptr{Int64}, Ptr{Int64}, Ptr{Int32}, Ptr{Int64}, Ptr{Int32}, Int32, Ptr{Int32}),
            ctx, length(verts), off, nbr, bond, C_NULL, phys, 2, C_NULL))
        check(ctx, ccall((:itn_tensors_upload_strided, libitn), Int32,
            (Ptr{Cvoid}, Int32, Ptr{Ptr{Cvoid}}, Ptr{Int64}), ctx, eltype_code(elt), ptrs, strides))
    end
    moff = cumsum(vcat(Int64(0), Int64.(bond) .^ 2))
    d = DeviceNetwork(ctx, verts, slot, off, bond, moff, elt)
    finalizer(destroy!, d)
    return d
end

# Messages: D x D operator with (bra, ket) names; packed as m[bra][ket] row-major.
function upload_messages!(d::DeviceNetwork, nn::NormNetwork, cache)
    packed = Vector{d.elt}(undef, d.moff[end])
    for ((a, b), s) in d.slot
        m = cache[a => b]
        ket = only(linknames(nn.ket, a => b))
        bra = braname(nn, ket)
        M = unnamed(permutedims(m, (bra, ket)))   # rows bra, columns ket
        packed[(d.moff[s + 1] + 1):d.moff[s + 2]] .= vec(permutedims(M, (2, 1)))
    end
    check(d.ctx, ccall((:itn_messages_upload, libitn), Int32, (Ptr{Cvoid}, Int32, Ptr{Cvoid}),
        d.ctx, eltype_code(d.elt), packed))
    return d
end

function download_messages!(cache, d::DeviceNetwork, nn::NormNetwork)
    packed = Vector{d.elt}(undef, d.moff[end])
    check(d.ctx, ccall((:itn_messages_download, libitn), Int32, (Ptr{Cvoid}, Int32, Ptr{Cvoid}),
        d.ctx, eltype_code(d.elt), packed))
    for ((a, b), s) in d.slot
        D = Int(d.bond[s + 1])
        M = permutedims(reshape(packed[(d.moff[s + 1] + 1):d.moff[s + 2]], D, D), (2, 1))
        ket = only(linknames(nn.ket, a => b))
        copyto!(unnamed(permutedims(cache[a => b], (braname(nn, ket), ket))), M)
    end
    return cache
end

precision_code(p::Symbol) = p === :native ? Int32(0) : p === :bf16 ? Int32(1) :
    p === :tf32 ? Int32(2) : p === :tf32x3 ? Int32(3) : throw(ArgumentError("unknown precision $p"))

# The whole solve in one call: beliefpropagation(nn, messages; edges, stopping_criterion,
# message_update_algorithm = GPUMessageUpdate(...)) dispatches here through AI.solve.
function gpu_beliefpropagation(nn::NormNetwork, messages, alg::GPUMessageUpdate;
        maxiter = nothing, tol = nothing, edges = nothing)
    isnothing(maxiter) && isnothing(tol) &&
        throw(ArgumentError("At least one of `maxiter` or `tol` must be specified."))
    d = DeviceNetwork(nn; device = alg.device)
    cache = MessageCache(messages)
    upload_messages!(d, nn, cache)
    seq = alg.schedule === :sequential
    eslots = seq ? Int64[d.slot[src(e) => dst(e)] for e in something(edges, collect(keys(cache)))] : Int64[]
    res = Ref{ItnBpResult}()
    GC.@preserve eslots begin
        opts = ItnBpOpts(seq ? 1 : 0, isnothing(maxiter) ? -1 : maxiter,
            isnothing(tol) ? -1.0 : tol, 1, precision_code(alg.precision), alg.split_sweeps, 0,
            seq ? pointer(eslots) : C_NULL, length(eslots))
        check(d.ctx, ccall((:itn_bp_run, libitn), Int32,
            (Ptr{Cvoid}, Ref{ItnBpOpts}, Ref{ItnBpResult}), d.ctx, opts, res))
    end
    download_messages!(cache, d, nn)
    destroy!(d)
    return cache
end

# bethe_free_energy(nn, messages) on the device (FP64 log-scalars).
function gpu_bethe_free_energy(nn::NormNetwork, cache; device = 0)
    d = DeviceNetwork(nn; device)
    upload_messages!(d, nn, cache)
    tot = zeros(Float64, 2); flags = zeros(Int32, 1)
    check(d.ctx, ccall((:itn_logscalars, libitn), Int32,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Int32}),
        d.ctx, C_NULL, C_NULL, C_NULL, C_NULL, tot, flags))
    destroy!(d)
    (flags[1] & 4) != 0 && return -Inf
    cplx = d.elt <: Complex || (flags[1] & 3) != 0
    return cplx ? complex(tot[1], tot[2]) : tot[1]
end

"""
    bp_logz(nn; maxiter, tol, alg = GPUMessageUpdate()) -> log Z_BP

Converged BP log-norm of `nn`; differentiable through the rrule below.
"""
function bp_logz(nn::NormNetwork, messages; alg = GPUMessageUpdate(), kwargs...)
    cache = gpu_beliefpropagation(nn, messages, alg; kwargs...)
    return gpu_bethe_free_energy(nn, cache; device = alg.device)
end

# rrule: the pullback of the converged log-norm w.r.t. every ket tensor comes from the
# implicit (adjoint BP) gradient, itn_bp_grad.
function ChainRulesCore.rrule(::typeof(bp_logz), nn::NormNetwork, messages; alg = GPUMessageUpdate(), kwargs...)
    cache = gpu_beliefpropagation(nn, messages, alg; kwargs...)
    d = DeviceNetwork(nn; device = alg.device)
    upload_messages!(d, nn, cache)
    y = gpu_bethe_free_energy(nn, cache; device = alg.device)
    function bp_logz_pullback(ȳ)
        n = d.off  # tensor sizes follow the upload order
        total = sum(length(unnamed(kettensor(nn, v))) for v in d.verts)
        g = Vector{d.elt}(undef, total)
        res = Ref{ItnGradResult}()
        check(d.ctx, ccall((:itn_bp_grad, libitn), Int32,
            (Ptr{Cvoid}, Ref{ItnGradOpts}, Ptr{Cvoid}, Ref{ItnGradResult}),
            d.ctx, ItnGradOpts(1, 200, 1e-10, 1, 0), g, res))
        destroy!(d)
        # g is in canonical [site, legs...] row-major order per vertex; the caller maps it
        # back onto each ket tensor's index order (the inverse of the upload strides).
        return NoTangent(), ȳ .* g, NoTangent()
    end
    return y, bp_logz_pullback
end

# ---- gate application (src/apply/apply_operators.jl:209-283) -------------------------------
# Mirrors itn_gate_desc (216 bytes).  A BPApplyGate-compatible strategy permutes each site to
# [other legs..., site index, shared bond] (column-major Julia arrays are passed reversed:
# the C side reads row-major), packs env[e] as M[bra, ket] per other leg and the operator
# as op[s1', s2', s1, s2], fills one descriptor per gate of a layer and calls
# gpu_apply_gates! once for the whole layer.
struct ItnGateDesc
    nsite::Int32
    d::NTuple{2,Int32}
    nleg::NTuple{2,Int32}
    bond::Int32
    leg_dim::NTuple{2,NTuple{6,Int32}}
    site_off::NTuple{2,Int64}
    env_off::NTuple{2,NTuple{6,Int64}}
    op_off::Int64
    out_off::NTuple{2,Int64}
    s_off::Int64
end

function gpu_apply_gates!(out::Vector{T}, svals::Vector{Float64}, chis::Vector{Int32},
                          descs::Vector{ItnGateDesc}, sites::Vector{T}, envs::Vector{T},
                          ops::Vector{T}; maxrank::Integer = 0, cutoff::Real = 0.0,
                          normalize::Bool = false, device::Integer = 0) where {T}
    ctx = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:itn_create, libitn), Int32, (Ptr{Ptr{Cvoid}}, Int32, Int32), ctx, device, 0)
    st == ITN_OK || error("itn_create failed with status $st")
    try
        GC.@preserve out svals chis descs sites envs ops begin
            check(ctx[], ccall((:itn_apply_gates, libitn), Int32,
                (Ptr{Cvoid}, Int32, Int64, Ptr{ItnGateDesc}, Ptr{Cvoid}, Int64, Ptr{Cvoid}, Int64,
                 Ptr{Cvoid}, Int64, Int32, Float64, Int32, Ptr{Cvoid}, Int64, Ptr{Float64}, Int64,
                 Ptr{Int32}, Ptr{Float64}),
                ctx[], eltype_code(T), length(descs), descs, sites, length(sites), envs, length(envs),
                ops, length(ops), maxrank, cutoff, normalize, out, length(out), svals, length(svals),
                chis, C_NULL))
        end
    finally
        ccall((:itn_destroy, libitn), Int32, (Ptr{Cvoid},), ctx[])
    end
    return out, svals, chis
end

end # module
