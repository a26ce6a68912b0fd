# ITensorNetworksNextGPU.jl -- Julia side of the drop-in: GPU strategies for
# ITensorNetworksNext.jl that call libitn_gpu.so through `ccall`.
#
# Plug-in points of the reference used here (paths inside ITensorNetworksNext.jl):
#   * `GPUMessageUpdate <: MessageUpdateAlgorithm` with a `message_update!(alg, cache,
#     factors, edge)` method (src/beliefpropagation/beliefpropagation.jl:214-235): the
#     per-edge strategy, one device update per call (itn_message_update).
#   * `AI.solve` specialised on `BeliefPropagationAlgorithm` whose sweep algorithm carries a
#     `GPUMessageUpdate` (beliefpropagation.jl:96-210): `beliefpropagation(factors, messages;
#     edges, stopping_criterion, message_update_algorithm = GPUMessageUpdate())`
#     (beliefpropagation.jl:69-92) keeps its signature, goes down in one call (itn_bp_run)
#     and returns a `MessageCache`.
#   * `GPUExact` with `contract_network(::GPUExact, tn)` (src/contract_network.jl:12-17, the
#     method table the unknown-algorithm fallback guards): exact contraction by pairwise GPU
#     contractions (itn_contract_network).
#   * `bethe_free_energy(factors, ::DeviceMessageCache)` (src/beliefpropagation/
#     messagecache.jl:185): the log-norm of messages that stayed on the device after the
#     solve (itn_logscalars, FP64 log-scalars, no re-upload).
#   * `ChainRulesCore.rrule(::typeof(bp_logz), nn, messages)`: the converged BP log-norm and
#     its gradient (no reference counterpart: the reference has no AD); the tangent of the
#     NormNetwork is a structural tangent of its ket tensors, each in its own index order.
#
# Not exercised here: no Julia toolchain exists where this repository is built and tested.
# tests/c/julia_shim_replay.c replays every ccall below (argument lists, struct layouts,
# packing and index orders) against the library from C.
module ITensorNetworksNextGPU

using ITensorNetworksNext: ITensorNetworksNext, MessageUpdateAlgorithm, MessageCache,
    NormNetwork, linknames, sitenames, kettensor, conj_bratensor, braname
using ITensorNetworksNext.AlgorithmsInterfaceExtensions: StopWhenConverged
using AlgorithmsInterface: AlgorithmsInterface as AI
using Graphs: vertices, src, dst, neighbors
using ITensorBase: dimnames, unnamed, inds, name
using ChainRulesCore: ChainRulesCore, NoTangent, Tangent

const INN = ITensorNetworksNext

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
eltype_code(::Type{T}) where {T} =
    throw(ArgumentError("no GPU arithmetic for element type $T (use SimpleMessageUpdate)"))

# C layouts of itn_bp_opts / itn_bp_result / itn_grad_opts / itn_grad_result
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
    sweeps::Int32
    checkpoint::Int32
    reserved0::Int32
end

struct ItnGradResult
    adjoint_iterations::Int32
    reserved0::Int32
    adjoint_residual::Float64
    device_ms::Float64
end

precision_code(p::Symbol) = p === :native ? Int32(0) : p === :bf16 ? Int32(1) :
    p === :tf32 ? Int32(2) : p === :tf32x3 ? Int32(3) : throw(ArgumentError("unknown precision $p"))

# ---- the message-update strategy ------------------------------------------------------------
"""
    GPUMessageUpdate(; normalize = true, precision = :native, split_sweeps = 0,
                       schedule = :sequential, device = 0)

`MessageUpdateAlgorithm` whose updates run on the GPU.  Through `beliefpropagation` the whole
solve is one device call: `schedule = :sequential` follows the `edges` order exactly (the
reference's Gauss-Seidel sweep), `:parallel` updates every edge from the previous sweep's
messages (Jacobi; `edges` only fixes the edge set).  `precision = :bf16` / `:tf32` run the
tcgen05 tensor-core sweep on Float32 networks whose vertices have at most four legs, bond
dimensions of at most 8 and a site index of dimension at most 2 (anything smaller than four
legs of 8 with d = 2, e.g. an open boundary, runs zero-padded to that shape), with
`split_sweeps` final hi/lo sweeps; `:tf32x3` runs every sweep with TF32 hi/lo operands.
"""
Base.@kwdef struct GPUMessageUpdate <: MessageUpdateAlgorithm
    normalize::Bool = true
    precision::Symbol = :native
    split_sweeps::Int = 0
    schedule::Symbol = :sequential
    device::Int = 0
end

# A flattened norm network on the device: CSR graph (one leg per neighbour), ket tensors
# uploaded with their own strides (permuted to the canonical [site, legs...] on the device).
mutable struct DeviceNetwork{V}
    ctx::Ptr{Cvoid}
    verts::Vector{V}
    slot::Dict{Pair{V, V}, Int}          # directed edge -> CSR slot
    off::Vector{Int64}
    bond::Vector{Int32}
    moff::Vector{Int64}
    elt::DataType
    # per vertex: canonical axis names (site name or nothing, then the link of each leg)
    canon::Vector{Vector{Any}}
    # host arrays of a solve queued by gpu_solve_submit! (kept alive until gpu_solve_wait!)
    pending::Any
    n_nets::Int
end

function destroy!(d::DeviceNetwork)
    d.ctx == C_NULL || ccall((:itn_destroy, libitn), Int32, (Ptr{Cvoid},), d.ctx)
    d.ctx = C_NULL
    return nothing
end

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
    canon = Vector{Vector{Any}}()
    elt = eltype(unnamed(kettensor(nn, first(verts))))
    keep = Any[]
    for v in verts
        A = kettensor(nn, v)
        names = dimnames(A)
        data = unnamed(A)                       # Julia array, column-major
        st_of = Dict(n => stride(data, i) for (i, n) in enumerate(names))
        sz_of = Dict(n => size(data, i) for (i, n) in enumerate(names))
        sites = sitenames(nn.ket, v)
        length(sites) <= 1 || throw(ArgumentError("vertex $v has several site indices"))
        push!(phys, isempty(sites) ? 1 : sz_of[only(sites)])
        push!(strides, isempty(sites) ? 0 : st_of[only(sites)])
        cv = Any[isempty(sites) ? nothing : only(sites)]
        for w in neighbors(nn, v)
            ln = collect(linknames(nn.ket, v => w))
            length(ln) == 1 || throw(ArgumentError("edge $v => $w carries $(length(ln)) links; fuse them first"))
            slot[v => w] = length(nbr)
            push!(nbr, vidx[w]); push!(bond, sz_of[only(ln)]); push!(strides, st_of[only(ln)])
            push!(cv, only(ln))
        end
        push!(off, length(nbr))
        push!(ptrs, pointer(data)); push!(keep, data)
        push!(canon, cv)
    end
    GC.@preserve keep off nbr bond phys ptrs strides begin
        check(ctx, ccall((:itn_graph_upload, libitn), Int32,
            (Ptr{Cvoid}, Int64, Ptr{Int64}, Ptr{Int64}, Ptr{Int32}, Ptr{Int64}, Ptr{Int32}, Int32, Ptr{Int32}),
            ctx, length(verts), off, nbr, bond, C_NULL, phys, 2, C_NULL))
        check(ctx, ccall((:itn_tensors_upload_strided, libitn), Int32,
            (Ptr{Cvoid}, Int32, Ptr{Ptr{Cvoid}}, Ptr{Int64}), ctx, eltype_code(elt), ptrs, strides))
    end
    moff = cumsum(vcat(Int64(0), Int64.(bond) .^ 2))
    d = DeviceNetwork(ctx, verts, slot, off, bond, moff, elt, canon, nothing, 1)
    finalizer(destroy!, d)
    return d
end

# Messages: D x D operator with (bra, ket) names, packed as m[bra][ket] row-major
# (the C layout): column-major M[bra, ket] is written out transposed.
function pack_messages(d::DeviceNetwork, nn::NormNetwork, cache)
    packed = Vector{d.elt}(undef, d.moff[end])
    for ((a, b), s) in d.slot
        m = cache[a => b]
        ket = only(linknames(nn.ket, a => b))
        M = unnamed(permutedims(m, (braname(nn, ket), ket)))   # rows bra, columns ket
        packed[(d.moff[s + 1] + 1):d.moff[s + 2]] .= vec(permutedims(M, (2, 1)))
    end
    return packed
end

function upload_messages!(d::DeviceNetwork, nn::NormNetwork, cache)
    packed = pack_messages(d, nn, cache)
    GC.@preserve packed check(d.ctx, ccall((:itn_messages_upload, libitn), Int32,
        (Ptr{Cvoid}, Int32, Ptr{Cvoid}), d.ctx, eltype_code(d.elt), packed))
    return d
end

function message_block(d::DeviceNetwork, packed, s)
    D = Int(d.bond[s + 1])
    return permutedims(reshape(packed[(d.moff[s + 1] + 1):d.moff[s + 2]], D, D), (2, 1))  # M[bra, ket]
end

function store_message!(cache, nn::NormNetwork, edge::Pair, M)
    ket = only(linknames(nn.ket, edge))
    copyto!(unnamed(permutedims(cache[edge], (braname(nn, ket), ket))), M)
    return cache
end

function download_messages!(cache, d::DeviceNetwork, nn::NormNetwork)
    packed = Vector{d.elt}(undef, d.moff[end])
    GC.@preserve packed check(d.ctx, ccall((:itn_messages_download, libitn), Int32,
        (Ptr{Cvoid}, Int32, Ptr{Cvoid}), d.ctx, eltype_code(d.elt), packed))
    for ((a, b), s) in d.slot
        store_message!(cache, nn, a => b, message_block(d, packed, s))
    end
    return cache
end

# One device context per (norm network, device) for the per-edge strategy, so that a
# sequence of message_update! calls on the same factors uploads the tensors once.
const EDGE_CONTEXTS = WeakKeyDict{Any, DeviceNetwork}()

"""
    message_update!(alg::GPUMessageUpdate, cache, factors::NormNetwork, edge)

The reference's strategy entry point (beliefpropagation.jl:214-257): recompute the message
on `edge` from its incoming neighbours on the GPU (itn_message_update), normalised by its
sum when `alg.normalize`, and write it into `cache`.
"""
function INN.message_update!(alg::GPUMessageUpdate, cache, factors::NormNetwork, edge)
    d = get!(() -> DeviceNetwork(factors; device = alg.device), EDGE_CONTEXTS, factors)
    upload_messages!(d, factors, cache)
    e = src(edge) => dst(edge)
    s = d.slot[e]
    check(d.ctx, ccall((:itn_message_update, libitn), Int32, (Ptr{Cvoid}, Int64, Int32),
        d.ctx, s, Int32(alg.normalize)))
    packed = Vector{d.elt}(undef, d.moff[end])
    GC.@preserve packed check(d.ctx, ccall((:itn_messages_download, libitn), Int32,
        (Ptr{Cvoid}, Int32, Ptr{Cvoid}), d.ctx, eltype_code(d.elt), packed))
    store_message!(cache, factors, e, message_block(d, packed, s))
    return cache
end

# (maxiter, tol) of the reference's stopping criteria (beliefpropagation.jl:16-55):
# AI.StopAfterIteration, StopWhenConverged and their `|` combination.
gpu_stopping(c::StopWhenConverged) = (nothing, c.tol)
function gpu_stopping(c::AI.StopAfterIteration)
    n = hasproperty(c, :max_iterations) ? c.max_iterations : getfield(c, 1)
    return (Int(n), nothing)
end
function gpu_stopping(c::AI.StopWhenAny)
    maxiter = nothing; tol = nothing
    for x in c.criteria
        m, t = gpu_stopping(x)
        isnothing(m) || (maxiter = m)
        isnothing(t) || (tol = t)
    end
    return (maxiter, tol)
end
gpu_stopping(c) = throw(ArgumentError("stopping criterion $c is not supported by GPUMessageUpdate"))

"""
    DeviceMessageCache

A `MessageCache` together with the device context that holds the same messages (and the
network's tensors), as returned by [`gpu_solve`](@ref); `bethe_free_energy(factors, ::DeviceMessageCache)`
reads the messages where they are.
"""
struct DeviceMessageCache{C}
    cache::C
    dev::DeviceNetwork
end

const SweepGPU = INN.BeliefPropagationSweepAlgorithm{<:GPUMessageUpdate}

# The whole solve as one device call; returns the messages on the host and keeps them on the
# device (DeviceMessageCache).
function gpu_solve(problem::INN.BeliefPropagationProblem{<:NormNetwork},
                   algorithm::INN.BeliefPropagationAlgorithm{<:Any, <:SweepGPU}, iterate)
    nn = problem.factors
    alg = algorithm.subalgorithm.message_update_algorithm
    maxiter, tol = gpu_stopping(algorithm.stopping_criterion)
    d = DeviceNetwork(nn; device = alg.device)
    cache = copy(MessageCache(iterate))
    upload_messages!(d, nn, cache)
    seq = alg.schedule === :sequential
    eslots = seq ? Int64[d.slot[src(e) => dst(e)] for e in algorithm.edges] : Int64[]
    res = Ref{ItnBpResult}()
    GC.@preserve eslots begin
        opts = ItnBpOpts(seq ? 1 : 0, isnothing(maxiter) ? -1 : maxiter,
            isnothing(tol) ? -1.0 : tol, Int32(alg.normalize), precision_code(alg.precision),
            alg.split_sweeps, 0, seq ? pointer(eslots) : C_NULL, length(eslots))
        check(d.ctx, ccall((:itn_bp_run, libitn), Int32,
            (Ptr{Cvoid}, Ref{ItnBpOpts}, Ref{ItnBpResult}), d.ctx, opts, res))
    end
    download_messages!(cache, d, nn)
    return DeviceMessageCache(cache, d)
end

"""
    gpu_solve_submit!(d::DeviceNetwork, tensors::Vector{T}, messages_in::Vector{T},
                      messages_out::Vector{T}; maxiter, precision = :native, split_sweeps = 0,
                      logz = true)
    gpu_solve_wait!(d::DeviceNetwork) -> (ItnBpResult, totals)

A serving loop over many networks of the same graph: `gpu_solve_submit!` queues the uploads of
the packed canonical tensors and messages (the layouts of `itn_tensors_upload` /
`itn_messages_upload`), a parallel solve of `maxiter` sweeps, the log-norm and the download of
the final messages into `messages_out`, and returns at once (`itn_bp_solve_submit`);
`gpu_solve_wait!` waits for them (`itn_bp_solve_wait`) and returns the run result and, with
`logz`, the per-network (re, im) log-norm totals.  With several `DeviceNetwork`s in flight the
uploads of later networks overlap the solves of earlier ones.  The arrays must stay alive and
unchanged until the wait; they are kept in `d` until then.
"""
function gpu_solve_submit!(d::DeviceNetwork, tensors::Vector{T}, messages_in::Vector{T},
                           messages_out::Vector{T}; maxiter::Integer, precision::Symbol = :native,
                           split_sweeps::Integer = 0, logz::Bool = true) where {T}
    opts = ItnBpOpts(0, Int32(maxiter), -1.0, Int32(1), precision_code(precision),
        Int32(split_sweeps), 0, C_NULL, 0)
    check(d.ctx, ccall((:itn_bp_solve_submit, libitn), Int32,
        (Ptr{Cvoid}, Int32, Ptr{Cvoid}, Ptr{Cvoid}, Ref{ItnBpOpts}, Ptr{Cvoid}, Int32),
        d.ctx, eltype_code(T), tensors, messages_in, opts, messages_out, Int32(logz)))
    d.pending = (tensors, messages_in, messages_out, logz)
    return nothing
end

function gpu_solve_wait!(d::DeviceNetwork)
    isnothing(d.pending) && throw(ArgumentError("no solve was submitted on this DeviceNetwork"))
    logz = d.pending[4]
    res = Ref{ItnBpResult}()
    totals = logz ? zeros(Float64, 2 * d.n_nets) : Float64[]
    flags = logz ? zeros(Int32, d.n_nets) : Int32[]
    GC.@preserve totals flags begin
        st = ccall((:itn_bp_solve_wait, libitn), Int32,
            (Ptr{Cvoid}, Ref{ItnBpResult}, Ptr{Float64}, Ptr{Int32}),
            d.ctx, res, logz ? pointer(totals) : C_NULL, logz ? pointer(flags) : C_NULL)
        d.pending = nothing
        check(d.ctx, st)
    end
    return res[], totals
end

"""
    AI.solve(problem::BeliefPropagationProblem{<:NormNetwork}, algorithm; iterate)

Specialisation for a sweep algorithm that carries a `GPUMessageUpdate`: the outer loop
(StopAfterIteration(maxiter) | StopWhenConverged(tol), iteration 0 skipped, delta < tol),
every sweep and the convergence test run on the device in one itn_bp_run call; returns the
`MessageCache`, as `beliefpropagation` promises.
"""
function AI.solve(problem::INN.BeliefPropagationProblem{<:NormNetwork},
                  algorithm::INN.BeliefPropagationAlgorithm{<:Any, <:SweepGPU}; iterate, kwargs...)
    return gpu_solve(problem, algorithm, iterate).cache
end

"""
    bethe_free_energy(factors::NormNetwork, messages::DeviceMessageCache)

messagecache.jl:185-201 on the device: FP64 log-scalars, complex promotion when a real part is
negative, -Inf when an edge scalar is zero.
"""
function INN.bethe_free_energy(nn::NormNetwork, messages::DeviceMessageCache)
    d = messages.dev
    tot = zeros(Float64, 2); flags = zeros(Int32, 1)
    GC.@preserve tot flags check(d.ctx, ccall((:itn_logscalars, libitn), Int32,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Int32}),
        d.ctx, C_NULL, C_NULL, C_NULL, C_NULL, tot, flags))
    (flags[1] & 4) != 0 && return -Inf
    cplx = d.elt <: Complex || (flags[1] & 3) != 0
    return cplx ? complex(tot[1], tot[2]) : tot[1]
end

# ---- contract_network ------------------------------------------------------------------------
"""
    GPUExact(; order = nothing, order_alg = :greedy, precision = :native, device = 0)

`contract_network` algorithm (the counterpart of `Exact`, contract_network.jl:7-10) that
contracts pairwise on the GPU.  `order` is an explicit list of steps in the
itn_contraction_order format or `nothing`; `order_alg` is `:greedy`, `:left`
(LeftAssociative) or `:sweep` (the cheaper of the greedy order and running-product boundary
sweeps: far fewer operations on lattices); `precision = :bf16` uses tcgen05 BF16 hi/lo products on Float32 data,
`:tf32x3` TF32 hi/lo products (FP32 accuracy on the tensor cores).
"""
Base.@kwdef struct GPUExact
    order::Union{Nothing, Vector{Int32}} = nothing
    order_alg::Symbol = :greedy
    precision::Symbol = :native
    device::Int = 0
end

network_tensors(tn::AbstractVector) = collect(tn)
network_tensors(tn::NormNetwork) =
    reduce(vcat, [[kettensor(tn, v), conj_bratensor(tn, v)] for v in vertices(tn)])
network_tensors(tn) = [tn[k] for k in keys(tn)]

"""
    contract_network(alg::GPUExact, tn)

Exact contraction of a vector of ITensors, an `ITensorNetwork` or a `NormNetwork` by pairwise
GPU contractions (itn_contract_network).  Column-major Julia arrays are handed over as
row-major arrays of the reversed axis order; the result comes back the same way.
"""
function INN.contract_network(alg::GPUExact, tn)
    ts = network_tensors(tn)
    T = promote_type(map(t -> eltype(unnamed(t)), ts)...)
    code = Dict{Any, Int64}()
    index_of = Dict{Any, Any}()
    ranks = Int32[]; labels = Int64[]; dims = Int64[]; datas = Any[]
    for t in ts
        names = dimnames(t)
        for (n, i) in zip(names, inds(t))
            index_of[n] = i
        end
        a = convert(Array{T}, unnamed(t))
        push!(datas, a)
        push!(ranks, length(names))
        for k in length(names):-1:1                    # column-major = reversed row-major
            push!(labels, get!(code, names[k], length(code)))
            push!(dims, size(a, k))
        end
    end
    ptrs = Ptr{Cvoid}[pointer(a) for a in datas]
    out_rank = Ref{Int32}(0)
    # the result holds the open indices (labels that occur once)
    count = Dict{Int64, Int}()
    for l in labels
        count[l] = get(count, l, 0) + 1
    end
    cap = prod((dims[k] for k in eachindex(labels) if count[labels[k]] == 1); init = Int64(1))
    out = Vector{T}(undef, cap)
    out_labels = zeros(Int64, 48); out_dims = zeros(Int64, 48)
    steps = isnothing(alg.order) ? C_NULL : alg.order
    order_code = !isnothing(alg.order) ? Int32(2) : alg.order_alg === :left ? Int32(1) :
                 alg.order_alg === :sweep ? Int32(3) : alg.order_alg === :greedy ? Int32(0) :
                 throw(ArgumentError("unknown order_alg $(alg.order_alg)"))
    ctxr = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:itn_create, libitn), Int32, (Ptr{Ptr{Cvoid}}, Int32, Int32), ctxr, alg.device, 0)
    st == ITN_OK || error("itn_create failed with status $st")
    try
        GC.@preserve datas ptrs ranks labels dims out out_labels out_dims steps begin
            check(ctxr[], ccall((:itn_contract_network, libitn), Int32,
                (Ptr{Cvoid}, Int32, Int32, Ptr{Int32}, Ptr{Int64}, Ptr{Int64}, Ptr{Ptr{Cvoid}}, Int32,
                 Ptr{Int32}, Int32, Ptr{Cvoid}, Int64, Ref{Int32}, Ptr{Int64}, Ptr{Int64}, Ptr{Float64}),
                ctxr[], eltype_code(T), length(ts), ranks, labels, dims, ptrs, order_code, steps,
                precision_code(alg.precision), out, cap, out_rank, out_labels, out_dims, C_NULL))
        end
    finally
        ccall((:itn_destroy, libitn), Int32, (Ptr{Cvoid},), ctxr[])
    end
    r = Int(out_rank[])
    name_of = Dict(c => n for (n, c) in code)
    names = [name_of[out_labels[k]] for k in r:-1:1]    # back to column-major order
    shape = Tuple(Int(out_dims[k]) for k in r:-1:1)
    data = reshape(out[1:prod(shape; init = 1)], shape)
    return data[(index_of[n] for n in names)...]
end

# ---- the converged log-norm and its gradient ----------------------------------------------------
"""
    bp_logz(nn, messages; alg = GPUMessageUpdate(schedule = :parallel), edges, maxiter, tol)

Converged BP log-norm of `nn` (beliefpropagation followed by bethe_free_energy), on the GPU;
differentiable through the rrule below.
"""
function bp_logz(nn::NormNetwork, messages; alg = GPUMessageUpdate(; schedule = :parallel),
                 edges = collect(keys(MessageCache(messages))), maxiter = nothing, tol = nothing)
    problem = INN.BeliefPropagationProblem(nn)
    sub = INN.BeliefPropagationSweepAlgorithm(; message_update_algorithm = alg,
        stopping_criterion = AI.StopAfterIteration(length(edges)))
    crit = INN.select_beliefpropagation_stopping_criterion((; maxiter, tol))
    algorithm = INN.BeliefPropagationAlgorithm(; edges, subalgorithm = sub, stopping_criterion = crit)
    dc = gpu_solve(problem, algorithm, messages)
    y = INN.bethe_free_energy(nn, dc)
    return y, dc
end

# The packed canonical gradient (per vertex row-major [site, legs in CSR order]) as an array
# in the ket tensor's own (column-major) index order.
function unpack_gradient(d::DeviceNetwork, nn::NormNetwork, g::Vector, k::Int, toff::Int)
    v = d.verts[k]
    A = kettensor(nn, v)
    names = dimnames(A)
    data = unnamed(A)
    cnames = [n for n in d.canon[k] if !isnothing(n)]
    cdims = Tuple(size(data, findfirst(==(n), collect(names))) for n in cnames)
    n = prod(cdims; init = 1)
    # row-major [c1, c2, ...] = column-major [..., c2, c1]
    blk = reshape(g[(toff + 1):(toff + n)], reverse(cdims))
    pos = [length(cnames) + 1 - findfirst(==(nm), cnames) for nm in names]
    return permutedims(blk, pos), toff + n
end

function ChainRulesCore.rrule(::typeof(bp_logz), nn::NormNetwork, messages; kwargs...)
    y, dc = bp_logz(nn, messages; kwargs...)
    d = dc.dev
    function bp_logz_pullback(ȳ)
        ȳ = ChainRulesCore.unthunk(ȳ)
        total = sum(length(unnamed(kettensor(nn, v))) for v in d.verts)
        g = Vector{d.elt}(undef, total)
        res = Ref{ItnGradResult}()
        GC.@preserve g check(d.ctx, ccall((:itn_bp_grad, libitn), Int32,
            (Ptr{Cvoid}, Ref{ItnGradOpts}, Ptr{Cvoid}, Ref{ItnGradResult}),
            d.ctx, ItnGradOpts(1, 200, 1e-10, 1, 0, 1, 0), g, res))
        # d log Z / d A_v for every ket tensor, each in its own index order: the tangent of
        # the NormNetwork's ket network (its bra is a function of the ket)
        toff = 0
        ket_tangents = Dict{eltype(d.verts), Any}()
        for k in eachindex(d.verts)
            arr, toff = unpack_gradient(d, nn, g, k, toff)
            ket_tangents[d.verts[k]] = ȳ .* arr
        end
        nn_tangent = Tangent{typeof(nn)}(; ket = ket_tangents)
        return NoTangent(), nn_tangent, NoTangent()
    end
    return (y, dc), bp_logz_pullback
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
