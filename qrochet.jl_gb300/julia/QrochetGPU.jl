# QrochetGPU.jl -- Julia binding of libqrochet_gpu.so (include/qrochet_gpu.h).
#
# Adds methods of Qrochet's Chain API on a device-resident `GPUChain`, so existing Julia code
# that calls canonize!/evolve!/expect/overlap/norm on a Chain can run them on a GB300.  Every
# method is a thin `ccall`; status codes become the exceptions Qrochet throws.
#
# Not executed in this repository's CI: the build image has no Julia.  The Python package in
# ../qrochet calls the same symbols with the same arguments and is tested on the GPU.
module QrochetGPU

using LinearAlgebra
import Qrochet
using Qrochet: Chain, Site, Dense, Open, State, MissingSchmidtCoefficientsException

const libqrochet = get(ENV, "QROCHET_GPU_LIB", joinpath(@__DIR__, "..", "lib", "libqrochet_gpu.so"))

const QR_OK, QR_EINVAL, QR_EASSERT, QR_ENO_SCHMIDT, QR_EDIM = 0, 1, 2, 3, 4
const QR_FP64, QR_MIXED, QR_SPLIT_CONTRACT = 0, 1, 2
const QR_DIR_LEFT, QR_DIR_RIGHT = 0, 1
const QR_METHOD_QR, QR_METHOD_SVD = 0, 1

lasterror() = unsafe_string(ccall((:qr_last_error_string, libqrochet), Cstring, ()))

function check(rc::Cint, bond = nothing)
    rc == QR_OK && return nothing
    msg = lasterror()
    rc == QR_EINVAL && throw(ArgumentError(msg))
    rc == QR_EASSERT && throw(AssertionError(msg))
    rc == QR_ENO_SCHMIDT && throw(MissingSchmidtCoefficientsException(bond))
    rc == QR_EDIM && throw(DimensionMismatch(msg))
    error("libqrochet_gpu: status $rc: $msg")
end

"""
    GPUChain(arrays; order = (:o, :l, :r), precision = :fp64)

MPS resident on the GPU, built from the same arrays as `MPS(arrays)`
(`Chain(State(), Open(), arrays; order)`) or, with `boundary = Periodic()`, as `pMPS(arrays)`.
"""
mutable struct GPUChain
    handle::Ptr{Cvoid}
    n::Int
    d::Int
    periodic::Bool
end
GPUChain(h::Ptr{Cvoid}, n::Int, d::Int) = GPUChain(h, n, d, false)

function GPUChain(arrays::Vector{<:AbstractArray}; order = (:o, :l, :r), precision = :fp64,
                  boundary = Qrochet.Open())
    n = length(arrays)
    ord = collect(order)
    periodic = boundary isa Qrochet.Periodic
    # the reference constructor's checks (Chain.jl:36-41, 64-68), plus matching bond sizes, which the
    # library relies on when it reads each array (cl * d * cr elements)
    n >= 2 || throw(ArgumentError("a Chain needs at least 2 sites"))
    if periodic
        @assert all(==(3) ∘ ndims, arrays) "All arrays must have 3 dimensions"
    else
        @assert ndims(arrays[1]) == 2 "First array must have 2 dimensions"
        @assert all(==(3) ∘ ndims, arrays[2:end-1]) "All arrays must have 3 dimensions"
        @assert ndims(arrays[end]) == 2 "Last array must have 2 dimensions"
    end
    issetequal(ord, [:o, :l, :r]) || throw(ArgumentError("order must be a permutation of [\"o\", \"l\", \"r\"]"))
    dims = map(enumerate(arrays)) do (i, a)
        sub = filter(x -> periodic || !((i == 1 && x == :l) || (i == n && x == :r)), ord)
        Dict(zip(sub, size(a)))
    end
    d = dims[1][:o]
    all(x -> x[:o] == d, dims) || throw(DimensionMismatch("all sites must share the physical dimension"))
    for i in 1:(periodic ? n : n - 1)
        r, l = dims[i][:r], dims[mod1(i + 1, n)][:l]
        r == l || throw(DimensionMismatch("bond $i: $r != $l"))
    end
    h = Ref{Ptr{Cvoid}}(C_NULL)
    if periodic
        bonds = Cint[dims[i][:r] for i in 1:n]
        check(ccall((:qr_chain_create_periodic, libqrochet), Cint, (Cint, Cint, Ptr{Cint}, Ref{Ptr{Cvoid}}),
                    n, d, bonds, h))
    else
        bonds = Cint[dims[i][:r] for i in 1:n-1]
        check(ccall((:qr_chain_create, libqrochet), Cint, (Cint, Cint, Ptr{Cint}, Ref{Ptr{Cvoid}}), n, d, bonds, h))
    end
    chain = GPUChain(h[], n, d, periodic)
    finalizer(c -> ccall((:qr_chain_free, libqrochet), Cint, (Ptr{Cvoid},), c.handle), chain)
    ordstr = join(String.(ord))
    for (i, a) in enumerate(arrays)
        buf = convert(Array{ComplexF64}, a)
        check(ccall((:qr_chain_upload_site, libqrochet), Cint, (Ptr{Cvoid}, Cint, Ptr{ComplexF64}, Cstring),
                    chain.handle, i - 1, buf, ordstr))
    end
    setprecision!(chain, precision)
    return chain
end

# :fp64 (all ComplexF64), :mixed (the mixed-precision SVD and theta GEMM of two-site gates),
# :split (environment contractions on the tensor cores as BF16x3 products), :mixed_split (both)
const PRECISIONS = Dict(:fp64 => QR_FP64, :mixed => QR_MIXED, :split => QR_SPLIT_CONTRACT,
                        :mixed_split => QR_MIXED | QR_SPLIT_CONTRACT)

function setprecision!(c::GPUChain, p::Symbol)
    haskey(PRECISIONS, p) || throw(ArgumentError("Unknown precision=:$p"))
    check(ccall((:qr_chain_set_precision, libqrochet), Cint, (Ptr{Cvoid}, Cint), c.handle, PRECISIONS[p]))
    return c
end

function Base.copy(c::GPUChain)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:qr_chain_copy, libqrochet), Cint, (Ptr{Cvoid}, Ref{Ptr{Cvoid}}), c.handle, h))
    out = GPUChain(h[], c.n, c.d, c.periodic)
    finalizer(x -> ccall((:qr_chain_free, libqrochet), Cint, (Ptr{Cvoid},), x.handle), out)
    return out
end

function wrap(h::Ptr{Cvoid})
    n, cl, d, cr, per = Ref{Cint}(0), Ref{Cint}(0), Ref{Cint}(0), Ref{Cint}(0), Ref{Cint}(0)
    check(ccall((:qr_chain_nsites, libqrochet), Cint, (Ptr{Cvoid}, Ref{Cint}), h, n))
    check(ccall((:qr_chain_site_dims, libqrochet), Cint, (Ptr{Cvoid}, Cint, Ref{Cint}, Ref{Cint}, Ref{Cint}),
                h, 0, cl, d, cr))
    check(ccall((:qr_chain_boundary, libqrochet), Cint, (Ptr{Cvoid}, Ref{Cint}), h, per))
    out = GPUChain(h, Int(n[]), Int(d[]), per[] != 0)
    finalizer(x -> ccall((:qr_chain_free, libqrochet), Cint, (Ptr{Cvoid},), x.handle), out)
    return out
end

"""`rand(Chain, Open, State; n, p, χ, eltype)` generated on the GPU (the reference's bond pattern
and Gram-Schmidt isometries; the random stream is the library's own, keyed by `seed`)."""
function Base.rand(::Type{GPUChain}, ::Type{Qrochet.Open}, ::Type{Qrochet.State}; n::Integer, χ::Integer,
                   p::Integer = 2, eltype = Float64, seed::Integer = 0)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:qr_chain_random, libqrochet), Cint, (Cint, Cint, Cint, UInt64, Cint, Ref{Ptr{Cvoid}}),
                n, p, χ, UInt64(seed), eltype <: Complex ? 1 : 0, h))
    return wrap(h[])
end

"""Checkpoint: sites in the reference's (:o, :l, :r) layout, bond dimensions, Λ, precision."""
save(c::GPUChain, path::AbstractString) =
    check(ccall((:qr_chain_save, libqrochet), Cint, (Ptr{Cvoid}, Cstring), c.handle, path))

function load(path::AbstractString)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:qr_chain_load, libqrochet), Cint, (Cstring, Ref{Ptr{Cvoid}}), path, h))
    return wrap(h[])
end

"""Reads a checkpoint on the host (no GPU needed): returns `(arrays, Λs, periodic)` with the arrays
exactly as `MPS(arrays)` / `pMPS(arrays)` take them.  Layout (little-endian): "QRCHAIN1", Int32 n, d,
precision, periodic, Int32 bond dimensions, UInt8 Λ flags per bond, the site arrays in (o, l, r)
column-major order, then Float64 Λ for every flagged bond."""
function read_checkpoint(path::AbstractString)
    open(path, "r") do io
        String(read(io, 8)) == "QRCHAIN1" || throw(ArgumentError("not a chain checkpoint"))
        n, d, _, per = (Int(read(io, Int32)) for _ in 1:4)
        nb = per == 1 ? n : n - 1
        bonds = [Int(read(io, Int32)) for _ in 1:nb]
        flags = [read(io, UInt8) for _ in 1:n-1]
        shapes = if per == 1
            [(d, bonds[mod1(i - 1, n)], bonds[i]) for i in 1:n]
        else
            [i == 1 ? (d, bonds[1]) : i == n ? (d, bonds[n-1]) : (d, bonds[i-1], bonds[i]) for i in 1:n]
        end
        arrays = [(a = Array{ComplexF64}(undef, shp...); read!(io, a); a) for shp in shapes]
        lams = [flags[b] == 1 ? (v = Vector{Float64}(undef, bonds[b]); read!(io, v); v) : nothing for b in 1:n-1]
        return arrays, lams, per == 1
    end
end

Qrochet.nsites(c::GPUChain) = c.n
# the lane queries of a Quantum network (src/Quantum.jl:118-143, 228-239): a GPUChain is a state
Qrochet.socket(::GPUChain) = State()
Qrochet.boundary(c::GPUChain) = c.periodic ? Qrochet.Periodic() : Qrochet.Open()
Qrochet.sites(c::GPUChain) = [Site(i) for i in 1:c.n]
Qrochet.outputs(c::GPUChain) = Qrochet.sites(c)
Qrochet.inputs(::GPUChain) = Site[]
Qrochet.noutputs(c::GPUChain) = c.n
Qrochet.ninputs(::GPUChain) = 0

function bond_dims(c::GPUChain)
    out = Vector{Cint}(undef, c.periodic ? c.n : c.n - 1)
    check(ccall((:qr_chain_bond_dims, libqrochet), Cint, (Ptr{Cvoid}, Ptr{Cint}), c.handle, out))
    return Int.(out)
end

"""Site tensor `i` back on the host, dims in `order` (`arrays(::Chain)` layout)."""
function sitearray(c::GPUChain, i::Integer; order = (:o, :l, :r))
    cl, d, cr = Ref{Cint}(0), Ref{Cint}(0), Ref{Cint}(0)
    check(ccall((:qr_chain_site_dims, libqrochet), Cint, (Ptr{Cvoid}, Cint, Ref{Cint}, Ref{Cint}, Ref{Cint}),
                c.handle, i - 1, cl, d, cr))
    dims = Dict(:l => cl[], :o => d[], :r => cr[])
    sub = filter(x -> c.periodic || !((i == 1 && x == :l) || (i == c.n && x == :r)), collect(order))
    out = Array{ComplexF64}(undef, (dims[x] for x in sub)...)
    check(ccall((:qr_chain_download_site, libqrochet), Cint, (Ptr{Cvoid}, Cint, Ptr{ComplexF64}, Cstring),
                c.handle, i - 1, out, join(String.(collect(order)))))
    return out
end

"""Λ on the bond between sites `i` and `i+1` (`tensors(tn; between)`), or `nothing`."""
function spectrum(c::GPUChain, i::Integer)
    flag = Ref{Cint}(0)
    check(ccall((:qr_chain_has_lambda, libqrochet), Cint, (Ptr{Cvoid}, Cint, Ref{Cint}), c.handle, i - 1, flag))
    flag[] == 0 && return nothing
    len = Ref{Cint}(0)
    check(ccall((:qr_chain_get_lambda, libqrochet), Cint, (Ptr{Cvoid}, Cint, Ptr{Float64}, Ref{Cint}),
                c.handle, i - 1, C_NULL, len))
    out = Vector{Float64}(undef, len[])
    check(ccall((:qr_chain_get_lambda, libqrochet), Cint, (Ptr{Cvoid}, Cint, Ptr{Float64}, Ref{Cint}),
                c.handle, i - 1, out, len))
    return out
end

# ---- the reference's Chain methods ----------------------------------------------------------
_dir(d::Symbol) = d === :left ? QR_DIR_LEFT : d === :right ? QR_DIR_RIGHT : throw(ArgumentError("Unknown direction=:$d"))
_method(m::Symbol) = m === :qr ? QR_METHOD_QR : m === :svd ? QR_METHOD_SVD : throw(ArgumentError("Unknown factorization method=:$m"))

function Qrochet.canonize_site!(c::GPUChain, site::Site; direction::Symbol, method = :qr)
    check(ccall((:qr_canonize_site, libqrochet), Cint, (Ptr{Cvoid}, Cint, Cint, Cint), c.handle,
                Qrochet.id(site) - 1, _dir(direction), _method(method)))
    return c
end

Qrochet.canonize!(c::GPUChain) = (check(ccall((:qr_canonize, libqrochet), Cint, (Ptr{Cvoid},), c.handle)); c)
Qrochet.canonize(c::GPUChain) = Qrochet.canonize!(copy(c))

Qrochet.mixed_canonize!(c::GPUChain, center::Site) =
    (check(ccall((:qr_mixed_canonize, libqrochet), Cint, (Ptr{Cvoid}, Cint), c.handle, Qrochet.id(center) - 1)); c)

# normalize!(tn, root; p) (Chain.jl:532-536): p = 2 on the device; another p re-scales the Lambda
# between root - 1 and root on the host after the mixed canonization
function LinearAlgebra.normalize!(c::GPUChain, root::Site; p::Real = 2)
    if p == 2
        check(ccall((:qr_normalize, libqrochet), Cint, (Ptr{Cvoid}, Cint), c.handle, Qrochet.id(root) - 1))
        return c
    end
    Qrochet.mixed_canonize!(c, root)
    r = Qrochet.id(root)
    λ = spectrum(c, r - 1)
    λ === nothing && throw(MissingSchmidtCoefficientsException((Site(r - 1), root)))
    normalize!(λ, p)
    check(ccall((:qr_chain_set_lambda, libqrochet), Cint, (Ptr{Cvoid}, Cint, Ptr{Float64}, Cint), c.handle, r - 2, λ,
                length(λ)))
    return c
end

# the non-mutating forms (Chain.jl:335, 378, 460, 499)
Qrochet.canonize_site(c::GPUChain, args...; kwargs...) = Qrochet.canonize_site!(copy(c), args...; kwargs...)
Qrochet.mixed_canonize(c::GPUChain, args...; kwargs...) = Qrochet.mixed_canonize!(copy(c), args...; kwargs...)
Qrochet.truncate(c::GPUChain, args...; kwargs...) = Qrochet.truncate!(copy(c), args...; kwargs...)

"""||A^H A - I||_F of site `site` viewed [(l,o) x r] (`QR_DIR_LEFT`) or ||A A^H - I||_F over
[l x (o,r)] (`QR_DIR_RIGHT`); the open ends get the reference's dummy dimension of size 1."""
function canonicality_error(c::GPUChain, site::Site, dir)
    err = Ref{Float64}(0)
    check(ccall((:qr_canonicality_error, libqrochet), Cint, (Ptr{Cvoid}, Cint, Cint, Ref{Float64}), c.handle,
                Qrochet.id(site) - 1, dir, err))
    return err[]
end

# isapprox(A^H A, I; atol) with atol > 0 compares the Frobenius norm of the difference (Chain.jl:424-458)
Qrochet.isleftcanonical(c::GPUChain, site::Site; atol::Real = 1e-12) = canonicality_error(c, site, QR_DIR_LEFT) <= atol
Qrochet.isrightcanonical(c::GPUChain, site::Site; atol::Real = 1e-12) = canonicality_error(c, site, QR_DIR_RIGHT) <= atol

# contract!(tn, Val(:between), site1, site2; direction, delete_Λ) (Chain.jl:309-333)
function Qrochet.Tenet.contract!(c::GPUChain, ::Val{:between}, site1::Site, site2::Site; direction::Symbol = :left,
                                 delete_Λ = true)
    check(ccall((:qr_contract_between, libqrochet), Cint, (Ptr{Cvoid}, Cint, Cint, Cint, Cint), c.handle,
                Qrochet.id(site1) - 1, Qrochet.id(site2) - 1, _dir(direction), delete_Λ))
    return c
end

function Qrochet.truncate!(c::GPUChain, bond; threshold = nothing, maxdim = nothing)
    s1, s2 = Qrochet.id.(bond)
    # -1 tells the C ABI "no maxdim"; a maxdim below 1 keeps nothing, as 1:min(dim, maxdim) does
    check(ccall((:qr_truncate, libqrochet), Cint, (Ptr{Cvoid}, Cint, Cint, Cdouble, Cint), c.handle, s1 - 1, s2 - 1,
                isnothing(threshold) ? NaN : Float64(threshold), isnothing(maxdim) ? -1 : max(0, maxdim)), Tuple(bond))
    return c
end

"""M[(o_1..o_k),(i_1..i_k)] (left lane slowest) of a Dense gate for `lanes`, returned as its
transpose so that the array's column-major memory is M in row-major order, which is how every
gate crosses the C ABI (`qr_evolve_1site`, `qr_evolve_2site`, `qr_evolve_layer`, `qr_expect`)."""
function gatematrix(gate::Dense, lanes)
    arr = only(Qrochet.arrays(gate))
    ind = Qrochet.inds(gate; at = Site(first(lanes)))  # dims follow `sites` (Dense.jl:21-34)
    sites = [s for s in Qrochet.sites(gate)]
    perm = vcat([findfirst(==(Site(l)), sites) for l in lanes], [findfirst(==(Site(l; dual = true)), sites) for l in lanes])
    t = permutedims(arr, perm)
    d = size(t, 1)
    k = length(lanes)
    # column-major reshape groups the first lane fastest; reverse lanes to make it slowest
    t = permutedims(t, vcat(reverse(1:k), reverse(k+1:2k)))
    M = reshape(t, d^k, d^k)
    return collect(transpose(M))  # row-major storage of M
end

# the checks evolve! makes before it touches the chain (Chain.jl:552-581); returns the sorted lanes
function checkgate(c::GPUChain, gate::Dense)
    Qrochet.socket(gate) isa Qrochet.Operator ||
        throw(ArgumentError("Gate must be an operator, but got $(Qrochet.socket(gate))"))
    issetequal(adjoint.(Qrochet.inputs(gate)), Qrochet.outputs(gate)) ||
        throw(ArgumentError("Gate inputs ($(Qrochet.inputs(gate))) and outputs ($(Qrochet.outputs(gate))) must be the same"))
    all(s -> 1 <= Qrochet.id(s) <= c.n, Qrochet.outputs(gate)) ||
        throw(ArgumentError("Gate inputs ($(Qrochet.inputs(gate))) must be a subset of the TN sites"))
    lanes = sort!(map(Qrochet.id, Qrochet.outputs(gate)))
    length(lanes) > 2 && throw(ArgumentError("Invalid number of lanes $(length(lanes)), maximum is 2"))
    length(lanes) == 2 && lanes[2] != lanes[1] + 1 && throw(ArgumentError("Gate lanes must be contiguous"))
    return lanes
end

function Qrochet.evolve!(c::GPUChain, gate::Dense; threshold = nothing, maxdim = nothing, iscanonical = false,
                         renormalize = false)
    lanes = checkgate(c, gate)
    M = ComplexF64.(gatematrix(gate, lanes))
    if length(lanes) == 1
        check(ccall((:qr_evolve_1site, libqrochet), Cint, (Ptr{Cvoid}, Cint, Ptr{ComplexF64}), c.handle, lanes[1] - 1, M))
    else
        check(ccall((:qr_evolve_2site, libqrochet), Cint,
                    (Ptr{Cvoid}, Cint, Ptr{ComplexF64}, Cdouble, Cint, Cint, Cint), c.handle, lanes[1] - 1, M,
                    isnothing(threshold) ? NaN : Float64(threshold), isnothing(maxdim) ? -1 : max(0, maxdim),
                    iscanonical, renormalize))
    end
    return c
end

# A brick-wall layer of two-site gates on disjoint site pairs, several at a time (the inner loop of
# a TEBD evolve! over one layer); the result is that of evolve! on each gate in turn.
function evolve_layer!(c::GPUChain, gates::AbstractVector{<:Dense}; threshold = nothing, maxdim = nothing,
                       iscanonical = false, renormalize = false, lanes = 0)
    sites = Cint[]
    mats = ComplexF64[]
    for gate in gates
        ls = checkgate(c, gate)
        length(ls) == 2 || throw(ArgumentError("evolve_layer! takes two-site gates"))
        push!(sites, ls[1] - 1)
        append!(mats, vec(ComplexF64.(gatematrix(gate, ls))))  # memory order as qr_evolve_2site takes it
    end
    check(ccall((:qr_evolve_layer, libqrochet), Cint,
                (Ptr{Cvoid}, Cint, Ptr{Cint}, Ptr{ComplexF64}, Cdouble, Cint, Cint, Cint, Cint),
                c.handle, length(sites), sites, mats, isnothing(threshold) ? NaN : Float64(threshold),
                isnothing(maxdim) ? -1 : max(0, maxdim), iscanonical, renormalize, lanes))
    return c
end

function Qrochet.overlap(a::GPUChain, b::GPUChain)
    out = Ref{ComplexF64}(0)
    check(ccall((:qr_overlap, libqrochet), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ref{ComplexF64}), a.handle, b.handle, out))
    return out[]
end
# the socket-dispatched form overlap(a, b) forwards to (Chain.jl:737-740)
Qrochet.overlap(::State, a::GPUChain, ::State, b::GPUChain) = Qrochet.overlap(a, b)

function LinearAlgebra.norm(c::GPUChain, p::Real = 2)
    p == 2 || throw(ArgumentError("only L2-norm is implemented yet"))
    out = Ref{Float64}(0)
    check(ccall((:qr_norm, libqrochet), Cint, (Ptr{Cvoid}, Ref{Float64}), c.handle, out))
    return out[]
end

function Qrochet.expect(c::GPUChain, observables)
    firsts, nl, mats = Cint[], Cint[], ComplexF64[]
    for o in observables
        lanes = checkgate(c, o)
        push!(firsts, lanes[1] - 1)
        push!(nl, length(lanes))
        append!(mats, vec(ComplexF64.(gatematrix(o, lanes))))  # row-major M, as for qr_evolve_2site
    end
    out = Ref{ComplexF64}(0)
    check(ccall((:qr_expect, libqrochet), Cint, (Ptr{Cvoid}, Cint, Ptr{Cint}, Ptr{Cint}, Ptr{ComplexF64}, Ref{ComplexF64}),
                c.handle, length(firsts), firsts, nl, mats, out))
    return out[]
end

"""
    GPUMPO(arrays; order = (:o, :i, :l, :r))

Open-boundary MPO resident on the GPU, built from the same arrays as `MPO(arrays)`
(`Chain(Operator(), Open(), arrays; order)`, Chain.jl:133-172): the ends drop `:l` / `:r`.
"""
mutable struct GPUMPO
    handle::Ptr{Cvoid}
    n::Int
    d::Int
end

function GPUMPO(arrays::Vector{<:AbstractArray}; order = (:o, :i, :l, :r))
    n = length(arrays)
    ord = collect(order)
    n >= 2 || throw(ArgumentError("an MPO needs at least 2 sites"))
    @assert ndims(arrays[1]) == 3 "First array must have 3 dimensions"
    @assert all(==(4) ∘ ndims, arrays[2:end-1]) "All arrays must have 4 dimensions"
    @assert ndims(arrays[end]) == 3 "Last array must have 3 dimensions"
    issetequal(ord, [:o, :i, :l, :r]) || throw(ArgumentError("order must be a permutation of [\"o\", \"i\", \"l\", \"r\"]"))
    dims = map(enumerate(arrays)) do (i, a)
        sub = filter(x -> !((i == 1 && x == :l) || (i == n && x == :r)), ord)
        Dict(zip(sub, size(a)))
    end
    d = dims[1][:o]
    all(x -> x[:o] == d && x[:i] == d, dims) || throw(DimensionMismatch("all sites must share the physical dimension"))
    for i in 1:n-1
        dims[i][:r] == dims[i+1][:l] || throw(DimensionMismatch("MPO bond $i: $(dims[i][:r]) != $(dims[i+1][:l])"))
    end
    h = Ref{Ptr{Cvoid}}(C_NULL)
    bonds = Cint[dims[i][:r] for i in 1:n-1]
    check(ccall((:qr_mpo_create, libqrochet), Cint, (Cint, Cint, Ptr{Cint}, Ref{Ptr{Cvoid}}), n, d, bonds, h))
    w = GPUMPO(h[], n, d)
    finalizer(x -> ccall((:qr_mpo_free, libqrochet), Cint, (Ptr{Cvoid},), x.handle), w)
    ordstr = join(String.(ord))
    for (i, a) in enumerate(arrays)
        buf = convert(Array{ComplexF64}, a)
        check(ccall((:qr_mpo_upload_site, libqrochet), Cint, (Ptr{Cvoid}, Cint, Ptr{ComplexF64}, Cstring),
                    w.handle, i - 1, buf, ordstr))
    end
    return w
end

"""`<ψ|H|ψ>`: `contract(merge(Quantum(ψ), Quantum(H), Quantum(ψ)'))` (src/Quantum.jl:330-348) as one
environment sweep on the device."""
function mpo_expect(ψ::GPUChain, H::GPUMPO)
    out = Ref{ComplexF64}(0)
    check(ccall((:qr_mpo_expect, libqrochet), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ref{ComplexF64}), ψ.handle, H.handle, out))
    return out[]
end

export GPUChain, GPUMPO, mpo_expect, bond_dims, sitearray, spectrum, setprecision!, save, load, read_checkpoint

end # module
