"""
    KPMGB300

Julia binding of libkpmgb for KPM.jl.  Wrapping a Hamiltonian as `GB300CSR`
routes `kpm_1d!` / `kpm_2d!` (and therefore `kpm_1d`, `kpm_2d`,
`dos_moments`, `cond_moments` on a `RescaledHamiltonian{GB300CSR}`) to the
GB300 kernels through `ccall`; everything else in KPM.jl is untouched.  The
methods are defined on a new type, so nothing in KPM.jl is overwritten.

    using KPM, KPMGB300
    h = KPM.rescale(H; center = true)
    hg = KPM.RescaledHamiltonian(GB300CSR(h.H), h.a, h.b)
    m = KPM.dos_moments(hg; NC = 4096, psi_in = psi)        # GPU moments
    m2 = KPM.cond_moments(hg, GB300CSR(Jx), GB300CSR(Jy); NC = 512, psi_in = psi)

`precision = :ff` selects the emulated-double recurrence (FP32 pipe).
"""
module KPMGB300

using KPM
using LinearAlgebra
using SparseArrays
import ChainRulesCore

export GB300CSR, dos_moments_ad, cond_moments_ad, kubo_bastin_cond_ad, kpm_1d_ensemble,
       pinned_probes

const libkpmgb = get(ENV, "KPMGB_LIB", joinpath(@__DIR__, "..", "kpm_gb300", "_lib", "libkpmgb.so"))

const OK, ERR_ARGUMENT, ERR_NUMERICAL = 0, 1, 2

struct Kpm1dOptions
    precision::Int32
    stability_check::Int32
    use_graph::Int32
    kernel_variant::Int32
end

struct Kpm2dOptions
    arr_size::Int64
    right_block::Int64
    workspace_bytes::Int64
    moment_parity::Int32
    mn_sym::Int32
    precision::Int32
    contraction::Int32
end

_prec(p::Symbol) = p === :fp64 ? Int32(0) : p === :ff ? Int32(1) :
                   throw(ArgumentError("precision must be :fp64 or :ff"))
_contract(c::Symbol) = c === :fp64 ? Int32(0) : c === :split ? Int32(1) :
                       throw(ArgumentError("contraction must be :fp64 or :split"))

function _check(rc::Cint)
    rc == OK && return nothing
    msg = unsafe_string(ccall((:kpmgb_last_error, libkpmgb), Cstring, ()))
    rc == ERR_ARGUMENT && throw(ArgumentError(msg))
    error(msg)  # numerical (stability guard) and device failures
end

"""
    GB300CSR(H::SparseMatrixCSC)

Sparse operator resident on the GPU (uploaded once; the reference converts and
uploads `H` on every moment call).
"""
mutable struct GB300CSR
    handle::Ptr{Cvoid}
    n::Int
    function GB300CSR(H::SparseMatrixCSC)
        Hc = SparseMatrixCSC{ComplexF64,Int64}(H)
        out = Ref{Ptr{Cvoid}}(C_NULL)
        rc = ccall((:kpmgb_operator_create, libkpmgb), Cint,
                   (Int64, Int64, Ptr{Int64}, Ptr{Int64}, Ptr{ComplexF64}, Int32, Ref{Ptr{Cvoid}}),
                   size(Hc, 1), nnz(Hc), Hc.colptr, Hc.rowval, Hc.nzval, Int32(1), out)
        _check(rc)
        op = new(out[], size(Hc, 1))
        finalizer(o -> ccall((:kpmgb_operator_destroy, libkpmgb), Cint, (Ptr{Cvoid},), o.handle), op)
        return op
    end
end
GB300CSR(H::GB300CSR) = H
Base.size(H::GB300CSR) = (H.n, H.n)
Base.size(H::GB300CSR, i::Integer) = H.n
_op(J) = J isa GB300CSR ? J : GB300CSR(sparse(J))

# kpm_1d! equal-vector doubling path (src/moment.jl:420-492)
function KPM.kpm_1d!(H::GB300CSR, NC::Int64, NR::Int64, NH::Int64, mu_all, psi_in;
                     verbose = 0, precision::Symbol = :fp64, stability_check::Bool = false,
                     kwargs...)
    @assert size(mu_all) == (NR, NC)
    @assert (mod(NC, 2) == 0) "Invalid NC: NC should be even."
    @assert (size(psi_in) == (NH, NR)) "Invalid `psi_in` with size $(size(psi_in)). Expecting $(NH), $(NR)"
    psi = Matrix{ComplexF64}(psi_in)
    out = Matrix{ComplexF64}(undef, NR, NC)
    opts = Ref(Kpm1dOptions(_prec(precision), Int32(stability_check), Int32(0), Int32(0)))
    _check(ccall((:kpmgb_kpm1d, libkpmgb), Cint,
                 (Ptr{Cvoid}, Int64, Int64, Int64, Ptr{ComplexF64}, Ptr{ComplexF64}, Ref{Kpm1dOptions}),
                 H.handle, NC, NR, NH, psi, out, opts))
    mu_all .= out
    return nothing
end

# kpm_1d! independent bra/ket path (src/moment.jl:498-556)
function KPM.kpm_1d!(H::GB300CSR, NC::Int64, NR::Int64, NH::Int64, mu_all, psi_in_l, psi_in_r;
                     verbose = 0, precision::Symbol = :fp64, stability_check::Bool = false,
                     kwargs...)
    @assert size(mu_all) == (NR, NC)
    @assert NC >= 2 "Invalid NC: NC should be at least 2."
    pl = Matrix{ComplexF64}(psi_in_l)
    pr = Matrix{ComplexF64}(psi_in_r)
    out = Matrix{ComplexF64}(undef, NR, NC)
    opts = Ref(Kpm1dOptions(_prec(precision), Int32(stability_check), Int32(0), Int32(0)))
    _check(ccall((:kpmgb_kpm1d_lr, libkpmgb), Cint,
                 (Ptr{Cvoid}, Int64, Int64, Int64, Ptr{ComplexF64}, Ptr{ComplexF64},
                  Ptr{ComplexF64}, Ref{Kpm1dOptions}),
                 H.handle, NC, NR, NH, pl, pr, out, opts))
    mu_all .= out
    return nothing
end

_parity(p::Symbol) = p === :NONE ? Int32(0) : p === :ODD ? Int32(1) : p === :EVEN ? Int32(2) :
                     throw(ArgumentError("moment_parity=$(p) not understood."))
_blk(x) = x === :auto ? Int64(0) : Int64(x)

# kpm_2d! (src/moment.jl:887-1088)
function KPM.kpm_2d!(H::GB300CSR, Jα, Jβ, NC::Int64, NR::Int64, NH::Int64, μ, psi_in_l, psi_in_r;
                     arr_size = :auto, right_block = :auto, workspace_bytes = :auto,
                     verbose = 0, mn_sym = false, moment_parity = :NONE,
                     precision::Symbol = :fp64, contraction::Symbol = :fp64, kwargs...)
    arr_size === :auto || arr_size >= 2 ||
        throw(ArgumentError("arr_size must be :auto or an integer at least 2"))
    wb = workspace_bytes === :auto ? Int64(-1) : Int64(workspace_bytes)
    opts = Ref(Kpm2dOptions(_blk(arr_size), _blk(right_block), wb, _parity(moment_parity),
                            Int32(mn_sym), _prec(precision), _contract(contraction)))
    pl = Matrix{ComplexF64}(psi_in_l)
    pr = Matrix{ComplexF64}(psi_in_r)
    out = Matrix{ComplexF64}(undef, NC, NC)
    A, B = _op(Jα), _op(Jβ)
    _check(ccall((:kpmgb_kpm2d, libkpmgb), Cint,
                 (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Int64, Int64, Int64, Ptr{ComplexF64},
                  Ptr{ComplexF64}, Ptr{ComplexF64}, Ref{Kpm2dOptions}),
                 H.handle, A.handle, B.handle, NC, NR, NH, pl, pr, out, opts))
    μ .= out
    return nothing
end

# kpm_1d_current! (src/moment.jl:656-714): the adjoint of Jα is uploaded as its
# own handle and the bra J†ψ is formed on the device.
function KPM.kpm_1d_current!(H::GB300CSR, Jα, NC::Int64, NR::Int64, NH::Int64, mu_all, psi_in;
                             precision::Symbol = :fp64, kwargs...)
    Jadj = Jα isa GB300CSR ? Jα : GB300CSR(sparse(Jα'))
    out = Matrix{ComplexF64}(undef, NR, NC)
    opts = Ref(Kpm1dOptions(_prec(precision), 0, 0, 0))
    _check(ccall((:kpmgb_kpm1d_current, libkpmgb), Cint,
                 (Ptr{Cvoid}, Ptr{Cvoid}, Int64, Int64, Int64, Ptr{ComplexF64}, Ptr{ComplexF64},
                  Ref{Kpm1dOptions}),
                 H.handle, Jadj.handle, NC, NR, NH, Matrix{ComplexF64}(psi_in), out, opts))
    mu_all .= out
    return nothing
end

# chebyshev_action! (src/utils/chebyshev_action.jl:47-122)
function KPM.chebyshev_action!(out::AbstractArray{<:Complex,3}, Hn::GB300CSR, V::AbstractMatrix,
                               C::AbstractMatrix; check_every::Integer = 16, kwargs...)
    NH, NR = size(V)
    NC, K = size(C)
    res = Array{ComplexF64,3}(undef, NH, NR, K)
    _check(ccall((:kpmgb_chebyshev_action, libkpmgb), Cint,
                 (Ptr{Cvoid}, Int64, Int64, Ptr{ComplexF64}, Int64, Int64, Ptr{ComplexF64}, Int64,
                  Ptr{ComplexF64}),
                 Hn.handle, NH, NR, Matrix{ComplexF64}(V), NC, K, Matrix{ComplexF64}(C),
                 Int64(check_every), res))
    out .= res
    return nothing
end

# kpm_3d! (src/moment.jl:1105-1228): mu[:, :, p] = kpm_2d(H, Jγ, Jβ; ψl, T_p(H) Jα ψr)
function KPM.kpm_3d!(H::GB300CSR, Jα, Jβ, Jγ, NC::Int64, NR::Int64, NH::Int64, μ, psi_in_l,
                     psi_in_r; arr_size = :auto, right_block = :auto, precision::Symbol = :fp64,
                     contraction::Symbol = :fp64, kwargs...)
    opts = Ref(Kpm2dOptions(_blk(arr_size), _blk(right_block), Int64(-1), _parity(:NONE),
                            Int32(0), _prec(precision), _contract(contraction)))
    out = Array{ComplexF64,3}(undef, NC, NC, NC)
    A, B, Cg = _op(Jα), _op(Jβ), _op(Jγ)
    _check(ccall((:kpmgb_kpm3d, libkpmgb), Cint,
                 (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Int64, Int64, Int64,
                  Ptr{ComplexF64}, Ptr{ComplexF64}, Ptr{ComplexF64}, Ref{Kpm2dOptions}),
                 H.handle, A.handle, B.handle, Cg.handle, NC, NR, NH,
                 Matrix{ComplexF64}(psi_in_l), Matrix{ComplexF64}(psi_in_r), out, opts))
    μ .= out
    return nothing
end

# DOS reconstruction on the device (src/applications/dos.jl:76-161), or its
# dE_order-th energy derivative (dos.jl:128-139; exact Taylor-series arithmetic
# on the device where the reference nests ForwardDiff), dE_order = 0..4.
function dos_gpu(μ::AbstractVector, a::Real, E_grid::AbstractVector; b::Real = 0.0,
                 kernel = KPM.JacksonKernel, NC::Int64 = length(μ), dE_order::Integer = 0)
    NC = min(NC, length(μ))
    g = Float64[kernel(n, NC) for n = 0:(NC-1)]
    ρ = Vector{Float64}(undef, length(E_grid))
    _check(ccall((:kpmgb_dos_derivative, libkpmgb), Cint,
                 (Ptr{Float64}, Int64, Float64, Float64, Ptr{Float64}, Ptr{Float64}, Int64,
                  Int32, Ptr{Float64}),
                 Vector{Float64}(real.(μ[1:NC])), NC, a, b, g, Vector{Float64}(E_grid),
                 length(E_grid), Int32(dE_order), ρ))
    return ρ
end

# kubo_bastin_cond (src/applications/conductivity.jl:101-157) for a vector of
# Fermi energies in one device pass.
function kubo_bastin_cond_gpu(mu2D, a::Real, Efs::AbstractVector; b::Real = 0.0, NH::Integer,
                              area::Real, beta::Real = Inf, kernel = KPM.JacksonKernel,
                              NC::Int64 = size(mu2D, 1), quad_N::Int64 = 8 * NC,
                              edge_cutoff::Real = 1e-3)
    NC = min(NC, size(mu2D, 1), size(mu2D, 2))
    g = Float64[kernel(n, NC) for n = 0:(NC-1)]
    σ = Vector{Float64}(undef, length(Efs))
    _check(ccall((:kpmgb_kubo_bastin, libkpmgb), Cint,
                 (Ptr{ComplexF64}, Int64, Int64, Float64, Float64, Ptr{Float64}, Int64, Int64,
                  Float64, Float64, Ptr{Float64}, Int64, Float64, Ptr{Float64}),
                 Matrix{ComplexF64}(mu2D), size(mu2D, 1), NC, a, b, Vector{Float64}(Efs),
                 length(Efs), NH, area, beta, g, quad_N, edge_cutoff, σ))
    return σ
end

# dL/dH on the sparsity pattern of H for L = sum_m g[m] mu_m (doubling moments);
# no reference counterpart.  Returns a SparseMatrixCSC with H's pattern.
function kpm_1d_grad(H::SparseMatrixCSC, NC::Int64, psi_in::AbstractMatrix, g::AbstractVector;
                     checkpoint_every::Int64 = 0)
    Hc = SparseMatrixCSC{ComplexF64,Int64}(H)
    op = GB300CSR(Hc)
    NH, NR = size(psi_in)
    out = Vector{ComplexF64}(undef, nnz(Hc))
    _check(ccall((:kpmgb_kpm1d_grad, libkpmgb), Cint,
                 (Ptr{Cvoid}, Int64, Int64, Int64, Ptr{ComplexF64}, Ptr{Float64}, Int64,
                  Ptr{ComplexF64}),
                 op.handle, NC, NR, NH, Matrix{ComplexF64}(psi_in), Vector{Float64}(g),
                 checkpoint_every, out))
    return SparseMatrixCSC(size(Hc, 1), size(Hc, 2), copy(Hc.colptr), copy(Hc.rowval), out)
end

# Batched ensemble: the doubling moments of independent members in one call
# (kpmgb_kpm1d_ensemble; it replaces a loop of kpm_1d! calls over disorder
# realisations).  Hs: rescaled members; psis: their NH_i × NR probe blocks
# (common NR).  Returns one NR × NC moment matrix per member.
function kpm_1d_ensemble(Hs::AbstractVector{<:SparseMatrixCSC}, NC::Int64,
                         psis::AbstractVector{<:AbstractMatrix}; precision::Symbol = :fp64)
    @assert (mod(NC, 2) == 0) "Invalid NC: NC should be even."
    @assert length(Hs) == length(psis) "one probe block per member"
    NR = size(psis[1], 2)
    seg = Int64[0; cumsum([size(H, 1) for H in Hs])]
    op = GB300CSR(blockdiag((SparseMatrixCSC{ComplexF64,Int64}(H) for H in Hs)...))
    psi = vcat((Matrix{ComplexF64}(p) for p in psis)...)
    @assert size(psi) == (seg[end], NR) "every probe block must be (NH_i, NR) with a common NR"
    out = Array{ComplexF64}(undef, NR, NC, length(Hs))
    opts = Ref(Kpm1dOptions(_prec(precision), Int32(0), Int32(0), Int32(0)))
    _check(ccall((:kpmgb_kpm1d_ensemble, libkpmgb), Cint,
                 (Ptr{Cvoid}, Int32, Ptr{Int64}, Int64, Int64, Ptr{ComplexF64},
                  Ptr{ComplexF64}, Ref{Kpm1dOptions}),
                 op.handle, Int32(length(Hs)), seg, NC, NR, psi, out, opts))
    return [out[:, :, i] for i in 1:length(Hs)]
end

# Page-locked host buffer for probe blocks (kpmgb_host_alloc): the library
# reads pinned inputs of 1 MiB or more with a copy kernel over NVLink-C2C.
function pinned_probes(NH::Integer, NR::Integer)
    out = Ref{Ptr{Cvoid}}(C_NULL)
    _check(ccall((:kpmgb_host_alloc, libkpmgb), Cint, (Int64, Ref{Ptr{Cvoid}}),
                 Int64(NH) * NR * sizeof(ComplexF64), out))
    A = unsafe_wrap(Matrix{ComplexF64}, Ptr{ComplexF64}(out[]), (NH, NR); own = false)
    finalizer(_ -> ccall((:kpmgb_host_free, libkpmgb), Cint, (Ptr{Cvoid},), out[]), A)
    return A
end

# Directional derivative of the kpm_1d moments along H + t dH (forward mode):
# the l/r recurrence over [H 0; dH H] with ket [ψ; 0] and bra [0; ψ], the
# direction pre-scaled by a power of two near sqrt(NC) |dH|.  Returns NR × NC.
function kpm_1d_derivative(H::SparseMatrixCSC, dH, NC::Int64, NR::Int64, NH::Int64,
                           psi_in::AbstractMatrix; kwargs...)
    Z = spzeros(ComplexF64, NH, NH)
    g = sqrt(NC) * opnorm(dH, Inf)
    s = g > 0 ? exp2(-round(log2(g))) : 1.0
    Haug = GB300CSR([H Z; s .* SparseMatrixCSC{ComplexF64,Int64}(dH) H])
    z = zeros(ComplexF64, NH, NR)
    dμ = Matrix{ComplexF64}(undef, NR, NC)
    KPM.kpm_1d!(Haug, NC, NR, 2NH, dμ, [z; psi_in], [psi_in; z]; kwargs...)
    return dμ ./ s
end

# Directional derivative of the kpm_2d moments along (H, Jα, Jβ) + t (dH, dJα, dJβ)
# (forward mode; no reference counterpart): one kpm_2d over the 2NH block operators
# [H 0; dH H], [Jα 0; dJα Jα], [dJβ Jβ; Jβ 0] with probes [ψl; 0], [ψr; 0], the
# direction pre-scaled by a power of two that balances the two halves.
function kpm_2d_derivative(H::SparseMatrixCSC, dH, Jα, dJα, Jβ, dJβ, NC::Int64, NR::Int64,
                           NH::Int64, psi_in_l::AbstractMatrix, psi_in_r::AbstractMatrix;
                           kwargs...)
    Z = spzeros(ComplexF64, NH, NH)
    nrm(M) = M === nothing ? 0.0 : opnorm(M, Inf)
    g = sqrt(NC) * nrm(dH)
    for (J, dJ) in ((Jα, dJα), (Jβ, dJβ))
        nrm(J) > 0 && (g = max(g, nrm(dJ) / nrm(J)))
    end
    s = g > 0 ? exp2(-round(log2(g))) : 1.0
    sc(M) = M === nothing ? Z : s .* SparseMatrixCSC{ComplexF64,Int64}(M)
    Haug = GB300CSR([H Z; sc(dH) H])
    Aaug = [Jα Z; sc(dJα) Jα]
    Baug = [sc(dJβ) Jβ; Jβ Z]
    z = zeros(ComplexF64, NH, NR)
    dμ = Matrix{ComplexF64}(undef, NC, NC)
    KPM.kpm_2d!(Haug, Aaug, Baug, NC, NR, 2NH, dμ, [psi_in_l; z], [psi_in_r; z]; kwargs...)
    return dμ ./ s
end

# ---------------------------------------------------------------------------
# Reverse-mode differentiation (no reference counterpart: KPM.jl pushes
# ForwardDiff duals through its recurrences).  The pullbacks call the adjoint
# Chebyshev recurrences of libkpmgb; a cotangent X̄ of a complex array X obeys
# dL = real(dot(X̄, dX)), the ChainRulesCore convention, which is also the
# library's (gradient entry k = dL/dRe(X_k) + i dL/dIm(X_k)).

"""
    kubo_bastin_weights(NC, a, Ef; b, NH, area, beta, kernel, quad_N, edge_cutoff)

NC × NC complex W with `kubo_bastin_cond(μ, a, Ef; ...) == real(sum(W .* μ))`
(src/applications/conductivity.jl:101-157 as a linear map, computed on the GPU).
"""
function kubo_bastin_weights(NC::Int64, a::Real, Ef::Real; b::Real = 0.0, NH::Integer,
                             area::Real, beta::Real = Inf, kernel = KPM.JacksonKernel,
                             quad_N::Int64 = 8 * NC, edge_cutoff::Real = 1e-3)
    g = Float64[kernel(n, NC) for n = 0:(NC-1)]
    W = Matrix{ComplexF64}(undef, NC, NC)
    _check(ccall((:kpmgb_kubo_bastin_weights, libkpmgb), Cint,
                 (Int64, Float64, Float64, Float64, Int64, Float64, Float64, Ptr{Float64}, Int64,
                  Float64, Ptr{ComplexF64}),
                 NC, a, b, Ef, NH, area, beta, g, quad_N, edge_cutoff, W))
    return W
end

"""
    kpm_2d_grad(H, Jα, Jβ, NC, G, psi_in_l, psi_in_r; moment_parity = :NONE)

Gradients (SparseMatrixCSC on each operator's pattern) of
F = real(sum(G .* μ)) with μ = kpm_2d(H, Jα, Jβ, NC, NR, NH; psi_in_l, psi_in_r).
"""
function kpm_2d_grad(H::SparseMatrixCSC, Jα::SparseMatrixCSC, Jβ::SparseMatrixCSC, NC::Int64,
                     G::AbstractMatrix, psi_in_l::AbstractMatrix, psi_in_r::AbstractMatrix;
                     moment_parity::Symbol = :NONE)
    ops = map(M -> SparseMatrixCSC{ComplexF64,Int64}(M), (H, Jα, Jβ))
    Hg, Ag, Bg = map(GB300CSR, ops)
    BHg = GB300CSR(SparseMatrixCSC{ComplexF64,Int64}(sparse(Jβ')))
    NH, NR = size(psi_in_r)
    outs = map(M -> Vector{ComplexF64}(undef, nnz(M)), ops)
    _check(ccall((:kpmgb_kpm2d_grad, libkpmgb), Cint,
                 (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Int64, Int64, Int64,
                  Ptr{ComplexF64}, Ptr{ComplexF64}, Ptr{ComplexF64}, Int32, Ptr{ComplexF64},
                  Ptr{ComplexF64}, Ptr{ComplexF64}),
                 Hg.handle, Ag.handle, Bg.handle, BHg.handle, NC, NR, NH,
                 Matrix{ComplexF64}(psi_in_l), Matrix{ComplexF64}(psi_in_r),
                 Matrix{ComplexF64}(G), _parity(moment_parity), outs[1], outs[2], outs[3]))
    return map((M, g) -> SparseMatrixCSC(size(M, 1), size(M, 2), copy(M.colptr), copy(M.rowval), g),
               ops, outs)
end

"""
    dos_moments_ad(H, NC, psi_in)

Probe-averaged real kpm_1d moments of the (rescaled) sparse H, differentiable
with respect to H's stored entries through `ChainRulesCore.rrule`.
"""
function dos_moments_ad(H::SparseMatrixCSC, NC::Int64, psi_in::AbstractMatrix)
    NH, NR = size(psi_in)
    mu = Matrix{ComplexF64}(undef, NR, NC)
    KPM.kpm_1d!(GB300CSR(H), NC, NR, NH, mu, psi_in)
    return vec(real.(sum(mu; dims = 1))) ./ NR
end

function ChainRulesCore.rrule(::typeof(dos_moments_ad), H::SparseMatrixCSC, NC::Int64,
                              psi_in::AbstractMatrix)
    μ = dos_moments_ad(H, NC, psi_in)
    function dos_moments_pullback(μ̄)
        H̄ = kpm_1d_grad(H, NC, psi_in, Vector{Float64}(ChainRulesCore.unthunk(μ̄)))
        return (ChainRulesCore.NoTangent(), H̄, ChainRulesCore.NoTangent(),
                ChainRulesCore.NoTangent())
    end
    return μ, dos_moments_pullback
end

"""
    cond_moments_ad(H, Jα, Jβ, NC, psi_in_l, psi_in_r)

The NC × NC kpm_2d moment matrix, differentiable with respect to the stored
entries of H, Jα and Jβ through `ChainRulesCore.rrule`.
"""
function cond_moments_ad(H::SparseMatrixCSC, Jα::SparseMatrixCSC, Jβ::SparseMatrixCSC,
                         NC::Int64, psi_in_l::AbstractMatrix, psi_in_r::AbstractMatrix)
    NH, NR = size(psi_in_r)
    μ = Matrix{ComplexF64}(undef, NC, NC)
    KPM.kpm_2d!(GB300CSR(H), Jα, Jβ, NC, NR, NH, μ, psi_in_l, psi_in_r)
    return μ
end

function ChainRulesCore.rrule(::typeof(cond_moments_ad), H::SparseMatrixCSC,
                              Jα::SparseMatrixCSC, Jβ::SparseMatrixCSC, NC::Int64,
                              psi_in_l::AbstractMatrix, psi_in_r::AbstractMatrix)
    μ = cond_moments_ad(H, Jα, Jβ, NC, psi_in_l, psi_in_r)
    function cond_moments_pullback(μ̄)
        # dL = real(dot(μ̄, dμ)) = real(sum(conj(μ̄) .* dμ)): G = conj(μ̄)
        G = conj.(Matrix{ComplexF64}(ChainRulesCore.unthunk(μ̄)))
        H̄, J̄α, J̄β = kpm_2d_grad(H, Jα, Jβ, NC, G, psi_in_l, psi_in_r)
        return (ChainRulesCore.NoTangent(), H̄, J̄α, J̄β, ChainRulesCore.NoTangent(),
                ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent())
    end
    return μ, cond_moments_pullback
end

"""
    kubo_bastin_cond_ad(μ, a, Ef; b, NH, area, kwargs...)

sigma(Ef) from the moment matrix (src/applications/conductivity.jl:101-157),
differentiable with respect to μ through `ChainRulesCore.rrule`; chained with
`cond_moments_ad` it gives d sigma / d(H, Jα, Jβ) by reverse mode.
"""
function kubo_bastin_cond_ad(μ::AbstractMatrix, a::Real, Ef::Real; b::Real = 0.0,
                             NH::Integer, area::Real, kwargs...)
    return only(kubo_bastin_cond_gpu(μ, a, [Ef]; b = b, NH = NH, area = area, kwargs...))
end

function ChainRulesCore.rrule(::typeof(kubo_bastin_cond_ad), μ::AbstractMatrix, a::Real,
                              Ef::Real; b::Real = 0.0, NH::Integer, area::Real, kwargs...)
    σ = kubo_bastin_cond_ad(μ, a, Ef; b = b, NH = NH, area = area, kwargs...)
    W = kubo_bastin_weights(size(μ, 1), a, Ef; b = b, NH = NH, area = area, kwargs...)
    # σ = real(sum(W .* μ)) = real(dot(conj(W), μ)): μ̄ = σ̄ conj(W)
    kubo_pullback(σ̄) = (ChainRulesCore.NoTangent(), ChainRulesCore.unthunk(σ̄) .* conj.(W),
                        ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent())
    return σ, kubo_pullback
end

end # module
