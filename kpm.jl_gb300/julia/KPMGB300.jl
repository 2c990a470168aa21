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

export GB300CSR

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

end # module
