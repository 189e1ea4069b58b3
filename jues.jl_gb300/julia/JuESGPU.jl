"""
    JuESGPU

Julia binding of libjuesgpu.so: GB300 implementations of the JuES hot path behind the same
`Wfn`-taking entry points.  `JuESGPU.get_eri`, `tei_transform`, `do_rmp2`, `do_rccd` and
`do_rccsd` take and return what `JuES.IntegralTransformation.get_eri`,
`JuES.Transformation.tei_transform`, `JuES.MollerPlesset.do_rmp2`,
`JuES.CoupledCluster.{mRCCD,RCCD}.do_rccd` and `JuES.CoupledCluster.{RCCSD,mRCCSD}.do_rccsd`
do.  Arrays are passed as they are (Julia is column-major, as is the library); `Wfn{Float32}`
is promoted to Float64.  Non-zero status codes become `error(...)` with the library message.

Set `ENV["JUESGPU_LIB"]` to the path of libjuesgpu.so (default: ../lib/libjuesgpu.so).
"""
module JuESGPU

using JuES.Wavefunction

const LIB = get(ENV, "JUESGPU_LIB", joinpath(@__DIR__, "..", "lib", "libjuesgpu.so"))
# :split is the split form at <= 1 uEh (three integer planes for contractions that produce
# integrals, two for the CC sweeps); :split_bf16 is its earlier name; :split3 / :split2 use
# three / two planes everywhere
const PREC = Dict(:fp64 => Cint(0), :split => Cint(1), :split_bf16 => Cint(1), :split3 => Cint(2),
                  :split2 => Cint(3))
const GUESS = Dict(:zero => Cint(0), :mp2 => Cint(1), :ovov => Cint(2))
const ENOTCONV = 4

struct CCOpts
    maxit::Cint
    e_conv::Cdouble
    r_conv::Cdouble
    diis::Cint
    diis_size::Cint
    precision::Cint
    guess::Cint
    refine::Cint
    transform_precision::Cint
    ccsd_fae::Cint      # 0: Fae's t1 term with <ma|ef> (RCCSD.jl:190); 1: <me|af> (mRCCSD.jl:140)
end

struct IterLog
    iter::Cint
    precision::Cint
    energy::Cdouble
    rnorm::Cdouble
    ms::Cdouble
end

function lasterror()
    buf = Vector{UInt8}(undef, 4096)
    ccall((:jues_last_error, LIB), Cint, (Ptr{UInt8}, Csize_t), buf, length(buf))
    return unsafe_string(pointer(buf))
end

check(st) = st == 0 ? nothing : error("libjuesgpu: " * lasterror())

const CTX = Ref{Ptr{Cvoid}}(C_NULL)
function ctx(device::Integer = 0)
    if CTX[] == C_NULL
        r = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:jues_ctx_create, LIB), Cint, (Cint, Ref{Ptr{Cvoid}}), device, r))
        CTX[] = r[]
    end
    return CTX[]
end

f64(x) = convert(Array{Float64}, x)

"tei_transform(gao, C1, C2, C3, C4, name) -- Transformation.jl:39-93"
function tei_transform(gao::AbstractArray{<:Real,4}, C1, C2, C3, C4, name::String = "default";
                       precision::Symbol = :fp64)
    g = f64(gao); c1, c2, c3, c4 = f64(C1), f64(C2), f64(C3), f64(C4)
    n = size(g, 1)
    out = Array{Float64}(undef, size(c1, 2), size(c2, 2), size(c3, 2), size(c4, 2))
    check(ccall((:jues_tei_transform, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint,
                 Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint, Cint, Ptr{Cdouble}),
                ctx(), g, n, c1, size(c1, 2), c2, size(c2, 2), c3, size(c3, 2), c4, size(c4, 2),
                PREC[precision], out))
    return out
end
tei_transform(gao::AbstractArray{<:Real,4}, C::AbstractMatrix, name::String = "default"; kw...) =
    tei_transform(gao, C, C, C, C, name; kw...)

"get_eri(wfn, spec; notation, fcn) -- IntegralTransformation.jl:38-101"
function get_eri(wfn::Wfn, eri_string::String; notation::String = "phys", fcn::Int = 0,
                 precision::Symbol = :fp64)
    sizeof(eri_string) == 4 || error("Invalid string given to JuES.IntegralTransformation.get_eri: $eri_string")
    s = notation == "phys" ? eri_string[[1, 3, 2, 4]] : eri_string
    d = [c in ('o', 'O') ? wfn.nalpha - fcn : wfn.nvira for c in s]
    shape = notation == "phys" ? (d[1], d[3], d[2], d[4]) : Tuple(d)
    out = Array{Float64}(undef, shape...)
    Co, Cv = f64(wfn.Cao), f64(wfn.Cav)
    check(ccall((:jues_get_eri, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint, Cstring,
                 Cint, Cint, Cint, Ptr{Cdouble}),
                ctx(), f64(wfn.ao_eri), size(Co, 1), Co, size(Co, 2), Cv, size(Cv, 2), eri_string,
                notation == "phys" ? 1 : 0, fcn, PREC[precision], out))
    return out
end

"do_rmp2(refWfn) -- RMP2.jl:11-45"
function do_rmp2(refWfn::Wfn; precision::Symbol = :fp64, kwargs...)
    e = Ref{Cdouble}(0.0)
    Co, Cv = f64(refWfn.Cao), f64(refWfn.Cav)
    check(ccall((:jues_rmp2, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint,
                 Ptr{Cdouble}, Cint, Ref{Cdouble}, Ptr{Cdouble}),
                ctx(), f64(refWfn.ao_eri), size(Co, 1), Co, size(Co, 2), Cv, size(Cv, 2),
                f64(refWfn.epsa), PREC[precision], e, C_NULL))
    return e[]
end

"""
    rmp2_energy(gao, C, nocc, eps; precision = :fp64)

Closed-shell MP2 energy from AO integrals and the full MO matrix; differentiable through the
`rrule` below (dE/dgao and dE/dC from jues_rmp2_adjoint).
"""
function rmp2_energy(gao::AbstractArray{<:Real,4}, C::AbstractMatrix, nocc::Integer,
                     eps::AbstractVector; precision::Symbol = :fp64)
    E, _, _ = rmp2_adjoint(gao, C, nocc, eps, 1.0; want_gao = false, want_C = false, precision)
    return E
end

function rmp2_adjoint(gao, C, nocc, eps, ebar; want_gao = true, want_C = true, precision = :fp64)
    g, Cm, e = f64(gao), f64(C), f64(eps)
    n = size(g, 1)
    gb = want_gao ? similar(g) : nothing
    cb = want_C ? similar(Cm) : nothing
    E = Ref{Cdouble}(0.0)
    check(ccall((:jues_rmp2_adjoint, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint, Cdouble,
                 Ref{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}),
                ctx(), g, n, Cm, nocc, e, PREC[precision], ebar, E,
                gb === nothing ? C_NULL : gb, cb === nothing ? C_NULL : cb))
    return E[], gb, cb
end

# ChainRulesCore rule (loaded when ChainRulesCore is available in the environment)
try
    @eval import ChainRulesCore
    @eval function ChainRulesCore.rrule(::typeof(rmp2_energy), gao, C, nocc, eps; precision = :fp64)
        E, gb, cb = rmp2_adjoint(gao, C, nocc, eps, 1.0; precision)
        function rmp2_pullback(Ebar)
            s = ChainRulesCore.unthunk(Ebar)
            return (ChainRulesCore.NoTangent(), s .* gb, s .* cb, ChainRulesCore.NoTangent(),
                    ChainRulesCore.NoTangent())
        end
        return E, rmp2_pullback
    end
catch
end

function cc_solve(method, refWfn; maxit, r_conv, e_conv, diis, diis_size, precision, guess, refine, ccsd_fae = 0)
    Co, Cv = f64(refWfn.Cao), f64(refWfn.Cav)
    o, v = size(Co, 2), size(Cv, 2)
    opts = Ref(CCOpts(maxit, e_conv, r_conv, diis, diis_size, PREC[precision], GUESS[guess], refine, Cint(-1),
                      Cint(ccsd_fae)))
    e = Ref{Cdouble}(0.0)
    nit = Ref{Cint}(0)
    T2 = Array{Float64}(undef, o, o, v, v)
    t1 = Array{Float64}(undef, o, v)
    log = Vector{IterLog}(undef, max(1, maxit))
    if method == 0
        st = ccall((:jues_rccd, LIB), Cint,
                   (Ptr{Cvoid}, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint,
                    Ptr{Cdouble}, Ref{CCOpts}, Ref{Cdouble}, Ptr{Cdouble}, Ptr{IterLog}, Cint, Ref{Cint}),
                   ctx(), f64(refWfn.ao_eri), size(Co, 1), Co, o, Cv, v, f64(refWfn.epsa), opts, e,
                   T2, log, length(log), nit)
    else
        st = ccall((:jues_rccsd, LIB), Cint,
                   (Ptr{Cvoid}, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint,
                    Ptr{Cdouble}, Ref{CCOpts}, Ref{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble},
                    Ptr{IterLog}, Cint, Ref{Cint}),
                   ctx(), f64(refWfn.ao_eri), size(Co, 1), Co, o, Cv, v, f64(refWfn.epsa), opts, e,
                   t1, T2, log, length(log), nit)
    end
    st == ENOTCONV ? @warn(lasterror()) : check(st)   # mRCCD.jl stops silently at maxit
    return e[], t1, T2, log[1:nit[]]
end

"mRCCD.do_rccd(refWfn; maxit=40, doprint=false, return_T2=false) -- mRCCD.jl:38-118"
function do_rccd(refWfn::Wfn; maxit = 40, doprint = false, return_T2 = false, precision = :fp64,
                 guess = :zero, r_conv = 1e-7, e_conv = 0.0, diis = true, diis_size = 6, refine = 2)
    E, _, T2, log = cc_solve(0, refWfn; maxit, r_conv, e_conv, diis = Cint(diis), diis_size,
                             precision, guess, refine)
    doprint && foreach(r -> println("@CCD ", r.energy), log)
    return return_T2 ? (E, T2) : E
end

"""
    do_rccsd(refWfn; maxit=40, return_T=false) -- RCCSD.jl:33-116 (`ccsd_fae = 0`) and
    mRCCSD.jl:35-101 (`ccsd_fae = 1`: Fae's t1 term as mRCCSD.jl:140)
"""
function do_rccsd(refWfn::Wfn; maxit = 40, return_T = false, precision = :fp64, diis = false,
                  r_conv = 0.0, e_conv = 0.0, diis_size = 6, refine = 0, ccsd_fae = 0, kwargs...)
    E, t1, T2, _ = cc_solve(1, refWfn; maxit, r_conv, e_conv, diis = Cint(diis), diis_size,
                            precision, guess = :mp2, refine, ccsd_fae)
    return return_T ? (E, T2) : E
end

"""
    do_df_rmp2(refWfn, pqP, Jpqh = nothing; precision = :fp64) -- DF-RMP2.jl:1-46

`pqP` and `Jpqh` are what `DF.setup_df(refWfn)` returns (DF.jl:30-51); with `Jpqh ===
nothing`, `pqP` is taken as the fitted b[mu,nu,Q].
"""
function do_df_rmp2(refWfn::Wfn, pqP::AbstractArray{<:Real,3}, Jpqh = nothing; precision::Symbol = :fp64)
    b = f64(pqP)
    J = Jpqh === nothing ? C_NULL : f64(Jpqh)
    Co, Cv = f64(refWfn.Cao), f64(refWfn.Cav)
    e = Ref{Cdouble}(0.0)
    check(ccall((:jues_df_rmp2, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cdouble}, Cint, Cint, Ptr{Cdouble}, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint,
                 Ptr{Cdouble}, Cint, Ref{Cdouble}),
                ctx(), b, size(b, 1), size(b, 3), J, Co, size(Co, 2), Cv, size(Cv, 2), f64(refWfn.epsa),
                PREC[precision], e))
    return e[]
end

"""
    do_df_rccd(refWfn, pqP, Jpqh = nothing; maxit = 40, return_T2 = false) -- DF-RCCD.jl:11-54

The reference's settings by default: T2 = (ia|jb)/D, `maxit` Jacobi sweeps, no DIIS, and
DF-RCCD.jl's WmBeJ (`variant = :reference`; `:rccd` for RCCD.jl's index order).
"""
function do_df_rccd(refWfn::Wfn, pqP::AbstractArray{<:Real,3}, Jpqh = nothing; maxit = 40, doprint = false,
                    return_T2 = false, precision = :fp64, variant = :reference, diis = false, r_conv = 0.0,
                    e_conv = 0.0, diis_size = 6, refine = 0)
    b = f64(pqP)
    J = Jpqh === nothing ? C_NULL : f64(Jpqh)
    Co, Cv = f64(refWfn.Cao), f64(refWfn.Cav)
    o, v = size(Co, 2), size(Cv, 2)
    opts = Ref(CCOpts(maxit, e_conv, r_conv, Cint(diis), diis_size, PREC[precision], GUESS[:mp2], refine, Cint(-1), Cint(0)))
    e = Ref{Cdouble}(0.0)
    nit = Ref{Cint}(0)
    T2 = Array{Float64}(undef, o, o, v, v)
    log = Vector{IterLog}(undef, max(1, maxit))
    st = ccall((:jues_df_rccd, LIB), Cint,
               (Ptr{Cvoid}, Ptr{Cdouble}, Cint, Cint, Ptr{Cdouble}, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint,
                Ptr{Cdouble}, Ref{CCOpts}, Cint, Ref{Cdouble}, Ptr{Cdouble}, Ptr{IterLog}, Cint, Ref{Cint}),
               ctx(), b, size(b, 1), size(b, 3), J, Co, o, Cv, v, f64(refWfn.epsa), opts,
               Cint(variant === :reference ? 0 : 1), e, T2, log, length(log), nit)
    st == ENOTCONV ? @warn(lasterror()) : check(st)
    doprint && foreach(r -> println(r.iter - 1, " @CCD ", r.energy), log[1:nit[]])
    return return_T2 ? (e[], T2) : e[]
end

"compute_pT(; T1, T2, Vvvvo, Vvooo, Vvovo, fo, fv) -- PerturbativeTriples.jl:35-138"
function compute_pT(; T1, T2, Vvvvo, Vvooo, Vvovo, fo, fv, precision::Symbol = :fp64)
    o, v = size(T1)
    e = Ref{Cdouble}(0.0)
    check(ccall((:jues_pT, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble},
                 Ptr{Cdouble}, Cint, Cint, Cint, Ref{Cdouble}),
                ctx(), f64(T1), f64(T2), f64(Vvvvo), f64(Vvooo), f64(Vvovo), f64(fo), f64(fv), o, v,
                PREC[precision], e))
    return e[]
end

"get_fock(wfn; spin = \"alpha\") -- IntegralTransformation.jl:119-141"
function get_fock(wfn::Wfn; spin = "alpha")
    sp = lowercase(spin)
    C, Co = sp in ("alpha", "up", "a") ? (wfn.Ca, wfn.Cao) :
            sp in ("beta", "down", "b") ? (wfn.Cb, wfn.Cbo) :
            error("Invalid Spin option given to JuES.IntegralTransformation.get_fock: $spin")
    Cm = f64(C)
    n, nmo = size(Cm)
    f = Array{Float64}(undef, nmo, nmo)
    check(ccall((:jues_get_fock, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint, Cint, Ptr{Cdouble}),
                ctx(), f64(wfn.ao_eri), f64(wfn.hao), n, Cm, nmo, size(Co, 2), f))
    return f
end

"""
    auto_rccsd(wfn; cc_max_iter = 50, cc_max_rms = 1e-10, cc_e_conv = 1e-10, diis = false,
               do_pT = false, fcn = 0, precision = :fp64) -- AutoRCCSD.jl:193-300

CCSD from the Fock matrix of the orbitals (non-canonical and non-HF references); returns the
correlation energy, or `(E, E_T)` with `do_pT`.
"""
function auto_rccsd(wfn::Wfn; cc_max_iter = 50, cc_max_rms = 1e-10, cc_e_conv = 1e-10, diis = false,
                    do_pT = false, fcn = 0, precision::Symbol = :fp64)
    Cm = f64(wfn.Ca)
    n, nmo = size(Cm)
    ndocc = (wfn.nalpha + wfn.nbeta) ÷ 2
    opts = Ref(CCOpts(cc_max_iter, cc_e_conv, cc_max_rms, Cint(diis), 6, PREC[precision], GUESS[:mp2], 0, Cint(-1), Cint(0)))
    e = Ref{Cdouble}(0.0)
    ept = Ref{Cdouble}(0.0)
    nit = Ref{Cint}(0)
    st = ccall((:jues_auto_rccsd, LIB), Cint,
               (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint, Cint, Cint, Ref{CCOpts}, Cint,
                Ref{Cdouble}, Ref{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{IterLog}, Cint, Ref{Cint}),
               ctx(), f64(wfn.ao_eri), f64(wfn.hao), n, Cm, nmo, ndocc, fcn, opts, Cint(do_pT), e, ept,
               C_NULL, C_NULL, C_NULL, 0, nit)
    st == ENOTCONV ? @warn(lasterror()) : check(st)
    return do_pT ? (e[], ept[]) : e[]
end

end # module
