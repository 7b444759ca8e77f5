"""
    DPFEHMGPU

Julia binding of libdpfehm_gpu.so (C ABI in include/dpfehm_gpu.h): drop-in
versions of `DPFEHM.groundwater_steadystate` and its `ChainRulesCore.rrule`
(DPFEHM src/groundwater.jl:75-109) that solve on a GB300 through `ccall`.

Not exercised in this repository's tests (no Julia toolchain is available where
they run); the same C entry points are exercised through ctypes.
"""
module DPFEHMGPU

import ChainRulesCore

const libdpf = get(ENV, "DPFEHM_GPU_LIB", joinpath(@__DIR__, "..", "_build", "libdpfehm_gpu.so"))

const DPF_OK = Cint(0)
const DPF_NOT_CONVERGED = Cint(2)

mutable struct Options
    reltol::Cdouble
    maxiter::Cint
    precision::Cint
    cheb_degree::Cint
    cheb_lo::Cdouble
    coarse_scale::Cdouble
    max_coarse::Cint
    max_outer::Cint
    use_graphs::Cint
    check_every::Cint
    blocks_per_sm::Cint
    tail_cells::Cint
    plane::Cint
    plane_cells::Cint
    plane_blocks_per_sm::Cint
    df_plane_cells::Cint
    df_plane_blocks_per_sm::Cint
    tail_cluster::Cint
    plane_levels::Cint
    streams::Cint
    fuse::Cint
    solver::Cint
end

"""The library defaults with any `dpf_options` field overridden by keyword (`precision` as
`:fp64` or `:mixed`)."""
function default_options(; kwargs...)
    o = Options(0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0)
    ccall((:dpf_default_options, libdpf), Cvoid, (Ref{Options},), o)
    for (k, v) in pairs(kwargs)
        if k === :precision
            o.precision = v == :mixed ? 1 : 0
        else
            setfield!(o, k, convert(fieldtype(Options, k), v))
        end
    end
    return o
end

lasterror(h) = unsafe_string(ccall((:dpf_last_error, libdpf), Cstring, (Ptr{Cvoid},), h))

function check(h, rc)
    rc == DPF_OK && return nothing
    rc == DPF_NOT_CONVERGED && (@warn "solve did not reach its tolerance: $(lasterror(h))"; return nothing)
    error("libdpfehm_gpu status $rc: $(lasterror(h))")
end

"""A problem handle: topology, multigrid hierarchy and the last forward state on the GPU."""
mutable struct Problem
    ptr::Ptr{Cvoid}
    N::Int
    F::Int
end

function Problem(neighbors, areasoverlengths, dirichletnodes, N; volumes=nothing, kwargs...)
    F = length(neighbors)
    a = Int64[p[1] - 1 for p in neighbors]          # 1-based pairs -> 0-based arrays
    b = Int64[p[2] - 1 for p in neighbors]
    aol = Vector{Float64}(areasoverlengths[1:F])
    dn = Int64[d - 1 for d in dirichletnodes]
    vol = volumes === nothing ? Ptr{Float64}(C_NULL) : Vector{Float64}(volumes)  # ccall roots a Vector argument
    opts = default_options(; kwargs...)
    out = Ref{Ptr{Cvoid}}(C_NULL)
    rc = ccall((:dpf_create, libdpf), Cint,
        (Int64, Int64, Ptr{Int64}, Ptr{Int64}, Ptr{Float64}, Ptr{Float64}, Int64, Ptr{Int64}, Ref{Options},
         Ref{Ptr{Cvoid}}), N, F, a, b, aol, vol, length(dn), dn, opts, out)
    rc == DPF_OK || error("dpf_create failed ($rc): $(lasterror(C_NULL))")
    p = Problem(out[], N, F)
    finalizer(p) do q
        q.ptr == C_NULL || ccall((:dpf_destroy, libdpf), Cvoid, (Ptr{Cvoid},), q.ptr)
        q.ptr = C_NULL
    end
    return p
end

# Array arguments. A host Vector{Float64} is passed as is and any other host vector as a
# Float64 copy. A device array (CUDA.jl's CuArray{Float64}, whose `pointer` is a CuPtr) is
# passed by its device address: the library recognises device pointers and reads and writes
# them in place, so a CuArray never goes through host memory. Outputs are allocated with
# `similar`, on the side (host or device) of the input they follow.
isdevice(x) = nameof(typeof(x)) === :CuArray
floatbuf(x::Vector{Float64}) = x
floatbuf(x) = isdevice(x) && eltype(x) === Float64 ? x : Vector{Float64}(x)
rawptr(x::Array{Float64}) = pointer(x)
rawptr(x) = Ptr{Float64}(reinterpret(UInt, pointer(x)))   # a device array's address
outbuf(like, n) = isdevice(like) ? similar(like, Float64, n) : Vector{Float64}(undef, n)

function forward(p::Problem, Ks, dirichleths, Qs)
    K = floatbuf(Ks); d = floatbuf(dirichleths); q = floatbuf(Qs)
    h = outbuf(K, p.N)
    rc = GC.@preserve K d q h ccall((:dpf_steady_forward, libdpf), Cint,
                                    (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                                    p.ptr, rawptr(K), rawptr(d), rawptr(q), rawptr(h))
    check(p.ptr, rc)
    return h
end

function adjoint(p::Problem, delta)
    dl = floatbuf(delta)
    dKs = outbuf(dl, p.F)
    ddh = outbuf(dl, p.N)
    dQs = outbuf(dl, p.N)
    rc = GC.@preserve dl dKs ddh dQs ccall((:dpf_steady_adjoint, libdpf), Cint,
                                           (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                                           p.ptr, rawptr(dl), rawptr(dKs), rawptr(ddh), rawptr(dQs))
    check(p.ptr, rc)
    return dKs, ddh, dQs
end

"""Selectors for the `linear_solver` keyword: `amg_solver` (CG + AMG to reltol, the default)
and `cholesky_solver` (a banded Cholesky factorisation of the operator on the GPU; a band too
wide for the device falls back to the CG solver run to the FP64 rounding floor)."""
function amg_solver end
function cholesky_solver end

solver_kwargs(ls, kwargs) = ls === cholesky_solver ?
    merge((; max_outer=12), kwargs, (; solver=1, precision=:mixed, reltol=1e-30)) : kwargs

"""Drop-in for `DPFEHM.groundwater_steadystate`."""
function groundwater_steadystate(Ks, neighbors, areasoverlengths, dirichletnodes, dirichleths, Qs;
                                 linear_solver=amg_solver, kwargs...)
    p = Problem(neighbors, areasoverlengths, dirichletnodes, length(Qs); solver_kwargs(linear_solver, values(kwargs))...)
    return forward(p, Ks, dirichleths, Qs)
end

"""Drop-in for `DPFEHM.solvepressure` (src/twophase.jl:48): the steady system with
transmissibility 2 aol K, i.e. the steady solve at conductances 2K."""
solvepressure(Ks, neighbors, areasoverlengths, dirichletnodes, dirichleths, Qs; kwargs...) =
    groundwater_steadystate(2 .* Ks, neighbors, areasoverlengths, dirichletnodes, dirichleths, Qs; kwargs...)

function ChainRulesCore.rrule(::typeof(solvepressure), Ks, neighbors, areasoverlengths, dirichletnodes,
                              dirichleths, Qs; kwargs...)
    h, pb = ChainRulesCore.rrule(groundwater_steadystate, 2 .* Ks, neighbors, areasoverlengths, dirichletnodes,
                                 dirichleths, Qs; kwargs...)
    function pullback(delta)
        t = pb(delta)
        return (t[1], ChainRulesCore.@thunk(2 .* ChainRulesCore.unthunk(t[2])), t[3:end]...)
    end
    return h, pullback
end

function ChainRulesCore.rrule(::typeof(groundwater_steadystate), Ks, neighbors, areasoverlengths, dirichletnodes,
                              dirichleths, Qs; kwargs...)
    p = Problem(neighbors, areasoverlengths, dirichletnodes, length(Qs); kwargs...)
    h = forward(p, Ks, dirichleths, Qs)
    function pullback(delta)
        dKs, ddh, dQs = adjoint(p, delta)     # the closure keeps the GPU handle alive
        return (ChainRulesCore.NoTangent(),
                ChainRulesCore.@thunk(dKs),
                ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent(),
                ChainRulesCore.@thunk(ddh),
                ChainRulesCore.@thunk(dQs))
    end
    return h, pullback
end

"""A face-list handle on the CSR path (the Richards solver needs one)."""
function GeneralProblem(neighbors, areasoverlengths, dirichletnodes, N; volumes=nothing, kwargs...)
    F = length(neighbors)
    a = Int64[p[1] - 1 for p in neighbors]
    b = Int64[p[2] - 1 for p in neighbors]
    aol = Vector{Float64}(areasoverlengths[1:F])
    dn = Int64[d - 1 for d in dirichletnodes]
    vol = volumes === nothing ? Ptr{Float64}(C_NULL) : Vector{Float64}(volumes)
    opts = default_options(; kwargs...)
    out = Ref{Ptr{Cvoid}}(C_NULL)
    rc = ccall((:dpf_create_general, libdpf), Cint,
        (Int64, Int64, Ptr{Int64}, Ptr{Int64}, Ptr{Float64}, Ptr{Float64}, Int64, Ptr{Int64}, Ref{Options},
         Ref{Ptr{Cvoid}}), N, F, a, b, aol, vol, length(dn), dn, opts, out)
    rc == DPF_OK || error("dpf_create_general failed ($rc): $(lasterror(C_NULL))")
    p = Problem(out[], N, F)
    finalizer(p) do q
        q.ptr == C_NULL || ccall((:dpf_destroy, libdpf), Cvoid, (Ptr{Cvoid},), q.ptr)
        q.ptr = C_NULL
    end
    return p
end

function richards_forward(p::Problem, psi0, Ks, dirichletpsis, coords, alphas, Ns, Qs; tol=1e-10, maxiter=200)
    psi = Vector{Float64}(undef, p.N)
    z = Vector{Float64}(coords[3, :])
    rc = ccall((:dpf_richards_steady, libdpf), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
         Cdouble, Cint, Ptr{Float64}), p.ptr, Vector{Float64}(psi0), Vector{Float64}(Ks),
        Vector{Float64}(dirichletpsis), z, Vector{Float64}(alphas), Vector{Float64}(Ns), Vector{Float64}(Qs), tol, maxiter,
        psi)
    check(p.ptr, rc)
    return psi
end

"""Fixed-step backward Euler of S V dpsi/dt = richards_residuals(psi) on a `GeneralProblem`:
psi at the final step and the (N, nsteps) states."""
function richards_transient(p::Problem, psi0, Ks, dirichletpsis, coords, alphas, Ns, Qs, specificstorage, dt, nsteps;
                            tol=1e-10, maxiter=200)
    psiT = Vector{Float64}(undef, p.N)
    states = Matrix{Float64}(undef, p.N, nsteps)
    z = Vector{Float64}(coords[3, :])
    rc = ccall((:dpf_richards_transient_forward, libdpf), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
         Ptr{Float64}, Cdouble, Cint, Cdouble, Cint, Ptr{Float64}, Ptr{Float64}), p.ptr, Vector{Float64}(psi0),
        Vector{Float64}(Ks), Vector{Float64}(dirichletpsis), z, Vector{Float64}(alphas), Vector{Float64}(Ns),
        Vector{Float64}(Qs), Vector{Float64}(specificstorage), dt, nsteps, tol, maxiter, states, psiT)
    check(p.ptr, rc)
    return psiT, states
end

"""Tangents (dKs, ddirichletpsis, dalphas, dNs, dQs, dpsi0) of the last `richards_transient` run for
J = sum_n sum_k w_k psi^n[obs_k]^2 + gT . psi^T (obs 1-based; gT may be `nothing`)."""
function richards_transient_adjoint(p::Problem, obs, w=nothing, gT=nothing; tol=1e-10, maxiter=200)
    o = Int64[k - 1 for k in obs]
    ww = w === nothing ? Ptr{Float64}(C_NULL) : Vector{Float64}(w)
    gg = gT === nothing ? Ptr{Float64}(C_NULL) : Vector{Float64}(gT)
    dKs = Vector{Float64}(undef, p.F); dal = Vector{Float64}(undef, p.F); dN = Vector{Float64}(undef, p.F)
    ddp = Vector{Float64}(undef, p.N); dQs = Vector{Float64}(undef, p.N); d0 = Vector{Float64}(undef, p.N)
    rc = ccall((:dpf_richards_transient_adjoint, libdpf), Cint,
        (Ptr{Cvoid}, Int64, Ptr{Int64}, Ptr{Float64}, Ptr{Float64}, Cdouble, Cint, Ptr{Float64}, Ptr{Float64},
         Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}), p.ptr, length(o), o, ww, gg, tol, maxiter, dKs, ddp,
        dal, dN, dQs, d0)
    check(p.ptr, rc)
    return dKs, ddp, dal, dN, dQs, d0
end

"""Drop-in for `DPFEHM.richards_steadystate` (src/richards.jl:148-167)."""
richards_steadystate(psi0, Ks, neighbors, areasoverlengths, dirichletnodes, dirichletpsis, coords, alphas, Ns, Qs;
                     tol=1e-10, maxiter=200, kwargs...) =
    richards_forward(GeneralProblem(neighbors, areasoverlengths, dirichletnodes, length(Qs); kwargs...), psi0, Ks,
                     dirichletpsis, coords, alphas, Ns, Qs; tol=tol, maxiter=maxiter)

function ChainRulesCore.rrule(::typeof(richards_steadystate), psi0, Ks, neighbors, areasoverlengths, dirichletnodes,
                              dirichletpsis, coords, alphas, Ns, Qs; tol=1e-10, maxiter=200, kwargs...)
    p = GeneralProblem(neighbors, areasoverlengths, dirichletnodes, length(Qs); kwargs...)
    psi = richards_forward(p, psi0, Ks, dirichletpsis, coords, alphas, Ns, Qs; tol=tol, maxiter=maxiter)
    function pullback(delta)
        dKs = Vector{Float64}(undef, p.F); dal = Vector{Float64}(undef, p.F); dN = Vector{Float64}(undef, p.F)
        ddp = Vector{Float64}(undef, p.N); dQs = Vector{Float64}(undef, p.N)
        rc = ccall((:dpf_richards_adjoint, libdpf), Cint,
            (Ptr{Cvoid}, Ptr{Float64}, Cdouble, Cint, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
             Ptr{Float64}), p.ptr, Vector{Float64}(delta), tol, maxiter, dKs, ddp, dal, dN, dQs)
        check(p.ptr, rc)
        return (ChainRulesCore.NoTangent(), ChainRulesCore.@thunk(zeros(length(psi0))), ChainRulesCore.@thunk(dKs),
                ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent(),
                ChainRulesCore.@thunk(ddp), ChainRulesCore.NoTangent(), ChainRulesCore.@thunk(dal),
                ChainRulesCore.@thunk(dN), ChainRulesCore.@thunk(dQs))
    end
    return psi, pullback
end

end # module
