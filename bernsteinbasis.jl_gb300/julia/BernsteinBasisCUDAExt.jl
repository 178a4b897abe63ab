# BernsteinBasisCUDAExt: GPU methods for BernsteinBasis.jl's operator types.
#
# A package extension (loaded when CUDA.jl is loaded next to BernsteinBasis) that sends
# `mul!` on CuArrays, and the wave/Maxwell right-hand side and LSRK time stepping, to
# libbbdg.so through its C ABI (include/bbdg.h). The reference's CPU methods stay as they
# are; only device arrays take these methods.
#
#   mul!(out, D::BernsteinDerivativeMatrix_3D_{r,s,t}, x)  -> bb_deriv_apply
#       (src/BernsteinDerivativeMatrix_3D.jl:134,176,218,222-231)
#   mul!(out, L::BernsteinLift, x)                          -> bb_lift_apply
#       (src/BernsteinLift.jl:191-220,264-269)
#   bernstein_rhs!(du, q, solver)                           -> bb_rhs
#       (examples/3d_wave.jl:36-84, examples/3d_maxwell.jl:36-93)
#   lsrk_run!(q, res, solver, dt, nsteps)                   -> bb_lsrk_run
module BernsteinBasisCUDAExt

using BernsteinBasis
using CUDA
using LinearAlgebra
using StaticArrays

const libbbdg = get(ENV, "BBDG_LIB", joinpath(@__DIR__, "..", "_build", "libbbdg.so"))

const BB_F32 = Cint(0)
const BB_F64 = Cint(1)
const BB_WAVE = Cint(0)
const BB_MAXWELL = Cint(1)
const BB_ADVECTION = Cint(2)   # examples/3d_advec_scalar.jl
const BB_ADVECTION3 = Cint(3)  # examples/3d_advec.jl (u, v, w)

dtype_code(::Type{Float32}) = BB_F32
dtype_code(::Type{Float64}) = BB_F64

# one bb_ctx per device, created on first use
const CONTEXTS = Dict{Int,Ptr{Cvoid}}()
function context()
    dev = CUDA.deviceid(CUDA.device())
    get!(CONTEXTS, dev) do
        r = Ref{Ptr{Cvoid}}(C_NULL)
        rc = ccall((:bb_ctx_create, libbbdg), Cint, (Cint, Ptr{Ptr{Cvoid}}), dev, r)
        rc == 0 || error("bb_ctx_create failed with status $rc")
        r[]
    end
end

function check(rc::Cint)
    rc == 0 && return nothing
    msg = unsafe_string(ccall((:bb_ctx_last_error, libbbdg), Cstring, (Ptr{Cvoid},), context()))
    error("libbbdg status $rc: $msg")
end

stream_handle() = CUDA.stream().handle

axis(::BernsteinDerivativeMatrix_3D_r) = Cint(0)
axis(::BernsteinDerivativeMatrix_3D_s) = Cint(1)
axis(::BernsteinDerivativeMatrix_3D_t) = Cint(2)
const DerivOp = Union{BernsteinDerivativeMatrix_3D_r,BernsteinDerivativeMatrix_3D_s,
                      BernsteinDerivativeMatrix_3D_t}

# Matrix form: one column per element (Np x K), exactly the reference's layout.
function LinearAlgebra.mul!(out::CuMatrix{T}, D::DerivOp, x::CuMatrix{T}) where {T<:Union{Float32,Float64}}
    size(out) == size(x) || throw(DimensionMismatch("out and x must have the same size"))
    check(ccall((:bb_deriv_apply, libbbdg), Cint,
                (Ptr{Cvoid}, Cint, Cint, Int64, Cint, CuPtr{T}, CuPtr{T}, Ptr{Cvoid}),
                context(), axis(D), D.N, size(x, 2), dtype_code(T), x, out, stream_handle()))
    return out
end

function LinearAlgebra.mul!(out::CuMatrix{T}, L::BernsteinLift, x::CuMatrix{T}) where {T<:Union{Float32,Float64}}
    size(out, 2) == size(x, 2) || throw(DimensionMismatch("column counts differ"))
    check(ccall((:bb_lift_apply, libbbdg), Cint,
                (Ptr{Cvoid}, Cint, Int64, Cint, CuPtr{T}, CuPtr{T}, Ptr{Cvoid}),
                context(), L.N, size(x, 2), dtype_code(T), x, out, stream_handle()))
    return out
end

# Vector form (one element) goes through the matrix form.
LinearAlgebra.mul!(out::CuVector{T}, D::DerivOp, x::CuVector{T}) where {T<:Union{Float32,Float64}} =
    (mul!(reshape(out, :, 1), D, reshape(x, :, 1)); out)
LinearAlgebra.mul!(out::CuVector{T}, L::BernsteinLift, x::CuVector{T}) where {T<:Union{Float32,Float64}} =
    (mul!(reshape(out, :, 1), L, reshape(x, :, 1)); out)

# Per-element views of device arrays would mean one launch per element: refuse them.
LinearAlgebra.mul!(::SubArray{<:Any,1,<:CuArray}, ::Union{DerivOp,BernsteinLift}, ::AbstractVector) =
    error("apply BernsteinBasis operators to whole Np x K CuMatrix columns, not per-element views")

# ---- solver --------------------------------------------------------------------------
# conn: K*4 Int32 (nbr << 5 | nbr_face << 3 | orientation); geo: K*24 values (rxJ..tzJ,
# 1/J, J, pad, nxJ[4], nyJ[4], nzJ[4]); both on the device and alive as long as the solver.
mutable struct BBSolver{T}
    handle::Ptr{Cvoid}
    nf::Int
    conn::CuVector{Int32}
    geo::CuVector{T}
end

function BBSolver(physics::Symbol, N::Integer, conn::CuVector{Int32}, geo::CuVector{T};
                  tau::Real = 1.0) where {T<:Union{Float32,Float64}}
    code = physics === :wave ? BB_WAVE : physics === :maxwell ? BB_MAXWELL :
           physics === :advection ? BB_ADVECTION : physics === :advection3 ? BB_ADVECTION3 :
           throw(ArgumentError("physics must be :wave, :maxwell, :advection or :advection3"))
    r = Ref{Ptr{Cvoid}}(C_NULL)
    K = length(conn) ÷ 4
    check(ccall((:bb_solver_create, libbbdg), Cint,
                (Ptr{Cvoid}, Cint, Cint, Int64, Cint, CuPtr{Int32}, CuPtr{T}, Cdouble, Ptr{Ptr{Cvoid}}),
                context(), code, N, K, dtype_code(T), conn, geo, tau, r))
    s = BBSolver{T}(r[], physics === :wave ? 4 : physics === :maxwell ? 6 : 1, conn, geo)
    finalizer(s -> ccall((:bb_solver_destroy, libbbdg), Cint, (Ptr{Cvoid},), s.handle), s)
    return s
end

# State as an (Np, K, nf) CuArray: field m is q[:, :, m], the reference's Np x K matrix of
# that component; in memory this is the library's [nf][K][Np] layout.
function bernstein_rhs!(du::CuArray{T,3}, q::CuArray{T,3}, s::BBSolver{T}) where {T}
    check(ccall((:bb_rhs, libbbdg), Cint, (Ptr{Cvoid}, CuPtr{T}, CuPtr{T}, Ptr{Cvoid}),
                s.handle, q, du, stream_handle()))
    return du
end

# OrdinaryDiffEq interop: the examples' `rhs_matvec!(du, u, params, t)` signature with the
# solver as `params`, so any integrator drives the GPU right-hand side on a CuArray state:
#     prob = ODEProblem(gpu_rhs!, to_device_state(modal_u0), tspan, s)
#     sol  = solve(prob, Tsit5(), dt = 0.01)          # examples/3d_wave.jl:133-134
# (The solver's own fused LSRK45 loop, `lsrk_run!`, avoids the integrator's extra passes.)
gpu_rhs!(du::CuArray{T,3}, u::CuArray{T,3}, s::BBSolver{T}, t) where {T} =
    (bernstein_rhs!(du, u, s); nothing)

function lsrk_run!(q::CuArray{T,3}, res::CuArray{T,3}, s::BBSolver{T}, dt::Real, nsteps::Integer;
                   graph::Bool = true) where {T}
    check(ccall((:bb_lsrk_run, libbbdg), Cint,
                (Ptr{Cvoid}, Cdouble, Cint, CuPtr{T}, CuPtr{T}, Cint, Ptr{Cvoid}),
                s.handle, dt, nsteps, q, res, graph, stream_handle()))
    return q
end

# AoS Matrix{SVector{nf,T}} (the examples' state) <-> the device SoA layout, once at upload.
to_device_state(q::AbstractMatrix{<:AbstractVector{T}}) where {T} =
    CuArray(permutedims(reshape(reinterpret(T, q), :, size(q)...), (2, 3, 1)))
from_device_state(q::CuArray{T,3}, ::Val{nf}) where {T,nf} =
    map(v -> SVector{nf,T}(v), eachslice(permutedims(Array(q), (3, 1, 2)); dims = (2, 3)))

export bernstein_rhs!, gpu_rhs!, lsrk_run!, BBSolver, to_device_state, from_device_state

end # module
