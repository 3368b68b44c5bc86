# KMHodlrGPU: the Julia side of the drop-in.  It binds libkmhodlr.so through `ccall` and adds
# methods for the KernelMatrices.jl HODLR API on a GPU-resident HODLR type.
#
# Covered calls (reference file:line):
#   HODLR.KernelHODLR(K, ep, maxrank, lvl; nystrom)   src/HODLR/src/constructor.jl:6-58
#   HODLR.symmetricfactorize!(K)                      src/HODLR/src/symfact.jl:6-49
#   mul!, *, ldiv!, \, logdet                          src/HODLR/src/baseoverloads.jl:152-263
#   ldiv!(t, K.W, v), ldiv!(t, K.W', v), mul!(t, K.W, v) baseoverloads.jl:95-150
#   HODLR.stoch_gradient, HODLR.negloglik             stochasticgradient.jl:30-44, maxlikfunctions.jl:2-9
#   HODLR.stoch_profile_gradient, profile_negloglik   stochasticgradient.jl:68-86, maxlikfunctions.jl:11-19
#   grad_and_fisher_matrix, stoch_fisher              stochastichessian.jl:91-115,152-181
#   stoch_hessian (profile = false / true)            stochastichessian.jl:15-31, 117-147
#   maxlikdata(...; sortmethod=:KDTree)               constructor.jl:171-181 (own k-d ordering)
#   RKernelHODLR(K, tol, maxrank, lvl), R * v         constructor.jl:130-161, baseoverloads.jl:301-305
#
# Kernels are callable structs, so the same object runs in the reference's CPU path
# (k(x, y, p) like any kernel function) and is recognised by type here.
module KMHodlrGPU

using LinearAlgebra, StaticArrays
import LinearAlgebra: mul!, ldiv!, logdet, adjoint
import KernelMatrices: KernelMatrix
import KernelMatrices.HODLR: HierLevel, FixedLevel, LogLevel, symmetricfactorize!

const libkm = joinpath(@__DIR__, "..", "kmhodlr", "libkmhodlr.so")

# ---- kernels ---------------------------------------------------------------------------------
struct RatQuad end    # p1^2/(1+(r/p2)^2)^2 + p3*(x == y)          (README.md:42-48)
struct Matern32 end   # p1*(1+sqrt3 r/p2)exp(-sqrt3 r/p2) + p3*(x == y)  (mtn_kernfun, nu = 3/2)

function (::RatQuad)(x, y, p)
  out = abs2(p[1]) / abs2(1.0 + abs2(norm(x - y) / p[2]))
  return x == y ? out + p[3] : out
end

function (::Matern32)(x, y, p)
  r = norm(x - y)
  out = p[1]
  if r > 0.0
    z = sqrt(3.0) * r / p[2]
    out = abs(r / p[2]) > 1.0e-8 ? p[1] * (1.0 + z) * exp(-z) : p[1]
  end
  return x == y ? out + p[3] : out
end

kernel_id(::RatQuad) = Cint(0)
kernel_id(::Matern32) = Cint(1)

# ---- library ---------------------------------------------------------------------------------
struct KmConfig
  device::Cint
  precision::Cint
  hbm_budget_fraction::Cdouble
  refine_max_iter::Cint
  refine_tol::Cdouble
end

struct PosDefGPU <: Exception
  msg::String
end

function check(h::Ptr{Cvoid}, rc::Cint)
  rc == 0 && return nothing
  msg = h == C_NULL ? "libkmhodlr error $rc" : unsafe_string(ccall((:km_last_error, libkm), Cstring, (Ptr{Cvoid},), h))
  rc == 2 && throw(PosDefException(-1))   # KM_ERR_NOT_SPD
  error(msg)
end

mutable struct GPUKernelHODLR
  h::Ptr{Cvoid}
  n::Int64
  nys::Bool
  factorized::Bool
end

level_args(l::FixedLevel) = (Cint(0), Int64(l.lv))
level_args(l::LogLevel) = (Cint(1), Int64(l.lv))

function GPUKernelHODLR(K::KernelMatrix, ep::Float64, maxrank::Int64, lvl::HierLevel;
                        nystrom::Bool=false, device::Int=0, precision::Int=0)
  K.x1 == K.x2 || error("This function builds symmetric matrices.")
  pts = Vector{SVector{2,Float64}}(K.x1)          # (x, y) pairs, contiguous
  prm = Vector{Float64}(K.parms)
  cfg = Ref(KmConfig(device, precision, 0.8, 0, 0.0))
  hr = Ref{Ptr{Cvoid}}(C_NULL)
  check(C_NULL, ccall((:km_create, libkm), Cint, (Ptr{KmConfig}, Ptr{Ptr{Cvoid}}), cfg, hr))
  out = GPUKernelHODLR(hr[], length(pts), nystrom, false)
  finalizer(x -> ccall((:km_destroy, libkm), Cint, (Ptr{Cvoid},), x.h), out)
  kind, lv = level_args(lvl)
  check(out.h, ccall((:km_assemble, libkm), Cint,
                     (Ptr{Cvoid}, Ptr{SVector{2,Float64}}, Int64, Cint, Ptr{Float64}, Cint, Cint, Cdouble,
                      Int64, Cint, Int64),
                     out.h, pts, length(pts), kernel_id(K.kernel), prm, length(prm), nystrom ? 1 : 0, ep,
                     maxrank, kind, lv))
  return out
end

function symmetricfactorize!(K::GPUKernelHODLR; plel::Bool=false, verbose::Bool=false)
  check(K.h, ccall((:km_factorize, libkm), Cint, (Ptr{Cvoid},), K.h))
  K.factorized = true
  return nothing
end

# symmetricfactorize!(K) then K \ src in one call (the forward half of the solve overlaps the
# factorisation); the same factor and result as the two calls.
function factorize_solve!(target::StridedVecOrMat{Float64}, K::GPUKernelHODLR, src::StridedVecOrMat{Float64})
  check(K.h, ccall((:km_factorize_solve, libkm), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int64),
                   K.h, src, target, size(src, 2)))
  K.factorized = true
  return target
end

function mul!(target::StridedVecOrMat{Float64}, K::GPUKernelHODLR, src::StridedVecOrMat{Float64})
  check(K.h, ccall((:km_matvec, libkm), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int64),
                   K.h, src, target, size(src, 2)))
  return target
end

function ldiv!(target::StridedVecOrMat{Float64}, K::GPUKernelHODLR, src::StridedVecOrMat{Float64})
  check(K.h, ccall((:km_solve, libkm), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int64),
                   K.h, src, target, size(src, 2)))
  return target
end

Base.:*(K::GPUKernelHODLR, x::VecOrMat{Float64}) = mul!(similar(x), K, x)
Base.:\(K::GPUKernelHODLR, x::VecOrMat{Float64}) = ldiv!(similar(x), K, x)

function logdet(K::GPUKernelHODLR)
  out = Ref{Cdouble}(0.0)
  check(K.h, ccall((:km_logdet, libkm), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), K.h, out))
  return out[]
end

# K.W and K.W' (FactorHODLR products and solves, baseoverloads.jl:95-150)
struct GPUFactor
  K::GPUKernelHODLR
  t::Bool
end
Base.getproperty(K::GPUKernelHODLR, s::Symbol) = s === :W ? GPUFactor(K, false) : getfield(K, s)
adjoint(W::GPUFactor) = GPUFactor(W.K, !W.t)

function ldiv!(target::StridedVecOrMat{Float64}, W::GPUFactor, src::StridedVecOrMat{Float64})
  check(W.K.h, ccall((:km_factor_solve, libkm), Cint, (Ptr{Cvoid}, Cint, Ptr{Float64}, Ptr{Float64}, Int64),
                     W.K.h, W.t, src, target, size(src, 2)))
  return target
end

function mul!(target::StridedVecOrMat{Float64}, W::GPUFactor, src::StridedVecOrMat{Float64})
  check(W.K.h, ccall((:km_factor_mul, libkm), Cint, (Ptr{Cvoid}, Cint, Ptr{Float64}, Ptr{Float64}, Int64),
                     W.K.h, W.t, src, target, size(src, 2)))
  return target
end

# negloglik (maxlikfunctions.jl:2-9) and stoch_gradient (stochasticgradient.jl:30-44): the
# derivative functions are the kernel's own parameter derivatives, so `dfuns` is not needed.
function negloglik(K::GPUKernelHODLR, dat::Vector{Float64})
  nll = Ref{Cdouble}(0.0)
  check(K.h, ccall((:km_nll_grad, libkm), Cint,
                   (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int64, Ptr{Cdouble}, Ptr{Cdouble}),
                   K.h, dat, C_NULL, 0, nll, C_NULL))
  return nll[]
end

function stoch_gradient(K::GPUKernelHODLR, dat::Vector{Float64}, vecs::Vector{Vector{Float64}})
  probes = reduce(hcat, vecs)
  nll = Ref{Cdouble}(0.0)
  grad = zeros(3)
  check(K.h, ccall((:km_nll_grad, libkm), Cint,
                   (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int64, Ptr{Cdouble}, Ptr{Cdouble}),
                   K.h, dat, probes, size(probes, 2), nll, grad))
  return grad
end

# profile_negloglik (maxlikfunctions.jl:11-19) and stoch_profile_gradient
# (stochasticgradient.jl:68-86): the scale parameter profiled out.
function profile_negloglik(K::GPUKernelHODLR, dat::Vector{Float64})
  nll = Ref{Cdouble}(0.0)
  check(K.h, ccall((:km_profile_nll_grad, libkm), Cint,
                   (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int64, Ptr{Cdouble}, Ptr{Cdouble}),
                   K.h, dat, C_NULL, 0, nll, C_NULL))
  return nll[]
end

function stoch_profile_gradient(K::GPUKernelHODLR, dat::Vector{Float64}, vecs::Vector{Vector{Float64}})
  probes = reduce(hcat, vecs)
  nll = Ref{Cdouble}(0.0)
  grad = zeros(3)
  check(K.h, ccall((:km_profile_nll_grad, libkm), Cint,
                   (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int64, Ptr{Cdouble}, Ptr{Cdouble}),
                   K.h, dat, probes, size(probes, 2), nll, grad))
  return grad
end

# grad_and_fisher_matrix (stochastichessian.jl:152-181) / stoch_fisher (:91-115) on a factorised
# GPU HODLR: (nll, gradient, 3 x 3 Fisher matrix) from one set of probes.
function grad_and_fisher(K::GPUKernelHODLR, dat::Vector{Float64}, vecs::Vector{Vector{Float64}})
  probes = reduce(hcat, vecs)
  nll = Ref{Cdouble}(0.0)
  grad = zeros(3)
  fisher = zeros(3, 3)
  check(K.h, ccall((:km_grad_fisher, libkm), Cint,
                   (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int64, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}),
                   K.h, dat, probes, size(probes, 2), nll, grad, fisher))
  return nll[], grad, Symmetric(fisher)
end

# stoch_hessian(K, HK, dat, d1funs, d2funs, vecs; profile) (stochastichessian.jl:117-147,
# shuffle = false) with the built-in kernels' second derivatives: (nll, gradient, 3 x 3 Hessian);
# profile = true takes HODLR_p_hess_slv (:15-31), the Hessian of nlpl_hessian.
function stoch_hessian(K::GPUKernelHODLR, dat::Vector{Float64}, vecs::Vector{Vector{Float64}};
                       profile::Bool=false)
  probes = reduce(hcat, vecs)
  nll = Ref{Cdouble}(0.0)
  grad = zeros(3)
  hess = zeros(3, 3)
  if profile
    check(K.h, ccall((:km_stoch_profile_hessian, libkm), Cint,
                     (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int64, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}),
                     K.h, dat, probes, size(probes, 2), nll, grad, hess))
  else
    check(K.h, ccall((:km_stoch_hessian, libkm), Cint,
                     (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int64, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}),
                     K.h, dat, probes, size(probes, 2), nll, grad, hess))
  end
  return nll[], grad, Symmetric(hess)
end

# maxlikdata(pts=, data=, sortmethod=:KDTree) (constructor.jl:171-181) with the library's own k-d
# ordering computed on the GPU (NearestNeighbors' permutation is not reproduced).
function maxlikdata_gpu(pts::Vector{SVector{2,Float64}}, data::Vector{Float64}; leaf::Int64=32, device::Int=0)
  length(pts) == length(data) || error("points and data disagree in length")
  h = Ref{Ptr{Cvoid}}(C_NULL)
  cfg = Ref(KmConfig(device, Cint(0), 0.8, 0, 0.0))
  check(C_NULL, ccall((:km_create, libkm), Cint, (Ptr{KmConfig}, Ptr{Ptr{Cvoid}}), cfg, h))
  pts_s = similar(pts)
  data_s = similar(data)
  try
    check(h[], ccall((:km_maxlikdata, libkm), Cint,
                     (Ptr{Cvoid}, Ptr{SVector{2,Float64}}, Ptr{Float64}, Int64, Int64,
                      Ptr{SVector{2,Float64}}, Ptr{Float64}, Ptr{Int64}),
                     h[], pts, data, length(pts), leaf, pts_s, data_s, C_NULL))
  finally
    ccall((:km_destroy, libkm), Cint, (Ptr{Cvoid},), h[])
  end
  return pts_s, data_s
end

# RKernelHODLR(K, tol, maxrank, lvl) (constructor.jl:130-161) for K(x1, x2) of any shape, held on
# the GPU; only products, as in the reference (baseoverloads.jl:301-305).
mutable struct GPURKernelHODLR
  r::Ptr{Cvoid}
  n1::Int64
  n2::Int64
end

function GPURKernelHODLR(K::KernelMatrix, tol::Float64, maxrank::Int64=0, lvl::HierLevel=LogLevel(7);
                         device::Int=0)
  kind, lv = lvl isa FixedLevel ? (Cint(0), Int64(lvl.lv)) : (Cint(1), Int64(lvl.lv))
  cfg = Ref(KmConfig(device, Cint(0), 0.8, 0, 0.0))
  prm = Vector{Float64}(collect(K.parms))
  r = Ref{Ptr{Cvoid}}(C_NULL)
  rc = ccall((:km_rhodlr_create, libkm), Cint,
             (Ptr{KmConfig}, Ptr{SVector{2,Float64}}, Int64, Ptr{SVector{2,Float64}}, Int64, Cint, Ptr{Float64},
              Cint, Float64, Int64, Cint, Int64, Ptr{Ptr{Cvoid}}),
             cfg, K.x1, length(K.x1), K.x2, length(K.x2), kernel_id(K.kernel), prm, length(prm), tol, maxrank,
             kind, lv, r)
  rc == 0 || error(unsafe_string(ccall((:km_rhodlr_create_error, libkm), Cstring, ())))
  R = GPURKernelHODLR(r[], length(K.x1), length(K.x2))
  finalizer(x -> ccall((:km_rhodlr_destroy, libkm), Cint, (Ptr{Cvoid},), x.r), R)
  return R
end

function Base.:*(R::GPURKernelHODLR, v::Vector{Float64})
  length(v) == R.n2 || error("dimension mismatch")
  out = Vector{Float64}(undef, R.n1)
  rc = ccall((:km_rhodlr_matvec, libkm), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int64), R.r, v, out, 1)
  rc == 0 || error(unsafe_string(ccall((:km_rhodlr_last_error, libkm), Cstring, (Ptr{Cvoid},), R.r)))
  return out
end

# ---- batched form: nll_objective over many independent datasets ------------------------------
struct KmProblem
  n::Int64
  pts::Ptr{SVector{2,Float64}}
  y::Ptr{Float64}
  params::NTuple{3,Float64}
end

struct KmBatchOpts
  kernel_id::Cint
  rank::Int64
  level_kind::Cint
  level::Int64
  nprobe::Int64
  probe_seed::UInt64
  profile::Cint
end

# One call for many (points, data, parameters) triples; returns (nll, grad (3 x m), status).
# Probes are drawn on the device (problem b uses seed + b).
function batch_nll_grad(pts::Vector{Vector{SVector{2,Float64}}}, dat::Vector{Vector{Float64}},
                        prms::Vector{NTuple{3,Float64}}, kernel, rank::Int64, lvl::HierLevel;
                        nprobe::Int64=72, seed::UInt64=UInt64(0), nworkers::Int=8, precision::Int=0,
                        profile::Bool=false)
  m = length(pts)
  b = Ref{Ptr{Cvoid}}(C_NULL)
  cfg = Ref(KmConfig(0, Cint(precision), 0.8, 0, 0.0))
  check(C_NULL, ccall((:km_batch_create, libkm), Cint, (Ptr{KmConfig}, Cint, Ptr{Ptr{Cvoid}}), cfg, nworkers, b))
  kind, lv = lvl isa HODLR.FixedLevel ? (Cint(0), Int64(lvl.lv)) : (Cint(1), Int64(lvl.lv))
  opts = Ref(KmBatchOpts(kernel_id(kernel), rank, kind, lv, nprobe, seed, Cint(profile)))
  probs = [KmProblem(length(pts[i]), pointer(pts[i]), pointer(dat[i]), prms[i]) for i in 1:m]
  nll = zeros(m); grad = zeros(3, m); status = zeros(Cint, m)
  GC.@preserve pts dat begin
    rc = ccall((:km_batch_nll_grad, libkm), Cint,
               (Ptr{Cvoid}, Ptr{KmBatchOpts}, Int64, Ptr{KmProblem}, Ptr{Float64}, Ptr{Float64}, Ptr{Cint}),
               b[], opts, m, probs, nll, grad, status)
  end
  ccall((:km_batch_destroy, libkm), Cint, (Ptr{Cvoid},), b[])
  return nll, grad, status
end

end # module
