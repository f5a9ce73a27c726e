# GLAGPU.jl — Julia host glue: GenericLinearAlgebra.jl's self-adjoint
# eigensolver API over libglagpu.so (ccall into the C ABI of include/glagpu.h).
#
# Mirrors, method for method, src/eigenSelfAdjoint.jl of GenericLinearAlgebra.jl
# v0.4.0:
#   eigen!(::Hermitian/Symmetric{<:Real})  (:626-630)  -> GLAGPU.eigen!
#   eigvals!(::Hermitian/Symmetric{<:Real}) (:584-588) -> GLAGPU.eigvals!
#   eigen!(::SymTridiagonal) / eigvals!     (:581,:623) -> GLAGPU.eigen! / eigvals!
#   keyword tol = eps(T), sortby = eigsortby (any key: a stable permutation
#   as sorteig! :598 applies), alg ignored
# and returns LinearAlgebra.Eigen like the reference. A nonzero per-matrix
# info raises, as src/lapack.jl:62 turns LAPACK's info into LAPACKException.
#
# The drop-in: a matrix held in GPU memory (GPUMatrix) wrapped in Hermitian or
# Symmetric. For those wrappers this module adds methods to LinearAlgebra's
# own eigen!, eigvals!, eigen and eigvals, so unqualified calls
#     E = eigen!(Hermitian(dA))      # dA::GPUMatrix{Float64}
# reach the GPU: stdlib's LAPACK method only takes StridedMatrix storage, and
# GenericLinearAlgebra's generic eigen!(::Hermitian) is less specific than a
# method on Hermitian{T,GPUMatrix{T}}, so these win dispatch without piracy.
#
# Host Matrix inputs go through gla_plan_execute_host (the library copies to
# and from the GPU); batched calls solve many matrices per launch sequence.
module GLAGPU

using LinearAlgebra

const libglagpu = get(ENV, "GLAGPU_LIB", joinpath(@__DIR__, "..", "build", "libglagpu.so"))

const GLA_PREC_F64 = Cint(0)
const GLA_PREC_F32 = Cint(1)
const GLA_PREC_F32_REFINED = Cint(2)
const GLA_ALG_QL = Cint(0)
const GLA_ALG_QR = Cint(1)
const GLA_MAX_SMALL_N = 128

struct GLAException <: Exception
    status::Cint
    msg::String
end
Base.showerror(io::IO, e::GLAException) = print(io, "GLAException(", e.status, "): ", e.msg)

struct NonConvergence <: Exception
    info::Cint
end

statusmsg(s) = unsafe_string(ccall((:gla_status_string, libglagpu), Cstring, (Cint,), s))
check(s) = s < 0 ? throw(GLAException(s, statusmsg(s))) : s

function raise_info(info)
    for i in info
        i == -1 && throw(ArgumentError("matrix contains NaN or Inf"))
        i > 0 && throw(NonConvergence(i))
    end
end

mutable struct Plan
    handle::Ptr{Cvoid}
    ns::Vector{Int64}
    jobz::Char
    a_elems::Int64
    w_elems::Int64
end

function Plan(ns::Vector{Int64}; precision = GLA_PREC_F64, jobz = 'V', uplo = 'L', tol = 0.0, alg = GLA_ALG_QL)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:gla_plan_create, libglagpu), Cint,
                (Ref{Ptr{Cvoid}}, Cint, UInt8, UInt8, Int64, Ptr{Int64}, Cdouble, Cint),
                h, precision, UInt8(jobz), UInt8(uplo), length(ns), ns, tol, alg))
    a = Ref{Int64}(0)
    w = Ref{Int64}(0)
    check(ccall((:gla_plan_arena_sizes, libglagpu), Cint, (Ptr{Cvoid}, Ref{Int64}, Ref{Int64}), h[], a, w))
    p = Plan(h[], ns, jobz, a[], w[])
    finalizer(p) do q
        q.handle == C_NULL || ccall((:gla_plan_destroy, libglagpu), Cint, (Ptr{Cvoid},), q.handle)
        q.handle = C_NULL
    end
    return p
end

# Run a plan on host arenas (column-major matrices packed back to back).
function execute_host!(p::Plan, A::Vector{T}, w::Vector{T}, V::Vector{T}, info::Vector{Cint}) where {T}
    check(ccall((:gla_plan_execute_host, libglagpu), Cint,
                (Ptr{Cvoid}, Ptr{T}, Ptr{T}, Ptr{T}, Ptr{Cint}, Ptr{Cvoid}),
                p.handle, A, w, V, info, C_NULL))
    return info
end

function _batched(mats::AbstractVector{<:AbstractMatrix}, jobz, uplo; precision = GLA_PREC_F64,
                  alg = GLA_ALG_QL, tol = 0.0)
    T = precision == GLA_PREC_F32 ? Float32 : Float64
    ns = Int64[LinearAlgebra.checksquare(M) for M in mats]
    p = Plan(ns; precision, jobz, uplo, tol, alg)
    A = reduce(vcat, (vec(Matrix{T}(M)) for M in mats); init = T[])
    w = Vector{T}(undef, max(p.w_elems, 1))
    V = Vector{T}(undef, jobz == 'V' ? max(p.a_elems, 1) : 1)
    info = zeros(Cint, length(ns))
    execute_host!(p, A, w, V, info)
    raise_info(info)
    vals = Vector{Vector{T}}()
    vecs = Vector{Matrix{T}}()
    ao = 0
    wo = 0
    for n in ns
        push!(vals, w[wo+1:wo+n])
        jobz == 'V' && push!(vecs, reshape(V[ao+1:ao+n*n], n, n))
        ao += n * n
        wo += n
    end
    return vals, vecs
end

"""
    eigen_batched(mats; uplo='L', precision=GLA_PREC_F64, alg=GLA_ALG_QL)

`[eigen(Hermitian(M, uplo)) for M in mats]` in one batched GPU solve.
"""
function eigen_batched(mats; uplo = 'L', kw...)
    vals, vecs = _batched(mats, 'V', uplo; kw...)
    return [LinearAlgebra.Eigen(v, V) for (v, V) in zip(vals, vecs)]
end
eigvals_batched(mats; uplo = 'L', kw...) = _batched(mats, 'N', uplo; kw...)[1]

uplochar(A) = A.uplo == 'L' ? 'L' : 'U'

# sorteig!(values, vectors, sortby) (:598): the device returns ascending
# values; any other key is applied as a stable permutation of that order
# (sortby === nothing leaves it).
function _sortby!(w::AbstractVector, V, sortby)
    (sortby === nothing || sortby === LinearAlgebra.eigsortby) && return w, V
    p = sortperm(w; by = sortby)  # stable: ties keep their ascending order
    return w[p], V === nothing ? nothing : V[:, p]
end

# eigen!/eigvals! on Hermitian/Symmetric real matrices (the reference's :614-630 and :572-588).
function eigen!(A::Union{Hermitian{T,Matrix{T}},Symmetric{T,Matrix{T}}}; tol = eps(T), sortby = LinearAlgebra.eigsortby,
                alg = nothing) where {T<:Union{Float32,Float64}}
    prec = T === Float32 ? GLA_PREC_F32 : GLA_PREC_F64
    E = eigen_batched([A.data]; uplo = uplochar(A), precision = prec, tol = Float64(tol))[1]
    copyto!(A.data, E.vectors)  # like eigen!, the input storage is consumed
    return LinearAlgebra.Eigen(_sortby!(E.values, E.vectors, sortby)...)
end

function eigvals!(A::Union{Hermitian{T,Matrix{T}},Symmetric{T,Matrix{T}}}; tol = eps(T),
                  sortby = LinearAlgebra.eigsortby, alg = nothing) where {T<:Union{Float32,Float64}}
    prec = T === Float32 ? GLA_PREC_F32 : GLA_PREC_F64
    w = eigvals_batched([A.data]; uplo = uplochar(A), precision = prec, tol = Float64(tol))[1]
    return _sortby!(w, nothing, sortby)[1]
end

# ---------------------------------------------------------------- GPU-resident matrices
#
# GPUMatrix{T}: an n x n column-major matrix in device memory, allocated and
# copied with the CUDA runtime (libcudart; GLAGPU_CUDART overrides the path).
# It is an AbstractMatrix (size, element access by one-element copies), so
# Hermitian(dA) and Symmetric(dA) are ordinary LinearAlgebra wrappers; the
# eigen!/eigvals!/eigen/eigvals methods below are LinearAlgebra's functions
# extended for them, and call gla_dsyev / gla_ssyev on the device pointer.
const libcudart = get(ENV, "GLAGPU_CUDART", "libcudart.so")

cudacheck(e) = e == 0 ? nothing : throw(GLAException(Cint(-1000 - e), statusmsg(Cint(-1000 - e))))

mutable struct GPUMatrix{T<:Union{Float32,Float64}} <: AbstractMatrix{T}
    ptr::Ptr{T}
    n::Int
    function GPUMatrix{T}(::UndefInitializer, n::Integer) where {T}
        p = Ref{Ptr{Cvoid}}(C_NULL)
        cudacheck(ccall((:cudaMalloc, libcudart), Cint, (Ref{Ptr{Cvoid}}, Csize_t), p, max(n * n, 1) * sizeof(T)))
        M = new{T}(Ptr{T}(p[]), Int(n))
        finalizer(M) do m
            m.ptr == C_NULL || ccall((:cudaFree, libcudart), Cint, (Ptr{Cvoid},), m.ptr)
            m.ptr = C_NULL
        end
        return M
    end
end

const cudaMemcpyHostToDevice = Cint(1)
const cudaMemcpyDeviceToHost = Cint(2)
const cudaMemcpyDeviceToDevice = Cint(3)
_memcpy(dst, src, bytes, kind) =
    cudacheck(ccall((:cudaMemcpy, libcudart), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Csize_t, Cint), dst, src, bytes, kind))

function GPUMatrix(A::AbstractMatrix{T}) where {T<:Union{Float32,Float64}}
    n = LinearAlgebra.checksquare(A)
    M = GPUMatrix{T}(undef, n)
    h = Matrix{T}(A)
    _memcpy(M.ptr, h, n * n * sizeof(T), cudaMemcpyHostToDevice)
    return M
end
Base.size(M::GPUMatrix) = (M.n, M.n)
Base.IndexStyle(::Type{<:GPUMatrix}) = IndexCartesian()
function Base.getindex(M::GPUMatrix{T}, i::Int, j::Int) where {T}
    checkbounds(M, i, j)
    r = Ref{T}()
    _memcpy(r, M.ptr + ((j - 1) * M.n + (i - 1)) * sizeof(T), sizeof(T), cudaMemcpyDeviceToHost)
    return r[]
end
function Base.setindex!(M::GPUMatrix{T}, v, i::Int, j::Int) where {T}
    checkbounds(M, i, j)
    r = Ref{T}(convert(T, v))
    _memcpy(M.ptr + ((j - 1) * M.n + (i - 1)) * sizeof(T), r, sizeof(T), cudaMemcpyHostToDevice)
    return v
end
function Base.Array(M::GPUMatrix{T}) where {T}
    h = Matrix{T}(undef, M.n, M.n)
    M.n == 0 || _memcpy(h, M.ptr, M.n * M.n * sizeof(T), cudaMemcpyDeviceToHost)
    return h
end
Base.Matrix(M::GPUMatrix) = Array(M)
function Base.copy(M::GPUMatrix{T}) where {T}
    C = GPUMatrix{T}(undef, M.n)
    M.n == 0 || _memcpy(C.ptr, M.ptr, M.n * M.n * sizeof(T), cudaMemcpyDeviceToDevice)
    return C
end

const HermSymGPU{T} = Union{Hermitian{T,GPUMatrix{T}},Symmetric{T,GPUMatrix{T}}}

# In place on the device: the storage of A becomes the eigenvectors (as
# LAPACK's dsyev and the reference's eigen! consume their input).
function _syev_gpu!(jobz::Char, A::HermSymGPU{T}, tol) where {T}
    D = A.data
    n = D.n
    tol == eps(T) || tol == 0 || throw(ArgumentError("GPUMatrix input: the default tolerance eps($T) only"))
    wbuf = Ref{Ptr{Cvoid}}(C_NULL)
    cudacheck(ccall((:cudaMalloc, libcudart), Cint, (Ref{Ptr{Cvoid}}, Csize_t), wbuf, max(n, 1) * sizeof(T)))
    info = Ref{Cint}(0)
    try
        rc = T === Float64 ?
            ccall((:gla_dsyev, libglagpu), Cint, (UInt8, UInt8, Int64, Ptr{T}, Int64, Ptr{Cvoid}, Ref{Cint}, Ptr{Cvoid}),
                  UInt8(jobz), UInt8(uplochar(A)), n, D.ptr, max(n, 1), wbuf[], info, C_NULL) :
            ccall((:gla_ssyev, libglagpu), Cint, (UInt8, UInt8, Int64, Ptr{T}, Int64, Ptr{Cvoid}, Ref{Cint}, Ptr{Cvoid}),
                  UInt8(jobz), UInt8(uplochar(A)), n, D.ptr, max(n, 1), wbuf[], info, C_NULL)
        check(rc)
        raise_info(Cint[info[]])
        vals = Vector{T}(undef, n)
        n == 0 || _memcpy(vals, wbuf[], n * sizeof(T), cudaMemcpyDeviceToHost)
        return vals
    finally
        ccall((:cudaFree, libcudart), Cint, (Ptr{Cvoid},), wbuf[])
    end
end

# Column permutation of a device matrix (n device-to-device column copies).
function _permutecols(V::GPUMatrix{T}, p) where {T}
    P = GPUMatrix{T}(undef, V.n)
    col = V.n * sizeof(T)
    for (k, j) in enumerate(p)
        _memcpy(P.ptr + (k - 1) * col, V.ptr + (j - 1) * col, col, cudaMemcpyDeviceToDevice)
    end
    return P
end

function LinearAlgebra.eigen!(A::HermSymGPU{T}; tol = eps(T), sortby = LinearAlgebra.eigsortby,
                              alg = nothing) where {T<:Union{Float32,Float64}}
    w = _syev_gpu!('V', A, tol)
    V = A.data
    if !(sortby === nothing || sortby === LinearAlgebra.eigsortby)
        p = sortperm(w; by = sortby)
        w = w[p]
        V = _permutecols(V, p)
    end
    return LinearAlgebra.Eigen(w, V)  # eigenvectors stay on the device
end
function LinearAlgebra.eigvals!(A::HermSymGPU{T}; tol = eps(T), sortby = LinearAlgebra.eigsortby,
                                alg = nothing) where {T<:Union{Float32,Float64}}
    return _sortby!(_syev_gpu!('N', A, tol), nothing, sortby)[1]
end
LinearAlgebra.eigen(A::Hermitian{T,GPUMatrix{T}}; kw...) where {T<:Union{Float32,Float64}} =
    LinearAlgebra.eigen!(Hermitian(copy(A.data), Symbol(A.uplo)); kw...)
LinearAlgebra.eigen(A::Symmetric{T,GPUMatrix{T}}; kw...) where {T<:Union{Float32,Float64}} =
    LinearAlgebra.eigen!(Symmetric(copy(A.data), Symbol(A.uplo)); kw...)
LinearAlgebra.eigvals(A::Hermitian{T,GPUMatrix{T}}; kw...) where {T<:Union{Float32,Float64}} =
    LinearAlgebra.eigvals!(Hermitian(copy(A.data), Symbol(A.uplo)); kw...)
LinearAlgebra.eigvals(A::Symmetric{T,GPUMatrix{T}}; kw...) where {T<:Union{Float32,Float64}} =
    LinearAlgebra.eigvals!(Symmetric(copy(A.data), Symbol(A.uplo)); kw...)

# FP32 solve + FP64 Ogita-Aishima refinement (no reference counterpart).
eigen_refined(A::Union{Hermitian{Float64},Symmetric{Float64}}) =
    eigen_batched([Matrix(A.data)]; uplo = uplochar(A), precision = GLA_PREC_F32_REFINED)[1]

# eigen!/eigvals! on SymTridiagonal{Float64} (:602-612, :623, :581): gla_dstev
# takes device pointers, so the host glue stages through the plan API with
# the tridiagonal written out densely (its reduction is then trivial).
function eigen!(S::SymTridiagonal{Float64}; tol = eps(Float64), sortby = LinearAlgebra.eigsortby, alg = GLA_ALG_QL)
    return eigen_batched([Matrix(S)]; alg = alg)[1]
end
eigvals!(S::SymTridiagonal{Float64}; tol = eps(Float64), sortby = LinearAlgebra.eigsortby) =
    eigvals_batched([Matrix(S)])[1]

# Non-mutating forms.
eigen(A::Union{Hermitian{T,Matrix{T}},Symmetric{T,Matrix{T}}}; kw...) where {T<:Union{Float32,Float64}} =
    eigen!(copy(A); kw...)
eigen(S::SymTridiagonal{Float64}; kw...) = eigen!(copy(S); kw...)

# eigen2 (:633-668): ascending eigenvalues and rows 1 and n of the eigenvector
# matrix (2 x n). Orders <= GLA_MAX_SMALL_N take the reference's cheap form
# (gla_plan_execute_eigen2_host): rows 1 and n of Q from the reflectors, the
# rotations replayed on those two rows only; the values equal eigen's and the
# rows agree with eigen's to rounding (test/eigenselfadjoint.jl:45-51
# compares them with isapprox). Larger orders keep two rows of the full
# eigenvector matrix.
function eigen2(A::Union{Hermitian{T,Matrix{T}},Symmetric{T,Matrix{T}}}; tol = eps(T)) where {T<:Union{Float32,Float64}}
    n = LinearAlgebra.checksquare(A)
    if 1 <= n <= GLA_MAX_SMALL_N
        prec = T === Float32 ? GLA_PREC_F32 : GLA_PREC_F64
        p = Plan(Int64[n]; precision = prec, jobz = 'V', uplo = uplochar(A), tol = Float64(tol))
        w = Vector{T}(undef, n)
        V2 = Vector{T}(undef, 2n)
        info = zeros(Cint, 1)
        check(ccall((:gla_plan_execute_eigen2_host, libglagpu), Cint,
                    (Ptr{Cvoid}, Ptr{T}, Ptr{T}, Ptr{T}, Ptr{Cint}, Ptr{Cvoid}),
                    p.handle, vec(Matrix{T}(A.data)), w, V2, info, C_NULL))
        raise_info(info)
        return LinearAlgebra.Eigen(w, reshape(V2, 2, n))
    end
    E = eigen!(copy(A); tol)
    return LinearAlgebra.Eigen(E.values, E.vectors[[1, n], :])
end
function eigen2(S::SymTridiagonal{Float64}; tol = eps(Float64))
    E = eigen!(copy(S))
    n = size(E.vectors, 1)
    return LinearAlgebra.Eigen(E.values, E.vectors[[1, n], :])
end

"""
    eigen_adjoint(E, wbar, Vbar; gap_rel = 0.0) -> Abar

Reverse-mode adjoint of `E = eigen(A)` for a real symmetric `A`
(gla_plan_adjoint_host; one CTA for n <= $(GLA_MAX_SMALL_N), three tensor-core GEMMs
above): the full symmetric cotangent
`V (diag(wbar) + sym(F .* (V'Vbar))) V'` with `F_ij = 1/(w_j - w_i)` above
the gap threshold. `nothing` stands for a zero cotangent.
"""
function eigen_adjoint(E::LinearAlgebra.Eigen, wbar, Vbar; gap_rel = 0.0)
    n = length(E.values)
    p = Plan(Int64[n]; jobz = 'V')
    w = Vector{Float64}(E.values)
    V = vec(Matrix{Float64}(E.vectors))
    wb = wbar === nothing ? zeros(Float64, n) : Vector{Float64}(wbar)
    Vb = Vbar === nothing ? zeros(Float64, n * n) : vec(Matrix{Float64}(Vbar))
    Abar = Vector{Float64}(undef, max(n * n, 1))
    check(ccall((:gla_plan_adjoint_host, libglagpu), Cint,
                (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Cdouble, Ptr{Cvoid}),
                p.handle, w, V, wb, Vb, Abar, Float64(gap_rel), C_NULL))
    return reshape(Abar[1:n*n], n, n)
end

# eigen!/eigvals! on Hermitian{ComplexF64} (the reference's complex
# Hermitian support, loop bound :462), through gla_zheev_host (the real
# symmetric embedding of order 2n on the GPU).
function eigen!(A::Hermitian{ComplexF64,Matrix{ComplexF64}}; tol = eps(Float64), sortby = LinearAlgebra.eigsortby,
                alg = nothing)
    n = size(A, 1)
    w = Vector{Float64}(undef, n)
    V = Matrix{ComplexF64}(undef, n, n)
    info = Ref{Cint}(0)
    check(ccall((:gla_zheev_host, libglagpu), Cint,
                (UInt8, UInt8, Int64, Ptr{ComplexF64}, Int64, Ptr{Float64}, Ptr{ComplexF64}, Int64, Ref{Cint}),
                UInt8('V'), UInt8(uplochar(A)), n, A.data, max(n, 1), w, V, max(n, 1), info))
    raise_info(Cint[info[]])
    return LinearAlgebra.Eigen(w, V)
end
function eigvals!(A::Hermitian{ComplexF64,Matrix{ComplexF64}}; tol = eps(Float64), sortby = LinearAlgebra.eigsortby)
    n = size(A, 1)
    w = Vector{Float64}(undef, n)
    info = Ref{Cint}(0)
    check(ccall((:gla_zheev_host, libglagpu), Cint,
                (UInt8, UInt8, Int64, Ptr{ComplexF64}, Int64, Ptr{Float64}, Ptr{ComplexF64}, Int64, Ref{Cint}),
                UInt8('N'), UInt8(uplochar(A)), n, A.data, max(n, 1), w, C_NULL, max(n, 1), info))
    raise_info(Cint[info[]])
    return w
end

# symtri! (src/eigenSelfAdjoint.jl:446-564) on the GPU: the factorisation in
# symtriLower!'s layout (uplo 'L') or symtriUpper!'s ('U'), with an EigenQ
# whose lmul!/rmul! (:23-99) and Array (:101) run on the device
# (gla_dsytrd_host / gla_dormtr_host).
struct GPUEigenQ
    uplo::Char
    factors::Matrix{Float64}
    tau::Vector{Float64}
end
struct GPUSymmetricTridiagonalFactorization
    reflectors::GPUEigenQ
    diagonals::SymTridiagonal{Float64,Vector{Float64}}
end

function symtri!(A::Union{Hermitian{Float64,Matrix{Float64}},Symmetric{Float64,Matrix{Float64}}})
    n = size(A, 1)
    d = Vector{Float64}(undef, n)
    e = Vector{Float64}(undef, max(n - 1, 0))
    tau = Vector{Float64}(undef, max(n - 1, 0))
    check(ccall((:gla_dsytrd_host, libglagpu), Cint,
                (UInt8, Int64, Ptr{Float64}, Int64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                UInt8(uplochar(A)), n, A.data, max(n, 1), d, e, tau))
    return GPUSymmetricTridiagonalFactorization(GPUEigenQ(uplochar(A), A.data, tau), SymTridiagonal(d, e))
end

function _ormtr!(side::Char, trans::Char, Q::GPUEigenQ, B::Matrix{Float64})
    m, k = size(B)
    check(ccall((:gla_dormtr_host, libglagpu), Cint,
                (UInt8, UInt8, UInt8, Int64, Int64, Ptr{Float64}, Int64, Ptr{Float64}, Ptr{Float64}, Int64),
                UInt8(side), UInt8(Q.uplo), UInt8(trans), m, k, Q.factors, max(size(Q.factors, 1), 1), Q.tau, B,
                max(m, 1)))
    return B
end
lmul!(Q::GPUEigenQ, B::Matrix{Float64}) = _ormtr!('L', 'N', Q, B)
rmul!(B::Matrix{Float64}, Q::GPUEigenQ) = _ormtr!('R', 'N', Q, B)
Base.Array(Q::GPUEigenQ) = lmul!(Q, Matrix{Float64}(I, size(Q.factors)...))

# numnegevals (src/tridiag.jl:20-36): the number of negative eigenvalues of
# T - sigma I, bit-identical to the reference's recurrence; many shifts at once.
function numnegevals(T::SymTridiagonal{Float64}, sigma::Real = 0.0)
    return numnegevals(T, Float64[sigma])[1]
end
function numnegevals(T::SymTridiagonal{Float64}, sigmas::AbstractVector{<:Real})
    s = Vector{Float64}(sigmas)
    counts = Vector{Int64}(undef, length(s))
    check(ccall((:gla_numnegevals_host, libglagpu), Cint,
                (Int64, Ptr{Float64}, Ptr{Float64}, Int64, Ptr{Float64}, Ptr{Int64}),
                length(T.dv), Vector{Float64}(T.dv), Vector{Float64}(T.ev), length(s), s, counts))
    return counts
end

# eigvals(T, il:iu) and eigvals(T, vl, vu) (LinearAlgebra's subset methods)
# by Sturm-count multisection on the GPU.
function eigvals(T::SymTridiagonal{Float64}, irange::UnitRange; abstol = 0.0)
    n = length(T.dv)
    il, iu = first(irange), last(irange)
    w = Vector{Float64}(undef, max(iu - il + 1, 0))
    check(ccall((:gla_dstebz_host, libglagpu), Cint,
                (Int64, Ptr{Float64}, Ptr{Float64}, Int64, Int64, Cdouble, Ptr{Float64}),
                n, Vector{Float64}(T.dv), Vector{Float64}(T.ev), il, iu, Float64(abstol), w))
    return w
end
function eigvals(T::SymTridiagonal{Float64}, vl::Real, vu::Real; abstol = 0.0)
    il = numnegevals(T, vl) + 1
    iu = numnegevals(T, vu)
    return iu < il ? Float64[] : eigvals(T, il:iu; abstol)
end

export GPUMatrix

end # module
