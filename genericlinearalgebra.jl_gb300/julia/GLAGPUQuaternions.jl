# eigen!/eigvals! on Hermitian{Quaternion{Float64}} (the reference's
# quaternion Hermitian support, test/eigenselfadjoint.jl:54-84) through
# gla_qheev_host: the real symmetric matrix of left multiplication, of order
# 4n, on the GPU. Include after GLAGPU.jl in an environment that has
# Quaternions (v0.7: Quaternion{Float64} is the four Float64 fields s, v1,
# v2, v3, the layout gla_qheev reads):
#
#     include("GLAGPU.jl"); include("GLAGPUQuaternions.jl")
#     vals, vecs = GLAGPU.eigen!(Hermitian(A))   # A::Matrix{QuaternionF64}
using LinearAlgebra
using Quaternions

function GLAGPU.eigen!(A::Hermitian{Quaternion{Float64},Matrix{Quaternion{Float64}}}; tol = eps(Float64),
                       sortby = LinearAlgebra.eigsortby, alg = nothing)
    n = size(A, 1)
    w = Vector{Float64}(undef, n)
    V = Matrix{Quaternion{Float64}}(undef, n, n)
    info = Ref{Cint}(0)
    GLAGPU.check(ccall((:gla_qheev_host, GLAGPU.libglagpu), Cint,
                       (UInt8, UInt8, Int64, Ptr{Quaternion{Float64}}, Int64, Ptr{Float64}, Ptr{Quaternion{Float64}},
                        Int64, Ref{Cint}),
                       UInt8('V'), UInt8(GLAGPU.uplochar(A)), n, A.data, max(n, 1), w, V, max(n, 1), info))
    GLAGPU.raise_info(Cint[info[]])
    return LinearAlgebra.Eigen(w, V)
end

function GLAGPU.eigvals!(A::Hermitian{Quaternion{Float64},Matrix{Quaternion{Float64}}}; tol = eps(Float64),
                         sortby = LinearAlgebra.eigsortby)
    n = size(A, 1)
    w = Vector{Float64}(undef, n)
    info = Ref{Cint}(0)
    GLAGPU.check(ccall((:gla_qheev_host, GLAGPU.libglagpu), Cint,
                       (UInt8, UInt8, Int64, Ptr{Quaternion{Float64}}, Int64, Ptr{Float64}, Ptr{Quaternion{Float64}},
                        Int64, Ref{Cint}),
                       UInt8('N'), UInt8(GLAGPU.uplochar(A)), n, A.data, max(n, 1), w, C_NULL, max(n, 1), info))
    GLAGPU.raise_info(Cint[info[]])
    return w
end

GLAGPU.eigen(A::Hermitian{Quaternion{Float64},Matrix{Quaternion{Float64}}}; kw...) = GLAGPU.eigen!(copy(A); kw...)
GLAGPU.eigvals(A::Hermitian{Quaternion{Float64},Matrix{Quaternion{Float64}}}; kw...) = GLAGPU.eigvals!(copy(A); kw...)
