# SeveroGPU.jl -- Julia glue that routes Severo.jl's embedding hot path to
# libseverogpu.so through ccall.  Written against the reference's call sites
# (src/normalize.jl, src/scaling.jl, src/irlba.jl, src/embedding.jl,
# src/neighbours.jl); not executed in this repository's test environment, which
# has no Julia.  The C entry points it calls are tested from Python.
module SeveroGPU

using SparseArrays, NamedArrays, LinearAlgebra, Random

const libsv = get(ENV, "SEVERO_GPU_LIB", joinpath(@__DIR__, "..", "lib", "libseverogpu.so"))
const SV_I32, SV_I64, SV_F32, SV_F64, SV_BF16 = Cint(1), Cint(2), Cint(3), Cint(4), Cint(5)

function svcheck(st::Cint)
    st == 0 && return nothing
    buf = Vector{UInt8}(undef, 2048)
    ccall((:sv_last_error, libsv), Cint, (Ptr{UInt8}, Csize_t), buf, length(buf))
    msg = unsafe_string(pointer(buf))
    st == -4 && error("convergence failed")            # src/irlba.jl:73
    error("severo_gpu: $msg")
end

mutable struct Context
    h::Ptr{Cvoid}
    function Context(device::Integer=0)
        r = Ref{Ptr{Cvoid}}(C_NULL)
        svcheck(ccall((:sv_context_create, libsv), Cint, (Cint, Ref{Ptr{Cvoid}}), device, r))
        c = new(r[])
        finalizer(c -> ccall((:sv_context_destroy, libsv), Cint, (Ptr{Cvoid},), c.h), c)
    end
end
const CTX = Ref{Context}()
ctx() = (isassigned(CTX) || (CTX[] = Context()); CTX[].h)

# device handles released by finalizers
mutable struct Handle
    h::Ptr{Cvoid}
    free::Symbol
    parent::Any          # keeps the handle this one reads from alive
    function Handle(h, free, parent=nothing)
        x = new(h, free, parent)
        finalizer(x -> ccall((x.free, libsv), Cint, (Ptr{Cvoid},), x.h), x)
    end
end

# ---- normalize_cells (src/normalize.jl:40-55,76-79) ---------------------------
function upload_counts(A::SparseMatrixCSC{<:Integer,Int64})
    r = Ref{Ptr{Cvoid}}(C_NULL)
    vt = sizeof(eltype(A)) == 8 ? SV_I64 : SV_I32
    svcheck(ccall((:sv_counts_upload_csc, libsv), Cint,
        (Ptr{Cvoid}, Int64, Int64, Int64, Ptr{Int64}, Cint, Ptr{Int64}, Cint, Ptr{Cvoid}, Cint, Cint, Ref{Ptr{Cvoid}}),
        ctx(), size(A, 1), size(A, 2), nnz(A), A.colptr, SV_I64, A.rowval, SV_I64, A.nzval, vt, 1, r))
    Handle(r[], :sv_counts_free)
end

# ---- readers (src/input.jl) ------------------------------------------------------
# readMM / the matrix of read_10X (src/input.jl:78-115,199-208): parsed on the
# device; rows_are_features for the 10X layout (features x barcodes).
function read_mtx(path::AbstractString; rows_are_features::Bool=true)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    svcheck(ccall((:sv_counts_read_mtx, libsv), Cint, (Ptr{Cvoid}, Cstring, Cint, Ref{Ptr{Cvoid}}),
        ctx(), path, rows_are_features, r))
    Handle(r[], :sv_counts_free)
end

_svtype(::Type{Int32}) = SV_I32
_svtype(::Type{Int64}) = SV_I64
_svtype(::Type{Float32}) = SV_F32
_svtype(::Type{Float64}) = SV_F64

# _read_10X_h5 / _read_h5 (src/input.jl:158-187,210-225): the stored features x
# barcodes CSC (0-based indptr over barcodes) is the cells x genes CSR.
function upload_10x_arrays(indptr::Vector, indices::Vector, data::Vector, dim)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    svcheck(ccall((:sv_counts_upload_csr, libsv), Cint,
        (Ptr{Cvoid}, Int64, Int64, Int64, Ptr{Cvoid}, Cint, Ptr{Cvoid}, Cint, Ptr{Cvoid}, Cint, Cint, Ref{Ptr{Cvoid}}),
        ctx(), dim[2], dim[1], length(indices), indptr, _svtype(eltype(indptr)), indices,
        _svtype(eltype(indices)), data, _svtype(eltype(data)), 0, r))
    Handle(r[], :sv_counts_free)
end

const DATA = WeakKeyDict{Any,Handle}()   # normalised matrix -> its device handle

function normalize_cells(X::NamedArray; method=:lognormalize, scale_factor::Real=1.0,
                         dtype::Type{T}=Float64) where {T<:AbstractFloat}
    method isa AbstractString && (method = Symbol(method))
    m = method == :lognormalize ? 0 : method == :relativecounts ? 1 :
        error("unknown normalization method: $method")
    counts = upload_counts(X.array)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    svcheck(ccall((:sv_normalize_cells, libsv), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cdouble, Cint, Ref{Ptr{Cvoid}}),
        ctx(), counts.h, m, convert(T, scale_factor), T == Float64 ? SV_F64 : SV_F32, r))
    data = Handle(r[], :sv_data_free, counts)
    A = X.array
    B = SparseMatrixCSC(size(A, 1), size(A, 2), A.colptr, A.rowval, Vector{T}(undef, nnz(A)))
    svcheck(ccall((:sv_data_download_csc, libsv), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{T}), ctx(), data.h, B.nzval))
    N = NamedArray(B, X.dicts, X.dimnames)
    DATA[N] = data
    N
end

# ---- filter_counts (src/filtering.jl:15-35,98-103) ------------------------------
# Cells, then genes, on the device; the kept matrix comes back as a labelled
# SparseMatrixCSC like the reference's X[CI, FI].
function filter_counts(A::NamedArray; min_cells=0, min_features=0, min_feature_count=0, min_umi=0)
    counts = upload_counts(A.array)
    CI = Vector{UInt8}(undef, size(A, 1)); FI = Vector{UInt8}(undef, size(A, 2))
    r = Ref{Ptr{Cvoid}}(C_NULL)
    svcheck(ccall((:sv_filter_counts, libsv), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Int64, Int64, Int64, Int64, Ptr{UInt8}, Ptr{UInt8}, Ref{Ptr{Cvoid}}),
        ctx(), counts.h, min_cells, min_features, min_feature_count, min_umi, CI, FI, r))
    kept = Handle(r[], :sv_counts_free)
    ci, fi = CI .!= 0, FI .!= 0
    m, n = count(ci), count(fi)
    nz = Ref{Int64}(0)
    svcheck(ccall((:sv_counts_info, libsv), Cint, (Ptr{Cvoid}, Ptr{Int64}, Ptr{Int64}, Ref{Int64}),
        kept.h, C_NULL, C_NULL, nz))
    colptr = Vector{Int64}(undef, n + 1); rowval = Vector{Int32}(undef, nz[]); nzval = Vector{Int32}(undef, nz[])
    svcheck(ccall((:sv_counts_download_csc, libsv), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Int64}, Ptr{Int32}, Ptr{Int32}),
        ctx(), kept.h, colptr, rowval, nzval))
    X = SparseMatrixCSC(m, n, colptr .+ 1, Int64.(rowval) .+ 1, eltype(A.array).(nzval))
    barcodes, features = names(A)
    NamedArray(X, (barcodes[ci], features[fi]), A.dimnames)
end

# ---- find_variable_features(:vst) (src/variablefeatures.jl:19-50,128-160) -------
# loess_surface: :interpolate (Loess.jl's kd-tree vertex fits blended linearly,
# what the reference's loess / predict give), :hermite, :direct.
const LOESS_SURFACE = Dict(:interpolate => Cint(0), :hermite => Cint(1), :direct => Cint(2))
function find_variable_features(X::NamedArray, nfeatures=2000; method=:vst, loess_span::Real=0.5,
                                loess_surface::Symbol=:interpolate)
    method isa AbstractString && (method = Symbol(method))
    method == :vst || error("unknown selection method: $method")
    counts = upload_counts(X.array)
    selected = Vector{Int64}(undef, nfeatures); metric = Vector{Float64}(undef, size(X, 2))
    svcheck(ccall((:sv_find_variable_features_vst_surface, libsv), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Int64, Cdouble, Cint, Ptr{Int64}, Ptr{Float64}),
        ctx(), counts.h, nfeatures, loess_span, LOESS_SURFACE[loess_surface], selected, metric))
    NamedArray(selected, (names(X, 2)[selected],), (dimnames(X, 2),))
end

# ---- scale_features / CenteredMatrix (src/scaling.jl:219-357) ------------------
struct GPUCenteredMatrix{T} <: AbstractMatrix{T}
    h::Handle
    m::Int
    n::Int
    mu::Vector{Float64}
end
Base.size(S::GPUCenteredMatrix) = (S.m, S.n)

function scale_features(X::NamedArray; scale_max::Real=Inf, features=nothing)
    data = DATA[X]
    f = features === nothing ? collect(Int64, 1:size(X, 2)) : collect(Int64, features)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    svcheck(ccall((:sv_scale_features, libsv), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Int64}, Int64, Cdouble, Ref{Ptr{Cvoid}}),
        ctx(), data.h, f, length(f), scale_max, r))
    h = Handle(r[], :sv_centered_free, data)
    mu = Vector{Float64}(undef, length(f))
    svcheck(ccall((:sv_centered_stats, libsv), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Ptr{Cvoid}, Ptr{Cvoid}),
        ctx(), h.h, mu, C_NULL, C_NULL))
    GPUCenteredMatrix{Float64}(h, size(X, 1), length(f), mu)
end

function _mul!(C::StridedVecOrMat{Float64}, S::GPUCenteredMatrix, trans::Char, v::StridedVecOrMat{Float64}, α, β)
    svcheck(ccall((:sv_centered_mul, libsv), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Cchar, Int64, Cdouble, Ptr{Float64}, Int64, Cdouble, Ptr{Float64}, Int64),
        ctx(), S.h.h, trans, size(v, 2), α, v, stride(v, 2), β, C, stride(C, 2)))
    C
end
LinearAlgebra.mul!(C::StridedVecOrMat{Float64}, S::GPUCenteredMatrix, v::StridedVecOrMat{Float64}, α::Number, β::Number) =
    _mul!(C, S, 'N', v, α, β)
LinearAlgebra.mul!(C::StridedVecOrMat{Float64}, S::Adjoint{<:Any,<:GPUCenteredMatrix}, v::StridedVecOrMat{Float64}, α::Number, β::Number) =
    _mul!(C, S.parent, 'T', v, α, β)

# ---- irlba / pca (src/irlba.jl:78-99, src/embedding.jl:46-94) ------------------
function irlba(S::GPUCenteredMatrix, nu::Integer; tol=1e-5, maxit=1000, init=randn(S.n))
    U = zeros(S.m, nu); s = zeros(nu); V = zeros(S.n, nu)
    it = Ref{Int64}(0); nmv = Ref{Int64}(0)
    svcheck(ccall((:sv_irlba, libsv), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Int64, Int64, Int64, Cdouble, Ptr{Float64}, UInt64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ref{Int64}, Ref{Int64}),
        ctx(), S.h.h, nu, 0, maxit, tol, init, rand(UInt64), s, U, V, it, nmv))
    SVD(U, s, Matrix(V'))
end

struct GPUEmbedding
    h::Handle
    coordinates::Matrix{Float64}
    stdev::Vector{Float64}
    basis::Matrix{Float64}
end

function pca(S::GPUCenteredMatrix, npcs::Integer; tol=1e-5, maxit=1000, init=randn(S.n))
    k = min(S.m, S.n, npcs)
    Z = zeros(S.m, k); stdev = zeros(k); load = zeros(S.n, k)
    e = Ref{Ptr{Cvoid}}(C_NULL); it = Ref{Int64}(0); nmv = Ref{Int64}(0)
    svcheck(ccall((:sv_pca, libsv), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Int64, Int64, Cdouble, Ptr{Float64}, UInt64, Ref{Ptr{Cvoid}}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ref{Int64}, Ref{Int64}),
        ctx(), S.h.h, k, maxit, tol, init, rand(UInt64), e, Z, stdev, load, it, nmv))
    GPUEmbedding(Handle(e[], :sv_embed_free, S.h), Z, stdev, load)
end

# ---- neighbours (src/neighbours.jl:19-349) --------------------------------------
function ann(em::GPUEmbedding, k::Integer; include_self::Bool=true, bf16::Bool=true)
    n = size(em.coordinates, 1)
    idx = Matrix{Int32}(undef, n, k); dist = Matrix{Float64}(undef, n, k)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    svcheck(ccall((:sv_knn_embed, libsv), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Int64, Int64, Cint, Cint, Cint, Ptr{Int32}, Ptr{Float64}, Ref{Ptr{Cvoid}}),
        ctx(), em.h.h, 0, k, 0, include_self, bf16 ? 1 : 0, idx, dist, r))
    idx, dist, Handle(r[], :sv_knn_free, em.h)
end

function nearest_neighbours(em::GPUEmbedding, k::Integer; include_self::Bool=true)
    idx, _, _ = ann(em, k; include_self=include_self)
    n = size(idx, 1)
    sparse(vec(idx'), repeat(1:n, inner=k), trues(length(idx)))   # src/neighbours.jl:79
end

function shared_nearest_neighbours(em::GPUEmbedding, k::Integer; prune::Real=1/15,
                                   include_self::Bool=true, dtype::Type{T}=Float64) where {T}
    _, _, kn = ann(em, k; include_self=include_self)
    g = Ref{Ptr{Cvoid}}(C_NULL)
    svcheck(ccall((:sv_snn_knn, libsv), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Int64, Cdouble, Cint, Ref{Ptr{Cvoid}}),
        ctx(), kn.h, k, prune, T == Float64 ? SV_F64 : SV_F32, g))
    gh = Handle(g[], :sv_graph_free)
    n = Ref{Int64}(0); nz = Ref{Int64}(0)
    svcheck(ccall((:sv_graph_info, libsv), Cint, (Ptr{Cvoid}, Ref{Int64}, Ref{Int64}), gh.h, n, nz))
    colptr = Vector{Int64}(undef, n[] + 1); rowval = Vector{Int64}(undef, nz[]); nzval = Vector{T}(undef, nz[])
    svcheck(ccall((:sv_graph_download, libsv), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Int64}, Ptr{Int64}, Ptr{T}),
        ctx(), gh.h, colptr, rowval, nzval))
    SparseMatrixCSC(n[], n[], colptr, rowval, nzval)
end

end # module
