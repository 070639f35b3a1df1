"""
    RBFFDGPU

Julia host side of librbffd (include/rbffd.h): the methods of
RadialBasisFiniteDifferences.jl's operator API -- `generate_operator`,
`hyperviscosity_operator`, `calculateneighbors` -- with the same arguments and return
values (`SparseMatrixCSC{Float64,Int64}`), computed on a GB300 through `ccall`.

The library writes the CSC arrays (1-based `colptr`/`rowval`, `nzval`) straight into
Julia-owned vectors, so no copy is made on the Julia side.  A singular local system
raises `LinearAlgebra.SingularException` as `inv` does in the reference
(src/interpolationmatrix.jl:8); every other failure raises `ErrorException`.
"""
module RBFFDGPU

using LinearAlgebra
using SparseArrays
using StaticArrays

const LIB = get(ENV, "RBFFD_LIB", joinpath(@__DIR__, "..", "_lib", "librbffd.so"))

const OP = (E = 0, Dx = 1, Dy = 2, Dxx = 3, Dyy = 4, Dxy = 5, Lap = 6, Dxk = 7, Dyk = 8, HV = 9)
const PREC = (fp64 = Cint(0), mixed = Cint(1))
mask(ops) = reduce(|, (UInt32(1) << getfield(OP, o) for o in ops))
const GENERATE = (:E, :Dx, :Dy, :Dxx, :Dyy, :Dxy)

struct Options
    device::Cint
    warps_per_block::Cint
    max_refine::Cint
    refine_tol::Cdouble
end

struct Stats
    ms_upload::Cdouble
    ms_grid::Cdouble
    ms_knn::Cdouble
    ms_solve::Cdouble
    ms_fallback::Cdouble
    ms_csr::Cdouble
    ms_total::Cdouble
    n_systems::Int64
    n_rows::Int64
    n_fallback::Int64
    first_bad_node::Int64
    refine_hist::NTuple{8,Int64}
    nnz::Int64
    kernel_launches::Int64
end
Stats() = Stats(0, 0, 0, 0, 0, 0, 0, 0, 0, 0, -1, ntuple(_ -> 0, 8), 0, 0)

struct CSC
    colptr::Ptr{Int64}
    rowval::Ptr{Int64}
    nzval::Ptr{Float64}
end

mutable struct Handle
    ptr::Ptr{Cvoid}
end

function Handle(; device::Integer = 0, warps_per_block::Integer = 0)
    ref = Ref{Ptr{Cvoid}}(C_NULL)
    opt = Ref(Options(device, warps_per_block, 0, 0.0))
    rc = ccall((:rbffd_create, LIB), Cint, (Ref{Options}, Ref{Ptr{Cvoid}}), opt, ref)
    rc == 0 || error("rbffd_create: ", unsafe_string(ccall((:rbffd_last_error, LIB), Cstring, (Ptr{Cvoid},), C_NULL)))
    h = Handle(ref[])
    finalizer(h) do x
        x.ptr == C_NULL || ccall((:rbffd_destroy, LIB), Cvoid, (Ptr{Cvoid},), x.ptr)
        x.ptr = C_NULL
    end
    return h
end

const _handle = Ref{Union{Nothing,Handle}}(nothing)
handle() = something(_handle[], (_handle[] = Handle()))

function check(h::Handle, rc, stats::Ref{Stats})
    rc == 0 && return nothing
    msg = unsafe_string(ccall((:rbffd_last_error, LIB), Cstring, (Ptr{Cvoid},), h.ptr))
    rc == 3 && throw(SingularException(Int(stats[].first_bad_node) + 1))
    error("librbffd error $rc: $msg")
end

points(X) = convert(Vector{SVector{2,Float64}}, X)

"Node classes from the index ranges of calculateneighbors: 0 interior, +b boundary b, -b ghost of b."
function node_class(N, X_idx_in, X_idx_bc, X_idx_bc_g)
    c = fill(typemin(Int32), N)
    c[X_idx_in] .= 0
    for (b, r) in enumerate(X_idx_bc)
        c[r] .= b
    end
    for (b, r) in enumerate(X_idx_bc_g)
        c[r] .= -b
    end
    any(==(typemin(Int32)), c) && throw(ArgumentError("every node must be in X_idx_in, X_idx_bc or X_idx_bc_g"))
    return c
end

function alloc_csc(M, N, n, nops)
    mats = [(Vector{Int64}(undef, N + 1), Vector{Int64}(undef, M * n), Vector{Float64}(undef, M * n)) for _ in 1:nops]
    structs = [CSC(pointer(a), pointer(b), pointer(c)) for (a, b, c) in mats]
    return mats, structs
end

tocsc(M, N, m) = SparseMatrixCSC(M, N, m[1], m[2], m[3])

function _generate(X, Y, p, n, polydeg, cls, ops; precision = :fp64, h = handle())
    Xv = points(X)
    Yv = Y === X ? Xv : points(Y)
    N, M = length(Xv), length(Yv)
    order = sort(collect(ops); by = o -> getfield(OP, o))
    mats, structs = alloc_csc(M, N, n, length(order))
    stats = Ref(Stats())
    GC.@preserve Xv Yv cls mats begin
        rc = ccall((:rbffd_generate_operator, LIB), Cint,
            (Ptr{Cvoid}, Ptr{Float64}, Int64, Ptr{Float64}, Int64, Cint, Cint, Cint, Ptr{Int32}, UInt32, Cint,
             Ptr{CSC}, Ref{Stats}),
            h.ptr, pointer(reinterpret(Float64, Xv)), N, pointer(reinterpret(Float64, Yv)), M, p, n, polydeg,
            cls === nothing ? C_NULL : pointer(cls), mask(order), getfield(PREC, precision), structs, stats)
    end
    check(h, rc, stats)
    byop = Dict(o => tocsc(M, N, m) for (o, m) in zip(order, mats))
    return Tuple(byop[o] for o in ops)
end

"generate_operator(X, Y, p, n, polydeg) -- src/generate_operator.jl:29-190"
generate_operator(X, Y, p, n, polydeg; kw...) = _generate(X, Y, p, n, polydeg, nothing, GENERATE; kw...)

"Boundary-aware overload -- src/generate_operator.jl:192-352"
function generate_operator(X, Y, p, n, polydeg, X_idx_in, X_idx_bc, X_idx_bc_g, Y_idx_in, Y_idx_bc, Y_idx_bc_g; kw...)
    cls = node_class(length(X), X_idx_in, X_idx_bc, X_idx_bc_g)
    return _generate(X, Y, p, n, polydeg, cls, GENERATE; kw...)
end

"Collocated, unscaled overload -- src/generate_operator.jl:354-491 (reproduced as computed there)"
function generate_operator(X, p::Integer, n::Integer, polydeg::Integer; h = handle())
    Xv = points(X)
    N = length(Xv)
    mats, structs = alloc_csc(N, N, n, 6)
    stats = Ref(Stats())
    GC.@preserve Xv mats begin
        rc = ccall((:rbffd_generate_operator_unscaled, LIB), Cint,
            (Ptr{Cvoid}, Ptr{Float64}, Int64, Cint, Cint, Cint, UInt32, Cint, Ptr{CSC}, Ref{Stats}),
            h.ptr, pointer(reinterpret(Float64, Xv)), N, p, n, polydeg, mask(GENERATE), 0, structs, stats)
    end
    check(h, rc, stats)
    return Tuple(tocsc(N, N, m) for m in mats)
end

function _hyper(k_deriv, X, Y, p, n, polydeg, cls; precision = :fp64, h = handle())
    Xv = points(X)
    Yv = Y === X ? Xv : points(Y)
    N, M = length(Xv), length(Yv)
    mats, structs = alloc_csc(M, N, n, 2)
    stats = Ref(Stats())
    GC.@preserve Xv Yv cls mats begin
        rc = ccall((:rbffd_hyperviscosity_operator, LIB), Cint,
            (Ptr{Cvoid}, Cint, Ptr{Float64}, Int64, Ptr{Float64}, Int64, Cint, Cint, Cint, Ptr{Int32}, Cint,
             Ptr{CSC}, Ref{Stats}),
            h.ptr, k_deriv, pointer(reinterpret(Float64, Xv)), N, pointer(reinterpret(Float64, Yv)), M, p, n,
            polydeg, cls === nothing ? C_NULL : pointer(cls), getfield(PREC, precision), structs, stats)
    end
    check(h, rc, stats)
    return tocsc(M, N, mats[1]), tocsc(M, N, mats[2])
end

"hyperviscosity_operator(k_deriv, X, Y, p, n, polydeg) -- src/hyperviscosity_operator.jl:26-175"
hyperviscosity_operator(k_deriv, X, Y, p, n, polydeg; kw...) = _hyper(k_deriv, X, Y, p, n, polydeg, nothing; kw...)

"Boundary-aware overload -- src/hyperviscosity_operator.jl:177-312"
function hyperviscosity_operator(k_deriv, X, Y, p, n, polydeg, X_idx_in, X_idx_bc, X_idx_bc_g, Y_idx_in, Y_idx_bc,
                                 Y_idx_bc_g; kw...)
    cls = node_class(length(X), X_idx_in, X_idx_bc, X_idx_bc_g)
    return _hyper(k_deriv, X, Y, p, n, polydeg, cls; kw...)
end

"Collocated, unscaled overload -- src/hyperviscosity_operator.jl:314-440"
function hyperviscosity_operator(k_deriv::Integer, X, p::Integer, n::Integer, polydeg::Integer; h = handle())
    Xv = points(X)
    N = length(Xv)
    mats, structs = alloc_csc(N, N, n, 2)
    stats = Ref(Stats())
    GC.@preserve Xv mats begin
        rc = ccall((:rbffd_generate_operator_unscaled, LIB), Cint,
            (Ptr{Cvoid}, Ptr{Float64}, Int64, Cint, Cint, Cint, UInt32, Cint, Ptr{CSC}, Ref{Stats}),
            h.ptr, pointer(reinterpret(Float64, Xv)), N, p, n, polydeg, mask((:Dxk, :Dyk)), k_deriv, structs, stats)
    end
    check(h, rc, stats)
    return tocsc(N, N, mats[1]), tocsc(N, N, mats[2])
end

"calculateneighbors(X, Y, n, X_idx_in, X_idx_bc, X_idx_bc_g, Y_idx_in, Y_idx_bc, Y_idx_bc_g) -- src/calculateneighbors.jl:1-97"
function calculateneighbors(X, Y, n, X_idx_in, X_idx_bc, X_idx_bc_g, Y_idx_in, Y_idx_bc, Y_idx_bc_g; h = handle())
    Xv, Yv = points(X), points(Y)
    N, M = length(Xv), length(Yv)
    cls = node_class(N, X_idx_in, X_idx_bc, X_idx_bc_g)
    ix = Matrix{Int64}(undef, n, N)   # column i = stencil of node i (row-major N x n on the C side)
    dx = Matrix{Float64}(undef, n, N)
    iy = Vector{Int64}(undef, M)
    dy = Vector{Float64}(undef, M)
    GC.@preserve Xv Yv cls ix dx iy dy begin
        rc = ccall((:rbffd_calculateneighbors, LIB), Cint,
            (Ptr{Cvoid}, Ptr{Float64}, Int64, Ptr{Float64}, Int64, Cint, Ptr{Int32}, Ptr{Int64}, Ptr{Float64},
             Ptr{Int64}, Ptr{Float64}),
            h.ptr, pointer(reinterpret(Float64, Xv)), N, pointer(reinterpret(Float64, Yv)), M, n, pointer(cls),
            pointer(ix), pointer(dx), pointer(iy), pointer(dy))
    end
    check(h, rc, Ref(Stats()))
    idxs_x = [SVector{n}(view(ix, :, i)) for i in 1:N]
    dists_x = [SVector{n}(view(dx, :, i)) for i in 1:N]
    idxs_y_x = [SVector{1}(iy[i]) for i in 1:M]
    dists_y_x = [SVector{1}(dy[i]) for i in 1:M]
    return idxs_x, idxs_y_x, dists_x, dists_y_x
end

# processmesh(meshname, markernames) (src/processmesh.jl:1-192) after its HDF5/CGNS reads,
# which stay in Julia (HDF5.jl): vertices from Base/dom-1/GridCoordinates, the triangles'
# and every marker's ElementConnectivity.  Returns the reference's Y, Y_idx_in, Y_idx_bc,
# Y_idx_bc_g, bc_normals and bc_tangents (the VTK cells are the caller's), plus the ghost
# offset.
function processmesh_arrays(vertices, tri_conn::AbstractMatrix{<:Integer},
                            bc_conns::AbstractVector{<:AbstractMatrix{<:Integer}}; h = handle())
    V = points(vertices)
    T = Matrix{Int64}(tri_conn)                        # 3 x ntri, 1-based (CGNS order)
    B = reduce(hcat, [Matrix{Int64}(b) for b in bc_conns])  # 2 x nbc, markers in element-range order
    ntri, nbc = size(T, 2), size(B, 2)
    Y = Vector{SVector{2,Float64}}(undef, ntri + 2nbc)
    nrm = Vector{SVector{2,Float64}}(undef, nbc)
    tng = Vector{SVector{2,Float64}}(undef, nbc)
    off = Ref{Float64}(0.0)
    GC.@preserve V T B Y nrm tng begin
        rc = ccall((:rbffd_process_mesh, LIB), Cint,
            (Ptr{Cvoid}, Ptr{Float64}, Int64, Ptr{Int64}, Int64, Ptr{Int64}, Int64, Ptr{Float64}, Ptr{Float64},
             Ptr{Float64}, Ref{Float64}),
            h.ptr, pointer(reinterpret(Float64, V)), length(V), pointer(T), ntri, pointer(B), nbc,
            pointer(reinterpret(Float64, Y)), pointer(reinterpret(Float64, nrm)), pointer(reinterpret(Float64, tng)),
            off)
    end
    check(h, rc, Ref(Stats()))
    Y_idx_bc, Y_idx_bc_g, bc_normals, bc_tangents = UnitRange{Int}[], UnitRange{Int}[], [], []
    a = 0
    for b in bc_conns
        m = size(b, 2)
        push!(Y_idx_bc, (ntri + a + 1):(ntri + a + m))
        push!(Y_idx_bc_g, (ntri + nbc + a + 1):(ntri + nbc + a + m))
        push!(bc_normals, nrm[(a + 1):(a + m)])
        push!(bc_tangents, tng[(a + 1):(a + m)])
        a += m
    end
    return Y, 1:ntri, Y_idx_bc, Y_idx_bc_g, bc_normals, bc_tangents, off[]
end

# ----------------------------------------------------------------------------------------
# Device-resident operators and time stepping (examples/adv_diff_test.jl:144-199).  Field
# arguments are device buffers: any object whose `pointer` is a device address (a CUDA.jl
# CuArray, row-major [rows][nfields] as a permuted/transposed view of Julia's column-major
# storage: `CuArray{Float64}(undef, nfields, rows)`).

struct Problem
    X::Ptr{Float64}
    N::Int64
    Y::Ptr{Float64}
    M::Int64
    p::Cint
    n::Cint
    polydeg::Cint
    node_class::Ptr{Int32}
    n_per_node::Ptr{Int32}
    deg_per_node::Ptr{Int32}
    op_mask::UInt32
    k_deriv::Cint
    precision::Cint
    memspace::Cint
    row_begin::Int64
    row_end::Int64
end

devptr(a) = reinterpret(Ptr{Cvoid}, UInt(pointer(a)))

mutable struct OperatorSet
    ptr::Ptr{Cvoid}
    h::Handle
    ops::Vector{Symbol}
end

"Operators `ops` of the collocated node set X kept in GPU memory (rbffd_opset_create)."
function OperatorSet(X, p, n, polydeg, ops; precision = :mixed, k_deriv = 0, node_class = nothing, h = handle())
    Xv = points(X)
    order = sort(collect(ops); by = o -> getfield(OP, o))
    ref = Ref{Ptr{Cvoid}}(C_NULL)
    stats = Ref(Stats())
    GC.@preserve Xv node_class begin
        prob = Ref(Problem(pointer(reinterpret(Float64, Xv)), length(Xv), C_NULL, 0, p, n, polydeg,
                           node_class === nothing ? C_NULL : pointer(node_class), C_NULL, C_NULL, mask(order),
                           k_deriv, getfield(PREC, precision), 0, 0, 0))
        rc = ccall((:rbffd_opset_create, LIB), Cint, (Ptr{Cvoid}, Ref{Problem}, Ref{Ptr{Cvoid}}, Ref{Stats}),
                   h.ptr, prob, ref, stats)
    end
    check(h, rc, stats)
    s = OperatorSet(ref[], h, order)
    finalizer(x -> (x.ptr == C_NULL || ccall((:rbffd_opset_destroy, LIB), Cvoid, (Ptr{Cvoid}, Ptr{Cvoid}),
                                             x.h.ptr, x.ptr); x.ptr = C_NULL), s)
    return s
end

"y = A_op x on the GPU (x, y device vectors of Float64), the `D * u` of cons_sys."
function spmv!(y, s::OperatorSet, op::Symbol, x)
    q = findfirst(==(op), s.ops) - 1
    rc = ccall((:rbffd_spmv, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Cvoid}, Ptr{Cvoid}),
               s.h.ptr, s.ptr, q, devptr(x), devptr(y))
    check(s.h, rc, Ref(Stats()))
    return y
end

mutable struct RK4
    ptr::Ptr{Cvoid}
    h::Handle
    sets::Vector{OperatorSet}
end

"RK4 for du/dt = L u, L = sum(coef .* operators of `sets`); rows with fixed_rows[i] != 0 held."
function RK4(sets::Vector{OperatorSet}, coef::Vector{Float64}, nfields; fixed_rows = nothing, dtype = :f64)
    h = sets[1].h
    ref = Ref{Ptr{Cvoid}}(C_NULL)
    ptrs = [s.ptr for s in sets]
    fx = fixed_rows === nothing ? nothing : UInt8.(fixed_rows .!= 0)
    GC.@preserve ptrs coef fx begin
        rc = ccall((:rbffd_rk4_create, LIB), Cint,
                   (Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Cint, Ptr{Float64}, Ptr{UInt8}, Cint, Cint, Ref{Ptr{Cvoid}}),
                   h.ptr, pointer(ptrs), length(sets), pointer(coef), fx === nothing ? C_NULL : pointer(fx),
                   nfields, dtype === :f64 ? 0 : 1, ref)
    end
    check(h, rc, Ref(Stats()))
    rk = RK4(ref[], h, sets)
    finalizer(x -> (x.ptr == C_NULL || ccall((:rbffd_rk4_destroy, LIB), Cvoid, (Ptr{Cvoid}, Ptr{Cvoid}),
                                             x.h.ptr, x.ptr); x.ptr = C_NULL), rk)
    return rk
end

"Advance the device fields u in place by nsteps RK4 steps of size dt."
function step!(rk::RK4, u, dt, nsteps)
    rc = ccall((:rbffd_rk4_run, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cdouble, Int64),
               rk.h.ptr, rk.ptr, devptr(u), dt, nsteps)
    check(rk.h, rc, Ref(Stats()))
    ccall((:rbffd_synchronize, LIB), Cint, (Ptr{Cvoid},), rk.h.ptr)
    return u
end

"""
    DeviceOperator(set, op)

One operator of a device-resident set as a lazily materialised matrix: products with device
vectors run on the GPU (`mul!` -> rbffd_spmv) and the host `SparseMatrixCSC` is built only
when asked for (`SparseMatrixCSC(A)` -> rbffd_opset_export_csc into Julia-owned arrays, the
same 1-based CSC the reference's `sparse(I, J, V)` returns), so a time loop never copies the
operator to the host.
"""
struct DeviceOperator <: AbstractMatrix{Float64}
    set::OperatorSet
    op::Symbol
end

function shape(s::OperatorSet)
    r, c, z, q = Ref{Int64}(0), Ref{Int64}(0), Ref{Int64}(0), Ref{Cint}(0)
    ccall((:rbffd_opset_shape, LIB), Cint, (Ptr{Cvoid}, Ref{Int64}, Ref{Int64}, Ref{Int64}, Ref{Cint}),
          s.ptr, r, c, z, q)
    return r[], c[], z[]
end

Base.size(A::DeviceOperator) = shape(A.set)[1:2]
Base.getindex(A::DeviceOperator, i::Int, j::Int) = SparseMatrixCSC(A)[i, j]  # host access materialises

LinearAlgebra.mul!(y, A::DeviceOperator, x) = spmv!(y, A.set, A.op, x)

function SparseArrays.SparseMatrixCSC(A::DeviceOperator)
    rows, cols, nnz = shape(A.set)
    colptr, rowval, nzval = Vector{Int64}(undef, cols + 1), Vector{Int64}(undef, nnz), Vector{Float64}(undef, nnz)
    q = findfirst(==(A.op), A.set.ops) - 1
    GC.@preserve colptr rowval nzval begin
        out = Ref(CSC(pointer(colptr), pointer(rowval), pointer(nzval)))
        rc = ccall((:rbffd_opset_export_csc, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ref{CSC}),
                   A.set.h.ptr, A.set.ptr, q, out)
    end
    check(A.set.h, rc, Ref(Stats()))
    return SparseMatrixCSC(rows, cols, colptr, rowval, nzval)
end

export generate_operator, hyperviscosity_operator, calculateneighbors, processmesh_arrays, OperatorSet, spmv!, RK4, step!,
       DeviceOperator

end # module
