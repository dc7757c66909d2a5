"""
    AdFemGPU

Julia bindings of libadfem_gpu.so for AdFem.jl users.

* The legacy symbols (init_nnfem_mesh, mfem_get_*, *_forward_Julia) have the
  signatures AdFem already ccalls, so pointing AdFem's `LIBMFEM` at this library
  makes `Mesh`, `compute_fem_laplace_matrix1`, `compute_fem_source_term1` and
  `compute_fem_stiffness_matrix` run on the GPU unchanged.
* This module adds the direct SparseMatrixCSC outputs (no COO + `sparse` round trip)
  for P1 and P2 meshes (Laplace, mass, stiffness), the Gauss-point interpolation ops,
  the Dirichlet imposition, `K\\F` on the GPU, and resident Poisson systems that keep
  the operator and the solver on the GPU across solves.
"""
module AdFemGPU

using SparseArrays

const LIB = get(ENV, "ADFEM_GPU_LIB", joinpath(@__DIR__, "..", "lib", "libadfem_gpu.so"))

function check(st::Integer)
    st == 0 && return nothing
    msg = unsafe_string(ccall((:adfem_last_error, LIB), Cstring, ()))
    error("libadfem_gpu: $msg (status $st)")
end

"""GPU-resident mesh; `coords` (n,2), `elems` (m,3) 1-based, as `AdFem.Mesh(coords, elems; degree)`
(degree 1: P1 with the order-2 rule; degree 2: P2 with the order-4 rule)."""
mutable struct GMesh
    h::Ptr{Cvoid}
    nnode::Int
    nelem::Int
    ndof::Int
    ngauss::Int
    nnz::Int
    function GMesh(coords::Matrix{Float64}, elems::Matrix{Int64}; degree::Integer = 1)
        xyz = vec([coords zeros(size(coords, 1))]')
        e0 = Int32.(vec(elems' .- 1))
        h = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:adfem_mesh_create, LIB), Cint, (Ptr{Cdouble}, Clonglong, Ptr{Cint}, Clonglong, Cint, Ptr{Ptr{Cvoid}}),
                    xyz, size(coords, 1), e0, size(elems, 1), degree, h))
        ng, nnz = Ref{Clonglong}(0), Ref{Clonglong}(0)
        check(ccall((:adfem_mesh_sizes, LIB), Cint, (Ptr{Cvoid}, Ptr{Clonglong}, Ptr{Clonglong}, Ptr{Clonglong}, Ptr{Clonglong}),
                    h[], C_NULL, C_NULL, ng, nnz))
        ndof = Ref{Clonglong}(0)
        check(ccall((:adfem_mesh_space, LIB), Cint, (Ptr{Cvoid}, Ptr{Cint}, Ptr{Cint}, Ptr{Cint}, Ptr{Clonglong}, Ptr{Clonglong}),
                    h[], C_NULL, C_NULL, C_NULL, ndof, C_NULL))
        m = new(h[], size(coords, 1), size(elems, 1), ndof[], ng[], nnz[])
        finalizer(x -> ccall((:adfem_mesh_destroy, LIB), Cint, (Ptr{Cvoid},), x.h), m)
        return m
    end
end

function pattern(m::GMesh)
    colptr = Vector{Int64}(undef, m.ndof + 1)
    rowval = Vector{Int64}(undef, m.nnz)
    check(ccall((:adfem_mesh_pattern, LIB), Cint, (Ptr{Cvoid}, Ptr{Clonglong}, Ptr{Clonglong}), m.h, colptr, rowval))
    colptr, rowval
end

"""compute_fem_laplace_matrix1(κ, mesh) with the SparseMatrixCSC built on the GPU (MCore.jl:112-120)."""
function compute_fem_laplace_matrix1(kappa::Vector{Float64}, m::GMesh)
    colptr, rowval = pattern(m)
    nzval = Vector{Float64}(undef, length(rowval))
    check(ccall((:adfem_laplace_csc, LIB), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Clonglong, Ptr{Cdouble}),
                m.h, kappa, length(kappa), nzval))
    SparseMatrixCSC(m.ndof, m.ndof, colptr, rowval, nzval)
end

"""compute_fem_stiffness_matrix(D, mesh) (MCore.jl:296-315): the 2ndof x 2ndof operator in the
reference's [x block; y block] ordering, with D[i, :, :] the 3x3 material matrix at Gauss point i,
built on the GPU as a SparseMatrixCSC."""
function compute_fem_stiffness_matrix(D::Array{Float64,3}, m::GMesh)
    size(D) == (m.ngauss, 3, 3) || error("D must be ngauss x 3 x 3")
    hmat = vec(permutedims(D, (3, 2, 1)))  # row-major 3x3 per Gauss point, as MCore.jl:298-307
    n2 = 2 * m.ndof
    colptr = Vector{Int64}(undef, n2 + 1)
    rowval = Vector{Int64}(undef, 4 * m.nnz)
    check(ccall((:adfem_mesh_pattern_elasticity, LIB), Cint, (Ptr{Cvoid}, Ptr{Clonglong}, Ptr{Clonglong}),
                m.h, colptr, rowval))
    nzval = Vector{Float64}(undef, length(rowval))
    check(ccall((:adfem_stiffness_csc, LIB), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Clonglong, Ptr{Cdouble}),
                m.h, hmat, length(hmat), nzval))
    SparseMatrixCSC(n2, n2, colptr, rowval, nzval)
end

"""compute_fem_mass_matrix1(ρ, mesh) (MCore.jl:170-181)."""
function compute_fem_mass_matrix1(rho::Vector{Float64}, m::GMesh)
    colptr, rowval = pattern(m)
    nzval = Vector{Float64}(undef, length(rowval))
    check(ccall((:adfem_mass_csc, LIB), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Clonglong, Ptr{Cdouble}),
                m.h, rho, length(rho), nzval))
    SparseMatrixCSC(m.ndof, m.ndof, colptr, rowval, nzval)
end

"""fem_to_gauss_points(u, mesh) (MUtils.jl:241-246): nodal values at the Gauss points."""
function fem_to_gauss_points(u::Vector{Float64}, m::GMesh)
    out = Vector{Float64}(undef, m.ngauss)
    check(ccall((:adfem_fem_to_gauss, LIB), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Clonglong, Ptr{Cdouble}),
                m.h, u, length(u), out))
    out
end

"""dof_to_gauss_points(u, mesh) (MUtils.jl:264-270): DOF values at the Gauss points."""
function dof_to_gauss_points(u::Vector{Float64}, m::GMesh)
    out = Vector{Float64}(undef, m.ngauss)
    check(ccall((:adfem_dof_to_gauss, LIB), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Clonglong, Ptr{Cdouble}),
                m.h, u, length(u), out))
    out
end

"""compute_fem_source_term1(f, mesh) (MCore.jl:77-82)."""
function compute_fem_source_term1(f::Vector{Float64}, m::GMesh)
    out = zeros(m.ndof)
    check(ccall((:adfem_source, LIB), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Clonglong, Ptr{Cdouble}, Cint),
                m.h, f, length(f), out, 0))
    out
end

"""impose_Dirichlet_boundary_conditions(A, rhs, bdnode, bdval) for a SparseMatrixCSC (MUtils.jl:184-199)."""
function impose_Dirichlet_boundary_conditions(A::SparseMatrixCSC{Float64,Int64}, rhs::Vector{Float64},
                                              bdnode::Vector{Int64}, bdval::Vector{Float64})
    n = size(A, 1)
    onnz = Ref{Clonglong}(0)
    args = (n, A.colptr, A.rowval, A.nzval, rhs, bdnode, length(bdnode), bdval, 0)
    check(ccall((:adfem_dirichlet_csc, LIB), Cint,
                (Clonglong, Ptr{Clonglong}, Ptr{Clonglong}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Clonglong}, Clonglong,
                 Ptr{Cdouble}, Cint, Ptr{Clonglong}, Ptr{Clonglong}, Ptr{Cdouble}, Ptr{Clonglong}, Ptr{Cdouble}),
                args..., C_NULL, C_NULL, C_NULL, onnz, C_NULL))
    colptr = Vector{Int64}(undef, n + 1)
    rowval = Vector{Int64}(undef, onnz[])
    nzval = Vector{Float64}(undef, onnz[])
    r = Vector{Float64}(undef, n)
    check(ccall((:adfem_dirichlet_csc, LIB), Cint,
                (Clonglong, Ptr{Clonglong}, Ptr{Clonglong}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Clonglong}, Clonglong,
                 Ptr{Cdouble}, Cint, Ptr{Clonglong}, Ptr{Clonglong}, Ptr{Cdouble}, Ptr{Clonglong}, Ptr{Cdouble}),
                args..., colptr, rowval, nzval, onnz, r))
    SparseMatrixCSC(n, n, colptr, rowval, nzval), r
end

# adfem_solver_opts / adfem_solver_stats (include/adfem_gpu.h)
struct SolverOpts
    rtol::Cdouble
    max_iter::Cint
    precision::Cint      # 0 FP64, 1 mixed
    ru_delta::Cdouble
    chunk::Cint
    warm_start::Cint
end
SolverOpts(; rtol = 1e-12, max_iter = 200000, mixed = false, ru_delta = 0.1, chunk = 32) =
    SolverOpts(rtol, max_iter, mixed ? 1 : 0, ru_delta, chunk, 0)

struct SolverStats
    iterations::Cint
    updates::Cint
    relres::Cdouble
    ms::Cdouble
    status::Cint
    launches::Clonglong
end

"""`K\\F` on the GPU for a symmetric positive definite K (Jacobi-CG, FP64 or mixed)."""
function gpu_solve(K::SparseMatrixCSC{Float64,Int64}, F::Vector{Float64}; kw...)
    u = zeros(length(F))
    o = Ref(SolverOpts(; kw...))
    s = Ref{SolverStats}()
    check(ccall((:adfem_csc_solve, LIB), Cint,
                (Clonglong, Ptr{Clonglong}, Ptr{Clonglong}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ref{SolverOpts},
                 Ref{SolverStats}), size(K, 1), K.colptr, K.rowval, K.nzval, F, u, o, s))
    u
end

"""A resident Poisson system: the operator's pattern, the solver's layout and its vectors stay on
the GPU between calls, so repeated solves on one mesh (an inverse problem, a parameter sweep) pay
only for the new coefficients.  `set_dirichlet!` fixes the Dirichlet DOFs and values once;
`poisson_solve!` then assembles K(κ) and F(f), imposes the Dirichlet values and solves K\\F in one
call (mixed precision by default: FP32 iterations with FP64 residual replacement)."""
mutable struct PoissonSystem
    h::Ptr{Cvoid}
    mesh::GMesh  # the system refers to the mesh: keep it alive as long as the system
    ndof::Int
    function PoissonSystem(m::GMesh)
        h = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:adfem_system_create, LIB), Cint, (Ptr{Cvoid}, Cint, Ptr{Ptr{Cvoid}}), m.h, 0, h))
        s = new(h[], m, m.ndof)
        finalizer(x -> ccall((:adfem_system_destroy, LIB), Cint, (Ptr{Cvoid},), x.h), s)
        return s
    end
end

"""Dirichlet DOFs `bd` (1-based, e.g. `bcnode(mesh)`) with values `bdval`."""
function set_dirichlet!(s::PoissonSystem, bd::Vector{Int64}, bdval::Vector{Float64} = zeros(length(bd)))
    length(bdval) == length(bd) || error("bd and bdval lengths differ")
    check(ccall((:adfem_system_set_dirichlet, LIB), Cint, (Ptr{Cvoid}, Ptr{Clonglong}, Clonglong, Ptr{Cdouble}),
                s.h, bd, length(bd), bdval))
    s
end

"""u = K(κ) \\ F(f) with the Dirichlet values imposed, κ and f at the Gauss points; returns
(u, stats).  `warm_start = true` starts from the u passed in."""
function poisson_solve!(u::Vector{Float64}, s::PoissonSystem, kappa::Vector{Float64}, f::Vector{Float64};
                        mixed::Bool = true, rtol::Real = 3e-10, max_iter::Integer = 200000, warm_start::Bool = false)
    length(u) == s.ndof || error("u must have ndof entries")
    length(kappa) == s.mesh.ngauss && length(f) == s.mesh.ngauss || error("kappa and f: one value per Gauss point")
    o = Ref(SolverOpts(rtol, max_iter, mixed ? 1 : 0, 0.1, 32, warm_start ? 1 : 0))
    st = Ref{SolverStats}()
    check(ccall((:adfem_poisson_solve, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ref{SolverOpts}, Ref{SolverStats}),
                s.h, kappa, f, u, o, st))
    u, st[]
end

end # module
