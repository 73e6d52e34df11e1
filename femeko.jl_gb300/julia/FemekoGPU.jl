#=
    FemekoGPU -- Julia bindings of libfemeko_gpu.so (GB300 / sm_103a) for Femeko's
    FEM hot path.  Drop-in replacements, taking Femeko's own `MESH` struct
    (src/mesh.jl:9-59) and returning the same types as the functions they replace:

        stiffnessMatrix(mesh, f)            src/FEM3D.jl:40-56      -> SparseMatrixCSC
        massMatrix(mesh)                    src/FEM3D.jl:466-492    -> SparseMatrixCSC
        tangentialStiffnessMatrix(mesh,H,dmu) src/FEM3D.jl:79-119   -> SparseMatrixCSC
        stiffnessMatrix2D / massMatrix2D    src/FEM2D.jl:48-161     -> SparseMatrixCSC
        quadraticStiffnessMatrix(mesh, S, mu)  src/FEM3D.jl:378-395 (S is ignored: the
                                            basis is built on the GPU)
        quadraticMassMatrix(mesh, S, F)     src/FEM3D.jl:494-561
        cg(A, b)                            IterativeSolvers.cg      -> Vector{Float64}
        newton_magnetostatics(...)          Magnetostatics/NewtonRaphson.jl:109-214

    The library is called through `ccall`, the pattern Femeko_jl_C++/Magnetostatics/run.jl:66-79
    uses for scalarPotential.  mesh.t is passed as-is (Int32, 1-based): index_base = 1,
    no copy.  Each MESH gets one device handle, cached in a WeakKeyDict and released
    by a finalizer.

    A ChainRulesCore.rrule makes `mean_Hx(mesh, mur, ...)` differentiable with respect
    to the per-element relative permeability through the GPU adjoint (fg_adjoint_dJdmu).
=#
module FemekoGPU

using SparseArrays
using LinearAlgebra

const LIB = Ref{String}(joinpath(@__DIR__, "..", "libfemeko_gpu.so"))
libpath() = LIB[]

# ---------------------------------------------------------------- C structs
struct SolveOpts
    precision::Int32
    rtol::Float64
    maxiter::Int32
    inner_rtol::Float64
    check_every::Int32
    use_graph::Int32
    spmv::Int32
    reserved_::Int32
end

struct SolveStats
    iterations::Int32
    refinements::Int32
    converged::Int32
    pad_::Int32
    relres::Float64
    ms::Float64
end

struct NewtonOpts
    precision::Int32
    maxit::Int32
    tol_update::Float64
    inner_rtol::Float64
    cg_maxiter::Int32
    line_search::Int32
    min_step::Float64
    Ms::Float64
    Hk::Float64
    check_every::Int32
    use_graph::Int32
    forcing::Int32          # 0 fixed inner_rtol, 1 Eisenstat-Walker
    picard_steps::Int32     # first iterations without the tangent term
    eta_min::Float64
    eta_max::Float64
end

struct NewtonStats
    newton_iters::Int32
    cg_iters::Int32
    converged::Int32
    trials::Int32
    update_ratio::Float64
    residual::Float64
    alpha::Float64
    energy::Float64
    ms::Float64
    setup_ms::Float64
    cg_ms::Float64
end

const FG_OK = Cint(0)
const FG_NOT_CONVERGED = Cint(1)

function check(st::Cint; allow_not_converged::Bool=false)
    if st == FG_OK || (allow_not_converged && st == FG_NOT_CONVERGED)
        return st
    end
    msg = unsafe_string(ccall((:fg_last_error, libpath()), Cstring, ()))
    error("libfemeko_gpu status $(st): $(msg)")
end

function solve_opts(; precision::Symbol=:fp64, rtol=1e-10, maxiter=1_000_000, inner_rtol=1e-5)
    o = Ref{SolveOpts}()
    ccall((:fg_solve_opts_default, libpath()), Cvoid, (Ref{SolveOpts},), o)
    d = o[]
    return SolveOpts(precision == :mixed ? 1 : 0, rtol, maxiter, inner_rtol, d.check_every, d.use_graph,
                     d.spmv, 0)
end

function newton_opts(; precision::Symbol=:mixed, tol_update=1e-8, maxit=100, inner_rtol=1e-4,
                     line_search::Symbol=:residual, Ms=1.2e6, Hk=500.0)
    o = Ref{NewtonOpts}()
    ccall((:fg_newton_opts_default, libpath()), Cvoid, (Ref{NewtonOpts},), o)
    d = o[]
    ls = line_search == :none ? 0 : line_search == :reference ? 1 : line_search == :quadratic ? 3 : 2
    return NewtonOpts(precision == :mixed ? 1 : 0, maxit, tol_update, inner_rtol, d.cg_maxiter, ls,
                      d.min_step, Ms, Hk, d.check_every, d.use_graph, d.forcing, d.picard_steps, d.eta_min,
                      d.eta_max)
end

# ---------------------------------------------------------------- mesh handle
mutable struct GPUMesh
    h::Ptr{Cvoid}
    nv::Int
    nt::Int
    nnz::Int
    colptr::Vector{Int64}      # 1-based, SparseMatrixCSC-ready
    rowval::Vector{Int32}
end

const HANDLES = WeakKeyDict{Any,GPUMesh}()

function GPUMesh(mesh; dirichlet::Union{Nothing,AbstractVector{UInt8}}=nothing)
    npe = size(mesh.t, 1)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:fg_mesh_create, libpath()), Cint,
                (Ptr{Float64}, Int64, Ptr{Int32}, Int64, Int32, Int32, Ref{Ptr{Cvoid}}),
                mesh.p, size(mesh.p, 2), mesh.t, size(mesh.t, 2), npe, 1, h))
    nnz = Ref{Int64}(0); mr = Ref{Int32}(0)
    check(ccall((:fg_mesh_nnz, libpath()), Cint, (Ptr{Cvoid}, Ref{Int64}, Ref{Int32}), h[], nnz, mr))
    colptr = zeros(Int64, size(mesh.p, 2) + 1)
    rowval = zeros(Int32, nnz[])
    check(ccall((:fg_csc_pattern, libpath()), Cint, (Ptr{Cvoid}, Ptr{Int64}, Ptr{Int32}, Int32),
                h[], colptr, rowval, 1))
    g = GPUMesh(h[], size(mesh.p, 2), size(mesh.t, 2), nnz[], colptr, rowval)
    finalizer(g) do x
        x.h != C_NULL && ccall((:fg_mesh_destroy, libpath()), Cint, (Ptr{Cvoid},), x.h)
        x.h = C_NULL
    end
    dirichlet === nothing || set_dirichlet!(g, dirichlet)
    return g
end

gpu(mesh) = get!(() -> GPUMesh(mesh), HANDLES, mesh)

function set_dirichlet!(g::GPUMesh, fixed::AbstractVector{UInt8})
    check(ccall((:fg_mesh_set_dirichlet, libpath()), Cint, (Ptr{Cvoid}, Ptr{UInt8}), g.h, fixed))
end

# CG kernel variant of one precision (:mixed or :fp64): fix one (0 = autotune again)
# or read the one the handle's solves use
precision_code(p::Symbol) = p === :mixed ? Int32(1) : Int32(0)
function set_cg_variant!(g::GPUMesh, precision::Symbol, variant::Integer)
    check(ccall((:fg_set_cg_variant, libpath()), Cint, (Ptr{Cvoid}, Int32, Int32), g.h,
                precision_code(precision), Int32(variant)))
end
function cg_variant(g::GPUMesh, precision::Symbol)
    v = Ref{Int32}(0)
    check(ccall((:fg_get_cg_variant, libpath()), Cint, (Ptr{Cvoid}, Int32, Ref{Int32}), g.h,
                precision_code(precision), v))
    return Int(v[])
end

csc(g::GPUMesh, vals::Vector{Float64}) =
    SparseMatrixCSC(g.nv, g.nv, copy(g.colptr), Int64.(g.rowval), vals)

# ---------------------------------------------------------------- assembly drop-ins
function stiffnessMatrix(mesh, f::Vector{Float64}=ones(size(mesh.t, 2)))
    g = gpu(mesh); v = zeros(g.nnz)
    check(ccall((:fg_stiffness, libpath()), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}), g.h, f, v))
    return csc(g, v)
end
stiffnessMatrix2D(mesh, mu::Vector{Float64}=ones(size(mesh.t, 2))) = stiffnessMatrix(mesh, mu)
quadraticStiffnessMatrix(mesh, S, mu::Vector{Float64}=ones(size(mesh.t, 2))) = stiffnessMatrix(mesh, mu)
quadraticStiffnessMatrix2D(mesh, mu::Vector{Float64}=ones(size(mesh.t, 2))) = stiffnessMatrix(mesh, mu)

function massMatrix(mesh; F::Vector{Float64}=ones(size(mesh.t, 2)), full_phi::Bool=false)
    g = gpu(mesh); v = zeros(g.nnz)
    check(ccall((:fg_mass, libpath()), Cint, (Ptr{Cvoid}, Ptr{Float64}, Int32, Ptr{Float64}),
                g.h, F, full_phi ? 1 : 0, v))
    return csc(g, v)
end
massMatrix2D(mesh) = massMatrix(mesh)
quadraticMassMatrix(mesh, S, F::Vector{Float64}=ones(size(mesh.t, 2))) = massMatrix(mesh; F=F)

# ---------------------------------------------------------------- Nedelec edge elements
const EDGE_HANDLES = WeakKeyDict{Any,GPUMesh}()

"""A handle over the edges of a second-order mesh (the unknowns of
Magnetostatics/nedelec3D.jl): mesh.edge2localMap[mesh.t[5:10, :]], 1-based."""
function EdgeGPUMesh(mesh)
    edges = Int32.(mesh.edge2localMap[mesh.t[5:10, :]])
    t4 = Int32.(mesh.t[1:4, :])
    ne = Int(mesh.ne)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:fg_edge_mesh_create, libpath()), Cint,
                (Ptr{Float64}, Int64, Ptr{Int32}, Ptr{Int32}, Int64, Int64, Int32, Ref{Ptr{Cvoid}}),
                mesh.p, size(mesh.p, 2), t4, edges, size(mesh.t, 2), ne, 1, h))
    nnz = Ref{Int64}(0); mr = Ref{Int32}(0)
    check(ccall((:fg_mesh_nnz, libpath()), Cint, (Ptr{Cvoid}, Ref{Int64}, Ref{Int32}), h[], nnz, mr))
    colptr = zeros(Int64, ne + 1)
    rowval = zeros(Int32, nnz[])
    check(ccall((:fg_csc_pattern, libpath()), Cint, (Ptr{Cvoid}, Ptr{Int64}, Ptr{Int32}, Int32),
                h[], colptr, rowval, 1))
    g = GPUMesh(h[], ne, size(mesh.t, 2), nnz[], colptr, rowval)
    finalizer(g) do x
        x.h != C_NULL && ccall((:fg_mesh_destroy, libpath()), Cint, (Ptr{Cvoid},), x.h)
        x.h = C_NULL
    end
    return g
end

edgegpu(mesh) = get!(() -> EdgeGPUMesh(mesh), EDGE_HANDLES, mesh)

"""nedelecLocalStiffness(mesh) -- src/FEM3D.jl:155-191 on the GPU (36 x nt)."""
function nedelecLocalStiffness(mesh)
    g = edgegpu(mesh); Ak = zeros(36, g.nt)
    check(ccall((:fg_nedelec_local_stiffness, libpath()), Cint, (Ptr{Cvoid}, Ptr{Float64}), g.h, Ak))
    return Ak
end

"""nedelecTangentialStiffness(mesh, dnu, Bfield, B) -- src/FEM3D.jl:194-271 on the GPU."""
function nedelecTangentialStiffness(mesh, dnu::Vector{Float64}, Bfield::Matrix{Float64}, B::Vector{Float64})
    g = edgegpu(mesh); v = zeros(g.nnz)
    check(ccall((:fg_nedelec_tangent, libpath()), Cint,
                (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}), g.h, dnu, Bfield, B, v))
    return csc(g, v)
end

"""nedelec_newton(mesh, Bext, curve_B, curve_nu) -- the Newton loop of
Magnetostatics/nedelec3D.jl:149-231 on the GPU, nu(B) the not-a-knot cubic through the
table (Spline1D(B, nu)); returns (u, Bfield, B, nu, steps, stats)."""
function nedelec_newton(mesh, Bext::Vector{Float64}, curve_B::Vector{Float64}, curve_nu::Vector{Float64};
                        tol=1e-4, maxAtt::Integer=100, minStep=1e-4, rtol=sqrt(eps(Float64)),
                        precision::Symbol=:mixed)
    g = edgegpu(mesh)
    nl = zeros(UInt8, g.nt); nl[mesh.InsideElements] .= 1
    u = zeros(g.nv); Bf = zeros(3, g.nt); B = zeros(g.nt); nu = zeros(g.nt); it = Ref{Int32}(0)
    o = Ref(solve_opts(precision=precision, rtol=rtol))
    s = Ref{SolveStats}()
    st = ccall((:fg_nedelec_newton, libpath()), Cint,
               (Ptr{Cvoid}, Ptr{Float64}, Ptr{UInt8}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Int32, Float64, Int32,
                Float64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ref{Int32}, Ref{SolveOpts},
                Ref{SolveStats}),
               g.h, Bext, nl, C_NULL, curve_B, curve_nu, length(curve_B), tol, maxAtt, minStep, u, Bf, B, nu, it, o, s)
    check(st; allow_not_converged=true)
    return u, Bf, B, nu, Int(it[]), s[]
end

"""quadraticConvectionMatrix(mesh, S, u, F) -- src/FEM3D.jl:563-648 on the GPU (S is
not used: the basis is built per element on the device).  u: 3 x nv velocity."""
function quadraticConvectionMatrix(mesh, S, u::Matrix{Float64}, F::Vector{Float64}=ones(size(mesh.t, 2));
                                   full_phi::Bool=false)
    g = gpu(mesh); v = zeros(g.nnz)
    check(ccall((:fg_convection, libpath()), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int32, Ptr{Float64}),
                g.h, u, F, full_phi ? 1 : 0, v))
    return csc(g, v)
end

"""quadraticConvectionMatrix2D(mesh, u) -- src/FEM2D.jl:231-319 on the GPU (u: 2 x nv)."""
function quadraticConvectionMatrix2D(mesh, u::Matrix{Float64})
    g = gpu(mesh); v = zeros(g.nnz)
    u3 = vcat(u[1:2, :], zeros(1, size(u, 2)))
    check(ccall((:fg_convection, libpath()), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int32, Ptr{Float64}),
                g.h, u3, C_NULL, 0, v))
    return csc(g, v)
end

"""quadraticMassMatrix1D(mesh, h) -- src/FEM2D.jl:394-419 on the GPU (surfaceT rows 1-3)."""
function quadraticMassMatrix1D(mesh, h::Vector{Float64}=ones(mesh.ns))
    g = gpu(mesh); v = zeros(g.nnz)
    faces = Int32.(mesh.surfaceT[1:3, :] .- 1)
    check(ccall((:fg_boundary_mass, libpath()), Cint,
                (Ptr{Cvoid}, Ptr{Int32}, Ptr{Float64}, Ptr{Float64}, Int64, Ptr{Float64}),
                g.h, faces, mesh.AE, h, size(faces, 2), v))
    return csc(g, v)
end

"""quadraticBoundaryMassMatrix(mesh, F) -- src/FEM3D.jl:300-322 on the GPU; reads the
six node rows of the P2 mesh.surfaceT (1-based) and mesh.AE."""
function quadraticBoundaryMassMatrix(mesh, F::Vector{Float64}=ones(mesh.ns))
    g = gpu(mesh); v = zeros(g.nnz)
    faces = Int32.(mesh.surfaceT[1:6, :] .- 1)
    check(ccall((:fg_boundary_mass, libpath()), Cint,
                (Ptr{Cvoid}, Ptr{Int32}, Ptr{Float64}, Ptr{Float64}, Int64, Ptr{Float64}),
                g.h, faces, mesh.AE, F, size(faces, 2), v))
    return csc(g, v)
end

"""transport_be(mesh, T0, rhoCp, conductivity, u, intakeBC; dt, nsteps) -- the time
loop of Transport/main3D.jl:155-213 (LM = M + dt (A + R + C), T = LM \\ (M T)) on the
GPU, one Jacobi-BiCGStab solve per step; returns (T, snapshots every `every` steps, stats)."""
function transport_be(mesh, T0::Vector{Float64}, rhoCp::Vector{Float64}, conductivity::Vector{Float64},
                      u::Matrix{Float64}, intakeBC::Vector{Float64}; dt=0.01, nsteps::Integer=100,
                      every::Integer=0, full_phi::Bool=true, rtol=1e-10, maxiter::Integer=10_000)
    g = gpu(mesh)
    T = copy(T0)
    snaps = zeros(g.nv, every > 0 ? nsteps ÷ every : 0)
    faces = Int32.(mesh.surfaceT[1:(size(mesh.t, 1) == 10 ? 6 : 3), :] .- 1)
    o = Ref(solve_opts(precision=:fp64, rtol=rtol, maxiter=maxiter))
    s = Ref{SolveStats}()
    st = ccall((:fg_transport_be, libpath()), Cint,
               (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Int32}, Ptr{Float64}, Ptr{Float64}, Int64,
                Float64, Int32, Int32, Ptr{Float64}, Int32, Ptr{Float64}, Ref{SolveOpts}, Ref{SolveStats}),
               g.h, rhoCp, conductivity, u, faces, mesh.AE, intakeBC, size(faces, 2), dt, nsteps,
               full_phi ? 1 : 0, T, every, isempty(snaps) ? C_NULL : snaps, o, s)
    check(st; allow_not_converged=true)
    return T, snaps, s[]
end
quadraticMassMatrix2D(mesh) = massMatrix(mesh)

function tangentialStiffnessMatrix(mesh, H_vec::Matrix{Float64}, dmu::Vector{Float64})
    g = gpu(mesh); v = zeros(g.nnz)
    check(ccall((:fg_tangent, libpath()), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                g.h, H_vec, dmu, v))
    return csc(g, v)
end

function localStiffnessMatrix(mesh, f::Vector{Float64}=ones(size(mesh.t, 2)))
    g = gpu(mesh); Ak = zeros(16, g.nt)
    check(ccall((:fg_local_stiffness, libpath()), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}), g.h, f, Ak))
    return Ak
end

# ---------------------------------------------------------------- solvers
"""cg(A, b; reltol, maxiter, precision) -- Jacobi-PCG on a symmetric SparseMatrixCSC."""
function cg(A::SparseMatrixCSC{Float64,Int64}, b::Vector{Float64}; reltol=sqrt(eps(Float64)),
            maxiter=size(A, 2), precision::Symbol=:fp64, x0=zeros(length(b)))
    x = copy(x0)
    o = Ref(solve_opts(precision=precision, rtol=reltol, maxiter=maxiter))
    s = Ref{SolveStats}()
    st = ccall((:fg_cg_csc, libpath()), Cint,
               (Int64, Ptr{Int64}, Ptr{Int64}, Ptr{Float64}, Int32, Ptr{Float64}, Ptr{Float64},
                Ref{SolveOpts}, Ref{SolveStats}),
               size(A, 1), A.colptr, A.rowval, A.nzval, 1, b, x, o, s)
    check(st; allow_not_converged=true)
    return x
end

"""lagrange(mesh) -- the Lagrange-multiplier row of src/FEM3D.jl:274-281."""
function lagrange(mesh)
    g = gpu(mesh)
    C = zeros(g.nv)
    check(ccall((:fg_lagrange, libpath()), Cint, (Ptr{Cvoid}, Ptr{Float64}), g.h, C))
    return C
end

"""BoundaryIntegral(mesh, F, shell_id) -- Neumann right-hand side of src/FEM3D.jl:284-297
(mesh.surfaceT is 4 x ns, 1-based, boundary id in row 4)."""
function BoundaryIntegral(mesh, F::Vector{Float64}, shell_id)
    g = gpu(mesh)
    RHS = zeros(g.nv)
    ids = Int32.(collect(shell_id))
    check(ccall((:fg_boundary_integral, libpath()), Cint,
                (Ptr{Cvoid}, Ptr{Int32}, Int64, Int32, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Int32}, Int32,
                 Ptr{Float64}),
                g.h, Int32.(mesh.surfaceT), size(mesh.surfaceT, 2), 1, mesh.normal, mesh.AE, F, ids, length(ids),
                RHS))
    return RHS
end

"""magnetostaticField(mesh, M, inside; precision=:fp64, rtol=1e-10) -- the demagnetising
field on the nodes of Micromagnetics/LL.jl:162-211 (M is 3 x nv, inside an nt UInt8
mask of the magnetic body).  The stiffness operator stays on the device between
calls, as the reference's A between Landau-Lifshitz steps."""
function magnetostaticField(mesh, M::Matrix{Float64}, inside::Vector{UInt8}; precision::Symbol=:fp64, rtol=1e-10)
    g = gpu(mesh)
    Hn = zeros(3, g.nv)
    o = Ref(solve_opts(precision=precision, rtol=rtol))
    s = Ref{SolveStats}()
    st = ccall((:fg_demag_field, libpath()), Cint,
               (Ptr{Cvoid}, Ptr{UInt8}, Ptr{Float64}, Ref{SolveOpts}, Ptr{Float64}, Ptr{Float64}, Ref{SolveStats}),
               g.h, inside, M, o, Hn, C_NULL, s)
    check(st; allow_not_converged=true)
    return Hn
end

"""heat_be(mesh, T, kappa, fixed; rho_c=1.0, dt=1e-3, nsteps=100, every=10, precision=:mixed)
-- the backward-Euler loop of Heat/heat3D.jl:83-89 with T = 0 on the `fixed` nodes.
Returns (T after nsteps, snapshots nv x (nsteps ÷ every), stats)."""
function heat_be(mesh, T0::Vector{Float64}, kappa::Vector{Float64}, fixed::Vector{UInt8}; rho_c=1.0, dt=1e-3,
                 nsteps::Integer=100, every::Integer=10, precision::Symbol=:mixed, rtol=1e-10)
    g = gpu(mesh)
    set_dirichlet!(g, fixed)
    T = copy(T0)
    snaps = zeros(g.nv, every > 0 ? nsteps ÷ every : 0)
    o = Ref(solve_opts(precision=precision, rtol=rtol))
    s = Ref{SolveStats}()
    st = ccall((:fg_heat_be, libpath()), Cint,
               (Ptr{Cvoid}, Ptr{Float64}, Float64, Float64, Int32, Ptr{Float64}, Int32, Ptr{Float64},
                Ref{SolveOpts}, Ref{SolveStats}),
               g.h, kappa, rho_c, dt, nsteps, T, every, isempty(snaps) ? C_NULL : snaps, o, s)
    check(st; allow_not_converged=true)
    return T, snaps, s[]
end

"""magnetostatics_sweep(mesh, mu, H0, fixed) -- potentials for every applied field
(columns of H0, 3 x nfield, nfield <= 256) of the linear problem
Magnetostatics/magneticField.jl:89-132, solved together; returns U (nv x nfield)."""
function magnetostatics_sweep(mesh, mu::Vector{Float64}, H0::Matrix{Float64}, fixed::Vector{UInt8}; rtol=1e-10)
    g = gpu(mesh)
    set_dirichlet!(g, fixed)
    U = zeros(g.nv, size(H0, 2))
    o = Ref(solve_opts(precision=:mixed, rtol=rtol))
    s = Ref{SolveStats}()
    st = ccall((:fg_magnetostatics_sweep, libpath()), Cint,
               (Ptr{Cvoid}, Ptr{Float64}, Int32, Ptr{Float64}, Ref{SolveOpts}, Ptr{Float64}, Ref{SolveStats}),
               g.h, mu, size(H0, 2), H0, o, U, s)
    check(st; allow_not_converged=true)
    return U
end

"""Newton-Raphson magnetostatics (Magnetostatics/NewtonRaphson.jl:109-214) with
Dirichlet nodes `fixed` holding u0.  Returns (u, Hfield 3 x nt, mu, stats)."""
function newton_magnetostatics(mesh, fixed::Vector{UInt8}, nl::Vector{UInt8}, mu_lin::Vector{Float64},
                               u0::Vector{Float64}; kw...)
    g = gpu(mesh)
    set_dirichlet!(g, fixed)
    u = zeros(g.nv); H = zeros(3, g.nt); mu = zeros(g.nt)
    o = Ref(newton_opts(; kw...))
    s = Ref{NewtonStats}()
    st = ccall((:fg_newton_magnetostatics, libpath()), Cint,
               (Ptr{Cvoid}, Ptr{UInt8}, Ptr{Float64}, Ptr{Float64}, Ref{NewtonOpts}, Ptr{Float64},
                Ptr{Float64}, Ptr{Float64}, Ref{NewtonStats}),
               g.h, nl, mu_lin, u0, o, u, H, mu, s)
    check(st; allow_not_converged=true)
    return u, H, mu, s[]
end

# ---------------------------------------------------------------- mesh files
# The arrays Femeko's `Mesh(...; saveMesh=true)` writes with save2file
# (src/mesh.jl:233-242, src/geometry.jl:237-245: one line per row, entries joined by
# " , "), read back as the fields of a MESH (1-based, as Julia holds them), so that a
# mesh saved on a machine with Gmsh can be solved on the GPU elsewhere.
function read_save2file(path::AbstractString, ::Type{T}=Float64) where {T}
    rows = [parse.(T, strip.(split(l, ","))) for l in eachline(path) if !isempty(strip(l))]
    isempty(rows) && return T[]
    all(length(r) == length(rows[1]) for r in rows) || error("$path: rows of different lengths")
    length(rows[1]) == 1 && return [r[1] for r in rows]
    return permutedims(reduce(hcat, rows))
end

function load_saved_mesh(folder::AbstractString)
    rd(name, T=Float64) = read_save2file(joinpath(folder, name * ".txt"), T)
    asmat(a) = a isa AbstractVector ? reshape(a, :, 1) : a
    return (t = Int32.(asmat(rd("t", Int64))), p = asmat(rd("p")), surfaceT = Int32.(asmat(rd("surfaceT", Int64))),
            InsideNodes = Int32.(rd("InsideNodes", Int64)), InsideElements = Int32.(rd("InsideElements", Int64)),
            VE = rd("VE"), AE = rd("AE"), normal = asmat(rd("normal")))
end

# ---------------------------------------------------------------- differentiation
struct AdjointStats
    forward_iters::Int32
    adjoint_iters::Int32
    newton_iters::Int32
    converged::Int32
    forward_ms::Float64
    adjoint_ms::Float64
end

"""mean_Hx(mesh, mur, fixed, u0, target; nl=nothing, precision=:mixed, rtol=1e-12) --
volume-weighted mean H_x over the target elements (Magnetostatics/NewtonRaphson.jl:234-240)
of the magnetostatic solution with relative permeability mur, and its gradient dJ/dmur
from the GPU adjoint.  nl === nothing: linear problem; else the Newton problem with
Froehlich elements nl[k] != 0."""
function mean_Hx(mesh, mur::Vector{Float64}, fixed::Vector{UInt8}, u0::Vector{Float64}, target::Vector{UInt8};
                 nl::Union{Nothing,Vector{UInt8}}=nothing, precision::Symbol=:mixed, rtol=1e-12)
    g = gpu(mesh)
    set_dirichlet!(g, fixed)
    J = Ref{Float64}(0.0)
    grad = zeros(g.nt)
    o = Ref(newton_opts(precision=precision))
    s = Ref{AdjointStats}()
    nlp = nl === nothing ? Ptr{UInt8}(C_NULL) : pointer(nl)
    GC.@preserve nl begin
        check(ccall((:fg_adjoint_dJdmu, libpath()), Cint,
                    (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{UInt8}, Ptr{UInt8}, Ref{NewtonOpts}, Float64,
                     Ref{Float64}, Ptr{Float64}, Ptr{Float64}, Ref{AdjointStats}),
                    g.h, mur, u0, target, nlp, o, rtol, J, grad, C_NULL, s); allow_not_converged=true)
    end
    return J[], grad
end

# ChainRulesCore is an optional dependency: the rule is defined when it is loaded.
function __init__()
    if Base.find_package("ChainRulesCore") !== nothing
        @eval begin
            import ChainRulesCore
            # keywords (nl for the Newton problem, precision, rtol) pass through to the
            # adjoint: with nl given, the gradient comes through the converged Newton Jacobian
            function ChainRulesCore.rrule(::typeof(mean_Hx_value), mesh, mur, fixed, u0, target; kw...)
                J, grad = mean_Hx(mesh, mur, fixed, u0, target; kw...)
                pullback(dJ) = (ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent(), dJ .* grad,
                                ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent())
                return J, pullback
            end
        end
    end
end

"""The scalar J alone (the function the rrule differentiates); keywords as mean_Hx
(nl = Froehlich mask for the nonlinear problem)."""
mean_Hx_value(mesh, mur, fixed, u0, target; kw...) = mean_Hx(mesh, mur, fixed, u0, target; kw...)[1]

end # module
