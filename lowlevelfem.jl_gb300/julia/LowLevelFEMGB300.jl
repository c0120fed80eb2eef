# LowLevelFEMGB300 — drop-in GPU methods for LowLevelFEM.jl's assembly/solve
# hot path, calling libllfem_gb300.so through ccall.
#
# Usage (after `using LowLevelFEM`):
#     include("LowLevelFEMGB300.jl"); using .LowLevelFEMGB300
#     K = LowLevelFEMGB300.stiffnessMatrix(problem)      # same result type as
#     u = LowLevelFEMGB300.solveDisplacement(problem; load=[ld], support=[bc])
#
# Mesh data and quadrature/shape tables are read from gmsh exactly as
# src/linear.jl:232-243 reads them, so the GPU integrates with gmsh's own
# rule and node ordering (llf_tables_upload).  Every non-zero status of the
# library becomes `error(msg)`, the reference's error behaviour.
module LowLevelFEMGB300

using LowLevelFEM
using LowLevelFEM: gmsh, SystemMatrix, VectorField, ScalarField, BoundaryCondition, LoadCondition
using SparseArrays

const LIB = get(ENV, "LLFEM_GB300_LIB", joinpath(@__DIR__, "..", "libllfem_gb300.so"))

const CTX = Ref{Ptr{Cvoid}}(C_NULL)

function ctx()
    if CTX[] == C_NULL
        r = Ref{Ptr{Cvoid}}(C_NULL)
        st = ccall((:llf_ctx_create, LIB), Cint, (Cint, Ref{Ptr{Cvoid}}), 0, r)
        st == 0 || error("llf_ctx_create failed with status $st (no CUDA device?)")
        CTX[] = r[]
    end
    return CTX[]
end

function check(st::Cint)
    st == 0 && return nothing
    msg = unsafe_string(ccall((:llf_last_error, LIB), Cstring, (Ptr{Cvoid},), ctx()))
    error(msg)
end

const FAMILY = Dict(1 => 1, 2 => 2, 3 => 3, 4 => 4, 5 => 5, 8 => 1, 9 => 2, 10 => 3, 11 => 4, 12 => 5,
                    26 => 1, 21 => 2, 36 => 3, 29 => 4, 92 => 5, 27 => 1, 23 => 2, 37 => 3, 35 => 4, 93 => 5)

ptype(p) = p.type == :Solid ? 0 : p.type == :PlaneStress ? 1 : p.type == :PlaneStrain ? 2 :
           p.type == :HeatConduction ? 3 : p.type == :PlaneHeatConduction ? 4 :
           p.type == :VectorField ? (p.dim == 3 ? 0 : 2) : p.type == :ScalarField ? (p.dim == 3 ? 3 : 4) :
           error("LowLevelFEMGB300: problem type $(p.type) is not on the accelerated path")

# ---------------------------------------------------------------- mesh
struct DevMesh
    h::Ptr{Cvoid}
    nel::Int
    npe::Int
    etype::Int
end

const MESHES = IdDict{Any,DevMesh}()
const PATTERNS = IdDict{Any,Dict{Int,Ptr{Cvoid}}}()

function device_mesh(problem)
    haskey(MESHES, problem) && return MESHES[problem]
    gmsh.model.setCurrent(problem.name)
    nodeTags, coord, _ = gmsh.model.mesh.getNodes()
    non = length(nodeTags)
    xyz = zeros(3non)
    for (i, t) in enumerate(nodeTags)
        xyz[3t-2:3t] .= coord[3i-2:3i]
    end
    conn = Int64[]; emat = Int32[]; et0 = 0; npe = 0
    for (imat, mat) in enumerate(problem.material)
        for (edim, etag) in gmsh.model.getEntitiesForPhysicalName(mat.phName)
            edim == problem.dim || continue
            types, _, ntags = gmsh.model.mesh.getElements(edim, etag)
            for (k, et) in enumerate(types)
                et0 == 0 && (et0 = et)
                et == et0 || error("LowLevelFEMGB300: one element type per problem")
                _, _, _, npe, _, _ = gmsh.model.mesh.getElementProperties(et)
                append!(conn, ntags[k])
                append!(emat, fill(Int32(imat - 1), length(ntags[k]) ÷ npe))
            end
        end
    end
    _, _, order, npe, _, _ = gmsh.model.mesh.getElementProperties(et0)
    nel = length(conn) ÷ npe
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:llf_mesh_upload, LIB), Cint,
                (Ptr{Cvoid}, Cint, Int64, Ptr{Float64}, Int64, Cint, Ptr{Int64}, Cint, Cint, Ref{Ptr{Cvoid}}),
                ctx(), problem.dim, non, xyz, nel, npe, conn, FAMILY[et0], order, h))
    # gmsh's own quadrature and shape tables (src/linear.jl:235-239)
    ip, w = gmsh.model.mesh.getIntegrationPoints(et0, "Gauss" * string(2order + 1))
    _, N, _ = gmsh.model.mesh.getBasisFunctions(et0, ip, "Lagrange")
    _, dN, _ = gmsh.model.mesh.getBasisFunctions(et0, ip, "GradLagrange")
    check(ccall((:llf_tables_upload, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                ctx(), h[], length(w), w, N, dN))
    if length(problem.material) > 1
        check(ccall((:llf_mesh_set_materials, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Int32}), ctx(), h[], emat))
    end
    return MESHES[problem] = DevMesh(h[], nel, npe, et0)
end

function pattern(problem, pdim::Int=problem.pdim)
    m = device_mesh(problem)
    d = get!(PATTERNS, problem, Dict{Int,Ptr{Cvoid}}())
    haskey(d, pdim) && return d[pdim]
    nnz = Ref{Int64}(0); h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:llf_pattern_build, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ref{Int64}, Ref{Ptr{Cvoid}}),
                ctx(), m.h, pdim, nnz, h))
    return d[pdim] = h[]
end

# Matrices assembled here stay on the device until the SparseMatrixCSC that
# was returned for them is collected: solveField / FDM use the device copy
# instead of uploading the host arrays again, as long as those arrays still
# hold what was returned (same arrays, same sum of values; a caller that
# edits K.A in place gets a fresh upload).
struct DevCopy
    h::Ptr{Cvoid}
    pat::Ptr{Cvoid}
    nnz::Int
    checksum::Float64
end
const DEVICE = WeakKeyDict{SparseMatrixCSC{Float64,Int64},DevCopy}()

function keep_on_device!(A::SparseMatrixCSC{Float64,Int64}, hm::Ptr{Cvoid}, pat::Ptr{Cvoid})
    DEVICE[A] = DevCopy(hm, pat, nnz(A), sum(nonzeros(A)))
    finalizer(A) do _
        ccall((:llf_matrix_destroy, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), ctx(), hm)
    end
    return A
end

# The device matrix of K if K.A is unchanged since it was returned, else
# nothing.
function device_copy(K::SystemMatrix, pat::Ptr{Cvoid})
    d = get(DEVICE, K.A, nothing)
    d === nothing && return nothing
    (d.pat == pat && d.nnz == nnz(K.A) && d.checksum == sum(nonzeros(K.A))) || return nothing
    return d.h
end

# device matrix -> SparseMatrixCSC{Float64,Int64} (two-phase copy); the
# device matrix is kept for the solves (keep_on_device!)
function fetch(hm::Ptr{Cvoid}, n::Int, pat::Ptr{Cvoid})
    nnz = Ref{Int64}(0)
    check(ccall((:llf_matrix_nnz, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ref{Int64}), ctx(), hm, nnz))
    colptr = Vector{Int64}(undef, n + 1); rowval = Vector{Int64}(undef, nnz[]); nzval = Vector{Float64}(undef, nnz[])
    check(ccall((:llf_matrix_copy_csc, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Int64}, Ptr{Int64}, Ptr{Float64}),
                ctx(), hm, colptr, rowval, nzval))
    return keep_on_device!(SparseMatrixCSC(n, n, colptr, rowval, nzval), hm, pat)
end

# ---------------------------------------------------------------- assembly
# stiffnessMatrix: assembled on the device, the stored CSC copied into the
# SparseMatrixCSC arrays, the device matrix kept for the solves.  With
# keep_device=false: one call straight into the host arrays
# (llf_assemble_stiffness_csc, the device work hidden behind the copy).
function stiffnessMatrix(problem; elements=[], forceOneThread=true, keep_device=true)
    m = device_mesh(problem); pat = pattern(problem)
    E = Float64[mat.E for mat in problem.material]; ν = Float64[mat.ν for mat in problem.material]
    n = problem.pdim * problem.non
    if keep_device
        h = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:llf_assemble_stiffness, LIB), Cint,
                    (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Float64}, Ptr{Float64}, Cint, Float64, Cint,
                     Ref{Ptr{Cvoid}}),
                    ctx(), m.h, pat, ptype(problem), E, ν, length(E), problem.thickness, 0, h))
        return SystemMatrix(fetch(h[], n, pat), problem)
    end
    snnz = Ref{Int64}(0); ndof = Ref{Int64}(0); pd = Ref{Cint}(0)
    ccall((:llf_pattern_info, LIB), Cint, (Ptr{Cvoid}, Ref{Int64}, Ref{Int64}, Ref{Cint}), pat, ndof, snnz, pd)
    colptr = Vector{Int64}(undef, n + 1); rowval = Vector{Int64}(undef, snnz[]); nzval = Vector{Float64}(undef, snnz[])
    nnz = Ref{Int64}(0)
    check(ccall((:llf_assemble_stiffness_csc, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Float64}, Ptr{Float64}, Cint, Float64, Cint, Int64,
                 Ptr{Int64}, Ptr{Int64}, Ptr{Float64}, Ref{Int64}),
                ctx(), m.h, pat, ptype(problem), E, ν, length(E), problem.thickness, 0, snnz[],
                colptr, rowval, nzval, nnz))
    resize!(rowval, nnz[]); resize!(nzval, nnz[])
    return SystemMatrix(SparseMatrixCSC(n, n, colptr, rowval, nzval), problem)
end

function massMatrix(problem; lumped=true)
    m = device_mesh(problem); pat = pattern(problem)
    ρ = Float64[mat.ρ for mat in problem.material]
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:llf_assemble_mass, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Float64}, Cint, Float64, Cint, Cint, Ref{Ptr{Cvoid}}),
                ctx(), m.h, pat, ptype(problem), ρ, length(ρ), problem.thickness, lumped ? 1 : 0, 0, h))
    return SystemMatrix(fetch(h[], problem.pdim * problem.non, pat), problem)
end

function heatConductionMatrix(problem; elements=[])
    m = device_mesh(problem); pat = pattern(problem, 1)
    k = Float64[mat.k for mat in problem.material]
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:llf_assemble_heat, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Float64}, Cint, Float64, Cint, Ref{Ptr{Cvoid}}),
                ctx(), m.h, pat, ptype(problem), k, length(k), problem.thickness, 0, h))
    return SystemMatrix(fetch(h[], problem.non, pat), problem)
end

function heatCapacityMatrix(problem; elements=[], lumped=false)
    m = device_mesh(problem); pat = pattern(problem, 1)
    cρ = Float64[mat.c * mat.ρ for mat in problem.material]
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:llf_assemble_mass, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Float64}, Cint, Float64, Cint, Cint, Ref{Ptr{Cvoid}}),
                ctx(), m.h, pat, ptype(problem), cρ, length(cρ), 1.0, lumped ? 1 : 0, 0, h))
    return SystemMatrix(fetch(h[], problem.non, pat), problem)
end

# Boundary elements of the conditions' physical groups, in condition order,
# with gmsh's own tables for their element type (src/linear.jl:2896-2907).
function boundary_mesh(problem, conds)
    gmsh.model.setCurrent(problem.name)
    nodeTags, coord, _ = gmsh.model.mesh.getNodes()
    non = length(nodeTags)
    xyz = zeros(3non)
    for (i, t) in enumerate(nodeTags)
        xyz[3t-2:3t] .= coord[3i-2:3i]
    end
    conn = Int64[]; owner = Int[]; et0 = 0; npe = 0
    for (c, bc) in enumerate(conds)
        for (edim, etag) in gmsh.model.getEntitiesForPhysicalName(bc.phName)
            edim == problem.dim - 1 || error("LowLevelFEMGB300: supports on groups of dimension $(problem.dim - 1) only")
            types, _, ntags = gmsh.model.mesh.getElements(edim, etag)
            for (k, et) in enumerate(types)
                et0 == 0 && (et0 = et)
                et == et0 || error("LowLevelFEMGB300: one boundary element type per call")
                _, _, _, npe, _, _ = gmsh.model.mesh.getElementProperties(et)
                append!(conn, ntags[k]); append!(owner, fill(c, length(ntags[k]) ÷ npe))
            end
        end
    end
    _, _, order, npe, _, _ = gmsh.model.mesh.getElementProperties(et0)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:llf_mesh_upload, LIB), Cint,
                (Ptr{Cvoid}, Cint, Int64, Ptr{Float64}, Int64, Cint, Ptr{Int64}, Cint, Cint, Ref{Ptr{Cvoid}}),
                ctx(), problem.dim, non, xyz, length(owner), npe, conn, FAMILY[et0], order, h))
    ip, w = gmsh.model.mesh.getIntegrationPoints(et0, "Gauss" * string(2order + 1))
    _, N, _ = gmsh.model.mesh.getBasisFunctions(et0, ip, "Lagrange")
    _, dN, _ = gmsh.model.mesh.getBasisFunctions(et0, ip, "GradLagrange")
    check(ccall((:llf_tables_upload, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                ctx(), h[], length(w), w, N, dN))
    return h[], owner
end

# elasticSupportMatrix (src/linear.jl:2859-3005) with constant kx, ky, kz (or
# h for heat convection, src/heat.jl:562-567), one value set per condition.
function support_matrix(problem, conds, keys)
    pat = pattern(problem)
    bm, owner = boundary_mesh(problem, conds)
    pd = problem.pdim
    ke = zeros(pd * length(owner))
    for (e, c) in enumerate(owner), i in 1:pd
        v = get(conds[c].values, keys[i], 0)
        v isa Function && error("LowLevelFEMGB300: function-valued supports go through the Python mirror")
        ke[pd*(e-1)+i] = v
    end
    h = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:llf_assemble_support, LIB), Cint,
               (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Float64, Ref{Ptr{Cvoid}}),
               ctx(), pat, bm, ke, C_NULL, problem.dim == 2 ? problem.thickness : 1.0, h)
    ccall((:llf_mesh_destroy, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), ctx(), bm)
    check(st)
    return SystemMatrix(fetch(h[], pd * problem.non, pat), problem)
end

elasticSupportMatrix(problem, elSupports) = support_matrix(problem, elSupports, (:kx, :ky, :kz))
heatConvectionMatrix(problem, heatConvection) = support_matrix(problem, heatConvection, (:h,))

# externalTangentFollower (src/nonlinear.jl:3053-3258) with constant fx, fy,
# fz per load; F nodal (9 per node) after elementsToNodes.
function externalTangentFollower(problem, loads; F)
    pat = pattern(problem)
    Fn = vec(LowLevelFEM.elementsToNodes(F).a[:, 1])
    bm, owner = boundary_mesh(problem, loads)
    te = zeros(3 * length(owner))
    for (e, c) in enumerate(owner), (i, k) in enumerate((:fx, :fy, :fz))
        v = get(loads[c].values, k, 0)
        v isa Number || error("LowLevelFEMGB300: function-valued follower loads go through the Python mirror")
        te[3*(e-1)+i] = v
    end
    h = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:llf_follower_tangent, LIB), Cint,
               (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ref{Ptr{Cvoid}}),
               ctx(), pat, bm, Fn, te, C_NULL, h)
    ccall((:llf_mesh_destroy, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), ctx(), bm)
    check(st)
    return SystemMatrix(fetch(h[], 3problem.non, pat), problem)
end

# energy: pass :NeoHookeCompressible or :StVenantKirchhoff; params = (μ=.., λ=..)
law(energy) = energy === :NeoHookeCompressible ? 1 : energy === :StVenantKirchhoff ? 2 :
              error("LowLevelFEMGB300: built-in laws are :NeoHookeCompressible and :StVenantKirchhoff")
lawparams(p) = Float64[p.μ, p.λ]

elementwise(T) = reduce(vcat, [vec(T.A[i][:, 1]) for i in eachindex(T.A)])

function materialTangentMatrix(problem; F, C=nothing, energy=nothing, params=nothing)
    @assert xor(C !== nothing, energy !== nothing)
    m = device_mesh(problem); pat = pattern(problem)
    Fe = elementwise(LowLevelFEM.nodesToElements(F))
    lw, prm = C === nothing ? (law(energy), lawparams(params)) : (0, vec(Float64.(C)))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:llf_tl_material_tangent, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Cint, Ptr{Float64}, Cint, Ref{Ptr{Cvoid}}),
                ctx(), m.h, pat, Fe, lw, prm, length(prm), h))
    return SystemMatrix(fetch(h[], 3problem.non, pat), problem)
end

function initialStressMatrix(problem; S=nothing, energy=nothing, params=nothing, C=nothing)
    @assert xor(S !== nothing, energy !== nothing)
    m = device_mesh(problem); pat = pattern(problem)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    if S !== nothing
        Se = elementwise(LowLevelFEM.nodesToElements(S))
        check(ccall((:llf_tl_initial_stress, LIB), Cint,
                    (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Cint, Ptr{Float64}, Cint, Ref{Ptr{Cvoid}}),
                    ctx(), m.h, pat, Se, C_NULL, 0, C_NULL, 0, h))
    else
        Ce = elementwise(LowLevelFEM.nodesToElements(C)); prm = lawparams(params)
        check(ccall((:llf_tl_initial_stress, LIB), Cint,
                    (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Cint, Ptr{Float64}, Cint, Ref{Ptr{Cvoid}}),
                    ctx(), m.h, pat, C_NULL, Ce, law(energy), prm, length(prm), h))
    end
    return SystemMatrix(fetch(h[], 3problem.non, pat), problem)
end

function internalForceVector(problem; P=nothing, F=nothing, energy=nothing, params=nothing)
    @assert xor(P !== nothing, energy !== nothing)
    m = device_mesh(problem)
    f = zeros(3problem.non)
    if P !== nothing
        Pe = elementwise(LowLevelFEM.nodesToElements(P))
        check(ccall((:llf_tl_internal_force, LIB), Cint,
                    (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Cint, Ptr{Float64}, Cint, Ptr{Float64}),
                    ctx(), m.h, Pe, C_NULL, 0, C_NULL, 0, f))
    else
        Fe = elementwise(LowLevelFEM.nodesToElements(F)); prm = lawparams(params)
        check(ccall((:llf_tl_internal_force, LIB), Cint,
                    (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Cint, Ptr{Float64}, Cint, Ptr{Float64}),
                    ctx(), m.h, C_NULL, Fe, law(energy), prm, length(prm), f))
    end
    return VectorField([], reshape(f, :, 1), [0.0], [], 1, :v3D, problem)
end

# ---------------------------------------------------------------- solve
# Condensed Dirichlet solve by PCG on the device (the iterative branch of
# src/linear.jl:3827-3833).  K is re-uploaded from its CSC arrays through the
# pattern of the problem; the prescribed values come from
# applyBoundaryConditions!.
function solveField(K::SystemMatrix, f; support=BoundaryCondition[], iterative=false,
                    reltol=sqrt(eps()), maxiter=K.model.non * K.model.dim, preconditioner=nothing, ordering=true)
    problem = K.model
    n = problem.pdim * problem.non
    u = copy(f); fill!(u.a, 0.0)
    LowLevelFEM.applyBoundaryConditions!(u, support)
    fixed = zeros(UInt8, n)
    fixed[LowLevelFEM.constrainedDoFs(problem, support)] .= 1
    hm, owned = device_matrix(K)
    x = vec(u.a[:, 1]); its = Ref{Int64}(0); rr = Ref{Float64}(0.0)
    prec = iterative ? (preconditioner === nothing ? 0 : 1) : 2
    tol = iterative ? reltol : 1e-13
    st = ccall((:llf_pcg, LIB), Cint,
               (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{UInt8}, Cint, Float64, Int64, Ref{Int64}, Ref{Float64}),
               ctx(), hm, vec(f.a[:, 1]), x, fixed, prec, tol, iterative ? maxiter : 20n, its, rr)
    owned && ccall((:llf_matrix_destroy, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), ctx(), hm)
    (st == 0 || (iterative && st == -4)) || check(st)
    u.a[:, 1] .= x
    return u
end

solveDisplacement(K::SystemMatrix, f; kw...) = solveField(K, f; kw...)

function solveDisplacement(problem; load=LoadCondition[], support=BoundaryCondition[], kw...)
    K = stiffnessMatrix(problem)
    f = LowLevelFEM.loadVector(problem, load)
    return solveField(K, f; support=support, kw...)
end

function solveTemperature(problem; heatFlux=LoadCondition[], temperatureConstraint=BoundaryCondition[], kw...)
    K = heatConductionMatrix(problem)
    q = LowLevelFEM.heatFluxVector(problem, heatFlux)
    return solveField(K, q; support=temperatureConstraint, kw...)
end

# FDM (src/heat.jl:1466-1616): the whole theta-method loop on the device.
# K and C re-enter through the problem's pattern; a lumped C (diagonal only)
# keeps its diagonal in the structural values.
function FDM(K::SystemMatrix, C::SystemMatrix, q::ScalarField, bc, TT0::ScalarField, n::Int, Δt::Float64; ϑ=0.5)
    problem = K.model
    nd = problem.pdim * problem.non
    T = zeros(nd, n)
    T[:, 1] .= TT0.a[:, 1]
    TT = ScalarField([], T, collect(0:Δt:(n-1)*Δt), [], n, :scalar, problem)
    LowLevelFEM.applyBoundaryConditions!(TT, bc)
    fixed = zeros(UInt8, nd)
    fixed[LowLevelFEM.constrainedDoFs(problem, bc)] .= 1
    (hK, oK) = device_matrix(K); (hC, oC) = device_matrix(C)
    qa = Matrix{Float64}(q.a)
    its = Ref{Int64}(0)
    st = ccall((:llf_heat_fdm, LIB), Cint,
               (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Cint, Ptr{Float64}, Ptr{UInt8}, Int64, Float64,
                Float64, Cint, Float64, Int64, Ref{Int64}),
               ctx(), hK, hC, qa, size(qa, 2), TT.a, fixed, n, Δt, ϑ, 2, 1e-13, 20nd, its)
    oK && ccall((:llf_matrix_destroy, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), ctx(), hK)
    oC && ccall((:llf_matrix_destroy, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), ctx(), hC)
    check(st)
    return TT
end

# The device matrix of a SystemMatrix: the one kept when it was assembled
# here (and is unchanged), else an upload.  Returns (handle, owned): an
# owned handle is the caller's to destroy.
function device_matrix(K::SystemMatrix)
    pat = pattern(K.model, size(K.A, 1) == K.model.non ? 1 : K.model.pdim)
    h = device_copy(K, pat)
    h === nothing || return (h, false)
    return (upload(K, pat), true)
end

# A host SystemMatrix re-enters the device through the structural pattern of
# its problem: per column, the stored rows (a sorted subset of the
# structural rows, or the same set) are merged into the structural rows in
# one pass, and the values go up as structural values.
const STRUCT_ROWS = IdDict{Ptr{Cvoid},Tuple{Vector{Int64},Vector{Int64}}}()

function upload(K::SystemMatrix, pat::Ptr{Cvoid})
    colptr, rowval = get!(STRUCT_ROWS, pat) do
        nnz = Ref{Int64}(0); ndof = Ref{Int64}(0); pd = Ref{Cint}(0)
        ccall((:llf_pattern_info, LIB), Cint, (Ptr{Cvoid}, Ref{Int64}, Ref{Int64}, Ref{Cint}), pat, ndof, nnz, pd)
        c = Vector{Int64}(undef, ndof[] + 1); r = Vector{Int64}(undef, nnz[])
        check(ccall((:llf_pattern_copy, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Int64}, Ptr{Int64}), ctx(), pat, c, r))
        (c, r)
    end
    A = K.A
    size(A, 2) == length(colptr) - 1 || error("LowLevelFEMGB300: matrix size does not match the problem's pattern")
    vals = zeros(length(rowval))
    Ar, Av, Ac = rowvals(A), nonzeros(A), SparseArrays.getcolptr(A)
    @inbounds for j in 1:size(A, 2)
        q = colptr[j]; qe = colptr[j+1]
        for p in Ac[j]:(Ac[j+1]-1)
            r = Ar[p]
            while q < qe && rowval[q] < r
                q += 1
            end
            (q < qe && rowval[q] == r) ||
                error("LowLevelFEMGB300: entry ($r, $j) is outside the problem's structural pattern")
            vals[q] = Av[p]
        end
    end
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:llf_matrix_from_structural, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Ref{Ptr{Cvoid}}),
                ctx(), pat, vals, h))
    return h[]
end

end # module
