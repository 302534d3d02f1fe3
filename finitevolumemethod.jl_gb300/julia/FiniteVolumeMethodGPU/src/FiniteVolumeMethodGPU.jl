"""
    FiniteVolumeMethodGPU

Julia binding of libfvmgpu.so (include/fvm_gpu.h).  A problem is built with
FiniteVolumeMethod.jl exactly as before (`FVMGeometry`, `BoundaryConditions`,
`InternalConditions`, `FVMProblem`, the templates); `GPUProblem(prob)` flattens it once
(triangles, boundary edges, the merged `Conditions` dictionaries, closures sampled at the
dual-edge midpoints and boundary quarter points) and every `fvm_eqs!` / `solve` then runs on
the GPU through `ccall`.  Closures must be functions of (x, y), or polynomials of degree <= 2
in u with (x, y) coefficients; other forms raise `ArgumentError`.  `GPUSystem(sys)` does the
same for an `FVMSystem`, whose sources and conditions may be polynomials of total degree <= 3
in the component tuple and whose fluxes may couple the components linearly.
Indices passed to the C ABI are 0-based.

Also bound: the four templates (`GPUTemplate`: `DiffusionEquation`,
`LinearReactionDiffusionEquation`, `PoissonsEquation`, `MeanExitTimeProblem`, with time stepping
or the steady Krylov solve), batched instances (`GPUBatch`), the discrete adjoint of the time
templates (`GPUAdjoint`, with a `ChainRulesCore.rrule` for `adjoint_solve`) and device point
location / interpolation (`locate`, `interpolate`).  With OrdinaryDiffEqTsit5 loaded, the package
extension adds `CommonSolve.solve(prob, Tsit5(); saveat, ...)` methods for `FVMProblem`,
`FVMSystem`, `DiffusionEquation` and `LinearReactionDiffusionEquation`, and
`CommonSolve.solve(prob, TRBDF2(...))` for the same four types, so scripts written
for the reference run unchanged; `CommonSolve.solve(tmpl, GPUKrylov())` solves the steady
templates and `CommonSolve.solve(SteadyFVMProblem(prob), GPUSteady(...))` a steady problem.

This layer has not been executed: Julia was not available where the library was developed and
measured.  A CPU test checks every ccall's argument types and every struct's layout against the
C header.
"""
module FiniteVolumeMethodGPU

using FiniteVolumeMethod
using DelaunayTriangulation
using ChainRulesCore
import CommonSolve
const FVM = FiniteVolumeMethod
const DT = DelaunayTriangulation

export GPUProblem, GPUSystem, GPUTemplate, GPUBatch, GPUAdjoint, GPUKrylov, GPUSteady, steady_state, adjoint_solve,
    adjoint_pullback,
    set_log_diffusion!, locate, interpolate, steady_solve, jvp!, solve_trbdf2

const libfvmgpu = get(ENV, "FVMGPU_LIB", joinpath(@__DIR__, "..", "..", "..", "fvmgpu", "_lib", "libfvmgpu.so"))

const FVM_OK = Cint(0)
const FVM_PTR_HOST = Cint(0)
const FVM_PTR_DEVICE = Cint(1)
const FVM_PTR_DEVICE_INTERNAL = Cint(2)
const FVM_VERTEX_FREE, FVM_VERTEX_DIRICHLET, FVM_VERTEX_DUDT, FVM_VERTEX_NOT_A_VERTEX = Int8(0), Int8(1), Int8(2), Int8(3)
const FVM_PROBLEM_CONDITIONS_ONLY = Int32(1)
const FVM_TEMPLATE_DIFFUSION, FVM_TEMPLATE_LINEAR_REACTION_DIFFUSION, FVM_TEMPLATE_POISSON, FVM_TEMPLATE_MEAN_EXIT_TIME =
    Int32(0), Int32(1), Int32(2), Int32(3)
const FVM_SOLVER_AUTO, FVM_SOLVER_CG, FVM_SOLVER_BICGSTAB = Int32(0), Int32(1), Int32(2)
const FVM_PRECOND_JACOBI, FVM_PRECOND_CHEBYSHEV = Int32(0), Int32(1)
const FVM_SOLVE_FP64, FVM_SOLVE_MIXED, FVM_SOLVE_FP32_PRECOND = Int32(0), Int32(1), Int32(2)

struct ProblemDesc
    vertex_code::Ptr{Int8}
    bedge_neumann::Ptr{Int8}
    diffusion_degree::Int32
    dual_edge_D::Ptr{Float64}
    quarter_D::Ptr{Float64}
    neumann_degree::Int32
    quarter_neumann::Ptr{Float64}
    source_degree::Int32
    source::Ptr{Float64}
    dudt_degree::Int32
    dudt::Ptr{Float64}
    dirichlet::Ptr{Float64}
    precision::Int32
    dual_edge_flux::Ptr{Float64}
    quarter_flux::Ptr{Float64}
    ntime::Int32
    time_factor::Ptr{Float64}
    time_dirichlet::Ptr{Float64}
    time_neumann::Ptr{Float64}
    time_source::Ptr{Float64}
    time_dudt::Ptr{Float64}
    options::Int32
end

struct OdeOptions
    t0::Float64
    tf::Float64
    dt::Float64
    adaptive::Int32
    abstol::Float64
    reltol::Float64
    max_steps::Int64
    saveat::Ptr{Float64}
    nsave::Int64
    use_graph::Int32
    precision::Int32
end

mutable struct OdeStats
    naccept::Int64
    nreject::Int64
    nrhs::Int64
    t_final::Float64
    elapsed_ms::Float64
    driver::Int32
end

function last_error()
    buf = Vector{UInt8}(undef, 4096)
    ccall((:fvm_last_error, libfvmgpu), Cint, (Ptr{UInt8}, Csize_t), buf, length(buf))
    return unsafe_string(pointer(buf))
end

function check(status::Cint)
    status == FVM_OK && return nothing
    msg = last_error()
    status == Cint(3) && throw(ArgumentError("unsupported closure form: " * msg))
    status == Cint(7) && throw(ArgumentError(msg))
    return error("libfvmgpu status $(status): $(msg)")
end

# ---- mesh: FVMGeometry(tri) (src/geometry.jl:99-169) -------------------------------------
mutable struct GPUMesh
    handle::Ptr{Cvoid}
    triangles::Matrix{Int32}      # 3 x ntri, 0-based, as each_solid_triangle iterates
    bedges::Matrix{Int32}         # 2 x nbe, 0-based, keys of get_boundary_edge_map
    npoints::Int
end

function GPUMesh(mesh::FVM.FVMGeometry)
    tri = mesh.triangulation
    np = DT.num_points(tri)
    pts = Vector{Float64}(undef, 2np)
    for i in 1:np
        x, y = DT.getxy(DT.get_point(tri, i))
        pts[2i-1], pts[2i] = x, y
    end
    tris = Int32[]
    for T in DT.each_solid_triangle(tri)
        i, j, k = DT.triangle_vertices(T)
        push!(tris, i - 1, j - 1, k - 1)
    end
    be = Int32[]
    badj = Int32[]
    for e in keys(DT.get_boundary_edge_map(tri))
        i, j = DT.edge_vertices(e)
        push!(be, i - 1, j - 1)
        push!(badj, DT.get_adjacent(tri, i, j) - 1)
    end
    nt = length(tris) ÷ 3
    nbe = length(be) ÷ 2
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:fvm_mesh_create, libfvmgpu), Cint,
        (Ptr{Float64}, Int64, Ptr{Int32}, Int64, Ptr{Int32}, Ptr{Int32}, Int64, Int32, Int32, Ref{Ptr{Cvoid}}),
        pts, np, tris, nt, be, badj, nbe, 0, 0, h))
    m = GPUMesh(h[], reshape(tris, 3, nt), reshape(be, 2, nbe), np)
    finalizer(m) do x
        ccall((:fvm_mesh_destroy, libfvmgpu), Cint, (Ptr{Cvoid},), x.handle)
    end
    return m
end

function sample_points(m::GPUMesh)
    nt, nbe = size(m.triangles, 2), size(m.bedges, 2)
    dual = Vector{Float64}(undef, 6nt)
    quarter = Vector{Float64}(undef, 4nbe)
    check(ccall((:fvm_mesh_sample_points, libfvmgpu), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}),
        m.handle, dual, quarter))
    return reshape(dual, 2, :), reshape(quarter, 2, :)
end

# ---- closure classification: (x, y) samples, or polynomials of degree <= 2 in u -------------
function classify(f, xs, ys, t0; maxdeg = 2, what = "function")
    n = length(xs)
    g(u, t) = [Float64(f(xs[m], ys[m], t, u)) for m in 1:n]
    g0, g1, gm = g(0.0, t0), g(1.0, t0), g(-1.0, t0)
    c0 = g0
    c1 = (g1 .- gm) ./ 2
    c2 = (g1 .+ gm) ./ 2 .- c0
    sc = max.(abs.(c0), abs.(c1), abs.(c2), 1e-300)
    for u in (2.0, -0.5, 3.25)
        all(abs.(g(u, t0) .- (c0 .+ u .* (c1 .+ u .* c2))) .<= 1e-10 .* sc .* (1 + abs(u))^2) ||
            throw(ArgumentError("$(what) is not a polynomial of degree <= 2 in u"))
    end
    all(abs.(g(1.0, t0 + 1.37) .- g1) .<= 1e-10 .* sc .* 4) || throw(ArgumentError("$(what) depends on t"))
    deg = any(!iszero, c2) ? 2 : any(!iszero, c1) ? 1 : 0
    deg > maxdeg && throw(ArgumentError("$(what) has degree $(deg) > $(maxdeg) in u"))
    return permutedims(hcat(c0, c1, c2)[:, 1:deg+1]), deg
end

# FVM_VERTEX_* per point (Dirichlet before Dudt: source_contributions.jl:5-11) and the
# Neumann flag of each boundary edge, from the merged Conditions
function vertex_codes(tri, conds, np)
    code = fill(FVM_VERTEX_FREE, np)
    for i in 1:np
        if !DT.has_vertex(tri, i)
            code[i] = FVM_VERTEX_NOT_A_VERTEX
        elseif FVM.is_dirichlet_node(conds, i)
            code[i] = FVM_VERTEX_DIRICHLET
        elseif FVM.is_dudt_node(conds, i)
            code[i] = FVM_VERTEX_DUDT
        end
    end
    return code
end

neumann_flags(conds, m::GPUMesh) =
    Int8[FVM.is_neumann_edge(conds, m.bedges[1, e] + 1, m.bedges[2, e] + 1) for e in 1:size(m.bedges, 2)]

# ---- problem: FVMProblem(mesh, BCs, ICs; ...) (src/problem.jl:118-163) ---------------------
mutable struct GPUProblem{P}
    prob::P
    mesh::GPUMesh
    handle::Ptr{Cvoid}
    keep::Vector{Any}
end

function GPUProblem(prob::FVM.FVMProblem; precision = :fp64)
    m = GPUMesh(prob.mesh)
    tri = prob.mesh.triangulation
    conds = prob.conditions
    np = m.npoints
    t0 = prob.initial_time
    code = vertex_codes(tri, conds, np)
    neu = neumann_flags(conds, m)
    dual, quarter = sample_points(m)
    # q(x, y, t, alpha, beta, gamma) = -D(x, y, u) (alpha, beta): D is recovered as -q_x(1, 0, 0)
    q = (x, y, t, u) -> -prob.flux_function(x, y, t, 1.0, 0.0, u, prob.flux_parameters)[1]
    allp = hcat(dual, quarter)
    Dc, ddeg = classify(q, allp[1, :], allp[2, :], t0; what = "diffusion")
    nd = size(dual, 2)
    dualD, quarterD = vec(Dc[:, 1:nd]), vec(Dc[:, nd+1:end])
    # Neumann functions at quarter points, Dudt / Dirichlet at vertices, source at free vertices
    quarterN = zeros(0); ndeg = 0
    if any(!iszero, neu)
        qN = zeros(3, size(quarter, 2))
        for e in 1:size(m.bedges, 2)
            neu[e] == 1 || continue
            fidx = FVM.get_neumann_fidx(conds, m.bedges[1, e] + 1, m.bedges[2, e] + 1)
            f = (x, y, t, u) -> FVM.eval_condition_fnc(conds, fidx, x, y, t, u)
            c, d = classify(f, quarter[1, (2*e-1):(2*e)], quarter[2, (2*e-1):(2*e)], t0; what = "Neumann function $(fidx)")
            qN[1:d+1, (2*e-1):(2*e)] .= c
            ndeg = max(ndeg, d)
        end
        quarterN = vec(qN[1:ndeg+1, :])
    end
    pts = [DT.getxy(DT.get_point(tri, i)) for i in 1:np]
    xs, ys = first.(pts), last.(pts)
    S = (x, y, t, u) -> prob.source_function(x, y, t, u, prob.source_parameters)
    Sc, sdeg = classify(S, xs, ys, t0; what = "source")
    dud = zeros(3, np); dir = zeros(np); udeg = 0
    for i in 1:np
        if code[i] == FVM_VERTEX_DUDT
            fidx = FVM.get_dudt_fidx(conds, i)
            c, d = classify((x, y, t, u) -> FVM.eval_condition_fnc(conds, fidx, x, y, t, u), xs[i:i], ys[i:i], t0)
            dud[1:d+1, i] .= c[:, 1]
            udeg = max(udeg, d)
        elseif code[i] == FVM_VERTEX_DIRICHLET
            fidx = FVM.get_dirichlet_fidx(conds, i)
            c, _ = classify((x, y, t, u) -> FVM.eval_condition_fnc(conds, fidx, x, y, t, u), xs[i:i], ys[i:i], t0;
                maxdeg = 0, what = "Dirichlet function $(fidx)")
            dir[i] = c[1, 1]
        end
    end
    dudt = vec(dud[1:udeg+1, :])
    keep = Any[code, neu, dualD, quarterD, quarterN, Sc, dudt, dir]
    desc = ProblemDesc(pointer(code), pointer(neu), Int32(ddeg), pointer(dualD), pointer(quarterD), Int32(ndeg),
        isempty(quarterN) ? Ptr{Float64}(C_NULL) : pointer(quarterN), Int32(sdeg), pointer(Sc), Int32(udeg),
        pointer(dudt), pointer(dir), precision == :fp32 ? Int32(1) : Int32(0), Ptr{Float64}(C_NULL),
        Ptr{Float64}(C_NULL), Int32(0), Ptr{Float64}(C_NULL), Ptr{Float64}(C_NULL), Ptr{Float64}(C_NULL),
        Ptr{Float64}(C_NULL), Ptr{Float64}(C_NULL), Int32(0))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve keep check(ccall((:fvm_problem_create, libfvmgpu), Cint,
        (Ptr{Cvoid}, Ref{ProblemDesc}, Ref{Ptr{Cvoid}}), m.handle, desc, h))
    gp = GPUProblem(prob, m, h[], keep)
    finalizer(gp) do x
        ccall((:fvm_problem_destroy, libfvmgpu), Cint, (Ptr{Cvoid},), x.handle)
    end
    return gp
end

"""
    fvm_eqs!(du, u, gp::GPUProblem, t)

`fvm_eqs!` (src/equations/main_equations.jl:28-81) on the GPU; `du`, `u` are host vectors.
"""
function fvm_eqs!(du::Vector{Float64}, u::Vector{Float64}, gp::GPUProblem, t)
    check(ccall((:fvm_rhs, libfvmgpu), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Float64, Int32, Ptr{Cvoid}),
        gp.handle, u, du, t, FVM_PTR_HOST, C_NULL))
    return du
end

"""
    solve(gp::GPUProblem; saveat, dt = nothing, abstol = 1e-6, reltol = 1e-3)

Tsit5 on the GPU with the Dirichlet update after every step (src/solve.jl:133-183).
Returns `(t, u)` with `u[k]` the state at `t[k]`.
"""
function solve(gp::GPUProblem; saveat, dt = nothing, abstol = 1e-6, reltol = 1e-3, max_steps = 0)
    prob = gp.prob
    t0, tf = prob.initial_time, prob.final_time
    ts = saveat isa Number ? collect(t0:saveat:tf) : collect(Float64, saveat)
    np = gp.mesh.npoints
    out = Vector{Float64}(undef, np * length(ts))
    u0 = collect(Float64, prob.initial_condition)
    opt = OdeOptions(t0, tf, dt === nothing ? 0.0 : dt, dt === nothing ? Int32(1) : Int32(0), abstol, reltol,
        max_steps, pointer(ts), length(ts), Int32(1), Int32(0))
    st = OdeStats(0, 0, 0, 0.0, 0.0, Int32(0))
    GC.@preserve ts check(ccall((:fvm_tsit5_solve, libfvmgpu), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ref{OdeOptions}, Ptr{Float64}, Ref{OdeStats}, Ptr{Cvoid}),
        gp.handle, u0, opt, out, st, C_NULL))
    return ts, [out[(k-1)*np+1:k*np] for k in eachindex(ts)]
end

# ---- implicit stepping: TR-BDF2 with the device Jacobian-vector product ---------------------
mutable struct ImplicitStats
    newton_iters::Int64
    krylov_iters::Int64
    jvps::Int64
    newton_failures::Int64
end

"""
    jvp!(jv, u, v, gp::GPUProblem, t)

J(u) v, the Jacobian-vector product of `fvm_eqs!` (exact for every device-coded form): what a
Newton-Krylov solve of the reference's implicit methods needs (src/solve.jl:50-131 gives J's
sparsity).
"""
function jvp!(jv::Vector{Float64}, u::Vector{Float64}, v::Vector{Float64}, gp::GPUProblem, t)
    check(ccall((:fvm_jvp, libfvmgpu), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Float64, Int32, Ptr{Cvoid}),
        gp.handle, u, v, jv, t, FVM_PTR_HOST, C_NULL))
    return jv
end

"""
    solve_trbdf2(gp::GPUProblem; saveat, dt = nothing, abstol = 1e-6, reltol = 1e-3)

TR-BDF2 on the device (simplified Newton, matrix-free BiCGStab on I - d h J): the reference
tutorials' `solve(prob, TRBDF2(linsolve = KLUFactorization()))`.  Returns `(t, u, stats)`.
"""
function solve_trbdf2(gp::GPUProblem; saveat, dt = nothing, abstol = 1e-6, reltol = 1e-3, max_steps = 0)
    prob = gp.prob
    t0, tf = prob.initial_time, prob.final_time
    ts = saveat isa Number ? collect(t0:saveat:tf) : collect(Float64, saveat)
    np = gp.mesh.npoints
    out = Vector{Float64}(undef, np * length(ts))
    u0 = collect(Float64, prob.initial_condition)
    opt = OdeOptions(t0, tf, dt === nothing ? 0.0 : dt, dt === nothing ? Int32(1) : Int32(0), abstol, reltol,
        max_steps, pointer(ts), length(ts), Int32(0), Int32(0))
    st = OdeStats(0, 0, 0, 0.0, 0.0, Int32(0))
    ist = ImplicitStats(0, 0, 0, 0)
    GC.@preserve ts check(ccall((:fvm_trbdf2_solve, libfvmgpu), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ref{OdeOptions}, Ptr{Float64}, Ref{OdeStats}, Ref{ImplicitStats}, Ptr{Cvoid}),
        gp.handle, u0, opt, out, st, ist, C_NULL))
    return ts, [out[(k-1)*np+1:k*np] for k in eachindex(ts)], ist
end



# ---- systems: FVMSystem(prob1, ..., probN) (src/problem.jl:190-365) -----------------------
struct SystemDesc
    neq::Int32
    vertex_code::Ptr{Int8}
    bedge_neumann::Ptr{Int8}
    dual_edge_D::Ptr{Float64}
    quarter_D::Ptr{Float64}
    nmono::Int32
    mono_exp::Ptr{Int8}
    source::Ptr{Float64}
    dudt::Ptr{Float64}
    quarter_neumann::Ptr{Float64}
    dirichlet::Ptr{Float64}
    ntime::Int32
    time_factor::Ptr{Float64}
    time_dirichlet::Ptr{Float64}
    time_neumann::Ptr{Float64}
    time_source::Ptr{Float64}
    time_dudt::Ptr{Float64}
end

# exponent vectors of the monomials in N variables of total degree <= 3, by degree
function monomials(N)
    out = Vector{Vector{Int8}}()
    for e in Iterators.product(ntuple(_ -> 0:3, N)...)
        sum(e) <= 3 && push!(out, Int8[e...])
    end
    sort!(out; by = e -> (sum(e), map(-, e)))
    return out
end

vandermonde(us, es) = [prod(Float64(u[c])^e[c] for c in eachindex(e)) for u in us, e in es]

# f(x, y, t, u) with u the N-tuple of component values as a polynomial of total degree <= maxdeg
# with (x, y) coefficients: (exponents, coefficients (monomials x points)), fitted by least
# squares at seeded tuples (the constant term exactly, from u = 0) and verified at fresh tuples
# and at a second time
function classify_system(f, xs, ys, t0, N; maxdeg = 3, what = "function")
    E = filter(e -> sum(e) <= maxdeg, monomials(N))
    seed = UInt64(11)
    rnd() = (seed = seed * 6364136223846793005 + 1442695040888963407; Float64(seed >> 11) / 2.0^53)
    U = [zeros(N)]
    for _ in 1:length(E)+5
        push!(U, [3rnd() - 1.5 for _ in 1:N])
    end
    ev(u, t) = [Float64(f(xs[m], ys[m], t, Tuple(u))) for m in eachindex(xs)]
    F = permutedims(reduce(hcat, [ev(u, t0) for u in U]))
    c0 = F[1, :]
    G = F[2:end, :] .- permutedims(c0)
    rest = E[2:end]
    coef = isempty(rest) ? zeros(0, length(xs)) : vandermonde(U[2:end], rest) \ G
    big = max(isempty(coef) ? 0.0 : maximum(abs, coef), isempty(c0) ? 0.0 : maximum(abs, c0), 1e-300)
    keep = [maximum(abs, coef[k, :]; init = 0.0) > 1e-12 * big for k in eachindex(rest)]
    rest = rest[keep]
    coef = isempty(rest) ? zeros(0, length(xs)) : vandermonde(U[2:end], rest) \ G
    sc = max.(abs.(c0), [maximum(abs, coef[:, m]; init = 0.0) for m in eachindex(xs)], 1e-300)
    for (u, t) in (([4rnd() - 2 for _ in 1:N], t0), (U[2], t0 + 1.37))
        pred = isempty(rest) ? c0 : c0 .+ vec(vandermonde([u], rest) * coef)
        all(abs.(ev(u, t) .- pred) .<= 1e-10 .* sc .* length(E) .* (1 + maximum(abs, u))^maxdeg) ||
            throw(ArgumentError("$(what) is not a polynomial of total degree <= $(maxdeg) in the components, or depends on t"))
    end
    return vcat([E[1]], rest), vcat(permutedims(c0), coef)
end

# D[c] of q(x, y, t, alpha, beta, gamma) = -sum_c D[c](x, y) (alpha[c], beta[c]) at the points, or an error
function classify_system_flux(q, xs, ys, t0, N; what = "flux function")
    z = ntuple(_ -> 0.0, N)
    unit(c) = ntuple(k -> k == c ? 1.0 : 0.0, N)
    D = zeros(length(xs), N)
    for m in eachindex(xs), c in 1:N
        qa = q(xs[m], ys[m], t0, unit(c), z, z)
        qb = q(xs[m], ys[m], t0, z, unit(c), z)
        qg = q(xs[m], ys[m], t0, z, z, unit(c))
        D[m, c] = -qa[1]
        s = max(abs(D[m, c]), 1e-300)
        ok = abs(qa[2]) <= 1e-10s && abs(qb[1]) <= 1e-10s && abs(qb[2] + D[m, c]) <= 1e-10s &&
             maximum(abs, qg) <= 1e-10s
        ok || throw(ArgumentError("$(what) is not of the form -sum_c D_c(x, y) (alpha[c], beta[c])"))
    end
    return D
end

mutable struct GPUSystem{S}
    sys::S
    mesh::GPUMesh
    handle::Ptr{Cvoid}
    keep::Vector{Any}
end

"""
    GPUSystem(sys::FVMSystem)

The system flattened once for `fvm_system_*`: per-component conditions from the system's own
`SimpleConditions`, per-block diffusivities probed from each component's flux, sources, Dudt,
Neumann (affine) and Dirichlet values classified as polynomials in the component tuple.
"""
function GPUSystem(sys::FVM.FVMSystem{N}) where {N}
    m = GPUMesh(sys.mesh)
    tri = sys.mesh.triangulation
    np, nt, nbe = m.npoints, size(m.triangles, 2), size(m.bedges, 2)
    t0 = sys.initial_time
    dual, quarter = sample_points(m)
    pts = [DT.getxy(DT.get_point(tri, i)) for i in 1:np]
    xs, ys = first.(pts), last.(pts)
    code = fill(FVM_VERTEX_FREE, np, N)             # [component][point]
    neu = zeros(Int8, nbe, N)                       # [component][edge]
    Dd = zeros(3nt, N * N)                          # [block][dual edge]
    Dq = zeros(2nbe, N * N)                         # [block][quarter point]
    E = monomials(N)
    col = Dict(e => k for (k, e) in enumerate(E))
    src = zeros(length(E), np, N)                   # [component][point][monomial]
    dud = zeros(length(E), np, N)
    qn = zeros(1 + N, 2nbe, N)                      # [component][quarter point][n0, n_1 .. n_N]
    dir = zeros(np, N)
    for r in 1:N
        for i in 1:np
            if !DT.has_vertex(tri, i)
                code[i, r] = FVM_VERTEX_NOT_A_VERTEX
            elseif FVM.is_dirichlet_node(sys, i, r)
                code[i, r] = FVM_VERTEX_DIRICHLET
            elseif FVM.is_dudt_node(sys, i, r)
                code[i, r] = FVM_VERTEX_DUDT
            end
        end
        for e in 1:nbe
            neu[e, r] = FVM.is_neumann_edge(sys, m.bedges[1, e] + 1, m.bedges[2, e] + 1, r) ? 1 : 0
        end
        q = (x, y, t, a, b, g) -> FVM.eval_flux_function(sys, x, y, t, a, b, g)[r]
        D = classify_system_flux(q, dual[1, :], dual[2, :], t0, N; what = "flux function $(r)")
        for c in 1:N
            Dd[:, (r-1)*N+c] .= D[:, c]
        end
        if nbe > 0
            D = classify_system_flux(q, quarter[1, :], quarter[2, :], t0, N; what = "flux function $(r)")
            for c in 1:N
                Dq[:, (r-1)*N+c] .= D[:, c]
            end
        end
        free = [i for i in 1:np if code[i, r] == FVM_VERTEX_FREE]
        if !isempty(free)
            S = (x, y, t, u) -> FVM.eval_source_fnc(sys, r, x, y, t, u)
            es, cs = classify_system(S, xs[free], ys[free], t0, N; what = "source function $(r)")
            for (k, ek) in enumerate(es)
                src[col[ek], free, r] .= cs[k, :]
            end
        end
        for i in 1:np
            c = code[i, r]
            if c == FVM_VERTEX_DUDT || c == FVM_VERTEX_DIRICHLET
                isdudt = c == FVM_VERTEX_DUDT
                fidx = isdudt ? FVM.get_dudt_fidx(sys, i, r) : FVM.get_dirichlet_fidx(sys, i, r)
                f = (x, y, t, u) -> FVM.eval_condition_fnc(sys, fidx, r, x, y, t, u)
                es, cs = classify_system(f, xs[i:i], ys[i:i], t0, N; maxdeg = isdudt ? 3 : 0,
                    what = "condition function $(fidx) of component $(r)")
                for (k, ek) in enumerate(es)
                    isdudt ? (dud[col[ek], i, r] = cs[k, 1]) : (dir[i, r] = cs[k, 1])
                end
            end
        end
        for e in 1:nbe
            neu[e, r] == 1 || continue
            i, j = m.bedges[1, e] + 1, m.bedges[2, e] + 1
            fidx = FVM.get_neumann_fidx(sys, i, j, r)
            f = (x, y, t, u) -> FVM.eval_condition_fnc(sys, fidx, r, x, y, t, u)
            es, cs = classify_system(f, quarter[1, (2*e-1):(2*e)], quarter[2, (2*e-1):(2*e)], t0, N; maxdeg = 1,
                what = "Neumann function $(fidx) of component $(r)")
            for (k, ek) in enumerate(es)
                slot = sum(ek) == 0 ? 1 : 1 + findfirst(!iszero, ek)
                qn[slot, (2*e-1):(2*e), r] .= cs[k, :]
            end
        end
    end
    used = [k for k in eachindex(E) if any(!iszero, src[k, :, :]) || any(!iszero, dud[k, :, :])]
    mexp = isempty(used) ? zeros(Int8, N, 0) : reduce(hcat, E[used])
    srcu = src[used, :, :]
    dudu = dud[used, :, :]
    keep = Any[code, neu, Dd, Dq, mexp, srcu, dudu, qn, dir]
    ptrf(a, use) = use ? pointer(a) : Ptr{Float64}(C_NULL)
    desc = SystemDesc(Int32(N), pointer(code), nbe > 0 ? pointer(neu) : Ptr{Int8}(C_NULL), pointer(Dd),
        ptrf(Dq, nbe > 0), Int32(length(used)), isempty(used) ? Ptr{Int8}(C_NULL) : pointer(mexp),
        ptrf(srcu, !isempty(used) && any(!iszero, srcu)), ptrf(dudu, !isempty(used) && any(!iszero, dudu)),
        ptrf(qn, nbe > 0 && any(!iszero, qn)), ptrf(dir, any(!iszero, dir)), Int32(0), Ptr{Float64}(C_NULL),
        Ptr{Float64}(C_NULL), Ptr{Float64}(C_NULL), Ptr{Float64}(C_NULL), Ptr{Float64}(C_NULL))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve keep check(ccall((:fvm_system_create, libfvmgpu), Cint,
        (Ptr{Cvoid}, Ref{SystemDesc}, Ref{Ptr{Cvoid}}), m.handle, desc, h))
    gs = GPUSystem(sys, m, h[], keep)
    finalizer(gs) do x
        ccall((:fvm_system_destroy, libfvmgpu), Cint, (Ptr{Cvoid},), x.handle)
    end
    return gs
end

"""
    fvm_eqs!(du, u, gs::GPUSystem, t)

`fvm_eqs!` on an `FVMSystem`; `du`, `u` are N x npoints matrices, whose column-major memory
is the library's `[point][component]` layout.
"""
function fvm_eqs!(du::Matrix{Float64}, u::Matrix{Float64}, gs::GPUSystem, t)
    check(ccall((:fvm_system_rhs, libfvmgpu), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Float64, Int32, Ptr{Cvoid}),
        gs.handle, u, du, t, FVM_PTR_HOST, C_NULL))
    return du
end

"""
    solve(gs::GPUSystem; saveat, dt = nothing, abstol = 1e-6, reltol = 1e-3)

Tsit5 on the system with the Dirichlet update after every step.  Returns `(t, u)` with `u[k]`
the N x npoints state at `t[k]`.
"""
function solve(gs::GPUSystem; saveat, dt = nothing, abstol = 1e-6, reltol = 1e-3, max_steps = 0)
    sys = gs.sys
    t0, tf = sys.initial_time, sys.final_time
    ts = saveat isa Number ? collect(t0:saveat:tf) : collect(Float64, saveat)
    N, np = size(sys.initial_condition)
    out = Array{Float64}(undef, N, np, length(ts))
    u0 = Matrix{Float64}(sys.initial_condition)
    opt = OdeOptions(t0, tf, dt === nothing ? 0.0 : dt, dt === nothing ? Int32(1) : Int32(0), abstol, reltol,
        max_steps, pointer(ts), length(ts), Int32(1), Int32(0))
    st = OdeStats(0, 0, 0, 0.0, 0.0, Int32(0))
    GC.@preserve ts check(ccall((:fvm_system_tsit5_solve, libfvmgpu), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ref{OdeOptions}, Ptr{Float64}, Ref{OdeStats}, Ptr{Cvoid}),
        gs.handle, u0, opt, out, st, C_NULL))
    return ts, [out[:, :, k] for k in eachindex(ts)]
end

"""
    jvp!(jv, u, v, gs::GPUSystem, t)

`jv = J(u) v` for the system's `fvm_eqs!` (N x npoints matrices), exact.
"""
function jvp!(jv::Matrix{Float64}, u::Matrix{Float64}, v::Matrix{Float64}, gs::GPUSystem, t)
    check(ccall((:fvm_system_jvp, libfvmgpu), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Float64, Int32, Ptr{Cvoid}),
        gs.handle, u, v, jv, t, FVM_PTR_HOST, C_NULL))
    return jv
end

"""
    solve_trbdf2(gs::GPUSystem; saveat, dt = nothing, abstol = 1e-6, reltol = 1e-3)

TR-BDF2 on the system (the Brusselator and Gray-Scott tutorials' `solve(system, TRBDF2(...))`).
Returns `(t, u, stats)` with `u[k]` the N x npoints state at `t[k]`.
"""
function solve_trbdf2(gs::GPUSystem; saveat, dt = nothing, abstol = 1e-6, reltol = 1e-3, max_steps = 0)
    sys = gs.sys
    t0, tf = sys.initial_time, sys.final_time
    ts = saveat isa Number ? collect(t0:saveat:tf) : collect(Float64, saveat)
    N, np = size(sys.initial_condition)
    out = Array{Float64}(undef, N, np, length(ts))
    u0 = Matrix{Float64}(sys.initial_condition)
    opt = OdeOptions(t0, tf, dt === nothing ? 0.0 : dt, dt === nothing ? Int32(1) : Int32(0), abstol, reltol,
        max_steps, pointer(ts), length(ts), Int32(0), Int32(0))
    st = OdeStats(0, 0, 0, 0.0, 0.0, Int32(0))
    ist = ImplicitStats(0, 0, 0, 0)
    GC.@preserve ts check(ccall((:fvm_system_trbdf2_solve, libfvmgpu), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ref{OdeOptions}, Ptr{Float64}, Ref{OdeStats}, Ref{ImplicitStats}, Ptr{Cvoid}),
        gs.handle, u0, opt, out, st, ist, C_NULL))
    return ts, [out[:, :, k] for k in eachindex(ts)], ist
end

# ---- templates (src/specific_problems/) ----------------------------------------------------
mutable struct GPUTemplate{T}
    tmpl::T
    mesh::GPUMesh
    problem::Ptr{Cvoid}   # the conditions carrier (FVM_PROBLEM_CONDITIONS_ONLY)
    handle::Ptr{Cvoid}
    keep::Vector{Any}
end

template_kind(::FVM.DiffusionEquation) = FVM_TEMPLATE_DIFFUSION
template_kind(::FVM.LinearReactionDiffusionEquation) = FVM_TEMPLATE_LINEAR_REACTION_DIFFUSION
template_kind(::FVM.PoissonsEquation) = FVM_TEMPLATE_POISSON
template_kind(::FVM.LaplacesEquation) = FVM_TEMPLATE_POISSON  # the Poisson template with f = 0
template_kind(::FVM.MeanExitTimeProblem) = FVM_TEMPLATE_MEAN_EXIT_TIME

"""
    GPUTemplate(tmpl)

A `DiffusionEquation`, `LinearReactionDiffusionEquation`, `PoissonsEquation` or
`MeanExitTimeProblem` assembled on the device (`fvm_template_create`): D(x, y, p) sampled at the
dual-edge midpoints and boundary quarter points, the conditions evaluated with t = u = nothing
(src/specific_problems/abstract_templates.jl), the source (Poisson's f, the reaction
coefficient) at the vertices.
"""
function GPUTemplate(tmpl::FVM.AbstractFVMTemplate)
    m = GPUMesh(tmpl.mesh)
    tri = tmpl.mesh.triangulation
    conds = tmpl.conditions
    np = m.npoints
    kind = template_kind(tmpl)
    code = vertex_codes(tri, conds, np)
    neu = neumann_flags(conds, m)
    dual, quarter = sample_points(m)
    D, Dp = tmpl.diffusion_function, tmpl.diffusion_parameters
    dualD = Float64[D(dual[1, k], dual[2, k], Dp) for k in axes(dual, 2)]
    quarterD = Float64[D(quarter[1, k], quarter[2, k], Dp) for k in axes(quarter, 2)]
    qn = zeros(size(quarter, 2))
    for e in 1:size(m.bedges, 2)
        neu[e] == 1 || continue
        fidx = FVM.get_neumann_fidx(conds, m.bedges[1, e] + 1, m.bedges[2, e] + 1)
        for k in (2 * e - 1, 2 * e)
            qn[k] = Float64(FVM.eval_condition_fnc(conds, fidx, quarter[1, k], quarter[2, k], nothing, nothing))
        end
    end
    dudt = zeros(np)
    dir = zeros(np)
    for i in 1:np
        (code[i] == FVM_VERTEX_DUDT || code[i] == FVM_VERTEX_DIRICHLET) || continue
        x, y = DT.getxy(DT.get_point(tri, i))
        isdudt = code[i] == FVM_VERTEX_DUDT
        fidx = isdudt ? FVM.get_dudt_fidx(conds, i) : FVM.get_dirichlet_fidx(conds, i)
        v = Float64(FVM.eval_condition_fnc(conds, fidx, x, y, nothing, nothing))
        isdudt ? (dudt[i] = v) : (dir[i] = v)
    end
    src = zeros(0)
    sdeg = Int32(0)
    if kind == FVM_TEMPLATE_POISSON || kind == FVM_TEMPLATE_LINEAR_REACTION_DIFFUSION
        S, Sp = tmpl isa FVM.LaplacesEquation ? ((x, y, p) -> 0.0, nothing) :
                (tmpl.source_function, tmpl.source_parameters)
        sv = Float64[S(DT.getxy(DT.get_point(tri, i))..., Sp) for i in 1:np]
        if kind == FVM_TEMPLATE_LINEAR_REACTION_DIFFUSION  # the reaction coefficient: source c1 u
            src = vec(permutedims(hcat(zeros(np), sv)))
            sdeg = Int32(1)
        else
            src = sv
        end
    end
    keep = Any[code, neu, dualD, quarterD, qn, src, dudt, dir]
    nbe = size(m.bedges, 2)
    pf(a, use) = use ? pointer(a) : Ptr{Float64}(C_NULL)
    desc = ProblemDesc(pointer(code), nbe > 0 ? pointer(neu) : Ptr{Int8}(C_NULL), Int32(0), pointer(dualD),
        pf(quarterD, nbe > 0), Int32(0), pf(qn, any(==(1), neu)), sdeg, pf(src, !isempty(src)), Int32(0), pointer(dudt),
        pointer(dir), Int32(0), Ptr{Float64}(C_NULL), Ptr{Float64}(C_NULL), Int32(0), Ptr{Float64}(C_NULL),
        Ptr{Float64}(C_NULL), Ptr{Float64}(C_NULL), Ptr{Float64}(C_NULL), Ptr{Float64}(C_NULL),
        FVM_PROBLEM_CONDITIONS_ONLY)
    hp = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve keep check(ccall((:fvm_problem_create, libfvmgpu), Cint,
        (Ptr{Cvoid}, Ref{ProblemDesc}, Ref{Ptr{Cvoid}}), m.handle, desc, hp))
    ht = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:fvm_template_create, libfvmgpu), Cint, (Ptr{Cvoid}, Int32, Ref{Ptr{Cvoid}}), hp[], kind, ht)
    if st != FVM_OK
        msg = last_error()
        ccall((:fvm_problem_destroy, libfvmgpu), Cint, (Ptr{Cvoid},), hp[])
        error("libfvmgpu status $(st): $(msg)")
    end
    gt = GPUTemplate(tmpl, m, hp[], ht[], keep)
    finalizer(gt) do x
        ccall((:fvm_template_destroy, libfvmgpu), Cint, (Ptr{Cvoid},), x.handle)
        ccall((:fvm_problem_destroy, libfvmgpu), Cint, (Ptr{Cvoid},), x.problem)
    end
    return gt
end

"""
    apply!(du, u, gt::GPUTemplate; precision = :fp64)

du = A u + b, the template's MatrixOperator product (diffusion_equation.jl:93-94); vectors of
length npoints.
"""
function apply!(du::Vector{Float64}, u::Vector{Float64}, gt::GPUTemplate; precision = :fp64)
    check(ccall((:fvm_template_apply, libfvmgpu), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int32, Int32, Ptr{Cvoid}),
        gt.handle, u, du, precision == :fp32 ? Int32(1) : Int32(0), FVM_PTR_HOST, C_NULL))
    return du
end

"""
    export_operator(gt::GPUTemplate) -> (A::SparseMatrixCSC-ready (rowptr, col, val), b)

A in CSR (0-based, caller numbering, sorted columns) and b, as assembled on the device.
"""
function export_operator(gt::GPUTemplate)
    nnz = Ref{Int64}(0)
    check(ccall((:fvm_template_export, libfvmgpu), Cint,
        (Ptr{Cvoid}, Ref{Int64}, Ptr{Int32}, Ptr{Int32}, Ptr{Float64}, Ptr{Float64}),
        gt.handle, nnz, C_NULL, C_NULL, C_NULL, C_NULL))
    np = gt.mesh.npoints
    rowptr = Vector{Int32}(undef, np + 1)
    col = Vector{Int32}(undef, nnz[])
    val = Vector{Float64}(undef, nnz[])
    b = Vector{Float64}(undef, np)
    check(ccall((:fvm_template_export, libfvmgpu), Cint,
        (Ptr{Cvoid}, Ref{Int64}, Ptr{Int32}, Ptr{Int32}, Ptr{Float64}, Ptr{Float64}),
        gt.handle, nnz, rowptr, col, val, b))
    return (rowptr, col, val), b
end

"""
    solve(gt::GPUTemplate; saveat, dt = nothing, abstol = 1e-6, reltol = 1e-3)

Tsit5 on du/dt = A u + b of a `DiffusionEquation` / `LinearReactionDiffusionEquation`.  Returns
`(t, u)` with `u[k]` of length npoints + 1, the reference's augmented state (last entry 1).
"""
function solve(gt::GPUTemplate; saveat, dt = nothing, abstol = 1e-6, reltol = 1e-3, max_steps = 0)
    tmpl = gt.tmpl
    t0, tf = tmpl.initial_time, tmpl.final_time
    ts = saveat isa Number ? collect(t0:saveat:tf) : collect(Float64, saveat)
    np = gt.mesh.npoints
    out = Vector{Float64}(undef, np * length(ts))
    u0 = collect(Float64, tmpl.initial_condition)[1:np]
    opt = OdeOptions(t0, tf, dt === nothing ? 0.0 : dt, dt === nothing ? Int32(1) : Int32(0), abstol, reltol,
        max_steps, pointer(ts), length(ts), Int32(1), Int32(0))
    st = OdeStats(0, 0, 0, 0.0, 0.0, Int32(0))
    GC.@preserve ts check(ccall((:fvm_template_tsit5_solve, libfvmgpu), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ref{OdeOptions}, Ptr{Float64}, Ref{OdeStats}, Ptr{Cvoid}),
        gt.handle, u0, opt, out, st, C_NULL))
    return ts, [vcat(out[(k-1)*np+1:k*np], 1.0) for k in eachindex(ts)]
end

"""
    solve_trbdf2(gt::GPUTemplate; saveat, dt = nothing, abstol = 1e-6, reltol = 1e-3)

TR-BDF2 on a time-dependent template (J = A).  Returns `(t, u, stats)`, `u[k]` of length
npoints + 1 (the reference's augmented state).
"""
function solve_trbdf2(gt::GPUTemplate; saveat, dt = nothing, abstol = 1e-6, reltol = 1e-3, max_steps = 0)
    tmpl = gt.tmpl
    t0, tf = tmpl.initial_time, tmpl.final_time
    ts = saveat isa Number ? collect(t0:saveat:tf) : collect(Float64, saveat)
    np = gt.mesh.npoints
    out = Vector{Float64}(undef, np * length(ts))
    u0 = collect(Float64, tmpl.initial_condition)[1:np]
    opt = OdeOptions(t0, tf, dt === nothing ? 0.0 : dt, dt === nothing ? Int32(1) : Int32(0), abstol, reltol,
        max_steps, pointer(ts), length(ts), Int32(0), Int32(0))
    st = OdeStats(0, 0, 0, 0.0, 0.0, Int32(0))
    ist = ImplicitStats(0, 0, 0, 0)
    GC.@preserve ts check(ccall((:fvm_template_trbdf2_solve, libfvmgpu), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ref{OdeOptions}, Ptr{Float64}, Ref{OdeStats}, Ref{ImplicitStats}, Ptr{Cvoid}),
        gt.handle, u0, opt, out, st, ist, C_NULL))
    return ts, [vcat(out[(k-1)*np+1:k*np], 1.0) for k in eachindex(ts)], ist
end

# ---- steady solve (LinearProblem(A, b), poissons_equation.jl:81, mean_exit_time.jl:76) -----
struct SolverOptions
    rtol::Float64
    max_iters::Int64
    method::Int32
    precond::Int32
    cheb_degree::Int32
    mode::Int32
    inner_reduction::Float64
end

mutable struct SolverStats
    iterations::Int64
    refinements::Int64
    rel_residual::Float64
    elapsed_ms::Float64
    method_used::Int32
    symmetric::Int32
    fallback_fp64::Int32
end

"""
    GPUKrylov(; rtol = 1e-10, method = :auto, precond = :jacobi, cheb_degree = 4, mode = :fp64,
              max_iters = 1_000_000, inner_reduction = 1e-3)

The device steady solver, an algorithm for `solve(tmpl, GPUKrylov())` on a `PoissonsEquation` or
`MeanExitTimeProblem` in place of a LinearSolve factorisation: CG (symmetric reduced operator)
or BiCGStab, Jacobi or Chebyshev preconditioning, FP64 or mixed precision, stopped on the FP64
residual ||b - A x|| / ||b|| <= rtol.
"""
Base.@kwdef struct GPUKrylov
    rtol::Float64 = 1e-10
    method::Symbol = :auto
    precond::Symbol = :jacobi
    cheb_degree::Int = 4
    mode::Symbol = :fp64
    max_iters::Int = 1_000_000
    inner_reduction::Float64 = 1e-3
end

"""
    steady_solve(gt::GPUTemplate, alg::GPUKrylov = GPUKrylov(); u0 = zeros) -> (x, stats)

Solves A x = b of a Poisson or mean-exit-time template on the device.
"""
function steady_solve(gt::GPUTemplate, alg::GPUKrylov = GPUKrylov(); u0 = nothing)
    np = gt.mesh.npoints
    x = u0 === nothing ? zeros(np) : collect(Float64, u0)[1:np]
    method = Dict(:auto => FVM_SOLVER_AUTO, :cg => FVM_SOLVER_CG, :bicgstab => FVM_SOLVER_BICGSTAB)[alg.method]
    precond = Dict(:jacobi => FVM_PRECOND_JACOBI, :chebyshev => FVM_PRECOND_CHEBYSHEV)[alg.precond]
    mode = Dict(:fp64 => FVM_SOLVE_FP64, :mixed => FVM_SOLVE_MIXED, :fp32_precond => FVM_SOLVE_FP32_PRECOND)[alg.mode]
    opt = SolverOptions(alg.rtol, alg.max_iters, method, precond, Int32(alg.cheb_degree), mode, alg.inner_reduction)
    st = SolverStats(0, 0, 0.0, 0.0, Int32(0), Int32(0), Int32(0))
    status = ccall((:fvm_template_steady_solve, libfvmgpu), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ref{SolverOptions}, Ref{SolverStats}, Int32, Ptr{Cvoid}),
        gt.handle, x, opt, st, FVM_PTR_HOST, C_NULL)
    status == Cint(6) && @warn "steady solve stopped before rtol" st.rel_residual st.iterations
    status == Cint(6) || check(status)
    return x, st
end

"""
    solve(tmpl::Union{PoissonsEquation, MeanExitTimeProblem}, alg::GPUKrylov)

The steady template solved on the device in place of `solve(tmpl, KLUFactorization())`
(src/specific_problems/abstract_templates.jl:58-60): a named tuple with `u` (the solution) and
`stats`.
"""
function CommonSolve.solve(tmpl::Union{FVM.PoissonsEquation, FVM.LaplacesEquation, FVM.MeanExitTimeProblem},
                           alg::GPUKrylov; kwargs...)
    x, st = steady_solve(gpu_object(tmpl), alg)
    return (u = x, stats = st)
end

# ---- steady states: SteadyFVMProblem (src/problem.jl:166-180, src/solve.jl:184-196) ----------
struct SteadyOptions
    method::Int32
    abstol::Float64
    reltol::Float64
    t::Float64
    tmax::Float64
    ode_abstol::Float64
    ode_reltol::Float64
    max_iters::Int64
end

mutable struct SteadyStats
    iterations::Int64
    krylov_iters::Int64
    jvps::Int64
    nrhs::Int64
    residual::Float64
    t_final::Float64
    elapsed_ms::Float64
end

"""
    GPUSteady(method = :dynamic; abstol, reltol, tspan = Inf, ode_abstol = 1e-6, ode_reltol = 1e-3,
              max_iters = 0)

The device steady solver for `solve(SteadyFVMProblem(prob), GPUSteady(...))`, in place of the
tutorials' `DynamicSS(TRBDF2(...))` / `DynamicSS(Rosenbrock23())` (`method = :dynamic`: TR-BDF2 in
pseudo-time until max|du/dt| <= abstol or <= reltol max|du/dt + u|; abstol 1e-8, reltol 1e-6 by
default) or `NewtonRaphson()` (`method = :newton`: Newton-Krylov with the exact device JVP, the
rows the problem fixes held; abstol = reltol = 1e-10 by default).
"""
struct GPUSteady
    method::Symbol
    abstol::Float64
    reltol::Float64
    tspan::Float64
    ode_abstol::Float64
    ode_reltol::Float64
    max_iters::Int
end
function GPUSteady(method::Symbol = :dynamic; abstol = method === :newton ? 1e-10 : 1e-8,
                   reltol = method === :newton ? 1e-10 : 1e-6, tspan = Inf, ode_abstol = 1e-6, ode_reltol = 1e-3,
                   max_iters = 0)
    method in (:dynamic, :newton) || throw(ArgumentError("GPUSteady method is :dynamic or :newton"))
    return GPUSteady(method, abstol, reltol, tspan, ode_abstol, ode_reltol, max_iters)
end

steady_options(alg::GPUSteady, t0) = SteadyOptions(alg.method === :newton ? Int32(1) : Int32(0), alg.abstol,
    alg.reltol, t0, t0 + alg.tspan, alg.ode_abstol, alg.ode_reltol, alg.max_iters)

"""
    steady_state(g::Union{GPUProblem, GPUSystem}, alg::GPUSteady = GPUSteady()) -> (u, stats)

The steady state from the problem's initial condition (the initial guess), on the device
(`fvm_steady_solve` / `fvm_system_steady_solve`).  Not converged: a warning, and the last iterate.
"""
function steady_state(gp::GPUProblem, alg::GPUSteady = GPUSteady())
    prob = gp.prob
    u0 = collect(Float64, prob.initial_condition)
    out = similar(u0)
    opt = steady_options(alg, prob.initial_time)
    st = SteadyStats(0, 0, 0, 0, 0.0, 0.0, 0.0)
    status = ccall((:fvm_steady_solve, libfvmgpu), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ref{SteadyOptions}, Ptr{Float64}, Ref{SteadyStats}, Ptr{Cvoid}),
        gp.handle, u0, opt, out, st, C_NULL)
    status == Cint(6) && @warn "steady state not reached" st.residual st.iterations
    status == Cint(6) || check(status)
    return out, st
end
function steady_state(gs::GPUSystem, alg::GPUSteady = GPUSteady())
    sys = gs.sys
    u0 = Matrix{Float64}(sys.initial_condition)
    out = similar(u0)
    opt = steady_options(alg, sys.initial_time)
    st = SteadyStats(0, 0, 0, 0, 0.0, 0.0, 0.0)
    status = ccall((:fvm_system_steady_solve, libfvmgpu), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ref{SteadyOptions}, Ptr{Float64}, Ref{SteadyStats}, Ptr{Cvoid}),
        gs.handle, u0, opt, out, st, C_NULL)
    status == Cint(6) && @warn "steady state not reached" st.residual st.iterations
    status == Cint(6) || check(status)
    return out, st
end

"""
    solve(prob::SteadyFVMProblem, alg::GPUSteady)

The steady state on the device: a named tuple with `u` (vector, or N x npoints matrix for a
system) and `stats`.
"""
function CommonSolve.solve(prob::FVM.SteadyFVMProblem, alg::GPUSteady; kwargs...)
    u, st = steady_state(gpu_object(prob.problem), alg)
    return (u = u, stats = st)
end

# ---- batched instances (an EnsembleProblem over D on one mesh) ------------------------------
mutable struct GPUBatch
    gp::GPUProblem
    handle::Ptr{Cvoid}
    batch::Int
end

"""
    GPUBatch(gp::GPUProblem, dualD::Matrix, quarterD::Matrix; precision = :fp64)

`batch` instances of the linear problem `gp` that differ in their diffusion field: `dualD` is
batch x (3 ntri) (the field at the dual-edge midpoints, `sample_points` order), `quarterD`
batch x (2 nbedge) (or empty without boundary samples).  States are batch x npoints matrices
(the library's [point][instance] memory).
"""
function GPUBatch(gp::GPUProblem, dualD::Matrix{Float64}, quarterD::Matrix{Float64}; precision = :fp64)
    B = size(dualD, 1)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    dT = permutedims(dualD)   # [instance][sample] rows, each instance contiguous
    qT = permutedims(quarterD)
    GC.@preserve dT qT check(ccall((:fvm_batch_create, libfvmgpu), Cint,
        (Ptr{Cvoid}, Int32, Ptr{Float64}, Ptr{Float64}, Int32, Ref{Ptr{Cvoid}}),
        gp.handle, Int32(B), dT, isempty(qT) ? Ptr{Float64}(C_NULL) : pointer(qT),
        precision == :fp32 ? Int32(1) : Int32(0), h))
    gb = GPUBatch(gp, h[], B)
    finalizer(gb) do x
        ccall((:fvm_batch_destroy, libfvmgpu), Cint, (Ptr{Cvoid},), x.handle)
    end
    return gb
end

function fvm_eqs!(du::Matrix{Float64}, u::Matrix{Float64}, gb::GPUBatch, t)
    check(ccall((:fvm_batch_rhs, libfvmgpu), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Float64, Int32, Ptr{Cvoid}),
        gb.handle, u, du, t, FVM_PTR_HOST, C_NULL))
    return du
end

"""
    solve(gb::GPUBatch, u0::Matrix; dt, saveat)

Fixed-step Tsit5 on every instance (u0 batch x npoints).  Returns `(t, u)`, `u[k]` batch x npoints.
"""
function solve(gb::GPUBatch, u0::Matrix{Float64}; dt, saveat)
    prob = gb.gp.prob
    t0, tf = prob.initial_time, prob.final_time
    ts = saveat isa Number ? collect(t0:saveat:tf) : collect(Float64, saveat)
    B, np = size(u0)
    out = Array{Float64}(undef, B, np, length(ts))
    opt = OdeOptions(t0, tf, dt, Int32(0), 1e-6, 1e-3, 0, pointer(ts), length(ts), Int32(1), Int32(0))
    st = OdeStats(0, 0, 0, 0.0, 0.0, Int32(0))
    GC.@preserve ts check(ccall((:fvm_batch_tsit5_solve, libfvmgpu), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ref{OdeOptions}, Ptr{Float64}, Ref{OdeStats}, Ptr{Cvoid}),
        gb.handle, u0, opt, out, st, C_NULL))
    return ts, [out[:, :, k] for k in eachindex(ts)]
end

# ---- discrete adjoint of the time templates ----------------------------------------------
mutable struct AdjointStats
    steps::Int64
    checkpoints::Int64
    rhs_evals::Int64
    transpose_evals::Int64
    forward_ms::Float64
    reverse_ms::Float64
end

mutable struct GPUAdjoint
    gt::GPUTemplate
    handle::Ptr{Cvoid}
    batch::Int
end

"""
    GPUAdjoint(gt::GPUTemplate, batch)

`batch` instances of a `DiffusionEquation` / `LinearReactionDiffusionEquation` template whose
diffusion field is exp(theta) interpolated from per-vertex values theta (batch x npoints), for
gradients of fixed-step Tsit5 solves by the discrete adjoint (`adjoint_solve` and its rrule).
"""
function GPUAdjoint(gt::GPUTemplate, batch::Integer)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:fvm_adjoint_create, libfvmgpu), Cint, (Ptr{Cvoid}, Int32, Ref{Ptr{Cvoid}}), gt.handle, Int32(batch), h))
    ga = GPUAdjoint(gt, h[], Int(batch))
    finalizer(ga) do x
        ccall((:fvm_adjoint_destroy, libfvmgpu), Cint, (Ptr{Cvoid},), x.handle)
    end
    return ga
end

function set_log_diffusion!(ga::GPUAdjoint, theta::Matrix{Float64})
    check(ccall((:fvm_adjoint_set_log_diffusion, libfvmgpu), Cint, (Ptr{Cvoid}, Ptr{Float64}, Int32, Ptr{Cvoid}),
        ga.handle, theta, FVM_PTR_HOST, C_NULL))
    return ga
end

"""
    adjoint_solve(ga::GPUAdjoint, theta, u0, dt, nsteps) -> uT

u(T) of every instance after `nsteps` Tsit5 steps of `dt` (theta, u0, uT: batch x npoints).
Differentiable: `ChainRulesCore.rrule` runs the discrete adjoint on the device.
"""
function adjoint_solve(ga::GPUAdjoint, theta::Matrix{Float64}, u0::Matrix{Float64}, dt::Real, nsteps::Integer)
    set_log_diffusion!(ga, theta)
    uT = similar(u0)
    check(ccall((:fvm_adjoint_forward, libfvmgpu), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Float64, Int64, Ptr{Float64}, Int32, Ptr{Cvoid}),
        ga.handle, u0, Float64(dt), Int64(nsteps), uT, FVM_PTR_HOST, C_NULL))
    return uT
end

"""
    adjoint_pullback(ga, theta, u0, dt, nsteps, uT_bar; checkpoint_every = 20) -> (theta_bar, u0_bar, stats)
"""
function adjoint_pullback(ga::GPUAdjoint, theta::Matrix{Float64}, u0::Matrix{Float64}, dt::Real, nsteps::Integer,
                          uT_bar::AbstractMatrix; checkpoint_every::Integer = 20)
    set_log_diffusion!(ga, theta)
    tb = similar(theta)
    ub = similar(u0)
    ubar = Matrix{Float64}(uT_bar)
    st = AdjointStats(0, 0, 0, 0, 0.0, 0.0)
    check(ccall((:fvm_adjoint_pullback, libfvmgpu), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Float64, Int64, Int32, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ref{AdjointStats},
         Int32, Ptr{Cvoid}),
        ga.handle, u0, Float64(dt), Int64(nsteps), Int32(checkpoint_every), ubar, tb, ub, st, FVM_PTR_HOST, C_NULL))
    return tb, ub, st
end

function ChainRulesCore.rrule(::typeof(adjoint_solve), ga::GPUAdjoint, theta::Matrix{Float64}, u0::Matrix{Float64},
                              dt::Real, nsteps::Integer)
    uT = adjoint_solve(ga, theta, u0, dt, nsteps)
    function adjoint_solve_pullback(uT_bar)
        tb, ub, _ = adjoint_pullback(ga, theta, u0, dt, nsteps, ChainRulesCore.unthunk(uT_bar))
        return ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent(), tb, ub, ChainRulesCore.NoTangent(),
               ChainRulesCore.NoTangent()
    end
    return uT, adjoint_solve_pullback
end

# ---- post-processing: point location and pl_interpolate for many points -------------------
"""
    locate(m::GPUMesh, xs, ys) -> Vector{Int}

The (1-based) index, in `each_solid_triangle` order, of a triangle holding each point, 0 outside
the mesh; the device counterpart of the tutorials' jump_and_march.
"""
function locate(m::GPUMesh, xs::AbstractVector, ys::AbstractVector)
    xy = Vector{Float64}(undef, 2length(xs))
    for q in eachindex(xs)
        xy[2q-1], xy[2q] = xs[q], ys[q]
    end
    out = Vector{Int64}(undef, length(xs))
    check(ccall((:fvm_mesh_locate, libfvmgpu), Cint, (Ptr{Cvoid}, Int64, Ptr{Float64}, Ptr{Int64}, Int32, Ptr{Cvoid}),
        m.handle, Int64(length(xs)), xy, out, FVM_PTR_HOST, C_NULL))
    return out .+ 1
end

"""
    interpolate(m::GPUMesh, u, xs, ys) -> Vector{Float64}

pl_interpolate (src/utils.jl:23-27) of the nodal values u at every point, NaN outside the mesh.
"""
function interpolate(m::GPUMesh, u::AbstractVector, xs::AbstractVector, ys::AbstractVector)
    tri = locate(m, xs, ys) .- 1
    xy = Vector{Float64}(undef, 2length(xs))
    for q in eachindex(xs)
        xy[2q-1], xy[2q] = xs[q], ys[q]
    end
    uu = collect(Float64, u)
    out = Vector{Float64}(undef, length(xs))
    check(ccall((:fvm_pl_interpolate, libfvmgpu), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Int32, Int64, Ptr{Int64}, Ptr{Float64}, Ptr{Float64}, Int32, Ptr{Cvoid}),
        m.handle, uu, Int32(1), Int64(length(xs)), tri, xy, out, FVM_PTR_HOST, C_NULL))
    return out
end

# GPU objects of the reference's problems, built once per problem object (CommonSolve methods)
const _CACHE = IdDict{Any, Any}()
gpu_object(prob::FVM.FVMProblem) = get!(() -> GPUProblem(prob), _CACHE, prob)
gpu_object(sys::FVM.FVMSystem) = get!(() -> GPUSystem(sys), _CACHE, sys)
gpu_object(tmpl::FVM.AbstractFVMTemplate) = get!(() -> GPUTemplate(tmpl), _CACHE, tmpl)
clear_gpu_cache!() = empty!(_CACHE)

function __init__()
    isfile(libfvmgpu) || @warn "libfvmgpu.so not found at $(libfvmgpu); build it (python -c 'import fvmgpu; fvmgpu.build()') or set FVMGPU_LIB"
end

end # module
