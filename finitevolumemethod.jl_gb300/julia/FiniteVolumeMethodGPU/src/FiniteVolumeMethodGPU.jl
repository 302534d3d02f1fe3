"""
    FiniteVolumeMethodGPU

Julia binding of libfvmgpu.so (include/fvm_gpu.h).  A problem is built with
FiniteVolumeMethod.jl exactly as before (`FVMGeometry`, `BoundaryConditions`,
`InternalConditions`, `FVMProblem`, the templates); `GPUProblem(prob)` flattens it once
(triangles, boundary edges, the merged `Conditions` dictionaries, closures sampled at the
dual-edge midpoints and boundary quarter points) and every `fvm_eqs!` / `solve` then runs on
the GPU through `ccall`.  Closures must be functions of (x, y), or polynomials of degree <= 2
in u with (x, y) coefficients; other forms raise `ArgumentError`.
Indices passed to the C ABI are 0-based.

This layer has not been executed: Julia is not installed on the machines this build was
developed and measured on.
"""
module FiniteVolumeMethodGPU

using FiniteVolumeMethod
using DelaunayTriangulation
const FVM = FiniteVolumeMethod
const DT = DelaunayTriangulation

const libfvmgpu = get(ENV, "FVMGPU_LIB", joinpath(@__DIR__, "..", "..", "..", "fvmgpu", "_lib", "libfvmgpu.so"))

const FVM_OK = Cint(0)
const FVM_PTR_HOST = Cint(0)
const FVM_PTR_DEVICE = Cint(1)
const FVM_VERTEX_FREE, FVM_VERTEX_DIRICHLET, FVM_VERTEX_DUDT, FVM_VERTEX_NOT_A_VERTEX = Int8(0), Int8(1), Int8(2), Int8(3)

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
    neu = Int8[FVM.is_neumann_edge(conds, m.bedges[1, e] + 1, m.bedges[2, e] + 1) for e in 1:size(m.bedges, 2)]
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
            c, d = classify(f, quarter[1, 2e-1:2e], quarter[2, 2e-1:2e], t0; what = "Neumann function $(fidx)")
            qN[1:d+1, 2e-1:2e] .= c
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
        pointer(dudt), pointer(dir), precision == :fp32 ? Int32(1) : Int32(0))
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

end # module
