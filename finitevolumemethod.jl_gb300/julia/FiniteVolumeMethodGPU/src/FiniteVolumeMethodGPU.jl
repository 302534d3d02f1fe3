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
            es, cs = classify_system(f, quarter[1, 2e-1:2e], quarter[2, 2e-1:2e], t0, N; maxdeg = 1,
                what = "Neumann function $(fidx) of component $(r)")
            for (k, ek) in enumerate(es)
                slot = sum(ek) == 0 ? 1 : 1 + findfirst(!iszero, ek)
                qn[slot, 2e-1:2e, r] .= cs[k, :]
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

end # module
