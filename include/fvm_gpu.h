/*
 * fvm_gpu.h - C ABI of the GB300 vertex-centred finite-volume library (libfvmgpu.so).
 *
 * Every entry point returns an int status (FVM_OK = 0) and never aborts the
 * process; fvm_last_error() gives the message of the last failure on the
 * calling thread.  Handles are opaque and owned by the library; free them with
 * the matching *_destroy.  A mesh and every handle built on it (its problems,
 * templates, systems, batches) are used by one host thread at a time: they share
 * per-mesh work state that is built and reused on demand.  Input host arrays are
 * copied at creation.  All
 * vertex, triangle and edge indices are 0-based and in the caller's
 * ("reference") numbering; internally the library renumbers vertices along a
 * Hilbert curve and maps back at the boundary.
 *
 * Reference interfaces replaced (FiniteVolumeMethod.jl 1.2.3, paths relative
 * to the project root) are cited beside each declaration.  The reference is
 * pure Julia and has no FFI of its own: the Julia layer in
 * julia/FiniteVolumeMethodGPU ccalls exactly these symbols.
 */
#ifndef FVM_GPU_H
#define FVM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------------------- */
#define FVM_OK 0
#define FVM_ERR_INVALID_ARGUMENT 1 /* null pointer, bad size, bad enum */
#define FVM_ERR_BAD_MESH 2         /* index out of range, clockwise or degenerate triangle, open boundary edge */
#define FVM_ERR_UNSUPPORTED_FORM 3 /* closure form outside the device-coded set */
#define FVM_ERR_CUDA 4             /* CUDA runtime error (message has the CUDA string) */
#define FVM_ERR_OUT_OF_MEMORY 5
#define FVM_ERR_NOT_CONVERGED 6    /* iterative solver hit its iteration limit */
#define FVM_ERR_UNSUPPORTED 7      /* condition type not allowed by a template (reference ArgumentError) */
#define FVM_ERR_STEP_LIMIT 8       /* ODE solver hit max_steps or dt underflow */

/* ---- vertex condition codes (per point) ------------------------------------------ */
#define FVM_VERTEX_FREE 0          /* no condition: du = (sum of fluxes)/V + S */
#define FVM_VERTEX_DIRICHLET 1     /* du = 0, u set by the Dirichlet update */
#define FVM_VERTEX_DUDT 2          /* du = a(x, y, t, u) */
#define FVM_VERTEX_NOT_A_VERTEX 3  /* point in no solid triangle: du = 0 */

/* ---- pointer-location flags ------------------------------------------------------- */
#define FVM_PTR_HOST 0             /* host arrays, reference numbering (copied in/out) */
#define FVM_PTR_DEVICE 1           /* device arrays, reference numbering */
#define FVM_PTR_DEVICE_INTERNAL 2  /* device arrays, internal (Hilbert) numbering */
#define FVM_RHS_FORCE_TRIANGLE 16  /* evaluate by the per-triangle flux kernel even for linear forms */
#define FVM_RHS_CONSERVATIVE 32    /* linear forms in difference form sum_j K_ij (u_j - u_i): constant fields
                                      carry exactly zero flux (one more FP64 instruction per neighbour) */

/* ---- precision ---------------------------------------------------------------------- */
#define FVM_FP64 0
#define FVM_FP32 1                 /* FP32 flux assembly / SpMV, FP64 control-volume division and output */

typedef struct fvm_mesh fvm_mesh;
typedef struct fvm_problem fvm_problem;
typedef struct fvm_template fvm_template;

int fvm_version(void);
/* Copies the last error message of the calling thread into buf (NUL-terminated). */
int fvm_last_error(char* buf, size_t len);
/* Number of CUDA devices visible (0 when none); a query, never an error. */
int fvm_device_count(int* count);

/* ---- mesh --------------------------------------------------------------------------- */
/* Replaces FVMGeometry(tri) (src/geometry.jl:99-169) and the triangulation queries of
 * the hot loop: each_solid_triangle (src/equations/triangle_contributions.jl:39),
 * get_boundary_edge_map / get_adjacent (src/equations/boundary_edge_contributions.jl:79,90).
 *   points            [2*npoints]   (x, y) interleaved
 *   triangles         [3*ntri]      counter-clockwise solid triangles
 *   boundary_edges    [2*nbedge]    (i, j) with the domain on the left
 *   boundary_adjacent [nbedge]      k = get_adjacent(tri, i, j), or NULL to look it up
 *   tile_vertices     vertices per tile of the triangle kernel (0 = default)
 *   flags             FVM_MESH_NO_RENUMBER keeps the caller's numbering internally;
 *                     FVM_MESH_HOST_INGEST builds the mesh data on the host */
#define FVM_MESH_NO_RENUMBER 1
/* FVM_MESH_HOST_INGEST builds the geometry, Hilbert order and operator pattern on the host
 * (by default they are built on the device; both builds give identical meshes) */
#define FVM_MESH_HOST_INGEST 2
int fvm_mesh_create(const double* points, int64_t npoints, const int32_t* triangles, int64_t ntri,
                    const int32_t* boundary_edges, const int32_t* boundary_adjacent, int64_t nbedge,
                    int32_t tile_vertices, int32_t flags, fvm_mesh** out);
int fvm_mesh_destroy(fvm_mesh* mesh);
/* info[0..9] = npoints, ntri, nbedge, nvertices, ntiles, ntile_elements, nbedge_elements,
 * tile_vertices, operator_slots (sliced-ELL, padded), operator_nnz (structural). */
int fvm_mesh_info(const fvm_mesh* mesh, int64_t* info);
/* FVMGeometry fields: cv_volumes [npoints] (src/geometry.jl:41,130-135) and, per triangle in
 * the caller's order, TriangleProperties (src/geometry.jl:21-26) as 24 doubles:
 * s1..s9, dual-edge midpoints (3 x (x,y)), unit normals (3 x (x,y)), lengths (3).
 * Either output may be NULL. */
int fvm_mesh_geometry(const fvm_mesh* mesh, double* cv_volumes, double* triangle_props);
/* Points where (x, y) closures are sampled: dual-edge midpoints [ntri*3*2] (edge order
 * (i,j), (j,k), (k,i): src/geometry.jl:149-151) and boundary quarter points [nbedge*2*2]
 * (m_i, m_j: src/equations/control_volumes.jl:47-49). Either output may be NULL. */
int fvm_mesh_sample_points(const fvm_mesh* mesh, double* dual_midpoints, double* quarter_points);
/* perm[internal] = caller index. */
int fvm_mesh_permutation(const fvm_mesh* mesh, int32_t* perm);
/* Reads the device-resident connectivity back and maps it to the caller's numbering:
 * triangles [3*ntri] in the caller's triangle order (rotation as given), boundary
 * elements [3*nbedge] = (i, j, k).  For the bit-exact connectivity check. */
int fvm_mesh_export_connectivity(const fvm_mesh* mesh, int32_t* triangles, int32_t* boundary_elements);

/* ---- problem -------------------------------------------------------------------------- */
/* Device-coded closure forms.  Closures of (x, y) are sampled by the host at the points
 * fvm_mesh_sample_points gives; closures of (u) are polynomials of degree <= 2 in u whose
 * coefficients are (x, y)-sampled: f = c0 + c1 u + c2 u^2.  Arrays are laid out
 * [entity][degree+1].  A NULL array means the form is identically zero. */
typedef struct fvm_problem_desc {
    /* conditions (src/conditions.jl:310-324 after merge_conditions!, :506-544) */
    const int8_t* vertex_code;      /* [npoints] FVM_VERTEX_* */
    const int8_t* bedge_neumann;    /* [nbedge] 1 if the edge has a Neumann condition, else 0 */
    /* diffusion flux q = -D(x, y, u) grad u (src/problem.jl:425-440), D at dual-edge midpoints
     * and boundary quarter points */
    int32_t diffusion_degree;       /* 0, 1 or 2 */
    const double* dual_edge_D;      /* [ntri*3][deg+1] */
    const double* quarter_D;        /* [nbedge*2][deg+1] */
    /* Neumann q.n = a(x, y, u(m)) at the quarter points (boundary_edge_contributions.jl:2-13) */
    int32_t neumann_degree;
    const double* quarter_neumann;  /* [nbedge*2][deg+1] */
    /* source S(x, y, u) at vertices (source_contributions.jl:2-14) */
    int32_t source_degree;
    const double* source;           /* [npoints][deg+1] */
    /* Dudt a(x, y, u) at vertices with code DUDT */
    int32_t dudt_degree;
    const double* dudt;             /* [npoints][deg+1] */
    /* Dirichlet u = a(x, y) at vertices with code DIRICHLET (dirichlet.jl:2-8) */
    const double* dirichlet;        /* [npoints] */
    int32_t precision;              /* FVM_FP64 or FVM_FP32 */
    /* A flux linear in (alpha, beta, gamma) (src/problem.jl:118-163, e.g. the advection-diffusion
     * q = nu u - D grad u with u = alpha x + beta y + gamma):
     *     q = (M0 alpha + M1 beta + M2 gamma, M3 alpha + M4 beta + M5 gamma)
     * with M sampled at the dual-edge midpoints and boundary quarter points.  When given,
     * dual_edge_D / quarter_D and diffusion_degree are ignored.  NULL: the diffusion form. */
    const double* dual_edge_flux;   /* [ntri*3][6] */
    const double* quarter_flux;     /* [nbedge*2][6] */
    /* Values that depend on t through a factor (src/conditions.jl:237-251 conditions a(x, y, t, u, p)
     * and source S(x, y, t, u, p) independent of u): value(x, y, t) = tau_g(t) v_g(x, y) for a time
     * factor from a fixed set, time_factor[g] = {kind, t_ref, a, b}:
     *   kind 1: tau(t) = exp(a (t - t_ref));  kind 2: tau(t) = 1 + a (t - t_ref) + b (t - t_ref)^2.
     * The v_g are added to the static values above (which hold 0 where a value is time-dependent).
     * Linear problems only.  ntime = 0: no time dependence (the arrays may be NULL). */
    int32_t ntime;                  /* at most FVM_MAX_TIME_FACTORS */
    const double* time_factor;      /* [ntime][4] */
    const double* time_dirichlet;   /* [ntime][npoints] Dirichlet values */
    const double* time_neumann;     /* [ntime][nbedge*2] Neumann values q.n at the quarter points */
    const double* time_source;      /* [ntime][npoints] source values on free vertices */
    const double* time_dudt;        /* [ntime][npoints] Dudt values */
    int32_t options;                /* FVM_PROBLEM_* bits */
} fvm_problem_desc;
/* The problem only carries a template's conditions and samples (fvm_template_create): no
 * operator is assembled, and the RHS and time-stepping calls refuse it. */
#define FVM_PROBLEM_CONDITIONS_ONLY 1
#define FVM_MAX_TIME_FACTORS 8

/* Replaces FVMProblem(mesh, BCs, ICs; ...) (src/problem.jl:118-163) together with
 * Conditions(mesh, BCs, ICs) (src/conditions.jl:546-552). */
int fvm_problem_create(fvm_mesh* mesh, const fvm_problem_desc* desc, fvm_problem** out);
int fvm_problem_destroy(fvm_problem* prob);
/* info[0..5] = linear (1 when the folded vertex-neighbour operator evaluates fvm_eqs!),
 * operator nonzeros, operator slots (padded), has constant term, has u^2 term, precision. */
int fvm_problem_info(const fvm_problem* prob, int64_t* info);
/* Reads the device-resident classification back in the caller's numbering. */
int fvm_problem_export_codes(const fvm_problem* prob, int8_t* vertex_code, int8_t* bedge_neumann);

/* Replaces fvm_eqs!(du, u, p, t) (src/equations/main_equations.jl:28-81): triangle fluxes,
 * boundary-edge fluxes and per-vertex source / condition finalisation.  stream is a
 * cudaStream_t (NULL = default stream).  flags: FVM_PTR_* | FVM_RHS_FORCE_TRIANGLE. */
int fvm_rhs(fvm_problem* prob, const double* u, double* du, double t, int32_t flags, void* stream);
/* fvm_rhs for callers that cannot call cudaMalloc: real-time loops whose allocator is frozen
 * after start-up, and hosts that hand all device memory to their own pool (where a cudaMalloc
 * behind the pool's back fails or fragments it).  This entry point has no counterpart in the
 * reference, which has no GPU path.
 *   u, du: device arrays in the caller's numbering.
 *   The mesh may have at most FVM_NOALLOC_MAX_POINTS points; larger meshes are rejected with
 *   FVM_ERR_INVALID_ARGUMENT (use fvm_rhs).
 *   u and du are staged through a fixed 4 MiB device array compiled into the library.  Every
 *   GPU that loads the library holds that array until exit, and all calls share it, so calls
 *   that overlap on the GPU (e.g. on two streams) race.
 *   The first call on each device looks up the array's device address (no allocation).  Make
 *   that first call before any stream capture.
 *   A nonlinear problem's per-triangle data is prepared by its first fvm_rhs call, so make one
 *   fvm_rhs call before using this entry point on such a problem (otherwise
 *   FVM_ERR_INVALID_ARGUMENT).  Call it with the device that was current when the mesh was
 *   created (otherwise FVM_ERR_INVALID_ARGUMENT). */
#define FVM_NOALLOC_MAX_POINTS 262144
int fvm_rhs_noalloc(fvm_problem* prob, const double* u, double* du, double t, void* stream);
/* Fault-path testing of the streamed operator kernel (no counterpart in the reference).  Every
 * wait of the library's kernels is bounded; a wait that runs out sets a bit in a device error
 * word, the kernel drains its copies in flight and returns, and the next synchronising call
 * returns FVM_ERR_CUDA.  This sets, for all later launches of the streamed kernel, the limit of
 * a consumer's wait for a stage (consumer_wait_ns, at least 100; 0 = the default 2 s) and a
 * delay of the producer before its second stage (producer_delay_ns, at most 10 ms; 0 = none),
 * so that a test can make the wait run out.  Not for production use; reset with (0, 0). */
int fvm_test_set_stream_waits(int64_t consumer_wait_ns, int64_t producer_delay_ns);
/* Replaces update_dirichlet_nodes! (src/equations/dirichlet.jl:78-86). */
int fvm_dirichlet_apply(fvm_problem* prob, double* u, double t, int32_t flags, void* stream);

/* ---- post-processing on the device ------------------------------------------------------ */
/* Point location, the step the reference's tutorials take with DelaunayTriangulation's
 * jump_and_march before pl_interpolate: tri_out[q] = the caller index of a solid triangle that
 * holds point (xy[2q], xy[2q+1]) -- the lowest such index, for points on shared edges -- or -1
 * outside the mesh.  xy [nq][2] and tri_out [nq] are host or device arrays (flags FVM_PTR_HOST
 * or FVM_PTR_DEVICE).  The first call builds a uniform grid of the triangles on the device. */
int fvm_mesh_locate(fvm_mesh* mesh, int64_t nq, const double* xy, int64_t* tri_out, int32_t flags, void* stream);
/* Replaces pl_interpolate(prob, T, u, x, y) (src/utils.jl:23-27) for nq points at once:
 * out[q][c] = alpha_c x + beta_c y + gamma_c, the shape-function coefficients of component c of
 * u on triangle tri[q] (a caller index; -1 gives NaN).  u [npoints][ncomp]; u, tri, xy and out
 * are host or device arrays per flags (FVM_PTR_HOST, FVM_PTR_DEVICE; FVM_PTR_DEVICE_INTERNAL
 * takes u in the internal numbering, the other arrays on the device). */
int fvm_pl_interpolate(fvm_mesh* mesh, const double* u, int32_t ncomp, int64_t nq, const int64_t* tri,
                       const double* xy, double* out, int32_t flags, void* stream);

/* ---- time stepping (solve(prob, Tsit5(); saveat), src/solve.jl:167-208) ---------------- */
typedef struct fvm_ode_options {
    double t0, tf;
    double dt;            /* fixed step, or initial step when adaptive (0 = automatic) */
    int32_t adaptive;     /* 0: fixed dt; 1: PI-controlled with the Tsit5 error estimate */
    double abstol, reltol;
    int64_t max_steps;
    const double* saveat; /* [nsave] output times (host); NULL with nsave = 1 saves tf */
    int64_t nsave;
    int32_t use_graph;    /* capture the fixed step in a CUDA graph */
    int32_t precision;    /* FVM_FP64 */
} fvm_ode_options;

typedef struct fvm_ode_stats {
    int64_t naccept, nreject, nrhs;
    double t_final;
    double elapsed_ms;    /* device time of the stepping loop (CUDA events) */
    int32_t driver;       /* FVM_DRIVER_*: which stepping loop ran after the first step */
} fvm_ode_stats;

/* stepping loops (fvm_ode_stats.driver) */
#define FVM_DRIVER_HOST 0          /* host-controlled loop, one launch sequence per step */
#define FVM_DRIVER_FIXED_GRAPH 1   /* fixed steps replayed as one captured CUDA graph */
#define FVM_DRIVER_DEVICE_LOOP 2   /* adaptive: CUDA graph with a conditional WHILE node */
#define FVM_DRIVER_CLUSTER 3       /* adaptive, small sliced-ELL problems: one thread-block cluster */

/* Tsit5 on a generic problem, with the Dirichlet callback after every step
 * (src/solve.jl:133-165).  u0 and out are host arrays in the caller's numbering;
 * out is [nsave][npoints]. */
int fvm_tsit5_solve(fvm_problem* prob, const double* u0, const fvm_ode_options* opt, double* out,
                    fvm_ode_stats* stats, void* stream);

/* ---- implicit stepping (solve(prob, TRBDF2()), the solver of the reference's tutorials) --- */
/* Jacobian-vector product of fvm_eqs! (the derivative that a Newton-Krylov solve of the
 * reference's implicit methods needs, src/solve.jl:50-131 gives its sparsity): jv = J(u) v,
 * exact for every device-coded form.  u, v, jv per flags (FVM_PTR_*). */
int fvm_jvp(fvm_problem* prob, const double* u, const double* v, double* jv, double t, int32_t flags, void* stream);
/* diag J(u), per flags (FVM_PTR_*). */
int fvm_jacobian_diagonal(fvm_problem* prob, const double* u, double* diag, double t, int32_t flags, void* stream);
typedef struct fvm_implicit_stats {
    int64_t newton_iters;     /* simplified-Newton iterations over all stages */
    int64_t krylov_iters;     /* BiCGStab iterations */
    int64_t jvps;             /* Jacobian-vector products */
    int64_t newton_failures;  /* steps retried with a quarter of the step after a Newton failure */
} fvm_implicit_stats;
/* TR-BDF2 (Hosea & Shampine 1996) on the problem, the Dirichlet update after every step:
 * simplified Newton per stage with W = I - d h J(u_n) applied by fvm_jvp and solved by
 * BiCGStab with the diagonal of W as preconditioner; adaptive with TR-BDF2's error estimate,
 * or fixed dt.  Options, u0 and out as fvm_tsit5_solve (use_graph is ignored); istats may be
 * NULL. */
int fvm_trbdf2_solve(fvm_problem* prob, const double* u0, const fvm_ode_options* opt, double* out,
                     fvm_ode_stats* stats, fvm_implicit_stats* istats, void* stream);
/* TR-BDF2 on a DiffusionEquation / LinearReactionDiffusionEquation template, du/dt = A u + b
 * (J = A): solve(template, TRBDF2()) (abstract_templates.jl:58-60). */
int fvm_template_trbdf2_solve(fvm_template* tmpl, const double* u0, const fvm_ode_options* opt, double* out,
                              fvm_ode_stats* stats, fvm_implicit_stats* istats, void* stream);


/* ---- systems of equations (FVMSystem, src/problem.jl:190-365) ---------------------------
 * N coupled components on one mesh.  State is laid out [npoints][neq] (component fastest),
 * the memory order of the reference's N x npoints solution matrix (column-major), in the
 * caller's point numbering.  Each component has its own conditions (vertex codes, Neumann
 * edges), as merge_problem_conditions keeps them (src/problem.jl:336-365).  Device-coded forms:
 *   flux of component r   q_r = -sum_c D_rc(x, y) (alpha_c, beta_c)  (linear, cross-diffusion
 *                         allowed), sampled at the dual-edge midpoints and boundary quarter
 *                         points;
 *   source / Dudt of r    a polynomial of total degree <= 3 in the node's component values,
 *                         sum_m coef_m(x, y) prod_c u_c^exp[m][c];
 *   Neumann value of r    affine in the quarter-point component values, n0 + sum_c n_c u_c(m);
 *   Dirichlet value of r  a(x, y).
 * Arrays are laid out as below; a NULL array means the form is identically zero. */
#define FVM_SYSTEM_MAX_EQ 8
#define FVM_SYSTEM_MAX_TERMS 64   /* non-zero (component, monomial) source / Dudt terms */
typedef struct fvm_system fvm_system;
typedef struct fvm_system_desc {
    int32_t neq;                    /* 1 .. FVM_SYSTEM_MAX_EQ */
    const int8_t* vertex_code;      /* [neq][npoints] FVM_VERTEX_* per component */
    const int8_t* bedge_neumann;    /* [neq][nbedge] 1 if the edge is Neumann for the component */
    const double* dual_edge_D;      /* [neq*neq][ntri*3], block (r, c) at r*neq + c */
    const double* quarter_D;        /* [neq*neq][nbedge*2] */
    int32_t nmono;                  /* monomials of the polynomial forms */
    const int8_t* mono_exp;         /* [nmono][neq] exponents, total degree <= 3 */
    const double* source;           /* [neq][npoints][nmono], used on FREE vertices */
    const double* dudt;             /* [neq][npoints][nmono], used on DUDT vertices */
    const double* quarter_neumann;  /* [neq][nbedge*2][1+neq]: n0, n_1 .. n_neq */
    const double* dirichlet;        /* [neq][npoints] */
    /* Time factors as in fvm_problem_desc, per component: the values v_g are added to the
     * constant terms (Dirichlet values, Neumann n0, the source's and Dudt's constant monomial). */
    int32_t ntime;                  /* at most FVM_MAX_TIME_FACTORS */
    const double* time_factor;      /* [ntime][4] */
    const double* time_dirichlet;   /* [ntime][neq][npoints] */
    const double* time_neumann;     /* [ntime][neq][nbedge*2] */
    const double* time_source;      /* [ntime][neq][npoints] */
    const double* time_dudt;        /* [ntime][neq][npoints] */
} fvm_system_desc;
/* Replaces FVMSystem(prob1, ..., probN) (src/problem.jl:318-334) with merge_problem_conditions
 * (:336-365). */
int fvm_system_create(fvm_mesh* mesh, const fvm_system_desc* desc, fvm_system** out);
int fvm_system_destroy(fvm_system* sys);
/* info[0..6] = neq, coupled (r, c) flux blocks, source / Dudt terms, terms with per-vertex
 * coefficients, Dirichlet entries, has Neumann constants, shared form (1 when every block is a
 * constant multiple of one stored operator: equal conditions, constant diffusivities, Neumann
 * values independent of u). */
int fvm_system_info(const fvm_system* sys, int64_t* info);
/* Replaces fvm_eqs!(du, u, p, t) on an FVMSystem (src/equations/main_equations.jl:38-44 with
 * the system methods of shape_functions.jl:12-19, triangle_contributions.jl:18-25,
 * individual_flux_contributions.jl:35-51, boundary_edge_contributions.jl:15-75,
 * source_contributions.jl:17-66).  u, du [npoints][neq]; flags FVM_PTR_*. */
int fvm_system_rhs(fvm_system* sys, const double* u, double* du, double t, int32_t flags, void* stream);
/* Replaces update_dirichlet_nodes! on an FVMSystem (src/equations/dirichlet.jl:54-61,73-86). */
int fvm_system_dirichlet_apply(fvm_system* sys, double* u, double t, int32_t flags, void* stream);
/* Tsit5 on the system with the Dirichlet callback after every step; u0 [npoints][neq] and
 * out [nsave][npoints][neq] are host arrays in the caller's numbering. */
int fvm_system_tsit5_solve(fvm_system* sys, const double* u0, const fvm_ode_options* opt, double* out,
                           fvm_ode_stats* stats, void* stream);
/* Jacobian-vector product of the system's fvm_eqs!: jv = J(u) v, exact (block operator plus the
 * derivatives of the source / Dudt polynomials).  u, v, jv [npoints][neq] per flags (FVM_PTR_*). */
int fvm_system_jvp(fvm_system* sys, const double* u, const double* v, double* jv, double t, int32_t flags,
                   void* stream);
/* diag J(u), [npoints][neq] per flags (FVM_PTR_*). */
int fvm_system_jacobian_diagonal(fvm_system* sys, const double* u, double* diag, double t, int32_t flags,
                                 void* stream);
/* TR-BDF2 on the system (solve(prob::FVMSystem, TRBDF2()), the integrator of the reference's
 * reaction-diffusion system tutorials), as fvm_trbdf2_solve; u0 [npoints][neq] and out
 * [nsave][npoints][neq] host arrays in the caller's numbering. */
int fvm_system_trbdf2_solve(fvm_system* sys, const double* u0, const fvm_ode_options* opt, double* out,
                            fvm_ode_stats* stats, fvm_implicit_stats* istats, void* stream);

/* ---- steady states (SteadyFVMProblem, src/problem.jl:166-180; solve, src/solve.jl:184-196) --
 * The reference wraps the problem's ODE right-hand side in a SteadyStateProblem and hands it to
 * SteadyStateDiffEq (DynamicSS(alg): integrate in pseudo-time until du/dt vanishes) or to
 * NonlinearSolve (NewtonRaphson: Newton on f(u) = 0).  Both run here on the device:
 *   FVM_STEADY_DYNAMIC  TR-BDF2 (as fvm_trbdf2_solve) from t, the Dirichlet update after every
 *                       step, stopped after the first accepted step whose u passes the test
 *   FVM_STEADY_NEWTON   Newton-Krylov on f(u, t) = 0: (F - J(u)) du = f(u) by BiCGStab with the
 *                       Jacobi preconditioner, F the identity on the rows the problem fixes
 *                       (Dirichlet, points outside the mesh), so those rows keep their values;
 *                       the Dirichlet update at t is applied to the initial guess first
 * Test on the returned u: max|f(u)| <= abstol, or max|f(u)| <= reltol max|f(u) + u|.  u0 and out
 * are host arrays in the caller's numbering (systems: [npoints][neq]).  Not converged within
 * max_iters (or tmax): FVM_ERR_NOT_CONVERGED, with the last iterate in out and stats filled. */
#define FVM_STEADY_DYNAMIC 0
#define FVM_STEADY_NEWTON 1
typedef struct fvm_steady_options {
    int32_t method;                 /* FVM_STEADY_* */
    double abstol, reltol;          /* the test above */
    double t;                       /* Newton: the time f is evaluated at; DynamicSS: the pseudo-time start */
    double tmax;                    /* DynamicSS: pseudo-time limit (INFINITY allowed) */
    double ode_abstol, ode_reltol;  /* DynamicSS: the TR-BDF2 step tolerances */
    int64_t max_iters;              /* Newton iterations or DynamicSS steps; 0: 50 or 100000 */
} fvm_steady_options;
typedef struct fvm_steady_stats {
    int64_t iterations;             /* Newton iterations, or accepted TR-BDF2 steps */
    int64_t krylov_iters, jvps, nrhs;
    double residual;                /* max|f(u)| at the returned u */
    double t_final;                 /* DynamicSS: the pseudo-time reached */
    double elapsed_ms;              /* device time (CUDA events) */
} fvm_steady_stats;
int fvm_steady_solve(fvm_problem* prob, const double* u0, const fvm_steady_options* opt, double* out,
                     fvm_steady_stats* stats, void* stream);
int fvm_system_steady_solve(fvm_system* sys, const double* u0, const fvm_steady_options* opt, double* out,
                            fvm_steady_stats* stats, void* stream);

/* ---- batched instances (many parameter sets on one mesh) -------------------------------- */
/* B instances of one linear problem that differ in their diffusion field D_b(x, y), the
 * batched counterpart of solving B FVMProblems (an EnsembleProblem over D in the reference).
 * State is laid out [npoints][batch] (batch fastest) so the mesh is read once for all
 * instances.  prob supplies conditions, Neumann / source / Dudt / Dirichlet forms (shared);
 * its own D is ignored.
 *   dual_edge_D [batch][ntri*3], quarter_D [batch][nbedge*2] (NULL when no boundary edge uses D)
 *   precision   FVM_FP64, or FVM_FP32 (FP32 values, state and accumulation) */
typedef struct fvm_batch fvm_batch;
int fvm_batch_create(fvm_problem* prob, int32_t batch, const double* dual_edge_D, const double* quarter_D,
                     int32_t precision, fvm_batch** out);
int fvm_batch_destroy(fvm_batch* b);
/* du_b = fvm_eqs!(u_b) for every instance; u, du [npoints][batch] of the batch's precision, in
 * the caller's numbering (FVM_PTR_HOST / FVM_PTR_DEVICE) or internal (FVM_PTR_DEVICE_INTERNAL). */
int fvm_batch_rhs(fvm_batch* b, const void* u, void* du, double t, int32_t flags, void* stream);
/* Fixed-step Tsit5 on every instance, one captured CUDA graph per step, Dirichlet update after
 * each step.  u0 [npoints][batch] and out [nsave][npoints][batch] are host FP64 arrays. */
int fvm_batch_tsit5_solve(fvm_batch* b, const double* u0, const fvm_ode_options* opt, double* out,
                          fvm_ode_stats* stats, void* stream);
/* Autotuned launch shape of the batched operator: tune[0..2] = block size, instances per thread,
 * grid blocks (chosen by timing the candidates on the first batched call). */
int fvm_batch_tuning(const fvm_batch* b, int32_t* tune);

/* ---- linear templates (src/specific_problems/) ------------------------------------------- */
#define FVM_TEMPLATE_DIFFUSION 0                 /* diffusion_equation.jl:69-101 */
#define FVM_TEMPLATE_LINEAR_REACTION_DIFFUSION 1 /* linear_reaction_diffusion_equations.jl:76-125 */
#define FVM_TEMPLATE_POISSON 2                   /* poissons_equation.jl:58-88 */
#define FVM_TEMPLATE_MEAN_EXIT_TIME 3            /* mean_exit_time.jl:57-94 */

/* Assembles A and b of a template straight into the device operator (no dense matrix).
 * The problem supplies D (degree 0), the source (Poisson f / reaction coefficient as
 * source c0 / c1), Neumann values, Dudt and Dirichlet values, all sampled with
 * t = u = nothing as the reference does. */
int fvm_template_create(fvm_problem* prob, int32_t kind, fvm_template** out);
int fvm_template_destroy(fvm_template* tmpl);
/* A in CSR (caller numbering, sorted columns, structural zeros dropped) and b.
 * Call with col = val = NULL to get nnz. */
int fvm_template_export(const fvm_template* tmpl, int64_t* nnz, int32_t* rowptr, int32_t* col,
                        double* val, double* b);
/* du = A u + b: the MatrixOperator product (diffusion_equation.jl:93-94). precision:
 * FVM_FP64 or FVM_FP32 (FP32 values, FP32 accumulation). */
int fvm_template_apply(fvm_template* tmpl, const double* u, double* du, int32_t precision,
                       int32_t flags, void* stream);
/* Tsit5 on du/dt = A u + b (the template's ODEProblem). */
int fvm_template_tsit5_solve(fvm_template* tmpl, const double* u0, const fvm_ode_options* opt,
                             double* out, fvm_ode_stats* stats, void* stream);

/* ---- steady solve (LinearProblem(A, b) + solve, poissons_equation.jl:81, mean_exit_time.jl:76) */
#define FVM_SOLVER_AUTO 0      /* CG when the reduced operator is symmetric, else BiCGStab */
#define FVM_SOLVER_CG 1
#define FVM_SOLVER_BICGSTAB 2
#define FVM_PRECOND_JACOBI 0
#define FVM_PRECOND_CHEBYSHEV 1
#define FVM_SOLVE_FP64 0       /* plain FP64 Krylov */
#define FVM_SOLVE_MIXED 1      /* FP32 inner iterations, FP64 reliable residual / refinement */
#define FVM_SOLVE_FP32_PRECOND 2 /* FP64 Krylov iteration and arithmetic; the Chebyshev
                                  * preconditioner reads its operator values stored in FP32 */

typedef struct fvm_solver_options {
    double rtol;           /* on ||b - A x|| / ||b|| with the reference operator, FP64 */
    int64_t max_iters;
    int32_t method;        /* FVM_SOLVER_* */
    int32_t precond;       /* FVM_PRECOND_* */
    int32_t cheb_degree;
    int32_t mode;          /* FVM_SOLVE_FP64 or FVM_SOLVE_MIXED */
    double inner_reduction;/* residual reduction between FP64 reliable updates (mixed), e.g. 1e-2 */
} fvm_solver_options;

typedef struct fvm_solver_stats {
    int64_t iterations;     /* Krylov iterations (all precisions) */
    int64_t refinements;    /* FP64 residual recomputations */
    double rel_residual;    /* final ||b - A x|| / ||b|| (FP64, reference operator) */
    double elapsed_ms;      /* device time (CUDA events) */
    int32_t method_used;
    int32_t symmetric;
    int32_t fallback_fp64;  /* mixed mode finished in FP64 after the FP32 inner iteration stalled */
} fvm_solver_stats;

/* Solves A x = b of a Poisson or mean-exit-time template.  x: in = initial guess,
 * out = solution, FVM_PTR_HOST or FVM_PTR_DEVICE (caller numbering). */
int fvm_template_steady_solve(fvm_template* tmpl, double* x, const fvm_solver_options* opt,
                              fvm_solver_stats* stats, int32_t flags, void* stream);

/* ---- differentiation: discrete adjoint of the time-dependent templates ---------------------
 * The reference differentiates its solves by running them under ForwardDiff (its closures are
 * generic in the number type) or through SciMLSensitivity; this is the device-side counterpart
 * for the DiffusionEquation / LinearReactionDiffusionEquation templates.  A batch of instances
 * shares the template's mesh, conditions and b; instance i has the diffusion field D_i(x, y) =
 * the P1 interpolant of per-vertex values exp(theta[v][i]) (a log-diffusivity field), sampled
 * where the reference samples D (dual-edge midpoints, boundary quarter points).  The template's
 * own D is ignored.  b must not depend on D (no Neumann edges).  Arrays are [npoints][batch]
 * (batch fastest), FP64, host (FVM_PTR_HOST) or device (FVM_PTR_DEVICE) in the caller's
 * numbering.  Time stepping is fixed-step Tsit5 (the templates' solve with adaptive = false). */
typedef struct fvm_adjoint fvm_adjoint;
typedef struct fvm_adjoint_stats {
    int64_t steps;            /* time steps of the forward solve */
    int64_t checkpoints;      /* states kept by the forward pass */
    int64_t rhs_evals;        /* batched A u + b products (forward pass and recomputation) */
    int64_t transpose_evals;  /* batched A^T products of the reverse pass */
    double forward_ms;        /* device time of the forward pass */
    double reverse_ms;        /* device time of the reverse pass, recomputation included */
} fvm_adjoint_stats;
int fvm_adjoint_create(fvm_template* tmpl, int32_t batch, fvm_adjoint** out);
int fvm_adjoint_destroy(fvm_adjoint* adj);
/* theta [npoints][batch]: assembles every instance's operator on the device. */
int fvm_adjoint_set_log_diffusion(fvm_adjoint* adj, const double* theta, int32_t flags, void* stream);
/* du = A(theta) u + b for every instance. */
int fvm_adjoint_rhs(fvm_adjoint* adj, const double* u, double* du, int32_t flags, void* stream);
/* u(T) after nsteps Tsit5 steps of dt from u0. */
int fvm_adjoint_forward(fvm_adjoint* adj, const double* u0, double dt, int64_t nsteps, double* uT,
                        int32_t flags, void* stream);
/* Vector-Jacobian product of the solve: theta_bar = (d uT / d theta)^T uT_bar and
 * u0_bar = (d uT / d u0)^T uT_bar (u0_bar may be NULL), by the discrete adjoint of the Tsit5
 * steps; the forward pass keeps u every checkpoint_every steps and the reverse pass recomputes
 * the states in between. */
int fvm_adjoint_pullback(fvm_adjoint* adj, const double* u0, double dt, int64_t nsteps, int32_t checkpoint_every,
                         const double* uT_bar, double* theta_bar, double* u0_bar, fvm_adjoint_stats* stats,
                         int32_t flags, void* stream);
/* loss[i] = sum_v (uT[v][i] - u_obs[v][i])^2 (host array [batch]) and its gradients with
 * respect to theta and u0 (u0_bar may be NULL). */
int fvm_adjoint_loss_grad(fvm_adjoint* adj, const double* u0, const double* u_obs, double dt, int64_t nsteps,
                          int32_t checkpoint_every, double* loss, double* theta_bar, double* u0_bar,
                          fvm_adjoint_stats* stats, int32_t flags, void* stream);
/* Vector-Jacobian product of the right-hand side f(u, theta) = A(theta) u + b:
 * u_bar = A^T w (may be NULL), theta_bar = (d f / d theta)^T w. */
int fvm_adjoint_rhs_vjp(fvm_adjoint* adj, const double* u, const double* w, double* u_bar, double* theta_bar,
                        int32_t flags, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* FVM_GPU_H */
