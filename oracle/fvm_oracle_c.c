/*
 * C restatement of the reference's CPU fvm_eqs! (TEST / BASELINE INFRASTRUCTURE).
 *
 * Only the tests and the CPU-baseline leg of bench.py load this file's library.  It follows
 * FiniteVolumeMethod.jl 1.2.3 (paths relative to the reference project root):
 *   serial_fvm_eqs!    src/equations/main_equations.jl:38-44
 *   parallel_fvm_eqs!  src/equations/main_equations.jl:47-81 (per-thread duplicated du, then
 *                      combine_duplicated_du!)
 *   triangle fluxes    src/equations/triangle_contributions.jl:2-15,28-35;
 *                      individual_flux_contributions.jl:2-6,27-33; shape_functions.jl:2-9;
 *                      construct_flux_function src/problem.jl:425-440
 *   boundary edges     src/equations/boundary_edge_contributions.jl:2-13,41-48,61-65,77-86;
 *                      control_volumes.jl:41-56
 *   sources            src/equations/source_contributions.jl:2-14,33-47
 * Geometry (TriangleProperties, 24 doubles per triangle) comes in precomputed as
 * FVMGeometry stores it (src/geometry.jl:99-169).  The diffusion closure is evaluated at
 * every dual edge on every call, as the reference's flux closure is.  Unlike the reference,
 * triangles are visited by index rather than through Dict lookups, so this restatement is
 * faster than the Julia original.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* closures of the benchmark configurations: D(x, y, t, u, p) */
enum { ORC_D_CONST = 0, ORC_D_SINE = 1, ORC_D_JUMP = 2 };

static inline double closure_D(int kind, const double* p, double x, double y, double t, double u) {
    (void)t;
    (void)u;
    switch (kind) {
        case ORC_D_SINE: return 1.0 + p[0] * sin(2.0 * M_PI * x) * sin(2.0 * M_PI * y);
        case ORC_D_JUMP: return (x * x + y * y < 0.25) ? p[0] : p[1];
        default: return p[0];
    }
}

typedef struct {
    int64_t np, nt, nbe;
    const int32_t* tri;     /* [3*nt] */
    const double* props;    /* [24*nt] s1..s9, mid(3x2), nrm(3x2), len(3) */
    const double* pts;      /* [2*np] */
    const double* vol;      /* [np] */
    const int32_t* bedge;   /* [3*nbe] i, j, stored triangle index */
    const int8_t* code;     /* [np] 0 free, 1 Dirichlet, 2 Dudt (value 0 here), 3 not a vertex */
    int d_kind;
    double d_param[4];
} orc_problem;

static inline void triangle_update(const orc_problem* P, int64_t t, const double* u, double* du, double tt) {
    const int32_t* T = P->tri + 3 * t;
    const double* pr = P->props + 24 * t;
    int32_t i = T[0], j = T[1], k = T[2];
    double ui = u[i], uj = u[j], uk = u[k];
    double a = pr[0] * ui + pr[1] * uj + pr[2] * uk;
    double b = pr[3] * ui + pr[4] * uj + pr[5] * uk;
    double g = pr[6] * ui + pr[7] * uj + pr[8] * uk;
    double Q[3];
    for (int e = 0; e < 3; ++e) {
        double x = pr[9 + 2 * e], y = pr[10 + 2 * e];
        double uu = a * x + b * y + g;
        double D = closure_D(P->d_kind, P->d_param, x, y, tt, uu);
        double qx = -D * a, qy = -D * b;
        double qn = qx * pr[15 + 2 * e] + qy * pr[16 + 2 * e];
        Q[e] = qn * pr[21 + e];
    }
    du[i] = du[i] + Q[2] - Q[0];
    du[j] = du[j] + Q[0] - Q[1];
    du[k] = du[k] + Q[1] - Q[2];
}

static inline void bedge_update(const orc_problem* P, int64_t e, const double* u, double* du, double tt) {
    int32_t i = P->bedge[3 * e], j = P->bedge[3 * e + 1], t = P->bedge[3 * e + 2];
    const int32_t* T = P->tri + 3 * (int64_t)t;
    const double* pr = P->props + 24 * (int64_t)t;
    double u0 = u[T[0]], u1 = u[T[1]], u2 = u[T[2]];
    double a = pr[0] * u0 + pr[1] * u1 + pr[2] * u2;
    double b = pr[3] * u0 + pr[4] * u1 + pr[5] * u2;
    double g = pr[6] * u0 + pr[7] * u1 + pr[8] * u2;
    double px = P->pts[2 * i], py = P->pts[2 * i + 1], qx = P->pts[2 * j], qy = P->pts[2 * j + 1];
    double lij = sqrt((qx - px) * (qx - px) + (qy - py) * (qy - py));
    double nx = (qy - py) / lij, ny = -(qx - px) / lij;
    double mijx = (px + qx) / 2, mijy = (py + qy) / 2;
    double mix = (px + mijx) / 2, miy = (py + mijy) / 2;
    double mjx = (qx + mijx) / 2, mjy = (qy + mijy) / 2;
    double l = sqrt((mijx - px) * (mijx - px) + (mijy - py) * (mijy - py));
    double Di = closure_D(P->d_kind, P->d_param, mix, miy, tt, a * mix + b * miy + g);
    double Dj = closure_D(P->d_kind, P->d_param, mjx, mjy, tt, a * mjx + b * mjy + g);
    double q1 = (-Di * a * nx + -Di * b * ny) * l;
    double q2 = (-Dj * a * nx + -Dj * b * ny) * l;
    du[i] = du[i] - q1;
    du[j] = du[j] - q2;
}

static inline void source_update(const orc_problem* P, int64_t i, double* du) {
    int c = P->code[i];
    if (c == 0)
        du[i] = du[i] / P->vol[i];
    else
        du[i] = 0.0;
}

void orc_rhs_serial(const orc_problem* P, const double* u, double* du, double t) {
    memset(du, 0, sizeof(double) * P->np);
    for (int64_t q = 0; q < P->nt; ++q) triangle_update(P, q, u, du, t);
    for (int64_t e = 0; e < P->nbe; ++e) bedge_update(P, e, u, du, t);
    for (int64_t i = 0; i < P->np; ++i) source_update(P, i, du);
}

/* parallel_fvm_eqs!: chunk c accumulates into column c of dup (np x nthreads), then the
 * columns are summed into du and the per-vertex sources run in parallel. */
void orc_rhs_threaded(const orc_problem* P, const double* u, double* du, double t, int nthreads, double* dup) {
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
    nthreads = 1;
#endif
    const int64_t np = P->np;
    memset(du, 0, sizeof(double) * np);
#pragma omp parallel num_threads(nthreads)
    {
#ifdef _OPENMP
        int c = omp_get_thread_num();
        int nth = omp_get_num_threads();
#else
        int c = 0, nth = 1;
#endif
        double* col = dup + (int64_t)c * np;
        memset(col, 0, sizeof(double) * np);
        int64_t t0 = P->nt * c / nth, t1 = P->nt * (c + 1) / nth;
        for (int64_t q = t0; q < t1; ++q) triangle_update(P, q, u, col, t);
        int64_t e0 = P->nbe * c / nth, e1 = P->nbe * (c + 1) / nth;
        for (int64_t e = e0; e < e1; ++e) bedge_update(P, e, u, col, t);
#pragma omp barrier
        int64_t v0 = np * c / nth, v1 = np * (c + 1) / nth;
        for (int w = 0; w < nth; ++w) {
            const double* cw = dup + (int64_t)w * np;
            for (int64_t i = v0; i < v1; ++i) du[i] += cw[i];
        }
        for (int64_t i = v0; i < v1; ++i) source_update(P, i, du);
    }
}

/* ---- FVMSystem: the Gray-Scott tutorial system ------------------------------------------
 * (docs/src/literate_tutorials/gray_scott_model_turing_patterns_from_a_coupled_reaction_diffusion_system.jl)
 * evaluated the way the reference evaluates an FVMSystem:
 *   alpha, beta, gamma tuples per triangle      src/equations/shape_functions.jl:12-19
 *   every component's flux closure per dual edge individual_flux_contributions.jl:35-51
 *   update_du! per component                     triangle_contributions.jl:18-25
 *   boundary edges: all fluxes evaluated, then the (zero) Neumann value replaces them
 *                                                boundary_edge_contributions.jl:15-75
 *   sources per component on free vertices       source_contributions.jl:17-30,49-66
 *   parallel_fvm_eqs! with duplicated du         main_equations.jl:47-81
 * State [point][component] (the reference's 2 x npoints matrix). */
typedef struct {
    double eps[2]; /* u_q = -eps_1 (alpha[1], beta[1]), v_q = -eps_2 (alpha[2], beta[2]) */
    double b, d;   /* u_S = b (1 - u) - u v^2, v_S = -d v + u v^2 */
} orc_gray_scott;

static inline void gs_flux(const orc_gray_scott* G, const double* a, const double* b, double q[2][2]) {
    q[0][0] = -a[0] * G->eps[0];
    q[0][1] = -b[0] * G->eps[0];
    q[1][0] = -a[1] * G->eps[1];
    q[1][1] = -b[1] * G->eps[1];
}

static inline void gs_triangle(const orc_problem* P, const orc_gray_scott* G, int64_t t, const double* u, double* du) {
    const int32_t* T = P->tri + 3 * t;
    const double* pr = P->props + 24 * t;
    int32_t i = T[0], j = T[1], k = T[2];
    double a[2], b[2], g[2], Q[2][3];
    for (int v = 0; v < 2; ++v) {
        double ui = u[2 * i + v], uj = u[2 * j + v], uk = u[2 * k + v];
        a[v] = pr[0] * ui + pr[1] * uj + pr[2] * uk;
        b[v] = pr[3] * ui + pr[4] * uj + pr[5] * uk;
        g[v] = pr[6] * ui + pr[7] * uj + pr[8] * uk;
    }
    (void)g;
    for (int e = 0; e < 3; ++e) {
        double q[2][2];
        gs_flux(G, a, b, q);
        for (int v = 0; v < 2; ++v) Q[v][e] = (q[v][0] * pr[15 + 2 * e] + q[v][1] * pr[16 + 2 * e]) * pr[21 + e];
    }
    for (int v = 0; v < 2; ++v) {
        du[2 * i + v] = du[2 * i + v] + Q[v][2] - Q[v][0];
        du[2 * j + v] = du[2 * j + v] + Q[v][0] - Q[v][1];
        du[2 * k + v] = du[2 * k + v] + Q[v][1] - Q[v][2];
    }
}

static inline void gs_bedge(const orc_problem* P, const orc_gray_scott* G, int64_t e, const double* u, double* du) {
    int32_t i = P->bedge[3 * e], j = P->bedge[3 * e + 1], t = P->bedge[3 * e + 2];
    const int32_t* T = P->tri + 3 * (int64_t)t;
    const double* pr = P->props + 24 * (int64_t)t;
    double a[2], b[2];
    for (int v = 0; v < 2; ++v) {
        double u0 = u[2 * T[0] + v], u1 = u[2 * T[1] + v], u2 = u[2 * T[2] + v];
        a[v] = pr[0] * u0 + pr[1] * u1 + pr[2] * u2;
        b[v] = pr[3] * u0 + pr[4] * u1 + pr[5] * u2;
    }
    double px = P->pts[2 * i], py = P->pts[2 * i + 1], qx = P->pts[2 * j], qy = P->pts[2 * j + 1];
    double mijx = (px + qx) / 2, mijy = (py + qy) / 2;
    double l = sqrt((mijx - px) * (mijx - px) + (mijy - py) * (mijy - py));
    double q[2][2];
    gs_flux(G, a, b, q); /* at m_i, then replaced by the zero Neumann value */
    gs_flux(G, a, b, q); /* at m_j */
    for (int v = 0; v < 2; ++v) {
        du[2 * i + v] = du[2 * i + v] - 0.0 * l;
        du[2 * j + v] = du[2 * j + v] - 0.0 * l;
    }
}

static inline void gs_source(const orc_problem* P, const orc_gray_scott* G, int64_t i, const double* u, double* du) {
    if (P->code[i] != 0) {
        du[2 * i] = du[2 * i + 1] = 0.0;
        return;
    }
    double uu = u[2 * i], vv = u[2 * i + 1];
    du[2 * i] = du[2 * i] / P->vol[i] + (G->b * (1 - uu) - uu * vv * vv);
    du[2 * i + 1] = du[2 * i + 1] / P->vol[i] + (-G->d * vv + uu * vv * vv);
}

void orc_gray_scott_rhs_threaded(const orc_problem* P, const orc_gray_scott* G, const double* u, double* du,
                                 int nthreads, double* dup) {
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
    nthreads = 1;
#endif
    const int64_t n = 2 * P->np;
    memset(du, 0, sizeof(double) * n);
#pragma omp parallel num_threads(nthreads)
    {
#ifdef _OPENMP
        int c = omp_get_thread_num();
        int nth = omp_get_num_threads();
#else
        int c = 0, nth = 1;
#endif
        double* col = dup + (int64_t)c * n;
        memset(col, 0, sizeof(double) * n);
        int64_t t0 = P->nt * c / nth, t1 = P->nt * (c + 1) / nth;
        for (int64_t q = t0; q < t1; ++q) gs_triangle(P, G, q, u, col);
        int64_t e0 = P->nbe * c / nth, e1 = P->nbe * (c + 1) / nth;
        for (int64_t e = e0; e < e1; ++e) gs_bedge(P, G, e, u, col);
#pragma omp barrier
        int64_t v0 = P->np * c / nth, v1 = P->np * (c + 1) / nth;
        for (int w = 0; w < nth; ++w) {
            const double* cw = dup + (int64_t)w * n;
            for (int64_t i = 2 * v0; i < 2 * v1; ++i) du[i] += cw[i];
        }
        for (int64_t i = v0; i < v1; ++i) gs_source(P, G, i, u, du);
    }
}

/* ---- steady linear solve on the host cores (CPU baseline of the steady templates) --------
 * The reference solves PoissonsEquation / MeanExitTimeProblem as LinearProblem(A, b)
 * (src/specific_problems/poissons_equation.jl:81, mean_exit_time.jl:76) with a sparse direct
 * method.  This baseline is a threaded FP64 BiCGStab with a Jacobi preconditioner (right
 * preconditioning, van der Vorst 1992) on the CSR matrix A, stopped when the true residual
 * ||b - A x|| / ||b|| reaches rtol (or after max_seconds): the same method and stopping test as
 * the GPU's plain FP64 solve, on all host threads, with the inner products summed in a fixed
 * order.  stats = {iterations, relative residual, converged}. */

/* Sum of the threads' partials in thread order (deterministic for a given thread count,
 * unlike an OpenMP reduction clause, whose combination order is unspecified). */
static double ordered_sum(const double* part, int nth, int q) {
    double s = 0.0;
    for (int c = 0; c < nth; ++c) s += part[4 * c + q];
    return s;
}

void orc_steady_bicgstab(int64_t n, const int64_t* rp, const int32_t* ci, const double* va, const double* b,
                         const double* w, double bnorm, double* x, double rtol, int64_t maxit, double max_seconds,
                         int nthreads, double* work, double* stats) {
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
    nthreads = 1;
#endif
    double *r = work, *rh = work + n, *p = work + 2 * n, *v = work + 3 * n, *ph = work + 4 * n, *sh = work + 5 * n,
           *t = work + 6 * n, *dinv = work + 7 * n;
    double part[4 * 512];
    if (nthreads > 512) nthreads = 512;
    /* the stopping norm ||w (b - A x)|| against rtol * bnorm (w = NULL: the plain 2-norm and
     * bnorm = ||b||) */
    double bn2 = 0.0;
    for (int64_t i = 0; i < n; ++i) bn2 += (w ? w[i] * b[i] : b[i]) * (w ? w[i] * b[i] : b[i]);
    if (!(bnorm > 0)) bnorm = sqrt(bn2);
    const double tol = rtol * bnorm;
    for (int64_t i = 0; i < n; ++i) {
        double d = 0.0;
        for (int64_t q = rp[i]; q < rp[i + 1]; ++q)
            if (ci[q] == i) d = va[q];
        dinv[i] = d != 0.0 ? 1.0 / d : 1.0;
    }
    int64_t it = 0;
    double rn = 0.0;
    int converged = 0;
    double rho = 1.0, alpha = 1.0, omega = 1.0;
    int restart = 1, stop = 0;
#ifdef _OPENMP
    const double t_start = omp_get_wtime();
#endif
#pragma omp parallel num_threads(nthreads)
    {
#ifdef _OPENMP
        const int c = omp_get_thread_num(), nth = omp_get_num_threads();
#else
        const int c = 0, nth = 1;
#endif
        /* each thread owns the contiguous rows [i0, i1) in every loop */
        const int64_t i0 = n * c / nth, i1 = n * (c + 1) / nth;
        double* my = part + 4 * c;
        while (!stop) {
            if (restart) {
                double a0 = 0.0;
                for (int64_t i = i0; i < i1; ++i) {
                    double sacc = 0.0;
                    for (int64_t q = rp[i]; q < rp[i + 1]; ++q) sacc += va[q] * x[ci[q]];
                    r[i] = b[i] - sacc;
                    rh[i] = r[i];
                    p[i] = v[i] = 0.0;
                    const double wr = w ? w[i] * r[i] : r[i];
                    a0 += wr * wr;
                }
                my[0] = a0;
#pragma omp barrier
#pragma omp single
                {
                    rn = sqrt(ordered_sum(part, nth, 0));
                    rho = alpha = omega = 1.0;
                    restart = 0;
                    if (rn <= tol) {
                        converged = 1;
                        stop = 1;
                    } else if (it >= maxit) {
                        stop = 1;
                    }
#ifdef _OPENMP
                    if (omp_get_wtime() - t_start > max_seconds) stop = 1;
#endif
                }
                if (stop) break;
            }
            double a0 = 0.0;
            for (int64_t i = i0; i < i1; ++i) a0 += rh[i] * r[i];
            my[0] = a0;
#pragma omp barrier
            const double rho_new = ordered_sum(part, nth, 0);
            const double beta = (rho_new / rho) * (alpha / omega);
            for (int64_t i = i0; i < i1; ++i) {
                p[i] = r[i] + beta * (p[i] - omega * v[i]);
                ph[i] = dinv[i] * p[i];
            }
#pragma omp barrier
            a0 = 0.0;
            for (int64_t i = i0; i < i1; ++i) {
                double sacc = 0.0;
                for (int64_t q = rp[i]; q < rp[i + 1]; ++q) sacc += va[q] * ph[ci[q]];
                v[i] = sacc;
                a0 += rh[i] * sacc;
            }
            my[1] = a0;
#pragma omp barrier
            const double al = rho_new / ordered_sum(part, nth, 1);
            for (int64_t i = i0; i < i1; ++i) {
                r[i] = r[i] - al * v[i]; /* s */
                sh[i] = dinv[i] * r[i];
            }
#pragma omp barrier
            double a1 = 0.0, a2 = 0.0;
            for (int64_t i = i0; i < i1; ++i) {
                double sacc = 0.0;
                for (int64_t q = rp[i]; q < rp[i + 1]; ++q) sacc += va[q] * sh[ci[q]];
                t[i] = sacc;
                a1 += sacc * r[i];
                a2 += sacc * sacc;
            }
            my[2] = a1;
            my[3] = a2;
#pragma omp barrier
            const double tt = ordered_sum(part, nth, 3);
            const double om = tt > 0.0 ? ordered_sum(part, nth, 2) / tt : 0.0;
            /* a breakdown (non-finite step) leaves x as it is and restarts from its residual */
            const int good = isfinite(al) && isfinite(om);
            double a3 = 0.0;
            if (good)
                for (int64_t i = i0; i < i1; ++i) {
                    x[i] += al * ph[i] + om * sh[i];
                    r[i] = r[i] - om * t[i];
                    const double wr = w ? w[i] * r[i] : r[i];
                    a3 += wr * wr;
                }
            else
                a3 = NAN;
            my[0] = a3;
#pragma omp barrier
#pragma omp single
            {
                const double rr = ordered_sum(part, nth, 0);
                rho = rho_new;
                alpha = al;
                omega = om;
                ++it;
                /* recurrence converged (or broke down): confirm with the true residual */
                if (sqrt(rr) <= tol || !(om != 0.0) || !isfinite(rr) || it >= maxit) restart = 1;
#ifdef _OPENMP
                if (it % 64 == 0 && omp_get_wtime() - t_start > max_seconds) restart = 1;
#endif
            }
        }
    }
    stats[0] = (double)it;
    stats[1] = bnorm > 0 ? rn / bnorm : rn;
    stats[2] = (double)converged;
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
