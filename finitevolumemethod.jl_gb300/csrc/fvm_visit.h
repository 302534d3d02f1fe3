// The linear-term visitor of the generic RHS as a template, so an assembly's emit callback is
// inlined (tens of millions of calls on a 1M-vertex mesh).  Host code only.
#pragma once
#include "fvm_internal.h"
#include <cmath>

namespace fvm {

// Linear terms of the generic RHS (fvm_eqs!).  Row i of a FREE vertex is
// (sum of triangle and boundary fluxes)/V_i + S_i (triangle_contributions.jl:10-15,
// boundary_edge_contributions.jl:61-65, source_contributions.jl:41), every flux linear in u:
//   triangle dual edge e of T = (a, b, c): Q_e = -D_e l_e (alpha n_x + beta n_y)
//   boundary half edge (non-Neumann):      Q_h = -D_h l_h (alpha n_x + beta n_y)
//   boundary half edge (Neumann, a = n0 + n1 u(m)): Q_h = l_h (n0 + n1 u(m)).
// With a linear flux q = M (alpha, beta, gamma) the dual-edge and half-edge fluxes are
//   Q = l ((n_x M0 + n_y M3) alpha + (n_x M1 + n_y M4) beta + (n_x M2 + n_y M5) gamma),
// alpha, beta, gamma being s1..s9 combinations of the triangle's values (shape_functions.jl:2-9);
// the alpha, beta part sums to zero along a row (a flux term), the gamma part does not.
// The visitor reports each coefficient as emit(row, col, coef, didx, flux) (caller numbering):
// the contribution to A_row,col is coef * D[didx] when didx >= 0 (D indexed over the dual edges,
// 3 per triangle, then the boundary quarter points, 2 per edge), coef otherwise.  `flux` marks
// dual-edge fluxes, whose coefficients along a row sum to zero.  Constant terms go to b,
// quadratic ones to q; rowscale is 1/V on FREE rows, 1 on Dudt rows.
template <class Emit>
void visit_linear_terms(const fvm_problem* p, Emit&& emit, std::vector<double>& b, std::vector<double>& q,
                        std::vector<double>& rowscale) {
    const fvm_mesh* m = p->mesh;
    b.assign(m->np, 0.0);
    q.assign(m->np, 0.0);
    rowscale.assign(m->np, 0.0);
    // l (n . q) per unit alpha, beta, gamma of a linear flux sampled as M[6] at the point
    auto nq = [](const double* M, double nx, double ny, double g[3]) {
        g[0] = nx * M[0] + ny * M[3];
        g[1] = nx * M[1] + ny * M[4];
        g[2] = nx * M[2] + ny * M[5];
    };
    for (int64_t t = 0; t < m->nt; ++t) {
        const int32_t* w = &m->tri[3 * t];
        const double* pr = &m->props[24 * t];
        for (int e = 0; e < 3; ++e) {
            int32_t e1 = w[e], e2 = w[(e + 1) % 3];
            double l = pr[21 + e], nx = pr[15 + 2 * e], ny = pr[16 + 2 * e];
            bool f1 = p->code[e1] == FVM_VERTEX_FREE, f2 = p->code[e2] == FVM_VERTEX_FREE;
            if (p->flux_linear) {  // e1 loses Q_e, e2 gains it
                double g[3];
                nq(&p->dualM[6 * (3 * t + e)], nx, ny, g);
                for (int v = 0; v < 3; ++v) {
                    const double cg = l * (g[0] * pr[v] + g[1] * pr[3 + v]), cz = l * g[2] * pr[6 + v];
                    if (f1) {
                        emit(e1, w[v], -cg / m->vol[e1], -1, true);
                        if (cz != 0) emit(e1, w[v], -cz / m->vol[e1], -1, false);
                    }
                    if (f2) {
                        emit(e2, w[v], cg / m->vol[e2], -1, true);
                        if (cz != 0) emit(e2, w[v], cz / m->vol[e2], -1, false);
                    }
                }
                continue;
            }
            for (int v = 0; v < 3; ++v) {
                double a = l * (pr[v] * nx + pr[3 + v] * ny);
                if (f1) emit(e1, w[v], a / m->vol[e1], 3 * t + e, true);
                if (f2) emit(e2, w[v], -a / m->vol[e2], 3 * t + e, true);
            }
        }
    }
    const int nn = p->neu_deg + 1;
    const int64_t q0 = 3 * m->nt;
    for (int64_t e = 0; e < m->nbe; ++e) {
        int32_t i = m->be[2 * e], j = m->be[2 * e + 1];
        double px = m->pts[2 * i], py = m->pts[2 * i + 1], qx = m->pts[2 * j], qy = m->pts[2 * j + 1];
        double lij = std::sqrt((qx - px) * (qx - px) + (qy - py) * (qy - py));
        double nx = (qy - py) / lij, ny = -(qx - px) / lij;
        double mijx = (px + qx) / 2, mijy = (py + qy) / 2;
        double lh = std::sqrt((mijx - px) * (mijx - px) + (mijy - py) * (mijy - py));
        bool fi = p->code[i] == FVM_VERTEX_FREE, fj = p->code[j] == FVM_VERTEX_FREE;
        if (p->bneu[e]) {
            double n0i = p->quarterN.empty() ? 0.0 : p->quarterN[(2 * e) * nn];
            double n0j = p->quarterN.empty() ? 0.0 : p->quarterN[(2 * e + 1) * nn];
            double n1i = (nn > 1 && !p->quarterN.empty()) ? p->quarterN[(2 * e) * nn + 1] : 0.0;
            double n1j = (nn > 1 && !p->quarterN.empty()) ? p->quarterN[(2 * e + 1) * nn + 1] : 0.0;
            if (fi) {
                b[m->iperm[i]] -= lh * n0i / m->vol[i];
                if (n1i != 0) {
                    emit(i, i, -lh * n1i * 0.75 / m->vol[i], -1, false);
                    emit(i, j, -lh * n1i * 0.25 / m->vol[i], -1, false);
                }
            }
            if (fj) {
                b[m->iperm[j]] -= lh * n0j / m->vol[j];
                if (n1j != 0) {
                    emit(j, i, -lh * n1j * 0.25 / m->vol[j], -1, false);
                    emit(j, j, -lh * n1j * 0.75 / m->vol[j], -1, false);
                }
            }
            continue;
        }
        int32_t t = m->btri[e];
        const int32_t* w = &m->tri[3 * t];
        const double* pr = &m->props[24 * t];
        if (p->flux_linear) {  // du_i -= Q(m_i), du_j -= Q(m_j)
            double gi[3], gj[3];
            nq(&p->quarterM[6 * (2 * e)], nx, ny, gi);
            nq(&p->quarterM[6 * (2 * e + 1)], nx, ny, gj);
            for (int v = 0; v < 3; ++v) {
                if (fi) {
                    emit(i, w[v], -lh * (gi[0] * pr[v] + gi[1] * pr[3 + v]) / m->vol[i], -1, true);
                    if (gi[2] != 0) emit(i, w[v], -lh * gi[2] * pr[6 + v] / m->vol[i], -1, false);
                }
                if (fj) {
                    emit(j, w[v], -lh * (gj[0] * pr[v] + gj[1] * pr[3 + v]) / m->vol[j], -1, true);
                    if (gj[2] != 0) emit(j, w[v], -lh * gj[2] * pr[6 + v] / m->vol[j], -1, false);
                }
            }
            continue;
        }
        for (int v = 0; v < 3; ++v) {
            double c = lh * (pr[v] * nx + pr[3 + v] * ny);
            if (fi) emit(i, w[v], c / m->vol[i], q0 + 2 * e, true);
            if (fj) emit(j, w[v], c / m->vol[j], q0 + 2 * e + 1, true);
        }
    }
    const int ns = p->src_deg + 1, nu = p->dudt_deg + 1;
    for (int64_t v = 0; v < m->np; ++v) {
        int32_t r = m->iperm[v];
        int c = p->code[v];
        if (c == FVM_VERTEX_FREE) {
            rowscale[r] = 1.0 / m->vol[v];
            if (!p->src.empty()) {
                b[r] += p->src[v * ns];
                if (ns > 1 && p->src[v * ns + 1] != 0) emit((int32_t)v, (int32_t)v, p->src[v * ns + 1], -1, false);
                if (ns > 2) q[r] = p->src[v * ns + 2];
            }
        } else if (c == FVM_VERTEX_DUDT) {
            rowscale[r] = 1.0;
            if (!p->dudt.empty()) {
                b[r] = p->dudt[v * nu];
                if (nu > 1 && p->dudt[v * nu + 1] != 0) emit((int32_t)v, (int32_t)v, p->dudt[v * nu + 1], -1, false);
                if (nu > 2) q[r] = p->dudt[v * nu + 2];
            }
        }
    }
}

}  // namespace fvm
