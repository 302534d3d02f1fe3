// Problem set-up: copies the sampled closure forms, folds linear forms into the
// vertex-neighbour operator, and prepares the per-triangle path for nonlinear forms.
#include "fvm_internal.h"
#include "fvm_visit.h"
#include <algorithm>
#include <cmath>

using namespace fvm;

static void check_deg(int d, const char* what) {
    if (d < 0 || d > 2) fail(FVM_ERR_UNSUPPORTED_FORM, std::string(what) + " degree must be 0, 1 or 2");
}

void fvm_problem::ensure_work() {
    const fvm_mesh* m = mesh;
    if (!d_u.p) d_u.alloc(sizeof(double) * m->np);
    if (!d_du.p) d_du.alloc(sizeof(double) * m->np);
    if (!d_ref.p) d_ref.alloc(sizeof(double) * m->np);
}

void fvm_visit_linear_terms(const fvm_problem* p, const LinearTermSink& emit, std::vector<double>& b,
                            std::vector<double>& q, std::vector<double>& rowscale) {
    visit_linear_terms(p, emit, b, q, rowscale);
}

// Constant terms of one time factor's values (time_neumann, time_source, time_dudt of the
// descriptor), in the internal numbering: the parts of fvm_visit_linear_terms that reach b.
std::vector<double> fvm_time_constant_terms(const fvm_problem* p, const double* neu, const double* src,
                                            const double* dudt) {
    const fvm_mesh* m = p->mesh;
    std::vector<double> b(m->np, 0.0);
    if (neu)
        for (int64_t e = 0; e < m->nbe; ++e) {
            if (!p->bneu[e]) continue;
            int32_t i = m->be[2 * e], j = m->be[2 * e + 1];
            double px = m->pts[2 * i], py = m->pts[2 * i + 1], qx = m->pts[2 * j], qy = m->pts[2 * j + 1];
            double mijx = (px + qx) / 2, mijy = (py + qy) / 2;
            double lh = std::sqrt((mijx - px) * (mijx - px) + (mijy - py) * (mijy - py));
            if (p->code[i] == FVM_VERTEX_FREE) b[m->iperm[i]] -= lh * neu[2 * e] / m->vol[i];
            if (p->code[j] == FVM_VERTEX_FREE) b[m->iperm[j]] -= lh * neu[2 * e + 1] / m->vol[j];
        }
    for (int64_t v = 0; v < m->np; ++v) {
        if (p->code[v] == FVM_VERTEX_FREE && src) b[m->iperm[v]] += src[v];
        if (p->code[v] == FVM_VERTEX_DUDT && dudt) b[m->iperm[v]] = dudt[v];
    }
    return b;
}

// Two equivalent storages are produced from the same contributions:
//  explicit (pattern with the diagonal): du_i = sum_j A_ij u_j + b_i + q_i u_i^2, one FP64
//    FMA per entry (GB300 runs FP64 at 1/58 of the FP32 rate, so this is the default);
//  difference form (off-diagonal pattern): du_i = sum_{j != i} K_ij (u_j - u_i) + d_i u_i
//    + b_i + q_i u_i^2.  A dual-edge flux is a combination of u whose coefficients sum to
//    zero (constant u carries no flux), so its diagonal coefficient is implied and dropped:
//    constant fields give exactly zero flux.  Non-flux terms (Neumann u(m) dependence, source,
//    Dudt) keep their full row sum in d_i.
static void assemble_generic(fvm_problem* p, std::vector<double>& E, std::vector<double>& A, std::vector<double>& dg,
                             std::vector<double>& b, std::vector<double>& q, std::vector<double>& rowscale) {
    const fvm_mesh* m = p->mesh;
    const SellPattern& pat = m->pat_off;
    const SellPattern& pate = m->pat;
    E.assign(pate.nslots, 0.0);
    A.assign(pat.nslots, 0.0);
    dg.assign(m->np, 0.0);
    const int nd = p->dif_deg + 1;
    const int64_t q0 = 3 * m->nt;
    auto Dval = [&](int64_t idx) {
        if (idx < q0) return p->dualD.empty() ? 0.0 : p->dualD[idx * nd];
        return p->quarterD.empty() ? 0.0 : p->quarterD[(idx - q0) * nd];
    };
    visit_linear_terms(
        p,
        [&](int32_t r, int32_t c, double coef, int64_t didx, bool flux) {
            const double v = didx >= 0 ? coef * Dval(didx) : coef;
            const int32_t ri = m->iperm[r], ci = m->iperm[c];
            const int64_t q = pate.find_csr(ri, ci);
            E[pate.csr_slot[q]] += v;
            // the off-diagonal row is the full row without its diagonal, in the same order
            if (r != c) A[pat.csr_slot[pat.rowptr[ri] + (q - pate.rowptr[ri]) - (ci > ri ? 1 : 0)]] += v;
            if (!flux) dg[ri] += v;
        },
        b, q, rowscale);
}

extern "C" int fvm_problem_create_impl(fvm_mesh* mesh, const fvm_problem_desc* d, fvm_problem** out) {
    if (!mesh || !d || !out) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    if (!d->vertex_code) fail(FVM_ERR_INVALID_ARGUMENT, "vertex_code is required");
    if (mesh->nbe > 0 && !d->bedge_neumann) fail(FVM_ERR_INVALID_ARGUMENT, "bedge_neumann is required");
    check_deg(d->diffusion_degree, "diffusion");
    check_deg(d->neumann_degree, "Neumann");
    check_deg(d->source_degree, "source");
    check_deg(d->dudt_degree, "Dudt");
    if (d->precision != FVM_FP64 && d->precision != FVM_FP32) fail(FVM_ERR_INVALID_ARGUMENT, "precision must be FVM_FP64 or FVM_FP32");
    SetupTrace tr("problem");
    std::unique_ptr<fvm_problem> p(new fvm_problem());
    const fvm_mesh* m = mesh;
    p->mesh = mesh;
    p->precision = d->precision;
    p->dif_deg = d->diffusion_degree;
    p->neu_deg = d->neumann_degree;
    p->src_deg = d->source_degree;
    p->dudt_deg = d->dudt_degree;
    p->code.assign(d->vertex_code, d->vertex_code + m->np);
    for (int64_t v = 0; v < m->np; ++v) {
        int c = p->code[v];
        if (c < 0 || c > 3) fail(FVM_ERR_INVALID_ARGUMENT, "vertex_code[" + std::to_string(v) + "] is not an FVM_VERTEX_* code");
        if (!m->has_vertex[v] && c != FVM_VERTEX_NOT_A_VERTEX)
            fail(FVM_ERR_INVALID_ARGUMENT, "point " + std::to_string(v) + " is in no triangle but its code is not FVM_VERTEX_NOT_A_VERTEX");
        if (m->has_vertex[v] && c == FVM_VERTEX_NOT_A_VERTEX)
            fail(FVM_ERR_INVALID_ARGUMENT, "point " + std::to_string(v) + " is a vertex but its code is FVM_VERTEX_NOT_A_VERTEX");
    }
    p->bneu.assign(m->nbe, 0);
    for (int64_t e = 0; e < m->nbe; ++e) p->bneu[e] = d->bedge_neumann[e] ? 1 : 0;
    auto copy = [](const double* src, size_t n, std::vector<double>& dst) {
        if (src) dst.assign(src, src + n);
    };
    copy(d->dual_edge_D, (size_t)m->nt * 3 * (p->dif_deg + 1), p->dualD);
    copy(d->quarter_D, (size_t)m->nbe * 2 * (p->dif_deg + 1), p->quarterD);
    copy(d->quarter_neumann, (size_t)m->nbe * 2 * (p->neu_deg + 1), p->quarterN);
    copy(d->source, (size_t)m->np * (p->src_deg + 1), p->src);
    copy(d->dudt, (size_t)m->np * (p->dudt_deg + 1), p->dudt);
    copy(d->dirichlet, (size_t)m->np, p->dirv);
    if (d->dual_edge_flux) {  // a flux linear in (alpha, beta, gamma): no diffusivity samples
        if (m->nbe > 0 && !d->quarter_flux) fail(FVM_ERR_INVALID_ARGUMENT, "quarter_flux is required with dual_edge_flux");
        p->flux_linear = true;
        p->dif_deg = 0;
        p->dualD.clear();
        p->quarterD.clear();
        copy(d->dual_edge_flux, (size_t)m->nt * 3 * 6, p->dualM);
        copy(d->quarter_flux, (size_t)m->nbe * 2 * 6, p->quarterM);
    }
    for (const auto* arr : {&p->dualD, &p->quarterD, &p->quarterN, &p->src, &p->dudt, &p->dirv, &p->dualM, &p->quarterM})
        for (double x : *arr)
            if (!std::isfinite(x)) fail(FVM_ERR_INVALID_ARGUMENT, "sampled closure values must be finite");
    // a form is linear when it is affine in u, except a u^2 term on a vertex's own value
    auto nonzero_deg = [](const std::vector<double>& a, int deg, int k) {
        if (a.empty() || deg < k) return false;
        for (size_t i = k; i < a.size(); i += deg + 1)
            if (a[i] != 0) return true;
        return false;
    };
    p->linear = !(nonzero_deg(p->dualD, p->dif_deg, 1) || nonzero_deg(p->dualD, p->dif_deg, 2) ||
                  nonzero_deg(p->quarterD, p->dif_deg, 1) || nonzero_deg(p->quarterD, p->dif_deg, 2) ||
                  nonzero_deg(p->quarterN, p->neu_deg, 2));

    // vertex classification and Dirichlet list (internal numbering)
    {
        std::vector<int8_t> code_int(m->np);
        for (int64_t v = 0; v < m->np; ++v) code_int[m->iperm[v]] = p->code[v];
        p->d_code.upload(code_int);
        std::vector<int32_t> idx;
        std::vector<double> val;
        for (int64_t v = 0; v < m->np; ++v)
            if (p->code[v] == FVM_VERTEX_DIRICHLET) {
                idx.push_back(m->iperm[v]);
                val.push_back(p->dirv.empty() ? 0.0 : p->dirv[v]);
            }
        p->ndir = (int64_t)idx.size();
        p->d_dir_idx.upload(idx);
        p->d_dir_val.upload(val);
        if (d->ntime < 0 || d->ntime > FVM_MAX_TIME_FACTORS)
            fail(FVM_ERR_INVALID_ARGUMENT, "ntime must lie in [0, FVM_MAX_TIME_FACTORS]");
        if (d->ntime > 0) {
            if (!p->linear)
                fail(FVM_ERR_UNSUPPORTED_FORM, "time-dependent values are supported for linear problems only");
            if (!d->time_factor) fail(FVM_ERR_INVALID_ARGUMENT, "time_factor is required when ntime > 0");
            p->ntime = d->ntime;
            p->tfac.assign(d->time_factor, d->time_factor + 4 * p->ntime);
            for (int g = 0; g < p->ntime; ++g) {
                const double* f = &p->tfac[4 * g];
                if (f[0] != 1.0 && f[0] != 2.0) fail(FVM_ERR_INVALID_ARGUMENT, "time_factor kind must be 1 or 2");
                if (!std::isfinite(f[1]) || !std::isfinite(f[2]) || !std::isfinite(f[3]))
                    fail(FVM_ERR_INVALID_ARGUMENT, "time_factor values must be finite");
            }
            auto finite = [](const double* a, size_t n) {
                for (size_t i = 0; a && i < n; ++i)
                    if (!std::isfinite(a[i])) fail(FVM_ERR_INVALID_ARGUMENT, "time-dependent values must be finite");
            };
            std::vector<double> tb((size_t)p->ntime * m->np), tdir((size_t)p->ntime * std::max<int64_t>(p->ndir, 1), 0.0);
            for (int g = 0; g < p->ntime; ++g) {
                const double* neu = d->time_neumann ? d->time_neumann + (size_t)g * 2 * m->nbe : nullptr;
                const double* src = d->time_source ? d->time_source + (size_t)g * m->np : nullptr;
                const double* dud = d->time_dudt ? d->time_dudt + (size_t)g * m->np : nullptr;
                finite(neu, 2 * m->nbe);
                finite(src, m->np);
                finite(dud, m->np);
                std::vector<double> bg = fvm_time_constant_terms(p.get(), neu, src, dud);
                std::copy(bg.begin(), bg.end(), tb.begin() + (size_t)g * m->np);
                if (d->time_dirichlet) {
                    const double* dv = d->time_dirichlet + (size_t)g * m->np;
                    finite(dv, m->np);
                    int64_t k = 0;
                    for (int64_t v = 0; v < m->np; ++v)
                        if (p->code[v] == FVM_VERTEX_DIRICHLET) {
                            p->tdir_varies |= dv[v] != 0.0;
                            tdir[(size_t)g * p->ndir + k++] = dv[v];
                        }
                }
            }
            p->d_tb.upload(tb);
            p->d_tdir.upload(tdir);
            p->d_beff.alloc(sizeof(double) * m->np);
        }
    }
    tr.mark("copy+codes+time");
    p->conditions_only = (d->options & FVM_PROBLEM_CONDITIONS_ONLY) != 0;
    if (p->linear && !p->conditions_only) {
        std::vector<double> E, A, dg, b, q, rs;
        assemble_generic(p.get(), E, A, dg, b, q, rs);
        tr.mark("assemble");
        p->d_val64.upload(E);
        p->d_kval64.upload(A);
        auto nz = [](double x) { return x != 0; };
        p->op_nonzeros = std::count_if(E.begin(), E.end(), nz);
        p->has_b = std::any_of(b.begin(), b.end(), nz);
        p->has_q = std::any_of(q.begin(), q.end(), nz);
        p->has_d = std::any_of(dg.begin(), dg.end(), nz);
        if (p->has_b) p->d_b.upload(b);
        if (p->has_q) p->d_q.upload(q);
        if (p->has_d) p->d_d.upload(dg);
        if (p->precision == FVM_FP32) {
            // FP32 values carry no 1/V (the control-volume division stays FP64 via rowscale)
            auto unscale = [&](const SellPattern& pat, const std::vector<double>& src) {
                std::vector<float> out(src.size(), 0.0f);
                for (int64_t s = 0; s < pat.nslices; ++s)
                    for (int lane = 0; lane < kSlice; ++lane) {
                        int64_t r = s * kSlice + lane;
                        if (r >= m->np) continue;
                        double sc = rs[r];
                        for (int32_t k = 0; k < pat.width[s]; ++k) {
                            int64_t slot = pat.slice_ptr[s] + (int64_t)k * kSlice + lane;
                            out[slot] = sc != 0 ? (float)(src[slot] / sc) : 0.0f;
                        }
                    }
                return out;
            };
            p->d_val32.upload(unscale(m->pat, E));
            p->d_kval32.upload(unscale(m->pat_off, A));
            p->d_rowscale.upload(rs);
            p->d_u32.alloc(sizeof(float) * m->np);
        }
    }
    tr.mark("upload");
    *out = p.release();
    return FVM_OK;
}

// Per-element data of the per-triangle flux kernel (used for nonlinear forms, or on request).
void fvm_problem::build_triangle_path() {
    if (tri_ready) return;
    if (ntime > 0)
        fail(FVM_ERR_UNSUPPORTED, "time-dependent values run on the operator path only (no force_triangle)");
    if (flux_linear)
        fail(FVM_ERR_UNSUPPORTED, "a flux linear in (alpha, beta, gamma) other than -D grad u runs on the operator "
                                  "path only: it needs affine Neumann, source and Dudt forms and no force_triangle");
    fvm_mesh* m = mesh;
    m->build_tiles();
    const Tiles& T = m->tiles;
    const int nd = dif_deg + 1;
    if (dif_deg == 0) {
        // fold D into the geometric coefficients: c[e][v] = D_e g[e][v]
        std::vector<double> g(6 * T.nelem);
        FVM_CUDA(cudaMemcpy(g.data(), T.d_g.p, g.size() * sizeof(double), cudaMemcpyDeviceToHost));
        for (int64_t e = 0; e < T.nelem; ++e)
            for (int d = 0; d < 3; ++d) {
                double D = dualD.empty() ? 0.0 : dualD[(3 * (size_t)T.etri[e] + d) * nd];
                g[(2 * d) * T.nelem + e] *= D;
                g[(2 * d + 1) * T.nelem + e] *= D;
            }
        d_ec.upload(g);
    } else {
        std::vector<double> c((size_t)3 * nd * T.nelem, 0.0);
        for (int64_t e = 0; e < T.nelem; ++e)
            for (int d = 0; d < 3; ++d)
                for (int k = 0; k < nd; ++k)
                    c[(size_t)(d * nd + k) * T.nelem + e] = dualD.empty() ? 0.0 : dualD[(3 * (size_t)T.etri[e] + d) * nd + k];
        d_ec.upload(c);
    }
    // boundary elements: [0] Neumann flag, D(m_i) poly, D(m_j) poly, N(m_i) poly (3), N(m_j) poly (3)
    const int nrow = 1 + 2 * nd + 6;
    std::vector<double> bc((size_t)nrow * std::max<int64_t>(T.nbelem, 1), 0.0);
    const int nn = neu_deg + 1;
    for (int64_t q = 0; q < T.nbelem; ++q) {
        int32_t e = T.ebedge[q];
        auto at = [&](int row) -> double& { return bc[(size_t)row * T.nbelem + q]; };
        at(0) = bneu[e] ? 1.0 : 0.0;
        for (int k = 0; k < nd; ++k) {
            at(1 + k) = quarterD.empty() ? 0.0 : quarterD[(2 * (size_t)e) * nd + k];
            at(1 + nd + k) = quarterD.empty() ? 0.0 : quarterD[(2 * (size_t)e + 1) * nd + k];
        }
        for (int k = 0; k < nn; ++k) {
            at(1 + 2 * nd + k) = quarterN.empty() ? 0.0 : quarterN[(2 * (size_t)e) * nn + k];
            at(1 + 2 * nd + 3 + k) = quarterN.empty() ? 0.0 : quarterN[(2 * (size_t)e + 1) * nn + k];
        }
    }
    bc.resize((size_t)nrow * T.nbelem);
    d_bc.upload(bc);
    // per-vertex polynomials (internal numbering), [3][np]
    std::vector<double> vs(3 * m->np, 0.0), vd(3 * m->np, 0.0);
    const int ns = src_deg + 1, nu = dudt_deg + 1;
    for (int64_t v = 0; v < m->np; ++v) {
        int32_t r = m->iperm[v];
        for (int k = 0; k < ns && !src.empty(); ++k) vs[k * m->np + r] = src[v * ns + k];
        for (int k = 0; k < nu && !dudt.empty(); ++k) vd[k * m->np + r] = dudt[v * nu + k];
    }
    d_vsrc.upload(vs);
    d_vdudt.upload(vd);
    tri_ready = true;
}
