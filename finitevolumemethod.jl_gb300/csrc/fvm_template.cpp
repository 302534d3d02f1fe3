// Linear templates (src/specific_problems/*.jl) assembled straight into the sliced-ELL
// operator of the mesh: no dense n x n matrix (the reference builds zeros(n, n) and calls
// sparse(), which cannot be allocated beyond a few 10^4 vertices).
#include "fvm_internal.h"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>

using namespace fvm;

// Terms of A and b, rows and columns in the caller's numbering; follows
// abstract_templates.jl:73-99 (triangles), :149-191 and :237-267 (boundary edges, including
// the reference's division of row j by V_i at :262), :127-135 (Dudt), :278-309 (Poisson b and
// steady Dirichlet rows), :317-325 (missing vertices), linear_reaction_diffusion_equations.jl:
// 115-125 and mean_exit_time.jl:84-94.  A diffusion term's coefficient multiplies the
// diffusion sample D[didx] (dual-edge midpoints 3 t + e, then boundary quarter points
// 3 nt + 2 e + side); a term with didx < 0 is a constant.  Every entry the reference assigns
// (Dirichlet and missing-vertex rows, Dudt and mean-exit-time b) receives no other term, so
// all terms add.
void fvm_template_visit_terms(const fvm_template* T, const TemplateTermSink& emitA, const TemplateTermSink& emitb) {
    const fvm_problem* p = T->prob;
    const fvm_mesh* m = p->mesh;
    const int kind = T->kind;
    if (p->dif_deg != 0) fail(FVM_ERR_UNSUPPORTED_FORM, "template diffusion functions are D(x, y): degree 0");
    bool has_dudt = false;
    for (int64_t v = 0; v < m->np; ++v) has_dudt |= p->code[v] == FVM_VERTEX_DUDT;
    if (has_dudt && kind == FVM_TEMPLATE_POISSON) fail(FVM_ERR_UNSUPPORTED, "PoissonsEquation does not support Dudt nodes.");
    if (has_dudt && kind == FVM_TEMPLATE_MEAN_EXIT_TIME)
        fail(FVM_ERR_UNSUPPORTED, "MeanExitTimeProblem does not support Dudt nodes.");
    auto hc = [&](int32_t v) { return p->code[v] == FVM_VERTEX_DIRICHLET || p->code[v] == FVM_VERTEX_DUDT; };
    auto dir = [&](int32_t v) { return p->code[v] == FVM_VERTEX_DIRICHLET; };
    const int ns = p->src_deg + 1, nn = p->neu_deg + 1;
    const int64_t qbase = 3 * m->nt;
    if (kind == FVM_TEMPLATE_POISSON)  // create_rhs_b
        for (int64_t v = 0; v < m->np; ++v)
            if (m->has_vertex[v] && !dir((int32_t)v)) emitb((int32_t)v, -1, p->src.empty() ? 0.0 : p->src[v * ns], -1);
    // triangle_contributions!
    for (int64_t t = 0; t < m->nt; ++t) {
        const int32_t* w = &m->tri[3 * t];
        const double* pr = &m->props[24 * t];
        for (int e = 0; e < 3; ++e) {
            int32_t e1 = w[e], e2 = w[(e + 1) % 3];
            double l = pr[21 + e];
            double nx = pr[15 + 2 * e], ny = pr[16 + 2 * e];
            bool h1 = hc(e1), h2 = hc(e2);
            for (int v = 0; v < 3; ++v) {
                double a = l * (pr[v] * nx + pr[3 + v] * ny);
                if (!h1) emitA(e1, w[v], a / m->vol[e1], 3 * t + e);
                if (!h2) emitA(e2, w[v], -a / m->vol[e2], 3 * t + e);
            }
        }
    }
    if (kind != FVM_TEMPLATE_MEAN_EXIT_TIME) {
        for (int64_t e = 0; e < m->nbe; ++e) {
            int32_t i = m->be[2 * e], j = m->be[2 * e + 1];
            double px = m->pts[2 * i], py = m->pts[2 * i + 1], qx = m->pts[2 * j], qy = m->pts[2 * j + 1];
            double lij = std::sqrt((qx - px) * (qx - px) + (qy - py) * (qy - py));
            double nx = (qy - py) / lij, ny = -(qx - px) / lij;
            double mijx = (px + qx) / 2, mijy = (py + qy) / 2;
            double lh = std::sqrt((mijx - px) * (mijx - px) + (mijy - py) * (mijy - py));
            if (p->bneu[e]) {  // neumann_boundary_edge_contributions! (b += D a l / V)
                double ai = p->quarterN.empty() ? 0.0 : p->quarterN[(2 * e) * nn];
                double aj = p->quarterN.empty() ? 0.0 : p->quarterN[(2 * e + 1) * nn];
                if (!hc(i)) emitb(i, -1, ai * lh / m->vol[i], qbase + 2 * e);
                if (!hc(j)) emitb(j, -1, aj * lh / m->vol[j], qbase + 2 * e + 1);
                continue;
            }
            int32_t t = m->btri[e];
            const int32_t* w = &m->tri[3 * t];
            const double* pr = &m->props[24 * t];
            for (int v = 0; v < 3; ++v) {
                double c = pr[v] * nx + pr[3 + v] * ny;
                if (!hc(i)) emitA(i, w[v], lh * c / m->vol[i], qbase + 2 * e);
                if (!hc(j)) emitA(j, w[v], lh * c / m->vol[i], qbase + 2 * e + 1);  // V_i, as the reference
            }
        }
    }
    if (kind == FVM_TEMPLATE_LINEAR_REACTION_DIFFUSION)  // linear_source_contributions!
        for (int64_t v = 0; v < m->np; ++v)
            if (m->has_vertex[v] && !hc((int32_t)v) && !p->src.empty() && ns > 1)
                emitA((int32_t)v, (int32_t)v, p->src[v * ns + 1], -1);
    if (kind == FVM_TEMPLATE_DIFFUSION || kind == FVM_TEMPLATE_LINEAR_REACTION_DIFFUSION) {
        const int nu = p->dudt_deg + 1;
        for (int64_t v = 0; v < m->np; ++v)  // apply_dudt_conditions!
            if (p->code[v] == FVM_VERTEX_DUDT) emitb((int32_t)v, -1, p->dudt.empty() ? 0.0 : p->dudt[v * nu], -1);
    }
    if (kind == FVM_TEMPLATE_POISSON)  // apply_steady_dirichlet_conditions!
        for (int64_t v = 0; v < m->np; ++v)
            if (dir((int32_t)v)) {
                emitb((int32_t)v, -1, p->dirv.empty() ? 0.0 : p->dirv[v], -1);
                emitA((int32_t)v, (int32_t)v, 1.0, -1);
            }
    if (kind == FVM_TEMPLATE_MEAN_EXIT_TIME)  // create_met_b!
        for (int64_t v = 0; v < m->np; ++v) {
            if (!m->has_vertex[v]) continue;
            if (!dir((int32_t)v))
                emitb((int32_t)v, -1, -1.0, -1);
            else
                emitA((int32_t)v, (int32_t)v, 1.0, -1);
        }
    for (int64_t v = 0; v < m->np; ++v)  // fix_missing_vertices! (b stays 0)
        if (!m->has_vertex[v]) emitA((int32_t)v, (int32_t)v, 1.0, -1);
}

// A and b in the internal numbering, from the terms above with the problem's D samples
static void assemble_template(fvm_template* T) {
    const fvm_problem* p = T->prob;
    const fvm_mesh* m = p->mesh;
    const SellPattern& pat = m->pat;
    std::vector<double>& A = T->val;
    std::vector<double>& b = T->b;
    A.assign(pat.nslots, 0.0);
    b.assign(m->np, 0.0);
    const int64_t qbase = 3 * m->nt;
    auto D = [&](int64_t didx) {
        if (didx < 0) return 1.0;
        if (didx < qbase) return p->dualD.empty() ? 0.0 : p->dualD[didx];
        return p->quarterD.empty() ? 0.0 : p->quarterD[didx - qbase];
    };
    fvm_template_visit_terms(
        T,
        [&](int32_t r, int32_t c, double coef, int64_t didx) {
            A[pat.find(m->iperm[r], m->iperm[c])] += D(didx) * coef;
        },
        [&](int32_t r, int32_t, double coef, int64_t didx) { b[m->iperm[r]] += D(didx) * coef; });
}

// FP32 copy of the template values and the FP32 gather buffer (first FP32 use)
static void ensure_fp32(fvm_template* T) {
    if (!T->d_val32.p) {
        std::vector<float> v32(T->val.size());
        for (size_t i = 0; i < v32.size(); ++i) v32[i] = (float)T->val[i];
        T->d_val32.upload(v32);
    }
    if (!T->d_u32.p) T->d_u32.alloc(sizeof(float) * T->prob->mesh->np);
}

extern "C" {

int fvm_template_create(fvm_problem* prob, int32_t kind, fvm_template** out) {
    return guard_call([&] {
        if (!prob || !out) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        if (kind < FVM_TEMPLATE_DIFFUSION || kind > FVM_TEMPLATE_MEAN_EXIT_TIME)
            fail(FVM_ERR_INVALID_ARGUMENT, "unknown template kind");
        if (prob->ntime > 0) fail(FVM_ERR_UNSUPPORTED_FORM, "templates take time-independent conditions");
        *out = nullptr;
        std::unique_ptr<fvm_template> T(new fvm_template());
        T->prob = prob;
        T->kind = kind;
        assemble_template(T.get());
        T->d_val64.upload(T->val);
        T->d_b.upload(T->b);
        *out = T.release();
        return FVM_OK;
    });
}

int fvm_template_destroy(fvm_template* T) {
    return guard_call([&] {
        delete T;
        return FVM_OK;
    });
}

int fvm_template_export(const fvm_template* T, int64_t* nnz, int32_t* rowptr, int32_t* col, double* val, double* b) {
    return guard_call([&] {
        if (!T || !nnz) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        const fvm_mesh* m = T->prob->mesh;
        const SellPattern& pat = m->pat;
        std::vector<std::pair<int32_t, double>> row;
        int64_t count = 0;
        if (rowptr) rowptr[0] = 0;
        for (int64_t r = 0; r < m->np; ++r) {
            int32_t ri = m->iperm[r];
            row.clear();
            for (int64_t q = pat.rowptr[ri]; q < pat.rowptr[ri + 1]; ++q) {
                double v = T->val[pat.csr_slot[q]];
                if (v != 0.0) row.push_back({m->perm[pat.csr_col[q]], v});
            }
            std::sort(row.begin(), row.end());
            if (col && val)
                for (size_t k = 0; k < row.size(); ++k) {
                    col[count + k] = row[k].first;
                    val[count + k] = row[k].second;
                }
            count += (int64_t)row.size();
            if (rowptr) rowptr[r + 1] = (int32_t)count;
        }
        *nnz = count;
        if (b)
            for (int64_t r = 0; r < m->np; ++r) b[r] = T->b[m->iperm[r]];
        return FVM_OK;
    });
}

int fvm_template_apply(fvm_template* T, const double* u, double* du, int32_t precision, int32_t flags, void* stream) {
    return guard_call([&] {
        if (!T || !u || !du) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        cudaStream_t s = (cudaStream_t)stream;
        fvm_problem* p = T->prob;
        fvm_mesh* m = p->mesh;
        int32_t loc = flags & 3;
        if (loc > FVM_PTR_DEVICE_INTERNAL) fail(FVM_ERR_INVALID_ARGUMENT, "bad pointer-location flag");
        const double* uin = u;
        double* dout = du;
        if (loc != FVM_PTR_DEVICE_INTERNAL) {
            p->ensure_work();
            if (loc == FVM_PTR_HOST) {
                FVM_CUDA(cudaMemcpyAsync(p->d_ref.p, u, sizeof(double) * m->np, cudaMemcpyHostToDevice, s));
                launch_permute_in(m->d_perm.as<int32_t>(), p->d_ref.as<double>(), p->d_u.as<double>(), m->np, s);
            } else {
                launch_permute_in(m->d_perm.as<int32_t>(), u, p->d_u.as<double>(), m->np, s);
            }
            uin = p->d_u.as<double>();
            dout = p->d_du.as<double>();
        }
        if (precision == FVM_FP32) {
            ensure_fp32(T);
            launch_to_f32(uin, T->d_u32.as<float>(), m->np, s);
            launch_sell_apply32(m->pat, T->d_val32.as<float>(), T->d_u32.as<float>(), uin, dout, nullptr,
                                T->d_b.as<double>(), nullptr, s);
        } else {
            launch_sell_apply64(m->pat, T->d_val64.as<double>(), uin, dout, nullptr, T->d_b.as<double>(), nullptr, s);
        }
        FVM_CUDA(cudaGetLastError());
        if (loc == FVM_PTR_HOST) {
            launch_permute_out(m->d_perm.as<int32_t>(), p->d_du.as<double>(), p->d_ref.as<double>(), m->np, s);
            FVM_CUDA(cudaMemcpyAsync(du, p->d_ref.p, sizeof(double) * m->np, cudaMemcpyDeviceToHost, s));
            FVM_CUDA(cudaStreamSynchronize(s));
        } else if (loc == FVM_PTR_DEVICE) {
            launch_permute_out(m->d_perm.as<int32_t>(), p->d_du.as<double>(), du, m->np, s);
        }
        return FVM_OK;
    });
}

int fvm_template_tsit5_solve(fvm_template* T, const double* u0, const fvm_ode_options* opt, double* out,
                             fvm_ode_stats* stats, void* stream) {
    return guard_call([&] {
        if (!T || !u0 || !opt || !out) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        if (T->kind != FVM_TEMPLATE_DIFFUSION && T->kind != FVM_TEMPLATE_LINEAR_REACTION_DIFFUSION)
            fail(FVM_ERR_INVALID_ARGUMENT, "only time-dependent templates can be stepped");
        cudaStream_t s = (cudaStream_t)stream;
        fvm_mesh* m = T->prob->mesh;
        const int64_t n = m->np;
        int64_t nsave = (opt->saveat && opt->nsave > 0) ? opt->nsave : 1;
        DBuf d_in, d_out;
        d_in.alloc(sizeof(double) * n * 2);
        d_out.alloc(sizeof(double) * n * nsave);
        double* d_ref = d_in.as<double>();
        double* d_u0 = d_ref + n;
        FVM_CUDA(cudaMemcpyAsync(d_ref, u0, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        launch_permute_in(m->d_perm.as<int32_t>(), d_ref, d_u0, n, s);
        const bool fp32 = opt->precision == FVM_FP32;
        if (fp32) ensure_fp32(T);
        OdeRhs rhs;
        rhs.f = [T, m, fp32](const double* u, double* du, double, cudaStream_t st) {
            if (fp32) {
                launch_to_f32(u, T->d_u32.as<float>(), m->np, st);
                launch_sell_apply32(m->pat, T->d_val32.as<float>(), T->d_u32.as<float>(), u, du, nullptr,
                                    T->d_b.as<double>(), nullptr, st);
            } else
                launch_sell_apply64(m->pat, T->d_val64.as<double>(), u, du, nullptr, T->d_b.as<double>(), nullptr, st);
        };
        if (!fp32) {
            rhs.sell.pat = &m->pat;
            rhs.sell.val = T->d_val64.as<double>();
            rhs.sell.b = T->d_b.as<double>();
        }
        tsit5_run_internal(rhs, n, d_u0, *opt, d_out.as<double>(), stats, s);
        snapshots_to_host(m->d_iperm.as<int32_t>(), d_out.as<double>(), out, n, nsave, s);
        FVM_CUDA(cudaStreamSynchronize(s));
        FVM_CUDA(cudaGetLastError());
        return FVM_OK;
    });
}

}  // extern "C"
