// FVMSystem: N coupled components on one mesh (fvm_system_*).
//
// Set-up folds each component's linear flux -sum_c D_rc(x, y) grad u_c, with its affine Neumann
// terms, into coupled blocks K_rc on the mesh's vertex-neighbour pattern (sliced ELL, the
// control-volume division folded in), through the same term visitor as the single-equation
// RHS.  The source and Dudt forms stay polynomials in the node's own component values and
// are evaluated in the kernel's epilogue.  One kernel then gives
//   du[i][r] = sum_c sum_j K_rc[i][j] u[j][c] + b[i][r] + P_r(u[i][0..N-1])
// for the state laid out [point][component], the reference's N x npoints matrix order.
#include "fvm_internal.h"
#include <algorithm>
#include <cmath>
#include <cstring>

namespace fvm {

constexpr int kSysMaxEq = FVM_SYSTEM_MAX_EQ;
constexpr int kSysMaxTerms = FVM_SYSTEM_MAX_TERMS;

// Terms of the polynomial epilogue: term t adds coef_t * prod_c u_c^e_tc to component var_t on
// the rows whose mask bit var_t is set.  exps packs e_tc in 2 bits per component.
struct SysTerms {
    int32_t n = 0;
    uint32_t exps[kSysMaxTerms];
    int32_t var[kSysMaxTerms];
    int32_t vary[kSysMaxTerms];  // row of the per-vertex coefficient table, or -1 (coef is uniform)
    double coef[kSysMaxTerms];
};

struct SysArgs {
    const int64_t* slice_ptr;
    const int32_t* width;
    const int32_t* col;
    int64_t nslices, nrows, nslots;
    const double* val;    // [stored blocks][nslots], blocks in (r, c) row-major order
    uint64_t blocks;      // bit r*N + c: block (r, c) is stored
    const double* u;      // [nrows][N]
    double* du;           // [nrows][N]
    const double* b;      // [nrows][N] or null (Neumann constants)
    const uint8_t* mask;  // [nrows]: bit r set when component r's row is FREE or DUDT
    const double* vcoef;  // [nvary][nrows]
};

// One warp per 32-row slice, one lane per row.  Each slot gathers the neighbour's N component
// values (contiguous) once and feeds every stored block of the row.
template <int N>
__global__ void __launch_bounds__(256) system_rhs_kernel(const SysArgs a, const SysTerms tm) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < a.nslices; s += nwarps) {
        const int64_t base = __ldg(&a.slice_ptr[s]) + lane;
        const int w = __ldg(&a.width[s]);
        double acc[N];
#pragma unroll
        for (int r = 0; r < N; ++r) acc[r] = 0.0;
#pragma unroll 2
        for (int k = 0; k < w; ++k) {
            const int64_t slot = base + (int64_t)k * 32;
            const int64_t c = __ldg(&a.col[slot]);
            double uc[N];
#pragma unroll
            for (int q = 0; q < N; ++q) uc[q] = __ldg(&a.u[c * N + q]);
            const double* v = a.val + slot;
#pragma unroll
            for (int r = 0; r < N; ++r)
#pragma unroll
                for (int q = 0; q < N; ++q)
                    if ((a.blocks >> (r * N + q)) & 1ull) {
                        acc[r] = fma(__ldg(v), uc[q], acc[r]);
                        v += a.nslots;
                    }
        }
        const int64_t row = s * 32 + lane;
        if (row >= a.nrows) continue;
        double ui[N];
#pragma unroll
        for (int q = 0; q < N; ++q) ui[q] = a.u[row * N + q];
        if (a.b) {
#pragma unroll
            for (int r = 0; r < N; ++r) acc[r] += a.b[row * N + r];
        }
        const unsigned m = a.mask[row];
        for (int t = 0; t < tm.n; ++t) {
            double x = tm.vary[t] < 0 ? tm.coef[t] : __ldg(&a.vcoef[(int64_t)tm.vary[t] * a.nrows + row]);
            const uint32_t e = tm.exps[t];
#pragma unroll
            for (int q = 0; q < N; ++q) {
                const uint32_t eq = (e >> (2 * q)) & 3u;
                if (eq >= 1) x *= ui[q];
                if (eq >= 2) x *= ui[q];
                if (eq >= 3) x *= ui[q];
            }
            const int rt = tm.var[t];
#pragma unroll
            for (int r = 0; r < N; ++r)
                if (r == rt && ((m >> r) & 1u)) acc[r] += x;
        }
#pragma unroll
        for (int r = 0; r < N; ++r) a.du[row * N + r] = acc[r];
    }
}

}  // namespace fvm

using namespace fvm;

struct fvm_system {
    fvm_mesh* mesh = nullptr;
    int neq = 0;
    int nblocks = 0;
    uint64_t blocks = 0;
    SysTerms terms;
    int nvary = 0;
    bool has_b = false;
    int64_t ndir = 0;
    DBuf d_val, d_b, d_mask, d_vcoef, d_dir_idx, d_dir_val;
    DBuf d_perm, d_iperm;  // flat [point][component] permutations: internal -> caller, caller -> internal
    DBuf d_u, d_du, d_ref;
    int64_t n() const { return (int64_t)neq * mesh->np; }
    void ensure_work() {
        if (!d_u.p) d_u.alloc(sizeof(double) * n());
        if (!d_du.p) d_du.alloc(sizeof(double) * n());
        if (!d_ref.p) d_ref.alloc(sizeof(double) * n());
    }
};

namespace fvm {

template <int N>
static void launch_system(const fvm_system* S, const double* u, double* du, cudaStream_t s) {
    const SellPattern& p = S->mesh->pat;
    if (p.nslices == 0) return;
    SysArgs a{p.d_slice_ptr.as<int64_t>(),
              p.d_width.as<int32_t>(),
              p.d_col.as<int32_t>(),
              p.nslices,
              p.nrows,
              p.nslots,
              S->d_val.as<double>(),
              S->blocks,
              u,
              du,
              S->has_b ? S->d_b.as<double>() : nullptr,
              S->d_mask.as<uint8_t>(),
              S->nvary ? S->d_vcoef.as<double>() : nullptr};
    // 8 warps per block, at most 8 resident blocks on each of the 152 SMs; slices are grid-strided
    const unsigned grid = (unsigned)std::min<int64_t>((p.nslices + 7) / 8, 152 * 8);
    system_rhs_kernel<N><<<grid, 256, 0, s>>>(a, S->terms);
}

static void system_rhs_internal(const fvm_system* S, const double* u, double* du, cudaStream_t s) {
    switch (S->neq) {
        case 1: launch_system<1>(S, u, du, s); break;
        case 2: launch_system<2>(S, u, du, s); break;
        case 3: launch_system<3>(S, u, du, s); break;
        case 4: launch_system<4>(S, u, du, s); break;
        case 5: launch_system<5>(S, u, du, s); break;
        case 6: launch_system<6>(S, u, du, s); break;
        case 7: launch_system<7>(S, u, du, s); break;
        case 8: launch_system<8>(S, u, du, s); break;
        default: fail(FVM_ERR_INVALID_ARGUMENT, "neq out of range");
    }
    FVM_CUDA(cudaGetLastError());
}

static void system_dirichlet_internal(const fvm_system* S, double* u, cudaStream_t s) {
    if (S->ndir) launch_dirichlet(S->d_dir_idx.as<int32_t>(), S->d_dir_val.as<double>(), u, S->ndir, s);
}

static void create_system(fvm_mesh* m, const fvm_system_desc* d, fvm_system** out) {
    if (!m || !d || !out) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    const int N = d->neq;
    if (N < 1 || N > kSysMaxEq)
        fail(FVM_ERR_INVALID_ARGUMENT, "neq must lie in 1.." + std::to_string(kSysMaxEq));
    if (!d->vertex_code) fail(FVM_ERR_INVALID_ARGUMENT, "vertex_code is required");
    if (m->nbe > 0 && !d->bedge_neumann) fail(FVM_ERR_INVALID_ARGUMENT, "bedge_neumann is required");
    const int64_t np = m->np, nt = m->nt, nbe = m->nbe;
    if ((int64_t)N * np >= (int64_t(1) << 31)) fail(FVM_ERR_INVALID_ARGUMENT, "neq * npoints must fit in int32");
    for (int r = 0; r < N; ++r)
        for (int64_t v = 0; v < np; ++v) {
            const int c = d->vertex_code[r * np + v];
            if (c < 0 || c > 3) fail(FVM_ERR_INVALID_ARGUMENT, "vertex_code holds a value that is not an FVM_VERTEX_* code");
            if (!m->has_vertex[v] != (c == FVM_VERTEX_NOT_A_VERTEX))
                fail(FVM_ERR_INVALID_ARGUMENT, "point " + std::to_string(v) + " of component " + std::to_string(r) +
                                                   ": FVM_VERTEX_NOT_A_VERTEX must mark exactly the points in no triangle");
        }
    const int nmono = d->nmono;
    if (nmono < 0 || (nmono > 0 && !d->mono_exp)) fail(FVM_ERR_INVALID_ARGUMENT, "nmono / mono_exp");
    if (nmono == 0 && (d->source || d->dudt)) fail(FVM_ERR_INVALID_ARGUMENT, "source / dudt given with nmono = 0");
    for (int mo = 0; mo < nmono; ++mo) {
        int deg = 0;
        for (int c = 0; c < N; ++c) {
            const int e = d->mono_exp[mo * N + c];
            if (e < 0 || e > 3) fail(FVM_ERR_UNSUPPORTED_FORM, "monomial exponents must lie in 0..3");
            deg += e;
        }
        if (deg > 3) fail(FVM_ERR_UNSUPPORTED_FORM, "source and Dudt polynomials must have total degree <= 3");
    }
    auto finite = [](const double* a, size_t n, const char* what) {
        if (!a) return;
        for (size_t i = 0; i < n; ++i)
            if (!std::isfinite(a[i])) fail(FVM_ERR_INVALID_ARGUMENT, std::string(what) + " values must be finite");
    };
    finite(d->dual_edge_D, (size_t)N * N * 3 * nt, "dual_edge_D");
    finite(d->quarter_D, (size_t)N * N * 2 * nbe, "quarter_D");
    finite(d->source, (size_t)N * np * nmono, "source");
    finite(d->dudt, (size_t)N * np * nmono, "dudt");
    finite(d->quarter_neumann, (size_t)N * 2 * nbe * (1 + N), "quarter_neumann");
    finite(d->dirichlet, (size_t)N * np, "dirichlet");

    std::unique_ptr<fvm_system> S(new fvm_system());
    S->mesh = m;
    S->neq = N;
    const SellPattern& pat = m->pat;
    const int64_t q0 = 3 * nt;

    // coupled flux blocks K_rc, and the Neumann constants of each component (from the (r, r) pass)
    std::vector<double> vals, B((size_t)np * N, 0.0);
    for (int r = 0; r < N; ++r)
        for (int c = 0; c < N; ++c) {
            fvm_problem tp;  // host-side view of component r's flux through u_c
            tp.mesh = m;
            tp.code.assign(d->vertex_code + r * np, d->vertex_code + (r + 1) * np);
            tp.bneu.assign(nbe, 0);
            for (int64_t e = 0; e < nbe; ++e) tp.bneu[e] = d->bedge_neumann[r * nbe + e] ? 1 : 0;
            tp.dif_deg = 0;
            const size_t blk = (size_t)r * N + c;
            if (d->dual_edge_D) tp.dualD.assign(d->dual_edge_D + blk * 3 * nt, d->dual_edge_D + (blk + 1) * 3 * nt);
            if (d->quarter_D) tp.quarterD.assign(d->quarter_D + blk * 2 * nbe, d->quarter_D + (blk + 1) * 2 * nbe);
            tp.neu_deg = 1;
            if (d->quarter_neumann) {
                tp.quarterN.assign((size_t)2 * nbe * 2, 0.0);
                for (int64_t qp = 0; qp < 2 * nbe; ++qp) {
                    const double* nq = d->quarter_neumann + ((size_t)r * 2 * nbe + qp) * (1 + N);
                    tp.quarterN[2 * qp] = c == r ? nq[0] : 0.0;
                    tp.quarterN[2 * qp + 1] = nq[1 + c];
                }
            }
            auto Dval = [&](int64_t idx) -> double {
                if (idx < q0) return tp.dualD.empty() ? 0.0 : tp.dualD[idx];
                return tp.quarterD.empty() ? 0.0 : tp.quarterD[idx - q0];
            };
            std::vector<double> E(pat.nslots, 0.0), b, qv, rs;
            fvm_visit_linear_terms(
                &tp,
                [&](int32_t row, int32_t col, double coef, int64_t didx, bool) {
                    const double v = didx >= 0 ? coef * Dval(didx) : coef;
                    E[pat.find(m->iperm[row], m->iperm[col])] += v;
                },
                b, qv, rs);
            if (c == r)
                for (int64_t i = 0; i < np; ++i) B[(size_t)i * N + r] = b[i];
            if (std::any_of(E.begin(), E.end(), [](double x) { return x != 0.0; })) {
                S->blocks |= 1ull << (r * N + c);
                ++S->nblocks;
                vals.insert(vals.end(), E.begin(), E.end());
            }
        }
    if (vals.empty()) vals.assign(pat.nslots, 0.0);  // keeps the value pointer valid; no block is read
    S->d_val.upload(vals);
    S->has_b = std::any_of(B.begin(), B.end(), [](double x) { return x != 0.0; });
    if (S->has_b) S->d_b.upload(B);

    // polynomial terms (source on FREE rows, Dudt on DUDT rows) and the row masks
    std::vector<uint8_t> mask(np, 0);
    for (int r = 0; r < N; ++r)
        for (int64_t v = 0; v < np; ++v) {
            const int c = d->vertex_code[r * np + v];
            if (c == FVM_VERTEX_FREE || c == FVM_VERTEX_DUDT) mask[m->iperm[v]] |= (uint8_t)(1u << r);
        }
    S->d_mask.upload(mask);
    std::vector<double> vtab, cf(np);
    for (int r = 0; r < N; ++r)
        for (int mo = 0; mo < nmono; ++mo) {
            bool any = false, uniform = true, first = true;
            double u0 = 0.0;
            for (int64_t v = 0; v < np; ++v) {
                const int c = d->vertex_code[r * np + v];
                const size_t at = ((size_t)r * np + v) * nmono + mo;
                double x = 0.0;
                if (c == FVM_VERTEX_FREE && d->source) x = d->source[at];
                if (c == FVM_VERTEX_DUDT && d->dudt) x = d->dudt[at];
                cf[v] = x;
                if (c != FVM_VERTEX_FREE && c != FVM_VERTEX_DUDT) continue;
                any = any || x != 0.0;
                if (first) {
                    u0 = x;
                    first = false;
                } else if (x != u0) {
                    uniform = false;
                }
            }
            if (!any) continue;
            SysTerms& T = S->terms;
            if (T.n == kSysMaxTerms)
                fail(FVM_ERR_UNSUPPORTED_FORM, "more than " + std::to_string(kSysMaxTerms) + " source / Dudt terms");
            uint32_t e = 0;
            for (int c = 0; c < N; ++c) e |= (uint32_t)d->mono_exp[mo * N + c] << (2 * c);
            T.exps[T.n] = e;
            T.var[T.n] = r;
            if (uniform) {
                T.vary[T.n] = -1;
                T.coef[T.n] = u0;
            } else {
                T.vary[T.n] = S->nvary++;
                T.coef[T.n] = 0.0;
                const size_t off = vtab.size();
                vtab.resize(off + np, 0.0);
                for (int64_t v = 0; v < np; ++v) vtab[off + m->iperm[v]] = cf[v];
            }
            ++T.n;
        }
    if (S->nvary) S->d_vcoef.upload(vtab);

    // Dirichlet entries on the flat internal state
    std::vector<int32_t> idx;
    std::vector<double> dval;
    for (int r = 0; r < N; ++r)
        for (int64_t v = 0; v < np; ++v)
            if (d->vertex_code[r * np + v] == FVM_VERTEX_DIRICHLET) {
                idx.push_back((int32_t)((int64_t)m->iperm[v] * N + r));
                dval.push_back(d->dirichlet ? d->dirichlet[r * np + v] : 0.0);
            }
    S->ndir = (int64_t)idx.size();
    S->d_dir_idx.upload(idx);
    S->d_dir_val.upload(dval);

    std::vector<int32_t> perm((size_t)np * N), iperm((size_t)np * N);
    for (int64_t i = 0; i < np; ++i)
        for (int r = 0; r < N; ++r) {
            perm[(size_t)i * N + r] = (int32_t)((int64_t)m->perm[i] * N + r);
            iperm[(size_t)i * N + r] = (int32_t)((int64_t)m->iperm[i] * N + r);
        }
    S->d_perm.upload(perm);
    S->d_iperm.upload(iperm);
    *out = S.release();
}

}  // namespace fvm

extern "C" {

int fvm_system_create(fvm_mesh* mesh, const fvm_system_desc* desc, fvm_system** out) {
    return guard_call([&] {
        create_system(mesh, desc, out);
        return FVM_OK;
    });
}

int fvm_system_destroy(fvm_system* sys) {
    delete sys;
    return FVM_OK;
}

int fvm_system_info(const fvm_system* S, int64_t* info) {
    return guard_call([&] {
        if (!S || !info) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        info[0] = S->neq;
        info[1] = S->nblocks;
        info[2] = S->terms.n;
        info[3] = S->nvary;
        info[4] = S->ndir;
        info[5] = S->has_b ? 1 : 0;
        return FVM_OK;
    });
}

int fvm_system_rhs(fvm_system* S, const double* u, double* du, double t, int32_t flags, void* stream) {
    return guard_call([&] {
        if (!S || !u || !du) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        (void)t;  // device-coded forms are time independent
        cudaStream_t s = (cudaStream_t)stream;
        const int32_t loc = flags & 3;
        if (loc > FVM_PTR_DEVICE_INTERNAL) fail(FVM_ERR_INVALID_ARGUMENT, "bad pointer-location flag");
        if (loc == FVM_PTR_DEVICE_INTERNAL) {
            system_rhs_internal(S, u, du, s);
            return FVM_OK;
        }
        S->ensure_work();
        const int64_t n = S->n();
        const int32_t* perm = S->d_perm.as<int32_t>();
        if (loc == FVM_PTR_HOST) {
            FVM_CUDA(cudaMemcpyAsync(S->d_ref.p, u, sizeof(double) * n, cudaMemcpyHostToDevice, s));
            launch_permute_in(perm, S->d_ref.as<double>(), S->d_u.as<double>(), n, s);
        } else {
            launch_permute_in(perm, u, S->d_u.as<double>(), n, s);
        }
        system_rhs_internal(S, S->d_u.as<double>(), S->d_du.as<double>(), s);
        if (loc == FVM_PTR_HOST) {
            launch_permute_out(perm, S->d_du.as<double>(), S->d_ref.as<double>(), n, s);
            FVM_CUDA(cudaMemcpyAsync(du, S->d_ref.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
            FVM_CUDA(cudaStreamSynchronize(s));
        } else {
            launch_permute_out(perm, S->d_du.as<double>(), du, n, s);
        }
        FVM_CUDA(cudaGetLastError());
        return FVM_OK;
    });
}

int fvm_system_dirichlet_apply(fvm_system* S, double* u, double t, int32_t flags, void* stream) {
    return guard_call([&] {
        if (!S || !u) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        (void)t;
        cudaStream_t s = (cudaStream_t)stream;
        const int32_t loc = flags & 3;
        if (loc > FVM_PTR_DEVICE_INTERNAL) fail(FVM_ERR_INVALID_ARGUMENT, "bad pointer-location flag");
        if (loc == FVM_PTR_DEVICE_INTERNAL) {
            system_dirichlet_internal(S, u, s);
        } else {
            S->ensure_work();
            const int64_t n = S->n();
            const int32_t* perm = S->d_perm.as<int32_t>();
            if (loc == FVM_PTR_HOST)
                FVM_CUDA(cudaMemcpyAsync(S->d_ref.p, u, sizeof(double) * n, cudaMemcpyHostToDevice, s));
            launch_permute_in(perm, loc == FVM_PTR_HOST ? S->d_ref.as<double>() : u, S->d_u.as<double>(), n, s);
            system_dirichlet_internal(S, S->d_u.as<double>(), s);
            launch_permute_out(perm, S->d_u.as<double>(), loc == FVM_PTR_HOST ? S->d_ref.as<double>() : u, n, s);
            if (loc == FVM_PTR_HOST) {
                FVM_CUDA(cudaMemcpyAsync(u, S->d_ref.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
                FVM_CUDA(cudaStreamSynchronize(s));
            }
        }
        FVM_CUDA(cudaGetLastError());
        return FVM_OK;
    });
}

int fvm_system_tsit5_solve(fvm_system* S, const double* u0, const fvm_ode_options* opt, double* out,
                           fvm_ode_stats* stats, void* stream) {
    return guard_call([&] {
        if (!S || !u0 || !opt || !out) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        cudaStream_t s = (cudaStream_t)stream;
        const int64_t n = S->n();
        const int64_t nsave = (opt->saveat && opt->nsave > 0) ? opt->nsave : 1;
        DBuf d_in, d_out;
        d_in.alloc(sizeof(double) * n * 2);
        d_out.alloc(sizeof(double) * n * nsave);
        double* d_ref = d_in.as<double>();
        double* d_u0 = d_ref + n;
        FVM_CUDA(cudaMemcpyAsync(d_ref, u0, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        launch_permute_in(S->d_perm.as<int32_t>(), d_ref, d_u0, n, s);
        OdeRhs rhs;
        rhs.f = [S](const double* u, double* du, double, cudaStream_t st) { system_rhs_internal(S, u, du, st); };
        if (S->ndir > 0) rhs.callback = [S](double* u, double, cudaStream_t st) { system_dirichlet_internal(S, u, st); };
        tsit5_run_internal(rhs, n, d_u0, *opt, d_out.as<double>(), stats, s);
        snapshots_to_host(S->d_iperm.as<int32_t>(), d_out.as<double>(), out, n, nsave, s);
        FVM_CUDA(cudaStreamSynchronize(s));
        FVM_CUDA(cudaGetLastError());
        return FVM_OK;
    });
}

}  // extern "C"
