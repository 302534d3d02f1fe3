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

// Terms of the polynomial epilogue, grouped by monomial: monomial m is u_{f_m0} * ... *
// u_{f_m(nf_m - 1)} (degree nf_m <= 3, written as its factors) and is evaluated once per row;
// term[m][r] >= 0 adds coef * monomial to component r on the rows whose mask bit r is set.
struct SysTerms {
    int32_t n = 0;      // terms
    int32_t nmono = 0;  // distinct monomials
    uint8_t nf[kSysMaxTerms];
    uint8_t f[kSysMaxTerms][3];
    int16_t term[kSysMaxTerms][kSysMaxEq];
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
    uint32_t cmask;       // shared form: bit c set when some block reads component c
    double dmat[kSysMaxEq * kSysMaxEq];  // shared form: block (r, c) is dmat[r*N + c] times the one operator
};

// The N component values of point c: 16-byte loads when N is even and u is 16-byte aligned.
template <int N, bool VEC>
__device__ __forceinline__ void load_point(const double* __restrict__ u, int64_t c, double (&out)[N]) {
    if constexpr (VEC && N % 2 == 0) {
        const double2* p = reinterpret_cast<const double2*>(u + c * N);
#pragma unroll
        for (int h = 0; h < N / 2; ++h) {
            const double2 t = __ldg(p + h);
            out[2 * h] = t.x;
            out[2 * h + 1] = t.y;
        }
    } else {
#pragma unroll
        for (int q = 0; q < N; ++q) out[q] = __ldg(&u[c * N + q]);
    }
}

// ui[f] for a warp-uniform runtime f: a chain of selects, no FP64 instruction and no local memory.
template <int N>
__device__ __forceinline__ double pick(const double (&ui)[N], int f) {
    double v = ui[0];
#pragma unroll
    for (int q = 1; q < N; ++q) v = f == q ? ui[q] : v;
    return v;
}

// One warp per 32-row slice, one lane per row, slices grid-strided.  For a compile-time
// maximum width MAXW the slot loop is unrolled in three phases -- every column load, then
// every gather of the neighbours' N component values, then the FMAs of each stored block in
// slot order -- so a warp waits for one DRAM round trip and one gather round trip per slice
// instead of two per slot.  MAXW = 0 keeps a rolled loop for wide rows or many components.
// SH (shared form): the blocks are constant multiples dmat[r][c] of one stored operator G, so
// each slot reads one value; the row sums S_c = sum_k G_k u_c(col_k) are combined at the end.
template <int N, int MAXW, bool VEC, bool SH>
__global__ void __launch_bounds__(256) system_rhs_kernel(const SysArgs a, const SysTerms tm) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < a.nslices; s += nwarps) {
        const int64_t base = __ldg(&a.slice_ptr[s]) + lane;
        const int w = __ldg(&a.width[s]);
        double acc[N];
#pragma unroll
        for (int r = 0; r < N; ++r) acc[r] = 0.0;
        if constexpr (MAXW > 0) {
            int32_t c[MAXW];
#pragma unroll
            for (int k = 0; k < MAXW; ++k)
                if (k < w) c[k] = __ldg(&a.col[base + (int64_t)k * 32]);
            double uc[MAXW][N];
#pragma unroll
            for (int k = 0; k < MAXW; ++k)
                if (k < w) load_point<N, VEC>(a.u, c[k], uc[k]);
            const double* v = a.val + base;
            if constexpr (SH) {
                double sc[N];
#pragma unroll
                for (int q = 0; q < N; ++q) sc[q] = 0.0;
#pragma unroll
                for (int k = 0; k < MAXW; ++k)
                    if (k < w) {
                        const double g = __ldg(&v[(int64_t)k * 32]);
#pragma unroll
                        for (int q = 0; q < N; ++q)
                            if ((a.cmask >> q) & 1u) sc[q] = fma(g, uc[k][q], sc[q]);
                    }
#pragma unroll
                for (int r = 0; r < N; ++r)
#pragma unroll
                    for (int q = 0; q < N; ++q)
                        if ((a.blocks >> (r * N + q)) & 1ull) acc[r] = fma(a.dmat[r * N + q], sc[q], acc[r]);
            } else {
#pragma unroll
                for (int r = 0; r < N; ++r)
#pragma unroll
                    for (int q = 0; q < N; ++q)
                        if ((a.blocks >> (r * N + q)) & 1ull) {
#pragma unroll
                            for (int k = 0; k < MAXW; ++k)
                                if (k < w) acc[r] = fma(__ldg(&v[(int64_t)k * 32]), uc[k][q], acc[r]);
                            v += a.nslots;
                        }
            }
        } else if constexpr (SH) {
            double sc[N];
#pragma unroll
            for (int q = 0; q < N; ++q) sc[q] = 0.0;
#pragma unroll 2
            for (int k = 0; k < w; ++k) {
                const int64_t slot = base + (int64_t)k * 32;
                double uc[N];
                load_point<N, VEC>(a.u, __ldg(&a.col[slot]), uc);
                const double g = __ldg(&a.val[slot]);
#pragma unroll
                for (int q = 0; q < N; ++q)
                    if ((a.cmask >> q) & 1u) sc[q] = fma(g, uc[q], sc[q]);
            }
#pragma unroll
            for (int r = 0; r < N; ++r)
#pragma unroll
                for (int q = 0; q < N; ++q)
                    if ((a.blocks >> (r * N + q)) & 1ull) acc[r] = fma(a.dmat[r * N + q], sc[q], acc[r]);
        } else {
#pragma unroll 2
            for (int k = 0; k < w; ++k) {
                const int64_t slot = base + (int64_t)k * 32;
                double uc[N];
                load_point<N, VEC>(a.u, __ldg(&a.col[slot]), uc);
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
        }
        const int64_t row = s * 32 + lane;
        if (row >= a.nrows) continue;
        double ui[N];
        load_point<N, VEC>(a.u, row, ui);
        if (a.b) {
#pragma unroll
            for (int r = 0; r < N; ++r) acc[r] += a.b[row * N + r];
        }
        // the source / Dudt polynomials.  Loop bounds and branches are warp-uniform, each
        // distinct monomial is formed once (degree - 1 multiplications) and each term is one FMA
        // into the row's running sum, which the row's mask then keeps or drops: FP64 is the
        // scarce pipe on this GPU.
        const unsigned m = a.mask[row];
        double p[N];
#pragma unroll
        for (int r = 0; r < N; ++r) p[r] = acc[r];
        for (int mo = 0; mo < tm.nmono; ++mo) {
            const int nf = tm.nf[mo];
            double x = 1.0;
            if (nf > 0) {
                x = pick<N>(ui, tm.f[mo][0]);
                for (int k = 1; k < nf; ++k) x *= pick<N>(ui, tm.f[mo][k]);
            }
#pragma unroll
            for (int r = 0; r < N; ++r) {
                const int t = tm.term[mo][r];
                if (t >= 0) {
                    const double c = tm.vary[t] < 0 ? tm.coef[t] : __ldg(&a.vcoef[(int64_t)tm.vary[t] * a.nrows + row]);
                    p[r] = fma(c, x, p[r]);
                }
            }
        }
#pragma unroll
        for (int r = 0; r < N; ++r)
            if ((m >> r) & 1u) acc[r] = p[r];
        if constexpr (VEC && N % 2 == 0) {
            double2* o = reinterpret_cast<double2*>(a.du + row * N);
#pragma unroll
            for (int h = 0; h < N / 2; ++h) o[h] = make_double2(acc[2 * h], acc[2 * h + 1]);
        } else {
#pragma unroll
            for (int r = 0; r < N; ++r) a.du[row * N + r] = acc[r];
        }
    }
}

// The polynomial epilogue's share of the Jacobian, one thread per row.  With v: y += P'(u) v,
// each monomial's derivative along v being sum_k v_{f_k} prod_{j != k} u_{f_j}.  Without v:
// y[r] += dP_r/du_r, the diagonal.  Rows and components outside the mask get nothing, as in
// the right-hand side.
template <int N>
__global__ void system_poly_jacobian_kernel(const double* __restrict__ u, const double* __restrict__ v,
                                            double* __restrict__ y, const uint8_t* __restrict__ mask,
                                            const double* __restrict__ vcoef, int64_t nrows, const SysTerms tm) {
    const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= nrows) return;
    double ui[N], vi[N], acc[N];
    load_point<N, false>(u, row, ui);
    if (v) load_point<N, false>(v, row, vi);
#pragma unroll
    for (int r = 0; r < N; ++r) acc[r] = 0.0;
    for (int mo = 0; mo < tm.nmono; ++mo) {
        const int nf = tm.nf[mo];
        if (nf == 0) continue;  // a constant
        // prod_{j != k} u_{f_j} for each factor k
        double rest[3];
        for (int k = 0; k < nf; ++k) {
            double x = 1.0;
            for (int j = 0; j < nf; ++j)
                if (j != k) x *= pick<N>(ui, tm.f[mo][j]);
            rest[k] = x;
        }
        double dv = 0.0;
        if (v)
            for (int k = 0; k < nf; ++k) dv = fma(pick<N>(vi, tm.f[mo][k]), rest[k], dv);
#pragma unroll
        for (int r = 0; r < N; ++r) {
            const int t = tm.term[mo][r];
            if (t < 0) continue;
            double d = dv;
            if (!v) {
                d = 0.0;
                for (int k = 0; k < nf; ++k)
                    if (tm.f[mo][k] == r) d += rest[k];
            }
            const double c = tm.vary[t] < 0 ? tm.coef[t] : vcoef[(int64_t)tm.vary[t] * nrows + row];
            acc[r] = fma(c, d, acc[r]);
        }
    }
    const unsigned m = mask[row];
#pragma unroll
    for (int r = 0; r < N; ++r)
        if ((m >> r) & 1u) y[row * N + r] += acc[r];
}

// 1 on the [point][component] rows the system fixes (mask bit clear: Dirichlet, no triangle), else 0
__global__ void system_fixed_kernel(const uint8_t* mask, int N, int64_t n, double* fixed) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t row = i / N;
    const int r = (int)(i - row * N);
    fixed[i] = ((mask[row] >> r) & 1u) ? 0.0 : 1.0;
}

// the shared form's diagonal multipliers dmat[r][r]
struct SysDiagMat {
    double d[kSysMaxEq];
};

// diag[i][r] = K_rr[i][i], the diagonal blocks' diagonal entries, one thread per row
__global__ void system_block_diag_kernel(const int64_t* slice_ptr, const int32_t* width, const int32_t* col,
                                         const double* val, int64_t nslots, uint64_t blocks, int N, bool shared,
                                         const SysDiagMat dm, int64_t nrows, double* diag) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nrows) return;
    const int64_t s = i / 32;
    const int lane = (int)(i - s * 32);
    double g[kSysMaxEq];
    for (int r = 0; r < N; ++r) g[r] = 0.0;
    for (int k = 0; k < width[s]; ++k) {
        const int64_t slot = slice_ptr[s] + (int64_t)k * 32 + lane;
        if (col[slot] != i) continue;
        for (int r = 0; r < N; ++r) {
            const int bit = r * N + r;
            if (!((blocks >> bit) & 1ull)) continue;
            if (shared) {
                g[r] += dm.d[r] * val[slot];
            } else {
                const int idx = __popcll(blocks & ((1ull << bit) - 1));  // rank among the stored blocks
                g[r] += val[(int64_t)idx * nslots + slot];
            }
        }
    }
    for (int r = 0; r < N; ++r) diag[i * N + r] = g[r];
}

}  // namespace fvm

using namespace fvm;

struct fvm_system {
    fvm_mesh* mesh = nullptr;
    int neq = 0;
    int nblocks = 0;
    uint64_t blocks = 0;
    SysTerms terms;
    bool shared = false;   // every block is dmat[r][c] times the one stored operator
    uint32_t cmask = 0;
    double dmat[kSysMaxEq * kSysMaxEq] = {};
    int nvary = 0;
    bool has_b = false;
    int64_t ndir = 0;
    DBuf d_val, d_b, d_mask, d_vcoef, d_dir_idx, d_dir_val;
    // time factors: b(t) = b + sum_g tau_g(t) b_g, Dirichlet values val + sum_g tau_g(t) val_g
    int ntime = 0;
    bool tdir_varies = false;
    std::vector<double> tfac;  // [ntime][4]
    DBuf d_tb, d_tdir, d_beff; // [ntime][np][N] internal, [ntime][ndir], [np][N]
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

// unrolled width for N components and a pattern whose widest slice has maxw slots (0: rolled):
// exact widths for the common vertex degrees (no predicated-off slot costs an FP64 issue), and
// at most 32 gathered values per lane in registers
static int system_bucket(int N, int maxw) {
    for (int w : {4, 6, 7, 8, 12, 16})
        if (maxw <= w) return w * N <= 32 ? w : 0;
    return 0;
}

template <int N, int MAXW, bool VEC, bool SH>
static void launch_system_shape(const SysArgs& a, const SysTerms& tm, int64_t nslices, cudaStream_t s) {
    // 8 warps per block, one warp per slice up to 8 blocks for each of the 152 SMs; beyond that
    // the warps stride over the slices
    const unsigned grid = (unsigned)std::min<int64_t>((nslices + 7) / 8, 152 * 8);
    system_rhs_kernel<N, MAXW, VEC, SH><<<grid, 256, 0, s>>>(a, tm);
}

template <int N, bool VEC, bool SH>
static void launch_system_vec(const SysArgs& a, const SysTerms& tm, int64_t nslices, int maxw, cudaStream_t s) {
    switch (system_bucket(N, maxw)) {
        case 4: launch_system_shape<N, 4, VEC, SH>(a, tm, nslices, s); break;
        case 6: if constexpr (N <= 5) launch_system_shape<N, 6, VEC, SH>(a, tm, nslices, s); break;
        case 7: if constexpr (N <= 4) launch_system_shape<N, 7, VEC, SH>(a, tm, nslices, s); break;
        case 8: if constexpr (N <= 4) launch_system_shape<N, 8, VEC, SH>(a, tm, nslices, s); break;
        case 12: if constexpr (N <= 2) launch_system_shape<N, 12, VEC, SH>(a, tm, nslices, s); break;
        case 16: if constexpr (N <= 2) launch_system_shape<N, 16, VEC, SH>(a, tm, nslices, s); break;
        default: launch_system_shape<N, 0, VEC, SH>(a, tm, nslices, s); break;
    }
}

template <int N>
static void launch_system(const fvm_system* S, const double* u, double* du, const double* b, cudaStream_t s,
                          const SysTerms* terms = nullptr) {
    const SysTerms& tm = terms ? *terms : S->terms;
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
              b,
              S->d_mask.as<uint8_t>(),
              S->nvary ? S->d_vcoef.as<double>() : nullptr,
              S->cmask,
              {}};
    std::copy(S->dmat, S->dmat + kSysMaxEq * kSysMaxEq, a.dmat);
    const bool vec = N % 2 == 0 && ((uintptr_t)u % 16) == 0 && ((uintptr_t)du % 16) == 0;
    if (S->shared) {
        if (vec)
            launch_system_vec<N, true, true>(a, tm, p.nslices, p.maxw, s);
        else
            launch_system_vec<N, false, true>(a, tm, p.nslices, p.maxw, s);
    } else if (vec) {
        launch_system_vec<N, true, false>(a, tm, p.nslices, p.maxw, s);
    } else {
        launch_system_vec<N, false, false>(a, tm, p.nslices, p.maxw, s);
    }
}

static TimeTaus system_taus(const fvm_system* S, double t) {
    TimeTaus tt{};
    for (int g = 0; g < S->ntime; ++g) tt.tau[g] = time_factor_value(&S->tfac[4 * g], t);
    return tt;
}

static void system_rhs_internal(const fvm_system* S, const double* u, double* du, cudaStream_t s, double t) {
    const double* b = S->has_b ? S->d_b.as<double>() : nullptr;
    if (S->ntime > 0) {  // b(t) = b + sum_g tau_g(t) b_g
        launch_time_b(b, S->d_tb.as<double>(), system_taus(S, t), S->ntime, S->d_beff.as<double>(), S->n(), s);
        b = S->d_beff.as<double>();
    }
    switch (S->neq) {
        case 1: launch_system<1>(S, u, du, b, s); break;
        case 2: launch_system<2>(S, u, du, b, s); break;
        case 3: launch_system<3>(S, u, du, b, s); break;
        case 4: launch_system<4>(S, u, du, b, s); break;
        case 5: launch_system<5>(S, u, du, b, s); break;
        case 6: launch_system<6>(S, u, du, b, s); break;
        case 7: launch_system<7>(S, u, du, b, s); break;
        case 8: launch_system<8>(S, u, du, b, s); break;
        default: fail(FVM_ERR_INVALID_ARGUMENT, "neq out of range");
    }
    FVM_CUDA(cudaGetLastError());
}

static void system_dirichlet_internal(const fvm_system* S, double* u, cudaStream_t s, double t) {
    if (!S->ndir) return;
    if (S->ntime > 0)
        launch_dirichlet_time(S->d_dir_idx.as<int32_t>(), S->d_dir_val.as<double>(), S->d_tdir.as<double>(),
                              system_taus(S, t), S->ntime, u, S->ndir, s);
    else
        launch_dirichlet(S->d_dir_idx.as<int32_t>(), S->d_dir_val.as<double>(), u, S->ndir, s);
}

// J(u) v = K v + P'(u) v: the block operator on v with no constants and no polynomial terms, then
// the polynomials' derivatives (time factors enter the constants only: J does not depend on t)
template <int N>
static void system_jacobian_n(const fvm_system* S, const double* u, const double* v, double* y, cudaStream_t s) {
    const int64_t np = S->mesh->np;
    const unsigned grid = (unsigned)((np + 255) / 256);
    if (v) {
        const SysTerms none{};
        launch_system<N>(S, v, y, nullptr, s, &none);
    } else {
        const SellPattern& p = S->mesh->pat;
        SysDiagMat dm{};
        for (int r = 0; r < N; ++r) dm.d[r] = S->dmat[r * N + r];
        system_block_diag_kernel<<<grid, 256, 0, s>>>(p.d_slice_ptr.as<int64_t>(), p.d_width.as<int32_t>(),
                                                      p.d_col.as<int32_t>(), S->d_val.as<double>(), p.nslots,
                                                      S->blocks, N, S->shared, dm, np, y);
    }
    if (S->terms.nmono > 0)
        system_poly_jacobian_kernel<N><<<grid, 256, 0, s>>>(u, v, y, S->d_mask.as<uint8_t>(),
                                                            S->nvary ? S->d_vcoef.as<double>() : nullptr, np, S->terms);
}

// v non-null: y = J(u) v; v null: y = diag J(u)
static void system_jacobian_internal(const fvm_system* S, const double* u, const double* v, double* y, cudaStream_t s) {
    switch (S->neq) {
        case 1: system_jacobian_n<1>(S, u, v, y, s); break;
        case 2: system_jacobian_n<2>(S, u, v, y, s); break;
        case 3: system_jacobian_n<3>(S, u, v, y, s); break;
        case 4: system_jacobian_n<4>(S, u, v, y, s); break;
        case 5: system_jacobian_n<5>(S, u, v, y, s); break;
        case 6: system_jacobian_n<6>(S, u, v, y, s); break;
        case 7: system_jacobian_n<7>(S, u, v, y, s); break;
        case 8: system_jacobian_n<8>(S, u, v, y, s); break;
        default: fail(FVM_ERR_INVALID_ARGUMENT, "neq out of range");
    }
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

    // One pass of the linear-term visitor over component r's conditions: the operator of D (dual
    // samples D3, quarter samples D2; null = 0) plus the Neumann terms n0 + n1 u(m) of the
    // per-quarter-point pairs NQ ([2*nbe][2], null = none), on the pattern; b gets the constants.
    auto visit = [&](int r, const double* D3, const double* D2, const std::vector<double>* NQ, std::vector<double>& E,
                     std::vector<double>& b) {
        fvm_problem tp;  // host-side view of component r
        tp.mesh = m;
        tp.code.assign(d->vertex_code + r * np, d->vertex_code + (r + 1) * np);
        tp.bneu.assign(nbe, 0);
        for (int64_t e = 0; e < nbe; ++e) tp.bneu[e] = d->bedge_neumann[r * nbe + e] ? 1 : 0;
        tp.dif_deg = 0;
        tp.neu_deg = 1;
        if (NQ) tp.quarterN = *NQ;
        E.assign(pat.nslots, 0.0);
        std::vector<double> qv, rs;
        fvm_visit_linear_terms(
            &tp,
            [&](int32_t row, int32_t col, double coef, int64_t didx, bool) {
                double v = coef;
                if (didx >= 0) v *= didx < q0 ? (D3 ? D3[didx] : 0.0) : (D2 ? D2[didx - q0] : 0.0);
                E[pat.find(m->iperm[row], m->iperm[col])] += v;
            },
            b, qv, rs);
    };
    // per-quarter-point (n0, n_c) pairs of component r for the block (r, c); n0 only on the diagonal
    auto neumann_pairs = [&](int r, int c, bool with_n0, bool with_n1) {
        std::vector<double> nq((size_t)2 * nbe * 2, 0.0);
        for (int64_t qp = 0; qp < 2 * nbe; ++qp) {
            const double* a = d->quarter_neumann + ((size_t)r * 2 * nbe + qp) * (1 + N);
            nq[2 * qp] = with_n0 ? a[0] : 0.0;
            nq[2 * qp + 1] = with_n1 ? a[1 + c] : 0.0;
        }
        return nq;
    };
    const double* DD = d->dual_edge_D;
    const double* DQ = d->quarter_D;

    // Shared form: when every component has the same conditions, no Neumann value depends on u and
    // every block's D is one constant d_rc at all its samples, block (r, c) is d_rc times the
    // operator G of those conditions with D = 1, and G is stored once.
    bool shared = true;
    for (int r = 1; r < N && shared; ++r)
        shared = std::equal(d->vertex_code + r * np, d->vertex_code + (r + 1) * np, d->vertex_code) &&
                 (nbe == 0 || std::equal(d->bedge_neumann + r * nbe, d->bedge_neumann + (r + 1) * nbe, d->bedge_neumann));
    if (shared && d->quarter_neumann)
        for (int r = 0; r < N && shared; ++r)
            for (int64_t qp = 0; qp < 2 * nbe && shared; ++qp)
                for (int c = 0; c < N && shared; ++c)
                    shared = d->quarter_neumann[((size_t)r * 2 * nbe + qp) * (1 + N) + 1 + c] == 0.0;
    std::vector<double> dconst((size_t)N * N, 0.0);
    for (size_t blk = 0; blk < (size_t)N * N && shared; ++blk) {
        bool first = true;
        double v0 = 0.0;
        auto scan = [&](const double* a, int64_t n) {
            for (int64_t i = 0; i < n && shared; ++i) {
                if (first) {
                    v0 = a[i];
                    first = false;
                } else if (a[i] != v0) {
                    shared = false;
                }
            }
        };
        if (DD) scan(DD + blk * 3 * nt, 3 * nt);
        if (DQ) scan(DQ + blk * 2 * nbe, 2 * nbe);
        dconst[blk] = (DD || DQ) ? v0 : 0.0;
    }

    // The shared form reads one value per slot but spends N FP64 FMAs per slot and one per block
    // and row; the stored blocks spend one per block and slot.  FP64 issue, not DRAM, bounds
    // these kernels on this GPU, so the shared form is kept only when it issues fewer.
    if (shared) {
        int nb = 0;
        uint32_t cols = 0;
        for (int r = 0; r < N; ++r)
            for (int c = 0; c < N; ++c)
                if (dconst[(size_t)r * N + c] != 0.0) {
                    ++nb;
                    cols |= 1u << c;
                }
        const double w = pat.nrows ? (double)pat.nslots / (double)pat.nrows : 0.0;
        shared = (double)__builtin_popcount(cols) * w + nb < (double)nb * w;
    }
    std::vector<double> vals, B((size_t)np * N, 0.0), E, b;
    if (shared) {
        std::vector<double> ones3(3 * nt, 1.0), ones2(2 * nbe, 1.0);
        visit(0, ones3.data(), ones2.data(), nullptr, E, b);
        vals = E;
        for (int r = 0; r < N; ++r) {
            if (d->quarter_neumann) {
                const std::vector<double> nq = neumann_pairs(r, r, true, false);
                visit(r, nullptr, nullptr, &nq, E, b);
                for (int64_t i = 0; i < np; ++i) B[(size_t)i * N + r] = b[i];
            }
            for (int c = 0; c < N; ++c)
                if (dconst[(size_t)r * N + c] != 0.0) {
                    S->blocks |= 1ull << (r * N + c);
                    S->cmask |= 1u << c;
                    S->dmat[r * N + c] = dconst[(size_t)r * N + c];
                    ++S->nblocks;
                }
        }
        S->shared = true;
    } else {
        // coupled blocks K_rc, stored one after another; the Neumann constants from the (r, r) pass
        for (int r = 0; r < N; ++r)
            for (int c = 0; c < N; ++c) {
                const size_t blk = (size_t)r * N + c;
                std::vector<double> nq;
                if (d->quarter_neumann) nq = neumann_pairs(r, c, c == r, true);
                visit(r, DD ? DD + blk * 3 * nt : nullptr, DQ ? DQ + blk * 2 * nbe : nullptr,
                      d->quarter_neumann ? &nq : nullptr, E, b);
                if (c == r)
                    for (int64_t i = 0; i < np; ++i) B[(size_t)i * N + r] = b[i];
                if (std::any_of(E.begin(), E.end(), [](double x) { return x != 0.0; })) {
                    S->blocks |= 1ull << (r * N + c);
                    ++S->nblocks;
                    vals.insert(vals.end(), E.begin(), E.end());
                }
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
    SysTerms& T = S->terms;
    for (int mo = 0; mo < nmono; ++mo) {
        bool used = false;
        for (int r = 0; r < N; ++r) {
            T.term[T.nmono][r] = -1;
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
            if (T.n == kSysMaxTerms)
                fail(FVM_ERR_UNSUPPORTED_FORM, "more than " + std::to_string(kSysMaxTerms) + " source / Dudt terms");
            used = true;
            T.term[T.nmono][r] = (int16_t)T.n;
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
        if (!used) continue;
        int nf = 0;
        for (int c = 0; c < N; ++c)
            for (int e = 0; e < d->mono_exp[mo * N + c]; ++e) T.f[T.nmono][nf++] = (uint8_t)c;
        for (int k = nf; k < 3; ++k) T.f[T.nmono][k] = 0;
        T.nf[T.nmono] = (uint8_t)nf;
        ++T.nmono;
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

    // time factors: per factor, the constant terms of each component (as the Neumann constants
    // above) and the Dirichlet values in the order of idx
    if (d->ntime < 0 || d->ntime > FVM_MAX_TIME_FACTORS)
        fail(FVM_ERR_INVALID_ARGUMENT, "ntime must lie in [0, FVM_MAX_TIME_FACTORS]");
    if (d->ntime > 0) {
        if (!d->time_factor) fail(FVM_ERR_INVALID_ARGUMENT, "time_factor is required when ntime > 0");
        S->ntime = d->ntime;
        S->tfac.assign(d->time_factor, d->time_factor + 4 * S->ntime);
        for (int g = 0; g < S->ntime; ++g) {
            const double* f = &S->tfac[4 * g];
            if (f[0] != 1.0 && f[0] != 2.0) fail(FVM_ERR_INVALID_ARGUMENT, "time_factor kind must be 1 or 2");
            if (!std::isfinite(f[1]) || !std::isfinite(f[2]) || !std::isfinite(f[3]))
                fail(FVM_ERR_INVALID_ARGUMENT, "time_factor values must be finite");
        }
        const size_t G = (size_t)S->ntime;
        finite(d->time_dirichlet, G * N * np, "time_dirichlet");
        finite(d->time_neumann, G * N * 2 * nbe, "time_neumann");
        finite(d->time_source, G * N * np, "time_source");
        finite(d->time_dudt, G * N * np, "time_dudt");
        std::vector<double> tb(G * np * N, 0.0), tdir(G * std::max<int64_t>(S->ndir, 1), 0.0);
        for (int g = 0; g < S->ntime; ++g) {
            for (int r = 0; r < N; ++r) {
                fvm_problem tp;  // host-side view of component r
                tp.mesh = m;
                tp.code.assign(d->vertex_code + r * np, d->vertex_code + (r + 1) * np);
                tp.bneu.assign(nbe, 0);
                for (int64_t e = 0; e < nbe; ++e) tp.bneu[e] = d->bedge_neumann[r * nbe + e] ? 1 : 0;
                const size_t gr = (size_t)g * N + r;
                std::vector<double> bg = fvm_time_constant_terms(
                    &tp, d->time_neumann ? d->time_neumann + gr * 2 * nbe : nullptr,
                    d->time_source ? d->time_source + gr * np : nullptr, d->time_dudt ? d->time_dudt + gr * np : nullptr);
                for (int64_t i = 0; i < np; ++i) tb[((size_t)g * np + i) * N + r] = bg[i];
            }
            if (d->time_dirichlet) {
                int64_t k = 0;
                for (int r = 0; r < N; ++r)
                    for (int64_t v = 0; v < np; ++v)
                        if (d->vertex_code[r * np + v] == FVM_VERTEX_DIRICHLET) {
                            const double x = d->time_dirichlet[((size_t)g * N + r) * np + v];
                            S->tdir_varies |= x != 0.0;
                            tdir[(size_t)g * S->ndir + k++] = x;
                        }
            }
        }
        S->d_tb.upload(tb);
        S->d_tdir.upload(tdir);
        S->d_beff.alloc(sizeof(double) * np * N);
    }

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
        info[6] = S->shared ? 1 : 0;
        return FVM_OK;
    });
}

int fvm_system_rhs(fvm_system* S, const double* u, double* du, double t, int32_t flags, void* stream) {
    return guard_call([&] {
        if (!S || !u || !du) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        cudaStream_t s = (cudaStream_t)stream;
        const int32_t loc = flags & 3;
        if (loc > FVM_PTR_DEVICE_INTERNAL) fail(FVM_ERR_INVALID_ARGUMENT, "bad pointer-location flag");
        if (loc == FVM_PTR_DEVICE_INTERNAL) {
            system_rhs_internal(S, u, du, s, t);
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
        system_rhs_internal(S, S->d_u.as<double>(), S->d_du.as<double>(), s, t);
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
        cudaStream_t s = (cudaStream_t)stream;
        const int32_t loc = flags & 3;
        if (loc > FVM_PTR_DEVICE_INTERNAL) fail(FVM_ERR_INVALID_ARGUMENT, "bad pointer-location flag");
        if (loc == FVM_PTR_DEVICE_INTERNAL) {
            system_dirichlet_internal(S, u, s, t);
        } else {
            S->ensure_work();
            const int64_t n = S->n();
            const int32_t* perm = S->d_perm.as<int32_t>();
            if (loc == FVM_PTR_HOST)
                FVM_CUDA(cudaMemcpyAsync(S->d_ref.p, u, sizeof(double) * n, cudaMemcpyHostToDevice, s));
            launch_permute_in(perm, loc == FVM_PTR_HOST ? S->d_ref.as<double>() : u, S->d_u.as<double>(), n, s);
            system_dirichlet_internal(S, S->d_u.as<double>(), s, t);
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
        rhs.f = [S](const double* u, double* du, double t, cudaStream_t st) { system_rhs_internal(S, u, du, st, t); };
        if (S->ndir > 0)
            rhs.callback = [S](double* u, double t, cudaStream_t st) { system_dirichlet_internal(S, u, st, t); };
        rhs.time_dependent = S->ntime > 0;
        rhs.callback_varies = S->tdir_varies;
        tsit5_run_internal(rhs, n, d_u0, *opt, d_out.as<double>(), stats, s);
        snapshots_to_host(S->d_iperm.as<int32_t>(), d_out.as<double>(), out, n, nsave, s);
        FVM_CUDA(cudaStreamSynchronize(s));
        FVM_CUDA(cudaGetLastError());
        return FVM_OK;
    });
}

}  // extern "C"

namespace {

// y = J(u) v (v non-null) or diag J(u), with u, v, y per the pointer-location flag
void system_jacobian_entry(fvm_system* S, const double* u, const double* v, double* y, int32_t flags,
                           cudaStream_t s) {
    const int32_t loc = flags & 3;
    if (loc > FVM_PTR_DEVICE_INTERNAL) fail(FVM_ERR_INVALID_ARGUMENT, "bad pointer-location flag");
    if (loc == FVM_PTR_DEVICE_INTERNAL) {
        system_jacobian_internal(S, u, v, y, s);
        FVM_CUDA(cudaGetLastError());
        return;
    }
    const int64_t n = S->n();
    const int32_t* perm = S->d_perm.as<int32_t>();
    DBuf w;
    w.alloc(sizeof(double) * 4 * n);
    double *ui = w.as<double>(), *vi = ui + n, *yi = ui + 2 * n, *st = ui + 3 * n;
    auto in = [&](const double* src, double* dst) {
        const double* from = src;
        if (loc == FVM_PTR_HOST) {
            FVM_CUDA(cudaMemcpyAsync(st, src, sizeof(double) * n, cudaMemcpyHostToDevice, s));
            from = st;
        }
        launch_permute_in(perm, from, dst, n, s);
    };
    in(u, ui);
    if (v) in(v, vi);
    system_jacobian_internal(S, ui, v ? vi : nullptr, yi, s);
    double* dst = loc == FVM_PTR_HOST ? st : y;
    launch_permute_out(perm, yi, dst, n, s);
    if (loc == FVM_PTR_HOST) FVM_CUDA(cudaMemcpyAsync(y, st, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    FVM_CUDA(cudaStreamSynchronize(s));
    FVM_CUDA(cudaGetLastError());
}

}  // namespace

extern "C" {

int fvm_system_jvp(fvm_system* S, const double* u, const double* v, double* jv, double t, int32_t flags,
                   void* stream) {
    return guard_call([&] {
        if (!S || !u || !v || !jv) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        (void)t;  // time factors enter the constants only
        system_jacobian_entry(S, u, v, jv, flags, (cudaStream_t)stream);
        return FVM_OK;
    });
}

int fvm_system_jacobian_diagonal(fvm_system* S, const double* u, double* diag, double t, int32_t flags,
                                 void* stream) {
    return guard_call([&] {
        if (!S || !u || !diag) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        (void)t;
        system_jacobian_entry(S, u, nullptr, diag, flags, (cudaStream_t)stream);
        return FVM_OK;
    });
}

int fvm_system_trbdf2_solve(fvm_system* S, const double* u0, const fvm_ode_options* opt, double* out,
                            fvm_ode_stats* stats, fvm_implicit_stats* istats, void* stream) {
    return guard_call([&] {
        if (!S) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        ImplicitRhs R;
        R.f = [S](const double* y, double* du, double t, cudaStream_t s) { system_rhs_internal(S, y, du, s, t); };
        R.jvp = [S](const double* u, const double* v, double* jv, cudaStream_t s) {
            system_jacobian_internal(S, u, v, jv, s);
        };
        R.diag = [S](const double* u, double* d, cudaStream_t s) { system_jacobian_internal(S, u, nullptr, d, s); };
        if (S->ndir > 0)
            R.callback = [S](double* u, double t, cudaStream_t s) { system_dirichlet_internal(S, u, s, t); };
        R.callback_varies = S->tdir_varies;
        bool affine = true;  // no monomial of degree two or more
        for (int mo = 0; mo < S->terms.nmono; ++mo) affine = affine && S->terms.nf[mo] <= 1;
        R.affine = affine;
        return trbdf2_run(R, S->d_perm.as<int32_t>(), S->d_iperm.as<int32_t>(), S->n(), u0, opt, out, stats, istats,
                          stream);
    });
}

int fvm_system_steady_solve(fvm_system* S, const double* u0, const fvm_steady_options* opt, double* out,
                            fvm_steady_stats* stats, void* stream) {
    return guard_call([&] {
        if (!S) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        const int64_t n = S->n();
        DBuf d_fixed;
        d_fixed.alloc(sizeof(double) * n);
        system_fixed_kernel<<<(unsigned)((n + 255) / 256), 256>>>(S->d_mask.as<uint8_t>(), S->neq, n,
                                                                  d_fixed.as<double>());
        FVM_CUDA(cudaGetLastError());
        FVM_CUDA(cudaDeviceSynchronize());
        ImplicitRhs R;
        R.f = [S](const double* y, double* du, double t, cudaStream_t s) { system_rhs_internal(S, y, du, s, t); };
        R.jvp = [S](const double* u, const double* v, double* jv, cudaStream_t s) {
            system_jacobian_internal(S, u, v, jv, s);
        };
        R.diag = [S](const double* u, double* d, cudaStream_t s) { system_jacobian_internal(S, u, nullptr, d, s); };
        if (S->ndir > 0)
            R.callback = [S](double* u, double t, cudaStream_t s) { system_dirichlet_internal(S, u, s, t); };
        R.callback_varies = S->tdir_varies;
        bool affine = true;
        for (int mo = 0; mo < S->terms.nmono; ++mo) affine = affine && S->terms.nf[mo] <= 1;
        R.affine = affine;
        R.fixed = d_fixed.as<double>();
        steady_run(R, S->d_perm.as<int32_t>(), S->d_iperm.as<int32_t>(), n, u0, opt, out, stats, stream);
        return FVM_OK;
    });
}

}  // extern "C"
