// Implicit time stepping on the device: the Jacobian-vector product of fvm_eqs! and TR-BDF2
// with simplified Newton and matrix-free BiCGStab.
//
// The reference hands its ODEProblem, with jac_prototype = jacobian_sparsity(prob)
// (src/solve.jl:50-131,167-183), to OrdinaryDiffEq's implicit solvers; its tutorials use TRBDF2
// (docs/src/literate_tutorials/diffusion_equation_on_an_annulus.jl:64,
// docs/src/tutorials/diffusion_equation_on_a_square_plate.md).  Here the Jacobian is never
// formed: J(u) v is one launch (the operator itself on the linear path, the derivative of the
// per-triangle kernel otherwise, fvm_kernels.cu), and each TR-BDF2 stage solves its Newton
// systems W d = r, W = I - d h J(u_n), with BiCGStab preconditioned by diag(W).
//
// TR-BDF2 as in Hosea & Shampine, "Analysis and implementation of TR-BDF2", Appl. Numer. Math.
// 20 (1996): gamma = 2 - sqrt 2, d = gamma / 2, w = sqrt 2 / 4, z = h f:
//   trapezoidal stage to t + gamma h:  z_g = h f(u_n + d z_n + d z_g)
//   BDF2 stage to t + h:              z_1 = h f(u_n + w z_n + w z_g + d z_1),
//                                     u_{n+1} = u_n + w z_n + w z_g + d z_1
//   error estimate (filtered by W):   est = W^-1 ((1 - sqrt 2)/3 z_n + 1/3 z_g + (sqrt 2 - 2)/3 z_1)
// Step control: accept when RMS(est / (abstol + reltol max(|u_n|, |u_{n+1}|))) <= 1, and
// h <- h min(10, max(0.2, 0.9 err^(-1/3))).  A stage whose Newton iteration does not converge
// in 10 iterations (or diverges) retries the step with h / 4.  saveat values inside a step
// are the cubic Hermite interpolant of (u_n, f_n), (u_{n+1}, f_{n+1}).  The Dirichlet update
// runs after every accepted step, as with Tsit5.
#include "fvm_internal.h"
#include "fvm_tma.cuh"
#include <algorithm>
#include <cmath>
#include <vector>

namespace fvm {
namespace {

constexpr int kThreads = 256;
constexpr int kParts = 304;  // blocks of the reductions (2 per SM): partials summed on the host in order

inline unsigned blocks_for(int64_t n) { return (unsigned)std::max<int64_t>(1, (n + kThreads - 1) / kThreads); }

// out = c0 x0 + c1 x1 + c2 x2 + c3 x3 (null terms skipped); out may alias an input
struct Lin {
    const double* x[4];
    double c[4];
};
__global__ void lin_kernel(double* out, Lin L, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (L.x[j]) acc += L.c[j] * L.x[j][i];
    out[i] = acc;
}
void lin(double* out, const Lin& L, int64_t n, cudaStream_t s) {
    lin_kernel<<<blocks_for(n), kThreads, 0, s>>>(out, L, n);
}
Lin lin2(const double* a, double ca, const double* b, double cb) {
    Lin L{};
    L.x[0] = a;
    L.c[0] = ca;
    L.x[1] = b;
    L.c[1] = cb;
    return L;
}

// two dot products per pass, partials per block: part[2 * b + k]
__global__ void dot2_kernel(const double* a0, const double* b0, const double* a1, const double* b1, int64_t n,
                            double* part) {
    __shared__ double red[2][kThreads];
    double s0 = 0.0, s1 = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        s0 += a0[i] * b0[i];
        if (a1) s1 += a1[i] * b1[i];
    }
    red[0][threadIdx.x] = s0;
    red[1][threadIdx.x] = s1;
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            red[0][threadIdx.x] += red[0][threadIdx.x + w];
            red[1][threadIdx.x] += red[1][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = red[0][0];
        part[2 * blockIdx.x + 1] = red[1][0];
    }
}

// sum of (x / (abstol + reltol max(|a|, |b|)))^2, partials per block (b may be null)
__global__ void wnorm_kernel(const double* x, const double* a, const double* b, double abstol, double reltol,
                             int64_t n, double* part) {
    __shared__ double red[kThreads];
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double sc = abstol + reltol * (b ? fmax(fabs(a[i]), fabs(b[i])) : fabs(a[i]));
        const double r = x[i] / sc;
        s += r * r;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// y = x / dw (Jacobi), dw = 1 - c diagJ
__global__ void jacobi_kernel(const double* x, const double* dw, double* y, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = x[i] / dw[i];
}
__global__ void wdiag_kernel(const double* dj, double c, double* dw, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dw[i] = 1.0 - c * dj[i];
}
// W = F - c J with F = diag(mask) (steady Newton): out = mask x - c out, out holding J x
__global__ void wmask_kernel(double* out, const double* x, const double* mask, double c, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = mask[i] * x[i] - c * out[i];
}
// its diagonal mask - c diagJ; a zero (a row that does not depend on its own value) taken as 1
__global__ void wdiag_mask_kernel(const double* dj, const double* mask, double c, double* dw, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double d = mask[i] - c * dj[i];
    dw[i] = d != 0.0 ? d : 1.0;
}
// max|f| and max|f + u|, partials per block: part[2 b], part[2 b + 1]
__global__ void maxabs2_kernel(const double* f, const double* u, int64_t n, double* part) {
    __shared__ double red[2][kThreads];
    double m0 = 0.0, m1 = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        m0 = fmax(m0, fabs(f[i]));
        m1 = fmax(m1, fabs(f[i] + u[i]));
    }
    red[0][threadIdx.x] = m0;
    red[1][threadIdx.x] = m1;
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            red[0][threadIdx.x] = fmax(red[0][threadIdx.x], red[0][threadIdx.x + w]);
            red[1][threadIdx.x] = fmax(red[1][threadIdx.x], red[1][threadIdx.x + w]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = red[0][0];
        part[2 * blockIdx.x + 1] = red[1][0];
    }
}
// the diagonal of a sliced-ELL operator: padding slots name the row itself with value 0
template <class V>
__global__ void sell_diag_kernel(const int64_t* slice_ptr, const int32_t* width, const int32_t* col, const V* val,
                                 const double* rowscale, int64_t nrows, double* diag) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    const int64_t s = r / kSlice;
    const int lane = (int)(r - s * kSlice);
    double d = 0.0;
    for (int k = 0; k < width[s]; ++k) {
        const int64_t slot = slice_ptr[s] + (int64_t)k * kSlice + lane;
        if (col[slot] == r) d += (double)val[slot];
    }
    diag[r] = rowscale ? d * rowscale[r] : d;
}

// BiCGStab with its scalars in device memory: each dot product's block partials are summed in a
// fixed order by one finalize kernel, which also updates the scalars; the vector kernels read
// them, and every kernel does nothing once `status` is set (1 converged, 2 breakdown), so the
// host checks only every few iterations.
struct KDev {
    double rho, rho_prev, alpha, omega, bb, tol2, rr;
    int32_t status, it;
};
// the two sums of the partials part[2 b + k] over the blocks, by a fixed tree over one block of
// kFin threads (deterministic); valid in thread 0
constexpr int kFin = 512;
static_assert(kParts <= kFin, "one finalize thread per partial");
__device__ void sum_parts2(const double* part, double& s0, double& s1) {
    __shared__ double a[kFin], b[kFin];
    const int t = threadIdx.x;
    a[t] = t < kParts ? part[2 * t] : 0.0;
    b[t] = t < kParts ? part[2 * t + 1] : 0.0;
    __syncthreads();
    for (int w = kFin / 2; w > 0; w >>= 1) {
        if (t < w) {
            a[t] += a[t + w];
            b[t] += b[t + w];
        }
        __syncthreads();
    }
    s0 = a[0];
    s1 = b[0];
}
__global__ void kd_init_kernel(KDev* kd, const double* part, double tol2) {
    double s0, s1;
    sum_parts2(part, s0, s1);
    if (threadIdx.x) return;
    kd->rho = s0;
    kd->bb = s1;
    kd->tol2 = tol2;
    kd->rho_prev = kd->alpha = kd->omega = 1.0;
    kd->rr = kd->bb;
    kd->it = 0;
    kd->status = kd->bb > 0.0 ? 0 : 1;
}
// p = r (first iteration) or p = r + beta (p - omega v), beta = (rho / rho_prev)(alpha / omega)
__global__ void kd_p_kernel(const KDev* kd, const double* r, double* p, const double* v, int64_t n) {
    if (kd->status) return;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (kd->it == 0) {
        p[i] = r[i];
    } else {
        const double beta = (kd->rho / kd->rho_prev) * (kd->alpha / kd->omega);
        p[i] = r[i] + beta * (p[i] - kd->omega * v[i]);
    }
}
__global__ void kd_alpha_kernel(KDev* kd, const double* part) {
    if (kd->status) return;  // uniform over the block: status changes only after the sums
    double rv, unused;
    sum_parts2(part, rv, unused);
    if (threadIdx.x) return;
    if (!(rv != 0.0) || !isfinite(rv)) {
        kd->status = 2;
        return;
    }
    kd->alpha = kd->rho / rv;
}
__global__ void kd_s_kernel(const KDev* kd, const double* r, const double* v, double* s, int64_t n) {
    if (kd->status) return;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) s[i] = r[i] - kd->alpha * v[i];
}
__global__ void kd_omega_kernel(KDev* kd, const double* part) {
    if (kd->status) return;
    double ts, tt;
    sum_parts2(part, ts, tt);
    if (threadIdx.x) return;
    kd->omega = tt > 0.0 ? ts / tt : 0.0;
}
// x += alpha ph + omega sh; r = s - omega t
__global__ void kd_xr_kernel(const KDev* kd, double* x, const double* ph, const double* sh, const double* s,
                             const double* t, double* r, int64_t n) {
    if (kd->status) return;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    x[i] = x[i] + kd->alpha * ph[i] + kd->omega * sh[i];
    r[i] = s[i] - kd->omega * t[i];
}
__global__ void kd_rho_kernel(KDev* kd, const double* part) {
    if (kd->status) return;
    double rho, rr;
    sum_parts2(part, rho, rr);
    if (threadIdx.x) return;
    kd->rho_prev = kd->rho;
    kd->rho = rho;
    kd->rr = rr;
    kd->it += 1;
    if (!isfinite(kd->rr))
        kd->status = 2;
    else if (kd->rr <= kd->tol2 * kd->bb)
        kd->status = 1;
    else if (!(kd->omega != 0.0) || !(kd->rho != 0.0))
        kd->status = 2;
}

// ---------------------------------------------------------------------------------------
// The whole BiCGStab solve in one cooperative launch, for an operator J = A (+ diag(2 q u))
// held as a sliced-ELL matrix (the linear problems and the time-dependent templates).  At
// small and medium sizes an iteration of the launch-per-step solver is a dozen launches of a
// few microseconds each; here it is three grid barriers.  CTA c owns the contiguous slices
// [S c / G, S (c+1) / G) for every vector operation and product, one warp per slice.  Each
// iteration has three phases, each ending in a grid barrier:
//   A  p = r + beta (p' - omega v') (ping-pong: p', v' are the previous iteration's, read by
//      the neighbours' gathers, which form p on the fly), v = W (p / dw), partial <rhat, v>
//   B  s = r - alpha v, t = W (s / dw) (the gathers form s on the fly), partials <t,s>, <t,t>
//   C  x += alpha p/dw + omega s/dw, r = s - omega t, partials <rhat,r>, <r,r>
// Every CTA sums the G partials in the same fixed tree, so every CTA holds the same scalars and
// takes the same branch (converged, breakdown, iteration limit).  Values another CTA wrote in
// this launch are read through L2 (ld.global.cg).  The grid barrier is a counter and a
// generation word; its wait is bounded, and a barrier that runs out sets the error word and
// ends the solve with a breakdown status.
// ---------------------------------------------------------------------------------------
constexpr int kCoopThreads = 256;
constexpr int kCoopMaxCtas = 256;             // one partial per thread of the final sum
constexpr unsigned kDevErrGridBarrier = 8u;   // a grid barrier of the cooperative solve ran out

struct CoopResult {
    int32_t status, it;  // 1 converged, 2 breakdown or iteration limit
};

struct CoopKrylov {
    const int64_t* slice_ptr;
    const int32_t* width;
    const int32_t* col;
    const double* val;   // A
    const double* q;     // J = A + diag(2 q u), or null
    const double* u;     // J's point (for q)
    const double* mask;  // W = diag(mask) - c J, or null for I - c J
    double c;
    const double* dw;    // diag(W), the Jacobi preconditioner
    const double* b;
    double* x;
    double *r, *rhat, *p0, *p1, *v0, *v1, *s, *t;
    double* part;        // [2][kCoopMaxCtas]
    unsigned *bar_count, *bar_gen, *err;
    CoopResult* res;
    int64_t n, nslices;
    double tol2;
    int maxit;
    unsigned long long wait_ns;
};

__device__ __forceinline__ unsigned coop_ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void coop_st_release(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// all CTAs of the (co-resident) grid; false when the wait ran out
__device__ bool coop_grid_barrier(const CoopKrylov& k, int* s_ok) {
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned g = coop_ld_acquire(k.bar_gen);
        if (atomicAdd(k.bar_count, 1u) + 1u == gridDim.x) {
            atomicExch(k.bar_count, 0u);
            __threadfence();
            coop_st_release(k.bar_gen, g + 1u);
        } else {
            const unsigned long long t0 = global_ns();
            while (coop_ld_acquire(k.bar_gen) == g) {
                __nanosleep(32);
                if (global_ns() - t0 > k.wait_ns) {
                    atomicOr(k.err, kDevErrGridBarrier);
                    ok = 0;
                    break;
                }
            }
        }
        __threadfence();
        *s_ok = ok;
    }
    __syncthreads();
    return *s_ok != 0;
}

// the CTA's partial sums of a0 (and a1) into part[0][cta] (part[1][cta]), fixed order
__device__ void coop_block_partials(double a0, double a1, const CoopKrylov& k, double (*red)[kCoopThreads / 32]) {
    for (int o = 16; o > 0; o >>= 1) {
        a0 += __shfl_down_sync(0xffffffffu, a0, o);
        a1 += __shfl_down_sync(0xffffffffu, a1, o);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        red[0][warp] = a0;
        red[1][warp] = a1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s0 = 0.0, s1 = 0.0;
        for (int w = 0; w < kCoopThreads / 32; ++w) {
            s0 += red[0][w];
            s1 += red[1][w];
        }
        k.part[blockIdx.x] = s0;
        k.part[kCoopMaxCtas + blockIdx.x] = s1;
    }
}

// the two sums over the grid's partials, by the same fixed tree in every CTA (after a barrier)
__device__ void coop_grid_sums(const CoopKrylov& k, double (*fin)[kCoopThreads], double& s0, double& s1) {
    const int t = threadIdx.x;
    fin[0][t] = t < (int)gridDim.x ? __ldcg(&k.part[t]) : 0.0;
    fin[1][t] = t < (int)gridDim.x ? __ldcg(&k.part[kCoopMaxCtas + t]) : 0.0;
    __syncthreads();
    for (int w = kCoopThreads / 2; w > 0; w >>= 1) {
        if (t < w) {
            fin[0][t] += fin[0][t + w];
            fin[1][t] += fin[1][t + w];
        }
        __syncthreads();
    }
    s0 = fin[0][0];
    s1 = fin[1][0];
    __syncthreads();  // fin is reused by the next sum
}

// the product W y at row i for y formed on the fly by ycol(col): y_i / dw_i times the mask (or 1)
// minus c (A y + 2 q u y)_i
template <class Y>
__device__ __forceinline__ double coop_w_row(const CoopKrylov& k, int64_t s, int lane, int64_t i, double yi,
                                             Y ycol) {
    const int64_t base = __ldg(&k.slice_ptr[s]) + lane;
    const int w = __ldg(&k.width[s]);
    double acc = 0.0;
#pragma unroll 4
    for (int j = 0; j < w; ++j) {
        const int64_t slot = base + (int64_t)j * 32;
        const int32_t c = __ldg(&k.col[slot]);
        acc += __ldg(&k.val[slot]) * (ycol(c) / __ldg(&k.dw[c]));
    }
    const double yh = yi / __ldg(&k.dw[i]);
    if (k.q) acc += 2.0 * __ldg(&k.q[i]) * __ldg(&k.u[i]) * yh;
    const double m = k.mask ? __ldg(&k.mask[i]) : 1.0;
    return m * yh - k.c * acc;
}

__global__ void __launch_bounds__(kCoopThreads) coop_bicgstab_kernel(const CoopKrylov k) {
    __shared__ double red[2][kCoopThreads / 32];
    __shared__ double fin[2][kCoopThreads];
    __shared__ int s_ok;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t s0 = k.nslices * blockIdx.x / gridDim.x, s1 = k.nslices * (blockIdx.x + 1) / gridDim.x;
    constexpr int kWarps = kCoopThreads / 32;
    // r = rhat = b, x = 0
    double a0 = 0.0, a1 = 0.0;
    for (int64_t s = s0 + warp; s < s1; s += kWarps) {
        const int64_t i = s * 32 + lane;
        if (i >= k.n) continue;
        const double bi = __ldg(&k.b[i]);
        k.r[i] = bi;
        k.rhat[i] = bi;
        k.x[i] = 0.0;
        a0 += bi * bi;
    }
    coop_block_partials(a0, a0, k, red);
    bool ok = coop_grid_barrier(k, &s_ok);
    double rho, bb;
    coop_grid_sums(k, fin, rho, bb);
    double rho_prev = 1.0, alpha = 1.0, omega = 1.0;
    int status = (ok && bb > 0.0) ? 0 : (ok ? 1 : 2);
    int it = 0;
    const double* po = k.p0;
    const double* vo = k.v0;
    double* pn = k.p1;
    double* vn = k.v1;
    while (status == 0) {
        if (it >= k.maxit) {
            status = 2;
            break;
        }
        const double beta = it == 0 ? 0.0 : (rho / rho_prev) * (alpha / omega);
        const bool first = it == 0;
        // A: p = r + beta (p' - omega v'), v = W (p / dw)
        const double* r = k.r;
        auto pcol = [&](int32_t c) {
            const double rc = __ldcg(&r[c]);
            return first ? rc : rc + beta * (__ldcg(&po[c]) - omega * __ldcg(&vo[c]));
        };
        a0 = 0.0;
        for (int64_t s = s0 + warp; s < s1; s += kWarps) {
            const int64_t i = s * 32 + lane;
            if (i >= k.n) continue;
            const double pi = pcol((int32_t)i);
            const double vi = coop_w_row(k, s, lane, i, pi, pcol);
            pn[i] = pi;
            vn[i] = vi;
            a0 += __ldcg(&k.rhat[i]) * vi;
        }
        coop_block_partials(a0, 0.0, k, red);
        ok = coop_grid_barrier(k, &s_ok);
        double rv, unused;
        coop_grid_sums(k, fin, rv, unused);
        if (!ok || !(rv != 0.0) || !isfinite(rv)) {
            status = 2;
            break;
        }
        alpha = rho / rv;
        // B: s = r - alpha v, t = W (s / dw)
        auto scol = [&](int32_t c) { return __ldcg(&r[c]) - alpha * __ldcg(&vn[c]); };
        a0 = a1 = 0.0;
        for (int64_t s = s0 + warp; s < s1; s += kWarps) {
            const int64_t i = s * 32 + lane;
            if (i >= k.n) continue;
            const double si = scol((int32_t)i);
            const double ti = coop_w_row(k, s, lane, i, si, scol);
            k.s[i] = si;
            k.t[i] = ti;
            a0 += ti * si;
            a1 += ti * ti;
        }
        coop_block_partials(a0, a1, k, red);
        ok = coop_grid_barrier(k, &s_ok);
        double ts, tt;
        coop_grid_sums(k, fin, ts, tt);
        if (!ok) {
            status = 2;
            break;
        }
        omega = tt > 0.0 ? ts / tt : 0.0;
        // C: x += alpha p/dw + omega s/dw, r = s - omega t
        a0 = a1 = 0.0;
        for (int64_t s = s0 + warp; s < s1; s += kWarps) {
            const int64_t i = s * 32 + lane;
            if (i >= k.n) continue;
            const double dwi = __ldg(&k.dw[i]);
            const double si = __ldcg(&k.s[i]);
            k.x[i] = __ldcg(&k.x[i]) + alpha * (__ldcg(&pn[i]) / dwi) + omega * (si / dwi);
            const double ri = si - omega * __ldcg(&k.t[i]);
            k.r[i] = ri;
            a0 += __ldcg(&k.rhat[i]) * ri;
            a1 += ri * ri;
        }
        coop_block_partials(a0, a1, k, red);
        ok = coop_grid_barrier(k, &s_ok);
        double rho_new, rr;
        coop_grid_sums(k, fin, rho_new, rr);
        ++it;
        rho_prev = rho;
        rho = rho_new;
        if (!ok || !isfinite(rr))
            status = 2;
        else if (rr <= k.tol2 * bb)
            status = 1;
        else if (!(omega != 0.0) || !(rho != 0.0))
            status = 2;
        // the next iteration reads this one's p and v
        const double* tp = po;
        po = pn;
        pn = const_cast<double*>(tp);
        const double* tv = vo;
        vo = vn;
        vn = const_cast<double*>(tv);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        k.res->status = status;
        k.res->it = it;
    }
}

// Hermite interpolation of a saved value inside a step
__global__ void hermite_kernel(double* out, const double* u0, const double* f0, const double* u1, const double* f1,
                               double h, double th, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double t2 = th * th, t3 = t2 * th;
    const double h00 = 2 * t3 - 3 * t2 + 1, h10 = t3 - 2 * t2 + th, h01 = -2 * t3 + 3 * t2, h11 = t3 - t2;
    out[i] = h00 * u0[i] + h10 * h * f0[i] + h01 * u1[i] + h11 * h * f1[i];
}

struct Reducer {
    DBuf part;
    std::vector<double> host;
    Reducer() {
        part.alloc(sizeof(double) * 2 * kParts);
        host.resize(2 * kParts);
    }
    void fetch(int count, cudaStream_t s) {
        FVM_CUDA(cudaMemcpyAsync(host.data(), part.p, sizeof(double) * count, cudaMemcpyDeviceToHost, s));
        FVM_CUDA(cudaStreamSynchronize(s));
    }
    void dot2(const double* a0, const double* b0, const double* a1, const double* b1, int64_t n, double& r0,
              double& r1, cudaStream_t s) {
        dot2_kernel<<<kParts, kThreads, 0, s>>>(a0, b0, a1, b1, n, part.as<double>());
        fetch(2 * kParts, s);
        r0 = r1 = 0.0;
        for (int b = 0; b < kParts; ++b) {
            r0 += host[2 * b];
            r1 += host[2 * b + 1];
        }
    }
    double dot(const double* a, const double* b, int64_t n, cudaStream_t s) {
        double r0, r1;
        dot2(a, b, nullptr, nullptr, n, r0, r1, s);
        return r0;
    }
    // max|f| and max|f + u| (NaN propagates as a failed test: fmax drops it, so check finiteness)
    void maxabs2(const double* f, const double* u, int64_t n, double& m0, double& m1, cudaStream_t s) {
        maxabs2_kernel<<<kParts, kThreads, 0, s>>>(f, u, n, part.as<double>());
        fetch(2 * kParts, s);
        m0 = m1 = 0.0;
        for (int b = 0; b < kParts; ++b) {
            m0 = std::max(m0, host[2 * b]);
            m1 = std::max(m1, host[2 * b + 1]);
        }
    }
    // RMS of x / (abstol + reltol max(|a|, |b|))
    double wrms(const double* x, const double* a, const double* b, double abstol, double reltol, int64_t n,
                cudaStream_t s) {
        wnorm_kernel<<<kParts, kThreads, 0, s>>>(x, a, b, abstol, reltol, n, part.as<double>());
        fetch(kParts, s);
        double r = 0.0;
        for (int k = 0; k < kParts; ++k) r += host[k];
        return std::sqrt(r / (double)std::max<int64_t>(1, n));
    }
};

}  // namespace

// J(u) v in the internal numbering (the linear path: A v + 2 q u v; otherwise the derivative of
// the per-triangle kernel)
void problem_jvp_internal(fvm_problem* p, const double* u, const double* v, double* jv, cudaStream_t s) {
    fvm_mesh* m = p->mesh;
    if (p->conditions_only) fail(FVM_ERR_INVALID_ARGUMENT, "this problem carries a template's conditions only");
    if (p->linear) {
        if (p->precision == FVM_FP32) {
            launch_to_f32(v, p->d_u32.as<float>(), m->np, s);
            launch_sell_apply32(m->pat, p->d_val32.as<float>(), p->d_u32.as<float>(), v, jv,
                                p->d_rowscale.as<double>(), nullptr, nullptr, s);
        } else {
            launch_sell_apply64(m->pat, p->d_val64.as<double>(), v, jv, nullptr, nullptr, nullptr, s);
        }
        if (p->has_q) launch_quad_jvp(p->d_q.as<double>(), u, v, nullptr, jv, m->np, s);
    } else {
        p->build_triangle_path();
        launch_triangle_jvp(m, p, u, v, jv, false, s);
    }
}

// diag J(u) in the internal numbering
void problem_jacobian_diagonal_internal(fvm_problem* p, const double* u, double* dj, cudaStream_t s) {
    fvm_mesh* m = p->mesh;
    if (p->conditions_only) fail(FVM_ERR_INVALID_ARGUMENT, "this problem carries a template's conditions only");
    if (p->linear) {
        const SellPattern& pat = m->pat;
        if (p->precision == FVM_FP32)
            sell_diag_kernel<float><<<blocks_for(m->np), kThreads, 0, s>>>(
                pat.d_slice_ptr.as<int64_t>(), pat.d_width.as<int32_t>(), pat.d_col.as<int32_t>(),
                p->d_val32.as<float>(), p->d_rowscale.as<double>(), m->np, dj);
        else
            sell_diag_kernel<double><<<blocks_for(m->np), kThreads, 0, s>>>(
                pat.d_slice_ptr.as<int64_t>(), pat.d_width.as<int32_t>(), pat.d_col.as<int32_t>(),
                p->d_val64.as<double>(), nullptr, m->np, dj);
        if (p->has_q) launch_quad_jvp(p->d_q.as<double>(), u, nullptr, dj, dj, m->np, s);
    } else {
        p->build_triangle_path();
        launch_triangle_jvp(m, p, u, nullptr, dj, true, s);
    }
}

namespace {

constexpr double kSqrt2 = 1.4142135623730951;
constexpr double kGamma = 2.0 - kSqrt2;
constexpr double kD = kGamma / 2.0;
constexpr double kW = kSqrt2 / 4.0;

struct Trbdf2 {
    ImplicitRhs* R;
    int64_t n;
    cudaStream_t s;
    double abstol, reltol;
    Reducer red;
    DBuf buf;
    double *u, *un, *fn, *f1, *zn, *zg, *z1, *base, *tmp, *dj, *dw, *est;
    double *r, *rhat, *pv, *ph, *v, *sv, *sh, *t, *x;  // BiCGStab
    int64_t nrhs = 0, newton = 0, krylov = 0, jvps = 0, newton_fail = 0;
    double wd = 0;  // d h of the current W
    const double* wu = nullptr;  // J's point
    const double* wmask = nullptr;  // null: W = I - wd J; else W = diag(wmask) - wd J

    Trbdf2(ImplicitRhs* R_, int64_t n_, cudaStream_t s_, double at, double rt)
        : R(R_), n(n_), s(s_), abstol(at), reltol(rt) {
        constexpr int nv = 21;
        buf.alloc(sizeof(double) * n * nv);
        double* q = buf.as<double>();
        double** slots[nv] = {&u, &un, &fn, &f1, &zn, &zg, &z1, &base, &tmp, &dj, &dw, &est,
                              &r, &rhat, &pv, &ph, &v, &sv, &sh, &t, &x};
        for (int k = 0; k < nv; ++k) *slots[k] = q + (int64_t)k * n;
        kdev.alloc(sizeof(KDev));
        if (R->op_pat && R->op_val && n > 0 && n <= kCoopMaxRows) {
            int per_sm = 0, sms = 0, dev = 0;
            FVM_CUDA(cudaGetDevice(&dev));
            FVM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            FVM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, coop_bicgstab_kernel, kCoopThreads, 0));
            // about one slice per warp, within what can be co-resident
            const int64_t want = (R->op_pat->nslices + kCoopThreads / 32 - 1) / (kCoopThreads / 32);
            coop_grid = (int)std::min<int64_t>({want, (int64_t)per_sm * sms, (int64_t)kCoopMaxCtas});
            if (coop_grid >= 1) {
                coop_buf.alloc(sizeof(double) * 2 * kCoopMaxCtas + 64);
                use_coop = true;
            }
        }
    }
    // the cooperative solve (one launch per Krylov solve) for small operators: measured faster up
    // to 15,625 unknowns (2-2.3x per TR-BDF2 solve), slower at 40,401 (its barriers and chained
    // gathers then cost more than the launches they save)
    static constexpr int64_t kCoopMaxRows = 1 << 15;
    bool use_coop = false;
    int coop_grid = 0;
    DBuf coop_buf;  // partials [2][kCoopMaxCtas], then the result and the barrier words
    bool solve_coop(const double* b, double* xo, double rtol, int maxit) {
        double* part = coop_buf.as<double>();
        CoopResult* res = reinterpret_cast<CoopResult*>(part + 2 * kCoopMaxCtas);
        unsigned* bar = reinterpret_cast<unsigned*>(res + 1);
        FVM_CUDA(cudaMemsetAsync(res, 0, sizeof(CoopResult) + 2 * sizeof(unsigned), s));
        const SellPattern& pat = *R->op_pat;
        CoopKrylov k{pat.d_slice_ptr.as<int64_t>(), pat.d_width.as<int32_t>(), pat.d_col.as<int32_t>(), R->op_val,
                     R->op_q, wu, wmask, wd, dw, b, xo, r, rhat, pv, ph, v, sh, sv, t, part, bar, bar + 1,
                     device_error_word(), res, n, pat.nslices, rtol * rtol, maxit, kWaitLimitNs};
        void* args[] = {&k};
        FVM_CUDA(cudaLaunchCooperativeKernel((const void*)coop_bicgstab_kernel, dim3((unsigned)coop_grid),
                                             dim3(kCoopThreads), args, 0, s));
        CoopResult h{};
        FVM_CUDA(cudaMemcpyAsync(&h, res, sizeof h, cudaMemcpyDeviceToHost, s));
        FVM_CUDA(cudaStreamSynchronize(s));
        if (unsigned e = take_device_error())
            fail(FVM_ERR_CUDA, "the cooperative Krylov solve timed out in a bounded wait (device error bits " +
                                   std::to_string(e) + ")");
        krylov += h.it;
        jvps += 2 * (int64_t)h.it;
        return h.status == 1;
    }
    void rhs(const double* y, double* out, double tt) {
        R->f(y, out, tt, s);
        ++nrhs;
    }
    void wmul(const double* xin, double* out) {  // out = xin - d h J(wu) xin (two per BiCGStab iteration)
        R->jvp(wu, xin, out, s);
        if (wmask)
            wmask_kernel<<<blocks_for(n), kThreads, 0, s>>>(out, xin, wmask, wd, n);
        else
            lin(out, lin2(xin, 1.0, out, -wd), n, s);
    }
    // W at u_n with d h: its diagonal for the preconditioner; the captured iteration chunk of
    // the previous W is dropped
    void set_w(const double* at, double dh) {
        drop_chunk();
        wu = at;
        wd = dh;
        R->diag(at, dj, s);
        if (wmask)
            wdiag_mask_kernel<<<blocks_for(n), kThreads, 0, s>>>(dj, wmask, dh, dw, n);
        else
            wdiag_kernel<<<blocks_for(n), kThreads, 0, s>>>(dj, dh, dw, n);
    }
    // x = W^-1 b by right-preconditioned BiCGStab to ||b - W x|| <= rtol ||b||; x starts at 0.
    // The iterations run without host round trips; the host reads the scalars every kCheck.
    static constexpr int kCheck = 8;
    bool solve(const double* b, double* xo, double rtol, int maxit) {
        if (use_coop) return solve_coop(b, xo, rtol, maxit);
        FVM_CUDA(cudaMemsetAsync(xo, 0, sizeof(double) * n, s));
        FVM_CUDA(cudaMemcpyAsync(r, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        FVM_CUDA(cudaMemcpyAsync(rhat, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        FVM_CUDA(cudaMemsetAsync(pv, 0, sizeof(double) * n, s));
        FVM_CUDA(cudaMemsetAsync(v, 0, sizeof(double) * n, s));
        KDev* kd = kdev.as<KDev>();
        double* part = red.part.as<double>();
        dot2_kernel<<<kParts, kThreads, 0, s>>>(rhat, r, b, b, n, part);
        kd_init_kernel<<<1, kFin, 0, s>>>(kd, part, rtol * rtol);
        if (xo != x) fail(FVM_ERR_INVALID_ARGUMENT, "the captured Krylov chunk writes the solver's x");
        if (!chunk) capture_chunk();
        for (int done = 0; done < maxit; done += kCheck) {
            FVM_CUDA(cudaGraphLaunch(chunk, s));
            KDev h{};
            FVM_CUDA(cudaMemcpyAsync(&h, kd, sizeof h, cudaMemcpyDeviceToHost, s));
            FVM_CUDA(cudaStreamSynchronize(s));
            krylov += h.it - (int64_t)done_its;
            jvps += 2 * (h.it - (int64_t)done_its);
            done_its = h.it;
            if (h.status == 1) {
                done_its = 0;
                return true;
            }
            if (h.status == 2) {
                done_its = 0;
                return false;
            }
        }
        done_its = 0;
        return false;
    }
    int64_t done_its = 0;
    DBuf kdev;
    // kCheck BiCGStab iterations on the current W, captured once per W and replayed
    cudaGraphExec_t chunk = nullptr;
    void iterations() {
        KDev* kd = kdev.as<KDev>();
        double* part = red.part.as<double>();
        const unsigned g = blocks_for(n);
        for (int j = 0; j < kCheck; ++j) {
            kd_p_kernel<<<g, kThreads, 0, s>>>(kd, r, pv, v, n);
            jacobi_kernel<<<g, kThreads, 0, s>>>(pv, dw, ph, n);
            wmul(ph, v);
            dot2_kernel<<<kParts, kThreads, 0, s>>>(rhat, v, nullptr, nullptr, n, part);
            kd_alpha_kernel<<<1, kFin, 0, s>>>(kd, part);
            kd_s_kernel<<<g, kThreads, 0, s>>>(kd, r, v, sv, n);
            jacobi_kernel<<<g, kThreads, 0, s>>>(sv, dw, sh, n);
            wmul(sh, t);
            dot2_kernel<<<kParts, kThreads, 0, s>>>(t, sv, t, t, n, part);
            kd_omega_kernel<<<1, kFin, 0, s>>>(kd, part);
            kd_xr_kernel<<<g, kThreads, 0, s>>>(kd, x, ph, sh, sv, t, r, n);
            dot2_kernel<<<kParts, kThreads, 0, s>>>(rhat, r, r, r, n, part);
            kd_rho_kernel<<<1, kFin, 0, s>>>(kd, part);
        }
    }
    void capture_chunk() {
        cudaGraph_t graph = nullptr;
        FVM_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        iterations();
        FVM_CUDA(cudaStreamEndCapture(s, &graph));
        const cudaError_t e = cudaGraphInstantiate(&chunk, graph, 0);
        cudaGraphDestroy(graph);
        FVM_CUDA(e);
    }
    void drop_chunk() {
        if (chunk) cudaGraphExecDestroy(chunk);
        chunk = nullptr;
    }
    ~Trbdf2() { drop_chunk(); }
    // z = h f(base + d z) by simplified Newton from the predictor already in z; exact_linear: one
    // iteration solves an affine f to the Krylov tolerance
    bool stage(double* z, double tt, double h, bool exact_linear) {
        double prev = 0.0;
        for (int it = 0; it < 10; ++it) {
            ++newton;
            lin(tmp, lin2(base, 1.0, z, kD), n, s);  // the stage's state
            rhs(tmp, r, tt);
            lin(r, lin2(r, h, z, -1.0), n, s);  // residual h f - z
            FVM_CUDA(cudaMemcpyAsync(est, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
            if (!solve(est, x, 1e-10, 1000)) return false;
            lin(z, lin2(z, 1.0, x, 1.0), n, s);
            if (exact_linear) return true;
            const double dn = red.wrms(x, u, nullptr, abstol, reltol, n, s);
            if (!std::isfinite(dn)) return false;
            if (dn <= 1e-10) return true;
            if (it > 0) {
                const double theta = dn / prev;
                if (theta >= 1.0) return false;
                if (theta / (1.0 - theta) * dn <= 1e-2) return true;
            }
            prev = dn;
        }
        return false;
    }
};

// a stream that can be captured (the legacy default stream cannot): the caller's, or one of ours
// ordered after the default stream's earlier work
struct CapturableStream {
    cudaStream_t s = nullptr, own = nullptr;
    explicit CapturableStream(void* stream) : s((cudaStream_t)stream) {
        if (!s || s == cudaStreamLegacy || s == cudaStreamPerThread) {
            FVM_CUDA(cudaDeviceSynchronize());
            FVM_CUDA(cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking));
            s = own;
        }
    }
    CapturableStream(const CapturableStream&) = delete;
    CapturableStream& operator=(const CapturableStream&) = delete;
    ~CapturableStream() {
        if (own) {
            cudaStreamSynchronize(own);
            cudaStreamDestroy(own);
        }
    }
};

}  // namespace
}  // namespace fvm

using namespace fvm;

// TR-BDF2 on R over n unknowns: u0 and out are host arrays in the caller's numbering, perm /
// iperm the device permutations between it and the internal one.
int fvm::trbdf2_run(ImplicitRhs& R, const int32_t* perm, const int32_t* iperm, int64_t n, const double* u0,
                    const fvm_ode_options* o, double* out, fvm_ode_stats* st, fvm_implicit_stats* ist, void* stream,
                    SteadyStop* stop) {
    {
        if (!u0 || !o || !out) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        if (!(o->tf > o->t0)) fail(FVM_ERR_INVALID_ARGUMENT, "final time must exceed the initial time");
        if (!stop && !std::isfinite(o->tf)) fail(FVM_ERR_INVALID_ARGUMENT, "the final time must be finite");
        if (!o->adaptive && !(o->dt > 0)) fail(FVM_ERR_INVALID_ARGUMENT, "dt must be positive for fixed steps");
        CapturableStream cs(stream);
        cudaStream_t s = cs.s;
        std::vector<double> saveat;
        if (stop)
            saveat.push_back(INFINITY);  // one output, the u that passes the test (saved at the end)
        else if (o->saveat && o->nsave > 0)
            saveat.assign(o->saveat, o->saveat + o->nsave);
        else
            saveat.push_back(o->tf);
        for (size_t i = 0; i < saveat.size() && !stop; ++i) {
            if (saveat[i] < o->t0 || saveat[i] > o->tf) fail(FVM_ERR_INVALID_ARGUMENT, "saveat times must lie in [t0, tf]");
            if (i && saveat[i] < saveat[i - 1]) fail(FVM_ERR_INVALID_ARGUMENT, "saveat must be sorted");
        }
        Trbdf2 M(&R, n, s, o->abstol, o->reltol);
        DBuf d_in, d_out;
        d_in.alloc(sizeof(double) * n);
        d_out.alloc(sizeof(double) * n * saveat.size());
        FVM_CUDA(cudaMemcpyAsync(d_in.p, u0, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        launch_permute_in(perm, d_in.as<double>(), M.u, n, s);
        double* outi = d_out.as<double>();
        size_t si = 0;
        auto save = [&](const double* src) {
            FVM_CUDA(cudaMemcpyAsync(outi + si * n, src, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
            ++si;
        };
        double t = o->t0;
        while (si < saveat.size() && saveat[si] == t) save(M.u);
        cudaEvent_t e0, e1;
        FVM_CUDA(cudaEventCreate(&e0));
        FVM_CUDA(cudaEventCreate(&e1));
        FVM_CUDA(cudaEventRecord(e0, s));
        M.rhs(M.u, M.fn, t);
        const double tspan = o->tf - o->t0;
        // affine f with an exact product: one Newton iteration solves each stage
        const bool exact_linear = R.affine;
        double h = o->dt;
        if (o->adaptive && !(h > 0)) {  // order-2 version of the Hairer-Wanner initial step
            const double d0 = M.red.wrms(M.u, M.u, nullptr, o->abstol, o->reltol, n, s);
            const double d1 = M.red.wrms(M.fn, M.u, nullptr, o->abstol, o->reltol, n, s);
            const double h0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * d0 / d1;
            h = std::min(h0, tspan);
        }
        const int64_t max_steps = o->max_steps > 0 ? o->max_steps : 100000000;
        int64_t nacc = 0, nrej = 0, step = 0;
        bool first_cb = true;
        while (t < o->tf) {
            if (step >= max_steps) {
                if (stop) break;  // not converged: the caller reports it
                fail(FVM_ERR_STEP_LIMIT, "TRBDF2 reached max_steps before tf");
            }
            const bool last = std::isfinite(o->tf) && t + h >= o->tf - 1e-12 * tspan;
            const double hh = last ? o->tf - t : h;
            ++step;
            // z_n = h f_n; W = I - d h J(u_n)
            lin(M.zn, lin2(M.fn, hh, nullptr, 0.0), n, s);
            M.set_w(M.u, kD * hh);
            // trapezoidal stage: base = u_n + d z_n, predictor z_g = z_n
            lin(M.base, lin2(M.u, 1.0, M.zn, kD), n, s);
            FVM_CUDA(cudaMemcpyAsync(M.zg, M.zn, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
            bool ok = M.stage(M.zg, t + kGamma * hh, hh, exact_linear);
            if (ok) {  // BDF2 stage: base = u_n + w z_n + w z_g, predictor z_1 = z_g
                Lin L{};
                L.x[0] = M.u;
                L.c[0] = 1.0;
                L.x[1] = M.zn;
                L.c[1] = kW;
                L.x[2] = M.zg;
                L.c[2] = kW;
                lin(M.base, L, n, s);
                FVM_CUDA(cudaMemcpyAsync(M.z1, M.zg, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
                ok = M.stage(M.z1, t + hh, hh, exact_linear);
            }
            if (!ok) {
                ++M.newton_fail;
                if (!o->adaptive) fail(FVM_ERR_STEP_LIMIT, "TRBDF2: the Newton iteration did not converge at the fixed dt");
                h = hh / 4;
                if (h < 1e-14 * std::max(1.0, std::fabs(t))) fail(FVM_ERR_STEP_LIMIT, "TRBDF2 step size underflow");
                continue;
            }
            lin(M.un, lin2(M.base, 1.0, M.z1, kD), n, s);  // u_{n+1}
            double err = 0.0;
            if (o->adaptive) {
                Lin L{};
                L.x[0] = M.zn;
                L.c[0] = (1.0 - kSqrt2) / 3.0;
                L.x[1] = M.zg;
                L.c[1] = 1.0 / 3.0;
                L.x[2] = M.z1;
                L.c[2] = (kSqrt2 - 2.0) / 3.0;
                lin(M.tmp, L, n, s);
                if (!M.solve(M.tmp, M.x, 1e-10, 1000)) fail(FVM_ERR_STEP_LIMIT, "TRBDF2: the error estimate's solve failed");
                err = M.red.wrms(M.x, M.u, M.un, o->abstol, o->reltol, n, s);
                if (!std::isfinite(err)) fail(FVM_ERR_STEP_LIMIT, "TRBDF2 error estimate is not finite");
                if (err > 1.0) {
                    ++nrej;
                    h = hh * std::min(10.0, std::max(0.2, 0.9 * std::pow(err, -1.0 / 3.0)));
                    if (h < 1e-14 * std::max(1.0, std::fabs(t))) fail(FVM_ERR_STEP_LIMIT, "TRBDF2 step size underflow");
                    continue;
                }
            }
            const double tn = last ? o->tf : t + hh;
            // f at u_{n+1} (before the Dirichlet update) for the interpolant
            M.rhs(M.un, M.f1, tn);
            while (si < saveat.size() && saveat[si] < tn) {
                const double th = (saveat[si] - t) / hh;
                hermite_kernel<<<blocks_for(n), kThreads, 0, s>>>(outi + si * n, M.u, M.fn, M.un, M.f1, hh, th, n);
                ++si;
            }
            std::swap(M.u, M.un);
            std::swap(M.fn, M.f1);
            t = tn;
            ++nacc;
            if (R.callback) {
                R.callback(M.u, t, s);
                if (first_cb || R.callback_varies) M.rhs(M.u, M.fn, t);
                first_cb = false;
            }
            while (si < saveat.size() && saveat[si] == t) save(M.u);
            if (stop) {  // f_n is f at the updated u
                double m0, m1;
                M.red.maxabs2(M.fn, M.u, n, m0, m1, s);
                stop->residual = m0;
                if (m0 <= stop->abstol || m0 <= stop->reltol * m1) {
                    stop->converged = true;
                    break;
                }
            }
            if (o->adaptive) {
                const double q = err > 0 ? 0.9 * std::pow(err, -1.0 / 3.0) : 10.0;
                h = std::min(tspan, hh * std::min(10.0, std::max(0.2, q)));
            }
            if (last) break;
        }
        while (si < saveat.size()) save(M.u);
        FVM_CUDA(cudaEventRecord(e1, s));
        FVM_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        FVM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        snapshots_to_host(iperm, outi, out, n, (int64_t)saveat.size(), s);
        FVM_CUDA(cudaStreamSynchronize(s));
        FVM_CUDA(cudaGetLastError());
        if (st) {
            st->naccept = nacc;
            st->nreject = nrej;
            st->nrhs = M.nrhs;
            st->t_final = t;
            st->elapsed_ms = ms;
            st->driver = FVM_DRIVER_HOST;
        }
        if (ist) {
            ist->newton_iters = M.newton;
            ist->krylov_iters = M.krylov;
            ist->jvps = M.jvps;
            ist->newton_failures = M.newton_fail;
        }
        return FVM_OK;
    }
}

// NewtonRaphson on f(u, t) = 0: (F - J(u)) du = f(u) by the Krylov solver of the stages, F the
// identity on the fixed rows (R.fixed), until the steady test passes
static void newton_run(ImplicitRhs& R, const int32_t* perm, const int32_t* iperm, int64_t n, const double* u0,
                       const fvm_steady_options* o, double* out, fvm_steady_stats* st, bool& converged,
                       void* stream) {
    CapturableStream cs(stream);
    cudaStream_t s = cs.s;
    if (!R.fixed) fail(FVM_ERR_INVALID_ARGUMENT, "Newton needs the fixed-row mask");
    Trbdf2 M(&R, n, s, 1.0, 0.0);
    M.wmask = R.fixed;
    DBuf d_in;
    d_in.alloc(sizeof(double) * n);
    FVM_CUDA(cudaMemcpyAsync(d_in.p, u0, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    launch_permute_in(perm, d_in.as<double>(), M.u, n, s);
    cudaEvent_t e0, e1;
    FVM_CUDA(cudaEventCreate(&e0));
    FVM_CUDA(cudaEventCreate(&e1));
    FVM_CUDA(cudaEventRecord(e0, s));
    if (R.callback) R.callback(M.u, o->t, s);
    const int64_t max_it = o->max_iters > 0 ? o->max_iters : 50;
    int64_t it = 0;
    double res = INFINITY;
    converged = false;
    for (;; ++it) {
        M.rhs(M.u, M.fn, o->t);
        double m1;
        M.red.maxabs2(M.fn, M.u, n, res, m1, s);
        if (!std::isfinite(res)) break;
        if (res <= o->abstol || res <= o->reltol * m1) {
            converged = true;
            break;
        }
        if (it >= max_it) break;
        ++M.newton;
        M.set_w(M.u, 1.0);  // W = F - J(u)
        FVM_CUDA(cudaMemcpyAsync(M.est, M.fn, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        if (!M.solve(M.est, M.x, 1e-10, 20000)) break;
        lin(M.u, lin2(M.u, 1.0, M.x, 1.0), n, s);
    }
    FVM_CUDA(cudaEventRecord(e1, s));
    FVM_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    FVM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    snapshots_to_host(iperm, M.u, out, n, 1, s);
    FVM_CUDA(cudaStreamSynchronize(s));
    FVM_CUDA(cudaGetLastError());
    if (st) {
        st->iterations = M.newton;
        st->krylov_iters = M.krylov;
        st->jvps = M.jvps;
        st->nrhs = M.nrhs;
        st->residual = res;
        st->t_final = o->t;
        st->elapsed_ms = ms;
    }
}

void fvm::steady_run(ImplicitRhs& R, const int32_t* perm, const int32_t* iperm, int64_t n, const double* u0,
                     const fvm_steady_options* o, double* out, fvm_steady_stats* st, void* stream) {
    if (!u0 || !o || !out) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!(o->abstol >= 0) || !(o->reltol >= 0)) fail(FVM_ERR_INVALID_ARGUMENT, "tolerances must be non-negative");
    if (st) *st = fvm_steady_stats{};
    bool converged = false;
    if (o->method == FVM_STEADY_NEWTON) {
        newton_run(R, perm, iperm, n, u0, o, out, st, converged, stream);
    } else if (o->method == FVM_STEADY_DYNAMIC) {
        if (!(o->tmax > o->t)) fail(FVM_ERR_INVALID_ARGUMENT, "tmax must exceed t");
        fvm_ode_options od{};
        od.t0 = o->t;
        od.tf = o->tmax;
        od.adaptive = 1;
        od.abstol = o->ode_abstol > 0 ? o->ode_abstol : 1e-6;
        od.reltol = o->ode_reltol > 0 ? o->ode_reltol : 1e-3;
        od.max_steps = o->max_iters > 0 ? o->max_iters : 100000;
        SteadyStop stop;
        stop.abstol = o->abstol;
        stop.reltol = o->reltol;
        stop.residual = INFINITY;
        fvm_ode_stats os{};
        fvm_implicit_stats is{};
        trbdf2_run(R, perm, iperm, n, u0, &od, out, &os, &is, stream, &stop);
        converged = stop.converged;
        if (st) {
            st->iterations = os.naccept;
            st->krylov_iters = is.krylov_iters;
            st->jvps = is.jvps;
            st->nrhs = os.nrhs;
            st->residual = stop.residual;
            st->t_final = os.t_final;
            st->elapsed_ms = os.elapsed_ms;
        }
    } else {
        fail(FVM_ERR_INVALID_ARGUMENT, "unknown steady method");
    }
    if (!converged) fail(FVM_ERR_NOT_CONVERGED, "the steady-state test was not met");
}

extern "C" {

int fvm_jvp(fvm_problem* p, const double* u, const double* v, double* jv, double t, int32_t flags, void* stream) {
    return guard_call([&] {
        if (!p || !u || !v || !jv) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        (void)t;  // time factors enter constant terms only: J does not depend on t
        const int32_t loc = flags & 3;
        if (loc > FVM_PTR_DEVICE_INTERNAL) fail(FVM_ERR_INVALID_ARGUMENT, "bad pointer-location flag");
        cudaStream_t s = (cudaStream_t)stream;
        fvm_mesh* m = p->mesh;
        const int64_t n = m->np;
        if (loc == FVM_PTR_DEVICE_INTERNAL) {
            problem_jvp_internal(p, u, v, jv, s);
            FVM_CUDA(cudaGetLastError());
            return FVM_OK;
        }
        DBuf w;
        w.alloc(sizeof(double) * 4 * n);
        double *ui = w.as<double>(), *vi = ui + n, *ji = ui + 2 * n, *st = ui + 3 * n;
        auto in = [&](const double* src, double* dst) {
            const double* from = src;
            if (loc == FVM_PTR_HOST) {
                FVM_CUDA(cudaMemcpyAsync(st, src, sizeof(double) * n, cudaMemcpyHostToDevice, s));
                from = st;
            }
            launch_permute_in(m->d_perm.as<int32_t>(), from, dst, n, s);
        };
        in(u, ui);
        in(v, vi);
        problem_jvp_internal(p, ui, vi, ji, s);
        double* dst = loc == FVM_PTR_HOST ? st : jv;
        launch_permute_out(m->d_perm.as<int32_t>(), ji, dst, n, s);
        if (loc == FVM_PTR_HOST) FVM_CUDA(cudaMemcpyAsync(jv, st, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
        FVM_CUDA(cudaStreamSynchronize(s));
        FVM_CUDA(cudaGetLastError());
        return FVM_OK;
    });
}

int fvm_jacobian_diagonal(fvm_problem* p, const double* u, double* diag, double t, int32_t flags, void* stream) {
    return guard_call([&] {
        if (!p || !u || !diag) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        (void)t;
        const int32_t loc = flags & 3;
        if (loc > FVM_PTR_DEVICE_INTERNAL) fail(FVM_ERR_INVALID_ARGUMENT, "bad pointer-location flag");
        cudaStream_t s = (cudaStream_t)stream;
        fvm_mesh* m = p->mesh;
        const int64_t n = m->np;
        if (loc == FVM_PTR_DEVICE_INTERNAL) {
            problem_jacobian_diagonal_internal(p, u, diag, s);
            FVM_CUDA(cudaGetLastError());
            return FVM_OK;
        }
        DBuf w;
        w.alloc(sizeof(double) * 3 * n);
        double *ui = w.as<double>(), *di = ui + n, *st = ui + 2 * n;
        const double* from = u;
        if (loc == FVM_PTR_HOST) {
            FVM_CUDA(cudaMemcpyAsync(st, u, sizeof(double) * n, cudaMemcpyHostToDevice, s));
            from = st;
        }
        launch_permute_in(m->d_perm.as<int32_t>(), from, ui, n, s);
        problem_jacobian_diagonal_internal(p, ui, di, s);
        double* dst = loc == FVM_PTR_HOST ? st : diag;
        launch_permute_out(m->d_perm.as<int32_t>(), di, dst, n, s);
        if (loc == FVM_PTR_HOST) FVM_CUDA(cudaMemcpyAsync(diag, st, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
        FVM_CUDA(cudaStreamSynchronize(s));
        FVM_CUDA(cudaGetLastError());
        return FVM_OK;
    });
}

int fvm_trbdf2_solve(fvm_problem* p, const double* u0, const fvm_ode_options* o, double* out, fvm_ode_stats* st,
                     fvm_implicit_stats* ist, void* stream) {
    return guard_call([&] {
        if (!p) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        if (p->conditions_only) fail(FVM_ERR_INVALID_ARGUMENT, "this problem carries a template's conditions only");
        ImplicitRhs R;
        R.f = [p](const double* y, double* du, double t, cudaStream_t s) {
            problem_rhs_internal(p, y, du, false, s, false, t);
        };
        R.jvp = [p](const double* u, const double* v, double* jv, cudaStream_t s) { problem_jvp_internal(p, u, v, jv, s); };
        R.diag = [p](const double* u, double* d, cudaStream_t s) { problem_jacobian_diagonal_internal(p, u, d, s); };
        if (p->ndir > 0)
            R.callback = [p](double* u, double t, cudaStream_t s) { problem_dirichlet_internal(p, u, t, s); };
        R.callback_varies = p->tdir_varies;
        R.affine = p->linear && !p->has_q && p->precision != FVM_FP32;
        fvm_mesh* m = p->mesh;
        if (p->linear && p->precision == FVM_FP64) {  // J v = A v + 2 q u v, the assembled operator
            R.op_pat = &m->pat;
            R.op_val = p->d_val64.as<double>();
            R.op_q = p->has_q ? p->d_q.as<double>() : nullptr;
        }
        return trbdf2_run(R, m->d_perm.as<int32_t>(), m->d_iperm.as<int32_t>(), m->np, u0, o, out, st, ist, stream);
    });
}

int fvm_template_trbdf2_solve(fvm_template* T, const double* u0, const fvm_ode_options* o, double* out,
                              fvm_ode_stats* st, fvm_implicit_stats* ist, void* stream) {
    return guard_call([&] {
        if (!T) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        if (T->kind != FVM_TEMPLATE_DIFFUSION && T->kind != FVM_TEMPLATE_LINEAR_REACTION_DIFFUSION)
            fail(FVM_ERR_INVALID_ARGUMENT, "only time-dependent templates can be stepped");
        fvm_mesh* m = T->prob->mesh;
        // du/dt = A u + b: J = A, the template's operator itself (its rows of Dirichlet and missing
        // vertices are zero, so those values stay as given)
        ImplicitRhs R;
        R.f = [T, m](const double* y, double* du, double, cudaStream_t s) {
            launch_sell_apply64(m->pat, T->d_val64.as<double>(), y, du, nullptr, T->d_b.as<double>(), nullptr, s);
        };
        R.jvp = [T, m](const double*, const double* v, double* jv, cudaStream_t s) {
            launch_sell_apply64(m->pat, T->d_val64.as<double>(), v, jv, nullptr, nullptr, nullptr, s);
        };
        R.diag = [T, m](const double*, double* d, cudaStream_t s) {
            const SellPattern& pat = m->pat;
            sell_diag_kernel<double><<<blocks_for(m->np), kThreads, 0, s>>>(
                pat.d_slice_ptr.as<int64_t>(), pat.d_width.as<int32_t>(), pat.d_col.as<int32_t>(),
                T->d_val64.as<double>(), nullptr, m->np, d);
        };
        R.affine = true;
        R.op_pat = &m->pat;
        R.op_val = T->d_val64.as<double>();
        return trbdf2_run(R, m->d_perm.as<int32_t>(), m->d_iperm.as<int32_t>(), m->np, u0, o, out, st, ist, stream);
    });
}

int fvm_steady_solve(fvm_problem* p, const double* u0, const fvm_steady_options* o, double* out,
                     fvm_steady_stats* st, void* stream) {
    return guard_call([&] {
        if (!p) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        if (p->conditions_only) fail(FVM_ERR_INVALID_ARGUMENT, "this problem carries a template's conditions only");
        fvm_mesh* m = p->mesh;
        // the rows the problem fixes: Dirichlet points and points in no triangle (du = 0 there)
        std::vector<double> fixed((size_t)m->np, 0.0);
        for (int64_t v = 0; v < m->np; ++v)
            if (p->code[v] == FVM_VERTEX_DIRICHLET || p->code[v] == FVM_VERTEX_NOT_A_VERTEX) fixed[m->iperm[v]] = 1.0;
        DBuf d_fixed;
        d_fixed.upload(fixed);
        ImplicitRhs R;
        R.f = [p](const double* y, double* du, double t, cudaStream_t s) {
            problem_rhs_internal(p, y, du, false, s, false, t);
        };
        R.jvp = [p](const double* u, const double* v, double* jv, cudaStream_t s) { problem_jvp_internal(p, u, v, jv, s); };
        R.diag = [p](const double* u, double* d, cudaStream_t s) { problem_jacobian_diagonal_internal(p, u, d, s); };
        if (p->ndir > 0)
            R.callback = [p](double* u, double t, cudaStream_t s) { problem_dirichlet_internal(p, u, t, s); };
        R.callback_varies = p->tdir_varies;
        R.affine = p->linear && !p->has_q && p->precision != FVM_FP32;
        R.fixed = d_fixed.as<double>();
        if (p->linear && p->precision == FVM_FP64) {
            R.op_pat = &m->pat;
            R.op_val = p->d_val64.as<double>();
            R.op_q = p->has_q ? p->d_q.as<double>() : nullptr;
        }
        steady_run(R, m->d_perm.as<int32_t>(), m->d_iperm.as<int32_t>(), m->np, u0, o, out, st, stream);
        return FVM_OK;
    });
}

}  // extern "C"
