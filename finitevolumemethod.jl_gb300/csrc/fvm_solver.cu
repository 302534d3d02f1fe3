// Steady solve of a Poisson / mean-exit-time template (LinearProblem(A, b) + solve,
// poissons_equation.jl:81, mean_exit_time.jl:76) on the GPU alone.
//
// Rows fixed by a Dirichlet condition or a missing vertex are identity rows of A; the
// remaining (free) rows are scaled by -V_i, which turns -div(D grad) into a symmetric
// positive definite operator B when D is constant on each triangle:
//     B z = rhs,  B_ij = -V_i A_ij (i, j free),  rhs_i = -V_i (b_i - sum_{j fixed} A_ij b_j),
//     x = z + x_fixed,  and  (b - A x)_i = -(rhs - B z)_i / V_i  on free rows.
// CG runs when B is symmetric, BiCGStab otherwise.  Mixed precision: FP32 values, vectors and
// inner products, FP32 accumulation, with FP64 reliable updates of the residual and the
// solution (x in FP64, true residual computed with the FP64 operator) every time the FP32
// recurrence residual has dropped by `inner_reduction`.  The stopping test is always the
// FP64 residual ||b - A x|| / ||b|| of the reference operator.
#include "fvm_internal.h"
#include "fvm_sell.cuh"
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <type_traits>
#include <utility>

namespace fvm {

constexpr int kRedBlock = 256;

struct KState {               // device-resident Krylov scalars
    double dot[8];            // reduction results
    double alpha, beta, omega, rho, rz, tol2, rn2;
    double div2;              // a cycle whose recurrence residual^2 exceeds this has diverged
    int done;
    int breakdown;
    int skip3;                // CG: the update step of this iteration did not run
    unsigned counter;
};

// last-block-done reduction: every block writes its partials; the last block to finish sums
// them in block order (deterministic) and runs `fin` on thread 0.
template <int NV>
__device__ void block_reduce_publish(double (&v)[NV], double* part, KState* st, int nblocks, bool& is_last) {
    __shared__ double red[NV][kRedBlock / 32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double x = v[q];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) red[q][wid] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double s = 0;
            for (int w = 0; w < kRedBlock / 32; ++w) s += red[q][w];
            part[q * nblocks + blockIdx.x] = s;
        }
        __threadfence();
        unsigned prev = atomicAdd(&st->counter, 1u);
        last = prev == (unsigned)nblocks - 1;
    }
    __syncthreads();
    is_last = last;
    if (!last) return;
    __threadfence();
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double s = 0;
        for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += __ldcg(&part[q * nblocks + b]);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) red[q][wid] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double s = 0;
            for (int w = 0; w < kRedBlock / 32; ++w) s += red[q][w];
            v[q] = s;
        }
        st->counter = 0;
    }
}

// ---- sliced-ELL SpMV with a fused inner product: y = B x, dot(w, y) --------------------
// x gathered and accumulated in T.  Each block covers 8 slices (256 rows).  Slices of at
// most 8 slots (every triangulation here) take the fully unrolled path; the branch is
// uniform across the warp.
template <class V, class T>
__device__ __forceinline__ T sell_row(const int64_t* slice_ptr, const int32_t* width, const int32_t* col, const V* val,
                                      const T* x, int64_t s, int lane) {
    if (__ldg(&width[s]) <= 8) return sell_row_product<V, T, T, false, 8>(slice_ptr, width, col, val, x, T(0), s, lane);
    return sell_row_product<V, T, T, false, 0>(slice_ptr, width, col, val, x, T(0), s, lane);
}

struct SpmvArgs {
    const int64_t* slice_ptr;
    const int32_t* width;
    const int32_t* col;
    int64_t n, nslices;
};

// (B x)_r of the lane's row.  rowsum == nullptr: explicit values.  Otherwise the difference
// form sum_j K_rj (x_j - x_r) + rowsum_r x_r, K with a zero diagonal: the FP32 operator.  On a
// smooth x the explicit FP32 sum cancels to eps32 |B||x| ~ eps32 / h^2 relative (interior rows
// of a diffusion operator sum to zero); the differences cut that to ~ eps32 / h.
template <class V, class T>
__device__ __forceinline__ T spmv_row(const SpmvArgs& A, const V* val, const T* rowsum, const T* x, int64_t s,
                                      int lane) {
    if (!rowsum) return sell_row<V, T>(A.slice_ptr, A.width, A.col, val, x, s, lane);
    const int64_t r = s * kSlice + lane;
    const int64_t rc = r < A.n ? r : A.n - 1;
    const T xr = x[rc];
    const T acc = __ldg(&A.width[s]) <= 8
                      ? sell_row_product<V, T, T, true, 8>(A.slice_ptr, A.width, A.col, val, x, xr, s, lane)
                      : sell_row_product<V, T, T, true, 0>(A.slice_ptr, A.width, A.col, val, x, xr, s, lane);
    return acc + rowsum[rc] * xr;
}

// The sparse-product kernels below are latency-bound one-warp-per-slice gathers: they are
// compiled for eight 256-thread blocks per SM (32 registers a thread, a few spilled to L1),
// full occupancy measured 17 % faster per Chebyshev BiCGStab iteration than four blocks of
// 60-register threads.

// CG step 1: Ap = B p; pAp; alpha = rz / pAp
template <class V, class T>
__global__ void __launch_bounds__(kRedBlock, 8) cg_spmv_kernel(SpmvArgs A, const V* val, const T* rowsum, const T* p, T* Ap,
                                                            double* part,
                                                            KState* st) {
    if (st->done) return;
    int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    double v[1] = {0.0};
    if (s < A.nslices) {
        T y = spmv_row<V, T>(A, val, rowsum, p, s, lane);
        int64_t r = s * kSlice + lane;
        if (r < A.n) {
            Ap[r] = y;
            v[0] = (double)(y * p[r]);
        }
    }
    bool last;
    block_reduce_publish<1>(v, part, st, gridDim.x, last);
    if (last && threadIdx.x == 0) {
        st->dot[0] = v[0];
        if (!(v[0] > 0) || !isfinite(v[0])) {
            st->done = 1;
            st->breakdown = 1;
            st->alpha = 0;
        } else {
            st->alpha = st->rz / v[0];
        }
    }
}

// CG step 2: x += alpha p; r -= alpha Ap; rn2 = sum (r invV)^2; with the Jacobi
// preconditioner also rz = r . (invD r) and beta (a polynomial preconditioner computes them
// after its own pass, cg_rz_kernel)
template <class T, bool JACOBI>
__global__ void __launch_bounds__(kRedBlock) cg_update_kernel(T* x, T* r, const T* p, const T* Ap, const T* invD,
                                                              const T* invV, int64_t n, double* part, KState* st) {
    if (st->done) {
        if (blockIdx.x == 0 && threadIdx.x == 0) st->skip3 = 1;
        return;
    }
    T alpha = (T)st->alpha;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double v[2] = {0.0, 0.0};
    if (i < n) {
        T xi = x[i] + alpha * p[i];
        T ri = r[i] - alpha * Ap[i];
        x[i] = xi;
        r[i] = ri;
        T rr = ri * ri;
        v[0] = (double)(rr * invD[i]);
        T w = ri * invV[i];
        v[1] = (double)(w * w);
    }
    bool last;
    block_reduce_publish<2>(v, part, st, gridDim.x, last);
    if (last && threadIdx.x == 0) {
        if (JACOBI) {
            double rz_old = st->rz;
            st->rz = v[0];
            st->beta = rz_old > 0 ? v[0] / rz_old : 0.0;
        }
        st->rn2 = v[1];
        st->skip3 = 0;
        if (v[1] <= st->tol2 || !isfinite(v[1])) st->done = 1;
        if (v[1] > st->div2) st->done = st->breakdown = 1;
    }
}

// CG step 3: p = invD r + beta p (runs whenever step 2 of the same iteration ran)
template <class T>
__global__ void cg_pupdate_kernel(T* p, const T* r, const T* invD, int64_t n, const KState* st) {
    if (st->skip3) return;
    T beta = (T)st->beta;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = invD[i] * r[i] + beta * p[i];
}

// ---- Chebyshev polynomial preconditioner -------------------------------------------------
// z = p(D^-1 B) D^-1 r: `degree` steps of the Chebyshev iteration for D^-1 B y = D^-1 r from
// y = 0 on an interval [lmin, lmax] that holds the spectrum of D^-1 B (Saad, Iterative Methods
// for Sparse Linear Systems, 2nd ed., Algorithm 12.1): with theta = (lmax + lmin) / 2,
// delta = (lmax - lmin) / 2, sigma = theta / delta,
//     w_0 = D^-1 r, d_0 = w_0 / theta, y_1 = d_0, rho_0 = 1 / sigma,
//     w_j = w_{j-1} - D^-1 B d_{j-1}, rho_j = 1 / (2 sigma - rho_{j-1}),
//     d_j = rho_j rho_{j-1} d_{j-1} + (2 rho_j / delta) w_j, y_{j+1} = y_j + d_j.
// A fixed polynomial in the Jacobi-scaled operator: linear, and symmetric positive definite
// when B is (the polynomial is positive on (0, lmax]), so CG and BiCGStab take it unchanged.
constexpr int kChebMax = 16;
struct ChebPlan {
    int degree = 0;                       // SpMVs per application: degree - 1
    double inv_theta = 0;
    double c1[kChebMax] = {}, c2[kChebMax] = {};
};

// lmax from Gershgorin on D^-1 B, lmin = lmax / 30 (the low end of the spectrum is left to
// the Krylov method)
static ChebPlan cheb_plan(double gershgorin, int degree) {
    ChebPlan P;
    P.degree = std::max(1, std::min(degree, kChebMax));
    const double lmax = 1.05 * gershgorin, lmin = lmax / 30.0;
    const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin), sigma = theta / delta;
    P.inv_theta = 1.0 / theta;
    double rho_prev = 1.0 / sigma;
    for (int j = 1; j < P.degree; ++j) {
        const double rho = 1.0 / (2.0 * sigma - rho_prev);
        P.c1[j] = rho * rho_prev;
        P.c2[j] = 2.0 * rho / delta;
        rho_prev = rho;
    }
    return P;
}

// gate: 0 = skip once the solve is done (BiCGStab, true residual); 1 = skip when this CG
// iteration's update did not run (the last update before `done` still completes its p)
__device__ __forceinline__ bool gated(const KState* st, int gate) { return gate ? st->skip3 != 0 : st->done != 0; }

template <class T>
__global__ void cheb_init_kernel(const T* r, const T* invD, T* w, T* d, T* y, T inv_theta, int64_t n,
                                 const KState* st, int gate) {
    if (gated(st, gate)) return;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const T wi = invD[i] * r[i];
        w[i] = wi;
        const T di = wi * inv_theta;
        d[i] = di;
        y[i] = di;
    }
}

template <class V, class T>
__global__ void __launch_bounds__(kRedBlock, 8) cheb_step_kernel(SpmvArgs A, const V* val, const T* rowsum, const T* d_in,
                                                              const T* invD,
                                                              T* w, T* d_out, T* y, T c1, T c2, const KState* st,
                                                              int gate) {
    if (gated(st, gate)) return;
    int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (s >= A.nslices) return;
    const T t = spmv_row<V, T>(A, val, rowsum, d_in, s, lane);
    int64_t i = s * kSlice + lane;
    if (i < A.n) {
        const T wi = w[i] - invD[i] * t;
        w[i] = wi;
        const T di = c1 * d_in[i] + c2 * wi;
        d_out[i] = di;
        y[i] += di;
    }
}

// ---- Chebyshev step on FP32-stored operator values, FP64 vectors and arithmetic -------------
// (FVM_SOLVE_FP32_PRECOND).  The stored values are B rounded to FP32, so the preconditioner is
// a fixed linear operator like the FP64 one, with a third less operator traffic per step.
// Each value is widened to FP64 by integer operations (sign, exponent rebias, fraction shift):
// on GB300 a float-to-double conversion instruction would occupy the scarce FP64 pipe once
// per stored entry.  FP32 subnormals (none in an assembled operator) read as zero.
__device__ __forceinline__ double widen_f32(float f) {
    const uint32_t b = __float_as_uint(f);
    const uint32_t e = (b >> 23) & 0xffu;
    const uint32_t sign = b & 0x80000000u;
    const uint32_t ed = e == 255u ? 2047u : e + 896u;
    const uint32_t hi = e ? (sign | (ed << 20) | ((b & 0x7fffffu) >> 3)) : sign;
    const uint32_t lo = e ? (b << 29) : 0u;
    return __hiloint2double((int)hi, (int)lo);
}

template <int MAXW>
__device__ __forceinline__ double sell_row_f32v(const SpmvArgs& A, const float* __restrict__ val,
                                                const double* __restrict__ x, int64_t s, int lane) {
    const int64_t base = __ldg(&A.slice_ptr[s]) + lane;
    const int w = __ldg(&A.width[s]);
    double acc = 0.0;
    if constexpr (MAXW > 0) {
        int32_t c[MAXW];
        float v[MAXW];
#pragma unroll
        for (int k = 0; k < MAXW; ++k)
            if (k < w) {
                c[k] = __ldg(&A.col[base + (int64_t)k * 32]);
                v[k] = __ldg(&val[base + (int64_t)k * 32]);
            }
        double xs[MAXW];
#pragma unroll
        for (int k = 0; k < MAXW; ++k)
            if (k < w) xs[k] = __ldg(&x[c[k]]);
#pragma unroll
        for (int k = 0; k < MAXW; ++k)
            if (k < w) acc += widen_f32(v[k]) * xs[k];
    } else {
        for (int k = 0; k < w; ++k) {
            const int64_t i = base + (int64_t)k * 32;
            acc += widen_f32(__ldg(&val[i])) * __ldg(&x[__ldg(&A.col[i])]);
        }
    }
    return acc;
}

__global__ void __launch_bounds__(kRedBlock, 8) cheb_step_f32v_kernel(SpmvArgs A, const float* val, const double* d_in,
                                                                   const double* invD, double* w, double* d_out,
                                                                   double* y, double c1, double c2, const KState* st,
                                                                   int gate) {
    if (gated(st, gate)) return;
    int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (s >= A.nslices) return;
    const double t = __ldg(&A.width[s]) <= 8 ? sell_row_f32v<8>(A, val, d_in, s, lane)
                                               : sell_row_f32v<0>(A, val, d_in, s, lane);
    int64_t i = s * kSlice + lane;
    if (i < A.n) {
        const double wi = w[i] - invD[i] * t;
        w[i] = wi;
        const double di = c1 * d_in[i] + c2 * wi;
        d_out[i] = di;
        y[i] += di;
    }
}

// CG with a polynomial preconditioner: rz = r . z, beta = rz / rz_old; p = z on a restart
template <class T>
__global__ void __launch_bounds__(kRedBlock) cg_rz_kernel(const T* r, const T* z, T* p, int set_p, int64_t n,
                                                          double* part, KState* st, int gate) {
    if (gated(st, gate)) return;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double v[1] = {0.0};
    if (i < n) {
        v[0] = (double)(r[i] * z[i]);
        if (set_p) p[i] = z[i];
    }
    bool last;
    block_reduce_publish<1>(v, part, st, gridDim.x, last);
    if (last && threadIdx.x == 0) {
        const double rz_old = st->rz;
        st->rz = v[0];
        st->beta = rz_old > 0 ? v[0] / rz_old : 0.0;
    }
}

// p = z + beta p (runs whenever the update step of the same iteration ran)
template <class T>
__global__ void cg_pupdate_z_kernel(T* p, const T* z, int64_t n, const KState* st) {
    if (st->skip3) return;
    T beta = (T)st->beta;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = z[i] + beta * p[i];
}

// residual r = rhs - B z (FP64), its FP32 copy, and the scalars that restart / continue CG
template <class T>
__global__ void __launch_bounds__(kRedBlock) residual_kernel(SpmvArgs A, const double* val, const double* z,
                                                             const double* rhs, const double* invV, const T* invD,
                                                             T* r_out, T* p_out, int set_p, double* part, KState* st) {
    int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    double v[2] = {0.0, 0.0};
    if (s < A.nslices) {
        double y = sell_row<double, double>(A.slice_ptr, A.width, A.col, val, z, s, lane);
        int64_t i = s * kSlice + lane;
        if (i < A.n) {
            double ri = rhs[i] - y;
            T rt = (T)ri;
            r_out[i] = rt;
            if (set_p) p_out[i] = invD[i] * rt;
            v[0] = (double)(rt * rt * invD[i]);
            double w = ri * invV[i];
            v[1] = w * w;
        }
    }
    bool last;
    block_reduce_publish<2>(v, part, st, gridDim.x, last);
    if (last && threadIdx.x == 0) {
        st->rz = v[0];
        st->rn2 = v[1];
        st->dot[1] = v[1];
        st->done = (v[1] <= st->tol2) ? 1 : 0;
        st->breakdown = 0;
    }
}

// z64 += sign * x (x in the inner precision)
template <class T>
__global__ void accumulate_kernel(double* z, const T* x, double sign, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) z[i] += sign * (double)x[i];
}

// ---- BiCGStab pieces --------------------------------------------------------------------
// p = r + beta (p - omega v); phat = invD p
template <class T>
__global__ void bicg_p_kernel(T* p, T* phat, const T* r, const T* v, const T* invD, int64_t n, const KState* st) {
    if (st->done) return;
    T beta = (T)st->beta, omega = (T)st->omega;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        T pi = r[i] + beta * (p[i] - omega * v[i]);
        p[i] = pi;
        phat[i] = invD[i] * pi;
    }
}
// v = B phat; alpha = rho / (rhat . v)
template <class V, class T>
__global__ void __launch_bounds__(kRedBlock, 8) bicg_v_kernel(SpmvArgs A, const V* val, const T* rowsum, const T* phat, T* v,
                                                           const T* rhat, double* part, KState* st) {
    if (st->done) return;
    int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    double d[1] = {0.0};
    if (s < A.nslices) {
        T y = spmv_row<V, T>(A, val, rowsum, phat, s, lane);
        int64_t i = s * kSlice + lane;
        if (i < A.n) {
            v[i] = y;
            d[0] = (double)(rhat[i] * y);
        }
    }
    bool last;
    block_reduce_publish<1>(d, part, st, gridDim.x, last);
    if (last && threadIdx.x == 0) {
        if (d[0] == 0.0 || !isfinite(d[0])) {
            st->done = 1;
            st->breakdown = 1;
        } else {
            st->alpha = st->rho / d[0];
        }
    }
}
// s = r - alpha v (into r); shat = invD s
template <class T>
__global__ void bicg_s_kernel(T* r, T* shat, const T* v, const T* invD, int64_t n, const KState* st) {
    if (st->done) return;
    T alpha = (T)st->alpha;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        T si = r[i] - alpha * v[i];
        r[i] = si;
        shat[i] = invD[i] * si;
    }
}
// t = B shat; omega = (t . s) / (t . t)
template <class V, class T>
__global__ void __launch_bounds__(kRedBlock, 8) bicg_t_kernel(SpmvArgs A, const V* val, const T* rowsum, const T* shat, T* t,
                                                           const T* s_vec,
                                                           double* part, KState* st) {
    if (st->done) return;
    int64_t sl = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    double d[2] = {0.0, 0.0};
    if (sl < A.nslices) {
        T y = spmv_row<V, T>(A, val, rowsum, shat, sl, lane);
        int64_t i = sl * kSlice + lane;
        if (i < A.n) {
            t[i] = y;
            d[0] = (double)(y * s_vec[i]);
            d[1] = (double)(y * y);
        }
    }
    bool last;
    block_reduce_publish<2>(d, part, st, gridDim.x, last);
    if (last && threadIdx.x == 0) st->omega = d[1] > 0 ? d[0] / d[1] : 0.0;
}
// x += alpha phat + omega shat; r = s - omega t; rho_new = rhat . r; rn2; beta
template <class T>
__global__ void __launch_bounds__(kRedBlock) bicg_x_kernel(T* x, T* r, const T* phat, const T* shat, const T* t,
                                                           const T* rhat, const T* invV, int64_t n, double* part,
                                                           KState* st) {
    if (st->done) return;
    T alpha = (T)st->alpha, omega = (T)st->omega;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double d[2] = {0.0, 0.0};
    if (i < n) {
        x[i] += alpha * phat[i] + omega * shat[i];
        T ri = r[i] - omega * t[i];
        r[i] = ri;
        d[0] = (double)(rhat[i] * ri);
        T w = ri * invV[i];
        d[1] = (double)(w * w);
    }
    bool last;
    block_reduce_publish<2>(d, part, st, gridDim.x, last);
    if (last && threadIdx.x == 0) {
        double rho_old = st->rho;
        st->rho = d[0];
        st->rn2 = d[1];
        if (d[1] <= st->tol2 || !isfinite(d[1])) st->done = 1;
        if (d[1] > st->div2) st->done = st->breakdown = 1;
        if (st->omega == 0.0 || rho_old == 0.0) {
            st->done = 1;
            st->breakdown = 1;
        } else {
            st->beta = (d[0] / rho_old) * (st->alpha / st->omega);
        }
    }
}
// BiCGStab (re)start: rhat = r, p = v = 0, rho = rhat . r, omega = 1, beta = 0
template <class T>
__global__ void __launch_bounds__(kRedBlock) bicg_start_kernel(T* rhat, const T* r, T* p, T* v, int64_t n,
                                                               double* part, KState* st) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double d[1] = {0.0};
    if (i < n) {
        T ri = r[i];
        rhat[i] = ri;
        p[i] = 0;
        v[i] = 0;
        d[0] = (double)(ri * ri);
    }
    bool last;
    block_reduce_publish<1>(d, part, st, gridDim.x, last);
    if (last && threadIdx.x == 0) {
        st->rho = d[0];
        st->beta = 0;
        st->omega = 1;
        st->alpha = 0;
        st->breakdown = 0;
        if (d[0] == 0.0) st->done = 1;
    }
}

// After a reliable update replaced r by the true residual: rho' = rhat . r, and the pending
// beta is rescaled to it (beta = (rho'/rho_old) (alpha/omega) with the recurrence rho replaced).
template <class T>
__global__ void __launch_bounds__(kRedBlock) bicg_rho_fix_kernel(const T* rhat, const T* r, int64_t n, double* part,
                                                                 KState* st) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double d[1] = {0.0};
    if (i < n) d[0] = (double)(rhat[i] * r[i]);
    bool last;
    block_reduce_publish<1>(d, part, st, gridDim.x, last);
    if (last && threadIdx.x == 0) {
        if (st->rho != 0.0) st->beta *= d[0] / st->rho;
        st->rho = d[0];
        if (d[0] == 0.0) st->breakdown = 1;
    }
}

template <class T>
__global__ void to_type_kernel(T* dst, const double* src, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = (T)src[i];
}

// x_out = z + xfix (internal)
__global__ void combine_kernel(double* x, const double* z, const double* xfix, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = z[i] + xfix[i];
}
// z = x - xfix on free rows, 0 on fixed rows
__global__ void split_kernel(double* z, const double* x, const double* xfix, const int8_t* fixed, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) z[i] = fixed[i] ? 0.0 : x[i];
}

static unsigned blocks_for(int64_t n) { return (unsigned)((n + kRedBlock - 1) / kRedBlock); }

}  // namespace fvm

using namespace fvm;

// reduced operator of the steady template
void fvm_template::build_steady() {
    if (steady_ready) return;
    if (kind != FVM_TEMPLATE_POISSON && kind != FVM_TEMPLATE_MEAN_EXIT_TIME)
        fail(FVM_ERR_INVALID_ARGUMENT, "steady solves apply to PoissonsEquation / MeanExitTimeProblem templates");
    const fvm_mesh* m = prob->mesh;
    const SellPattern& pat = m->pat;
    const int64_t n = m->np;
    std::vector<int8_t> fixed(n, 0);
    for (int64_t v = 0; v < n; ++v) {
        int32_t r = m->iperm[v];
        fixed[r] = (prob->code[v] == FVM_VERTEX_DIRICHLET || !m->has_vertex[v]) ? 1 : 0;
    }
    std::vector<double> xfix(n, 0.0), rhs(n, 0.0), Bv(pat.nslots, 0.0), invD(n, 1.0), Vr(n, 0.0);
    for (int64_t r = 0; r < n; ++r) {
        Vr[r] = m->vol[m->perm[r]];
        if (fixed[r]) xfix[r] = b[r];
    }
    double asym = 0, scale = 0;
    for (int64_t s = 0; s < pat.nslices; ++s)
        for (int lane = 0; lane < kSlice; ++lane) {
            int64_t r = s * kSlice + lane;
            if (r >= n) continue;
            int64_t len = pat.rowptr[r + 1] - pat.rowptr[r];
            double acc = b[r];
            for (int64_t q = 0; q < len; ++q) {
                int64_t slot = pat.slice_ptr[s] + q * kSlice + lane;
                int32_t c = pat.col[slot];
                double a = val[slot];
                if (fixed[r]) {
                    Bv[slot] = (c == r) ? 1.0 : 0.0;
                } else if (fixed[c]) {
                    acc -= a * b[c];
                } else {
                    Bv[slot] = -Vr[r] * a;
                }
            }
            rhs[r] = fixed[r] ? 0.0 : -Vr[r] * acc;
        }
    // symmetry of B and its diagonal
    for (int64_t r = 0; r < n; ++r) {
        for (int64_t q = pat.rowptr[r]; q < pat.rowptr[r + 1]; ++q) {
            int32_t c = pat.csr_col[q];
            double brc = Bv[pat.csr_slot[q]];
            scale = std::max(scale, std::fabs(brc));
            if (c == r) {
                invD[r] = brc != 0 ? 1.0 / brc : 1.0;
                continue;
            }
            int64_t t = pat.find(c, (int32_t)r);
            double bcr = t >= 0 ? Bv[t] : 0.0;
            asym = std::max(asym, std::fabs(brc - bcr));
        }
        if (!fixed[r] && !(invD[r] > 0)) fail(FVM_ERR_INVALID_ARGUMENT, "steady operator has a non-positive diagonal");
    }
    symmetric = asym <= 1e-12 * std::max(scale, 1e-300) ? 1 : 0;
    // Gershgorin bound on the spectrum of D^-1 B (for the Chebyshev preconditioner)
    cheb_gershgorin = 1.0;
    for (int64_t r = 0; r < n; ++r) {
        double row = 0;
        for (int64_t q = pat.rowptr[r]; q < pat.rowptr[r + 1]; ++q) row += std::fabs(Bv[pat.csr_slot[q]]);
        cheb_gershgorin = std::max(cheb_gershgorin, row * std::fabs(invD[r]));
    }
    double bn = 0;
    for (int64_t r = 0; r < n; ++r) bn += b[r] * b[r];
    bnorm = std::sqrt(bn);
    // FP32 operator in difference form: off-diagonal values (zero diagonal) and FP64 row sums
    std::vector<float> Bv32(Bv.size(), 0.0f), Bx32(Bv.size()), rs32(n), invD32(n), invV32(n);
    for (size_t k = 0; k < Bv.size(); ++k) Bx32[k] = (float)Bv[k];
    std::vector<double> invV(n);
    for (int64_t s = 0; s < pat.nslices; ++s)
        for (int lane = 0; lane < kSlice; ++lane) {
            const int64_t r = s * kSlice + lane;
            if (r >= n) continue;
            double rs = 0;
            for (int64_t q = 0; q < pat.width[s]; ++q) {
                const int64_t slot = pat.slice_ptr[s] + q * kSlice + lane;
                rs += Bv[slot];
                if (pat.col[slot] != r) Bv32[slot] = (float)Bv[slot];
            }
            rs32[r] = (float)rs;
        }
    for (int64_t r = 0; r < n; ++r) {
        invD32[r] = (float)invD[r];
        invV[r] = fixed[r] ? 0.0 : 1.0 / Vr[r];
        invV32[r] = (float)invV[r];
    }
    d_bval64.upload(Bv);
    d_bval32.upload(Bv32);
    d_bval32x.upload(Bx32);
    d_brow32.upload(rs32);
    d_bdiag_inv64.upload(invD);
    d_bdiag_inv32.upload(invD32);
    d_rhs_red.upload(rhs);
    d_xfix.upload(xfix);
    d_invV_free64.upload(invV);
    d_invV_free32.upload(invV32);
    d_fixed_mask.upload(fixed);
    steady_ready = true;
}

namespace {

struct Solver {
    fvm_template* T;
    const fvm_mesh* m;
    int64_t n;
    cudaStream_t s;
    SpmvArgs A;
    unsigned nb, nbs;  // blocks for vector kernels, for SpMV kernels
    DBuf ws;
    KState* st;
    double* part;
    double* z64;
    void* vec;  // typed work vectors

    Solver(fvm_template* t, cudaStream_t st_) : T(t), m(t->prob->mesh), n(m->np), s(st_) {
        A.slice_ptr = m->pat.d_slice_ptr.as<int64_t>();
        A.width = m->pat.d_width.as<int32_t>();
        A.col = m->pat.d_col.as<int32_t>();
        A.n = n;
        A.nslices = m->pat.nslices;
        nb = blocks_for(n);
        nbs = (unsigned)((m->pat.nslices * 32 + kRedBlock - 1) / kRedBlock);
    }
};

template <class T>
struct Vecs {
    T *x, *r, *p, *Ap, *rhat, *phat, *shat, *t;
    T *w, *d0, *d1;                    // Chebyshev work vectors
    const float* f32vals;              // FP32-stored operator of the preconditioner (FVM_SOLVE_FP32_PRECOND)
};

constexpr int kWorkVectors = 11;  // vectors of the Krylov type

// y = p(D^-1 B) D^-1 r (Chebyshev preconditioner; see cheb_plan)
template <class V, class T>
static void cheb_apply(const Solver& S, const ChebPlan& P, const V* val, const T* rowsum, const T* invD, const T* r,
                       T* y, Vecs<T>& v, int gate) {
    if constexpr (std::is_same_v<T, double>) {
        if (v.f32vals) {  // FP32-stored operator values, FP64 vectors and arithmetic
            cheb_init_kernel<double><<<S.nb, kRedBlock, 0, S.s>>>(r, invD, v.w, v.d0, y, P.inv_theta, S.n, S.st, gate);
            double *din = v.d0, *dout = v.d1;
            for (int j = 1; j < P.degree; ++j) {
                cheb_step_f32v_kernel<<<S.nbs, kRedBlock, 0, S.s>>>(S.A, v.f32vals, din, invD, v.w, dout, y, P.c1[j],
                                                                    P.c2[j], S.st, gate);
                std::swap(din, dout);
            }
            return;
        }
    }
    cheb_init_kernel<T><<<S.nb, kRedBlock, 0, S.s>>>(r, invD, v.w, v.d0, y, (T)P.inv_theta, S.n, S.st, gate);
    T *din = v.d0, *dout = v.d1;
    for (int j = 1; j < P.degree; ++j) {
        cheb_step_kernel<V, T><<<S.nbs, kRedBlock, 0, S.s>>>(S.A, val, rowsum, din, invD, v.w, dout, y, (T)P.c1[j],
                                                             (T)P.c2[j], S.st, gate);
        std::swap(din, dout);
    }
}

}  // namespace

template <class V, class T>
static void run_krylov(fvm_template* Tm, Solver& S, bool cg, bool mixed, const fvm_solver_options& o,
                       fvm_solver_stats& stats) {
    const int64_t n = S.n;
    cudaStream_t s = S.s;
    const V* val = mixed ? (const V*)Tm->d_bval32.p : (const V*)Tm->d_bval64.p;
    const T* invD = mixed ? (const T*)Tm->d_bdiag_inv32.p : (const T*)Tm->d_bdiag_inv64.p;
    const T* rowsum = mixed ? (const T*)Tm->d_brow32.p : nullptr;  // FP32 products in difference form
    const T* invV = mixed ? (const T*)Tm->d_invV_free32.p : (const T*)Tm->d_invV_free64.p;
    Vecs<T> v;
    T* base = (T*)S.vec;
    v.x = base;
    v.r = base + n;
    v.p = base + 2 * n;
    v.Ap = base + 3 * n;
    v.rhat = base + 4 * n;
    v.phat = base + 5 * n;
    v.shat = base + 6 * n;
    v.t = base + 7 * n;
    v.w = base + 8 * n;
    v.d0 = base + 9 * n;
    v.d1 = base + 10 * n;
    v.f32vals = (o.mode == FVM_SOLVE_FP32_PRECOND && !mixed) ? Tm->d_bval32x.as<float>() : nullptr;
    const bool cheb = o.precond == FVM_PRECOND_CHEBYSHEV;
    const ChebPlan plan = cheb ? cheb_plan(Tm->cheb_gershgorin, o.cheb_degree > 0 ? o.cheb_degree : 4) : ChebPlan{};
    T* zc = v.rhat;  // CG's preconditioned residual (BiCGStab's rhat is unused by CG)
    FVM_CUDA(cudaMemsetAsync(v.x, 0, sizeof(T) * n, s));
    const double tol = o.rtol * Tm->bnorm;
    const double tol2 = tol * tol;
    const int64_t maxit = o.max_iters > 0 ? o.max_iters : 1000000;
    // FP32 inner arithmetic (mixed) makes the iteration run in cycles: each cycle reduces the
    // residual by `inner_reduction`, then the FP64 true residual is recomputed.  The FP32
    // Krylov recurrences drift, which BiCGStab's short recurrences do not tolerate for long:
    // its cycles restart from the FP64 residual.  (fp32pc keeps FP64 arithmetic throughout:
    // its preconditioner is linear, so it runs like the FP64 iteration.)
    const bool fp32pc = o.mode == FVM_SOLVE_FP32_PRECOND && !mixed;
    const bool cycles = mixed;
    double red = o.inner_reduction > 0 && o.inner_reduction < 1 ? o.inner_reduction : 1e-2;
    KState h{};
    auto set_tol = [&](double t2) {
        FVM_CUDA(cudaMemcpyAsync(&S.st->tol2, &t2, sizeof(double), cudaMemcpyHostToDevice, s));
    };
    // cycles with FP32 inner arithmetic stop when their recurrence residual grows 1e4-fold
    auto set_div = [&](double rn0) {
        const double d2 = cycles ? 1e8 * rn0 * rn0 : std::numeric_limits<double>::infinity();
        FVM_CUDA(cudaMemcpyAsync(&S.st->div2, &d2, sizeof(double), cudaMemcpyHostToDevice, s));
    };
    auto read_state = [&]() {
        FVM_CUDA(cudaMemcpyAsync(&h, S.st, sizeof(KState), cudaMemcpyDeviceToHost, s));
        FVM_CUDA(cudaStreamSynchronize(s));
    };
    // true residual from z64 (FP64); sets r, optionally p, rz, rn2, done
    auto true_residual = [&](bool set_p) {
        set_tol(tol2);
        const bool poly_cg = cg && cheb;
        residual_kernel<T><<<S.nbs, kRedBlock, 0, s>>>(S.A, Tm->d_bval64.as<double>(), S.z64, Tm->d_rhs_red.as<double>(),
                                                      Tm->d_invV_free64.as<double>(), invD, v.r, v.p,
                                                      set_p && !poly_cg ? 1 : 0, S.part, S.st);
        if (poly_cg) {  // rz = r . M^-1 r, and p = M^-1 r on a restart
            cheb_apply<V, T>(S, plan, val, rowsum, invD, v.r, zc, v, 0);
            cg_rz_kernel<T><<<S.nb, kRedBlock, 0, s>>>(v.r, zc, v.p, set_p ? 1 : 0, n, S.part, S.st, 0);
        }
        FVM_CUDA(cudaGetLastError());
        read_state();
        ++stats.refinements;
        return std::sqrt(h.rn2);
    };
    double rn = true_residual(true);
    const int chunk = 16;
    int64_t it = 0;
    int stagnation = 0, rejects = 0;
    double rn_last_update = rn;
    double best = rn;
    double red_cur = red;
    static const bool trace = std::getenv("FVM_SOLVER_TRACE") != nullptr;
    // inner target: the FP32 recurrence is trusted down to `red_cur` of the last true residual
    auto inner_tol2 = [&]() {
        double t = cycles ? std::max(tol, red_cur * rn_last_update) : tol;
        return t * t;
    };
    bool need_start = !cg;
    while (rn > tol) {
        if (it >= maxit) break;
        set_tol(inner_tol2());
        set_div(rn);
        if (need_start) {
            // BiCGStab restart from the current residual: rhat = r, p = v = 0, rho = r.r
            bicg_start_kernel<T><<<S.nb, kRedBlock, 0, s>>>(v.rhat, v.r, v.p, v.Ap, n, S.part, S.st);
            need_start = false;
        }
        for (int c = 0; c < chunk; ++c) {
            if (cg) {
                cg_spmv_kernel<V, T><<<S.nbs, kRedBlock, 0, s>>>(S.A, val, rowsum, v.p, v.Ap, S.part, S.st);
                if (cheb) {
                    cg_update_kernel<T, false><<<S.nb, kRedBlock, 0, s>>>(v.x, v.r, v.p, v.Ap, invD, invV, n, S.part,
                                                                          S.st);
                    cheb_apply<V, T>(S, plan, val, rowsum, invD, v.r, zc, v, 1);
                    cg_rz_kernel<T><<<S.nb, kRedBlock, 0, s>>>(v.r, zc, v.p, 0, n, S.part, S.st, 1);
                    cg_pupdate_z_kernel<T><<<S.nb, kRedBlock, 0, s>>>(v.p, zc, n, S.st);
                } else {
                    cg_update_kernel<T, true><<<S.nb, kRedBlock, 0, s>>>(v.x, v.r, v.p, v.Ap, invD, invV, n, S.part,
                                                                         S.st);
                    cg_pupdate_kernel<T><<<S.nb, kRedBlock, 0, s>>>(v.p, v.r, invD, n, S.st);
                }
            } else {
                bicg_p_kernel<T><<<S.nb, kRedBlock, 0, s>>>(v.p, v.phat, v.r, v.Ap, invD, n, S.st);
                if (cheb) cheb_apply<V, T>(S, plan, val, rowsum, invD, v.p, v.phat, v, 0);  // phat = M^-1 p
                bicg_v_kernel<V, T><<<S.nbs, kRedBlock, 0, s>>>(S.A, val, rowsum, v.phat, v.Ap, v.rhat, S.part, S.st);
                bicg_s_kernel<T><<<S.nb, kRedBlock, 0, s>>>(v.r, v.shat, v.Ap, invD, n, S.st);
                if (cheb) cheb_apply<V, T>(S, plan, val, rowsum, invD, v.r, v.shat, v, 0);  // shat = M^-1 s
                bicg_t_kernel<V, T><<<S.nbs, kRedBlock, 0, s>>>(S.A, val, rowsum, v.shat, v.t, v.r, S.part, S.st);
                bicg_x_kernel<T><<<S.nb, kRedBlock, 0, s>>>(v.x, v.r, v.phat, v.shat, v.t, v.rhat, invV, n, S.part, S.st);
            }
        }
        FVM_CUDA(cudaGetLastError());
        read_state();
        it += chunk;  // iterations issued (kernels after convergence return at once)
        if (!h.done) continue;
        // reliable update: fold the correction into the FP64 solution, recompute the residual
        accumulate_kernel<T><<<S.nb, kRedBlock, 0, s>>>(S.z64, v.x, 1.0, n);
        bool restart = h.breakdown != 0 || (cycles && !cg);
        const double rec = std::sqrt(h.rn2);
        const int brk = h.breakdown;
        double rn_new = true_residual(restart);
        if (trace)
            std::fprintf(stderr, "[fvm solver] %s %s it=%lld rn=%.3e (recurrence %.3e) breakdown=%d\n",
                         cg ? "cg" : "bicgstab", mixed ? "mixed" : fp32pc ? "fp32-precond" : "fp64", (long long)it,
                         rn_new / Tm->bnorm,
                         rec / Tm->bnorm, brk);
        if (!(rn_new < rn)) {
            // the correction raised the true residual (inner-precision drift or breakdown):
            // undo it, restart from the FP64 residual with a milder inner reduction
            accumulate_kernel<T><<<S.nb, kRedBlock, 0, s>>>(S.z64, v.x, -1.0, n);
            rn_new = true_residual(true);
            restart = true;
            red_cur = std::min(0.5, red_cur * 4);
            if (++rejects > 6) break;
        }
        FVM_CUDA(cudaMemsetAsync(v.x, 0, sizeof(T) * n, s));
        rn = rn_new;
        if (!cg) {
            if (restart) {
                need_start = true;
            } else {
                // keep the BiCGStab recurrences; only rho (and the pending beta) follow the new r
                bicg_rho_fix_kernel<T><<<S.nb, kRedBlock, 0, s>>>(v.rhat, v.r, n, S.part, S.st);
                read_state();
                if (h.breakdown) need_start = true;
            }
        }
        if (rn < 0.9 * best) {
            best = rn;
            stagnation = 0;
        } else if (++stagnation > 8) {
            break;
        }
        rn_last_update = rn;
    }
    stats.iterations += it;
    stats.rel_residual = Tm->bnorm > 0 ? rn / Tm->bnorm : rn;
    if (rn > tol) {
        char msg[160];
        std::snprintf(msg, sizeof msg, "steady solve did not reach rtol %.3e (relative residual %.3e after %lld iterations)",
                      o.rtol, stats.rel_residual, (long long)stats.iterations);
        fail(FVM_ERR_NOT_CONVERGED, msg);
    }
}

extern "C" int fvm_template_steady_solve(fvm_template* Tm, double* x, const fvm_solver_options* opt,
                                         fvm_solver_stats* stats, int32_t flags, void* stream) {
    return guard_call([&] {
        if (!Tm || !x || !opt) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        Tm->build_steady();
        cudaStream_t s = (cudaStream_t)stream;
        const fvm_mesh* m = Tm->prob->mesh;
        const int64_t n = m->np;
        int32_t loc = flags & 3;
        if (loc == FVM_PTR_DEVICE_INTERNAL) fail(FVM_ERR_INVALID_ARGUMENT, "steady solve takes host or device arrays in the caller's numbering");
        fvm_solver_stats st{};
        bool mixed = opt->mode == FVM_SOLVE_MIXED;
        if (opt->mode == FVM_SOLVE_FP32_PRECOND && opt->precond != FVM_PRECOND_CHEBYSHEV)
            fail(FVM_ERR_INVALID_ARGUMENT, "the FP32 inner iteration is the Chebyshev preconditioner: set precond");
        bool cg = opt->method == FVM_SOLVER_CG || (opt->method == FVM_SOLVER_AUTO && Tm->symmetric);
        st.method_used = cg ? FVM_SOLVER_CG : FVM_SOLVER_BICGSTAB;
        st.symmetric = Tm->symmetric;
        if (opt->precond != FVM_PRECOND_JACOBI && opt->precond != FVM_PRECOND_CHEBYSHEV)
            fail(FVM_ERR_INVALID_ARGUMENT, "unknown preconditioner");
        if (opt->precond == FVM_PRECOND_CHEBYSHEV && opt->cheb_degree > kChebMax)
            fail(FVM_ERR_INVALID_ARGUMENT, "Chebyshev degree above 16");
        Solver S(Tm, s);
        // vectors sized for FP64 even in mixed mode: a stalled mixed solve finishes in FP64
        // (run_krylov<double, double>) on the same workspace
        size_t elem = sizeof(double);
        size_t bytes = sizeof(KState) + sizeof(double) * 8 * (size_t)std::max(S.nb, S.nbs) + sizeof(double) * 3 * n +
                       elem * kWorkVectors * n + 256;
        S.ws.alloc(bytes);
        char* w = S.ws.as<char>();
        S.st = (KState*)w;
        w += (sizeof(KState) + 255) / 256 * 256;
        S.part = (double*)w;
        w += sizeof(double) * 8 * std::max(S.nb, S.nbs);
        S.z64 = (double*)w;
        double* xref = S.z64 + n;
        double* xint = S.z64 + 2 * n;
        w += sizeof(double) * 3 * n;
        S.vec = w;
        FVM_CUDA(cudaMemsetAsync(S.st, 0, sizeof(KState), s));
        // initial guess -> z (free rows), internal numbering
        if (loc == FVM_PTR_HOST)
            FVM_CUDA(cudaMemcpyAsync(xref, x, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        else
            FVM_CUDA(cudaMemcpyAsync(xref, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        launch_permute_in(m->d_perm.as<int32_t>(), xref, xint, n, s);
        split_kernel<<<S.nb, kRedBlock, 0, s>>>(S.z64, xint, Tm->d_xfix.as<double>(), Tm->d_fixed_mask.as<int8_t>(), n);
        cudaEvent_t e0, e1;
        FVM_CUDA(cudaEventCreate(&e0));
        FVM_CUDA(cudaEventCreate(&e1));
        FVM_CUDA(cudaEventRecord(e0, s));
        int status = FVM_OK;
        std::string msg;
        try {
            if (mixed) {
                try {
                    run_krylov<float, float>(Tm, S, cg, true, *opt, st);
                } catch (const Error& e) {
                    if (e.code != FVM_ERR_NOT_CONVERGED) throw;
                    // the FP32 inner iteration stalled: finish in FP64 from the current solution
                    st.fallback_fp64 = 1;
                    run_krylov<double, double>(Tm, S, cg, false, *opt, st);
                }
            } else if (opt->mode == FVM_SOLVE_FP32_PRECOND) {
                try {
                    run_krylov<double, double>(Tm, S, cg, false, *opt, st);
                } catch (const Error& e) {
                    if (e.code != FVM_ERR_NOT_CONVERGED) throw;
                    // the FP32 polynomial stalled the iteration: finish with the FP64 polynomial
                    st.fallback_fp64 = 1;
                    fvm_solver_options o64 = *opt;
                    o64.mode = FVM_SOLVE_FP64;
                    run_krylov<double, double>(Tm, S, cg, false, o64, st);
                }
            } else {
                run_krylov<double, double>(Tm, S, cg, false, *opt, st);
            }
        } catch (const Error& e) {
            if (e.code != FVM_ERR_NOT_CONVERGED) {
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                throw;
            }
            status = e.code;
            msg = e.what();
        }
        FVM_CUDA(cudaEventRecord(e1, s));
        FVM_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        st.elapsed_ms = ms;
        combine_kernel<<<S.nb, kRedBlock, 0, s>>>(xint, S.z64, Tm->d_xfix.as<double>(), n);
        launch_permute_out(m->d_perm.as<int32_t>(), xint, xref, n, s);
        if (loc == FVM_PTR_HOST)
            FVM_CUDA(cudaMemcpyAsync(x, xref, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
        else
            FVM_CUDA(cudaMemcpyAsync(x, xref, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        FVM_CUDA(cudaStreamSynchronize(s));
        FVM_CUDA(cudaGetLastError());
        if (stats) *stats = st;
        if (status != FVM_OK) fail(status, msg);
        return FVM_OK;
    });
}
