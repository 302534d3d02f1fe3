// Steady solve of a Poisson / mean-exit-time template (LinearProblem(A, b) + solve,
// poissons_equation.jl:81, mean_exit_time.jl:76) on the GPU alone.
//
// Rows fixed by a Dirichlet condition or a missing vertex are identity rows of A; the
// remaining (free) rows are scaled by -V_i, which turns -div(D grad) into a symmetric
// positive definite operator B when D is constant on each triangle:
//     B z = rhs,  B_ij = -V_i A_ij (i, j free),  rhs_i = -V_i (b_i - sum_{j fixed} A_ij b_j),
//     x = z + x_fixed,  and  (b - A x)_i = -(rhs - B z)_i / V_i  on free rows.
// CG runs when B is symmetric, BiCGStab otherwise.  Mixed precision with the Chebyshev
// preconditioner: the Krylov iteration in FP64, its preconditioner polynomial in FP32 (values,
// vectors, difference-form products).  With Jacobi: FP32 Krylov cycles with FP64 reliable
// updates of the residual and the solution.  The stopping test is always the certified FP64
// residual ||b - A x|| / ||b|| of the reference operator (difference form, compensated row sums).
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

// Vector kernels that end in a grid-wide reduction run one wave of blocks that each walk a
// contiguous range of rows, so that each block pays the reduction's fence and atomic once for
// many rows instead of once for 256.
#define FVM_FOR_ROWS(i, n)                                                                            \
    for (int64_t i = (int64_t)(n) * blockIdx.x / gridDim.x + threadIdx.x,                             \
                 i##_end = (int64_t)(n) * (blockIdx.x + 1) / gridDim.x;                               \
         i < i##_end; i += blockDim.x)

struct KState {               // device-resident Krylov scalars
    double dot[8];            // reduction results
    double alpha, beta, omega, rho, rz, tol2, rn2;
    double div2;              // a cycle whose recurrence residual^2 exceeds this has diverged
    double grow2;             // ... or exceeds grow2 times the smallest one of the cycle
    double rmin2;             // smallest recurrence residual^2 of the cycle
    int done;
    int breakdown;
    int skip3;                // CG: the update step of this iteration did not run
    unsigned counter;
};

// Sum of part[0], part[stride], ... over the thread's share of n entries (entries b with
// b % step == first), four loads in flight: a single-block pass over thousands of partials
// otherwise waits one L2 round trip per entry.  The order is fixed by (n, step, first).
__device__ __forceinline__ double sum_strided(const double* part, int n, int first, int step) {
    double t0 = 0, t1 = 0, t2 = 0, t3 = 0;
    int b = first;
    for (; b + 3 * step < n; b += 4 * step) {
        t0 += __ldcg(&part[b]);
        t1 += __ldcg(&part[b + step]);
        t2 += __ldcg(&part[b + 2 * step]);
        t3 += __ldcg(&part[b + 3 * step]);
    }
    for (; b < n; b += step) t0 += __ldcg(&part[b]);
    return (t0 + t1) + (t2 + t3);
}

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
        double s = sum_strided(part + q * nblocks, nblocks, threadIdx.x, blockDim.x);
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

// Block partials of a grid-wide reduction, written without a fence or atomic: the sparse
// products run one slice per warp in many short blocks, and a fence and atomic per block cost
// them more than one small finalising launch (finalize_kernel) does.
template <int NV>
__device__ void block_partials(const double (&v)[NV], double* part) {
    __shared__ double red[NV][kRedBlock / 32];
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
            double t = 0;
            for (int w = 0; w < kRedBlock / 32; ++w) t += red[q][w];
            part[q * gridDim.x + blockIdx.x] = t;
        }
    }
}

// what a finalize_kernel launch computes from the sums of the partials
enum FinalizeOp { kFinCgAlpha, kFinBicgAlpha, kFinBicgOmega, kFinResidual };

// Sums the partials of the preceding launch in a fixed order (deterministic) and updates the
// Krylov scalars; one block of kFinThreads threads.
constexpr int kFinThreads = 1024;
__global__ void __launch_bounds__(kFinThreads) finalize_kernel(const double* part, int nblocks, int nv, int op,
                                                               KState* st) {
    if (op != kFinResidual && st->done) return;
    __shared__ double red[4][kFinThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    double v[4] = {0, 0, 0, 0};
    for (int q = 0; q < nv; ++q) {
        double t = sum_strided(part + q * nblocks, nblocks, threadIdx.x, blockDim.x);
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (lane == 0) red[q][wid] = t;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int q = 0; q < nv; ++q)
        for (int w = 0; w < kFinThreads / 32; ++w) v[q] += red[q][w];
    switch (op) {
        case kFinCgAlpha:  // v0 = p . B p
            st->dot[0] = v[0];
            if (!(v[0] > 0) || !isfinite(v[0])) {
                st->done = 1;
                st->breakdown = 1;
                st->alpha = 0;
            } else {
                st->alpha = st->rz / v[0];
            }
            break;
        case kFinBicgAlpha:  // v0 = rhat . v
            if (v[0] == 0.0 || !isfinite(v[0])) {
                st->done = 1;
                st->breakdown = 1;
            } else {
                st->alpha = st->rho / v[0];
            }
            break;
        case kFinBicgOmega:  // v0 = t . s, v1 = t . t
            st->omega = v[1] > 0 ? v[0] / v[1] : 0.0;
            break;
        default:  // kFinResidual: v0 = r . D^-1 r, v1 = sum (r / V)^2, v2 = sum r^2
            st->rz = v[0];
            st->rn2 = v[1];
            st->dot[1] = v[1];
            st->dot[2] = v[2];
            st->done = (v[1] <= st->tol2) ? 1 : 0;
            st->breakdown = 0;
            break;
    }
}

// ---- sliced-ELL SpMV with a fused inner product: y = B x, dot(w, y) --------------------
// Rows of 9-16 slots: two unrolled chunks of eight slots (the second predicated), so a warp
// still issues eight independent loads per round trip instead of one.
template <class V, class T, bool DIFF>
__device__ __forceinline__ T sell_row_chunks(const int64_t* slice_ptr, int w, const int32_t* col, const V* val,
                                             const T* x, T xr, int64_t s, int lane) {
    const int64_t base = __ldg(&slice_ptr[s]) + lane;
    T acc = 0;
#pragma unroll
    for (int c0 = 0; c0 < 16; c0 += 8) {
        int32_t c[8];
        V v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (c0 + k < w) {
                c[k] = __ldg(&col[base + (int64_t)(c0 + k) * 32]);
                v[k] = __ldg(&val[base + (int64_t)(c0 + k) * 32]);
            }
        T xs[8];
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (c0 + k < w) xs[k] = __ldg(&x[c[k]]);
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (c0 + k < w) {
                if constexpr (DIFF)
                    acc += (T)v[k] * (xs[k] - xr);
                else
                    acc += (T)v[k] * xs[k];
            }
    }
    return acc;
}

// x gathered and accumulated in T.  Each block covers 8 slices (256 rows).  Slices of at
// most 8 slots (every triangulation here) take the fully unrolled path; the branch is
// uniform across the warp.
template <class V, class T>
__device__ __forceinline__ T sell_row(const int64_t* slice_ptr, const int32_t* width, const int32_t* col, const V* val,
                                      const T* x, int64_t s, int lane) {
    const int w = __ldg(&width[s]);
    if (w <= 8) return sell_row_product<V, T, T, false, 8>(slice_ptr, width, col, val, x, T(0), s, lane);
    if (w <= 16) return sell_row_chunks<V, T, false>(slice_ptr, w, col, val, x, T(0), s, lane);
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
    const int w = __ldg(&A.width[s]);
    const T acc = w <= 8    ? sell_row_product<V, T, T, true, 8>(A.slice_ptr, A.width, A.col, val, x, xr, s, lane)
                  : w <= 16 ? sell_row_chunks<V, T, true>(A.slice_ptr, w, A.col, val, x, xr, s, lane)
                            : sell_row_product<V, T, T, true, 0>(A.slice_ptr, A.width, A.col, val, x, xr, s, lane);
    return acc + rowsum[rc] * xr;
}

// The sparse-product kernels below are one-warp-per-slice gathers.  The FP32 ones are compiled
// for eight 256-thread blocks per SM (32 registers a thread); the FP64 ones keep the eight
// gathers and eight values of a slot chunk in registers (64 a thread, four blocks per SM)
// instead of spilling them to local memory.
template <class T>
constexpr int kSpmvBlocks = sizeof(T) == 8 ? 4 : 8;

// CG step 1: Ap = B p; pAp; alpha = rz / pAp
template <class V, class T>
__global__ void __launch_bounds__(kRedBlock, kSpmvBlocks<T>) cg_spmv_kernel(SpmvArgs A, const V* val, const T* rowsum, const T* p, T* Ap,
                                                            double* part,
                                                            KState* st) {
    if (st->done) return;
    const int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    double v[1] = {0.0};
    if (s < A.nslices) {
        T y = spmv_row<V, T>(A, val, rowsum, p, s, lane);
        int64_t r = s * kSlice + lane;
        if (r < A.n) {
            Ap[r] = y;
            v[0] = (double)(y * p[r]);
        }
    }
    block_partials<1>(v, part);  // finalize_kernel(kFinCgAlpha) follows
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
    double v[2] = {0.0, 0.0};
    FVM_FOR_ROWS(i, n) {
        T xi = x[i] + alpha * p[i];
        T ri = r[i] - alpha * Ap[i];
        x[i] = xi;
        r[i] = ri;
        T rr = ri * ri;
        v[0] += (double)(rr * invD[i]);
        T w = ri * invV[i];
        v[1] += (double)(w * w);
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
        if (v[1] > st->div2 || v[1] > st->grow2 * st->rmin2) st->done = st->breakdown = 1;
        st->rmin2 = fmin(st->rmin2, v[1]);
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

// LAST (the FP32 polynomial of the mixed mode): the step's y is written to the FP64 output
// y_out instead of back into y
template <class V, class T, bool LAST = false>
__global__ void __launch_bounds__(kRedBlock, kSpmvBlocks<T>) cheb_step_kernel(SpmvArgs A, const V* val, const T* rowsum, const T* d_in,
                                                              const T* invD,
                                                              T* w, T* d_out, T* y, T c1, T c2, const KState* st,
                                                              int gate, double* y_out = nullptr) {
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
        if constexpr (LAST)
            y_out[i] = (double)(y[i] + di);
        else
            y[i] += di;
    }
}

// First step of the FP32 polynomial of the mixed mode: w = D^-1 r, d = w / theta, y = d in
// FP32 from the FP64 input (a degree-1 polynomial writes y straight to the FP64 output)
__global__ void cheb_init_mixed_kernel(const double* r, const float* invD, float* w, float* d, float* y, double* y_out,
                                       float inv_theta, int64_t n, const KState* st, int gate) {
    if (gated(st, gate)) return;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const float wi = invD[i] * (float)r[i];
        w[i] = wi;
        const float di = wi * inv_theta;
        d[i] = di;
        if (y_out)
            y_out[i] = (double)di;
        else
            y[i] = di;
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
    double v[1] = {0.0};
    FVM_FOR_ROWS(i, n) {
        v[0] += (double)(r[i] * z[i]);
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

// Certified residual r = rhs - B z in FP64.  B z is evaluated in difference form with the
// compensated row sums of the stored values,
//     (B z)_r = sum_j B_rj (z_j - z_r) + rowsum_r z_r,
// which equals the explicit product of the stored FP64 operator in exact arithmetic (the
// diagonal and padding slots multiply z_r - z_r = 0).  Each product then carries the rounding
// of a difference of neighbouring values, where the explicit sum cancels terms of size |B||z|:
// at 2M disk points that cancellation alone is ~1e-9 of ||b||, above the residuals asked for.
// Writes r (FP64) and, with set_p, p = D^-1 r; block partials of r . D^-1 r, sum (r / V)^2 and
// sum r^2 for finalize_kernel(kFinResidual).
__global__ void __launch_bounds__(kRedBlock, kSpmvBlocks<double>) cert_residual_kernel(
    SpmvArgs A, const double* val, const double* rowsum, const double* z, const double* rhs, const double* invV,
    const double* invD, double* r, double* p_out, int set_p, double* part) {
    const int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    double v[3] = {0.0, 0.0, 0.0};
    if (s < A.nslices) {
        const double y = spmv_row<double, double>(A, val, rowsum, z, s, lane);
        int64_t i = s * kSlice + lane;
        if (i < A.n) {
            const double ri = rhs[i] - y;
            r[i] = ri;
            if (set_p) p_out[i] = invD[i] * ri;
            v[0] = ri * ri * invD[i];
            const double w = ri * invV[i];
            v[1] = w * w;
            v[2] = ri * ri;
        }
    }
    block_partials<3>(v, part);
}

// The FP32 inner system of a refinement cycle: r32 = scale r64 (scale brings the residual to
// unit RMS, away from FP32's subnormal range as the cycles shrink it); with set_p p = D^-1 r32;
// reduces r32 . D^-1 r32 and sum (r32 / V)^2 for the inner iteration's start.
__global__ void __launch_bounds__(kRedBlock) scale_residual_kernel(const double* r64, float* r32, float* p_out,
                                                                   int set_p, const float* invD, const float* invV,
                                                                   double scale, int64_t n, double* part, KState* st) {
    double v[2] = {0.0, 0.0};
    FVM_FOR_ROWS(i, n) {
        const float ri = (float)(scale * r64[i]);
        r32[i] = ri;
        if (set_p) p_out[i] = invD[i] * ri;
        v[0] += (double)(ri * ri * invD[i]);
        const float w = ri * invV[i];
        v[1] += (double)(w * w);
    }
    bool last;
    block_reduce_publish<2>(v, part, st, gridDim.x, last);
    if (last && threadIdx.x == 0) {
        st->rz = v[0];
        st->rn2 = v[1];
        st->done = (v[1] <= st->tol2) ? 1 : 0;
        st->breakdown = 0;
    }
}

// z64 += scale * x (x: a cycle's correction in the inner precision and units)
template <class T>
__global__ void accumulate_kernel(double* z, const T* x, double scale, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) z[i] += scale * (double)x[i];
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
__global__ void __launch_bounds__(kRedBlock, kSpmvBlocks<T>) bicg_v_kernel(SpmvArgs A, const V* val, const T* rowsum, const T* phat, T* v,
                                                           const T* rhat, double* part, KState* st) {
    if (st->done) return;
    const int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    double d[1] = {0.0};
    if (s < A.nslices) {
        T y = spmv_row<V, T>(A, val, rowsum, phat, s, lane);
        int64_t i = s * kSlice + lane;
        if (i < A.n) {
            v[i] = y;
            d[0] = (double)(rhat[i] * y);
        }
    }
    block_partials<1>(d, part);  // finalize_kernel(kFinBicgAlpha) follows
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
__global__ void __launch_bounds__(kRedBlock, kSpmvBlocks<T>) bicg_t_kernel(SpmvArgs A, const V* val, const T* rowsum, const T* shat, T* t,
                                                           const T* s_vec,
                                                           double* part, KState* st) {
    if (st->done) return;
    const int64_t sl = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
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
    block_partials<2>(d, part);  // finalize_kernel(kFinBicgOmega) follows
}
// x += alpha phat + omega shat; r = s - omega t; rho_new = rhat . r; rn2; beta
template <class T>
__global__ void __launch_bounds__(kRedBlock) bicg_x_kernel(T* x, T* r, const T* phat, const T* shat, const T* t,
                                                           const T* rhat, const T* invV, int64_t n, double* part,
                                                           KState* st) {
    if (st->done) return;
    T alpha = (T)st->alpha, omega = (T)st->omega;
    double d[2] = {0.0, 0.0};
    FVM_FOR_ROWS(i, n) {
        x[i] += alpha * phat[i] + omega * shat[i];
        T ri = r[i] - omega * t[i];
        r[i] = ri;
        d[0] += (double)(rhat[i] * ri);
        T w = ri * invV[i];
        d[1] += (double)(w * w);
    }
    bool last;
    block_reduce_publish<2>(d, part, st, gridDim.x, last);
    if (last && threadIdx.x == 0) {
        double rho_old = st->rho;
        st->rho = d[0];
        st->rn2 = d[1];
        if (d[1] <= st->tol2 || !isfinite(d[1])) st->done = 1;
        if (d[1] > st->div2 || d[1] > st->grow2 * st->rmin2) st->done = st->breakdown = 1;
        st->rmin2 = fmin(st->rmin2, d[1]);
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
    double d[1] = {0.0};
    FVM_FOR_ROWS(i, n) {
        T ri = r[i];
        rhat[i] = ri;
        p[i] = 0;
        v[i] = 0;
        d[0] += (double)(ri * ri);
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
    double d[1] = {0.0};
    FVM_FOR_ROWS(i, n) d[0] += (double)(rhat[i] * r[i]);
    bool last;
    block_reduce_publish<1>(d, part, st, gridDim.x, last);
    if (last && threadIdx.x == 0) {
        if (st->rho != 0.0) st->beta *= d[0] / st->rho;
        st->rho = d[0];
        if (d[0] == 0.0) st->breakdown = 1;
    }
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

// Neumaier's compensated sum (Neumaier 1974): the running sum plus the rounding error of every
// addition, recovered exactly by TwoSum-style differences.
struct CompensatedSum {
    double s = 0, c = 0;
    void add(double x) {
        const double t = s + x;
        c += std::fabs(s) >= std::fabs(x) ? (s - t) + x : (x - t) + s;
        s = t;
    }
    double value() const { return s + c; }
};

// reduced operator of the steady template, on the solver's row order
void fvm_template::build_steady() {
    if (steady_ready) return;
    if (kind != FVM_TEMPLATE_POISSON && kind != FVM_TEMPLATE_MEAN_EXIT_TIME)
        fail(FVM_ERR_INVALID_ARGUMENT, "steady solves apply to PoissonsEquation / MeanExitTimeProblem templates");
    const fvm_mesh* m = prob->mesh;
    const SellPattern& pat = m->pat;
    const int64_t n = m->np;
    // 1. B on the mesh pattern (internal order): fixed rows are identity rows, columns of fixed
    //    rows move into the right-hand side, free rows are scaled by -V
    std::vector<int8_t> fixed(n, 0);
    for (int64_t v = 0; v < n; ++v) {
        int32_t r = m->iperm[v];
        fixed[r] = (prob->code[v] == FVM_VERTEX_DIRICHLET || !m->has_vertex[v]) ? 1 : 0;
    }
    std::vector<double> xfix(n, 0.0), rhs(n, 0.0), Vr(n, 0.0);
    for (int64_t r = 0; r < n; ++r) {
        Vr[r] = m->vol[m->perm[r]];
        if (fixed[r]) xfix[r] = b[r];
    }
    std::vector<int64_t> rp(n + 1, 0);  // CSR of B, internal order, vanishing entries dropped
    std::vector<int32_t> cc;
    std::vector<double> cv;
    cc.reserve(pat.nnz);
    cv.reserve(pat.nnz);
    for (int64_t r = 0; r < n; ++r) {
        double acc = b[r];
        for (int64_t q = pat.rowptr[r]; q < pat.rowptr[r + 1]; ++q) {
            const int32_t c = pat.csr_col[q];
            const double a = val[pat.csr_slot[q]];
            double bv;
            if (fixed[r]) {
                bv = c == r ? 1.0 : 0.0;
            } else if (fixed[c]) {
                acc -= a * b[c];
                bv = 0.0;
            } else {
                bv = -Vr[r] * a;
            }
            if (bv != 0.0 || c == r) {
                cc.push_back(c);
                cv.push_back(bv);
            }
        }
        rp[r + 1] = (int64_t)cc.size();
        rhs[r] = fixed[r] ? 0.0 : -Vr[r] * acc;
    }
    // 2. solver order: rows sorted by length, longest first, within windows of the mesh order
    std::vector<int32_t> sig(n);  // solver row -> internal row
    for (int64_t r = 0; r < n; ++r) sig[r] = (int32_t)r;
    for (int64_t w0 = 0; w0 < n; w0 += kSteadyWindow) {
        const int64_t w1 = std::min<int64_t>(n, w0 + kSteadyWindow);
        std::stable_sort(sig.begin() + w0, sig.begin() + w1, [&](int32_t x, int32_t y) {
            return rp[x + 1] - rp[x] > rp[y + 1] - rp[y];
        });
    }
    std::vector<int32_t> sinv(n);
    for (int64_t r = 0; r < n; ++r) sinv[sig[r]] = (int32_t)r;
    spat.nrows = n;
    spat.rowptr.assign(n + 1, 0);
    spat.csr_col.resize(cc.size());
    std::vector<double> csr_val(cc.size());
    {
        std::vector<std::pair<int32_t, double>> row;
        for (int64_t r2 = 0; r2 < n; ++r2) {
            const int32_t r = sig[r2];
            row.clear();
            for (int64_t q = rp[r]; q < rp[r + 1]; ++q) row.emplace_back(sinv[cc[q]], cv[q]);
            std::sort(row.begin(), row.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
            const int64_t o = spat.rowptr[r2];
            for (size_t k = 0; k < row.size(); ++k) {
                spat.csr_col[o + (int64_t)k] = row[k].first;
                csr_val[o + (int64_t)k] = row[k].second;
            }
            spat.rowptr[r2 + 1] = o + (int64_t)row.size();
        }
    }
    finalize_sell(spat, n);
    sperm.resize(n);
    for (int64_t r2 = 0; r2 < n; ++r2) sperm[r2] = m->perm[sig[r2]];
    // 3. values and per-row data in solver order
    std::vector<double> Bv(spat.nslots, 0.0), invD(n, 1.0), rs(n, 0.0), rhs2(n), xfix2(n), invV(n);
    std::vector<float> Bv32(spat.nslots, 0.0f), rs32(n), invD32(n), invV32(n);
    std::vector<int8_t> fixed2(n);
    double asym = 0, scale = 0, gersh = 1.0, bn = 0;
    for (int64_t r2 = 0; r2 < n; ++r2) {
        CompensatedSum sum;
        double row_abs = 0;
        for (int64_t q = spat.rowptr[r2]; q < spat.rowptr[r2 + 1]; ++q) {
            const double v = csr_val[q];
            Bv[spat.csr_slot[q]] = v;
            Bv32[spat.csr_slot[q]] = (float)v;
            sum.add(v);
            row_abs += std::fabs(v);
            scale = std::max(scale, std::fabs(v));
            if (spat.csr_col[q] == r2) invD[r2] = v != 0 ? 1.0 / v : 1.0;
        }
        rs[r2] = sum.value();
        const int32_t r = sig[r2];
        fixed2[r2] = fixed[r];
        rhs2[r2] = rhs[r];
        xfix2[r2] = xfix[r];
        invV[r2] = fixed[r] ? 0.0 : 1.0 / Vr[r];
        if (!fixed[r] && !(invD[r2] > 0)) fail(FVM_ERR_INVALID_ARGUMENT, "steady operator has a non-positive diagonal");
        gersh = std::max(gersh, row_abs * std::fabs(invD[r2]));
        rs32[r2] = (float)rs[r2];
        invD32[r2] = (float)invD[r2];
        invV32[r2] = (float)invV[r2];
    }
    for (int64_t r2 = 0; r2 < n; ++r2)  // symmetry of B
        for (int64_t q = spat.rowptr[r2]; q < spat.rowptr[r2 + 1]; ++q) {
            const int32_t c = spat.csr_col[q];
            if (c == r2) continue;
            const int64_t t = spat.find_csr(c, (int32_t)r2);
            asym = std::max(asym, std::fabs(csr_val[q] - (t >= 0 ? csr_val[t] : 0.0)));
        }
    for (int64_t r = 0; r < n; ++r) bn += b[r] * b[r];
    symmetric = asym <= 1e-12 * std::max(scale, 1e-300) ? 1 : 0;
    cheb_gershgorin = gersh;
    bnorm = std::sqrt(bn);
    d_sperm.upload(sperm);
    d_bval64.upload(Bv);
    d_bval32.upload(Bv32);
    d_brow64.upload(rs);
    d_brow32.upload(rs32);
    d_bdiag_inv64.upload(invD);
    d_bdiag_inv32.upload(invD32);
    d_rhs_red.upload(rhs2);
    d_xfix.upload(xfix2);
    d_invV_free64.upload(invV);
    d_invV_free32.upload(invV32);
    d_fixed_mask.upload(fixed2);
    steady_ready = true;
}

namespace {

struct Solver {
    fvm_template* T;
    int64_t n;
    cudaStream_t s;
    SpmvArgs A;
    unsigned nb, nbs;  // blocks for vector kernels, for SpMV kernels (a row / a slice per thread / warp)
    unsigned sms = 1;  // multiprocessors: the one-wave grids of the reducing vector kernels
    DBuf ws;
    KState* st;
    double* part;
    double* z64;   // solution of the reduced system (free rows), FP64
    double* r64;   // certified residual, FP64
    void* vec;     // typed work vectors

    Solver(fvm_template* t, cudaStream_t st_) : T(t), n(t->spat.nrows), s(st_) {
        const SellPattern& P = t->spat;
        A.slice_ptr = P.d_slice_ptr.as<int64_t>();
        A.width = P.d_width.as<int32_t>();
        A.col = P.d_col.as<int32_t>();
        A.n = n;
        A.nslices = P.nslices;
        nb = blocks_for(n);
        nbs = (unsigned)((P.nslices * 32 + kRedBlock - 1) / kRedBlock);
        int dev = 0, c = 1;
        FVM_CUDA(cudaGetDevice(&dev));
        FVM_CUDA(cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev));
        sms = (unsigned)std::max(1, c);
    }
    // one wave of the reducing vector kernels (eight blocks per SM)
    unsigned rgrid() const { return std::max(1u, std::min(nb, 8 * sms)); }
};

template <class T>
struct Vecs {
    T *x, *r, *p, *Ap, *rhat, *phat, *shat, *t;
    T *w, *d0, *d1;                    // Chebyshev work vectors
    const float* f32vals = nullptr;    // FP32-stored operator of the preconditioner (FVM_SOLVE_FP32_PRECOND)
    // the FP32 polynomial of the mixed mode: FP32 operator in difference form (values, row
    // sums), FP32 Jacobi scaling; its work vectors are FP32 views of w, d0, d1
    const float *pc_val = nullptr, *pc_rowsum = nullptr, *pc_invD = nullptr;
};

constexpr int kWorkVectors = 11;  // vectors of the Krylov type

// y = p(D^-1 B) D^-1 r (Chebyshev preconditioner; see cheb_plan)
template <class V, class T>
static void cheb_apply(const Solver& S, const ChebPlan& P, const V* val, const T* rowsum, const T* invD, const T* r,
                       T* y, Vecs<T>& v, int gate) {
    if constexpr (std::is_same_v<T, double>) {
        if (v.pc_val) {  // mixed: the polynomial in FP32 (values, vectors, difference-form products)
            float* w32 = reinterpret_cast<float*>(v.w);
            float* y32 = w32 + S.n;
            float* din = reinterpret_cast<float*>(v.d0);
            float* dout = reinterpret_cast<float*>(v.d1);
            cheb_init_mixed_kernel<<<S.nb, kRedBlock, 0, S.s>>>(r, v.pc_invD, w32, din, y32, P.degree == 1 ? y : nullptr,
                                                                (float)P.inv_theta, S.n, S.st, gate);
            for (int j = 1; j < P.degree; ++j) {
                if (j + 1 < P.degree)
                    cheb_step_kernel<float, float, false><<<S.nbs, kRedBlock, 0, S.s>>>(
                        S.A, v.pc_val, v.pc_rowsum, din, v.pc_invD, w32, dout, y32, (float)P.c1[j], (float)P.c2[j],
                        S.st, gate);
                else
                    cheb_step_kernel<float, float, true><<<S.nbs, kRedBlock, 0, S.s>>>(
                        S.A, v.pc_val, v.pc_rowsum, din, v.pc_invD, w32, dout, y32, (float)P.c1[j], (float)P.c2[j],
                        S.st, gate, y);
                std::swap(din, dout);
            }
            return;
        }
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

// One Krylov solve of the reduced system B z = rhs from the current z64, in iteration type T:
//   FP64 (T = double, explicit FP64 products): the iteration updates a correction x from the
//     certified residual and runs until its recurrence residual reaches rtol; x is then folded
//     into z64 and the certified residual decides (a reliable update: continue from the
//     certified residual while it is above rtol).  pc32: the Chebyshev preconditioner is
//     evaluated in FP32 (the mixed mode with the Chebyshev preconditioner);
//   FP32 cycles (T = float, FP32 values, vectors and products in difference form; the mixed
//     mode with the Jacobi preconditioner): each refinement cycle solves B x = s r for the
//     certified residual r scaled to unit RMS, from x = 0, until the FP32 recurrence residual
//     has dropped by inner_reduction; z64 += x / s.
// The stopping test is always the certified FP64 residual ||b - A x|| / ||b||.
template <class V, class T>
static void run_krylov(fvm_template* Tm, Solver& S, bool cg, bool mixed, const fvm_solver_options& o,
                       fvm_solver_stats& stats, bool pc32 = false) {
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
    v.f32vals = (o.mode == FVM_SOLVE_FP32_PRECOND && !mixed) ? Tm->d_bval32.as<float>() : nullptr;
    if (pc32) {
        v.pc_val = Tm->d_bval32.as<float>();
        v.pc_rowsum = Tm->d_brow32.as<float>();
        v.pc_invD = Tm->d_bdiag_inv32.as<float>();
    }
    const bool cheb = o.precond == FVM_PRECOND_CHEBYSHEV;
    const ChebPlan plan = cheb ? cheb_plan(Tm->cheb_gershgorin, o.cheb_degree > 0 ? o.cheb_degree : 4) : ChebPlan{};
    T* zc = v.rhat;  // CG's preconditioned residual (BiCGStab's rhat is unused by CG)
    FVM_CUDA(cudaMemsetAsync(v.x, 0, sizeof(T) * n, s));
    const double tol = o.rtol * Tm->bnorm;
    const double tol2 = tol * tol;
    const int64_t maxit = o.max_iters > 0 ? o.max_iters : 1000000;
    const bool fp32pc = o.mode == FVM_SOLVE_FP32_PRECOND && !mixed;
    double red = o.inner_reduction > 0 && o.inner_reduction < 1 ? o.inner_reduction : 1e-3;
    KState h{};
    auto set_tol = [&](double t2) {
        FVM_CUDA(cudaMemcpyAsync(&S.st->tol2, &t2, sizeof(double), cudaMemcpyHostToDevice, s));
    };
    // FP32 cycles stop when their recurrence residual grows 1e4-fold.  Any cycle in which FP32
    // rounding enters (FP32 cycles, or the FP32 polynomial, which varies by rounding from one
    // application to the next) also stops when its recurrence residual climbs 1e3-fold above
    // the lowest it reached, and the iteration restarts from the certified residual.
    // (BiCGStab's residual is not monotone: excursions of a few hundred above the running
    // minimum are part of normal convergence.)
    auto set_div = [&](double rn0) {
        const double inf = std::numeric_limits<double>::infinity();
        const double d[3] = {mixed ? 1e8 * rn0 * rn0 : inf, (mixed || pc32) ? 1e6 : inf, inf};
        FVM_CUDA(cudaMemcpyAsync(&S.st->div2, d, sizeof d, cudaMemcpyHostToDevice, s));
    };
    auto read_state = [&]() {
        FVM_CUDA(cudaMemcpyAsync(&h, S.st, sizeof(KState), cudaMemcpyDeviceToHost, s));
        FVM_CUDA(cudaStreamSynchronize(s));
    };
    double scale = 1.0;  // inner units = scale * FP64 units (FP32 cycles)
    // certified residual from z64; sets the iteration's r (and p on a restart), rz, rn2;
    // returns the FP64 residual norm in the reference operator's norm
    auto true_residual = [&](bool set_p) {
        set_tol(tol2);
        const bool poly_cg = cg && cheb;
        double rn_true;
        if constexpr (std::is_same_v<T, double>) {
            cert_residual_kernel<<<S.nbs, kRedBlock, 0, s>>>(S.A, Tm->d_bval64.as<double>(), Tm->d_brow64.as<double>(),
                                                             S.z64, Tm->d_rhs_red.as<double>(),
                                                             Tm->d_invV_free64.as<double>(), invD, v.r, v.p,
                                                             set_p && !poly_cg ? 1 : 0, S.part);
            finalize_kernel<<<1, kFinThreads, 0, s>>>(S.part, (int)S.nbs, 3, kFinResidual, S.st);
            FVM_CUDA(cudaGetLastError());
            read_state();
            rn_true = std::sqrt(h.rn2);
        } else {
            cert_residual_kernel<<<S.nbs, kRedBlock, 0, s>>>(S.A, Tm->d_bval64.as<double>(), Tm->d_brow64.as<double>(),
                                                             S.z64, Tm->d_rhs_red.as<double>(),
                                                             Tm->d_invV_free64.as<double>(),
                                                             Tm->d_bdiag_inv64.as<double>(), S.r64, nullptr, 0, S.part);
            finalize_kernel<<<1, kFinThreads, 0, s>>>(S.part, (int)S.nbs, 3, kFinResidual, S.st);
            FVM_CUDA(cudaGetLastError());
            read_state();
            rn_true = std::sqrt(h.rn2);
            const double rms = std::sqrt(h.dot[2] / std::max<int64_t>(1, n));
            scale = rms > 0 ? 1.0 / rms : 1.0;
            set_tol(tol2 * scale * scale);
            scale_residual_kernel<<<S.rgrid(), kRedBlock, 0, s>>>(S.r64, (float*)v.r, (float*)v.p,
                                                                  set_p && !poly_cg ? 1 : 0, (const float*)invD,
                                                                  (const float*)invV, scale, n, S.part, S.st);
        }
        if (poly_cg) {  // rz = r . M^-1 r, and p = M^-1 r on a restart
            cheb_apply<V, T>(S, plan, val, rowsum, invD, v.r, zc, v, 0);
            cg_rz_kernel<T><<<S.rgrid(), kRedBlock, 0, s>>>(v.r, zc, v.p, set_p ? 1 : 0, n, S.part, S.st, 0);
        }
        FVM_CUDA(cudaGetLastError());
        read_state();
        ++stats.refinements;
        return rn_true;
    };
    double rn = true_residual(true);
    const int chunk = 16;
    int64_t it = 0;
    int stagnation = 0, rejects = 0;
    double best = rn;
    double red_cur = red;
    static const bool trace = std::getenv("FVM_SOLVER_TRACE") != nullptr;
    static const bool trace_chunks = trace && std::getenv("FVM_SOLVER_TRACE")[0] == '2';
    // iteration target (iteration units): an FP32 cycle runs until its recurrence residual has
    // dropped by red_cur (never below rtol); the FP64 iteration runs to rtol
    auto inner_tol2 = [&]() {
        const double t = mixed ? std::max(tol, red_cur * rn) * scale : tol;
        return t * t;
    };
    bool need_start = !cg;
    bool cycle_start = true;  // the growth guard's running minimum restarts with each cycle
    while (rn > tol) {
        if (it >= maxit) break;
        if (cycle_start) {
            set_tol(inner_tol2());
            set_div(std::sqrt(h.rn2));
            cycle_start = false;
        }
        if (need_start) {
            // BiCGStab restart from the current residual: rhat = r, p = v = 0, rho = r.r
            bicg_start_kernel<T><<<S.rgrid(), kRedBlock, 0, s>>>(v.rhat, v.r, v.p, v.Ap, n, S.part, S.st);
            need_start = false;
        }
        for (int c = 0; c < chunk; ++c) {
            if (cg) {
                cg_spmv_kernel<V, T><<<S.nbs, kRedBlock, 0, s>>>(S.A, val, rowsum, v.p, v.Ap, S.part, S.st);
                finalize_kernel<<<1, kFinThreads, 0, s>>>(S.part, (int)S.nbs, 1, kFinCgAlpha, S.st);
                if (cheb) {
                    cg_update_kernel<T, false><<<S.rgrid(), kRedBlock, 0, s>>>(v.x, v.r, v.p, v.Ap, invD, invV, n,
                                                                               S.part, S.st);
                    cheb_apply<V, T>(S, plan, val, rowsum, invD, v.r, zc, v, 1);
                    cg_rz_kernel<T><<<S.rgrid(), kRedBlock, 0, s>>>(v.r, zc, v.p, 0, n, S.part, S.st, 1);
                    cg_pupdate_z_kernel<T><<<S.nb, kRedBlock, 0, s>>>(v.p, zc, n, S.st);
                } else {
                    cg_update_kernel<T, true><<<S.rgrid(), kRedBlock, 0, s>>>(v.x, v.r, v.p, v.Ap, invD, invV, n,
                                                                              S.part, S.st);
                    cg_pupdate_kernel<T><<<S.nb, kRedBlock, 0, s>>>(v.p, v.r, invD, n, S.st);
                }
            } else {
                bicg_p_kernel<T><<<S.nb, kRedBlock, 0, s>>>(v.p, v.phat, v.r, v.Ap, invD, n, S.st);
                if (cheb) cheb_apply<V, T>(S, plan, val, rowsum, invD, v.p, v.phat, v, 0);  // phat = M^-1 p
                bicg_v_kernel<V, T><<<S.nbs, kRedBlock, 0, s>>>(S.A, val, rowsum, v.phat, v.Ap, v.rhat, S.part, S.st);
                finalize_kernel<<<1, kFinThreads, 0, s>>>(S.part, (int)S.nbs, 1, kFinBicgAlpha, S.st);
                bicg_s_kernel<T><<<S.nb, kRedBlock, 0, s>>>(v.r, v.shat, v.Ap, invD, n, S.st);
                if (cheb) cheb_apply<V, T>(S, plan, val, rowsum, invD, v.r, v.shat, v, 0);  // shat = M^-1 s
                bicg_t_kernel<V, T><<<S.nbs, kRedBlock, 0, s>>>(S.A, val, rowsum, v.shat, v.t, v.r, S.part, S.st);
                finalize_kernel<<<1, kFinThreads, 0, s>>>(S.part, (int)S.nbs, 2, kFinBicgOmega, S.st);
                bicg_x_kernel<T><<<S.rgrid(), kRedBlock, 0, s>>>(v.x, v.r, v.phat, v.shat, v.t, v.rhat, invV, n, S.part,
                                                                 S.st);
            }
        }
        FVM_CUDA(cudaGetLastError());
        read_state();
        it += chunk;  // iterations issued (kernels after convergence return at once)
        if (trace_chunks)
            std::fprintf(stderr, "[fvm solver] it=%lld recurrence %.3e alpha %.3e omega %.3e rho %.3e\n", (long long)it,
                         std::sqrt(h.rn2) / scale / Tm->bnorm, h.alpha, h.omega, h.rho);
        if (!h.done) continue;
        // reliable update: fold the correction into the FP64 solution, recompute the residual
        const double scale_used = scale;
        accumulate_kernel<T><<<S.nb, kRedBlock, 0, s>>>(S.z64, v.x, 1.0 / scale_used, n);
        // CG restarts from every certified residual (its recurrence and the FP64 products drift
        // apart over thousands of iterations, and the old direction no longer matches the new
        // residual); BiCGStab keeps its recurrences unless it broke down
        bool restart = h.breakdown != 0 || mixed || cg;
        const double rec = std::sqrt(h.rn2) / scale_used;
        const int brk = h.breakdown;
        double rn_new = true_residual(restart);
        if (trace)
            std::fprintf(stderr, "[fvm solver] %s %s it=%lld rn=%.3e (recurrence %.3e) breakdown=%d\n",
                         cg ? "cg" : "bicgstab",
                         mixed ? "fp32-cycles" : pc32 ? "mixed" : fp32pc ? "fp32-precond" : "fp64", (long long)it,
                         rn_new / Tm->bnorm, rec / Tm->bnorm, brk);
        if (!(rn_new < rn)) {
            // the correction raised the certified residual (inner-precision drift or a
            // breakdown): undo it, restart from the FP64 residual with a milder inner reduction
            accumulate_kernel<T><<<S.nb, kRedBlock, 0, s>>>(S.z64, v.x, -1.0 / scale_used, n);
            rn_new = true_residual(true);
            restart = true;
            red_cur = std::min(0.5, red_cur * 4);
            // an FP32 polynomial that made a cycle diverge would do so again from the same
            // state: hand over to the FP64 polynomial (the caller's fallback)
            if (++rejects > 6 || pc32) break;
        }
        FVM_CUDA(cudaMemsetAsync(v.x, 0, sizeof(T) * n, s));
        rn = rn_new;
        cycle_start = true;
        if (!cg) {
            if (restart) {
                need_start = true;
            } else {
                // keep the BiCGStab recurrences; only rho (and the pending beta) follow the new r
                bicg_rho_fix_kernel<T><<<S.rgrid(), kRedBlock, 0, s>>>(v.rhat, v.r, n, S.part, S.st);
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
        const int64_t n = Tm->spat.nrows;
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
        // Krylov vectors sized for FP64 even for FP32 cycles: a stalled run finishes in FP64
        // (run_krylov<double, double>) on the same workspace
        size_t elem = sizeof(double);
        size_t bytes = sizeof(KState) + sizeof(double) * 8 * (size_t)std::max(S.nb, S.nbs) + sizeof(double) * 4 * n +
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
        S.r64 = S.z64 + 3 * n;
        w += sizeof(double) * 4 * n;
        S.vec = w;
        FVM_CUDA(cudaMemsetAsync(S.st, 0, sizeof(KState), s));
        // initial guess -> z (free rows), solver order
        if (loc == FVM_PTR_HOST)
            FVM_CUDA(cudaMemcpyAsync(xref, x, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        else
            FVM_CUDA(cudaMemcpyAsync(xref, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        launch_permute_in(Tm->d_sperm.as<int32_t>(), xref, xint, n, s);
        split_kernel<<<S.nb, kRedBlock, 0, s>>>(S.z64, xint, Tm->d_xfix.as<double>(), Tm->d_fixed_mask.as<int8_t>(), n);
        cudaEvent_t e0, e1;
        FVM_CUDA(cudaEventCreate(&e0));
        FVM_CUDA(cudaEventCreate(&e1));
        FVM_CUDA(cudaEventRecord(e0, s));
        int status = FVM_OK;
        std::string msg;
        try {
            if (mixed && opt->precond == FVM_PRECOND_CHEBYSHEV) {
                // FP64 Krylov iteration; its preconditioner, the Chebyshev polynomial, in FP32.
                // CG takes the slightly varying polynomial in its stride; BiCGStab's
                // bi-orthogonality can lose it on large non-symmetric systems, and a diverging
                // cycle hands over to the FP64 polynomial
                try {
                    run_krylov<double, double>(Tm, S, cg, false, *opt, st, true);
                } catch (const Error& e) {
                    if (e.code != FVM_ERR_NOT_CONVERGED) throw;
                    st.fallback_fp64 = 1;
                    fvm_solver_options o64 = *opt;
                    o64.mode = FVM_SOLVE_FP64;
                    run_krylov<double, double>(Tm, S, cg, false, o64, st);
                }
            } else if (mixed) {
                try {
                    run_krylov<float, float>(Tm, S, cg, true, *opt, st);
                } catch (const Error& e) {
                    if (e.code != FVM_ERR_NOT_CONVERGED) throw;
                    // the FP32 cycles stalled: finish in FP64 from the current solution
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
        launch_permute_out(Tm->d_sperm.as<int32_t>(), xint, xref, n, s);
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
