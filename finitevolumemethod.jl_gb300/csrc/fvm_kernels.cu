// Device kernels of libfvmgpu (sm_103a).  Every kernel here is HBM- or FP64-issue-bound
// gather/scatter/stream work; none is a dense contraction, so no tensor-core path exists.
#include "fvm_internal.h"
#include "fvm_sell.cuh"
#include "fvm_stream.cuh"
#include "fvm_tma.cuh"

#include <algorithm>
#include <atomic>
#include <vector>

namespace fvm {

static inline unsigned grid_for(int64_t threads, int block) { return (unsigned)((threads + block - 1) / block); }

// ---------------------------------------------------------------------------------------
// Sliced-ELL operators (one warp per 32-row slice; see fvm_sell.cuh).
//   explicit (templates, A u + b):  y_i = rowscale_i * sum_j A_ij x_j + b_i + q_i x_i^2
//   difference form (generic RHS):  y_i = rowscale_i * sum_{j != i} K_ij (x_j - x_i)
//                                         + d_i x_i + b_i + q_i x_i^2
// In the difference form padding slots point at the row itself (x_i - x_i = 0).  FP32
// variants gather an FP32 copy of x (converted once per row by to_f32_kernel: gathering
// doubles would spend an FP64-pipe conversion per entry), accumulate in FP32 and apply
// rowscale, d, b, q in FP64 with the row's FP64 value.
// ---------------------------------------------------------------------------------------
struct SellArgs {
    const int64_t* slice_ptr;
    const int32_t* width;
    const int32_t* col;
    const void* val;
    const void* xg;   // gathered x (double or float)
    const double* x;  // the row's own FP64 value
    double* y;
    const double* rowscale;
    const double* d;
    const double* b;
    const double* q;
    int64_t nrows, nslices;
};

template <class V, class Acc, class X, bool DIFF, int MAXW>
__global__ void __launch_bounds__(256) sell_kernel(SellArgs a) {
    const int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= a.nslices) return;
    const int64_t r = s * kSlice + lane;
    const int64_t rc = r < a.nrows ? r : a.nrows - 1;
    const X* xg = (const X*)a.xg;
    Acc xa = DIFF ? (Acc)__ldg(&xg[rc]) : Acc(0);
    Acc acc = sell_row_product<V, Acc, X, DIFF, MAXW>(a.slice_ptr, a.width, a.col, (const V*)a.val, xg, xa, s, lane);
    if (r >= a.nrows) return;
    double out = (double)acc;
    if (a.rowscale) out *= a.rowscale[r];
    if (a.d || a.q) {
        const double xr = a.x[r];
        if (a.d) out += a.d[r] * xr;
        if (a.q) out += a.q[r] * xr * xr;
    }
    if (a.b) out += a.b[r];
    a.y[r] = out;
}

// ---------------------------------------------------------------------------------------
// Streamed sliced-ELL operator (fvm_stream.cuh) with the RHS / template epilogue:
//   y_i = rowscale_i * (sum) + d_i x_i + q_i x_i^2 + b_i
// ---------------------------------------------------------------------------------------
__device__ unsigned g_dev_error = 0;

// Consumer stage-wait limit and producer delay of the streamed kernels (fault-path testing;
// fvm_test_set_stream_waits).  0 = the defaults: kWaitLimitNs and no delay.
static std::atomic<unsigned long long> g_stream_wait_ns{0}, g_producer_delay_ns{0};
static unsigned long long stream_wait_ns() {
    const unsigned long long w = g_stream_wait_ns.load();
    return w ? w : kWaitLimitNs;
}
}  // namespace fvm

extern "C" int fvm_test_set_stream_waits(int64_t consumer_wait_ns, int64_t producer_delay_ns) {
    // bounded: a delay never exceeds 10 ms, a wait limit never goes below 100 ns
    if (producer_delay_ns < 0 || producer_delay_ns > 10000000 || consumer_wait_ns < 0 ||
        (consumer_wait_ns != 0 && consumer_wait_ns < 100)) {
        fvm::set_last_error("fvm_test_set_stream_waits: delay outside [0, 10 ms] or wait limit below 100 ns");
        return FVM_ERR_INVALID_ARGUMENT;
    }
    fvm::g_stream_wait_ns.store((unsigned long long)consumer_wait_ns);
    fvm::g_producer_delay_ns.store((unsigned long long)producer_delay_ns);
    return FVM_OK;
}

namespace fvm {

unsigned* device_error_word() {
    static unsigned* p = nullptr;
    if (!p) FVM_CUDA(cudaGetSymbolAddress((void**)&p, g_dev_error));
    return p;
}

struct RhsEpilogue {
    static constexpr int NP = 0;
    static constexpr bool kOwnX = false;
    struct Pre {};
    __device__ Pre load(int64_t) const { return {}; }
    const double* x;  // the row's own FP64 value
    double* y;
    const double* rowscale;
    const double* d;
    const double* b;
    const double* q;
    __device__ bool skip() const { return false; }
    template <class Acc>
    __device__ void row(int64_t r, Acc acc, Acc, const Pre&, double*) const {
        double out = (double)acc;
        if (rowscale) out *= rowscale[r];
        if (d || q) {
            const double xr = x[r];
            if (d) out += d[r] * xr;
            if (q) out += q[r] * xr * xr;
        }
        if (b) out += b[r];
        y[r] = out;
    }
};

template <class V, class Acc, class X, bool DIFF>
static void launch_sell(const SellPattern& p, const V* val, const X* xg, const double* x, double* y,
                        const double* rowscale, const double* d, const double* b, const double* q, cudaStream_t s) {
    if (p.nslices == 0) return;
    if (p.maxw <= 16) {
        StreamArgs a{p.d_slice_ptr.as<int64_t>(), p.d_col.as<int32_t>(), val, xg, device_error_word(),
                     p.nrows, p.nslices, 0, 0, 0, stream_wait_ns(), g_producer_delay_ns.load()};
        const RhsEpilogue e{x, y, rowscale, d, b, q};
        // exact widths of the common vertex degrees: no predicated-off slot costs an FP64 issue
        if (p.maxw <= 4)
            launch_stream_any<V, Acc, X, DIFF, 4>(a, p.slice_ptr, e, s);
        else if (p.maxw <= 6)
            launch_stream_any<V, Acc, X, DIFF, 6>(a, p.slice_ptr, e, s);
        else if (p.maxw <= 7)
            launch_stream_any<V, Acc, X, DIFF, 7>(a, p.slice_ptr, e, s);
        else if (p.maxw <= 8)
            launch_stream_any<V, Acc, X, DIFF, 8>(a, p.slice_ptr, e, s);
        else if (p.maxw <= 12)
            launch_stream_any<V, Acc, X, DIFF, 12>(a, p.slice_ptr, e, s);
        else
            launch_stream_any<V, Acc, X, DIFF, 16>(a, p.slice_ptr, e, s);
        return;
    }
    SellArgs a{p.d_slice_ptr.as<int64_t>(), p.d_width.as<int32_t>(), p.d_col.as<int32_t>(), val, xg, x, y, rowscale,
               d, b, q, p.nrows, p.nslices};
    unsigned grid = grid_for(p.nslices * 32, 256);
    sell_kernel<V, Acc, X, DIFF, 0><<<grid, 256, 0, s>>>(a);
}

unsigned take_device_error() {
    unsigned e = 0;
    FVM_CUDA(cudaMemcpyFromSymbol(&e, g_dev_error, sizeof e));
    if (e) {
        const unsigned zero = 0;
        FVM_CUDA(cudaMemcpyToSymbol(g_dev_error, &zero, sizeof zero));
    }
    return e;
}

void launch_sell_apply64(const SellPattern& p, const double* val, const double* x, double* y, const double* rowscale,
                         const double* b, const double* q, cudaStream_t s) {
    launch_sell<double, double, double, false>(p, val, x, x, y, rowscale, nullptr, b, q, s);
}

void launch_sell_apply32(const SellPattern& p, const float* val, const float* x32, const double* x, double* y,
                         const double* rowscale, const double* b, const double* q, cudaStream_t s) {
    launch_sell<float, float, float, false>(p, val, x32, x, y, rowscale, nullptr, b, q, s);
}

void launch_sell_diff64(const SellPattern& p, const double* val, const double* x, double* y, const double* rowscale,
                        const double* d, const double* b, const double* q, cudaStream_t s) {
    launch_sell<double, double, double, true>(p, val, x, x, y, rowscale, d, b, q, s);
}

void launch_sell_diff32(const SellPattern& p, const float* val, const float* x32, const double* x, double* y,
                        const double* rowscale, const double* d, const double* b, const double* q, cudaStream_t s) {
    launch_sell<float, float, float, true>(p, val, x32, x, y, rowscale, d, b, q, s);
}

__global__ void to_f32_kernel(const double* __restrict__ x, float* __restrict__ y, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = (float)x[i];
}
void launch_to_f32(const double* x, float* y, int64_t n, cudaStream_t s) {
    if (n) to_f32_kernel<<<grid_for(n, 256), 256, 0, s>>>(x, y, n);
}

// ---------------------------------------------------------------------------------------
// Permutation between the caller's numbering and the internal (Hilbert) numbering.
// ---------------------------------------------------------------------------------------
__global__ void permute_in_kernel(const int32_t* __restrict__ perm, const double* __restrict__ xref,
                                  double* __restrict__ xint, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) xint[i] = __ldg(&xref[__ldg(&perm[i])]);
}
__global__ void permute_out_kernel(const int32_t* __restrict__ perm, const double* __restrict__ xint,
                                   double* __restrict__ xref, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) xref[__ldg(&perm[i])] = xint[i];
}
void launch_permute_in(const int32_t* perm, const double* xref, double* xint, int64_t n, cudaStream_t s) {
    if (n) permute_in_kernel<<<grid_for(n, 256), 256, 0, s>>>(perm, xref, xint, n);
}
void launch_permute_out(const int32_t* perm, const double* xint, double* xref, int64_t n, cudaStream_t s) {
    if (n) permute_out_kernel<<<grid_for(n, 256), 256, 0, s>>>(perm, xint, xref, n);
}

// The same permutations with the caller-numbered side walked in order: the form for arrays in
// pinned host memory, read or written by the kernel over the host link in whole lines.
__global__ void permute_in_seq_kernel(const int32_t* __restrict__ iperm, const double* __restrict__ xref,
                                      double* __restrict__ xint, int64_t n) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) xint[__ldg(&iperm[j])] = xref[j];
}
__global__ void permute_out_seq_kernel(const int32_t* __restrict__ iperm, const double* __restrict__ xint,
                                       double* __restrict__ xref, int64_t n) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) xref[j] = xint[__ldg(&iperm[j])];
}
void launch_permute_in_seq(const int32_t* iperm, const double* xref, double* xint, int64_t n, cudaStream_t s) {
    if (n) permute_in_seq_kernel<<<grid_for(n, 256), 256, 0, s>>>(iperm, xref, xint, n);
}
void launch_permute_out_seq(const int32_t* iperm, const double* xint, double* xref, int64_t n, cudaStream_t s) {
    if (n) permute_out_seq_kernel<<<grid_for(n, 256), 256, 0, s>>>(iperm, xint, xref, n);
}

// nsave snapshots at once, caller side in order: xref[k][j] = xint[k][iperm[j]]
__global__ void permute_out_snapshots_kernel(const int32_t* __restrict__ iperm, const double* __restrict__ xint,
                                             double* __restrict__ xref, int64_t n, int64_t total) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = i / n, j = i - k * n;
        xref[i] = xint[k * n + __ldg(&iperm[j])];
    }
}
void launch_permute_out_snapshots(const int32_t* iperm, const double* xint, double* xref, int64_t n, int64_t nsave,
                                  cudaStream_t s) {
    const int64_t total = n * nsave;
    if (total == 0) return;
    const unsigned grid = (unsigned)std::min<int64_t>(grid_for(total, 256), 152 * 16);
    permute_out_snapshots_kernel<<<grid, 256, 0, s>>>(iperm, xint, xref, n, total);
}

// Dirichlet update: u_i <- a(x_i, y_i) on the Dirichlet list (dirichlet.jl:20-26).
__global__ void dirichlet_kernel(const int32_t* __restrict__ idx, const double* __restrict__ val,
                                 double* __restrict__ u, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) u[idx[i]] = val[i];
}
void launch_dirichlet(const int32_t* idx, const double* val, double* u, int64_t n, cudaStream_t s) {
    if (n) dirichlet_kernel<<<grid_for(n, 256), 256, 0, s>>>(idx, val, u, n);
}

// Time-dependent values: v = v_static + sum_g tau_g(t) v_g, the tau_g evaluated on the host.
__global__ void time_b_kernel(const double* __restrict__ b, const double* __restrict__ tb, TimeTaus tt, int ntime,
                              double* __restrict__ out, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v = b ? b[i] : 0.0;
    for (int g = 0; g < ntime; ++g) v = fma(tt.tau[g], tb[g * n + i], v);
    out[i] = v;
}
void launch_time_b(const double* b, const double* tb, const TimeTaus& tt, int ntime, double* out, int64_t n,
                   cudaStream_t s) {
    if (n) time_b_kernel<<<grid_for(n, 256), 256, 0, s>>>(b, tb, tt, ntime, out, n);
}

__global__ void dirichlet_time_kernel(const int32_t* __restrict__ idx, const double* __restrict__ val,
                                      const double* __restrict__ tval, TimeTaus tt, int ntime, double* __restrict__ u,
                                      int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v = val[i];
    for (int g = 0; g < ntime; ++g) v = fma(tt.tau[g], tval[g * n + i], v);
    u[idx[i]] = v;
}
void launch_dirichlet_time(const int32_t* idx, const double* val, const double* tval, const TimeTaus& tt, int ntime,
                           double* u, int64_t n, cudaStream_t s) {
    if (n) dirichlet_time_kernel<<<grid_for(n, 256), 256, 0, s>>>(idx, val, tval, tt, ntime, u, n);
}

// ---------------------------------------------------------------------------------------
// Per-triangle flux kernel (generic fvm_eqs! for any device-coded form).
// One CTA per vertex tile; the CTA walks every triangle touching the tile (coalesced SoA
// streams), evaluates the three dual-edge fluxes, and accumulates the tile's du in shared
// memory; boundary half edges follow; then the tile's vertices are finalised in place
// (du/V + S, Dudt, Dirichlet / missing-vertex zero) and written once.
// ---------------------------------------------------------------------------------------
struct TriArgs {
    const int64_t* off;
    const int64_t* boff;
    const int32_t* ev;   // [3][nelem]
    const double* g;     // [6][nelem] geometric coefficients (DDEG>0)
    const double* ec;    // [6][nelem] folded coefficients (DDEG==0) or [3*(DDEG+1)][nelem] D polys
    const int32_t* bv;   // [3][nbelem]
    const double* bg;    // [3][nbelem] g_i, g_j, l_h
    const double* bc;    // [1 + 2(DDEG+1) + 6][nbelem]
    const int8_t* code;
    const double* invV;
    const double* vsrc;  // [3][np] or null
    const double* vdudt; // [3][np] or null
    const double* u;
    double* du;
    int64_t nelem, nbelem, np;
    int tv;
};

template <int DDEG>
__device__ __forceinline__ double dpoly(const double* c, int64_t stride, int64_t e, double x) {
    double r = __ldg(&c[e]);
    if (DDEG >= 1) {
        double c1 = __ldg(&c[stride + e]);
        if (DDEG >= 2) c1 += x * __ldg(&c[2 * stride + e]);
        r += x * c1;
    }
    return r;
}

template <int DDEG>
__global__ void __launch_bounds__(256) triangle_rhs_kernel(TriArgs a) {
    extern __shared__ double acc[];
    const int64_t tile = blockIdx.x;
    const int64_t v0 = tile * a.tv;
    for (int i = threadIdx.x; i < a.tv; i += blockDim.x) acc[i] = 0.0;
    __syncthreads();
    const int64_t N = a.nelem;
    const int64_t e0 = a.off[tile], e1 = a.off[tile + 1];
    for (int64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        int32_t va = __ldg(&a.ev[e]), vb = __ldg(&a.ev[N + e]), vc = __ldg(&a.ev[2 * N + e]);
        double ua = __ldg(&a.u[va]), ub = __ldg(&a.u[vb]), uc = __ldg(&a.u[vc]);
        double dac = ua - uc, dbc = ub - uc;
        double Q[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double* gc = DDEG == 0 ? a.ec : a.g;
            double G = __ldg(&gc[(2 * d) * N + e]) * dac + __ldg(&gc[(2 * d + 1) * N + e]) * dbc;
            if (DDEG == 0) {
                Q[d] = G;
            } else {
                // u at the dual-edge midpoint (5 p_a + 5 p_b + 2 p_c)/12 of edge d
                double us = d == 0 ? (5.0 * (ua + ub) + 2.0 * uc) / 12.0
                          : d == 1 ? (5.0 * (ub + uc) + 2.0 * ua) / 12.0
                                   : (5.0 * (uc + ua) + 2.0 * ub) / 12.0;
                Q[d] = dpoly<DDEG>(a.ec + (int64_t)(d * (DDEG + 1)) * N, N, e, us) * G;
            }
        }
        uint64_t la = (uint64_t)(va - v0), lb = (uint64_t)(vb - v0), lc = (uint64_t)(vc - v0);
        if (la < (uint64_t)a.tv) atomicAdd(&acc[la], Q[2] - Q[0]);
        if (lb < (uint64_t)a.tv) atomicAdd(&acc[lb], Q[0] - Q[1]);
        if (lc < (uint64_t)a.tv) atomicAdd(&acc[lc], Q[1] - Q[2]);
    }
    // boundary half edges (boundary_edge_contributions.jl:41-65)
    const int64_t NB = a.nbelem;
    const int nd = DDEG + 1;
    const int64_t b0 = a.boff[tile], b1 = a.boff[tile + 1];
    for (int64_t e = b0 + threadIdx.x; e < b1; e += blockDim.x) {
        int32_t vi = a.bv[e], vj = a.bv[NB + e], vk = a.bv[2 * NB + e];
        double ui = a.u[vi], uj = a.u[vj], uk = a.u[vk];
        double umi = (3.0 * ui + uj) / 4.0, umj = (ui + 3.0 * uj) / 4.0;
        double lh = a.bg[2 * NB + e];
        double Qi, Qj;
        if (a.bc[e] != 0.0) {  // Neumann: q.n = a(m, u(m))
            const double* n = a.bc + (int64_t)(1 + 2 * nd) * NB;
            Qi = (n[e] + umi * (n[NB + e] + umi * n[2 * NB + e])) * lh;
            Qj = (n[3 * NB + e] + umj * (n[4 * NB + e] + umj * n[5 * NB + e])) * lh;
        } else {
            double G = a.bg[e] * (ui - uk) + a.bg[NB + e] * (uj - uk);
            Qi = dpoly<DDEG>(a.bc + NB, NB, e, umi) * G;
            Qj = dpoly<DDEG>(a.bc + (int64_t)(1 + nd) * NB, NB, e, umj) * G;
        }
        uint64_t li = (uint64_t)(vi - v0), lj = (uint64_t)(vj - v0);
        if (li < (uint64_t)a.tv) atomicAdd(&acc[li], -Qi);
        if (lj < (uint64_t)a.tv) atomicAdd(&acc[lj], -Qj);
    }
    __syncthreads();
    // finalise (source_contributions.jl:33-47)
    for (int i = threadIdx.x; i < a.tv; i += blockDim.x) {
        int64_t v = v0 + i;
        if (v >= a.np) break;
        int c = a.code[v];
        double uu = a.u[v];
        double r = 0.0;
        if (c == FVM_VERTEX_FREE) {
            r = acc[i] * a.invV[v];
            if (a.vsrc) r += a.vsrc[v] + uu * (a.vsrc[a.np + v] + uu * a.vsrc[2 * a.np + v]);
        } else if (c == FVM_VERTEX_DUDT) {
            if (a.vdudt) r = a.vdudt[v] + uu * (a.vdudt[a.np + v] + uu * a.vdudt[2 * a.np + v]);
        }
        a.du[v] = r;
    }
}

// Derivative of a D polynomial c0 + c1 x + c2 x^2 at x.
template <int DDEG>
__device__ __forceinline__ double dpoly_prime(const double* c, int64_t stride, int64_t e, double x) {
    if (DDEG == 0) return 0.0;
    double r = __ldg(&c[stride + e]);
    if (DDEG >= 2) r += 2.0 * x * __ldg(&c[2 * stride + e]);
    return r;
}

// The derivative of fvm_eqs! on the per-triangle path.  JVP (DIAG false): du = J(u) v, with
// each dual-edge flux Q = D(u_s) G(u) giving dQ = D'(u_s) (s . v) G(u) + D(u_s) G(v), u_s the
// dual-edge midpoint value; the boundary and source terms likewise.  DIAG: du = diag J(u), the
// derivative of each vertex's row with respect to its own value.  Same tiles and order as
// triangle_rhs_kernel.
template <int DDEG, bool DIAG>
__global__ void __launch_bounds__(256) triangle_jvp_kernel(TriArgs a, const double* __restrict__ v) {
    extern __shared__ double acc[];
    const int64_t tile = blockIdx.x;
    const int64_t v0 = tile * a.tv;
    for (int i = threadIdx.x; i < a.tv; i += blockDim.x) acc[i] = 0.0;
    __syncthreads();
    const int64_t N = a.nelem;
    const int64_t e0 = a.off[tile], e1 = a.off[tile + 1];
    // dual-edge midpoint weights (in twelfths) of the corners a, b, c for edges 0, 1, 2
    const double W[3][3] = {{5.0, 5.0, 2.0}, {2.0, 5.0, 5.0}, {5.0, 2.0, 5.0}};
    for (int64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        const int32_t va = __ldg(&a.ev[e]), vb = __ldg(&a.ev[N + e]), vc = __ldg(&a.ev[2 * N + e]);
        const double ua = __ldg(&a.u[va]), ub = __ldg(&a.u[vb]), uc = __ldg(&a.u[vc]);
        double xa = 0, xb = 0, xc = 0;
        if (!DIAG) {
            xa = __ldg(&v[va]);
            xb = __ldg(&v[vb]);
            xc = __ldg(&v[vc]);
        }
        // dQ[d] (JVP), or dQ[d][corner] = dQ_d / du_corner (DIAG)
        double dQ[3][3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double* gc = DDEG == 0 ? a.ec : a.g;
            const double g0 = __ldg(&gc[(2 * d) * N + e]), g1 = __ldg(&gc[(2 * d + 1) * N + e]);
            const double dG[3] = {g0, g1, -g0 - g1};  // dG / d(ua, ub, uc)
            if (DDEG == 0) {
                if (DIAG) {
                    for (int k = 0; k < 3; ++k) dQ[d][k] = dG[k];
                } else {
                    dQ[d][0] = g0 * (xa - xc) + g1 * (xb - xc);
                }
            } else {
                const double G = g0 * (ua - uc) + g1 * (ub - uc);
                const double us = (W[d][0] * ua + W[d][1] * ub + W[d][2] * uc) / 12.0;
                const double* cd = a.ec + (int64_t)(d * (DDEG + 1)) * N;
                const double D = dpoly<DDEG>(cd, N, e, us), Dp = dpoly_prime<DDEG>(cd, N, e, us);
                if (DIAG) {
                    for (int k = 0; k < 3; ++k) dQ[d][k] = Dp * (W[d][k] / 12.0) * G + D * dG[k];
                } else {
                    const double sv = (W[d][0] * xa + W[d][1] * xb + W[d][2] * xc) / 12.0;
                    dQ[d][0] = Dp * sv * G + D * (g0 * (xa - xc) + g1 * (xb - xc));
                }
            }
        }
        const uint64_t la = (uint64_t)(va - v0), lb = (uint64_t)(vb - v0), lc = (uint64_t)(vc - v0);
        if (DIAG) {  // row a gets Q2 - Q0, row b Q0 - Q1, row c Q1 - Q2
            if (la < (uint64_t)a.tv) atomicAdd(&acc[la], dQ[2][0] - dQ[0][0]);
            if (lb < (uint64_t)a.tv) atomicAdd(&acc[lb], dQ[0][1] - dQ[1][1]);
            if (lc < (uint64_t)a.tv) atomicAdd(&acc[lc], dQ[1][2] - dQ[2][2]);
        } else {
            if (la < (uint64_t)a.tv) atomicAdd(&acc[la], dQ[2][0] - dQ[0][0]);
            if (lb < (uint64_t)a.tv) atomicAdd(&acc[lb], dQ[0][0] - dQ[1][0]);
            if (lc < (uint64_t)a.tv) atomicAdd(&acc[lc], dQ[1][0] - dQ[2][0]);
        }
    }
    const int64_t NB = a.nbelem;
    const int nd = DDEG + 1;
    const int64_t b0 = a.boff[tile], b1 = a.boff[tile + 1];
    for (int64_t e = b0 + threadIdx.x; e < b1; e += blockDim.x) {
        const int32_t vi = a.bv[e], vj = a.bv[NB + e], vk = a.bv[2 * NB + e];
        const double ui = a.u[vi], uj = a.u[vj], uk = a.u[vk];
        const double umi = (3.0 * ui + uj) / 4.0, umj = (ui + 3.0 * uj) / 4.0;
        const double lh = a.bg[2 * NB + e];
        double xi = 0, xj = 0, xk = 0;
        if (!DIAG) {
            xi = v[vi];
            xj = v[vj];
            xk = v[vk];
        }
        const double dmi = DIAG ? 0.75 : (3.0 * xi + xj) / 4.0, dmj = DIAG ? 0.75 : (xi + 3.0 * xj) / 4.0;
        double dQi, dQj;
        if (a.bc[e] != 0.0) {  // Neumann q.n = n0 + n1 u(m) + n2 u(m)^2
            const double* n = a.bc + (int64_t)(1 + 2 * nd) * NB;
            dQi = (n[NB + e] + 2.0 * umi * n[2 * NB + e]) * dmi * lh;
            dQj = (n[4 * NB + e] + 2.0 * umj * n[5 * NB + e]) * dmj * lh;
        } else {
            const double bg0 = a.bg[e], bg1 = a.bg[NB + e];
            const double G = bg0 * (ui - uk) + bg1 * (uj - uk);
            const double Gi = DIAG ? bg0 : bg0 * (xi - xk) + bg1 * (xj - xk);
            const double Gj = DIAG ? bg1 : Gi;
            dQi = dpoly_prime<DDEG>(a.bc + NB, NB, e, umi) * dmi * G + dpoly<DDEG>(a.bc + NB, NB, e, umi) * Gi;
            dQj = dpoly_prime<DDEG>(a.bc + (int64_t)(1 + nd) * NB, NB, e, umj) * dmj * G +
                  dpoly<DDEG>(a.bc + (int64_t)(1 + nd) * NB, NB, e, umj) * Gj;
        }
        const uint64_t li = (uint64_t)(vi - v0), lj = (uint64_t)(vj - v0);
        if (li < (uint64_t)a.tv) atomicAdd(&acc[li], -dQi);
        if (lj < (uint64_t)a.tv) atomicAdd(&acc[lj], -dQj);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < a.tv; i += blockDim.x) {
        const int64_t vv = v0 + i;
        if (vv >= a.np) break;
        const int c = a.code[vv];
        const double uu = a.u[vv];
        const double xv = DIAG ? 1.0 : v[vv];
        double r = 0.0;
        if (c == FVM_VERTEX_FREE) {
            r = acc[i] * a.invV[vv];
            if (a.vsrc) r += (a.vsrc[a.np + vv] + 2.0 * uu * a.vsrc[2 * a.np + vv]) * xv;
        } else if (c == FVM_VERTEX_DUDT) {
            if (a.vdudt) r = (a.vdudt[a.np + vv] + 2.0 * uu * a.vdudt[2 * a.np + vv]) * xv;
        }
        a.du[vv] = r;
    }
}

void launch_triangle_rhs(const fvm_mesh* m, const fvm_problem* p, const double* u, double* du, cudaStream_t s) {
    const Tiles& T = m->tiles;
    TriArgs a;
    a.off = T.d_off.as<int64_t>();
    a.boff = T.d_boff.as<int64_t>();
    a.ev = T.d_ev.as<int32_t>();
    a.g = T.d_g.as<double>();
    a.ec = p->d_ec.as<double>();
    a.bv = T.d_bv.as<int32_t>();
    a.bg = T.d_bg.as<double>();
    a.bc = p->d_bc.as<double>();
    a.code = p->d_code.as<int8_t>();
    a.invV = m->d_invV.as<double>();
    a.vsrc = p->src.empty() ? nullptr : p->d_vsrc.as<double>();
    a.vdudt = p->dudt.empty() ? nullptr : p->d_vdudt.as<double>();
    a.u = u;
    a.du = du;
    a.nelem = T.nelem;
    a.nbelem = T.nbelem;
    a.np = m->np;
    a.tv = T.tile_vertices;
    size_t smem = sizeof(double) * T.tile_vertices;
    switch (p->dif_deg) {
        case 0: triangle_rhs_kernel<0><<<(unsigned)T.ntiles, 256, smem, s>>>(a); break;
        case 1: triangle_rhs_kernel<1><<<(unsigned)T.ntiles, 256, smem, s>>>(a); break;
        default: triangle_rhs_kernel<2><<<(unsigned)T.ntiles, 256, smem, s>>>(a); break;
    }
}

void launch_triangle_jvp(const fvm_mesh* m, const fvm_problem* p, const double* u, const double* v, double* jv,
                         bool diag, cudaStream_t s) {
    const Tiles& T = m->tiles;
    TriArgs a;
    a.off = T.d_off.as<int64_t>();
    a.boff = T.d_boff.as<int64_t>();
    a.ev = T.d_ev.as<int32_t>();
    a.g = T.d_g.as<double>();
    a.ec = p->d_ec.as<double>();
    a.bv = T.d_bv.as<int32_t>();
    a.bg = T.d_bg.as<double>();
    a.bc = p->d_bc.as<double>();
    a.code = p->d_code.as<int8_t>();
    a.invV = m->d_invV.as<double>();
    a.vsrc = p->src.empty() ? nullptr : p->d_vsrc.as<double>();
    a.vdudt = p->dudt.empty() ? nullptr : p->d_vdudt.as<double>();
    a.u = u;
    a.du = jv;
    a.nelem = T.nelem;
    a.nbelem = T.nbelem;
    a.np = m->np;
    a.tv = T.tile_vertices;
    const size_t smem = sizeof(double) * T.tile_vertices;
    const unsigned g = (unsigned)T.ntiles;
    if (diag) {
        switch (p->dif_deg) {
            case 0: triangle_jvp_kernel<0, true><<<g, 256, smem, s>>>(a, v); break;
            case 1: triangle_jvp_kernel<1, true><<<g, 256, smem, s>>>(a, v); break;
            default: triangle_jvp_kernel<2, true><<<g, 256, smem, s>>>(a, v); break;
        }
    } else {
        switch (p->dif_deg) {
            case 0: triangle_jvp_kernel<0, false><<<g, 256, smem, s>>>(a, v); break;
            case 1: triangle_jvp_kernel<1, false><<<g, 256, smem, s>>>(a, v); break;
            default: triangle_jvp_kernel<2, false><<<g, 256, smem, s>>>(a, v); break;
        }
    }
}

// y += 2 q u v (the derivative of a quadratic diagonal term q u^2), or y = diag + 2 q u (DIAG)
__global__ void quad_jvp_kernel(const double* __restrict__ q, const double* __restrict__ u,
                                const double* __restrict__ v, const double* __restrict__ diag, double* __restrict__ y,
                                int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double qq = q ? q[i] : 0.0;
    if (diag)
        y[i] = diag[i] + 2.0 * qq * u[i];
    else
        y[i] += 2.0 * qq * u[i] * v[i];
}
void launch_quad_jvp(const double* q, const double* u, const double* v, const double* diag, double* y, int64_t n,
                     cudaStream_t s) {
    if (n) quad_jvp_kernel<<<grid_for(n, 256), 256, 0, s>>>(q, u, v, diag, y, n);
}

// ---------------------------------------------------------------------------------------
// Tsit5 stage combination, error norm, dense output
// ---------------------------------------------------------------------------------------
struct StageArgs {
    const double* k[7];
    double a[7];
};

__global__ void stage_kernel(double* __restrict__ y, const double* __restrict__ u, StageArgs sa, int nk, double dt,
                             int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j < 7; ++j)
        if (j < nk) acc += sa.a[j] * sa.k[j][i];
    y[i] = u[i] + dt * acc;
}

void launch_stage(double* y, const double* u, const double* const* k, const double* a, int nk, double dt, int64_t n,
                  cudaStream_t s) {
    StageArgs sa;
    for (int j = 0; j < 7; ++j) {
        sa.k[j] = j < nk ? k[j] : nullptr;
        sa.a[j] = j < nk ? a[j] : 0.0;
    }
    stage_kernel<<<grid_for(n, 256), 256, 0, s>>>(y, u, sa, nk, dt, n);
}

// Deterministic two-pass sum of squares of the scaled error (ODE_DEFAULT_NORM, RMS).
__global__ void error_partial_kernel(const double* __restrict__ u, const double* __restrict__ unew, StageArgs sa,
                                     double dt, double abstol, double reltol, int64_t n, double* __restrict__ part) {
    __shared__ double red[256];
    double acc = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double e = 0.0;
#pragma unroll
        for (int j = 0; j < 7; ++j) e += sa.a[j] * sa.k[j][i];
        e *= dt;
        double sc = abstol + fmax(fabs(u[i]), fabs(unew[i])) * reltol;
        double r = e / sc;
        acc += r * r;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}
__global__ void sum_partials_kernel(const double* __restrict__ part, int n, double* __restrict__ out) {
    __shared__ double red[256];
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) acc += part[i];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = red[0];
}
constexpr int kErrBlocks = 304;
void launch_error_norm(const double* u, const double* unew, const double* const* k, const double* bt, double dt,
                       double abstol, double reltol, int64_t n, double* d_acc, cudaStream_t s) {
    StageArgs sa;
    for (int j = 0; j < 7; ++j) {
        sa.k[j] = k[j];
        sa.a[j] = bt[j];
    }
    error_partial_kernel<<<kErrBlocks, 256, 0, s>>>(u, unew, sa, dt, abstol, reltol, n, d_acc + 1);
    sum_partials_kernel<<<1, 256, 0, s>>>(d_acc + 1, kErrBlocks, d_acc);
}

// saveat value inside a step from Tsit5's continuous extension: a stage combination with the
// weights w_j(theta)
void launch_tsit5_interp(double* out, const double* u, const double* const* k, double h, double theta, int64_t n,
                         cudaStream_t s) {
    double w[7];
    tsit5_interp_weights(theta, w);
    launch_stage(out, u, k, w, 7, h, n, s);
}

// w_i(theta) multiplied out: each is a constant times linear or quadratic factors times theta
// or theta^2
void tsit5_interp_poly(double beta[7][4]) {
    // coefficients of theta^0.. of a polynomial held as a vector, multiplied factor by factor
    auto mul = [](std::vector<double> p, std::initializer_list<double> f) {
        std::vector<double> r(p.size() + f.size() - 1, 0.0);
        size_t j = 0;
        for (double fj : f) {
            for (size_t i = 0; i < p.size(); ++i) r[i + j] += p[i] * fj;
            ++j;
        }
        return r;
    };
    std::vector<std::vector<double>> P(7);
    P[0] = mul(mul(mul({-1.0530884977290216}, {0.0, 1.0}), {-1.3299890189751412, 1.0}),
               {0.7139816917074209, -1.4364028541716351, 1.0});
    P[1] = mul(mul({0.1017}, {0.0, 0.0, 1.0}), {1.2949852507374631, -2.1966568338249754, 1.0});
    P[2] = mul(mul({2.490627285651252793}, {0.0, 0.0, 1.0}), {1.57803468208092486, -2.38535645472061657, 1.0});
    P[3] = mul(mul(mul({-16.54810288924490272}, {-1.21712927295533244, 1.0}), {-0.61620406037800089, 1.0}),
               {0.0, 0.0, 1.0});
    P[4] = mul(mul(mul({47.37952196281928122}, {-1.203071208372362603, 1.0}), {-0.658047292653547382, 1.0}),
               {0.0, 0.0, 1.0});
    P[5] = mul(mul(mul({-34.87065786149660974}, {-1.2, 1.0}), {-0.666666666666666667, 1.0}), {0.0, 0.0, 1.0});
    P[6] = mul(mul(mul({2.5}, {-1.0, 1.0}), {-0.6, 1.0}), {0.0, 0.0, 1.0});
    for (int i = 0; i < 7; ++i)
        for (int p = 0; p < 4; ++p) beta[i][p] = p + 1 < (int)P[i].size() ? P[i][p + 1] : 0.0;
}

// ---------------------------------------------------------------------------------------
// Device-controlled adaptive Tsit5: one attempted step per iteration of a graph WHILE loop.
// The step size lives in device memory (AdaptState), so the stage, error and output kernels
// read it there; a one-thread controller applies the PI step control of the host driver and
// sets the loop condition.  No host round trip per step.
// ---------------------------------------------------------------------------------------
__global__ void adapt_begin_kernel(AdaptState* st) {
    const double t = st->t, dt = st->dt;
    st->last = t + dt >= st->tf ? 1 : 0;
    st->h = st->last ? st->tf - t : dt;
}

__global__ void stage_dev_kernel(double* __restrict__ y, const double* __restrict__ u, StageArgs sa, int nk,
                                 const AdaptState* __restrict__ st, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j < 7; ++j)
        if (j < nk) acc += sa.a[j] * sa.k[j][i];
    y[i] = u[i] + st->h * acc;
}
void launch_stage_dev(double* y, const double* u, const double* const* k, const double* a, int nk,
                      const AdaptState* st, int64_t n, cudaStream_t s) {
    StageArgs sa;
    for (int j = 0; j < 7; ++j) {
        sa.k[j] = j < nk ? k[j] : nullptr;
        sa.a[j] = j < nk ? a[j] : 0.0;
    }
    stage_dev_kernel<<<grid_for(n, 256), 256, 0, s>>>(y, u, sa, nk, st, n);
}

__global__ void error_partial_dev_kernel(const double* __restrict__ u, const double* __restrict__ unew, StageArgs sa,
                                         const AdaptState* __restrict__ st, int64_t n, double* __restrict__ part) {
    __shared__ double red[256];
    const double dt = st->h, abstol = st->abstol, reltol = st->reltol;
    double acc = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double e = 0.0;
#pragma unroll
        for (int j = 0; j < 7; ++j) e += sa.a[j] * sa.k[j][i];
        e *= dt;
        double sc = abstol + fmax(fabs(u[i]), fabs(unew[i])) * reltol;
        double r = e / sc;
        acc += r * r;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// a graph-looped solve that runs this long stops with status 4 (a runaway step sequence)
constexpr unsigned long long kDeviceLoopTimeLimitNs = 600ull * 1000000000ull;

// PI control of OrdinaryDiffEq's Tsit5 defaults (the host driver's formulas)
// (256 threads: the partial sums are reduced in the order of sum_partials_kernel)
__global__ void adapt_control_kernel(AdaptState* st, const double* __restrict__ part, int nparts, int64_t n,
                                     cudaGraphConditionalHandle cond) {
    __shared__ double red[256];
    double acc = 0.0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) acc += part[i];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    const double sum = red[0];
    const double beta1 = 7.0 / 50.0, beta2 = 2.0 / 25.0, qmin = 0.2, qmax = 10.0, gamma = 0.9;
    const double EEst = sqrt(sum / (double)(n > 1 ? n : 1));
    const double h = st->h, t = st->t;
    st->accept = 0;
    if (!isfinite(EEst)) {
        st->status = 3;
        cudaGraphSetConditional(cond, 0);
        return;
    }
    double q11 = 0.0, q;
    if (EEst == 0.0) {
        q = 1.0 / qmax;
    } else {
        q11 = pow(EEst, beta1);
        q = q11 / pow(st->qold, beta2);
        q = fmax(1.0 / qmax, fmin(1.0 / qmin, q / gamma));
    }
    st->step += 1;
    if (EEst > 1.0) {  // reject
        st->nrej += 1;
        st->dt = h / fmin(1.0 / qmin, q11 / gamma);
        if (st->dt < 1e-14 * fmax(1.0, fabs(t))) st->status = 2;
    } else {
        st->accept = 1;
        st->t_prev = t;
        st->t = st->last ? st->tf : t + h;
        st->nacc += 1;
        st->qold = fmax(EEst, 1e-4);
        st->dt = fmin(h / q, st->tspan);
    }
    const bool finished = st->accept && st->last;
    if (!finished && st->status == 0 && st->step >= st->max_steps) st->status = 1;
    const unsigned long long now = global_ns();
    if (st->start_ns == 0) st->start_ns = now;
    if (!finished && st->status == 0 && now - st->start_ns > kDeviceLoopTimeLimitNs) st->status = 4;
    cudaGraphSetConditional(cond, (!finished && st->status == 0) ? 1u : 0u);
}

// saveat points strictly inside the accepted step: Tsit5's continuous extension of the step
// (the seven stage derivatives; the weights are the same for every row of a save)
__global__ void adapt_save_interp_kernel(double* __restrict__ out, const double* __restrict__ u, StageArgs sk,
                                         const double* __restrict__ saveat, const AdaptState* __restrict__ st,
                                         int64_t n) {
    if (!st->accept) return;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double h = st->h, t0 = st->t_prev, tn = st->t;
    double kv[7];
#pragma unroll
    for (int j = 0; j < 7; ++j) kv[j] = sk.k[j][i];
    const double ui = u[i];
    for (int64_t j = st->si; j < st->nsave && saveat[j] < tn; ++j) {
        double w[7];
        tsit5_interp_weights((saveat[j] - t0) / h, w);
        double acc = 0.0;
#pragma unroll
        for (int q = 0; q < 7; ++q) acc += w[q] * kv[q];
        out[j * n + i] = ui + h * acc;
    }
}
// accepted step: u <- unew, FSAL k0 <- k6
__global__ void adapt_commit_kernel(double* __restrict__ u, const double* __restrict__ unew, double* __restrict__ k0,
                                    const double* __restrict__ k6, const AdaptState* __restrict__ st, int64_t n) {
    if (!st->accept) return;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    u[i] = unew[i];
    k0[i] = k6[i];
}
// saveat points at the step's end (after the callback), then the save cursor moves past tn
__global__ void adapt_save_exact_kernel(double* __restrict__ out, const double* __restrict__ u,
                                        const double* __restrict__ saveat, const AdaptState* __restrict__ st,
                                        int64_t n) {
    if (!st->accept) return;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double tn = st->t;
    int64_t j = st->si;
    while (j < st->nsave && saveat[j] < tn) ++j;
    for (; j < st->nsave && saveat[j] == tn; ++j) out[j * n + i] = u[i];
}
__global__ void adapt_advance_kernel(AdaptState* st, const double* __restrict__ saveat) {
    if (!st->accept) return;
    int64_t j = st->si;
    while (j < st->nsave && saveat[j] <= st->t) ++j;
    st->si = j;
}

void launch_adaptive_step_tail(AdaptState* st, const double* part, int nparts, int64_t n,
                               cudaGraphConditionalHandle cond, double* out, double* u, const double* unew,
                               double* const* k, const double* saveat, cudaStream_t s) {
    StageArgs sk;
    for (int j = 0; j < 7; ++j) {
        sk.k[j] = k[j];
        sk.a[j] = 0.0;
    }
    adapt_control_kernel<<<1, 256, 0, s>>>(st, part, nparts, n, cond);
    adapt_save_interp_kernel<<<grid_for(n, 256), 256, 0, s>>>(out, u, sk, saveat, st, n);
    adapt_commit_kernel<<<grid_for(n, 256), 256, 0, s>>>(u, unew, k[0], k[6], st, n);
}
void launch_adaptive_step_end(AdaptState* st, double* out, const double* u, const double* saveat, int64_t n,
                              cudaStream_t s) {
    adapt_save_exact_kernel<<<grid_for(n, 256), 256, 0, s>>>(out, u, saveat, st, n);
    adapt_advance_kernel<<<1, 1, 0, s>>>(st, saveat);
}
void launch_adapt_begin(AdaptState* st, cudaStream_t s) { adapt_begin_kernel<<<1, 1, 0, s>>>(st); }
void launch_error_partial_dev(const double* u, const double* unew, const double* const* k, const double* bt,
                              const AdaptState* st, int64_t n, double* part, int nparts, cudaStream_t s) {
    StageArgs sa;
    for (int j = 0; j < 7; ++j) {
        sa.k[j] = k[j];
        sa.a[j] = bt[j];
    }
    error_partial_dev_kernel<<<nparts, 256, 0, s>>>(u, unew, sa, st, n, part);
}

__global__ void fill_kernel(double* x, double v, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = v;
}
void launch_fill(double* x, double v, int64_t n, cudaStream_t s) {
    if (n) fill_kernel<<<grid_for(n, 256), 256, 0, s>>>(x, v, n);
}

}  // namespace fvm
