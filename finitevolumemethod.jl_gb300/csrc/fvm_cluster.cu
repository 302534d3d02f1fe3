// Adaptive Tsit5 for small meshes in one thread-block cluster (sm_103a).
//
// On a few thousand vertices a Tsit5 step is ~20 tiny kernels whose launch gaps, not their
// work, set the step time.  Here the whole adaptive loop after the first accepted step runs
// in ONE launch of a cluster of up to 16 CTAs (one per SM):
//   - thread (CTA c, warp w, lane l) owns row ((c * spc + w) * 32 + l) of the sliced-ELL
//     pattern and keeps that row's u, the seven stage derivatives and the slot loop in
//     registers;
//   - every stage value y_i is broadcast into each CTA's shared memory (distributed shared
//     memory stores), so the right-hand side gathers y from local shared memory;
//   - one cluster barrier per stage (double-buffered y) and one per step for the error norm,
//     whose per-CTA partial sums are broadcast the same way; every thread then sums the
//     partials in the same order and applies the same PI control, so all threads take the
//     same accept/reject decision without another barrier.
// Arithmetic per row follows the graph-looped driver for the stage sums and the error-norm
// terms; the sliced-ELL product is summed as a balanced tree (a shorter dependent FP64 chain:
// on GB300 each dependent FP64 operation costs tens of nanoseconds), and the error norm and
// step control round differently in the last bits, so the solution agrees with the other
// drivers to rounding.
// The loop ends at tf, on an error status, after max_steps attempted steps, or when the
// kernel has run for kClusterTimeLimitNs (status 4) - no barrier waits on a thread that can
// leave the loop early, because the exit decision is the same in every thread.
#include <cooperative_groups.h>

#include <cstdlib>
#include <vector>

#include "fvm_internal.h"
#include "fvm_pow.h"
#include "fvm_tma.cuh"

namespace cg = cooperative_groups;

namespace fvm {

constexpr int kClusterMax = 16;
constexpr int kClusterWarps = 16;  // row warps plus one control warp per CTA
constexpr unsigned long long kClusterTimeLimitNs = 120ull * 1000000000ull;

struct ClusterTsit5Args {
    const int64_t* slice_ptr;
    const int32_t* width;
    const int32_t* col;
    const double* val;
    const double* b;        // may be null
    const double* q;        // may be null
    const double* dirval;   // per row: Dirichlet value, NaN elsewhere; may be null
    const uint32_t* dests;  // per row: bit c set when CTA c gathers the row
    double* u;              // [n] in/out
    double* k0;             // [n] in/out: f(u), first-same-as-last
    double* out;            // [nsave][n]
    const double* saveat;   // [nsave]
    AdaptState* st;
    int64_t n, nslices;
    int spc;   // slices per CTA (= warps per CTA)
    int npad;  // nslices * 32: rows held in each CTA's y buffers
    uint32_t expect_bytes[kClusterMax];  // per CTA: bytes of row values it receives per stage
    double a[7][6];
    double bt[7];
    double bi[7][4];  // continuous extension: w_i(theta) = sum_p bi[i][p] theta^(p+1)
};

// Step decision of one CTA's thread 0, read by the CTA's other threads after a __syncthreads.
struct ClusterCtl {
    double h, t0, tn;
    double x_acc;        // sum / n of the last accepted step: qold = max(sqrt(x_acc), 1e-4) is pending
    int64_t si, j1, j2;  // interpolated saves [si, j1), saves at the step end [j1, j2)
    int32_t last, accept, stop, qold_pending;
};

constexpr int kClusterInterp = 32;  // saveat points per step whose theta is shared

__constant__ PowTables c_pow;  // tables of pow_pos, uploaded once per device (launch_cluster_tsit5)

// PI control of OrdinaryDiffEq's Tsit5 defaults, applied by thread 0 of every CTA to the same
// inputs; sets the next step's h and last.  On GB300 a chain of dependent FP64 operations in
// one thread costs ~40 ns per operation, so the chain is kept short: EEst^beta1 is taken as
// (sum / n)^(beta1 / 2) without the square root and through pow_pos (fvm_pow.h, within about
// one ulp, a third of the dependent operations of the library pow), qold^beta2 (pq) was
// computed by another warp during the step's stages, and qold itself (a square root) is left
// pending for that warp.  These change results only in the last bits, like the order of the
// error-norm sum.
__device__ void cluster_control(AdaptState& S, ClusterCtl& c, double sum, double flags, double inv_n, double pq,
                                const double* __restrict__ saveat) {
    const double beta1_half = 7.0 / 100.0, qmin = 0.2, qmax = 10.0, inv_gamma = 1.0 / 0.9, gamma = 0.9;
    const double h = c.h;
    const bool last = c.last != 0;
    const double x = sum * inv_n;  // EEst^2
    c.accept = 0;
    c.stop = 0;
    if (!isfinite(x)) {
        S.status = 3;
        c.stop = 1;
        return;
    }
    double q11 = 0.0, qc;
    if (x == 0.0) {
        qc = 1.0 / qmax;
    } else {
        q11 = pow_pos(x, beta1_half, c_pow);
        qc = fmax(1.0 / qmax, fmin(1.0 / qmin, (q11 / pq) * inv_gamma));
    }
    S.step += 1;
    bool finished = false;
    if (x > 1.0) {  // reject
        S.nrej += 1;
        S.dt = h / fmin(1.0 / qmin, q11 / gamma);
        if (S.dt < 1e-14 * fmax(1.0, fabs(S.t))) {
            S.status = 2;
            c.stop = 1;
            return;
        }
    } else {
        const double t0 = S.t, tn = last ? S.tf : S.t + h;
        int64_t j = S.si;
        c.si = j;
        while (j < S.nsave && saveat[j] < tn) ++j;
        c.j1 = j;
        while (j < S.nsave && saveat[j] == tn) ++j;
        c.j2 = j;
        c.t0 = t0;
        c.tn = tn;
        c.accept = 1;
        S.si = j;
        S.t_prev = t0;
        S.t = tn;
        S.nacc += 1;
        c.x_acc = x;
        c.qold_pending = 1;
        S.dt = fmin(h / qc, S.tspan);
        finished = last;
    }
    if (finished) {
        c.stop = 1;
    } else if (S.step >= S.max_steps) {
        S.status = 1;
        c.stop = 1;
    } else if (flags > 0.0) {
        S.status = 4;
        c.stop = 1;
    }
    c.last = S.t + S.dt >= S.tf ? 1 : 0;
    c.h = c.last ? S.tf - S.t : S.dt;
}

// MAXW > 0: the row's slots (at most MAXW) stay in registers for the whole solve; MAXW = 0
// re-reads them from global memory (L1-resident) at every stage.
template <int MAXW>
__global__ void __launch_bounds__(32 * kClusterWarps, 1) tsit5_cluster_kernel(const __grid_constant__ ClusterTsit5Args a) {
    extern __shared__ __align__(16) double sm[];
    __shared__ AdaptState S;
    __shared__ ClusterCtl ctl;
    __shared__ double wsum[kClusterWarps];
    __shared__ double pq_sh;
    __shared__ double thsh[kClusterInterp];  // theta of the step's interior saves
    __shared__ __align__(8) uint64_t ybar[3];
    __shared__ __align__(8) uint64_t pbar[2];
    cg::cluster_group cl = cg::this_cluster();
    const unsigned crank = cl.block_rank(), csize = cl.num_blocks();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nrw = a.spc;                // row warps; warp nrw is the control warp (no rows)
    const int pw_thread = 32 * nrw;       // computes qold^beta2 during the stages
    const int64_t sl = (int64_t)crank * a.spc + warp;
    const int64_t r = sl * 32 + lane;
    const bool has_slice = warp < nrw && sl < a.nslices;
    const bool own = has_slice && r < a.n;
    double* ybuf[3] = {sm, sm + a.npad, sm + 2 * a.npad};
    double* part = sm + 3 * a.npad;  // [2][kClusterMax][2]: each CTA's partial sum and time flag

    const int64_t n = a.n;
    const double inv_n = 1.0 / (double)(n > 1 ? n : 1);
    double u = own ? a.u[r] : 0.0;
    double k0 = own ? a.k0[r] : 0.0, k6 = 0.0;
    const double dv = (own && a.dirval) ? a.dirval[r] : __longlong_as_double(0x7ff8000000000000ll);
    const uint32_t dest = own ? a.dests[r] : 0u;
    const int64_t base = has_slice ? __ldg(&a.slice_ptr[sl]) + lane : 0;
    const int w = own ? __ldg(&a.width[sl]) : 0;
    const double bq = (own && a.b) ? a.b[r] : 0.0;
    const double qq = (own && a.q) ? a.q[r] : 0.0;
    int32_t cc[MAXW > 0 ? MAXW : 1];
    double cv[MAXW > 0 ? MAXW : 1];
    if constexpr (MAXW > 0) {
#pragma unroll
        for (int kk = 0; kk < MAXW; ++kk) {
            cc[kk] = kk < w ? __ldg(&a.col[base + (int64_t)kk * 32]) : 0;
            cv[kk] = kk < w ? __ldg(&a.val[base + (int64_t)kk * 32]) : 0.0;
        }
    }
    const uint32_t ybytes = a.expect_bytes[crank];
    const unsigned long long t_start = global_ns();
    if (threadIdx.x == 0) {
        S = *a.st;
        ctl.last = S.t + S.dt >= S.tf ? 1 : 0;
        ctl.h = ctl.last ? S.tf - S.t : S.dt;
        ctl.qold_pending = 0;
        for (int i = 0; i < 3; ++i) mbar_init(&ybar[i], 1);
        for (int i = 0; i < 2; ++i) mbar_init(&pbar[i], 1);
        mbar_init_fence();
        mbar_arrive_expect_tx(&ybar[0], ybytes);         // stage 0
        mbar_arrive_expect_tx(&pbar[0], 16u * csize);    // step 0's partial sums
    }
    // every CTA's barriers are initialised and armed before the first remote store
    cl.sync();
    const double abstol = S.abstol, reltol = S.reltol;
    uint32_t g = 0;   // stages so far: buffer g % 3, phase parity (g / 3) & 1
    uint32_t ns = 0;  // steps so far: partial-sum buffer ns % 2, parity (ns / 2) & 1
    bool bad = false;
    for (;;) {
        const double h = ctl.h;
        if (threadIdx.x == pw_thread) {  // read by thread 0 only after the stages
            if (ctl.qold_pending) S.qold = fmax(sqrt(ctl.x_acc), 1e-4);
            pq_sh = pow_pos(S.qold, 2.0 / 25.0, c_pow);
        }
        // running stage sums: acc[s] = sum_j a[s][j] k_j over the k_j known so far (slot order
        // j = 0, 1, ... as in the stage kernels), err likewise with the error weights
        double acc[7], err;
#pragma unroll
        for (int s = 1; s <= 6; ++s) acc[s] = a.a[s][0] * k0;
        err = a.bt[0] * k0;
        // running sums of the continuous extension, m[p] = sum_i bi[i][p] k_i
        double m[4];
#pragma unroll
        for (int p = 0; p < 4; ++p) m[p] = a.bi[0][p] * k0;
        double unew = 0.0, inv_sc = 0.0;
#pragma unroll
        for (int s = 1; s <= 6; ++s) {
            const double y = u + h * acc[s];
            if (s == 6) unew = y;
            const uint32_t b = g % 3;
            // arm the buffer of stage g + 1 (its stage g - 2 contents were read before any
            // thread of this CTA could pass stage g - 1) before this CTA's stage-g values leave:
            // a remote stage g + 1 value needs one of them first
            if (threadIdx.x == 0) mbar_arrive_expect_tx(&ybar[(g + 1) % 3], ybytes);
            if (__syncthreads_or(bad)) break;
            if (own) {
                const uint32_t yaddr = smem_addr(ybuf[b] + r), baddr = smem_addr(&ybar[b]);
                const unsigned long long bits = (unsigned long long)__double_as_longlong(y);
                for (uint32_t m = dest; m; m &= m - 1) {
                    const uint32_t c = __ffs(m) - 1;
                    st_async_b64(cluster_map(yaddr, c), bits, cluster_map(baddr, c));
                }
                if (s == 6) inv_sc = 1.0 / (abstol + fmax(fabs(u), fabs(y)) * reltol);  // during the wait
                if (!mbar_wait_cluster(&ybar[b], (g / 3) & 1)) bad = true;
                // f(y) for the owned row: sliced-ELL slots in order, then q y^2, then b
                const double* yb = ybuf[b];
                double f = 0.0;
                if constexpr (MAXW > 0) {
                    // slots past the row's width hold value 0 and column 0
                    double t[MAXW / 2];
#pragma unroll
                    for (int kk = 0; kk < MAXW / 2; ++kk)
                        t[kk] = fma(cv[2 * kk + 1], yb[cc[2 * kk + 1]], cv[2 * kk] * yb[cc[2 * kk]]);
#pragma unroll
                    for (int span = 1; span < MAXW / 2; span *= 2)
#pragma unroll
                        for (int kk = 0; kk + span < MAXW / 2; kk += 2 * span) t[kk] += t[kk + span];
                    f = t[0];
                } else {
                    for (int kk = 0; kk < w; ++kk) {
                        const int64_t i = base + (int64_t)kk * 32;
                        f += __ldg(&a.val[i]) * yb[__ldg(&a.col[i])];
                    }
                }
                if (a.q) f += qq * y * y;
                if (a.b) f += bq;
#pragma unroll
                for (int s2 = s + 1; s2 <= 6; ++s2) acc[s2] += a.a[s2][s] * f;
                err += a.bt[s] * f;
#pragma unroll
                for (int p = 0; p < 4; ++p) m[p] += a.bi[s][p] * f;
                if (s == 6) k6 = f;
            }
            ++g;
        }
        if (__syncthreads_or(bad)) {
            if (threadIdx.x == 0) S.status = 5;
            break;
        }
        // scaled RMS error: this CTA's sum of squares, sent to every CTA
        double v = 0.0;
        if (own) {
            const double rr = (err * h) * inv_sc;
            v = rr * rr;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) wsum[warp] = v;
        __syncthreads();
        if (warp == 0) {  // tree sums in warp 0, the same order in every CTA
            const uint32_t pb = ns & 1;
            double cs = lane < nrw ? wsum[lane] : 0.0;
#pragma unroll
            for (int o = 8; o > 0; o >>= 1) cs += __shfl_xor_sync(0xffffffffu, cs, o);
            if (lane == 0) {
                const unsigned long long flag = (global_ns() - t_start > kClusterTimeLimitNs) ? 1ull : 0ull;
                // next step's partials can only follow this one's
                mbar_arrive_expect_tx(&pbar[pb ^ 1], 16u * csize);
                double* slot = part + (pb * kClusterMax + crank) * 2;
                const uint32_t a0 = smem_addr(slot), a1 = smem_addr(slot + 1), pba = smem_addr(&pbar[pb]);
                for (unsigned c = 0; c < csize; ++c) {
                    const uint32_t rb = cluster_map(pba, c);
                    st_async_b64(cluster_map(a0, c), (unsigned long long)__double_as_longlong(cs), rb);
                    st_async_b64(cluster_map(a1, c), flag, rb);
                }
                if (ctl.qold_pending) ctl.qold_pending = 0;  // resolved by pw_thread this step
            }
            const bool ok = __all_sync(0xffffffffu, mbar_wait_cluster(&pbar[pb], (ns / 2) & 1));
            double sum = (ok && lane < (int)csize) ? part[(pb * kClusterMax + lane) * 2] : 0.0;
            unsigned long long fl =
                (ok && lane < (int)csize)
                    ? (unsigned long long)__double_as_longlong(part[(pb * kClusterMax + lane) * 2 + 1])
                    : 0ull;
#pragma unroll
            for (int o = 8; o > 0; o >>= 1) {
                sum += __shfl_xor_sync(0xffffffffu, sum, o);
                fl |= __shfl_xor_sync(0xffffffffu, fl, o);
            }
            if (lane == 0) {
                if (!ok) {
                    S.status = 5;
                    ctl.accept = 0;
                    ctl.stop = 1;
                } else {
                    cluster_control(S, ctl, sum, fl ? 1.0 : 0.0, inv_n, pq_sh, a.saveat);
                }
            }
        }
        ++ns;
        __syncthreads();
        if (ctl.accept) {
            const int64_t nint = ctl.j1 - ctl.si;
            if (nint > 0) {  // the step's interior saves from the continuous extension
                if (threadIdx.x < kClusterInterp && threadIdx.x < nint)
                    thsh[threadIdx.x] = (__ldg(&a.saveat[ctl.si + threadIdx.x]) - ctl.t0) / h;
                __syncthreads();
                if (own) {
                    for (int64_t j = ctl.si; j < ctl.j1; ++j) {
                        const int64_t jj = j - ctl.si;
                        const double th = jj < kClusterInterp ? thsh[jj] : (__ldg(&a.saveat[j]) - ctl.t0) / h;
                        a.out[j * n + r] = u + h * (th * (m[0] + th * (m[1] + th * (m[2] + th * m[3]))));
                    }
                }
            }
            u = unew;
            if (!isnan(dv)) u = dv;  // Dirichlet callback
            k0 = k6;
            if (own)
                for (int64_t j = ctl.j1; j < ctl.j2; ++j) a.out[j * n + r] = u;
        }
        if (ctl.stop) break;
    }
    if (own) {
        a.u[r] = u;
        a.k0[r] = k0;
    }
    if (crank == 0 && threadIdx.x == 0) {
        if (ctl.qold_pending) S.qold = fmax(sqrt(ctl.x_acc), 1e-4);
        *a.st = S;
    }
    cl.sync();  // no CTA leaves while another could still address its shared memory
}

using ClusterKernel = void (*)(ClusterTsit5Args);

static ClusterKernel cluster_kernel_for(int maxw) {
    if (maxw <= 8) return tsit5_cluster_kernel<8>;
    if (maxw <= 12) return tsit5_cluster_kernel<12>;
    return tsit5_cluster_kernel<0>;
}

static size_t cluster_smem_bytes(int npad) { return sizeof(double) * ((size_t)3 * npad + 4 * kClusterMax); }

// Cluster size for a pattern, or 0 when the cluster driver does not apply (too many rows for
// one cluster's shared memory, or no cluster of that size can be resident).  FVM_CLUSTER_CTAS
// (2, 4, 8 or 16) caps the size.
static int cluster_size_for(const SellPattern& p) {
    if (p.nslices <= 0 || p.nrows > kClusterMaxRows) return 0;
    const size_t smem = cluster_smem_bytes((int)(p.nslices * 32));
    int dev = 0;
    FVM_CUDA(cudaGetDevice(&dev));
    int optin = 0;
    FVM_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    if (smem + 1024 > (size_t)optin) return 0;
    ClusterKernel kern = cluster_kernel_for(p.maxw);
    FVM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    FVM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    int cap = kClusterMax;
    if (const char* e = std::getenv("FVM_CLUSTER_CTAS")) cap = std::max(1, std::min(kClusterMax, std::atoi(e)));
    if (p.cluster_cap == cap) return p.cluster_size;
    p.cluster_cap = cap;
    p.cluster_size = 0;
    for (int cs = kClusterMax; cs >= 1; cs /= 2) {
        if (cs > cap) continue;
        if ((p.nslices + cs - 1) / cs > kClusterWarps - 1) break;
        const int spc = (int)((p.nslices + cs - 1) / cs);
        cudaLaunchConfig_t cfg{};
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = cs;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(cs);
        cfg.blockDim = dim3(32 * (spc + 1));
        cfg.dynamicSmemBytes = smem;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        if (nclusters >= 1) {
            p.cluster_size = cs;
            break;
        }
    }
    return p.cluster_size;
}

bool cluster_tsit5_available(const SellPattern& pat) { return cluster_size_for(pat) > 0; }

// dests[r]: the CTAs whose rows have a slot in column r (and the row's own CTA), so that y_r is
// stored only where it is gathered.  The CTA graph is then made symmetric: when CTA A stores
// into CTA B but B stores nothing into A, one row of B also goes to A.  With every link
// two-way, a CTA cannot pass stage g + 2 before each CTA it stores into has finished reading
// stage g, which is what makes three row buffers enough.  expect[c] = bytes CTA c receives
// per stage.  Computed once per pattern and cluster shape.
static const uint32_t* cluster_dests(const SellPattern& p, int cs, int spc, uint32_t* expect) {
    const int key = cs * 64 + spc;
    if (p.cluster_dest_key != key) {
        const int64_t npad = p.nslices * 32;
        std::vector<uint32_t> m((size_t)npad, 0u);
        auto owner = [&](int64_t row) { return (unsigned)((row / 32) / spc); };
        for (int64_t sl = 0; sl < p.nslices; ++sl) {
            const uint32_t bit = 1u << (unsigned)(sl / spc);
            for (int64_t i = p.slice_ptr[sl]; i < p.slice_ptr[sl + 1]; ++i) {
                const int32_t c = p.col[i];
                if (c >= 0 && c < (int32_t)npad) m[c] |= bit;
            }
        }
        for (int64_t rr = 0; rr < npad; ++rr) m[rr] |= 1u << owner(rr);
        uint32_t to[kClusterMax] = {0};  // to[a]: CTAs that CTA a stores into
        int64_t first[kClusterMax];
        for (int i = 0; i < kClusterMax; ++i) first[i] = -1;
        for (int64_t rr = 0; rr < p.nrows; ++rr) {
            to[owner(rr)] |= m[rr];
            if (first[owner(rr)] < 0) first[owner(rr)] = rr;
        }
        for (int a = 0; a < cs; ++a)
            for (int b = 0; b < cs; ++b)
                if (a != b && (to[a] >> b & 1u) && !(to[b] >> a & 1u) && first[b] >= 0) {
                    m[first[b]] |= 1u << a;
                    to[b] |= 1u << a;
                }
        std::vector<uint32_t> e(kClusterMax, 0u);
        for (int64_t rr = 0; rr < p.nrows; ++rr)
            for (int c = 0; c < cs; ++c)
                if (m[rr] >> c & 1u) e[c] += 8;
        p.d_cluster_dest.upload(m);
        p.cluster_expect = e;
        p.cluster_dest_key = key;
    }
    for (int c = 0; c < kClusterMax; ++c) expect[c] = p.cluster_expect[c];
    return p.d_cluster_dest.as<uint32_t>();
}

void launch_cluster_tsit5(const SellRhsDesc& d, const double* dirval, double* u, double* k0, double* out,
                          const double* saveat, AdaptState* st, const double (*A)[6], const double* bt,
                          cudaStream_t s) {
    const SellPattern& p = *d.pat;
    const int cs = cluster_size_for(p);
    if (cs == 0) fail(FVM_ERR_CUDA, "no thread-block cluster is available for the small-mesh Tsit5 driver");
    static int pow_dev = -1;  // device whose constant bank holds the pow tables
    int dev = 0;
    FVM_CUDA(cudaGetDevice(&dev));
    if (pow_dev != dev) {
        PowTables T;
        pow_build_tables(T);
        FVM_CUDA(cudaMemcpyToSymbol(c_pow, &T, sizeof T));
        pow_dev = dev;
    }
    ClusterTsit5Args a{};
    a.slice_ptr = p.d_slice_ptr.as<int64_t>();
    a.width = p.d_width.as<int32_t>();
    a.col = p.d_col.as<int32_t>();
    a.val = d.val;
    a.b = d.b;
    a.q = d.q;
    a.dirval = dirval;
    a.u = u;
    a.k0 = k0;
    a.out = out;
    a.saveat = saveat;
    a.st = st;
    a.n = p.nrows;
    a.nslices = p.nslices;
    a.spc = (int)((p.nslices + cs - 1) / cs);
    a.npad = (int)(p.nslices * 32);
    a.dests = cluster_dests(p, cs, a.spc, a.expect_bytes);
    for (int i = 0; i < 7; ++i) {
        for (int j = 0; j < 6; ++j) a.a[i][j] = A[i][j];
        a.bt[i] = bt[i];
    }
    tsit5_interp_poly(a.bi);
    cudaLaunchConfig_t cfg{};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(cs);
    cfg.blockDim = dim3(32 * (a.spc + 1));
    cfg.dynamicSmemBytes = cluster_smem_bytes(a.npad);
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    FVM_CUDA(cudaLaunchKernelEx(&cfg, cluster_kernel_for(p.maxw), a));
}

}  // namespace fvm
