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
// Arithmetic per row follows the graph-looped driver operation for operation (stage sums,
// slot order of the sliced-ELL product, error norm terms, Hermite output), so the solution
// differs from it only through the order of the error-norm sum.
// The loop ends at tf, on an error status, after max_steps attempted steps, or when the
// kernel has run for kClusterTimeLimitNs (status 4) - no barrier waits on a thread that can
// leave the loop early, because the exit decision is the same in every thread.
#include <cooperative_groups.h>

#include <cstdlib>
#include <vector>

#include "fvm_internal.h"
#include "fvm_tma.cuh"

namespace cg = cooperative_groups;

namespace fvm {

constexpr int kClusterMax = 16;
constexpr int kClusterWarps = 16;
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
    double a[7][6];
    double bt[7];
};

// Step decision of one CTA's thread 0, read by the CTA's other threads after a __syncthreads.
struct ClusterCtl {
    double h, t0, tn;
    int64_t si, j1, j2;  // interpolated saves [si, j1), saves at the step end [j1, j2)
    int32_t last, accept, stop;
};

// PI control of OrdinaryDiffEq's Tsit5 defaults (the formulas of the other drivers), applied
// by thread 0 of every CTA to the same inputs; sets the next step's h and last.
__device__ void cluster_control(AdaptState& S, ClusterCtl& c, double sum, double flags, int64_t n,
                                const double* __restrict__ saveat) {
    const double beta1 = 7.0 / 50.0, beta2 = 2.0 / 25.0, qmin = 0.2, qmax = 10.0, gamma = 0.9;
    const double h = c.h;
    const bool last = c.last != 0;
    const double EEst = sqrt(sum / (double)(n > 1 ? n : 1));
    c.accept = 0;
    c.stop = 0;
    if (!isfinite(EEst)) {
        S.status = 3;
        c.stop = 1;
        return;
    }
    double q11 = 0.0, qc;
    if (EEst == 0.0) {
        qc = 1.0 / qmax;
    } else {
        q11 = pow(EEst, beta1);
        qc = q11 / pow(S.qold, beta2);
        qc = fmax(1.0 / qmax, fmin(1.0 / qmin, qc / gamma));
    }
    S.step += 1;
    bool finished = false;
    if (EEst > 1.0) {  // reject
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
        S.qold = fmax(EEst, 1e-4);
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
    cg::cluster_group cl = cg::this_cluster();
    const unsigned crank = cl.block_rank(), csize = cl.num_blocks();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    const int64_t sl = (int64_t)crank * a.spc + warp;
    const int64_t r = sl * 32 + lane;
    const bool has_slice = sl < a.nslices;
    const bool own = has_slice && r < a.n;
    double* ybuf[2] = {sm, sm + a.npad};
    double* psum = sm + 2 * a.npad;           // [2][kClusterMax] per-CTA partial sums
    double* pflag = psum + 2 * kClusterMax;  // [2][kClusterMax] per-CTA time-limit flags

    const int64_t n = a.n;
    double u = own ? a.u[r] : 0.0;
    double k[7];
    k[0] = own ? a.k0[r] : 0.0;
#pragma unroll
    for (int j = 1; j < 7; ++j) k[j] = 0.0;
    const double dv = (own && a.dirval) ? a.dirval[r] : __longlong_as_double(0x7ff8000000000000ll);
    const uint32_t dest = own ? a.dests[r] : 0u;
    const int64_t base = has_slice ? __ldg(&a.slice_ptr[sl]) + lane : 0;
    const int w = has_slice ? __ldg(&a.width[sl]) : 0;
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
    const unsigned long long t_start = global_ns();
    if (threadIdx.x == 0) {
        S = *a.st;
        ctl.last = S.t + S.dt >= S.tf ? 1 : 0;
        ctl.h = ctl.last ? S.tf - S.t : S.dt;
    }
    cl.sync();  // every CTA of the cluster is running before the first remote store
    const double abstol = S.abstol, reltol = S.reltol;
    int pb = 0;
    for (;;) {
        const double h = ctl.h;
        double unew = 0.0;
#pragma unroll
        for (int s = 1; s <= 6; ++s) {
            double acc = 0.0;
#pragma unroll
            for (int j = 0; j < 6; ++j)
                if (j < s) acc += a.a[s][j] * k[j];
            const double y = u + h * acc;
            if (s == 6) unew = y;
            double* yb = ybuf[s & 1];
            for (uint32_t m = dest; m; m &= m - 1) cl.map_shared_rank(yb, __ffs(m) - 1)[r] = y;
            cl.sync();
            // f(y) for the owned row: sliced-ELL slots in order, then q y^2, then b
            double f = 0.0;
            if constexpr (MAXW > 0) {
                double xs[MAXW];
#pragma unroll
                for (int kk = 0; kk < MAXW; ++kk)
                    if (kk < w) xs[kk] = yb[cc[kk]];
#pragma unroll
                for (int kk = 0; kk < MAXW; ++kk)
                    if (kk < w) f += cv[kk] * xs[kk];
            } else {
                for (int kk = 0; kk < w; ++kk) {
                    const int64_t i = base + (int64_t)kk * 32;
                    f += __ldg(&a.val[i]) * yb[__ldg(&a.col[i])];
                }
            }
            if (a.q) f += qq * y * y;
            if (a.b) f += bq;
            k[s] = f;
        }
        // scaled RMS error: this CTA's sum of squares, broadcast to every CTA
        double e = 0.0;
#pragma unroll
        for (int j = 0; j < 7; ++j) e += a.bt[j] * k[j];
        e *= h;
        double v = 0.0;
        if (own) {
            const double sc = abstol + fmax(fabs(u), fabs(unew)) * reltol;
            const double rr = e / sc;
            v = rr * rr;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) wsum[warp] = v;
        __syncthreads();
        if (threadIdx.x == 0) {
            double cs = 0.0;
            for (int i = 0; i < nwarps; ++i) cs += wsum[i];
            const double flag = (global_ns() - t_start > kClusterTimeLimitNs) ? 1.0 : 0.0;
            for (unsigned c = 0; c < csize; ++c) {
                cl.map_shared_rank(psum, c)[pb * kClusterMax + crank] = cs;
                cl.map_shared_rank(pflag, c)[pb * kClusterMax + crank] = flag;
            }
        }
        cl.sync();
        if (threadIdx.x == 0) {
            double sum = 0.0, flags = 0.0;
            for (unsigned c = 0; c < csize; ++c) {
                sum += psum[pb * kClusterMax + c];
                flags += pflag[pb * kClusterMax + c];
            }
            cluster_control(S, ctl, sum, flags, n, a.saveat);
        }
        pb ^= 1;
        __syncthreads();
        if (ctl.accept) {
            if (own) {
                const double t0 = ctl.t0;
                for (int64_t j = ctl.si; j < ctl.j1; ++j) {
                    const double th = (__ldg(&a.saveat[j]) - t0) / h;
                    const double t2 = th * th, t3 = t2 * th;
                    const double h00 = 2 * t3 - 3 * t2 + 1, h10 = t3 - 2 * t2 + th, h01 = -2 * t3 + 3 * t2,
                                 h11 = t3 - t2;
                    a.out[j * n + r] = h00 * u + h10 * h * k[0] + h01 * unew + h11 * h * k[6];
                }
            }
            u = unew;
            if (!isnan(dv)) u = dv;  // Dirichlet callback
            k[0] = k[6];
            if (own)
                for (int64_t j = ctl.j1; j < ctl.j2; ++j) a.out[j * n + r] = u;
        }
        if (ctl.stop) break;
    }
    if (own) {
        a.u[r] = u;
        a.k0[r] = k[0];
    }
    if (crank == 0 && threadIdx.x == 0) *a.st = S;
    cl.sync();  // no CTA leaves while another could still address its shared memory
}

using ClusterKernel = void (*)(ClusterTsit5Args);

static ClusterKernel cluster_kernel_for(int maxw) {
    if (maxw <= 8) return tsit5_cluster_kernel<8>;
    if (maxw <= 12) return tsit5_cluster_kernel<12>;
    return tsit5_cluster_kernel<0>;
}

static size_t cluster_smem_bytes(int npad) { return sizeof(double) * ((size_t)2 * npad + 4 * kClusterMax); }

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
        if ((p.nslices + cs - 1) / cs > kClusterWarps) break;
        const int spc = (int)((p.nslices + cs - 1) / cs);
        cudaLaunchConfig_t cfg{};
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = cs;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(cs);
        cfg.blockDim = dim3(32 * spc);
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

// dests[r]: the CTAs whose rows have a slot in column r, so that y_r is stored only where it is
// gathered.  Computed once per pattern and cluster shape.
static const uint32_t* cluster_dests(const SellPattern& p, int cs, int spc) {
    const int key = cs * 64 + spc;
    if (p.cluster_dest_key == key) return p.d_cluster_dest.as<uint32_t>();
    std::vector<uint32_t> m((size_t)p.nslices * 32, 0u);
    for (int64_t sl = 0; sl < p.nslices; ++sl) {
        const uint32_t bit = 1u << (unsigned)(sl / spc);
        for (int64_t i = p.slice_ptr[sl]; i < p.slice_ptr[sl + 1]; ++i) {
            const int32_t c = p.col[i];
            if (c >= 0 && c < (int32_t)m.size()) m[c] |= bit;
        }
    }
    for (int64_t rr = 0; rr < (int64_t)m.size(); ++rr) m[rr] |= 1u << (unsigned)((rr / 32) / spc);
    p.d_cluster_dest.upload(m);
    p.cluster_dest_key = key;
    return p.d_cluster_dest.as<uint32_t>();
}

void launch_cluster_tsit5(const SellRhsDesc& d, const double* dirval, double* u, double* k0, double* out,
                          const double* saveat, AdaptState* st, const double (*A)[6], const double* bt,
                          cudaStream_t s) {
    const SellPattern& p = *d.pat;
    const int cs = cluster_size_for(p);
    if (cs == 0) fail(FVM_ERR_CUDA, "no thread-block cluster is available for the small-mesh Tsit5 driver");
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
    a.dests = cluster_dests(p, cs, a.spc);
    for (int i = 0; i < 7; ++i) {
        for (int j = 0; j < 6; ++j) a.a[i][j] = A[i][j];
        a.bt[i] = bt[i];
    }
    cudaLaunchConfig_t cfg{};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(cs);
    cfg.blockDim = dim3(32 * a.spc);
    cfg.dynamicSmemBytes = cluster_smem_bytes(a.npad);
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    FVM_CUDA(cudaLaunchKernelEx(&cfg, cluster_kernel_for(p.maxw), a));
}

}  // namespace fvm
