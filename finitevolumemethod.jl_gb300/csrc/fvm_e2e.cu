// fvm_eqs! on page-locked host arrays in one launch: the host link's reads, the operator and
// the link's writes overlapped.
//
// fvm_rhs with host u and du moves 8 bytes per point each way over the host link, in the
// caller's numbering, around the operator product in the internal (Hilbert) numbering.  Done
// as three launches (read and permute, product, permute and write) the two link transfers and
// the product run one after another.  Here one persistent kernel works through a queue of
// items of three kinds:
//   A  caller points [a C, (a+1) C): read u from the host array, scatter to the internal vector
//   B  slices [b S, (b+1) S): the operator rows of those slices into the internal du
//   C  caller points [c C, (c+1) C): gather du and write the host array
// Each B lists the A items holding its columns, each C the B items holding its rows, and A a
// lists A (a - r) (r items reading at once), so that the reads proceed in caller order at the
// link's rate instead of all finishing together: B items then start as soon as the rows they
// read have arrived.  CTAs
// take items in queue order from one atomic counter; an item waits (bounded) until every item
// it lists has published its flag, does its work, and publishes its own flag.  The queue puts
// every item after the items it lists and interleaves the kinds (each B right after its last
// A, each C right after its last B), so link reads, products and link writes of different
// parts of the mesh proceed at once.  An item only waits on items earlier in the queue, which
// CTAs that are running have already taken, and A items wait on nothing: every wait ends.
//
// Values written by one CTA and read by another in the same launch (the internal u and du) are
// read through L2 (ld.global.cg), never from a possibly stale L1 line.  The row sum is the
// streamed kernel's: slots in order, the same epilogue, so the result is bit-identical.
#include <algorithm>
#include <vector>

#include "fvm_internal.h"
#include "fvm_sell.cuh"
#include "fvm_tma.cuh"

namespace fvm {

constexpr unsigned kDevErrFlagWait = 4u;  // an item waited too long for an item it lists
constexpr int kE2eThreads = 256;
constexpr int kE2eUnroll = 8;  // link loads (A) and L2 gathers (C) in flight per thread

// the queue's sizes: caller points per A / C item, slices per B item, A items reading at once
// (A a also waits for A (a - readahead)); FVM_E2E_CHUNK, FVM_E2E_SLICES and FVM_E2E_READAHEAD
// override them when the mesh's queue is built
static int e2e_knob(const char* name, int dflt, int lo, int hi) {
    const char* v = std::getenv(name);
    if (!v) return dflt;
    const int x = std::atoi(v);
    return x < lo ? lo : x > hi ? hi : x;
}

struct E2eArgs {
    const int32_t* order;    // [nitems] item ids: A in [0, nA), B in [nA, nA + nB), C after
    const int32_t* dep_ptr;  // [nA + nB + nC + 1]
    const int32_t* dep;      // flag indices (an A or B item id)
    unsigned* flags;         // [nA + nB]: the call's epoch once the item is done
    int* counter;
    unsigned* err;
    unsigned epoch;
    int nA, nB, nitems, chunk, spi;  // chunk: caller points per A / C item; spi: slices per B item
    int64_t np, nslices;
    const int32_t* perm;   // internal -> caller
    const int32_t* iperm;  // caller -> internal
    const double* uh;      // host u (device address of the page-locked array)
    double* dh;            // host du
    double* ui;            // internal u
    double* di;            // internal du
    const int64_t* slice_ptr;
    const int32_t* width;
    const int32_t* col;
    const double* val;
    const double* b;
    const double* q;
    unsigned long long wait_ns;
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// false when the flag did not reach the epoch within the limit
__device__ bool wait_flag(const unsigned* f, unsigned epoch, unsigned long long limit_ns) {
    if (ld_acquire(f) == epoch) return true;
    const unsigned long long t0 = global_ns();
    for (;;) {
        __nanosleep(64);
        if (ld_acquire(f) == epoch) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}

// the streamed kernel's row sum (sell_row_product's order), x read through L2
template <int MAXW>
__device__ __forceinline__ double e2e_row(const E2eArgs& a, int64_t s, int lane) {
    const int64_t base = __ldg(&a.slice_ptr[s]) + lane;
    const int w = __ldg(&a.width[s]);
    double acc = 0;
    if constexpr (MAXW > 0) {
        int32_t c[MAXW];
        double v[MAXW];
#pragma unroll
        for (int k = 0; k < MAXW; ++k)
            if (k < w) {
                c[k] = __ldg(&a.col[base + (int64_t)k * 32]);
                v[k] = __ldg(&a.val[base + (int64_t)k * 32]);
            }
        double xs[MAXW];
#pragma unroll
        for (int k = 0; k < MAXW; ++k)
            if (k < w) xs[k] = __ldcg(&a.ui[c[k]]);
#pragma unroll
        for (int k = 0; k < MAXW; ++k)
            if (k < w) acc += v[k] * xs[k];
    } else {
        for (int k = 0; k < w; ++k) {
            const int64_t i = base + (int64_t)k * 32;
            const double xv = __ldcg(&a.ui[__ldg(&a.col[i])]);
            acc += __ldg(&a.val[i]) * xv;
        }
    }
    return acc;
}

template <int MAXW>
__global__ void __launch_bounds__(kE2eThreads) rhs_e2e_kernel(const E2eArgs a) {
    __shared__ int s_item;
    __shared__ int s_bad;
    const int tid = threadIdx.x;
    for (;;) {
        if (tid == 0) {
            s_item = atomicAdd(a.counter, 1);
            s_bad = 0;
        }
        __syncthreads();
        const int it = s_item;
        if (it >= a.nitems) break;  // uniform over the block
        const int w = __ldg(&a.order[it]);
        for (int d = __ldg(&a.dep_ptr[w]) + tid, d1 = __ldg(&a.dep_ptr[w + 1]); d < d1; d += kE2eThreads)
            if (!wait_flag(a.flags + __ldg(&a.dep[d]), a.epoch, a.wait_ns)) {
                atomicOr(a.err, kDevErrFlagWait);
                s_bad = 1;
            }
        __syncthreads();
        const bool bad = s_bad != 0;
        if (w < a.nA) {  // A: host u -> internal u, kE2eUnroll link loads in flight per thread
            const int64_t j0 = (int64_t)w * a.chunk;
            const int64_t j1 = j0 + a.chunk < a.np ? j0 + a.chunk : a.np;
            for (int64_t jb = j0 + tid; jb < j1; jb += kE2eThreads * kE2eUnroll) {
                double v[kE2eUnroll];
#pragma unroll
                for (int k = 0; k < kE2eUnroll; ++k) {
                    const int64_t j = jb + (int64_t)k * kE2eThreads;
                    v[k] = j < j1 ? a.uh[j] : 0.0;
                }
#pragma unroll
                for (int k = 0; k < kE2eUnroll; ++k) {
                    const int64_t j = jb + (int64_t)k * kE2eThreads;
                    if (j < j1) a.ui[__ldg(&a.iperm[j])] = v[k];
                }
            }
        } else if (w < a.nA + a.nB) {  // B: rows of slices [s0, s1)
            if (!bad) {
                const int warp = tid >> 5, lane = tid & 31;
                const int64_t s0 = (int64_t)(w - a.nA) * a.spi, s1 = s0 + a.spi < a.nslices ? s0 + a.spi : a.nslices;
                for (int64_t s = s0 + warp; s < s1; s += kE2eThreads / 32) {
                    const int64_t r = s * 32 + lane;
                    if (r >= a.np) continue;
                    double out = e2e_row<MAXW>(a, s, lane);
                    if (a.q) {
                        const double xr = __ldcg(&a.ui[r]);
                        out += a.q[r] * xr * xr;
                    }
                    if (a.b) out += a.b[r];
                    a.di[r] = out;
                }
            }
        } else if (!bad) {  // C: internal du -> host du, kE2eUnroll gathers in flight per thread
            const int64_t j0 = (int64_t)(w - a.nA - a.nB) * a.chunk;
            const int64_t j1 = j0 + a.chunk < a.np ? j0 + a.chunk : a.np;
            for (int64_t jb = j0 + tid; jb < j1; jb += kE2eThreads * kE2eUnroll) {
                double v[kE2eUnroll];
#pragma unroll
                for (int k = 0; k < kE2eUnroll; ++k) {
                    const int64_t j = jb + (int64_t)k * kE2eThreads;
                    v[k] = j < j1 ? __ldcg(&a.di[__ldg(&a.iperm[j])]) : 0.0;
                }
#pragma unroll
                for (int k = 0; k < kE2eUnroll; ++k) {
                    const int64_t j = jb + (int64_t)k * kE2eThreads;
                    if (j < j1) a.dh[j] = v[k];
                }
            }
        }
        if (w < a.nA + a.nB) {  // publish (also after a failed wait, so that no later wait hangs)
            __threadfence();
            __syncthreads();
            if (tid == 0) st_release(a.flags + w, a.epoch);
        }
        __syncthreads();  // s_item and s_bad are rewritten next
    }
}

// The queue and the lists of one mesh (host-built once, from the operator pattern and the
// permutation).
void E2ePlan::build(const fvm_mesh* m) {
    const SellPattern& p = m->pat;
    const int64_t np = m->np;
    // measured at 1M points: 4096 / 32 / 32 at 119-123 us per call; 8192 points per chunk 130 us,
    // all reads at once 139 us, 8 at once 210 us
    chunk = e2e_knob("FVM_E2E_CHUNK", 4096, 256, 1 << 20);
    spi = e2e_knob("FVM_E2E_SLICES", 32, 1, 4096);
    const int readahead = e2e_knob("FVM_E2E_READAHEAD", 32, 1, 1 << 20);
    nA = (int)((np + chunk - 1) / chunk);
    nB = (int)((p.nslices + spi - 1) / spi);
    nC = nA;
    const int nitems_ = nA + nB + nC;
    std::vector<std::vector<int32_t>> deps(nitems_);
    for (int a = readahead; a < nA; ++a) deps[a].push_back(a - readahead);  // reads in order
    std::vector<int32_t> mark(std::max(nA, nB), -1);
    for (int b = 0; b < nB; ++b) {  // the A items holding the columns of B's real rows
        auto& d = deps[nA + b];
        const int64_t s1 = std::min<int64_t>((int64_t)(b + 1) * spi, p.nslices);
        for (int64_t s = (int64_t)b * spi; s < s1; ++s)
            for (int k = 0; k < p.width[s]; ++k)
                for (int lane = 0; lane < kSlice; ++lane) {
                    if (s * kSlice + lane >= np) break;
                    const int32_t c = p.col[p.slice_ptr[s] + (int64_t)k * kSlice + lane];
                    const int a = (int)(m->perm[c] / chunk);
                    if (mark[a] != b) {
                        mark[a] = b;
                        d.push_back(a);
                    }
                }
        std::sort(d.begin(), d.end());
    }
    std::fill(mark.begin(), mark.end(), -1);
    for (int c = 0; c < nC; ++c) {  // the B items holding C's rows
        auto& d = deps[nA + nB + c];
        const int64_t j1 = std::min<int64_t>((int64_t)(c + 1) * chunk, np);
        for (int64_t j = (int64_t)c * chunk; j < j1; ++j) {
            const int b = (int)(m->iperm[j] / kSlice / spi);
            if (mark[b] != c) {
                mark[b] = c;
                d.push_back(nA + b);
            }
        }
        std::sort(d.begin(), d.end());
    }
    // queue: A in order, each B right after its last A, each C right after its last B
    std::vector<std::vector<int32_t>> after_a(nA), after_b(nB);
    for (int b = 0; b < nB; ++b) after_a[deps[nA + b].empty() ? 0 : deps[nA + b].back()].push_back(nA + b);
    std::vector<int32_t> q;
    q.reserve(nitems_);
    std::vector<int64_t> pos(nA + nB, -1);
    for (int a = 0; a < nA; ++a) {
        pos[a] = (int64_t)q.size();
        q.push_back(a);
        for (int32_t b : after_a[a]) {
            pos[b] = (int64_t)q.size();
            q.push_back(b);
        }
    }
    std::vector<std::vector<int32_t>> after(q.size());
    for (int c = 0; c < nC; ++c) {
        int64_t last = (int64_t)q.size() - 1;
        if (!deps[nA + nB + c].empty()) {
            last = 0;
            for (int32_t d : deps[nA + nB + c]) last = std::max(last, pos[d]);
        }
        after[last].push_back(nA + nB + c);
    }
    std::vector<int32_t> order;
    order.reserve(nitems_);
    for (size_t i = 0; i < q.size(); ++i) {
        order.push_back(q[i]);
        for (int32_t c : after[i]) order.push_back(c);
    }
    std::vector<int32_t> ptr(nitems_ + 1, 0), list;
    for (int i = 0; i < nitems_; ++i) {
        ptr[i + 1] = ptr[i] + (int32_t)deps[i].size();
        list.insert(list.end(), deps[i].begin(), deps[i].end());
    }
    if (list.empty()) list.push_back(0);
    nitems = nitems_;
    d_order.upload(order);
    d_dep_ptr.upload(ptr);
    d_dep.upload(list);
    d_flags.alloc(sizeof(unsigned) * (nA + nB));
    FVM_CUDA(cudaMemset(d_flags.p, 0, d_flags.bytes));
    d_counter.alloc(sizeof(int));
    epoch = 0;
    built = true;
}

template <int MAXW>
static void launch_e2e(const E2eArgs& a, cudaStream_t s) {
    static int grid = 0;
    if (!grid) {
        int per_sm = 0, sms = 0, dev = 0;
        FVM_CUDA(cudaGetDevice(&dev));
        FVM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        FVM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rhs_e2e_kernel<MAXW>, kE2eThreads, 0));
        grid = std::max(1, per_sm) * sms;
    }
    rhs_e2e_kernel<MAXW><<<(unsigned)std::min(grid, a.nitems), kE2eThreads, 0, s>>>(a);
}

bool problem_rhs_host_fused(fvm_problem* p, const double* uh, double* dh, double t, cudaStream_t s) {
    fvm_mesh* m = p->mesh;
    if (!p->linear || p->precision != FVM_FP64 || p->conditions_only || m->np == 0) return false;
    E2ePlan& P = m->e2e;
    if (!P.built) P.build(m);
    p->ensure_work();
    const double* b = p->has_b ? p->d_b.as<double>() : nullptr;
    if (p->ntime > 0) {
        launch_time_b(b, p->d_tb.as<double>(), problem_time_taus(p, t), p->ntime, p->d_beff.as<double>(), m->np, s);
        b = p->d_beff.as<double>();
    }
    if (++P.epoch == 0) {  // the epochs wrapped: clear the flags so no old value matches
        FVM_CUDA(cudaMemsetAsync(P.d_flags.p, 0, P.d_flags.bytes, s));
        P.epoch = 1;
    }
    FVM_CUDA(cudaMemsetAsync(P.d_counter.p, 0, sizeof(int), s));
    const SellPattern& pat = m->pat;
    E2eArgs a{P.d_order.as<int32_t>(), P.d_dep_ptr.as<int32_t>(), P.d_dep.as<int32_t>(), P.d_flags.as<unsigned>(),
              P.d_counter.as<int>(), device_error_word(), P.epoch, P.nA, P.nB, P.nitems, P.chunk, P.spi, m->np,
              pat.nslices, m->d_perm.as<int32_t>(), m->d_iperm.as<int32_t>(), uh, dh, p->d_u.as<double>(),
              p->d_du.as<double>(), pat.d_slice_ptr.as<int64_t>(), pat.d_width.as<int32_t>(), pat.d_col.as<int32_t>(),
              p->d_val64.as<double>(), b, p->has_q ? p->d_q.as<double>() : nullptr, kWaitLimitNs};
#define FVM_E2E_CALL(W) launch_e2e<W>(a, s)
    FVM_SELL_DISPATCH(pat.maxw, FVM_E2E_CALL)
#undef FVM_E2E_CALL
    FVM_CUDA(cudaGetLastError());
    return true;
}

}  // namespace fvm
