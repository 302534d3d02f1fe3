// Streamed sliced-ELL product with a per-row epilogue (sm_103a), shared by the RHS and
// template operators (fvm_kernels.cu) and the Krylov solver (fvm_solver.cu).
//
// An epilogue type Epi supplies, as __device__ const members:
//   skip()                      true: the whole launch does nothing (checked first)
//   Pre load(r)                 row r's operands, loaded with the slice's gathers so that
//                               their latency hides behind the previous slice's sums
//   row(r, acc, xa, pre, part)  row r's product acc (xa: the row's own x, gathered in the
//                               difference form or when kOwnX); part: per-lane scratch
//                               (NP doubles, zero-initialised)
#pragma once
#include <algorithm>
#include <cstdint>
#include <vector>

#include "fvm_internal.h"
#include "fvm_sell.cuh"
#include "fvm_tma.cuh"

namespace fvm {

// ---------------------------------------------------------------------------------------
// Streamed sliced-ELL operator (the default for slices up to 16 slots wide).
//
// A persistent grid (resident CTAs x SMs, more when a CTA's slice range would not fit its
// window); CTA c owns the contiguous slice range [nslices c / G, nslices (c+1) / G).  At start
// one bulk copy brings the range's slice offsets into shared memory, so no later step waits on
// a global load for them.  The slices are then processed in stages of NW consecutive slices,
// whose column and value slots are contiguous in HBM: one producer thread streams each stage
// into shared memory with two cp.async.bulk copies completing on the stage's `full` mbarrier,
// up to NST stages ahead of the consumers.  Consumer warp w takes slice w of each stage: it
// reads its slots from shared memory (lane = row, conflict-free), gathers x, releases the
// stage (`empty` mbarrier) and finishes the row while the next copies land.  When x is
// 16-byte aligned the launch runs one CTA of 16 consumer warps per SM and the CTA first
// bulk-copies its own rows of x into shared memory: on a Hilbert-ordered mesh almost every
// gather then reads shared memory, the rest go through L1/L2.  Otherwise two CTAs of 8
// consumer warps per SM gather through L1/L2, with the CTA's x rows prefetched into L2.
// The sum runs over the slots in the same order as sell_row_product; the stage loop is
// software-pipelined so that gathers overlap the previous slice's sums.
// ---------------------------------------------------------------------------------------
struct StreamArgs {
    const int64_t* slice_ptr;  // nslices + 1 offsets, padded with two more
    const int32_t* col;
    const void* val;
    const void* xg;            // the gathered vector
    unsigned* err;             // device error word (bits kDevErr*)
    int64_t nrows, nslices;
    int nst;    // pipeline stages held in shared memory
    int spwin;  // slice offsets held per CTA: its range plus alignment slack, a multiple of 16
    int xb;     // bytes of shared memory holding the CTA's own rows of x (0: gathers via L1/L2)
    // limit of a consumer's wait for a stage to land (kWaitLimitNs), and a delay of the producer
    // before its second stage (0): the fault-path test shortens the one and sets the other so
    // that the wait runs out, the CTA stops and the error word reports it
    unsigned long long wait_ns, producer_delay_ns;
};

constexpr int kSpWindowMax = 1024;

// First-stage slot range of each CTA, passed with the launch so that the producer issues the
// first bulk copies without waiting on a global load of the slice offsets (after an L2 flush
// that load is a DRAM round trip on the start-up path).  n = 0: not provided.
constexpr int kStage0Max = 640;
struct Stage0Table {
    int n;
    int32_t c0[kStage0Max], c1[kStage0Max];
};

template <class V, int MAXW, int NW>
struct StreamLayout {
    static constexpr int kSlots = NW * MAXW * kSlice;  // slots per stage
    static constexpr size_t kStageBytes = (size_t)kSlots * (sizeof(int32_t) + sizeof(V));
    __host__ __device__ static size_t sp_offset(int nst) { return (size_t)nst * kStageBytes; }
    __host__ __device__ static size_t x_offset(int nst, int spwin) {
        return sp_offset(nst) + (size_t)spwin * sizeof(int64_t);
    }
    __host__ __device__ static size_t bar_offset(int nst, int spwin, int xb) { return x_offset(nst, spwin) + xb; }
    __host__ __device__ static size_t bytes(int nst, int spwin, int xb) {
        return bar_offset(nst, spwin, xb) + (2 * (size_t)nst + 2) * sizeof(uint64_t);
    }
};

// one consumer warp's slice between its fetch and its sums (registers)
template <class Acc, int MAXW, class Pre>
struct SliceRegs {
    Acc x[MAXW];  // gathered x of the lane's slots
    Acc xa;       // the row's own x (difference form, or an epilogue that reads it)
    Pre pre;      // the epilogue's operands of the row
    int64_t r;    // row
    int st;       // stage buffer
    int off;      // shared-memory slot of the lane's first entry
    int cw;       // slots in the slice
    bool have;
};

// slices up to 8 slots wide are software-pipelined (two slices in registers per warp, two
// CTAs per SM); wider ones are summed as soon as they are fetched
template <int MAXW>
constexpr bool kStreamPipelined = MAXW <= 8;

template <class V, class Acc, class X, bool DIFF, int MAXW, int NW, class Epi>
__global__ void __launch_bounds__((NW + 1) * 32, kStreamPipelined<MAXW> && NW <= 8 ? 2 : 1)
    sell_stream_kernel(StreamArgs a, const __grid_constant__ Stage0Table t0, const __grid_constant__ Epi e) {
    using L = StreamLayout<V, MAXW, NW>;
    if (e.skip()) return;  // uniform over the grid (e.g. a converged Krylov iteration)
    extern __shared__ __align__(128) unsigned char smem[];
    const int nst = a.nst;
    int32_t* colbuf = reinterpret_cast<int32_t*>(smem);
    V* valbuf = reinterpret_cast<V*>(smem + (size_t)nst * L::kSlots * sizeof(int32_t));
    int64_t* spw = reinterpret_cast<int64_t*>(smem + L::sp_offset(nst));
    X* xs = reinterpret_cast<X*>(smem + L::x_offset(nst, a.spwin));
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + L::bar_offset(nst, a.spwin, a.xb));
    uint64_t* empty = full + nst;
    uint64_t* spbar = empty + nst;
    uint64_t* xbar = spbar + 1;
    __shared__ volatile int abort_flag;  // a consumer gave up: the producer stops issuing stages
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t G = gridDim.x;
    const int64_t sb = a.nslices * (int64_t)blockIdx.x / G, se = a.nslices * ((int64_t)blockIdx.x + 1) / G;
    const int64_t nstage = (se - sb + NW - 1) / NW;
    // window of slice offsets: from sb rounded down to even (16-byte aligned), an even count
    // covering sp[sb .. se]; the launcher keeps it within a.spwin entries and the array is
    // padded so that the rounded-up end stays inside it
    const int64_t w0 = sb & ~(int64_t)1;
    const uint32_t wcount = (uint32_t)(((se + 1 - w0) + 1) & ~(int64_t)1);
    // the CTA's own rows of x, staged once in shared memory (whole 16-byte units; the launcher
    // sizes a.xb for the longest range and checks the alignment of x): most gathers of a
    // Hilbert-ordered mesh fall inside the range and read shared memory instead of L1/L2
    const int64_t xr0 = sb * kSlice;
    uint32_t xbytes = 0;
    if (a.xb) {
        const int64_t r1 = min(se * kSlice, a.nrows);
        xbytes = r1 > xr0 ? (uint32_t)(((r1 - xr0) * (int64_t)sizeof(X)) & ~(int64_t)15) : 0u;
    }
    const uint64_t xcnt = xbytes / sizeof(X);
    if (threadIdx.x == 0) {
        abort_flag = 0;
        for (int i = 0; i < nst; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], NW);
        }
        mbar_init(spbar, 1);
        mbar_init(xbar, 1);
        mbar_init_fence();
        mbar_arrive_expect_tx(spbar, wcount * (uint32_t)sizeof(int64_t));
        bulk_copy_g2s(spw, a.slice_ptr + w0, wcount * (uint32_t)sizeof(int64_t), spbar);
        if (xbytes) {
            mbar_arrive_expect_tx(xbar, xbytes);
            bulk_copy_g2s(xs, (const X*)a.xg + xr0, xbytes, xbar);
        } else {
            mbar_arrive(xbar);
        }
    }
    __syncthreads();

    if (warp == NW) {  // producer
        if (lane != 0 || nstage == 0) return;
        // streams stage k (slots [c0, c1)) into its buffer once the buffer is free
        auto issue = [&](int64_t k, int64_t c0, int64_t c1) -> bool {
            const int st = (int)(k % nst);
            if (abort_flag) return false;
            if (k >= nst && !mbar_wait_for(&empty[st], (uint32_t)((k / nst - 1) & 1), kWaitLimitNs, &abort_flag))
                return false;
            const uint32_t n = (uint32_t)(c1 - c0);  // <= kSlots: NW slices of at most MAXW slots
            if (n == 0) {  // slices without slots: nothing to copy
                mbar_arrive(&full[st]);
                return true;
            }
            mbar_arrive_expect_tx(&full[st], n * (uint32_t)(sizeof(int32_t) + sizeof(V)));
            bulk_copy_g2s(colbuf + (size_t)st * L::kSlots, a.col + c0, n * (uint32_t)sizeof(int32_t), &full[st]);
            bulk_copy_g2s(valbuf + (size_t)st * L::kSlots, (const V*)a.val + c0, n * (uint32_t)sizeof(V), &full[st]);
            return true;
        };
        // the x entries of this CTA's rows into L2: the gathers of the CTA and of its
        // neighbours in the Hilbert order then hit L2 instead of HBM
        if (!a.xb) {  // a hint: the range is shrunk to 16-byte boundaries (x may be any caller's array)
            const uintptr_t p0 = (uintptr_t)((const X*)a.xg + sb * kSlice);
            const uintptr_t p1 = (uintptr_t)((const X*)a.xg + min(se * kSlice, a.nrows));
            const uintptr_t q0 = (p0 + 15) & ~(uintptr_t)15, q1 = p1 & ~(uintptr_t)15;
            if (q1 > q0) bulk_prefetch_l2((const void*)q0, (uint32_t)(q1 - q0));
        }
        // stage 0 from the launch's table, else from two global loads, in parallel with the
        // window copy
        bool ok = (int)blockIdx.x < t0.n ? issue(0, t0.c0[blockIdx.x], t0.c1[blockIdx.x])
                                         : issue(0, __ldg(&a.slice_ptr[sb]), __ldg(&a.slice_ptr[min(sb + NW, se)]));
        int64_t issued = ok ? 1 : 0;
        if (ok && !mbar_wait(spbar, 0)) ok = false;
        if (a.producer_delay_ns) {  // fault-path test only: hold back the second stage
            const unsigned long long d0 = global_ns();
            while (global_ns() - d0 < a.producer_delay_ns) {
            }
        }
        const int64_t* sp = spw - w0;
        for (int64_t k = 1; ok && k < nstage; ++k) {
            const int64_t s0 = sb + k * NW;
            if ((ok = issue(k, sp[s0], sp[min(s0 + NW, se)]))) issued = k + 1;
        }
        if (!ok || abort_flag) {  // a wait ran out here or in a consumer
            if (!ok && !abort_flag) atomicOr(a.err, kDevErrEmptyWait);
            // wait (bounded) for the copies already issued into the stages still in flight
            for (int64_t j = (issued > nst ? issued - nst : 0); j < issued; ++j)
                mbar_wait(&full[j % nst], (uint32_t)((j / nst) & 1));
            mbar_wait(xbar, 0);
        }
        return;
    }

    bool ok = mbar_wait(spbar, 0) && mbar_wait(xbar, 0);
    const int64_t* sp = spw - w0;  // sp[s] for s in [w0, w0 + wcount)
    double part[Epi::NP > 0 ? Epi::NP : 1] = {};  // per-lane epilogue scratch

    // consumers, software-pipelined by one stage: the gathers of stage k + 1 are in flight
    // while the FP64 sums of stage k run.  A warp holds two stages at a time (the one it
    // sums, the one it gathers for), so a CTA needs at least four.
    const X* __restrict__ xg = (const X*)a.xg;
    const V* __restrict__ vb0 = valbuf;
    auto gather = [&](int64_t c) -> Acc {
        const uint64_t rel = (uint64_t)(c - xr0);
        return rel < xcnt ? (Acc)xs[rel] : (Acc)__ldg(&xg[c]);
    };
    // waits for stage k, reads this warp's columns from shared memory and issues its gathers;
    // false when the wait ran out
    using Regs = SliceRegs<Acc, MAXW, typename Epi::Pre>;
    auto fetch = [&](int64_t k, Regs& R) -> bool {
        const int64_t s0 = sb + k * NW, s = s0 + warp;
        R.have = s < se;
        R.r = s * kSlice + lane;
        R.st = (int)(k % nst);
        R.cw = 0;
        R.xa = 0;
        if ((DIFF || Epi::kOwnX) && R.have) R.xa = gather(R.r < a.nrows ? R.r : a.nrows - 1);
        if (!mbar_wait_for(&full[R.st], (uint32_t)((k / nst) & 1), a.wait_ns, &abort_flag)) {
            abort_flag = 1;
            return false;
        }
        if (R.have) {
            const int64_t cb = sp[s];
            R.cw = (int)((sp[s + 1] - cb) / kSlice);
            R.off = R.st * L::kSlots + (int)(cb - sp[s0]) + lane;
            int32_t c[MAXW];
#pragma unroll
            for (int j = 0; j < MAXW; ++j)
                if (j < R.cw) c[j] = colbuf[R.off + j * kSlice];
#pragma unroll
            for (int j = 0; j < MAXW; ++j)
                if (j < R.cw) R.x[j] = gather(c[j]);
            if (R.r < a.nrows) R.pre = e.load(R.r);
        }
        return true;
    };
    // sums the slice with its values from shared memory (slot order, one FMA per slot: the
    // FP64 pipe is the kernel's floor), releases the stage and writes the lane's row
    auto finish = [&](const Regs& R) {
        Acc acc = 0;
        if (R.have) {
#pragma unroll
            for (int j = 0; j < MAXW; ++j)
                if (j < R.cw) {
                    const Acc v = (Acc)vb0[R.off + j * kSlice];
                    if constexpr (DIFF)
                        acc += v * (R.x[j] - R.xa);
                    else
                        acc += v * R.x[j];
                }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[R.st]);
        if (!R.have || R.r >= a.nrows) return;
        e.row(R.r, acc, R.xa, R.pre, part);
    };
    if constexpr (kStreamPipelined<MAXW>) {
        Regs A, B;
        ok = ok && (nstage == 0 || fetch(0, A));
        for (int64_t k = 0; ok && k < nstage; k += 2) {
            // A holds stage k
            if (k + 1 < nstage) ok = fetch(k + 1, B);
            finish(A);
            if (!ok || k + 1 >= nstage) break;
            // B holds stage k + 1
            if (k + 2 < nstage) ok = fetch(k + 2, A);
            finish(B);
        }
    } else {
        Regs A;
        for (int64_t k = 0; ok && k < nstage; ++k)
            if ((ok = fetch(k, A))) finish(A);
    }
    if (!ok && lane == 0) atomicOr(a.err, kDevErrFullWait);
}

constexpr int kStreamWarps = 8;

// Launch shape of one instantiation on one device: CTAs per SM.  The most consumer warps per
// SM wins, provided each CTA still holds enough stages with the largest slice-offset window
// (four for the software-pipelined widths, whose warps hold two stages each; three otherwise).
// The pipeline depth of a launch then fills the CTA's share of shared memory around its
// actual window.
struct StreamShape {
    int dev = -1, sms = 0, ctas = 0;
    long budget = 0;  // shared memory bytes per CTA
};

// Launch shape for NW consumer warps: CTAs per SM and the shared memory budget of a CTA.
// xstage: the CTA also stages its rows of x; one CTA per SM (the widest contiguous range, the
// fewest gathers outside it).  Returns false when the pipeline does not fit that way.
template <class V, class Acc, class X, bool DIFF, int MAXW, int NW, class Epi>
static bool launch_stream(const StreamArgs& a0, const std::vector<int64_t>& hsp, bool xstage, const Epi& e,
                          cudaStream_t s) {
    using L = StreamLayout<V, MAXW, NW>;
    auto kern = sell_stream_kernel<V, Acc, X, DIFF, MAXW, NW, Epi>;
    const int threads = (NW + 1) * 32;
    const long need = kStreamPipelined<MAXW> ? 4 : 3;
    static StreamShape shape;  // per instantiation
    int dev = 0;
    FVM_CUDA(cudaGetDevice(&dev));
    if (shape.dev != dev) {
        int smem_sm = 0, smem_cta = 0, reserved = 0, sms = 0;
        FVM_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
        FVM_CUDA(cudaDeviceGetAttribute(&smem_cta, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        FVM_CUDA(cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev));
        FVM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        // static shared memory (an epilogue's reduction scratch) comes out of the same budget
        cudaFuncAttributes fa;
        FVM_CUDA(cudaFuncGetAttributes(&fa, kern));
        const int dyn_max = smem_cta - (int)fa.sharedSizeBytes;
        FVM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_max));
        StreamShape best;
        for (int ctas = xstage ? 1 : 4; ctas >= 1 && best.ctas == 0; --ctas) {
            const long budget =
                std::min<long>(smem_sm / ctas - reserved - (long)fa.sharedSizeBytes, dyn_max);
            const long nst = (budget - (long)L::bytes(0, kSpWindowMax, 0)) / (long)L::kStageBytes;
            if (nst < (ctas == 1 && !kStreamPipelined<MAXW> ? 2 : need)) continue;
            int fit = 0;
            FVM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, kern, threads, (size_t)budget));
            if (fit >= ctas) best = {dev, sms, ctas, budget};
        }
        if (best.ctas == 0) {
            if (xstage) return false;
            fail(FVM_ERR_CUDA, "streamed operator kernel does not fit on an SM");
        }
        shape = best;
    }
    StreamArgs a = a0;
    // every CTA's range (ceil(nslices / G) slices, at most 3 more window entries after the
    // alignment rounding) must fit the window
    const int64_t stages = (a.nslices + NW - 1) / NW;
    int64_t grid = std::min<int64_t>((int64_t)shape.ctas * shape.sms, stages);
    grid = std::max<int64_t>(grid, (a.nslices + (kSpWindowMax - 4) - 1) / (kSpWindowMax - 4));
    grid = std::max<int64_t>(grid, 1);
    const int64_t range = (a.nslices + grid - 1) / grid;
    a.spwin = (int)std::min<int64_t>(kSpWindowMax, ((range + 3) + 15) & ~(int64_t)15);
    a.xb = 0;
    if (xstage) {
        a.xb = (int)(((range * kSlice * (int64_t)sizeof(X)) + 15) & ~(int64_t)15);
        const long nst = (shape.budget - (long)L::bytes(0, a.spwin, a.xb)) / (long)L::kStageBytes;
        if (nst < need) return false;
    }
    a.nst = (int)std::min<long>(6, (shape.budget - (long)L::bytes(0, a.spwin, a.xb)) / (long)L::kStageBytes);
    Stage0Table t0;  // copied into the launch's parameters
    t0.n = 0;
    if (grid <= kStage0Max && (int64_t)hsp.size() == a.nslices + 1 && hsp.back() < ((int64_t)1 << 31)) {
        for (int64_t c = 0; c < grid; ++c) {
            const int64_t sb = a.nslices * c / grid, se = a.nslices * (c + 1) / grid;
            t0.c0[c] = (int32_t)hsp[sb];
            t0.c1[c] = (int32_t)hsp[std::min(sb + NW, se)];
        }
        t0.n = (int)grid;
    }
    kern<<<(unsigned)grid, threads, L::bytes(a.nst, a.spwin, a.xb), s>>>(a, t0, e);
    return true;
}

// x staged in shared memory needs a 16-byte aligned x (bulk copies)
static bool stream_xstage(const void* xg) { return ((uintptr_t)xg & 15) == 0; }

template <class V, class Acc, class X, bool DIFF, int MAXW, class Epi>
static void launch_stream_any(const StreamArgs& a, const std::vector<int64_t>& hsp, const Epi& e, cudaStream_t s) {
    if (stream_xstage(a.xg) && launch_stream<V, Acc, X, DIFF, MAXW, 2 * kStreamWarps, Epi>(a, hsp, true, e, s)) return;
    launch_stream<V, Acc, X, DIFF, MAXW, kStreamWarps, Epi>(a, hsp, false, e, s);
}


}  // namespace fvm
