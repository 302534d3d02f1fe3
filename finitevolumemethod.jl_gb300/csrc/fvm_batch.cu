// Batched instances: B copies of one linear problem that differ in their diffusion field.
//
// State is [npoints][batch] with the batch index fastest, in the internal numbering.  The
// operator of instance b is A_b = C + sum_m coef_m D_b[idx_m] entrywise: the coefficients and
// the constant part come from the problem's linear terms (fvm_visit_linear_terms) and are the
// same for every instance, so the per-instance values are assembled on the device in one
// kernel from the per-instance D fields.  The batched operator runs one warp per (row, chunk
// of 32*VEC instances): the row's columns are warp-uniform (read once, broadcast), values and
// gathered u are consecutive across lanes (coalesced), and the mesh is read once for all
// instances.  Launch shape (block size, instances per thread) is picked by timing the
// candidates on the first call (cached per shape, optionally in the file named by
// FVM_AUTOTUNE_CACHE).
#include "fvm_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>

struct fvm_batch {
    fvm_problem* prob = nullptr;
    int B = 0;
    int precision = FVM_FP64;
    int64_t np = 0, nnz = 0;
    fvm::DBuf d_rowptr, d_col, d_val, d_b, d_q;
    fvm::DBuf d_dir_idx, d_dir_val;
    int64_t ndir = 0;
    fvm::DBuf d_work;  // caller-numbered IO staging: 3 x [np][B]
    fvm::BatchOp op;
};

namespace fvm {
namespace {

static inline unsigned blocks(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

// per-instance values: val[k][b] = cst[k] + sum_{m in map[k]} coef[m] * D[idx[m]][b]
template <class T>
__global__ void batch_assemble_kernel(const int64_t* __restrict__ mptr, const int32_t* __restrict__ midx,
                                      const double* __restrict__ mcoef, const double* __restrict__ cst,
                                      const double* __restrict__ D, T* __restrict__ val, int64_t nnz, int B) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nnz * B) return;
    int64_t k = i / B;
    int b = (int)(i - k * B);
    double v = cst[k];
    for (int64_t m = mptr[k]; m < mptr[k + 1]; ++m) v += mcoef[m] * D[(int64_t)midx[m] * B + b];
    val[i] = (T)v;
}

template <class T, int VEC>
struct Vec;
template <>
struct Vec<float, 1> { using type = float; };
template <>
struct Vec<float, 2> { using type = float2; };
template <>
struct Vec<float, 4> { using type = float4; };
template <>
struct Vec<double, 1> { using type = double; };
template <>
struct Vec<double, 2> { using type = double2; };

template <class T, int VEC>
__device__ __forceinline__ void vload(const T* p, T (&x)[VEC]) {
    using V = typename Vec<T, VEC>::type;
    V v = __ldg(reinterpret_cast<const V*>(p));
    const T* e = reinterpret_cast<const T*>(&v);
#pragma unroll
    for (int j = 0; j < VEC; ++j) x[j] = e[j];
}
template <class T, int VEC>
__device__ __forceinline__ void vstore(T* p, const T (&x)[VEC]) {
    using V = typename Vec<T, VEC>::type;
    V v;
    T* e = reinterpret_cast<T*>(&v);
#pragma unroll
    for (int j = 0; j < VEC; ++j) e[j] = x[j];
    *reinterpret_cast<V*>(p) = v;
}

// du[r][b] = sum_k val[k][b] u[col_k][b] + bvec[r] + q[r] u[r][b]^2 over the chunk of instances
// of each (row, chunk of 32 * VEC instances) work item; grid-stride over items (a persistent grid).
// EPI: the row's linear combination E (BatchEpi) is formed from the fresh product in the same
// pass; du may then be null (the product is not stored).
template <class T, int VEC, bool EPI = false>
__global__ void __launch_bounds__(512) batch_op_kernel(const int64_t* __restrict__ rowptr,
                                                       const int32_t* __restrict__ col, const T* __restrict__ val,
                                                       const T* __restrict__ u, T* __restrict__ du,
                                                       const T* __restrict__ bvec, const T* __restrict__ q, int64_t n,
                                                       int B, int64_t nchunk, BatchEpi<T> E = {}) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t item = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; item < n * nchunk; item += nwarp) {
        const int64_t r = item / nchunk;
        const int64_t b0 = ((item - r * nchunk) * 32 + lane) * VEC;
        if (b0 >= B) continue;
        T acc[VEC];
#pragma unroll
        for (int j = 0; j < VEC; ++j) acc[j] = 0;
        const int64_t k0 = __ldg(&rowptr[r]), k1 = __ldg(&rowptr[r + 1]);
        int64_t k = k0;
        for (; k + 1 < k1; k += 2) {  // two entries in flight
            const int32_t c0 = __ldg(&col[k]), c1 = __ldg(&col[k + 1]);
            T v0[VEC], v1[VEC], x0[VEC], x1[VEC];
            vload<T, VEC>(val + k * B + b0, v0);
            vload<T, VEC>(val + (k + 1) * B + b0, v1);
            vload<T, VEC>(u + (int64_t)c0 * B + b0, x0);
            vload<T, VEC>(u + (int64_t)c1 * B + b0, x1);
#pragma unroll
            for (int j = 0; j < VEC; ++j) {  // one fused multiply-add per entry (FP64 issue is scarce)
                acc[j] += v0[j] * x0[j];
                acc[j] += v1[j] * x1[j];
            }
        }
        if (k < k1) {
            const int32_t c0 = __ldg(&col[k]);
            T v0[VEC], x0[VEC];
            vload<T, VEC>(val + k * B + b0, v0);
            vload<T, VEC>(u + (int64_t)c0 * B + b0, x0);
#pragma unroll
            for (int j = 0; j < VEC; ++j) acc[j] += v0[j] * x0[j];
        }
        if (bvec) {
            const T bb = bvec[r];
#pragma unroll
            for (int j = 0; j < VEC; ++j) acc[j] += bb;
        }
        if (q) {
            const T qq = q[r];
            T ur[VEC];
            vload<T, VEC>(u + r * B + b0, ur);
#pragma unroll
            for (int j = 0; j < VEC; ++j) acc[j] += qq * ur[j] * ur[j];
        }
        if (!EPI || du) vstore<T, VEC>(du + r * B + b0, acc);
        if constexpr (EPI) {  // z = x0 + sum_t c_t v_t in list order, the fresh product where v_t is null
            T z[VEC];
            if (E.x0) {
                vload<T, VEC>(E.x0 + r * B + b0, z);
            } else {
#pragma unroll
                for (int j = 0; j < VEC; ++j) z[j] = 0;
            }
            for (int t = 0; t < E.nv; ++t) {
                T v[VEC];
                if (E.v[t]) {
                    vload<T, VEC>(E.v[t] + r * B + b0, v);
                } else {
#pragma unroll
                    for (int j = 0; j < VEC; ++j) v[j] = acc[j];
                }
                const T c = (T)E.c[t];
#pragma unroll
                for (int j = 0; j < VEC; ++j) z[j] += c * v[j];
            }
            vstore<T, VEC>(E.z + r * B + b0, z);
        }
    }
}

template <class T>
__global__ void batch_dirichlet_kernel(const int32_t* __restrict__ idx, const double* __restrict__ v, T* __restrict__ u,
                                       int64_t nd, int B) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nd * B) return;
    int64_t k = i / B;
    u[(int64_t)idx[k] * B + (i - k * B)] = (T)v[k];
}

// rows of [n][B]: out[r] = in[perm[r]] (gather) or out[perm[r]] = in[r] (scatter), with cast
template <class S, class D>
__global__ void batch_permute_kernel(const int32_t* __restrict__ perm, const S* __restrict__ in, D* __restrict__ out,
                                     int64_t n, int B, int gather) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * B) return;
    int64_t r = i / B, b = i - r * B;
    int64_t pr = perm[r];
    if (gather)
        out[i] = (D)in[pr * B + b];
    else
        out[pr * B + b] = (D)in[i];
}

// Tsit5 stage on [n*B] vectors: y = u + dt sum_j a_j k_j
template <class T>
struct BStage {
    const T* k[7];
    double a[7];
};
template <class T>
__global__ void batch_stage_kernel(T* y, const T* u, BStage<T> s, int nk, T dt, int64_t n) {  // y may be u
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    T acc = 0;
#pragma unroll
    for (int j = 0; j < 7; ++j)
        if (j < nk) acc += (T)s.a[j] * s.k[j][i];
    y[i] = u[i] + dt * acc;
}

// ---- launch shape autotuning ---------------------------------------------------------------
struct TuneKey {
    int64_t n, nnz;
    int B, prec;
    bool operator<(const TuneKey& o) const {
        return std::tie(n, nnz, B, prec) < std::tie(o.n, o.nnz, o.B, o.prec);
    }
};
struct TuneVal {
    int block, vec;
    int64_t grid;
};
std::mutex g_tune_mutex;
std::map<TuneKey, TuneVal> g_tune;
bool g_tune_loaded = false;

void tune_cache_load() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const char* f = std::getenv("FVM_AUTOTUNE_CACHE");
    if (!f) return;
    std::ifstream in(f);
    std::string line;
    while (std::getline(in, line)) {
        std::istringstream ss(line);
        TuneKey k;
        TuneVal v;
        if (ss >> k.n >> k.nnz >> k.B >> k.prec >> v.block >> v.vec >> v.grid) g_tune[k] = v;
    }
}
void tune_cache_store(const TuneKey& k, const TuneVal& v) {
    const char* f = std::getenv("FVM_AUTOTUNE_CACHE");
    if (!f) return;
    std::ofstream out(f, std::ios::app);
    out << k.n << ' ' << k.nnz << ' ' << k.B << ' ' << k.prec << ' ' << v.block << ' ' << v.vec << ' ' << v.grid << '\n';
}

template <class T>
void launch_op(const BatchOp& op, int block, int vec, int64_t grid, const T* u, T* du, cudaStream_t s) {
    const int64_t chunk = 32 * (int64_t)vec;
    const int64_t nchunk = (op.B + chunk - 1) / chunk;
    const T* bv = (const T*)op.b;
    const T* qv = (const T*)op.q;
    const T* val = (const T*)op.val;
    unsigned g = (unsigned)grid;
    if (vec == 4 && sizeof(T) == 4)
        batch_op_kernel<T, (sizeof(T) == 4 ? 4 : 2)><<<g, block, 0, s>>>(op.rowptr, op.col, val, u, du, bv, qv, op.np,
                                                                      op.B, nchunk);
    else if (vec == 2)
        batch_op_kernel<T, 2><<<g, block, 0, s>>>(op.rowptr, op.col, val, u, du, bv, qv, op.np, op.B, nchunk);
    else
        batch_op_kernel<T, 1><<<g, block, 0, s>>>(op.rowptr, op.col, val, u, du, bv, qv, op.np, op.B, nchunk);
}

int64_t persistent_grid(int block, int64_t items_warps) {
    int dev = 0, sms = 1, maxthr = 2048;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&maxthr, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
    int64_t full = (int64_t)sms * std::max(1, maxthr / block);
    int64_t need = (items_warps * 32 + block - 1) / block;
    return std::max<int64_t>(1, std::min(full, need));
}

// Widest vector (instances per thread) that the addresses of u and du allow, up to 16 bytes.
template <class T>
int max_vec_for(const void* a, const void* b) {
    const uintptr_t x = (uintptr_t)a | (uintptr_t)b;
    int v = 1;
    while (sizeof(T) * v * 2 <= 16 && x % (sizeof(T) * v * 2) == 0) v *= 2;
    return v;
}

// Times the candidate shapes on the real buffers (3 launches each) and keeps the fastest.
template <class T>
void autotune(BatchOp& op, const T* u, T* du, cudaStream_t s) {
    if (op.tuned) return;
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    tune_cache_load();
    TuneKey key{op.np, op.nnz, op.B, op.precision};
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
        op.block = it->second.block;
        op.vec = it->second.vec;
        op.grid = it->second.grid;
        op.tuned = true;
        return;
    }
    const int vmax = std::min(sizeof(T) == 4 ? 4 : 2, max_vec_for<T>(u, du));
    cudaEvent_t e0, e1;
    FVM_CUDA(cudaEventCreate(&e0));
    FVM_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    TuneVal bestv{256, 1, 1};
    for (int vec = 1; vec <= vmax; vec *= 2) {
        if (op.B % vec) continue;
        for (int block : {128, 256, 512}) {
            int64_t nchunk = (op.B + 32 * vec - 1) / (32 * vec);
            int64_t grid = persistent_grid(block, op.np * nchunk);
            launch_op<T>(op, block, vec, grid, u, du, s);  // warm
            FVM_CUDA(cudaEventRecord(e0, s));
            for (int r = 0; r < 3; ++r) launch_op<T>(op, block, vec, grid, u, du, s);
            FVM_CUDA(cudaEventRecord(e1, s));
            FVM_CUDA(cudaEventSynchronize(e1));
            float ms = 0;
            FVM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < best) {
                best = ms;
                bestv = {block, vec, grid};
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    op.block = bestv.block;
    op.vec = bestv.vec;
    op.grid = bestv.grid;
    op.tuned = true;
    g_tune[key] = bestv;
    tune_cache_store(key, bestv);
}

template <class T>
void batch_rhs_internal(fvm_batch* bt, const T* u, T* du, cudaStream_t s) {
    batch_op_apply<T>(bt->op, u, du, s);
}

template <class T>
void batch_dirichlet(fvm_batch* bt, T* u, cudaStream_t s) {
    if (bt->ndir)
        batch_dirichlet_kernel<T><<<blocks(bt->ndir * bt->B, 256), 256, 0, s>>>(
            bt->d_dir_idx.as<int32_t>(), bt->d_dir_val.as<double>(), u, bt->ndir, bt->B);
}

// Tsitouras (2011) tableau
const double kA[7][6] = {
    {0, 0, 0, 0, 0, 0},
    {0.161, 0, 0, 0, 0, 0},
    {-0.008480655492356989, 0.335480655492357, 0, 0, 0, 0},
    {2.897153057105493, -6.359448489975075, 4.3622954328695815, 0, 0, 0},
    {5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525, 0, 0},
    {5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383, 0},
    {0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774},
};

template <class T>
void stage(T* y, const T* u, T* const* k, int sidx, double dt, int64_t n, cudaStream_t s) {
    BStage<T> st;
    for (int j = 0; j < 7; ++j) {
        st.k[j] = j < sidx ? k[j] : nullptr;
        st.a[j] = j < sidx ? kA[sidx][j] : 0.0;
    }
    batch_stage_kernel<T><<<blocks(n, 256), 256, 0, s>>>(y, u, st, sidx, (T)dt, n);
}

// Fixed-step Tsit5 on the whole batch; u in place.  The Dirichlet update follows every step
// and the first step re-evaluates the FSAL derivative after it (later updates rewrite the same
// constant values).  Steps 2 .. n-1 replay one captured graph.
template <class T>
void batch_tsit5(fvm_batch* bt, T* u, T* work, int64_t nsteps, double dt, bool use_graph, cudaStream_t s) {
    const int64_t n = bt->np * bt->B;
    T* y = work;
    T* k[7];
    for (int j = 0; j < 7; ++j) k[j] = work + (1 + j) * n;
    auto f = [&](const T* x, T* out) { batch_rhs_internal<T>(bt, x, out, s); };
    auto one_step = [&](double h) {
        for (int sidx = 1; sidx < 6; ++sidx) {
            stage<T>(y, u, k, sidx, h, n, s);
            f(y, k[sidx]);
        }
        stage<T>(u, u, k, 6, h, n, s);
        f(u, k[0]);
        batch_dirichlet<T>(bt, u, s);
    };
    f(u, k[0]);
    if (nsteps <= 0) return;
    one_step(dt);
    if (bt->ndir) f(u, k[0]);  // the first Dirichlet update may change u
    int64_t done = 1;
    if (use_graph && nsteps > 1) {
        cudaGraph_t graph;
        cudaGraphExec_t exec;
        FVM_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        one_step(dt);
        FVM_CUDA(cudaStreamEndCapture(s, &graph));
        FVM_CUDA(cudaGraphInstantiate(&exec, graph, 0));
        for (; done < nsteps; ++done) FVM_CUDA(cudaGraphLaunch(exec, s));
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
    }
    for (; done < nsteps; ++done) one_step(dt);
}

}  // namespace

template <class T>
void batch_op_apply_epi(BatchOp& op, const T* u, T* du, const BatchEpi<T>& E, cudaStream_t s) {
    if (((uintptr_t)u | (uintptr_t)du | (uintptr_t)E.z) % sizeof(T))
        fail(FVM_ERR_INVALID_ARGUMENT, "batched state arrays must be aligned to their element size");
    if (!E.z || E.nv > 8) fail(FVM_ERR_INVALID_ARGUMENT, "bad batched epilogue");
    autotune<T>(op, u, du ? du : E.z, s);
    uintptr_t addr = (uintptr_t)u | (uintptr_t)E.z | (uintptr_t)E.x0 | (uintptr_t)du;
    for (int t = 0; t < E.nv; ++t) addr |= (uintptr_t)E.v[t];
    const int vec = std::min(op.vec, max_vec_for<T>((const void*)addr, (const void*)addr));
    const int64_t chunk = 32 * (int64_t)vec;
    const int64_t nchunk = (op.B + chunk - 1) / chunk;
    const unsigned g = (unsigned)op.grid;
    const T* val = (const T*)op.val;
    const T* bv = (const T*)op.b;
    const T* qv = (const T*)op.q;
    if (vec == 2)
        batch_op_kernel<T, 2, true><<<g, op.block, 0, s>>>(op.rowptr, op.col, val, u, du, bv, qv, op.np, op.B, nchunk, E);
    else
        batch_op_kernel<T, 1, true><<<g, op.block, 0, s>>>(op.rowptr, op.col, val, u, du, bv, qv, op.np, op.B, nchunk, E);
}
template void batch_op_apply_epi<double>(BatchOp&, const double*, double*, const BatchEpi<double>&, cudaStream_t);

template <class T>
void batch_op_apply(BatchOp& op, const T* u, T* du, cudaStream_t s) {
    if (((uintptr_t)u | (uintptr_t)du) % sizeof(T))
        fail(FVM_ERR_INVALID_ARGUMENT, "batched state arrays must be aligned to their element size");
    autotune<T>(op, u, du, s);
    // the grid-stride loop covers every item for any grid, so a narrower vector is always valid
    const int vec = std::min(op.vec, max_vec_for<T>(u, du));
    launch_op<T>(op, op.block, vec, op.grid, u, du, s);
}
template void batch_op_apply<float>(BatchOp&, const float*, float*, cudaStream_t);
template void batch_op_apply<double>(BatchOp&, const double*, double*, cudaStream_t);

void launch_batch_assemble(const int64_t* mptr, const int32_t* midx, const double* mcoef, const double* cst,
                           const double* D, void* val, int64_t nnz, int B, int precision, cudaStream_t s) {
    if (nnz * B == 0) return;
    const unsigned g = blocks(nnz * B, 256);
    if (precision == FVM_FP32)
        batch_assemble_kernel<float><<<g, 256, 0, s>>>(mptr, midx, mcoef, cst, D, (float*)val, nnz, B);
    else
        batch_assemble_kernel<double><<<g, 256, 0, s>>>(mptr, midx, mcoef, cst, D, (double*)val, nnz, B);
}

}  // namespace fvm

using namespace fvm;

extern "C" {

int fvm_batch_create(fvm_problem* p, int32_t batch, const double* dualD, const double* quarterD, int32_t precision,
                     fvm_batch** out) {
    return guard_call([&] {
        if (!p || !dualD || !out) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        if (batch < 1) fail(FVM_ERR_INVALID_ARGUMENT, "batch must be positive");
        if (precision != FVM_FP64 && precision != FVM_FP32) fail(FVM_ERR_INVALID_ARGUMENT, "bad precision");
        if (p->conditions_only) fail(FVM_ERR_INVALID_ARGUMENT, "this problem carries a template's conditions only");
        if (p->dif_deg != 0 || !p->linear || p->flux_linear || p->ntime > 0)
            fail(FVM_ERR_UNSUPPORTED_FORM, "batched instances need a linear, time-independent problem with a diffusion "
                                           "flux -D(x, y) grad u");
        *out = nullptr;
        const fvm_mesh* m = p->mesh;
        std::unique_ptr<fvm_batch> bt(new fvm_batch());
        bt->prob = p;
        bt->B = batch;
        bt->precision = precision;
        bt->np = m->np;
        const SellPattern& pat = m->pat;
        bt->nnz = pat.nnz;
        const int64_t nD = 3 * m->nt + 2 * m->nbe;
        // contribution map over the CSR entries of the pattern with the diagonal
        std::vector<double> cst(pat.nnz, 0.0);
        struct Ent {
            int64_t k;
            int32_t idx;
            double coef;
        };
        std::vector<Ent> ents;
        ents.reserve((size_t)m->nt * 18 + 8 * m->nbe);
        std::vector<double> bv, qv, rs;
        fvm_visit_linear_terms(
            p,
            [&](int32_t r, int32_t c, double coef, int64_t didx, bool) {
                int64_t k = pat.find_csr(m->iperm[r], m->iperm[c]);
                if (didx >= 0)
                    ents.push_back({k, (int32_t)didx, coef});
                else
                    cst[k] += coef;
            },
            bv, qv, rs);
        std::vector<int64_t> mptr(pat.nnz + 1, 0);
        for (const Ent& e : ents) mptr[e.k + 1]++;
        for (int64_t k = 0; k < pat.nnz; ++k) mptr[k + 1] += mptr[k];
        std::vector<int32_t> midx(ents.size());
        std::vector<double> mcoef(ents.size());
        {
            std::vector<int64_t> fill(mptr.begin(), mptr.end() - 1);
            for (const Ent& e : ents) {
                int64_t q = fill[e.k]++;
                midx[q] = e.idx;
                mcoef[q] = e.coef;
            }
        }
        // D transposed to [nD][batch]
        std::vector<double> Dt((size_t)nD * batch);
        for (int b = 0; b < batch; ++b) {
            const double* db = dualD + (size_t)b * 3 * m->nt;
            for (int64_t i = 0; i < 3 * m->nt; ++i) Dt[(size_t)i * batch + b] = db[i];
            for (int64_t i = 0; i < 2 * m->nbe; ++i)
                Dt[(size_t)(3 * m->nt + i) * batch + b] = quarterD ? quarterD[(size_t)b * 2 * m->nbe + i] : 0.0;
        }
        for (double x : Dt)
            if (!std::isfinite(x)) fail(FVM_ERR_INVALID_ARGUMENT, "D values must be finite");
        DBuf d_mptr, d_midx, d_mcoef, d_cst, d_D;
        d_mptr.upload(mptr);
        d_midx.upload(midx);
        d_mcoef.upload(mcoef);
        d_cst.upload(cst);
        d_D.upload(Dt);
        size_t es = precision == FVM_FP32 ? 4 : 8;
        bt->d_val.alloc(es * pat.nnz * batch);
        launch_batch_assemble(d_mptr.as<int64_t>(), d_midx.as<int32_t>(), d_mcoef.as<double>(), d_cst.as<double>(),
                              d_D.as<double>(), bt->d_val.p, pat.nnz, batch, precision, nullptr);
        FVM_CUDA(cudaGetLastError());
        FVM_CUDA(cudaDeviceSynchronize());
        bt->d_rowptr.upload(pat.rowptr);
        bt->d_col.upload(pat.csr_col);
        auto nz = [](double x) { return x != 0; };
        const bool has_b = std::any_of(bv.begin(), bv.end(), nz);
        const bool has_q = std::any_of(qv.begin(), qv.end(), nz);
        auto upload_t = [&](DBuf& dst, const std::vector<double>& src) {
            if (precision == FVM_FP32) {
                std::vector<float> f(src.begin(), src.end());
                dst.upload(f);
            } else {
                dst.upload(src);
            }
        };
        if (has_b) upload_t(bt->d_b, bv);
        if (has_q) upload_t(bt->d_q, qv);
        BatchOp& op = bt->op;
        op.np = bt->np;
        op.nnz = bt->nnz;
        op.B = batch;
        op.precision = precision;
        op.rowptr = bt->d_rowptr.as<int64_t>();
        op.col = bt->d_col.as<int32_t>();
        op.val = bt->d_val.p;
        op.b = has_b ? bt->d_b.p : nullptr;
        op.q = has_q ? bt->d_q.p : nullptr;
        // Dirichlet list shared by every instance
        std::vector<int32_t> idx;
        std::vector<double> val;
        for (int64_t v = 0; v < m->np; ++v)
            if (p->code[v] == FVM_VERTEX_DIRICHLET) {
                idx.push_back(m->iperm[v]);
                val.push_back(p->dirv.empty() ? 0.0 : p->dirv[v]);
            }
        bt->ndir = (int64_t)idx.size();
        bt->d_dir_idx.upload(idx);
        bt->d_dir_val.upload(val);
        *out = bt.release();
        return FVM_OK;
    });
}

int fvm_batch_destroy(fvm_batch* b) {
    return guard_call([&] {
        delete b;
        return FVM_OK;
    });
}

int fvm_batch_tuning(const fvm_batch* b, int32_t* tune) {
    return guard_call([&] {
        if (!b || !tune) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        tune[0] = b->op.block;
        tune[1] = b->op.vec;
        tune[2] = (int32_t)b->op.grid;
        return FVM_OK;
    });
}

int fvm_batch_rhs(fvm_batch* bt, const void* u, void* du, double t, int32_t flags, void* stream) {
    return guard_call([&] {
        if (!bt || !u || !du) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        (void)t;
        cudaStream_t s = (cudaStream_t)stream;
        const int32_t loc = flags & 3;
        const int64_t n = bt->np * bt->B;
        const size_t es = bt->precision == FVM_FP32 ? 4 : 8;
        const int32_t* perm = bt->prob->mesh->d_perm.as<int32_t>();
        auto run = [&](auto tag) {
            using T = decltype(tag);
            if (loc == FVM_PTR_DEVICE_INTERNAL) {
                batch_rhs_internal<T>(bt, (const T*)u, (T*)du, s);
                return;
            }
            if (!bt->d_work.p) bt->d_work.alloc(3 * es * n);
            T* ui = bt->d_work.as<T>();
            T* dui = ui + n;
            T* ref = ui + 2 * n;
            const T* src = (const T*)u;
            if (loc == FVM_PTR_HOST) {
                FVM_CUDA(cudaMemcpyAsync(ref, u, es * n, cudaMemcpyHostToDevice, s));
                src = ref;
            }
            batch_permute_kernel<T, T><<<blocks(n, 256), 256, 0, s>>>(perm, src, ui, bt->np, bt->B, 1);
            batch_rhs_internal<T>(bt, ui, dui, s);
            T* dst = loc == FVM_PTR_HOST ? ref : (T*)du;
            batch_permute_kernel<T, T><<<blocks(n, 256), 256, 0, s>>>(perm, dui, dst, bt->np, bt->B, 0);
            if (loc == FVM_PTR_HOST) {
                FVM_CUDA(cudaMemcpyAsync(du, ref, es * n, cudaMemcpyDeviceToHost, s));
                FVM_CUDA(cudaStreamSynchronize(s));
            }
        };
        if (bt->precision == FVM_FP32)
            run(float());
        else
            run(double());
        FVM_CUDA(cudaGetLastError());
        return FVM_OK;
    });
}

int fvm_batch_tsit5_solve(fvm_batch* bt, const double* u0, const fvm_ode_options* o, double* out,
                          fvm_ode_stats* st, void* stream) {
    return guard_call([&] {
        if (!bt || !u0 || !o || !out) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        if (o->adaptive) fail(FVM_ERR_INVALID_ARGUMENT, "batched Tsit5 uses fixed steps (adaptive = 0)");
        if (!(o->dt > 0) || !(o->tf > o->t0)) fail(FVM_ERR_INVALID_ARGUMENT, "need dt > 0 and tf > t0");
        const double span = o->tf - o->t0;
        const int64_t nsteps = (int64_t)std::llround(span / o->dt);
        if (std::fabs(nsteps * o->dt - span) > 1e-9 * span)
            fail(FVM_ERR_INVALID_ARGUMENT, "batched Tsit5 needs (tf - t0) to be a multiple of dt");
        std::vector<double> saveat;
        if (o->saveat && o->nsave > 0)
            saveat.assign(o->saveat, o->saveat + o->nsave);
        else
            saveat.push_back(o->tf);
        std::vector<int64_t> save_steps;
        for (double ts : saveat) {
            double kf = (ts - o->t0) / o->dt;
            int64_t kk = (int64_t)std::llround(kf);
            if (kk < 0 || kk > nsteps || std::fabs(kk - kf) > 1e-6)
                fail(FVM_ERR_INVALID_ARGUMENT, "batched saveat times must be step times t0 + k dt");
            if (!save_steps.empty() && kk < save_steps.back()) fail(FVM_ERR_INVALID_ARGUMENT, "saveat must be sorted");
            save_steps.push_back(kk);
        }
        CaptureStream cs((cudaStream_t)stream, o->use_graph != 0);
        cudaStream_t s = cs.s;
        const int64_t n = bt->np * bt->B;
        const size_t es = bt->precision == FVM_FP32 ? 4 : 8;
        const int32_t* perm = bt->prob->mesh->d_perm.as<int32_t>();
        DBuf ws, io;
        ws.alloc(es * n * 9);
        io.alloc(8 * n * 2);
        double* ref = io.as<double>();
        double* outd = ref + n;
        cudaEvent_t e0, e1;
        FVM_CUDA(cudaEventCreate(&e0));
        FVM_CUDA(cudaEventCreate(&e1));
        int64_t nrhs = 0;
        auto run = [&](auto tag) {
            using T = decltype(tag);
            T* u = ws.as<T>();
            T* work = u + n;
            FVM_CUDA(cudaMemcpyAsync(ref, u0, 8 * n, cudaMemcpyHostToDevice, s));
            batch_permute_kernel<double, T><<<blocks(n, 256), 256, 0, s>>>(perm, ref, u, bt->np, bt->B, 1);
            // autotune outside the timed loop and the graph capture
            batch_rhs_internal<T>(bt, u, work + n, s);
            FVM_CUDA(cudaEventRecord(e0, s));
            int64_t k = 0;
            for (size_t si = 0; si < save_steps.size(); ++si) {
                if (save_steps[si] > k) {
                    batch_tsit5<T>(bt, u, work, save_steps[si] - k, o->dt, o->use_graph != 0, s);
                    nrhs += 1 + 6 * (save_steps[si] - k) + (bt->ndir ? 1 : 0);
                    k = save_steps[si];
                }
                batch_permute_kernel<T, double><<<blocks(n, 256), 256, 0, s>>>(perm, u, outd, bt->np, bt->B, 0);
                FVM_CUDA(cudaMemcpyAsync(out + si * n, outd, 8 * n, cudaMemcpyDeviceToHost, s));
            }
            FVM_CUDA(cudaEventRecord(e1, s));
        };
        if (bt->precision == FVM_FP32)
            run(float());
        else
            run(double());
        FVM_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        FVM_CUDA(cudaGetLastError());
        if (st) {
            st->naccept = nsteps;
            st->nreject = 0;
            st->nrhs = nrhs;
            st->t_final = o->tf;
            st->elapsed_ms = ms;
            st->driver = o->use_graph ? FVM_DRIVER_FIXED_GRAPH : FVM_DRIVER_HOST;
        }
        return FVM_OK;
    });
}

}  // extern "C"
