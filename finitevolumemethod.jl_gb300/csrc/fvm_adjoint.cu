// Discrete adjoint of the batched template ODE du/dt = A(D) u + b, with D(x, y) the P1
// interpolant of per-vertex values exp(theta_v) (a log-diffusivity field per instance).
//
// The operator of a DiffusionEquation / LinearReactionDiffusionEquation template is affine in
// the diffusion samples: A_rc = C_rc + sum_m coef_m D[idx_m], the terms coming from
// fvm_template_visit_terms (the same visitor the template assembly runs).  Each sample is the
// P1 interpolant at a dual-edge midpoint (5/12, 5/12, 2/12 of the triangle's vertices) or at a
// boundary quarter point (3/4, 1/4 of the edge's end points).  So per instance
//   theta -> E = exp(theta) -> D = W E -> A(D) (values [nnz][B], and A^T's values)
// and the reverse of that chain is
//   Dbar[idx] = sum_m coef_m G[k_m],  thetabar_v = E_v sum_idx W[idx, v] Dbar[idx],
// where G[k] (one per operator entry) accumulates sum over stages and steps of
// kbar_r * Y_c: the cotangent of a stage derivative times the stage value it multiplied.
//
// Time stepping is fixed-step Tsit5 on the batch.  The reverse of one step, with cotangent
// lambda of u_{n+1}, stage values Y_i and stage derivatives k_i = A Y_i + b (i = 1..6):
//   kbar_i = h (b_i lambda + sum_{j > i} a_ji Ybar_j),  Ybar_i = A^T kbar_i   (i = 6 .. 1)
//   lambda_n = lambda + sum_i Ybar_i,  G += sum_i kbar_i (x) Y_i on the pattern.
// The forward pass keeps u every `checkpoint_every` steps; the reverse pass recomputes each
// segment's states from its checkpoint and each step's stages from its state.
#include "fvm_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>

struct fvm_adjoint {
    fvm_template* T = nullptr;
    int B = 0;
    int64_t np = 0, nnz = 0, nD = 0, nt = 0;
    fvm::DBuf d_rowptr, d_col, d_erow;        // A's CSR (internal numbering), row of each entry
    fvm::DBuf d_trowptr, d_tcol, d_tperm;     // A^T's CSR and entry -> A entry
    fvm::DBuf d_mptr, d_midx, d_mcoef, d_cst; // entry -> (sample, coef) terms, constant part
    fvm::DBuf d_sptr, d_sent, d_scoef;        // sample -> (entry, coef) terms
    fvm::DBuf d_svtx, d_sw;                   // sample -> 3 internal vertices, 3 weights
    fvm::DBuf d_vptr, d_vsmp, d_vw;           // vertex -> (sample, weight)
    fvm::DBuf d_b;                            // b (internal, independent of D)
    bool has_b = false;
    fvm::DBuf d_theta, d_E, d_D, d_val, d_valT;  // per instance
    fvm::BatchOp A, AT;
    // one instance: A and A^T in the mesh's sliced-ELL layout (the pattern is structurally
    // symmetric, so A^T has A's slots), applied by the single-instance streamed kernel
    fvm::DBuf d_slot, d_tslot, d_sell, d_sellT;
    bool theta_set = false;
};

namespace fvm {
namespace {

static inline unsigned blocks(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

// Tsitouras (2011) tableau: row s holds a_{s+1, j+1}; row 6 is b (b_7 = 0)
const double kA[7][6] = {
    {0, 0, 0, 0, 0, 0},
    {0.161, 0, 0, 0, 0, 0},
    {-0.008480655492356989, 0.335480655492357, 0, 0, 0, 0},
    {2.897153057105493, -6.359448489975075, 4.3622954328695815, 0, 0, 0},
    {5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525, 0, 0},
    {5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383, 0},
    {0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774},
};

// y = x0 + sum_j c_j v_j over n entries (x0 may be null); y may alias x0
struct LinComb {
    const double* v[8];
    double c[8];
    int nv;
};
__global__ void lincomb_kernel(double* y, const double* x0, LinComb L, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double acc = x0 ? x0[i] : 0.0;
#pragma unroll
    for (int j = 0; j < 8; ++j)
        if (j < L.nv) acc += L.c[j] * L.v[j][i];
    y[i] = acc;
}
void lincomb(double* y, const double* x0, const LinComb& L, int64_t n, cudaStream_t s) {
    if (n) lincomb_kernel<<<blocks(n, 256), 256, 0, s>>>(y, x0, L, n);
}

__global__ void exp_kernel(const double* __restrict__ th, double* __restrict__ E, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) E[i] = exp(th[i]);
}

// D[idx][b] = sum_j w[idx][j] E[v[idx][j]][b]
__global__ void sample_kernel(const int32_t* __restrict__ sv, const double* __restrict__ sw,
                              const double* __restrict__ E, double* __restrict__ D, int64_t nD, int B) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nD * B) return;
    int64_t idx = i / B;
    int b = (int)(i - idx * B);
    double acc = 0;
#pragma unroll
    for (int j = 0; j < 3; ++j) acc += sw[3 * idx + j] * E[(int64_t)sv[3 * idx + j] * B + b];
    D[i] = acc;
}

// valT[kT][b] = val[tperm[kT]][b]
__global__ void transpose_vals_kernel(const int64_t* __restrict__ tperm, const double* __restrict__ val,
                                      double* __restrict__ valT, int64_t nnz, int B) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nnz * B) return;
    int64_t k = i / B;
    valT[i] = val[tperm[k] * B + (i - k * B)];
}

// G[k][b] += sum_{i < ns} kb_i[row(k)][b] * Y_i[col(k)][b].  Every (entry, instance) pair is
// independent: with many instances a thread takes a pair (consecutive threads, consecutive
// instances: coalesced); with few, a thread takes an entry and loops over the instances.
struct StagePair {
    const double* kb[6];
    const double* Y[6];
    int ns;
};
__device__ __forceinline__ void grad_accum_one(const StagePair& P, double* G, int64_t k, int64_t r, int64_t c,
                                               int64_t b, int B) {
    double acc = G[k * B + b];
#pragma unroll
    for (int j = 0; j < 6; ++j)
        if (j < P.ns) acc += P.kb[j][r * B + b] * P.Y[j][c * B + b];
    G[k * B + b] = acc;
}
__global__ void grad_accum_elem_kernel(const int32_t* __restrict__ erow, const int32_t* __restrict__ col, StagePair P,
                                       double* __restrict__ G, int64_t nnz, int B) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nnz * B) return;
    const int64_t k = i / B;
    grad_accum_one(P, G, k, __ldg(&erow[k]), __ldg(&col[k]), i - k * B, B);
}
__global__ void grad_accum_thread_kernel(const int32_t* __restrict__ erow, const int32_t* __restrict__ col,
                                         StagePair P, double* __restrict__ G, int64_t nnz, int B) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nnz) return;
    const int64_t r = __ldg(&erow[k]), c = __ldg(&col[k]);
    for (int64_t b = 0; b < B; ++b) grad_accum_one(P, G, k, r, c, b, B);
}
void launch_grad_accum(const fvm_adjoint* a, const StagePair& P, double* G, cudaStream_t s) {
    if (a->B >= 16)
        grad_accum_elem_kernel<<<blocks(a->nnz * a->B, 256), 256, 0, s>>>(a->d_erow.as<int32_t>(),
                                                                           a->d_col.as<int32_t>(), P, G, a->nnz, a->B);
    else
        grad_accum_thread_kernel<<<blocks(a->nnz, 256), 256, 0, s>>>(a->d_erow.as<int32_t>(), a->d_col.as<int32_t>(), P,
                                                                     G, a->nnz, a->B);
}

// Dbar[idx][b] = sum coef * G[k][b] over the sample's terms
__global__ void dbar_kernel(const int64_t* __restrict__ sptr, const int64_t* __restrict__ sent,
                            const double* __restrict__ scoef, const double* __restrict__ G,
                            double* __restrict__ Dbar, int64_t nD, int B) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nD * B) return;
    int64_t idx = i / B;
    int64_t b = i - idx * B;
    double acc = 0;
    for (int64_t m = sptr[idx]; m < sptr[idx + 1]; ++m) acc += scoef[m] * G[sent[m] * B + b];
    Dbar[i] = acc;
}

// thetabar[v][b] = E[v][b] sum w * Dbar[idx][b] over the vertex's samples
__global__ void thetabar_kernel(const int64_t* __restrict__ vptr, const int32_t* __restrict__ vsmp,
                                const double* __restrict__ vw, const double* __restrict__ E,
                                const double* __restrict__ Dbar, double* __restrict__ tb, int64_t np, int B) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np * B) return;
    int64_t v = i / B;
    int64_t b = i - v * B;
    double acc = 0;
    for (int64_t m = vptr[v]; m < vptr[v + 1]; ++m) acc += vw[m] * Dbar[(int64_t)vsmp[m] * B + b];
    tb[i] = E[i] * acc;
}

// dst[map[k]] = src[k]
__global__ void scatter_kernel(const int64_t* __restrict__ map, const double* __restrict__ src, double* __restrict__ dst,
                               int64_t n) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) dst[map[k]] = src[k];
}

// rows of [n][B]: out[r] = in[perm[r]] (gather) or out[perm[r]] = in[r] (scatter)
__global__ void permute_rows_kernel(const int32_t* __restrict__ perm, const double* __restrict__ in,
                                    double* __restrict__ out, int64_t n, int B, int gather) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * B) return;
    int64_t r = i / B, b = i - r * B;
    int64_t pr = perm[r];
    if (gather)
        out[i] = in[pr * B + b];
    else
        out[pr * B + b] = in[i];
}

// partial[blk][b] = sum over the block's rows of (u - obs)^2; 32 instances x 8 row lanes
__global__ void loss_partial_kernel(const double* __restrict__ u, const double* __restrict__ obs,
                                    double* __restrict__ partial, int64_t n, int B, int64_t rows_per_block) {
    __shared__ double red[8][33];
    const int bl = threadIdx.x & 31, rl = threadIdx.x >> 5;
    const int64_t b = (int64_t)blockIdx.y * 32 + bl;
    const int64_t r0 = (int64_t)blockIdx.x * rows_per_block;
    const int64_t r1 = min(n, r0 + rows_per_block);
    double acc = 0;
    if (b < B)
        for (int64_t r = r0 + rl; r < r1; r += 8) {
            const double d = u[r * B + b] - obs[r * B + b];
            acc += d * d;
        }
    red[rl][bl] = acc;
    __syncthreads();
    if (rl == 0 && b < B) {
        double t = 0;
        for (int j = 0; j < 8; ++j) t += red[j][bl];
        partial[(int64_t)blockIdx.x * B + b] = t;
    }
}
__global__ void loss_final_kernel(const double* __restrict__ partial, double* __restrict__ loss, int64_t nblk,
                                  int B) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    double t = 0;
    for (int64_t j = 0; j < nblk; ++j) t += partial[j * B + b];
    loss[b] = t;
}

}  // namespace
}  // namespace fvm

using namespace fvm;

namespace {

// du = A u + b on the batch (A includes b)
void adj_rhs(fvm_adjoint* a, const double* u, double* du, cudaStream_t s) {
    if (a->B == 1)
        launch_sell_apply64(a->T->prob->mesh->pat, a->d_sell.as<double>(), u, du, nullptr,
                            a->has_b ? a->d_b.as<double>() : nullptr, nullptr, s);
    else
        batch_op_apply<double>(a->A, u, du, s);
}
// out = A^T w on the batch
void adj_rhs_t(fvm_adjoint* a, const double* w, double* out, cudaStream_t s) {
    if (a->B == 1)
        launch_sell_apply64(a->T->prob->mesh->pat, a->d_sellT.as<double>(), w, out, nullptr, nullptr, nullptr, s);
    else
        batch_op_apply<double>(a->AT, w, out, s);
}

// prod = A x (+ b), or A^T x (transpose), then z = x0 + sum_t c_t v_t with null v_t standing for
// prod: on a batch one fused pass (the combination in the product's row epilogue, run while the
// FP64 pipe works on the product), else the single-instance product and a separate pass.
void op_then(fvm_adjoint* a, bool transpose, const double* x, double* prod, double* z, const double* x0,
             const LinComb& L, int64_t n, cudaStream_t s) {
    if (a->B > 1) {
        BatchEpi<double> E;
        E.z = z;
        E.x0 = x0;
        E.nv = L.nv;
        for (int t = 0; t < L.nv; ++t) {
            E.v[t] = L.v[t];
            E.c[t] = L.c[t];
        }
        batch_op_apply_epi<double>(transpose ? a->AT : a->A, x, prod, E, s);
        return;
    }
    if (transpose)
        adj_rhs_t(a, x, prod, s);
    else
        adj_rhs(a, x, prod, s);
    LinComb M = L;
    for (int t = 0; t < M.nv; ++t)
        if (!M.v[t]) M.v[t] = prod;
    lincomb(z, x0, M, n, s);
}

// Y_1 = u + h a_21 k_0, the first stage combination of a Tsit5 step
void first_stage(double* Y1, const double* u, const double* k0, double h, int64_t n, cudaStream_t s) {
    LinComb L{};
    L.nv = 1;
    L.v[0] = k0;
    L.c[0] = h * kA[1][0];
    lincomb(Y1, u, L, n, s);
}

// One Tsit5 step in place: u <- u_{n+1}.  On entry k[0] = f(u_n) and Y[0] = u_n + h a_21 k_0
// (first_stage); on exit k[0] = f(u_{n+1}) and Y[0] = the next step's first stage.  Each stage
// combination is formed in the epilogue of the product before it (Y alternates between Y[0]
// and Y[1], as a product's input and its epilogue's output must differ).
void fwd_step(fvm_adjoint* a, double* u, double* const* k, double* const* Y, double h, int64_t n, cudaStream_t s) {
    for (int i = 1; i < 6; ++i) {
        // k_i = f(Y_i); then Y_{i+1} = u + sum_{j<=i} h a_{i+1,j} k_j, or u_{n+1} after k_5
        const int row = i + 1 < 6 ? i + 1 : 6;
        LinComb L{};
        L.nv = i + 1;
        for (int j = 0; j <= i; ++j) {
            L.v[j] = j < i ? k[j] : nullptr;
            L.c[j] = h * kA[row][j];
        }
        double* z = i < 5 ? Y[i % 2] : u;
        op_then(a, false, Y[(i - 1) % 2], k[i], z, u, L, n, s);
    }
    LinComb L{};
    L.nv = 1;
    L.v[0] = nullptr;
    L.c[0] = h * kA[1][0];
    op_then(a, false, u, k[0], Y[0], u, L, n, s);  // FSAL k_0 = f(u_{n+1}), the next first stage
}

struct Timer {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    Timer() {
        FVM_CUDA(cudaEventCreate(&e0));
        FVM_CUDA(cudaEventCreate(&e1));
    }
    ~Timer() {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    float ms() {
        FVM_CUDA(cudaEventSynchronize(e1));
        float t = 0;
        FVM_CUDA(cudaEventElapsedTime(&t, e0, e1));
        return t;
    }
};

void require_theta(const fvm_adjoint* a) {
    if (!a->theta_set) fail(FVM_ERR_INVALID_ARGUMENT, "set the log-diffusion field first (fvm_adjoint_set_log_diffusion)");
}

// caller-numbered [np][B] arrays in (host or device) -> internal device copies and back
struct Io {
    fvm_adjoint* a;
    int32_t loc;
    cudaStream_t s;
    DBuf stage;  // host staging (one [np][B] array)
    int64_t n;
    Io(fvm_adjoint* a_, int32_t flags, cudaStream_t s_) : a(a_), loc(flags & 3), s(s_), n(a_->np * a_->B) {
        if (loc != FVM_PTR_HOST && loc != FVM_PTR_DEVICE)
            fail(FVM_ERR_INVALID_ARGUMENT, "adjoint arrays are host or device arrays in the caller's numbering");
    }
    const int32_t* perm() const { return a->T->prob->mesh->d_perm.as<int32_t>(); }
    void in(const double* src, double* dst_int) {
        const double* from = src;
        if (loc == FVM_PTR_HOST) {
            if (!stage.p) stage.alloc(8 * n);
            FVM_CUDA(cudaMemcpyAsync(stage.p, src, 8 * n, cudaMemcpyHostToDevice, s));
            from = stage.as<double>();
        }
        permute_rows_kernel<<<blocks(n, 256), 256, 0, s>>>(perm(), from, dst_int, a->np, a->B, 1);
    }
    void out(const double* src_int, double* dst) {
        double* to = dst;
        if (loc == FVM_PTR_HOST) {
            if (!stage.p) stage.alloc(8 * n);
            to = stage.as<double>();
        }
        permute_rows_kernel<<<blocks(n, 256), 256, 0, s>>>(perm(), src_int, to, a->np, a->B, 0);
        if (loc == FVM_PTR_HOST) {
            FVM_CUDA(cudaMemcpyAsync(dst, to, 8 * n, cudaMemcpyDeviceToHost, s));
            FVM_CUDA(cudaStreamSynchronize(s));
        }
    }
};

// gradient of the operator-entry accumulator G with respect to theta (internal numbering)
void theta_from_G(fvm_adjoint* a, const double* G, double* tb, cudaStream_t s) {
    const int B = a->B;
    DBuf dbar;
    dbar.alloc(8 * a->nD * B);
    dbar_kernel<<<blocks(a->nD * B, 256), 256, 0, s>>>(a->d_sptr.as<int64_t>(), a->d_sent.as<int64_t>(),
                                                        a->d_scoef.as<double>(), G, dbar.as<double>(), a->nD, B);
    thetabar_kernel<<<blocks(a->np * B, 256), 256, 0, s>>>(a->d_vptr.as<int64_t>(), a->d_vsmp.as<int32_t>(),
                                                            a->d_vw.as<double>(), a->d_E.as<double>(),
                                                            dbar.as<double>(), tb, a->np, B);
    FVM_CUDA(cudaGetLastError());
    FVM_CUDA(cudaStreamSynchronize(s));  // dbar is freed on return
}

// Forward-and-reverse sweep on internal device arrays.  uTbar is the cotangent of u_N;
// on return tb = d/dtheta and u0b = d/du0 of <uTbar, u_N>; uT (optional) receives u_N.
void pullback_internal(fvm_adjoint* a, const double* u0, double dt, int64_t N, int64_t K, const double* uTbar,
                       double* uT, double* tb, double* u0b, fvm_adjoint_stats* st, cudaStream_t s,
                       const double* obs = nullptr, double* loss_dev = nullptr) {
    const int B = a->B;
    const int64_t n = a->np * B;
    const int64_t ncp = (N + K - 1) / K;
    const int64_t seglen = std::min<int64_t>(K, N);
    // workspace: u, k[7], Y, checkpoints, segment states, stage values/derivatives/cotangents, lambda, G
    const int64_t nvec = 1 + 7 + 2 + ncp + seglen + 5 + 6 + 6 + 6 + 1;
    DBuf ws, G;
    ws.alloc(8 * n * nvec);
    G.alloc(8 * a->nnz * B);
    double* p = ws.as<double>();
    auto take = [&](int64_t m) {
        double* q = p;
        p += m * n;
        return q;
    };
    double* u = take(1);
    double* k[7];
    for (int j = 0; j < 7; ++j) k[j] = take(1);
    double* Y[2];
    Y[0] = take(1);
    Y[1] = take(1);
    double* cps = take(ncp);
    double* seg = take(seglen);
    double* Ys[6];
    for (int j = 1; j < 6; ++j) Ys[j] = take(1);
    double* ks[6];
    for (int j = 0; j < 6; ++j) ks[j] = take(1);
    double* kb[6];
    for (int j = 0; j < 6; ++j) kb[j] = take(1);
    double* Yb[6];
    for (int j = 0; j < 6; ++j) Yb[j] = take(1);
    double* lam = take(1);
    Timer tf, tr;
    int64_t nrhs = 0, nadj = 0;
    // forward, keeping u every K steps
    FVM_CUDA(cudaEventRecord(tf.e0, s));
    FVM_CUDA(cudaMemcpyAsync(u, u0, 8 * n, cudaMemcpyDeviceToDevice, s));
    adj_rhs(a, u, k[0], s);
    first_stage(Y[0], u, k[0], dt, n, s);
    ++nrhs;
    for (int64_t step = 0; step < N; ++step) {
        if (step % K == 0) FVM_CUDA(cudaMemcpyAsync(cps + (step / K) * n, u, 8 * n, cudaMemcpyDeviceToDevice, s));
        fwd_step(a, u, k, Y, dt, n, s);
        nrhs += 6;
    }
    if (uT) FVM_CUDA(cudaMemcpyAsync(uT, u, 8 * n, cudaMemcpyDeviceToDevice, s));
    FVM_CUDA(cudaEventRecord(tf.e1, s));
    // the cotangent of u_N
    FVM_CUDA(cudaEventRecord(tr.e0, s));
    if (obs) {  // loss = sum (u_N - obs)^2, lambda = 2 (u_N - obs)
        LinComb L{};
        L.nv = 2;
        L.v[0] = u;
        L.c[0] = 2.0;
        L.v[1] = obs;
        L.c[1] = -2.0;
        lincomb(lam, nullptr, L, n, s);
        const int64_t rpb = 256;
        const int64_t nblk = (a->np + rpb - 1) / rpb;
        DBuf part;
        part.alloc(8 * nblk * B);
        loss_partial_kernel<<<dim3((unsigned)nblk, (unsigned)((B + 31) / 32)), 256, 0, s>>>(
            u, obs, part.as<double>(), a->np, B, rpb);
        loss_final_kernel<<<blocks(B, 128), 128, 0, s>>>(part.as<double>(), loss_dev, nblk, B);
        FVM_CUDA(cudaStreamSynchronize(s));  // part is freed on return
    } else {
        FVM_CUDA(cudaMemcpyAsync(lam, uTbar, 8 * n, cudaMemcpyDeviceToDevice, s));
    }
    FVM_CUDA(cudaMemsetAsync(G.p, 0, G.bytes, s));
    for (int64_t sg = ncp - 1; sg >= 0; --sg) {
        const int64_t s0 = sg * K, s1 = std::min(N, s0 + K);
        // states u_{s0} .. u_{s1 - 1} from the checkpoint
        FVM_CUDA(cudaMemcpyAsync(seg, cps + sg * n, 8 * n, cudaMemcpyDeviceToDevice, s));
        if (s1 - s0 > 1) {
            adj_rhs(a, seg, k[0], s);
            first_stage(Y[0], seg, k[0], dt, n, s);
            ++nrhs;
        }
        for (int64_t j = 1; j < s1 - s0; ++j) {
            FVM_CUDA(cudaMemcpyAsync(seg + j * n, seg + (j - 1) * n, 8 * n, cudaMemcpyDeviceToDevice, s));
            fwd_step(a, seg + j * n, k, Y, dt, n, s);
            nrhs += 6;
        }
        for (int64_t step = s1 - 1; step >= s0; --step) {
            const double* un = seg + (step - s0) * n;
            // stages of this step: Y_1 = u_n, Y_i = u_n + h sum_{j<i} a_ij k_j, k_i = A Y_i + b;
            // each Y_{i+1} is formed in the epilogue of k_i's product (k_6 forms no later stage)
            const double* Yi[6];
            Yi[0] = un;
            for (int i = 0; i < 5; ++i) {
                LinComb L{};
                L.nv = i + 1;
                for (int j = 0; j <= i; ++j) {
                    L.v[j] = j < i ? ks[j] : nullptr;
                    L.c[j] = dt * kA[i + 1][j];
                }
                op_then(a, false, Yi[i], ks[i], Ys[i + 1], un, L, n, s);
                Yi[i + 1] = Ys[i + 1];
            }
            nrhs += 5;
            // reverse through the stages: kb_i = h b_i lambda + sum_{j>i} h a_ji Yb_j, Yb_i = A^T kb_i;
            // kb_{i-1} is formed in the epilogue of Yb_i's product, and lambda += sum_i Yb_i in Yb_0's
            {
                LinComb L{};
                L.nv = 1;
                L.v[0] = lam;
                L.c[0] = dt * kA[6][5];
                lincomb(kb[5], nullptr, L, n, s);
            }
            for (int i = 5; i >= 0; --i) {
                LinComb L{};
                if (i > 0) {
                    const int m = i - 1;
                    L.v[L.nv] = lam;
                    L.c[L.nv++] = dt * kA[6][m];
                    for (int j = m + 1; j < 6; ++j) {
                        L.v[L.nv] = j == i ? nullptr : Yb[j];
                        L.c[L.nv++] = dt * kA[j][m];
                    }
                    op_then(a, true, kb[i], Yb[i], kb[m], nullptr, L, n, s);
                } else {
                    for (int j = 0; j < 6; ++j) {
                        L.v[L.nv] = j == 0 ? nullptr : Yb[j];
                        L.c[L.nv++] = 1.0;
                    }
                    op_then(a, true, kb[0], Yb[0], lam, lam, L, n, s);
                }
                ++nadj;
            }
            StagePair P{};
            P.ns = 6;
            for (int i = 0; i < 6; ++i) {
                P.kb[i] = kb[i];
                P.Y[i] = Yi[i];
            }
            launch_grad_accum(a, P, G.as<double>(), s);
        }
    }
    FVM_CUDA(cudaGetLastError());
    theta_from_G(a, G.as<double>(), tb, s);
    if (u0b) FVM_CUDA(cudaMemcpyAsync(u0b, lam, 8 * n, cudaMemcpyDeviceToDevice, s));
    FVM_CUDA(cudaEventRecord(tr.e1, s));
    const float fms = tf.ms(), rms = tr.ms();
    if (st) {
        st->steps = N;
        st->checkpoints = ncp;
        st->rhs_evals = nrhs;
        st->transpose_evals = nadj;
        st->forward_ms = fms;
        st->reverse_ms = rms;
    }
}

}  // namespace

extern "C" {

int fvm_adjoint_create(fvm_template* T, int32_t batch, fvm_adjoint** out) {
    return guard_call([&] {
        if (!T || !out) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        *out = nullptr;
        if (batch < 1) fail(FVM_ERR_INVALID_ARGUMENT, "batch must be positive");
        if (T->kind != FVM_TEMPLATE_DIFFUSION && T->kind != FVM_TEMPLATE_LINEAR_REACTION_DIFFUSION)
            fail(FVM_ERR_UNSUPPORTED, "the adjoint covers the time-dependent templates (DiffusionEquation, "
                                      "LinearReactionDiffusionEquation)");
        const fvm_mesh* m = T->prob->mesh;
        const SellPattern& pat = m->pat;
        std::unique_ptr<fvm_adjoint> a(new fvm_adjoint());
        a->T = T;
        a->B = batch;
        a->np = m->np;
        a->nnz = pat.nnz;
        a->nt = m->nt;
        a->nD = 3 * m->nt + 2 * m->nbe;
        // operator terms on the CSR entries (internal numbering) and the D-independent b
        struct Term {
            int64_t k;
            int32_t idx;
            double coef;
        };
        std::vector<Term> terms;
        terms.reserve((size_t)m->nt * 18 + 6 * m->nbe);
        std::vector<double> cst(pat.nnz, 0.0), b(m->np, 0.0);
        fvm_template_visit_terms(
            T,
            [&](int32_t r, int32_t c, double coef, int64_t didx) {
                const int64_t k = pat.find_csr(m->iperm[r], m->iperm[c]);
                if (didx >= 0)
                    terms.push_back({k, (int32_t)didx, coef});
                else
                    cst[k] += coef;
            },
            [&](int32_t r, int32_t, double coef, int64_t didx) {
                if (didx >= 0)
                    fail(FVM_ERR_UNSUPPORTED_FORM,
                         "the template's b depends on the diffusion field (Neumann edges); the adjoint needs a "
                         "b independent of D");
                b[m->iperm[r]] += coef;
            });
        // entry -> terms, and sample -> terms
        std::vector<int64_t> mptr(pat.nnz + 1, 0), sptr(a->nD + 1, 0);
        for (const Term& t : terms) {
            mptr[t.k + 1]++;
            sptr[t.idx + 1]++;
        }
        for (int64_t k = 0; k < pat.nnz; ++k) mptr[k + 1] += mptr[k];
        for (int64_t i = 0; i < a->nD; ++i) sptr[i + 1] += sptr[i];
        std::vector<int32_t> midx(terms.size());
        std::vector<double> mcoef(terms.size()), scoef(terms.size());
        std::vector<int64_t> sent(terms.size());
        {
            std::vector<int64_t> fm(mptr.begin(), mptr.end() - 1), fs(sptr.begin(), sptr.end() - 1);
            for (const Term& t : terms) {
                const int64_t q = fm[t.k]++, r = fs[t.idx]++;
                midx[q] = t.idx;
                mcoef[q] = t.coef;
                sent[r] = t.k;
                scoef[r] = t.coef;
            }
        }
        // rows of the entries, and A^T (entries of column c in row order)
        std::vector<int32_t> erow(pat.nnz);
        std::vector<int64_t> trowptr(m->np + 1, 0);
        for (int64_t r = 0; r < m->np; ++r)
            for (int64_t k = pat.rowptr[r]; k < pat.rowptr[r + 1]; ++k) {
                erow[k] = (int32_t)r;
                trowptr[pat.csr_col[k] + 1]++;
            }
        for (int64_t c = 0; c < m->np; ++c) trowptr[c + 1] += trowptr[c];
        std::vector<int32_t> tcol(pat.nnz);
        std::vector<int64_t> tperm(pat.nnz);
        {
            std::vector<int64_t> f(trowptr.begin(), trowptr.end() - 1);
            for (int64_t k = 0; k < pat.nnz; ++k) {
                const int64_t q = f[pat.csr_col[k]]++;
                tcol[q] = erow[k];
                tperm[q] = k;
            }
        }
        // P1 interpolation of the samples: dual-edge midpoint of edge e of triangle t is
        // (5 p_e + 5 p_{e+1} + 2 p_{e+2}) / 12; boundary quarter points are (3 p_i + p_j) / 4
        std::vector<int32_t> svtx(3 * a->nD);
        std::vector<double> sw(3 * a->nD);
        for (int64_t t = 0; t < m->nt; ++t)
            for (int e = 0; e < 3; ++e) {
                const int64_t i = 3 * t + e;
                for (int j = 0; j < 3; ++j) svtx[3 * i + j] = m->iperm[m->tri[3 * t + (e + j) % 3]];
                sw[3 * i] = 5.0 / 12.0;
                sw[3 * i + 1] = 5.0 / 12.0;
                sw[3 * i + 2] = 2.0 / 12.0;
            }
        for (int64_t e = 0; e < m->nbe; ++e)
            for (int side = 0; side < 2; ++side) {
                const int64_t i = 3 * m->nt + 2 * e + side;
                const int32_t near = m->iperm[m->be[2 * e + side]], far = m->iperm[m->be[2 * e + 1 - side]];
                svtx[3 * i] = near;
                svtx[3 * i + 1] = far;
                svtx[3 * i + 2] = near;
                sw[3 * i] = 0.75;
                sw[3 * i + 1] = 0.25;
                sw[3 * i + 2] = 0.0;
            }
        std::vector<int64_t> vptr(m->np + 1, 0);
        for (int64_t i = 0; i < 3 * a->nD; ++i)
            if (sw[i] != 0) vptr[svtx[i] + 1]++;
        for (int64_t v = 0; v < m->np; ++v) vptr[v + 1] += vptr[v];
        std::vector<int32_t> vsmp(vptr[m->np]);
        std::vector<double> vw(vptr[m->np]);
        {
            std::vector<int64_t> f(vptr.begin(), vptr.end() - 1);
            for (int64_t i = 0; i < 3 * a->nD; ++i)
                if (sw[i] != 0) {
                    const int64_t q = f[svtx[i]]++;
                    vsmp[q] = (int32_t)(i / 3);
                    vw[q] = sw[i];
                }
        }
        a->d_rowptr.upload(pat.rowptr);
        a->d_col.upload(pat.csr_col);
        a->d_erow.upload(erow);
        a->d_trowptr.upload(trowptr);
        a->d_tcol.upload(tcol);
        a->d_tperm.upload(tperm);
        a->d_mptr.upload(mptr);
        a->d_midx.upload(midx);
        a->d_mcoef.upload(mcoef);
        a->d_cst.upload(cst);
        a->d_sptr.upload(sptr);
        a->d_sent.upload(sent);
        a->d_scoef.upload(scoef);
        a->d_svtx.upload(svtx);
        a->d_sw.upload(sw);
        a->d_vptr.upload(vptr);
        a->d_vsmp.upload(vsmp);
        a->d_vw.upload(vw);
        if (batch == 1) {
            std::vector<int64_t> tslot(pat.nnz);
            for (int64_t k = 0; k < pat.nnz; ++k) {
                const int64_t t = pat.find(pat.csr_col[k], erow[k]);
                if (t < 0) fail(FVM_ERR_BAD_MESH, "vertex-neighbour pattern is not structurally symmetric");
                tslot[k] = t;
            }
            a->d_slot.upload(pat.csr_slot);
            a->d_tslot.upload(tslot);
            a->d_sell.alloc(8 * pat.nslots);
            a->d_sellT.alloc(8 * pat.nslots);
            FVM_CUDA(cudaMemset(a->d_sell.p, 0, a->d_sell.bytes));
            FVM_CUDA(cudaMemset(a->d_sellT.p, 0, a->d_sellT.bytes));
        }
        a->has_b = std::any_of(b.begin(), b.end(), [](double x) { return x != 0; });
        if (a->has_b) a->d_b.upload(b);
        const int64_t n = a->np * batch;
        a->d_theta.alloc(8 * n);
        a->d_E.alloc(8 * n);
        a->d_D.alloc(8 * a->nD * batch);
        a->d_val.alloc(8 * a->nnz * batch);
        a->d_valT.alloc(8 * a->nnz * batch);
        BatchOp& A = a->A;
        A.np = a->np;
        A.nnz = a->nnz;
        A.B = batch;
        A.rowptr = a->d_rowptr.as<int64_t>();
        A.col = a->d_col.as<int32_t>();
        A.val = a->d_val.p;
        A.b = a->has_b ? a->d_b.p : nullptr;
        BatchOp& AT = a->AT;
        AT = A;
        AT.rowptr = a->d_trowptr.as<int64_t>();
        AT.col = a->d_tcol.as<int32_t>();
        AT.val = a->d_valT.p;
        AT.b = nullptr;
        *out = a.release();
        return FVM_OK;
    });
}

int fvm_adjoint_destroy(fvm_adjoint* a) {
    return guard_call([&] {
        delete a;
        return FVM_OK;
    });
}

int fvm_adjoint_set_log_diffusion(fvm_adjoint* a, const double* theta, int32_t flags, void* stream) {
    return guard_call([&] {
        if (!a || !theta) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        cudaStream_t s = (cudaStream_t)stream;
        Io io(a, flags, s);
        if (io.loc == FVM_PTR_HOST)
            for (int64_t i = 0; i < io.n; ++i)
                if (!std::isfinite(theta[i])) fail(FVM_ERR_INVALID_ARGUMENT, "log-diffusion values must be finite");
        const int B = a->B;
        io.in(theta, a->d_theta.as<double>());
        exp_kernel<<<blocks(io.n, 256), 256, 0, s>>>(a->d_theta.as<double>(), a->d_E.as<double>(), io.n);
        sample_kernel<<<blocks(a->nD * B, 256), 256, 0, s>>>(a->d_svtx.as<int32_t>(), a->d_sw.as<double>(),
                                                              a->d_E.as<double>(), a->d_D.as<double>(), a->nD, B);
        launch_batch_assemble(a->d_mptr.as<int64_t>(), a->d_midx.as<int32_t>(), a->d_mcoef.as<double>(),
                              a->d_cst.as<double>(), a->d_D.as<double>(), a->d_val.p, a->nnz, B, FVM_FP64, s);
        transpose_vals_kernel<<<blocks(a->nnz * B, 256), 256, 0, s>>>(
            a->d_tperm.as<int64_t>(), a->d_val.as<double>(), a->d_valT.as<double>(), a->nnz, B);
        if (B == 1) {  // sliced-ELL copies: A's entry (r, c) at slot(r, c) and at A^T's slot(c, r)
            scatter_kernel<<<blocks(a->nnz, 256), 256, 0, s>>>(a->d_slot.as<int64_t>(), a->d_val.as<double>(),
                                                                a->d_sell.as<double>(), a->nnz);
            scatter_kernel<<<blocks(a->nnz, 256), 256, 0, s>>>(a->d_tslot.as<int64_t>(), a->d_val.as<double>(),
                                                                a->d_sellT.as<double>(), a->nnz);
        }
        FVM_CUDA(cudaGetLastError());
        a->theta_set = true;
        return FVM_OK;
    });
}

int fvm_adjoint_rhs(fvm_adjoint* a, const double* u, double* du, int32_t flags, void* stream) {
    return guard_call([&] {
        if (!a || !u || !du) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        require_theta(a);
        cudaStream_t s = (cudaStream_t)stream;
        Io io(a, flags, s);
        DBuf w;
        w.alloc(16 * io.n);
        double* ui = w.as<double>();
        io.in(u, ui);
        adj_rhs(a, ui, ui + io.n, s);
        io.out(ui + io.n, du);
        FVM_CUDA(cudaStreamSynchronize(s));
        return FVM_OK;
    });
}

int fvm_adjoint_forward(fvm_adjoint* a, const double* u0, double dt, int64_t nsteps, double* uT, int32_t flags,
                        void* stream) {
    return guard_call([&] {
        if (!a || !u0 || !uT) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        if (!(dt > 0) || nsteps < 0) fail(FVM_ERR_INVALID_ARGUMENT, "need dt > 0 and nsteps >= 0");
        require_theta(a);
        cudaStream_t s = (cudaStream_t)stream;
        Io io(a, flags, s);
        const int64_t n = io.n;
        DBuf w;
        w.alloc(8 * n * 10);
        double* u = w.as<double>();
        double* k[7];
        for (int j = 0; j < 7; ++j) k[j] = u + (1 + j) * n;
        double* Y[2] = {u + 8 * n, u + 9 * n};
        io.in(u0, u);
        adj_rhs(a, u, k[0], s);
        first_stage(Y[0], u, k[0], dt, n, s);
        for (int64_t step = 0; step < nsteps; ++step) fwd_step(a, u, k, Y, dt, n, s);
        io.out(u, uT);
        FVM_CUDA(cudaStreamSynchronize(s));
        FVM_CUDA(cudaGetLastError());
        return FVM_OK;
    });
}

int fvm_adjoint_pullback(fvm_adjoint* a, const double* u0, double dt, int64_t nsteps, int32_t checkpoint_every,
                         const double* uT_bar, double* theta_bar, double* u0_bar, fvm_adjoint_stats* stats,
                         int32_t flags, void* stream) {
    return guard_call([&] {
        if (!a || !u0 || !uT_bar || !theta_bar) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        if (!(dt > 0) || nsteps < 1) fail(FVM_ERR_INVALID_ARGUMENT, "need dt > 0 and nsteps >= 1");
        if (checkpoint_every < 1) fail(FVM_ERR_INVALID_ARGUMENT, "checkpoint_every must be positive");
        require_theta(a);
        cudaStream_t s = (cudaStream_t)stream;
        Io io(a, flags, s);
        const int64_t n = io.n;
        DBuf w;
        w.alloc(8 * n * 4);
        double* ui = w.as<double>();
        double* lb = ui + n;
        double* tb = ui + 2 * n;
        double* ub = ui + 3 * n;
        io.in(u0, ui);
        io.in(uT_bar, lb);
        pullback_internal(a, ui, dt, nsteps, checkpoint_every, lb, nullptr, tb, ub, stats, s);
        io.out(tb, theta_bar);
        if (u0_bar) io.out(ub, u0_bar);
        FVM_CUDA(cudaStreamSynchronize(s));
        return FVM_OK;
    });
}

int fvm_adjoint_loss_grad(fvm_adjoint* a, const double* u0, const double* u_obs, double dt, int64_t nsteps,
                          int32_t checkpoint_every, double* loss, double* theta_bar, double* u0_bar,
                          fvm_adjoint_stats* stats, int32_t flags, void* stream) {
    return guard_call([&] {
        if (!a || !u0 || !u_obs || !loss || !theta_bar) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        if (!(dt > 0) || nsteps < 1) fail(FVM_ERR_INVALID_ARGUMENT, "need dt > 0 and nsteps >= 1");
        if (checkpoint_every < 1) fail(FVM_ERR_INVALID_ARGUMENT, "checkpoint_every must be positive");
        require_theta(a);
        cudaStream_t s = (cudaStream_t)stream;
        Io io(a, flags, s);
        const int64_t n = io.n;
        DBuf w;
        w.alloc(8 * (n * 4 + a->B));
        double* ui = w.as<double>();
        double* ob = ui + n;
        double* tb = ui + 2 * n;
        double* ub = ui + 3 * n;
        double* ld = ui + 4 * n;
        io.in(u0, ui);
        io.in(u_obs, ob);
        pullback_internal(a, ui, dt, nsteps, checkpoint_every, nullptr, nullptr, tb, ub, stats, s, ob, ld);
        FVM_CUDA(cudaMemcpyAsync(loss, ld, 8 * a->B, cudaMemcpyDeviceToHost, s));
        io.out(tb, theta_bar);
        if (u0_bar) io.out(ub, u0_bar);
        FVM_CUDA(cudaStreamSynchronize(s));
        return FVM_OK;
    });
}

int fvm_adjoint_rhs_vjp(fvm_adjoint* a, const double* u, const double* w, double* u_bar, double* theta_bar,
                        int32_t flags, void* stream) {
    return guard_call([&] {
        if (!a || !u || !w || !theta_bar) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        require_theta(a);
        cudaStream_t s = (cudaStream_t)stream;
        Io io(a, flags, s);
        const int64_t n = io.n;
        DBuf buf, G;
        buf.alloc(8 * n * 4);
        G.alloc(8 * a->nnz * a->B);
        double* ui = buf.as<double>();
        double* wi = ui + n;
        double* ub = ui + 2 * n;
        double* tb = ui + 3 * n;
        io.in(u, ui);
        io.in(w, wi);
        if (u_bar) adj_rhs_t(a, wi, ub, s);
        FVM_CUDA(cudaMemsetAsync(G.p, 0, G.bytes, s));
        StagePair P{};
        P.ns = 1;
        P.kb[0] = wi;
        P.Y[0] = ui;
        launch_grad_accum(a, P, G.as<double>(), s);
        theta_from_G(a, G.as<double>(), tb, s);
        io.out(tb, theta_bar);
        if (u_bar) io.out(ub, u_bar);
        FVM_CUDA(cudaStreamSynchronize(s));
        return FVM_OK;
    });
}

}  // extern "C"
