// Internal declarations of libfvmgpu: handles, device buffers, kernel launchers.
#pragma once
struct fvm_mesh;
#include <cuda_runtime.h>
#include <cmath>
#include <cstdint>
#include <cstddef>
#include <string>
#include <vector>
#include <memory>
#include <stdexcept>
#include <functional>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include "../../include/fvm_gpu.h"

namespace fvm {

// ---- errors ------------------------------------------------------------------------
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};
void set_last_error(const std::string& msg);
[[noreturn]] void fail(int code, const std::string& msg);
void cuda_check(cudaError_t e, const char* what);
#define FVM_CUDA(x) ::fvm::cuda_check((x), #x)

// Set-up phase timing on stderr when FVM_SETUP_TRACE is set: mark("phase") prints the time
// since the previous mark (or construction).
struct SetupTrace {
    const char* scope;
    bool on;
    std::chrono::steady_clock::time_point t0;
    explicit SetupTrace(const char* s) : scope(s), on(std::getenv("FVM_SETUP_TRACE") != nullptr),
                                         t0(std::chrono::steady_clock::now()) {}
    void mark(const char* phase) {
        if (!on) return;
        auto t1 = std::chrono::steady_clock::now();
        std::fprintf(stderr, "[fvm setup] %s %s %.1f ms\n", scope, phase,
                     std::chrono::duration<double, std::milli>(t1 - t0).count());
        t0 = t1;
    }
};

// ---- device buffer (RAII) ------------------------------------------------------------
struct DBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept : p(o.p), bytes(o.bytes) {
        o.p = nullptr;
        o.bytes = 0;
    }
    DBuf& operator=(DBuf&& o) noexcept {
        if (this != &o) {
            release();
            p = o.p;
            bytes = o.bytes;
            o.p = nullptr;
            o.bytes = 0;
        }
        return *this;
    }
    ~DBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    void alloc(size_t n) {
        release();
        if (n == 0) return;
        cudaError_t e = cudaMalloc(&p, n);
        if (e != cudaSuccess) {
            p = nullptr;
            cudaGetLastError();
            fail(e == cudaErrorMemoryAllocation ? FVM_ERR_OUT_OF_MEMORY : FVM_ERR_CUDA,
                 std::string("cudaMalloc(") + std::to_string(n) + " bytes): " + cudaGetErrorString(e));
        }
        bytes = n;
    }
    template <class T> void upload(const std::vector<T>& v) {
        alloc(v.size() * sizeof(T));
        if (!v.empty()) FVM_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

// ---- sliced-ELL operator (slice height 32, one warp per slice, column-major slots) ----
constexpr int kSlice = 32;
constexpr int kSteadyWindow = 1024;  // rows sorted by length within windows of this many rows

struct SellPattern {
    int64_t nrows = 0, nslices = 0, nslots = 0, nnz = 0;
    int maxw = 0;                    // widest slice
    std::vector<int64_t> slice_ptr;  // [nslices+1] slot offsets (multiples of 32)
    std::vector<int32_t> width;      // [nslices]
    std::vector<int32_t> col;        // [nslots] internal column (pad: the row itself)
    std::vector<int64_t> rowptr;     // CSR view: [nrows+1]
    std::vector<int32_t> csr_col;    // CSR columns (sorted)
    std::vector<int64_t> csr_slot;   // CSR entry -> SELL slot
    DBuf d_slice_ptr, d_width, d_col;
    // per-row destination CTAs of the cluster Tsit5 driver (fvm_cluster.cu), for one shape
    mutable DBuf d_cluster_dest;
    mutable std::vector<uint32_t> cluster_expect;
    mutable int cluster_dest_key = -1;
    mutable int cluster_size = -1, cluster_cap = -1;  // chosen cluster size for the cap in force
    // slot of (row, col), or -1
    int64_t find(int32_t row, int32_t c) const;
    // CSR position of (row, col), or -1
    int64_t find_csr(int32_t row, int32_t c) const;
};

// ---- mesh ----------------------------------------------------------------------------
// Point location and interpolation data (fvm_post.cu), built on first use: a uniform grid
// over the bounding box, each cell listing (in ascending order) the triangles whose bounding
// box meets it; the points, triangles and shape coefficients in the caller's numbering.
struct Locator {
    bool ready = false;
    double xmin = 0, ymin = 0, h = 1;
    int64_t gx = 1, gy = 1;
    DBuf d_cell_start, d_cell_tri;  // [gx*gy+1], [pairs]
    DBuf d_pts, d_tri, d_shape;     // [np][2], [nt][3], [nt][9]
};

// The work queue of the fused host-array RHS (fvm_e2e.cu) for one mesh: A items read caller
// chunks of u from the host, B items compute blocks of slices, C items write caller chunks of
// du; each lists the items it waits for.
struct E2ePlan {
    bool built = false;
    int nA = 0, nB = 0, nC = 0, nitems = 0;
    int chunk = 0, spi = 0;  // caller points per A / C item, slices per B item
    DBuf d_order, d_dep_ptr, d_dep, d_flags, d_counter;
    unsigned epoch = 0;      // flags equal to the current call's epoch are done
    void build(const ::fvm_mesh* m);
};

struct Tiles {
    bool built = false;
    int tile_vertices = 0;
    int64_t ntiles = 0, nelem = 0, nbelem = 0;
    std::vector<int64_t> off, boff;            // [ntiles+1]
    std::vector<int32_t> etri, ebedge;         // element -> caller triangle / boundary edge
    std::vector<int32_t> ev;                   // [3][nelem] internal vertex ids (SoA)
    std::vector<int32_t> bv;                   // [3][nbelem] (i, j, k) internal
    DBuf d_off, d_boff, d_ev, d_bv;
    DBuf d_g, d_bg;                            // geometric flux coefficients [6][nelem], [3][nbelem]
};

}  // namespace fvm

struct fvm_mesh {
    int64_t np = 0, nt = 0, nbe = 0, nv = 0;   // points, triangles, boundary edges, vertices
    int device = -1;                            // device current at creation (holds the arrays)
    std::vector<double> pts;                    // [2*np] caller order
    std::vector<int32_t> tri;                   // [3*nt]
    std::vector<int32_t> be;                    // [2*nbe]
    std::vector<int32_t> badj;                  // [nbe]
    std::vector<int32_t> btri;                  // [nbe] triangle holding the boundary edge
    std::vector<uint8_t> has_vertex;            // [np]
    std::vector<double> vol;                    // [np] control-volume areas
    std::vector<double> props;                  // [24*nt] TriangleProperties
    std::vector<int32_t> perm, iperm;           // perm[internal] = caller, iperm[caller] = internal
    fvm::SellPattern pat;                       // vertex-neighbour pattern with the diagonal (templates)
    fvm::SellPattern pat_off;                   // off-diagonal neighbours only (difference-form RHS)
    fvm::Tiles tiles;
    fvm::Locator loc;
    fvm::E2ePlan e2e;
    fvm::DBuf d_perm, d_iperm, d_invV;          // d_invV internal order
    int tile_vertices_req = 0;
    void build_tiles();
};

struct fvm_problem {
    fvm_mesh* mesh = nullptr;
    int precision = FVM_FP64;
    int dif_deg = 0, neu_deg = 0, src_deg = 0, dudt_deg = 0;
    bool linear = true;                         // every form is affine in u (quadratic only on the diagonal)
    bool conditions_only = false;               // a template's conditions: no operator assembled
    std::vector<int8_t> code;                   // [np] caller order
    std::vector<int8_t> bneu;                   // [nbe]
    std::vector<double> dualD, quarterD, quarterN, src, dudt, dirv;  // copies of the descriptor arrays
    std::vector<double> dualM, quarterM;        // a linear flux q = M (alpha, beta, gamma), 6 per point
    bool flux_linear = false;
    // time factors: b(t) = b + sum_g tau_g(t) b_g, Dirichlet values val + sum_g tau_g(t) val_g
    int ntime = 0;
    bool tdir_varies = false;                   // some time-dependent Dirichlet value is nonzero
    std::vector<double> tfac;                   // [ntime][4] kind, t_ref, a, b
    fvm::DBuf d_tb, d_tdir, d_beff;             // [ntime][np] internal, [ntime][ndir], [np]
    // linear operator path, explicit form on the pattern with the diagonal (default):
    //   du_i = rowscale_i * sum_j A_ij u_j + b_i + q_i u_i^2
    // and difference form on the off-diagonal pattern (FVM_RHS_CONSERVATIVE):
    //   du_i = rowscale_i * sum_{j != i} K_ij (u_j - u_i) + d_i u_i + b_i + q_i u_i^2
    fvm::DBuf d_val64, d_val32;                 // explicit A (FP64; FP32 unscaled by 1/V)
    fvm::DBuf d_kval64, d_kval32, d_d;          // difference form K, d
    fvm::DBuf d_b, d_q, d_rowscale, d_u32;
    bool has_b = false, has_q = false, has_d = false;
    int64_t op_nonzeros = 0;
    // triangle path
    bool tri_ready = false;
    fvm::DBuf d_ec, d_bc;                       // element coefficients, boundary-element coefficients
    fvm::DBuf d_code, d_vsrc, d_vdudt;          // internal order vertex data
    // Dirichlet list
    int64_t ndir = 0;
    fvm::DBuf d_dir_idx, d_dir_val;
    // work buffers (internal order)
    fvm::DBuf d_u, d_du, d_ref;
    void ensure_work();
    void build_triangle_path();
};

struct fvm_template {
    fvm_problem* prob = nullptr;
    int kind = 0;
    fvm::DBuf d_val64, d_val32, d_b, d_u32;
    std::vector<double> val, b;                 // SELL values (internal), b internal
    // steady solve: the reduced system B z = rhs on the free rows (fixed rows are identity
    // rows), on its own row order: the mesh order with rows sorted by length (longest first)
    // within windows of kSteadyWindow rows, and entries that vanish (eliminated columns)
    // dropped, so slices are nearly full and mostly take the unrolled eight-slot path
    bool steady_ready = false;
    int symmetric = 0;
    double bnorm = 0;
    double cheb_gershgorin = 0;                  // Gershgorin bound on the spectrum of D^-1 B
    fvm::SellPattern spat;                       // pattern of B, solver order
    std::vector<int32_t> sperm;                  // solver row -> caller index
    fvm::DBuf d_sperm;
    fvm::DBuf d_bval64, d_bval32;                // B explicit (FP64, FP32)
    fvm::DBuf d_brow64, d_brow32;                // row sums of B, compensated, for the difference form
    fvm::DBuf d_bdiag_inv64, d_bdiag_inv32, d_rhs_red;
    fvm::DBuf d_xfix, d_invV_free64, d_invV_free32;
    fvm::DBuf d_fixed_mask;                      // 1 on rows fixed by Dirichlet / missing vertex
    void build_steady();
};

#ifdef __CUDACC__
#define FVM_HD __host__ __device__
#else
#define FVM_HD
#endif

namespace fvm {
// Tsit5's free 4th-order continuous extension (Tsitouras 2011, Comput. Math. Appl. 62:770-775),
// the dense output OrdinaryDiffEq's Tsit5 interpolates saveat with:
//     u(t_n + theta h) = u_n + h sum_i w_i(theta) k_i
// over the seven stage derivatives, k_7 = f(u_{n+1}).  w_i(1) are the step's weights.
FVM_HD inline void tsit5_interp_weights(double t, double w[7]) {
    w[0] = -1.0530884977290216 * t * (t - 1.3299890189751412) * (t * t - 1.4364028541716351 * t + 0.7139816917074209);
    w[1] = 0.1017 * t * t * (t * t - 2.1966568338249754 * t + 1.2949852507374631);
    w[2] = 2.490627285651252793 * t * t * (t * t - 2.38535645472061657 * t + 1.57803468208092486);
    w[3] = -16.54810288924490272 * (t - 1.21712927295533244) * (t - 0.61620406037800089) * t * t;
    w[4] = 47.37952196281928122 * (t - 1.203071208372362603) * (t - 0.658047292653547382) * t * t;
    w[5] = -34.87065786149660974 * (t - 1.2) * (t - 0.666666666666666667) * t * t;
    w[6] = 2.5 * (t - 1) * (t - 0.6) * t * t;
}
// The same weights as polynomials: w_i(theta) = sum_{p=1..4} beta[i][p-1] theta^p (the
// products above multiplied out), for drivers that keep running sums sum_i beta[i][p] k_i.
void tsit5_interp_poly(double beta[7][4]);

// Sliced ELL from a pattern's CSR view (rowptr, csr_col): slices of 32 rows, width = longest
// row of the slice, slots column-major, padding slots pointing at the row itself (fvm_mesh.cpp)
void finalize_sell(SellPattern& pat, int64_t nrows);
// kernels (fvm_kernels.cu)
void launch_sell_apply64(const SellPattern& p, const double* val, const double* x, double* y,
                         const double* rowscale, const double* b, const double* q, cudaStream_t s);
// FP32 variants gather x32 (an FP32 copy of x made by launch_to_f32) and use x for the row's own terms
void launch_sell_apply32(const SellPattern& p, const float* val, const float* x32, const double* x, double* y,
                         const double* rowscale, const double* b, const double* q, cudaStream_t s);
// y_i = rowscale_i * sum_j K_ij (x_j - x_i) + d_i x_i + b_i + q_i x_i^2 (any of rowscale, d, b, q may be null)
void launch_sell_diff64(const SellPattern& p, const double* val, const double* x, double* y, const double* rowscale,
                        const double* d, const double* b, const double* q, cudaStream_t s);
void launch_sell_diff32(const SellPattern& p, const float* val, const float* x32, const double* x, double* y,
                        const double* rowscale, const double* d, const double* b, const double* q, cudaStream_t s);
void launch_to_f32(const double* x, float* y, int64_t n, cudaStream_t s);
// error bits left by a kernel whose bounded wait ran out (0 = none); reading clears them
unsigned take_device_error();
unsigned* device_error_word();  // device address of the error word the streamed kernels set
void launch_permute_in(const int32_t* perm, const double* xref, double* xint, int64_t n, cudaStream_t s);
void launch_permute_out(const int32_t* perm, const double* xint, double* xref, int64_t n, cudaStream_t s);
// the same with iperm (caller -> internal) and the caller's side in order (host-mapped arrays)
void launch_permute_in_seq(const int32_t* iperm, const double* xref, double* xint, int64_t n, cudaStream_t s);
void launch_permute_out_seq(const int32_t* iperm, const double* xint, double* xref, int64_t n, cudaStream_t s);
void launch_permute_out_snapshots(const int32_t* iperm, const double* xint, double* xref, int64_t n, int64_t nsave,
                                  cudaStream_t s);
void launch_dirichlet(const int32_t* idx, const double* val, double* u, int64_t n, cudaStream_t s);
void launch_triangle_rhs(const fvm_mesh* m, const fvm_problem* p, const double* u, double* du, cudaStream_t s);
// Tsit5 stage: y = u + dt * sum_j a[j] * k[j]  (nk vectors)
void launch_stage(double* y, const double* u, const double* const* k, const double* a, int nk, double dt,
                  int64_t n, cudaStream_t s);
// err_i = dt * sum_j bt[j] k[j]; accumulates sum((err_i / (abstol + max(|u|,|unew|) reltol))^2)
void launch_error_norm(const double* u, const double* unew, const double* const* k, const double* bt,
                       double dt, double abstol, double reltol, int64_t n, double* d_acc, cudaStream_t s);
// saveat value inside a step: out = u + h sum_j w_j(theta) k_j (seven stage derivatives)
void launch_tsit5_interp(double* out, const double* u, const double* const* k, double h, double theta, int64_t n,
                         cudaStream_t s);
// Krylov helpers
void launch_fill(double* x, double v, int64_t n, cudaStream_t s);

// Device-side state of the graph-looped adaptive Tsit5 (fvm_kernels.cu, fvm_api.cpp)
struct AdaptState {
    double t, dt, h, tf, qold, t_prev, tspan, abstol, reltol;
    int64_t nacc, nrej, step, max_steps, si, nsave;
    uint64_t start_ns;             // device clock at the first attempted step (0: not started)
    int32_t accept, last, status;  // status: 0 running, 1 max_steps, 2 dt underflow, 3 non-finite
                                   // error, 4 device time limit
};
void launch_adapt_begin(AdaptState* st, cudaStream_t s);
// Jacobian of fvm_eqs!: J(u) v on the per-triangle path (diag: diag J(u), v unused)
void launch_triangle_jvp(const fvm_mesh* m, const fvm_problem* p, const double* u, const double* v, double* jv,
                         bool diag, cudaStream_t s);
// y += 2 q u v, or (diag non-null) y = diag + 2 q u
void launch_quad_jvp(const double* q, const double* u, const double* v, const double* diag, double* y, int64_t n,
                     cudaStream_t s);
void launch_stage_dev(double* y, const double* u, const double* const* k, const double* a, int nk,
                      const AdaptState* st, int64_t n, cudaStream_t s);
void launch_error_partial_dev(const double* u, const double* unew, const double* const* k, const double* bt,
                              const AdaptState* st, int64_t n, double* part, int nparts, cudaStream_t s);
void launch_adaptive_step_tail(AdaptState* st, const double* part, int nparts, int64_t n,
                               cudaGraphConditionalHandle cond, double* out, double* u, const double* unew,
                               double* const* k, const double* saveat, cudaStream_t s);
void launch_adaptive_step_end(AdaptState* st, double* out, const double* u, const double* saveat, int64_t n,
                              cudaStream_t s);

}  // namespace fvm

// The mesh build of fvm_mesh_create on the device (fvm_mesh_dev.cu): geometry, control volumes,
// boundary-edge triangles, Hilbert order and the vertex-neighbour pattern, identical to the host
// build; fills the host copies the set-up code reads.
namespace fvm {
void mesh_ingest_device(fvm_mesh* m, const int32_t* boundary_adjacent, bool renumber);
}

// Linear terms of a problem's RHS: emit(row, col, coef, didx, flux), rows and columns in the
// caller's numbering; the coefficient multiplies D[didx] when didx >= 0 (fvm_problem.cpp).
using LinearTermSink = std::function<void(int32_t, int32_t, double, int64_t, bool)>;
void fvm_visit_linear_terms(const fvm_problem* p, const LinearTermSink& emit, std::vector<double>& b,
                            std::vector<double>& q, std::vector<double>& rowscale);
// The constant terms that values neu [nbedge*2] (Neumann q.n), src [npoints] (source on FREE
// vertices) and dudt [npoints] (Dudt vertices) add to the RHS, internal numbering (any may be null).
std::vector<double> fvm_time_constant_terms(const fvm_problem* p, const double* neu, const double* src,
                                            const double* dudt);

// Terms of a linear template's A and b: emitA(row, col, coef, didx) adds coef * D[didx] (coef
// alone when didx < 0) to A[row][col]; emitb(row, -1, coef, didx) likewise to b[row].  Rows and
// columns in the caller's numbering; D[didx] are the dual-edge samples then the boundary
// quarter-point samples (fvm_template.cpp).
using TemplateTermSink = std::function<void(int32_t, int32_t, double, int64_t)>;
void fvm_template_visit_terms(const fvm_template* T, const TemplateTermSink& emitA, const TemplateTermSink& emitb);

namespace fvm {
// A stream that can be captured: the caller's, or a private one ordered after the legacy
// default stream (which cannot be captured) and joined back into it on destruction.
struct CaptureStream {
    cudaStream_t user, s, own = nullptr;
    CaptureStream(cudaStream_t u, bool need) : user(u), s(u) {
        if (!need || u != nullptr) return;
        FVM_CUDA(cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking));
        cudaEvent_t e;
        FVM_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        FVM_CUDA(cudaEventRecord(e, user));
        FVM_CUDA(cudaStreamWaitEvent(own, e, 0));
        cudaEventDestroy(e);
        s = own;
    }
    ~CaptureStream() {
        if (!own) return;
        cudaEvent_t e;
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess) {
            cudaEventRecord(e, own);
            cudaStreamWaitEvent(user, e, 0);
            cudaEventDestroy(e);
        }
        cudaStreamDestroy(own);
    }
};

// A batched CSR operator on [rows][B] state (instance index fastest) with per-instance values
// val[k][B]: du[r][b] = sum_k val[k][b] u[col_k][b] + bvec[r] + q[r] u[r][b]^2.  One warp per
// (row, chunk of instances); the launch shape is tuned on the first application (fvm_batch.cu).
struct BatchOp {
    int64_t np = 0, nnz = 0;
    int B = 0, precision = FVM_FP64;
    const int64_t* rowptr = nullptr;
    const int32_t* col = nullptr;
    const void* val = nullptr;
    const void* b = nullptr;  // per-row constant shared by the instances, or null
    const void* q = nullptr;  // per-row quadratic coefficient, or null
    int block = 256, vec = 1;
    int64_t grid = 0;
    bool tuned = false;
};
template <class T>
void batch_op_apply(BatchOp& op, const T* u, T* du, cudaStream_t s);
// A row epilogue of the batched product: z = x0 + sum_t c_t v_t over [np][B] arrays, in list
// order, where a null v_t stands for the product just formed (x0 may be null; z may alias x0
// but not the product's input).
template <class T>
struct BatchEpi {
    T* z = nullptr;
    const T* x0 = nullptr;
    const T* v[8] = {};
    double c[8] = {};
    int nv = 0;
};
// du = A u (+ b), and the epilogue E formed in the same pass (du may be null)
template <class T>
void batch_op_apply_epi(BatchOp& op, const T* u, T* du, const BatchEpi<T>& E, cudaStream_t s);
// val[k][b] = cst[k] + sum_{m in [mptr[k], mptr[k+1])} mcoef[m] D[midx[m]][b]  (FP64 or FP32 val)
void launch_batch_assemble(const int64_t* mptr, const int32_t* midx, const double* mcoef, const double* cst,
                           const double* D, void* val, int64_t nnz, int B, int precision, cudaStream_t s);

// An RHS that is the FP64 explicit sliced-ELL product f(u) = A u + q u^2 + b together with a
// Dirichlet callback u[dir_idx] = dir_val (both optional parts may be null).  With it, a small
// mesh's adaptive Tsit5 loop runs inside one thread-block cluster (fvm_cluster.cu).
struct SellRhsDesc {
    const SellPattern* pat = nullptr;
    const double* val = nullptr;
    const double* b = nullptr;
    const double* q = nullptr;
    const int32_t* dir_idx = nullptr;
    const double* dir_val = nullptr;
    int64_t ndir = 0;
};

// Right-hand side in the internal numbering plus the per-step callback (Dirichlet update).
struct OdeRhs {
    std::function<void(const double*, double*, double, cudaStream_t)> f;
    std::function<void(double*, double, cudaStream_t)> callback;  // may be empty
    SellRhsDesc sell;  // set when f (and callback) are exactly the described product and update
    // f depends on t: every step runs on the host-controlled loop (captured steps replay fixed t)
    bool time_dependent = false;
    // the callback's values depend on t: it changes u after every step, so the first-same-as-
    // last derivative is evaluated again after it (as after the first callback otherwise)
    bool callback_varies = false;
};

// the cluster-resident adaptive Tsit5 driver (fvm_cluster.cu); meshes up to kClusterMaxRows
constexpr int64_t kClusterMaxRows = 7680;
bool cluster_tsit5_available(const SellPattern& pat);
void launch_cluster_tsit5(const SellRhsDesc& d, const double* dirval, double* u, double* k0, double* out,
                          const double* saveat, AdaptState* st, const double (*A)[6], const double* bt,
                          cudaStream_t s);
// Copies nsave internal-order device snapshots [nsave][n] to the caller's host array in the
// caller's numbering: written directly when the array is page-locked, else through a device
// staging buffer in chunks of at most 64 MiB, one copy per chunk.  Does not synchronise.
void snapshots_to_host(const int32_t* iperm, const double* src, double* out, int64_t n, int64_t nsave,
                       cudaStream_t s);
void tsit5_run_internal(OdeRhs& rhs, int64_t n, const double* u0_int, const fvm_ode_options& o, double* out_int,
                        fvm_ode_stats* st, cudaStream_t s);
int guard_call(const std::function<int()>& f);
void problem_rhs_internal(fvm_problem* p, const double* u, double* du, bool force_triangle, cudaStream_t s,
                          bool conservative = false, double t = 0.0);
// the problem's Dirichlet update u_i = a(x_i, y_i, t) in the internal numbering
void problem_dirichlet_internal(const fvm_problem* p, double* u, double t, cudaStream_t s);
// tau(t) of a time factor {kind, t_ref, a, b}
inline double time_factor_value(const double* f, double t) {
    const double d = t - f[1];
    return f[0] == 1.0 ? std::exp(f[2] * d) : 1.0 + d * (f[2] + d * f[3]);
}
constexpr int kMaxTime = FVM_MAX_TIME_FACTORS;
struct TimeTaus {
    double tau[kMaxTime];
};
// out = b + sum_g tau_g tb[g] (b may be null); u[idx[k]] = val[k] + sum_g tau_g tval[g][k]
void launch_time_b(const double* b, const double* tb, const TimeTaus& tt, int ntime, double* out, int64_t n,
                   cudaStream_t s);
void launch_dirichlet_time(const int32_t* idx, const double* val, const double* tval, const TimeTaus& tt, int ntime,
                           double* u, int64_t n, cudaStream_t s);
// tau_g(t) of the problem's time factors
TimeTaus problem_time_taus(const fvm_problem* p, double t);
// fvm_eqs! from a page-locked host u into a page-locked host du (device addresses of both), one
// launch overlapping the link transfers with the product (fvm_e2e.cu); false when the problem
// is not on the FP64 operator path (the caller then takes the general path)
bool problem_rhs_host_fused(fvm_problem* p, const double* uh, double* dh, double t, cudaStream_t s);

// What the implicit integrator needs of a right-hand side, in the internal numbering: f(y, t),
// J(u) v, diag J(u), and the Dirichlet update after a step (optional).  callback_varies: the
// update changes u at every step (time-dependent values).  affine: f is affine in u with an
// exact J, so one Newton iteration solves a stage.
struct ImplicitRhs {
    std::function<void(const double*, double*, double, cudaStream_t)> f;
    std::function<void(const double*, const double*, double*, cudaStream_t)> jvp;
    std::function<void(const double*, double*, cudaStream_t)> diag;
    std::function<void(double*, double, cudaStream_t)> callback;
    bool callback_varies = false;
    bool affine = false;
    const double* fixed = nullptr;  // steady Newton: 1 on the rows the problem fixes, else 0 (internal)
    // when J v is exactly A v (+ 2 q u v) for a sliced-ELL A on op_pat: the Krylov solves may run
    // as one cooperative launch (fvm_implicit.cu) instead of a launch per vector operation
    const SellPattern* op_pat = nullptr;
    const double* op_val = nullptr;
    const double* op_q = nullptr;
};
// DynamicSS's stopping test on a TR-BDF2 run: after each accepted step, max|f(u)| <= abstol or
// <= reltol max|f(u) + u| ends the run with u as its one output
struct SteadyStop {
    double abstol = 0, reltol = 0;
    bool converged = false;
    double residual = 0;
};
// TR-BDF2 on R over n unknowns; u0 and out are host arrays in the caller's numbering, perm (internal
// -> caller) and iperm (caller -> internal) device index arrays.  Throws on error.
int trbdf2_run(ImplicitRhs& R, const int32_t* perm, const int32_t* iperm, int64_t n, const double* u0,
               const fvm_ode_options* o, double* out, fvm_ode_stats* st, fvm_implicit_stats* ist, void* stream,
               SteadyStop* stop = nullptr);
// fvm_steady_solve on R (either method); fills out and st, then throws FVM_ERR_NOT_CONVERGED if the
// test was not met
void steady_run(ImplicitRhs& R, const int32_t* perm, const int32_t* iperm, int64_t n, const double* u0,
                const fvm_steady_options* o, double* out, fvm_steady_stats* st, void* stream);
}  // namespace fvm
