// C ABI of libfvmgpu: handle management, fvm_rhs, the Dirichlet update and Tsit5.
#include "fvm_internal.h"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>

namespace fvm {

static thread_local std::string g_last_error;

void set_last_error(const std::string& msg) { g_last_error = msg; }

void fail(int code, const std::string& msg) { throw Error(code, msg); }

void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        cudaGetLastError();
        fail(e == cudaErrorMemoryAllocation ? FVM_ERR_OUT_OF_MEMORY : FVM_ERR_CUDA,
             std::string(what) + ": " + cudaGetErrorString(e));
    }
}

template <class F>
static int guard(F&& f) {
    try {
        return f();
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::bad_alloc&) {
        set_last_error("host out of memory");
        return FVM_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return FVM_ERR_INVALID_ARGUMENT;
    }
}

static void check_launch() { FVM_CUDA(cudaGetLastError()); }
// after a stream synchronisation: reports a kernel whose bounded wait ran out
static void check_device_error() {
    if (unsigned e = take_device_error())
        fail(FVM_ERR_CUDA, "a kernel timed out in a bounded wait (device error bits " + std::to_string(e) +
                               "; 1, 2: the streamed kernel's stages; 4: the host-array RHS's work items)");
}

// Tsit5 tableau (Tsitouras 2011, as published).
static const double kC[7] = {0.0, 0.161, 0.327, 0.9, 0.9800255409045097, 1.0, 1.0};
static const double kA[7][6] = {
    {0, 0, 0, 0, 0, 0},
    {0.161, 0, 0, 0, 0, 0},
    {-0.008480655492356989, 0.335480655492357, 0, 0, 0, 0},
    {2.897153057105493, -6.359448489975075, 4.3622954328695815, 0, 0, 0},
    {5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525, 0, 0},
    {5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383, 0},
    {0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774},
};
static const double kBt[7] = {-0.00178001105222577714, -0.0008164344596567469, 0.007880878010261995,
                              -0.1447110071732629,     0.5823571654525552,      -0.45808210592918697,
                              0.015151515151515152};

struct EventPair {
    cudaEvent_t a = nullptr, b = nullptr;
    EventPair() {
        FVM_CUDA(cudaEventCreate(&a));
        FVM_CUDA(cudaEventCreate(&b));
    }
    ~EventPair() {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
};

static double host_rms(const std::vector<double>& v, const std::vector<double>& sc) {
    double s = 0;
    for (size_t i = 0; i < v.size(); ++i) {
        double r = v[i] / sc[i];
        s += r * r;
    }
    return std::sqrt(s / std::max<size_t>(1, v.size()));
}

// Tsit5 driver.  u0_int: device, internal numbering.  out_int: device [nsave][n] internal.
static void tsit5_run(OdeRhs& rhs, int64_t n, const double* u0_int, const fvm_ode_options& o, double* out_int,
                      fvm_ode_stats* st, cudaStream_t user_stream) {
    if (!(o.tf > o.t0)) fail(FVM_ERR_INVALID_ARGUMENT, "final time must exceed the initial time");
    if (!std::isfinite(o.tf)) fail(FVM_ERR_INVALID_ARGUMENT, "the final time must be finite (a steady problem is solved by fvm_steady_solve)");
    CaptureStream cs(user_stream, o.use_graph != 0);
    cudaStream_t s = cs.s;
    std::vector<double> saveat;
    if (o.saveat && o.nsave > 0)
        saveat.assign(o.saveat, o.saveat + o.nsave);
    else
        saveat.push_back(o.tf);
    for (size_t i = 0; i < saveat.size(); ++i) {
        if (saveat[i] < o.t0 || saveat[i] > o.tf) fail(FVM_ERR_INVALID_ARGUMENT, "saveat times must lie in [t0, tf]");
        if (i && saveat[i] < saveat[i - 1]) fail(FVM_ERR_INVALID_ARGUMENT, "saveat must be sorted");
    }
    DBuf buf;
    buf.alloc(sizeof(double) * n * 10 + sizeof(double) * 512);
    double* base = buf.as<double>();
    double* u = base;
    double* unew = base + n;
    double* y = base + 2 * n;
    double* k[7];
    for (int j = 0; j < 7; ++j) k[j] = base + (3 + j) * n;
    double* d_acc = base + 10 * n;
    FVM_CUDA(cudaMemcpyAsync(u, u0_int, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    size_t si = 0;
    int64_t nrhs = 0, nacc = 0, nrej = 0;
    double t = o.t0;
    auto save_copy = [&](const double* src) {
        FVM_CUDA(cudaMemcpyAsync(out_int + si * n, src, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        ++si;
    };
    while (si < saveat.size() && saveat[si] == o.t0) save_copy(u);
    EventPair ev;
    FVM_CUDA(cudaEventRecord(ev.a, s));
    rhs.f(u, k[0], t, s);
    ++nrhs;
    double dt = o.dt;
    const double tspan = o.tf - o.t0;
    int64_t max_steps = o.max_steps > 0 ? o.max_steps : 100000000;
    // automatic initial step (Hairer-Wanner, as OrdinaryDiffEq's ode_determine_initdt, order 5)
    if (o.adaptive && !(dt > 0)) {
        std::vector<double> h_u(n), h_f0(n), h_f1(n), sc(n), tmp(n);
        FVM_CUDA(cudaMemcpyAsync(h_u.data(), u, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
        FVM_CUDA(cudaMemcpyAsync(h_f0.data(), k[0], sizeof(double) * n, cudaMemcpyDeviceToHost, s));
        FVM_CUDA(cudaStreamSynchronize(s));
        for (int64_t i = 0; i < n; ++i) sc[i] = o.abstol + std::fabs(h_u[i]) * o.reltol;
        double d0 = host_rms(h_u, sc), d1 = host_rms(h_f0, sc);
        double dt0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * d0 / d1;
        dt0 = std::min(dt0, tspan);
        for (int64_t i = 0; i < n; ++i) tmp[i] = h_u[i] + dt0 * h_f0[i];
        FVM_CUDA(cudaMemcpyAsync(y, tmp.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
        rhs.f(y, k[1], t + dt0, s);
        ++nrhs;
        FVM_CUDA(cudaMemcpyAsync(h_f1.data(), k[1], sizeof(double) * n, cudaMemcpyDeviceToHost, s));
        FVM_CUDA(cudaStreamSynchronize(s));
        for (int64_t i = 0; i < n; ++i) tmp[i] = h_f1[i] - h_f0[i];
        double d2 = host_rms(tmp, sc) / dt0;
        double md = std::max(d1, d2);
        double dt1 = md <= 1e-15 ? std::max(1e-6, dt0 * 1e-3) : std::pow(10.0, -(2.0 + std::log10(md)) / 5.0);
        dt = std::min({100 * dt0, dt1, tspan});
    }
    if (!(dt > 0)) fail(FVM_ERR_INVALID_ARGUMENT, "dt must be positive for fixed-step Tsit5");
    bool first_callback = true;
    const double beta1 = 7.0 / 50.0, beta2 = 2.0 / 25.0, qmin = 0.2, qmax = 10.0, gamma = 0.9;
    double qold = 1e-4;
    // fixed steps with nothing to save before tf run as a captured CUDA graph
    bool graph_ok = !o.adaptive && o.use_graph && si + 1 == saveat.size() && saveat.back() == o.tf &&
                    !rhs.time_dependent;
    int64_t nfixed = o.adaptive ? 0 : (int64_t)std::ceil(tspan / dt - 1e-9);
    if (!o.adaptive && nfixed > max_steps) fail(FVM_ERR_STEP_LIMIT, "fixed-step Tsit5 needs more than max_steps steps");
    int64_t step = 0;
    auto stages = [&](double* ydst7, double tt, double h) {
        for (int sidx = 1; sidx < 7; ++sidx) {
            double* dst = sidx == 6 ? ydst7 : y;
            launch_stage(dst, u, k, kA[sidx], sidx, h, n, s);
            if (sidx < 6) {
                rhs.f(y, k[sidx], tt + kC[sidx] * h, s);
                ++nrhs;
            }
        }
    };
    // Adaptive steps after the first accepted one run on the device: the step size, the PI
    // control and the saveat cursor live in device memory.  Small meshes with a sliced-ELL RHS
    // run the whole loop in one thread-block cluster; otherwise one graph launch loops over
    // attempted steps with a conditional WHILE node until tf (or an error status) is reached.
    auto device_loop = [&](bool cluster) {
        DBuf dstate;
        const size_t state_bytes = (sizeof(AdaptState) + 15) / 16 * 16;
        dstate.alloc(state_bytes + sizeof(double) * saveat.size());
        AdaptState* d_st = dstate.as<AdaptState>();
        double* d_saveat = reinterpret_cast<double*>(reinterpret_cast<char*>(dstate.p) + state_bytes);
        AdaptState hs{};
        hs.t = t;
        hs.dt = dt;
        hs.tf = o.tf;
        hs.qold = qold;
        hs.tspan = tspan;
        hs.abstol = o.abstol;
        hs.reltol = o.reltol;
        hs.nacc = nacc;
        hs.nrej = nrej;
        hs.step = step;
        hs.max_steps = max_steps;
        hs.si = (int64_t)si;
        hs.nsave = (int64_t)saveat.size();
        FVM_CUDA(cudaMemcpyAsync(d_st, &hs, sizeof hs, cudaMemcpyHostToDevice, s));
        FVM_CUDA(cudaMemcpyAsync(d_saveat, saveat.data(), sizeof(double) * saveat.size(), cudaMemcpyHostToDevice, s));
        cudaGraph_t g = nullptr;
        cudaGraphExec_t exec = nullptr;
        struct GraphGuard {
            cudaGraph_t& g;
            cudaGraphExec_t& e;
            ~GraphGuard() {
                if (e) cudaGraphExecDestroy(e);
                if (g) cudaGraphDestroy(g);
            }
        } guard_g{g, exec};
        DBuf dir;
        if (cluster) {
            const double* dirval = nullptr;
            if (rhs.sell.ndir > 0) {
                dir.alloc(sizeof(double) * n);
                launch_fill(dir.as<double>(), std::nan(""), n, s);
                launch_dirichlet(rhs.sell.dir_idx, rhs.sell.dir_val, dir.as<double>(), rhs.sell.ndir, s);
                dirval = dir.as<double>();
            }
            launch_cluster_tsit5(rhs.sell, dirval, u, k[0], out_int, d_saveat, d_st, kA, kBt, s);
        } else {
            FVM_CUDA(cudaGraphCreate(&g, 0));
            cudaGraphConditionalHandle cond;
            FVM_CUDA(cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault));
            cudaGraphNodeParams cp{};
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = cond;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            cudaGraphNode_t node;
            FVM_CUDA(cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp));
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            const int nparts = 304;
            FVM_CUDA(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
            launch_adapt_begin(d_st, s);
            for (int sidx = 1; sidx < 7; ++sidx) {
                launch_stage_dev(sidx == 6 ? unew : y, u, k, kA[sidx], sidx, d_st, n, s);
                if (sidx < 6) rhs.f(y, k[sidx], t, s);
            }
            rhs.f(unew, k[6], t, s);
            launch_error_partial_dev(u, unew, k, kBt, d_st, n, d_acc, nparts, s);
            launch_adaptive_step_tail(d_st, d_acc, nparts, n, cond, out_int, u, unew, k, d_saveat, s);
            if (rhs.callback) rhs.callback(u, t, s);
            launch_adaptive_step_end(d_st, out_int, u, d_saveat, n, s);
            cudaGraph_t captured = nullptr;
            FVM_CUDA(cudaStreamEndCapture(s, &captured));
            FVM_CUDA(cudaGraphInstantiate(&exec, g, 0));
            FVM_CUDA(cudaGraphLaunch(exec, s));
        }
        check_launch();
        FVM_CUDA(cudaMemcpyAsync(&hs, d_st, sizeof hs, cudaMemcpyDeviceToHost, s));
        FVM_CUDA(cudaStreamSynchronize(s));
        nrhs += 6 * (hs.step - step);
        t = hs.t;
        dt = hs.dt;
        step = hs.step;
        nacc = hs.nacc;
        nrej = hs.nrej;
        si = (size_t)hs.si;
        if (hs.status == 1) fail(FVM_ERR_STEP_LIMIT, "Tsit5 reached max_steps before tf");
        if (hs.status == 2) fail(FVM_ERR_STEP_LIMIT, "Tsit5 step size underflow");
        if (hs.status == 3) fail(FVM_ERR_STEP_LIMIT, "Tsit5 error estimate is not finite (instability)");
        if (hs.status == 4) fail(FVM_ERR_STEP_LIMIT, "Tsit5 device loop stopped at its time limit before tf");
    };
    int32_t driver = FVM_DRIVER_HOST;
    const bool use_cluster = o.adaptive && o.use_graph && rhs.sell.pat && rhs.sell.val &&
                             (rhs.callback == nullptr || rhs.sell.ndir > 0) && cluster_tsit5_available(*rhs.sell.pat);
    while (o.adaptive ? t < o.tf : step < nfixed) {
        if (o.adaptive && o.use_graph && nacc >= 1 && !rhs.time_dependent) {
            driver = use_cluster ? FVM_DRIVER_CLUSTER : FVM_DRIVER_DEVICE_LOOP;
            device_loop(use_cluster);
            break;
        }
        if (step >= max_steps) fail(FVM_ERR_STEP_LIMIT, "Tsit5 reached max_steps before tf");
        double h;
        bool last;
        if (o.adaptive) {
            last = t + dt >= o.tf;
            h = last ? o.tf - t : dt;
        } else {
            last = step + 1 == nfixed;
            double tn = last ? o.tf : o.t0 + (double)(step + 1) * dt;
            h = tn - t;
        }
        if (graph_ok && step >= 1 && step + 1 < nfixed) {
            // steps 2 .. nfixed-1 of a fixed-step run: u updated in place, FSAL through k[0],
            // one captured step replayed; the device-coded forms do not depend on t
            cudaGraph_t graph;
            cudaGraphExec_t exec;
            FVM_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            for (int sidx = 1; sidx < 6; ++sidx) {
                launch_stage(y, u, k, kA[sidx], sidx, dt, n, s);
                rhs.f(y, k[sidx], t + kC[sidx] * dt, s);
            }
            launch_stage(u, u, k, kA[6], 6, dt, n, s);  // u_{n+1} in place
            rhs.f(u, k[0], t + dt, s);                  // FSAL derivative
            if (rhs.callback) rhs.callback(u, t + dt, s);
            FVM_CUDA(cudaStreamEndCapture(s, &graph));
            FVM_CUDA(cudaGraphInstantiate(&exec, graph, 0));
            int64_t reps = nfixed - 1 - step;
            driver = FVM_DRIVER_FIXED_GRAPH;
            for (int64_t r = 0; r < reps; ++r) FVM_CUDA(cudaGraphLaunch(exec, s));
            check_launch();
            cudaGraphExecDestroy(exec);
            cudaGraphDestroy(graph);
            step += reps;
            nacc += reps;
            nrhs += 6 * reps;
            t = o.t0 + (double)step * dt;
            continue;
        }
        stages(unew, t, h);
        rhs.f(unew, k[6], t + h, s);  // k7 at u_{n+1}
        ++nrhs;
        double EEst = 0.0;
        if (o.adaptive) {
            launch_error_norm(u, unew, k, kBt, h, o.abstol, o.reltol, n, d_acc, s);
            double sum = 0;
            FVM_CUDA(cudaMemcpyAsync(&sum, d_acc, sizeof(double), cudaMemcpyDeviceToHost, s));
            FVM_CUDA(cudaStreamSynchronize(s));
            EEst = std::sqrt(sum / std::max<int64_t>(1, n));
            if (!std::isfinite(EEst)) fail(FVM_ERR_STEP_LIMIT, "Tsit5 error estimate is not finite (instability)");
        }
        double q11 = 0.0, q = 0.0;
        if (o.adaptive) {
            if (EEst == 0.0) {
                q = 1.0 / qmax;
            } else {
                q11 = std::pow(EEst, beta1);
                q = q11 / std::pow(qold, beta2);
                q = std::max(1.0 / qmax, std::min(1.0 / qmin, q / gamma));
            }
        }
        if (o.adaptive && EEst > 1.0) {  // reject
            ++nrej;
            ++step;
            dt = h / std::min(1.0 / qmin, q11 / gamma);
            if (dt < 1e-14 * std::max(1.0, std::fabs(t))) fail(FVM_ERR_STEP_LIMIT, "Tsit5 step size underflow");
            continue;
        }
        // accept: interpolate saveat points in (t, t+h), then take the step
        double tn = last ? o.tf : (o.adaptive ? t + h : o.t0 + (double)(step + 1) * dt);
        while (si < saveat.size() && saveat[si] < tn) {
            double th = (saveat[si] - t) / h;
            launch_tsit5_interp(out_int + si * n, u, k, h, th, n, s);
            ++si;
        }
        std::swap(u, unew);
        t = tn;
        ++nacc;
        ++step;
        bool reeval = false;
        if (rhs.callback) {
            rhs.callback(u, t, s);
            // later updates rewrite the same values unless they depend on t
            reeval = first_callback || rhs.callback_varies;
            first_callback = false;
        }
        while (si < saveat.size() && saveat[si] == t) save_copy(u);
        if (reeval) {
            rhs.f(u, k[0], t, s);
            ++nrhs;
        } else {
            std::swap(k[0], k[6]);
        }
        if (o.adaptive) {
            qold = std::max(EEst, 1e-4);
            dt = h / q;
            dt = std::min(dt, tspan);
        }
        if (last) break;
    }
    while (si < saveat.size()) save_copy(u);
    FVM_CUDA(cudaEventRecord(ev.b, s));
    check_launch();
    FVM_CUDA(cudaEventSynchronize(ev.b));
    float ms = 0;
    FVM_CUDA(cudaEventElapsedTime(&ms, ev.a, ev.b));
    if (st) {
        st->driver = driver;
        st->naccept = nacc;
        st->nreject = nrej;
        st->nrhs = nrhs;
        st->t_final = t;
        st->elapsed_ms = ms;
    }
}

// Device address of a page-locked host array (cudaHostAlloc / cudaHostRegister), or nullptr
// for pageable memory.  Kernels read and write such arrays directly over the host link.
static void* host_mapped(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// u/du pointer handling shared by fvm_rhs and fvm_template_apply
struct IoPlan {
    const double* uin = nullptr;  // internal-order input (device)
    double* dout = nullptr;       // internal-order output (device)
};

static void rhs_inputs(fvm_problem* p, const double* u, double* du, int32_t loc, IoPlan& io, cudaStream_t s) {
    fvm_mesh* m = p->mesh;
    if (loc == FVM_PTR_DEVICE_INTERNAL) {
        io.uin = u;
        io.dout = du;
        return;
    }
    p->ensure_work();
    if (loc == FVM_PTR_HOST) {
        if (const void* mapped = host_mapped(u)) {  // no staging copy: the permutation reads the host array
            launch_permute_in_seq(m->d_iperm.as<int32_t>(), (const double*)mapped, p->d_u.as<double>(), m->np, s);
        } else {
            FVM_CUDA(cudaMemcpyAsync(p->d_ref.p, u, sizeof(double) * m->np, cudaMemcpyHostToDevice, s));
            launch_permute_in(m->d_perm.as<int32_t>(), p->d_ref.as<double>(), p->d_u.as<double>(), m->np, s);
        }
    } else {
        launch_permute_in(m->d_perm.as<int32_t>(), u, p->d_u.as<double>(), m->np, s);
    }
    io.uin = p->d_u.as<double>();
    io.dout = p->d_du.as<double>();
}

static void rhs_outputs(fvm_problem* p, double* du, int32_t loc, cudaStream_t s) {
    fvm_mesh* m = p->mesh;
    if (loc == FVM_PTR_DEVICE_INTERNAL) return;
    if (loc == FVM_PTR_HOST) {
        if (void* mapped = host_mapped(du)) {  // the permutation writes the host array
            launch_permute_out_seq(m->d_iperm.as<int32_t>(), p->d_du.as<double>(), (double*)mapped, m->np, s);
        } else {
            launch_permute_out(m->d_perm.as<int32_t>(), p->d_du.as<double>(), p->d_ref.as<double>(), m->np, s);
            FVM_CUDA(cudaMemcpyAsync(du, p->d_ref.p, sizeof(double) * m->np, cudaMemcpyDeviceToHost, s));
        }
        FVM_CUDA(cudaStreamSynchronize(s));
        check_device_error();
    } else {
        launch_permute_out(m->d_perm.as<int32_t>(), p->d_du.as<double>(), du, m->np, s);
    }
}

TimeTaus problem_time_taus(const fvm_problem* p, double t) {
    TimeTaus tt{};
    for (int g = 0; g < p->ntime; ++g) tt.tau[g] = time_factor_value(&p->tfac[4 * g], t);
    return tt;
}
static TimeTaus time_taus(const fvm_problem* p, double t) { return problem_time_taus(p, t); }

void problem_dirichlet_internal(const fvm_problem* p, double* u, double t, cudaStream_t s) {
    if (p->ntime > 0)
        launch_dirichlet_time(p->d_dir_idx.as<int32_t>(), p->d_dir_val.as<double>(), p->d_tdir.as<double>(),
                              time_taus(p, t), p->ntime, u, p->ndir, s);
    else
        launch_dirichlet(p->d_dir_idx.as<int32_t>(), p->d_dir_val.as<double>(), u, p->ndir, s);
}

// fvm_eqs! in the internal numbering
void problem_rhs_internal(fvm_problem* p, const double* u, double* du, bool force_triangle, cudaStream_t s,
                          bool conservative, double t) {
    fvm_mesh* m = p->mesh;
    if (p->conditions_only)
        fail(FVM_ERR_INVALID_ARGUMENT, "this problem carries a template's conditions only (FVM_PROBLEM_CONDITIONS_ONLY)");
    if (p->ntime > 0 && force_triangle)
        fail(FVM_ERR_UNSUPPORTED, "time-dependent values run on the operator path only (no force_triangle)");
    if (p->linear && !force_triangle) {
        const double* dg = p->has_d ? p->d_d.as<double>() : nullptr;
        const double* b = p->has_b ? p->d_b.as<double>() : nullptr;
        if (p->ntime > 0) {  // b(t) = b + sum_g tau_g(t) b_g
            launch_time_b(b, p->d_tb.as<double>(), time_taus(p, t), p->ntime, p->d_beff.as<double>(), m->np, s);
            b = p->d_beff.as<double>();
        }
        const double* q = p->has_q ? p->d_q.as<double>() : nullptr;
        if (p->precision == FVM_FP32) {
            launch_to_f32(u, p->d_u32.as<float>(), m->np, s);
            if (conservative)
                launch_sell_diff32(m->pat_off, p->d_kval32.as<float>(), p->d_u32.as<float>(), u, du,
                                   p->d_rowscale.as<double>(), dg, b, q, s);
            else
                launch_sell_apply32(m->pat, p->d_val32.as<float>(), p->d_u32.as<float>(), u, du,
                                    p->d_rowscale.as<double>(), b, q, s);
        } else if (conservative) {
            launch_sell_diff64(m->pat_off, p->d_kval64.as<double>(), u, du, nullptr, dg, b, q, s);
        } else {
            launch_sell_apply64(m->pat, p->d_val64.as<double>(), u, du, nullptr, b, q, s);
        }
    } else {
        if (p->precision == FVM_FP32 && !p->linear)
            fail(FVM_ERR_UNSUPPORTED_FORM, "FP32 assembly is available for linear forms only");
        p->build_triangle_path();
        launch_triangle_rhs(m, p, u, du, s);
    }
}

}  // namespace fvm

using namespace fvm;

extern "C" int fvm_mesh_create_impl(const double*, int64_t, const int32_t*, int64_t, const int32_t*, const int32_t*,
                                     int64_t, int32_t, int32_t, fvm_mesh**);
extern "C" int fvm_problem_create_impl(fvm_mesh*, const fvm_problem_desc*, fvm_problem**);

extern "C" {

int fvm_version(void) { return 10000; }

int fvm_last_error(char* buf, size_t len) {
    if (!buf || len == 0) return FVM_ERR_INVALID_ARGUMENT;
    size_t n = std::min(len - 1, g_last_error.size());
    std::memcpy(buf, g_last_error.data(), n);
    buf[n] = 0;
    return FVM_OK;
}

int fvm_device_count(int* count) {
    if (!count) return FVM_ERR_INVALID_ARGUMENT;
    int c = 0;
    if (cudaGetDeviceCount(&c) != cudaSuccess) {
        cudaGetLastError();
        c = 0;
    }
    *count = c;
    return FVM_OK;
}

int fvm_mesh_create(const double* points, int64_t npoints, const int32_t* triangles, int64_t ntri,
                    const int32_t* boundary_edges, const int32_t* boundary_adjacent, int64_t nbedge,
                    int32_t tile_vertices, int32_t flags, fvm_mesh** out) {
    return guard([&] {
        return fvm_mesh_create_impl(points, npoints, triangles, ntri, boundary_edges, boundary_adjacent, nbedge,
                                    tile_vertices, flags, out);
    });
}

int fvm_mesh_destroy(fvm_mesh* mesh) {
    return guard([&] {
        delete mesh;
        return FVM_OK;
    });
}

int fvm_mesh_info(const fvm_mesh* m, int64_t* info) {
    return guard([&] {
        if (!m || !info) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        const_cast<fvm_mesh*>(m)->build_tiles();
        info[0] = m->np;
        info[1] = m->nt;
        info[2] = m->nbe;
        info[3] = m->nv;
        info[4] = m->tiles.ntiles;
        info[5] = m->tiles.nelem;
        info[6] = m->tiles.nbelem;
        info[7] = m->tiles.tile_vertices;
        info[8] = m->pat.nslots;
        info[9] = m->pat.nnz;
        return FVM_OK;
    });
}

int fvm_mesh_geometry(const fvm_mesh* m, double* cv, double* props) {
    return guard([&] {
        if (!m) fail(FVM_ERR_INVALID_ARGUMENT, "NULL mesh");
        if (cv) std::memcpy(cv, m->vol.data(), sizeof(double) * m->np);
        if (props) std::memcpy(props, m->props.data(), sizeof(double) * 24 * m->nt);
        return FVM_OK;
    });
}

int fvm_mesh_sample_points(const fvm_mesh* m, double* dual, double* quarter) {
    return guard([&] {
        if (!m) fail(FVM_ERR_INVALID_ARGUMENT, "NULL mesh");
        if (dual)
            for (int64_t t = 0; t < m->nt; ++t)
                for (int e = 0; e < 3; ++e) {
                    dual[6 * t + 2 * e] = m->props[24 * t + 9 + 2 * e];
                    dual[6 * t + 2 * e + 1] = m->props[24 * t + 10 + 2 * e];
                }
        if (quarter)
            for (int64_t e = 0; e < m->nbe; ++e) {
                int32_t i = m->be[2 * e], j = m->be[2 * e + 1];
                double px = m->pts[2 * i], py = m->pts[2 * i + 1], qx = m->pts[2 * j], qy = m->pts[2 * j + 1];
                double mx = (px + qx) / 2, my = (py + qy) / 2;
                quarter[4 * e] = (px + mx) / 2;
                quarter[4 * e + 1] = (py + my) / 2;
                quarter[4 * e + 2] = (qx + mx) / 2;
                quarter[4 * e + 3] = (qy + my) / 2;
            }
        return FVM_OK;
    });
}

int fvm_mesh_permutation(const fvm_mesh* m, int32_t* perm) {
    return guard([&] {
        if (!m || !perm) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        std::memcpy(perm, m->perm.data(), sizeof(int32_t) * m->np);
        return FVM_OK;
    });
}

int fvm_mesh_export_connectivity(const fvm_mesh* mc, int32_t* triangles, int32_t* belems) {
    return guard([&] {
        fvm_mesh* m = const_cast<fvm_mesh*>(mc);
        if (!m) fail(FVM_ERR_INVALID_ARGUMENT, "NULL mesh");
        m->build_tiles();
        const Tiles& T = m->tiles;
        std::vector<int32_t> ev(3 * T.nelem), bv(3 * T.nbelem);
        if (T.nelem) FVM_CUDA(cudaMemcpy(ev.data(), T.d_ev.p, ev.size() * 4, cudaMemcpyDeviceToHost));
        if (T.nbelem) FVM_CUDA(cudaMemcpy(bv.data(), T.d_bv.p, bv.size() * 4, cudaMemcpyDeviceToHost));
        if (triangles) {
            std::fill(triangles, triangles + 3 * m->nt, -1);
            for (int64_t e = 0; e < T.nelem; ++e) {
                int32_t t = T.etri[e];
                int32_t w[3] = {m->perm[ev[e]], m->perm[ev[T.nelem + e]], m->perm[ev[2 * T.nelem + e]]};
                if (triangles[3 * t] >= 0 &&
                    (triangles[3 * t] != w[0] || triangles[3 * t + 1] != w[1] || triangles[3 * t + 2] != w[2]))
                    fail(FVM_ERR_BAD_MESH, "tile copies of a triangle disagree");
                std::memcpy(&triangles[3 * t], w, sizeof(w));
            }
        }
        if (belems) {
            std::fill(belems, belems + 3 * m->nbe, -1);
            for (int64_t q = 0; q < T.nbelem; ++q) {
                int32_t e = T.ebedge[q];
                belems[3 * e] = m->perm[bv[q]];
                belems[3 * e + 1] = m->perm[bv[T.nbelem + q]];
                belems[3 * e + 2] = m->perm[bv[2 * T.nbelem + q]];
            }
        }
        return FVM_OK;
    });
}

int fvm_problem_create(fvm_mesh* mesh, const fvm_problem_desc* desc, fvm_problem** out) {
    return guard([&] { return fvm_problem_create_impl(mesh, desc, out); });
}

int fvm_problem_destroy(fvm_problem* p) {
    return guard([&] {
        delete p;
        return FVM_OK;
    });
}

int fvm_problem_info(const fvm_problem* p, int64_t* info) {
    return guard([&] {
        if (!p || !info) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        info[0] = p->linear ? 1 : 0;
        info[1] = p->op_nonzeros;
        info[2] = p->mesh->pat.nslots;
        info[3] = p->has_b ? 1 : 0;
        info[4] = p->has_q ? 1 : 0;
        info[5] = p->precision;
        return FVM_OK;
    });
}

int fvm_problem_export_codes(const fvm_problem* p, int8_t* code, int8_t* bneu) {
    return guard([&] {
        if (!p) fail(FVM_ERR_INVALID_ARGUMENT, "NULL problem");
        const fvm_mesh* m = p->mesh;
        if (code) {
            std::vector<int8_t> ci(m->np);
            FVM_CUDA(cudaMemcpy(ci.data(), p->d_code.p, m->np, cudaMemcpyDeviceToHost));
            for (int64_t v = 0; v < m->np; ++v) code[m->perm[v]] = ci[v];
        }
        if (bneu) {
            // the device copy lives with the triangle-path boundary elements
            const_cast<fvm_problem*>(p)->build_triangle_path();
            const Tiles& T = m->tiles;
            const int nrow = 1 + 2 * (p->dif_deg + 1) + 6;
            std::vector<double> bc((size_t)nrow * T.nbelem);
            if (T.nbelem) FVM_CUDA(cudaMemcpy(bc.data(), p->d_bc.p, bc.size() * 8, cudaMemcpyDeviceToHost));
            std::fill(bneu, bneu + m->nbe, (int8_t)-1);
            for (int64_t q = 0; q < T.nbelem; ++q) bneu[T.ebedge[q]] = bc[q] != 0.0 ? 1 : 0;
        }
        return FVM_OK;
    });
}

int fvm_rhs(fvm_problem* p, const double* u, double* du, double t, int32_t flags, void* stream) {
    return guard([&] {
        if (!p || !u || !du) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        cudaStream_t s = (cudaStream_t)stream;
        int32_t loc = flags & 3;
        if (loc > FVM_PTR_DEVICE_INTERNAL) fail(FVM_ERR_INVALID_ARGUMENT, "bad pointer-location flag");
        if (loc == FVM_PTR_HOST && !(flags & (FVM_RHS_FORCE_TRIANGLE | FVM_RHS_CONSERVATIVE))) {
            // page-locked host arrays: one launch overlaps the link transfers with the product
            const void* mu = host_mapped(u);
            void* md = mu ? host_mapped(du) : nullptr;
            if (md && problem_rhs_host_fused(p, (const double*)mu, (double*)md, t, s)) {
                FVM_CUDA(cudaStreamSynchronize(s));
                check_device_error();
                return FVM_OK;
            }
        }
        IoPlan io;
        rhs_inputs(p, u, du, loc, io, s);
        problem_rhs_internal(p, io.uin, io.dout, (flags & FVM_RHS_FORCE_TRIANGLE) != 0, s,
                             (flags & FVM_RHS_CONSERVATIVE) != 0, t);
        check_launch();
        rhs_outputs(p, du, loc, s);
        return FVM_OK;
    });
}

int fvm_dirichlet_apply(fvm_problem* p, double* u, double t, int32_t flags, void* stream) {
    return guard([&] {
        if (!p || !u) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        cudaStream_t s = (cudaStream_t)stream;
        fvm_mesh* m = p->mesh;
        int32_t loc = flags & 3;
        if (loc == FVM_PTR_DEVICE_INTERNAL) {
            problem_dirichlet_internal(p, u, t, s);
        } else {
            p->ensure_work();
            if (loc == FVM_PTR_HOST)
                FVM_CUDA(cudaMemcpyAsync(p->d_ref.p, u, sizeof(double) * m->np, cudaMemcpyHostToDevice, s));
            const double* src = loc == FVM_PTR_HOST ? p->d_ref.as<double>() : u;
            launch_permute_in(m->d_perm.as<int32_t>(), src, p->d_u.as<double>(), m->np, s);
            problem_dirichlet_internal(p, p->d_u.as<double>(), t, s);
            double* dst = loc == FVM_PTR_HOST ? p->d_ref.as<double>() : u;
            launch_permute_out(m->d_perm.as<int32_t>(), p->d_u.as<double>(), dst, m->np, s);
            if (loc == FVM_PTR_HOST) {
                FVM_CUDA(cudaMemcpyAsync(u, p->d_ref.p, sizeof(double) * m->np, cudaMemcpyDeviceToHost, s));
                FVM_CUDA(cudaStreamSynchronize(s));
            }
        }
        check_launch();
        return FVM_OK;
    });
}

int fvm_tsit5_solve(fvm_problem* p, const double* u0, const fvm_ode_options* opt, double* out, fvm_ode_stats* stats,
                    void* stream) {
    return guard([&] {
        if (!p || !u0 || !opt || !out) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        if (p->conditions_only) fail(FVM_ERR_INVALID_ARGUMENT, "this problem carries a template's conditions only");
        cudaStream_t s = (cudaStream_t)stream;
        fvm_mesh* m = p->mesh;
        const int64_t n = m->np;
        int64_t nsave = (opt->saveat && opt->nsave > 0) ? opt->nsave : 1;
        DBuf d_in, d_out;
        d_in.alloc(sizeof(double) * n * 2);
        d_out.alloc(sizeof(double) * n * nsave);
        double* d_ref = d_in.as<double>();
        double* d_u0 = d_ref + n;
        FVM_CUDA(cudaMemcpyAsync(d_ref, u0, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        launch_permute_in(m->d_perm.as<int32_t>(), d_ref, d_u0, n, s);
        OdeRhs rhs;
        rhs.f = [p](const double* u, double* du, double t, cudaStream_t st) {
            problem_rhs_internal(p, u, du, false, st, false, t);
        };
        if (p->ndir > 0)
            rhs.callback = [p](double* u, double t, cudaStream_t st) { problem_dirichlet_internal(p, u, t, st); };
        rhs.time_dependent = p->ntime > 0;
        rhs.callback_varies = p->tdir_varies;
        if (p->linear && p->precision != FVM_FP32 && p->ntime == 0) {  // problem_rhs_internal's explicit FP64 path
            rhs.sell.pat = &m->pat;
            rhs.sell.val = p->d_val64.as<double>();
            rhs.sell.b = p->has_b ? p->d_b.as<double>() : nullptr;
            rhs.sell.q = p->has_q ? p->d_q.as<double>() : nullptr;
            rhs.sell.dir_idx = p->d_dir_idx.as<int32_t>();
            rhs.sell.dir_val = p->d_dir_val.as<double>();
            rhs.sell.ndir = p->ndir;
        }
        tsit5_run(rhs, n, d_u0, *opt, d_out.as<double>(), stats, s);
        snapshots_to_host(m->d_iperm.as<int32_t>(), d_out.as<double>(), out, n, nsave, s);
        FVM_CUDA(cudaStreamSynchronize(s));
        check_launch();
        check_device_error();
        return FVM_OK;
    });
}

}  // extern "C"

// exported for the template / steady-solve translation unit
namespace fvm {
void snapshots_to_host(const int32_t* iperm, const double* src, double* out, int64_t n, int64_t nsave,
                       cudaStream_t s) {
    if (n == 0 || nsave == 0) return;
    if (double* mapped = static_cast<double*>(host_mapped(out))) {
        launch_permute_out_snapshots(iperm, src, mapped, n, nsave, s);
        return;
    }
    const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(nsave, (int64_t(64) << 20) / (8 * n)));
    DBuf tmp;
    tmp.alloc(sizeof(double) * n * chunk);
    for (int64_t k0 = 0; k0 < nsave; k0 += chunk) {
        const int64_t kc = std::min(chunk, nsave - k0);
        launch_permute_out_snapshots(iperm, src + k0 * n, tmp.as<double>(), n, kc, s);
        FVM_CUDA(cudaMemcpyAsync(out + k0 * n, tmp.p, sizeof(double) * n * kc, cudaMemcpyDeviceToHost, s));
    }
}

void tsit5_run_internal(OdeRhs& rhs, int64_t n, const double* u0_int, const fvm_ode_options& o, double* out_int,
                        fvm_ode_stats* st, cudaStream_t s) {
    tsit5_run(rhs, n, u0_int, o, out_int, st, s);
}
int guard_call(const std::function<int()>& f) { return guard(f); }
}  // namespace fvm
