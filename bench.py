"""Benchmark of the vertex-centred FVM hot path on GB300.

Headline workload (one "step" = one fvm_eqs! evaluation): the FVMProblem form of the
DiffusionEquation configuration - triangulate_rectangle(0, 1, 0, 1, 1000, 1000) (1M
vertices, 1,996,002 triangles), D(x, y) = 1 + 0.5 sin(2 pi x) sin(2 pi y), zero Dirichlet on
the four sides, u0 = exp(-50((x - 0.5)^2 + (y - 0.5)^2)).  Metric: vertex-flux evaluations per
second (3 per triangle + 2 per boundary edge, per RHS).  L2 is flushed (256 MiB read)
between timed steps; every step is timed with CUDA events on the launching stream.

`--impl reference` times the reference's CPU algorithm (the C restatement of
parallel_fvm_eqs!, the reference being Julia-only) on the host cores for the same workload.
Under torchrun every rank runs an independent replica on its own GPU ("replicas only").
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for _p in (ROOT / "finitevolumemethod.jl_gb300", ROOT / "oracle"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

WORKLOAD = ("fvm_eqs! of FVMProblem(diffusion) on triangulate_rectangle(0,1,0,1,1000,1000), "
            "D=1+0.5sin(2pi x)sin(2pi y), zero Dirichlet, u0 Gaussian bump")
METRIC = "vertex-flux evals/s"
UNIT = "flux-evals/s"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# --------------------------------------------------------------------------------------
# workloads
# --------------------------------------------------------------------------------------
def sine_D(x, y, t, u, p):
    return 1.0 + 0.5 * np.sin(2 * np.pi * x) * np.sin(2 * np.pi * y) + 0.0 * u


def zero_bc(x, y, t, u, p):
    return 0.0 * x


def c2_triangulation(n=1000):
    from fvmgpu.meshes import triangulate_rectangle

    return triangulate_rectangle(0.0, 1.0, 0.0, 1.0, n, n)


def c2_u0(tri):
    P = tri.points
    return np.exp(-50 * ((P[:, 0] - 0.5) ** 2 + (P[:, 1] - 0.5) ** 2))


def c2_problem(mesh, precision="fp64"):
    import fvmgpu as F

    tri = mesh.triangulation
    BCs = F.BoundaryConditions(mesh, (zero_bc,) * 4, (F.Dirichlet,) * 4)
    return F.FVMProblem(mesh, BCs, diffusion_function=sine_D, initial_condition=c2_u0(tri), final_time=1000 * 1e-7,
                        precision=precision)


def flux_evals(tri):
    return 3 * tri.num_triangles + 2 * tri.num_boundary_edges


# --------------------------------------------------------------------------------------
# measurement helpers
# --------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed regions run."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "50"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()
        return False

    def summary(self):
        rows = []
        for line in (self.out or "").splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                rows.append((float(parts[0]), float(parts[1]), parts[4:8]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for _, _, r in rows for k in range(4) if r[k].lower().startswith("active")})
        return {"sm_mhz": float(np.median([r[0] for r in rows])), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(name):
    """dram bytes per launch recorded by the committed ncu summary of `name`, or None."""
    p = ROOT / "profiles" / f"{name}.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.strip().startswith("dram_bytes_per_launch:"):
            try:
                return int(float(line.split(":", 1)[1].strip().split()[0]))
            except ValueError:
                return None
    return None


def timed_steps(fn, K, W, flush, torch):
    """W untimed warm-up calls, then K calls each bracketed by CUDA events (L2 flushed
    before each).  Returns per-step milliseconds."""
    for _ in range(W):
        fn()
    torch.cuda.synchronize()
    ev = []
    for _ in range(K):
        flush()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        ev.append((a, b))
    torch.cuda.synchronize()
    return np.array([a.elapsed_time(b) for a, b in ev])


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return None, 0, 1, 0
    import torch.distributed as dist

    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    dist.init_process_group("gloo")
    return dist, rank, ws, local


def aggregate(dist, units, seconds):
    """Whole-job throughput: units summed over ranks / slowest rank's time."""
    if dist is None:
        return units / seconds, seconds
    import torch

    t = torch.tensor([units, seconds], dtype=torch.float64)
    u = t[0:1].clone()
    s = t[1:2].clone()
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(s, op=dist.ReduceOp.MAX)
    return float(u[0]) / float(s[0]), float(s[0])


# --------------------------------------------------------------------------------------
# CPU baseline (oracle C restatement of parallel_fvm_eqs!)
# --------------------------------------------------------------------------------------
def cpu_baseline(tri, max_seconds=10.0, max_evals=200, nthreads=0):
    import build_oracle as B
    import fvm_oracle as O

    conds = O.Conditions(tri, [lambda x, y, t, u: 0.0 * x] * tri.num_ghost_vertices,
                         ["Dirichlet"] * tri.num_ghost_vertices)
    prob = O.Problem(tri, conds, D=lambda x, y, t, u: sine_D(x, y, t, u, None), u0=c2_u0(tri))
    cp = B.CProblem(prob.geo, tri, prob.code, B.D_SINE, (0.5,), prob.bnd_tri)
    nth = nthreads or B.max_threads()
    u = c2_u0(tri)
    du = np.empty_like(u)
    cp.rhs_threaded(u, 0.0, nth, du)  # warm-up
    t0 = time.perf_counter()
    k = 0
    while k < max_evals and time.perf_counter() - t0 < max_seconds:
        cp.rhs_threaded(u, 0.0, nth, du)
        k += 1
    dt = time.perf_counter() - t0
    return {"value": flux_evals(tri) * k / dt, "unit": UNIT, "cores": nth, "kind": "port",
            "sample": f"{k} threaded fvm_eqs! evaluations of the full 1000x1000 workload ({dt:.2f} s)",
            "ms_per_eval": 1e3 * dt / k}


def run_reference(args):
    dist, rank, ws, local = dist_setup()
    if rank != 0:
        return
    import build_oracle as B

    tri = c2_triangulation()
    import fvm_oracle as O

    conds = O.Conditions(tri, [lambda x, y, t, u: 0.0 * x] * 4, ["Dirichlet"] * 4)
    prob = O.Problem(tri, conds, D=lambda x, y, t, u: sine_D(x, y, t, u, None), u0=c2_u0(tri))
    cp = B.CProblem(prob.geo, tri, prob.code, B.D_SINE, (0.5,), prob.bnd_tri)
    nth = B.max_threads()
    u = c2_u0(tri)
    du = np.empty_like(u)
    for _ in range(args.warmup):
        cp.rhs_threaded(u, 0.0, nth, du)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cp.rhs_threaded(u, 0.0, nth, du)
    dt = time.perf_counter() - t0
    value = flux_evals(tri) * args.steps / dt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "nv": tri.num_points, "nt": tri.num_triangles,
                       "nbe": tri.num_boundary_edges, "flux_evals_per_step": flux_evals(tri)},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nth, "kind": "port",
                             "sample": f"{args.steps} threaded fvm_eqs! evaluations (C restatement of "
                                       "parallel_fvm_eqs!; the Julia reference is not installable here)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------------------
def run_gpu(args):
    import torch

    dist, rank, ws, local = dist_setup()
    torch.cuda.set_device(local)
    import fvmgpu as F
    from fvmgpu import _lib

    F.build()
    _lib.require_gpu()
    t_setup = time.perf_counter()
    tri = c2_triangulation()
    mesh = F.FVMGeometry(tri)
    prob = c2_problem(mesh)
    info = prob.info()
    n = tri.num_points
    units = flux_evals(tri)
    log(f"[bench] setup {time.perf_counter() - t_setup:.1f} s; operator nonzeros {info['operator_nonzeros']}, "
        f"slots {info['operator_slots']}")
    # L2 flush by a 256 MiB read: it evicts every line of the workload and, unlike a write,
    # leaves no dirty lines whose write-back the next timed kernel would pay for
    flush_src = torch.ones(64 << 20, dtype=torch.float32, device="cuda")
    flush = flush_src.sum  # noqa: E731
    perm = torch.as_tensor(mesh.permutation().astype(np.int64), device="cuda")
    u_ref = torch.as_tensor(c2_u0(tri), device="cuda")
    u_int = u_ref[perm].contiguous()
    du_int = torch.empty_like(u_int)
    K, W = args.steps, args.warmup
    step = lambda: F.fvm_eqs(du_int, u_int, prob, 0.0, internal=True)  # noqa: E731
    # e2e through the public API with pinned host buffers (H2D + kernels + D2H every step)
    u_h = torch.empty(n, dtype=torch.float64, pin_memory=True)
    du_h = torch.empty(n, dtype=torch.float64, pin_memory=True)
    u_h.copy_(torch.as_tensor(c2_u0(tri)))
    u_hn, du_hn = u_h.numpy(), du_h.numpy()
    e2e_step = lambda: F.fvm_eqs(du_hn, u_hn, prob, 0.0)  # noqa: E731
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(torch.cuda.current_device() if "CUDA_VISIBLE_DEVICES" in os.environ else local) as clk:
        ms = timed_steps(step, K, max(W, 3), flush, torch)
        torch.cuda.synchronize()
        ms_e2e = timed_steps(e2e_step, K, max(W, 3), flush, torch)
        torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    value, tmax = aggregate(dist, units * K, ms.sum() / 1e3)
    e2e_value, _ = aggregate(dist, units * K, ms_e2e.sum() / 1e3)
    peak, peak_kind = measured_peaks()
    alg_bytes = 12 * info["operator_nonzeros"] + 16 * n
    achieved = alg_bytes / (ms.mean() / 1e3) / 1e9
    traffic = profile_traffic("rhs_sell_stream_fp64_1000x1000")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": max(W, 3),
        "ms_per_step": float(ms.mean()), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "nv": n, "nt": tri.num_triangles, "nbe": tri.num_boundary_edges,
                   "flux_evals_per_step": units, "l2": "flushed between timed steps (256 MiB read)",
                   "layout": "device-resident u/du in the library's Hilbert numbering",
                   "parallelism": f"replicas x{ws}"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "kernel": "sell_stream_kernel<double,double,double,explicit,8,8>",
                     "alg_bytes_per_launch": alg_bytes, "peak_source": f"{peak_kind} hbm_gbs (burst copy)"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n,
                "ms_per_step": float(ms_e2e.mean()), "path": "fvm_rhs C ABI, pinned host buffers"},
        "clocks": clk.summary(),
        "gpu_launches": int(K + 3 * K),
    }
    extra = {}
    if rank == 0 and ws == 1 and not args.no_extras:
        extra = run_extras(args, F, torch, tri, mesh, prob, flush, perm, u_int, peak)
    if rank == 0:
        if ws == 1 and not args.no_cpu_baseline:
            try:
                line["cpu_baseline"] = cpu_baseline(tri)
            except Exception as e:  # noqa: BLE001
                line["cpu_baseline"] = {"value": None, "error": repr(e)}
        if extra:
            line["extra"] = extra
        print(json.dumps(line), flush=True)


def run_extras(args, F, torch, tri, mesh, prob, flush, perm, u_int, peak):
    """Secondary rows: FP32 assembly, per-triangle kernel, Tsit5, template SpMV, steady solve."""
    out = {}
    K = max(20, min(args.steps, 200))
    units = flux_evals(tri)
    n = tri.num_points
    du = torch.empty_like(u_int)
    try:
        p32 = c2_problem(mesh, precision="fp32")
        i32 = p32.info()
        ms = timed_steps(lambda: F.fvm_eqs(du, u_int, p32, 0.0, internal=True), K, 5, flush, torch)
        # to_f32 pass (read u 8 B, write u32 4 B) + operator 8 B / entry + u32 4 B + rowscale 8 B + du 8 B
        b32 = 8 * i32["operator_nonzeros"] + 32 * n
        out["rhs_fp32"] = {"value": units / (ms.mean() / 1e3), "unit": UNIT, "ms": float(ms.mean()),
                           "achieved_gbs": b32 / (ms.mean() / 1e3) / 1e9, "alg_bytes": b32}
        del p32
    except Exception as e:  # noqa: BLE001
        out["rhs_fp32"] = {"error": repr(e)}
    try:
        ms = timed_steps(lambda: F.fvm_eqs(du, u_int, prob, 0.0, internal=True, conservative=True), K, 5, flush,
                         torch)
        bc = 12 * (info_c := prob.info())["operator_nonzeros"] - 12 * n + 16 * n
        out["rhs_fp64_conservative"] = {"value": units / (ms.mean() / 1e3), "unit": UNIT, "ms": float(ms.mean()),
                                        "achieved_gbs": bc / (ms.mean() / 1e3) / 1e9, "alg_bytes": bc}
    except Exception as e:  # noqa: BLE001
        out["rhs_fp64_conservative"] = {"error": repr(e)}
    try:
        ms = timed_steps(lambda: F.fvm_eqs(du, u_int, prob, 0.0, internal=True, force_triangle=True), K, 5, flush,
                         torch)
        info = mesh.info()
        tb = 4 * 3 * info["ntile_elements"] + 8 * 6 * info["ntile_elements"] + 25 * n
        out["rhs_triangle_fp64"] = {"value": units / (ms.mean() / 1e3), "unit": UNIT, "ms": float(ms.mean()),
                                    "achieved_gbs": tb / (ms.mean() / 1e3) / 1e9, "alg_bytes": tb,
                                    "tile_elements": info["ntile_elements"]}
    except Exception as e:  # noqa: BLE001
        out["rhs_triangle_fp64"] = {"error": repr(e)}
    try:
        torch.cuda.synchronize()
        sol = F.solve(prob, F.Tsit5(), dt=1e-7, adaptive=False, saveat=[prob.final_time])
        st = sol.stats
        out["tsit5_1000_steps"] = {"elapsed_ms": st["elapsed_ms"], "steps": st["naccept"], "rhs_evals": st["nrhs"],
                                   "ms_per_step": st["elapsed_ms"] / max(1, st["naccept"]),
                                   "flux_evals_per_s": units * st["nrhs"] / (st["elapsed_ms"] / 1e3)}
    except Exception as e:  # noqa: BLE001
        out["tsit5_1000_steps"] = {"error": repr(e)}
    try:
        BCs = F.BoundaryConditions(mesh, (zero_bc,) * 4, (F.Dirichlet,) * 4)
        tmpl = F.DiffusionEquation(mesh, BCs, diffusion_function=lambda x, y, p: sine_D(x, y, 0, 0, p),
                                   initial_condition=c2_u0(tri), final_time=1e-4)
        A = tmpl.A
        for prec in ("fp64", "fp32"):
            ms = timed_steps(lambda: tmpl.apply(du, u_int, precision=prec, internal=True), K, 5, flush, torch)
            vb = 12 if prec == "fp64" else 8
            bb = vb * A.nnz + 4 * (n + 1) + 24 * n
            out[f"template_spmv_{prec}"] = {"ms": float(ms.mean()), "nnz": int(A.nnz),
                                            "achieved_gbs": bb / (ms.mean() / 1e3) / 1e9, "alg_bytes": bb}
        del tmpl
    except Exception as e:  # noqa: BLE001
        out["template_spmv"] = {"error": repr(e)}
    if not args.no_steady:
        out["steady"] = run_steady(args, F)
    return out


def run_steady(args, F):
    """Steady Poisson on the unit disk: Delaunay of N uniform random points (seed 0) plus 4096
    boundary points; D = 1 (r < 0.5), 10 otherwise; f = -1; zero Dirichlet; FP64 Krylov vs mixed
    precision (FP32 inner, FP64 reliable updates), both to ||b - A x|| / ||b|| <= 1e-10."""
    res = {}
    try:
        t0 = time.perf_counter()
        tri = F.triangulate_disk(args.steady_points, 4096, seed=0)
        mesh = F.FVMGeometry(tri)
        BCs = F.BoundaryConditions(mesh, zero_bc, F.Dirichlet)
        D = lambda x, y, p: np.where(x * x + y * y < 0.25, 1.0, 10.0)  # noqa: E731
        pois = F.PoissonsEquation(mesh, BCs, diffusion_function=D, source_function=lambda x, y, p: -1.0 + 0.0 * x)
        res["setup_s"] = time.perf_counter() - t0
        res["nv"] = tri.num_points
        res["nt"] = tri.num_triangles
        for mode in ("fp64", "mixed"):
            sol = F.solve(pois, F.KrylovSolver(mode=mode, rtol=1e-10))
            res[mode] = {k: sol.stats[k] for k in ("elapsed_ms", "iterations", "refinements", "rel_residual", "method",
                                                   "symmetric")}
        res["speedup_mixed_vs_fp64"] = res["fp64"]["elapsed_ms"] / res["mixed"]["elapsed_ms"]
    except Exception as e:  # noqa: BLE001
        res["error"] = repr(e)
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--no-steady", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--steady-points", type=int, default=2_000_000)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
