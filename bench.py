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


def read_stream_reference(torch, flush, nbytes, K):
    """What a plain read of the RHS's compulsory bytes costs on this GPU in one launch of the
    same size: the sum of an FP32 tensor of `nbytes` (a vectorised, fully occupied streaming
    reduction), timed like the RHS, L2 flushed before each launch.  The copy benchmark behind
    the roofline peak streams far more data per launch; this says how close the RHS kernel
    is to the read rate a launch of its size reaches."""
    t = torch.ones(nbytes // 4, dtype=torch.float32, device="cuda")
    ms = timed_steps(lambda: t.sum(), max(K, 20), 5, flush, torch)
    us = float(ms.mean()) * 1e3
    return {"bytes": int(t.numel() * 4), "us": us, "gbs": t.numel() * 4 / (us * 1e-6) / 1e9}


def canonical_roofline(tri, ms, peak):
    """The RHS against the canonical bytes of the reference's per-triangle layout
    (132 nt + 25 nv + 48 nbe: triangle connectivity, shape coefficients, normals times lengths,
    per-edge D; vertex u, du, 1/V, code; boundary-edge data), the figure the 70 % target is
    quoted on.  This layout never reads most of those arrays, so the ratio can exceed 1."""
    b = 132 * tri.num_triangles + 25 * tri.num_points + 48 * tri.num_boundary_edges
    t_peak_us = b / (peak * 1e9) * 1e6
    return {"bytes": b, "equivalent_gbs": b / (ms / 1e3) / 1e9, "equivalent_frac": b / (ms / 1e3) / 1e9 / peak,
            "time_at_peak_us": t_peak_us, "target_70pct_us": t_peak_us / 0.7, "measured_us": 1e3 * ms}


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


def timed_steps(fn, K, W, flush, torch, device_only=True):
    """W untimed warm-up calls, then K calls each bracketed by CUDA events (L2 flushed
    before each).  device_only: a device sleep of about half a millisecond after the flush
    keeps the GPU busy while the host enqueues the start event and the call, so the events
    bracket the device work and not the host's launch overhead, however slow the host is at
    that moment (end-to-end timings pass False and keep that overhead).  Returns per-step
    milliseconds."""
    for _ in range(W):
        fn()
    torch.cuda.synchronize()
    ev = []
    for _ in range(K):
        flush()
        if device_only:
            torch.cuda._sleep(1_000_000)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        ev.append((a, b))
    torch.cuda.synchronize()
    return np.array([a.elapsed_time(b) for a, b in ev])


_PROFILER_WARM = False


def count_launches(fn, torch):
    """Kernels launched by one call of `fn`, counted by the CUDA activity profiler (every
    kernel the process launches on the device, the library's included), or None if the
    profiler is unavailable.  Copies and memsets are not kernels and are not counted."""
    try:
        from torch.profiler import ProfilerActivity, profile

        torch.cuda.synchronize()
        global _PROFILER_WARM
        if not _PROFILER_WARM:  # the first session of a process can miss the device activity
            with profile(activities=[ProfilerActivity.CUDA]):
                fn()
                torch.cuda.synchronize()
            _PROFILER_WARM = True
        with profile(activities=[ProfilerActivity.CUDA]) as prof:
            fn()
            torch.cuda.synchronize()
        names = [e.name for e in prof.events() if e.device_type == torch.autograd.DeviceType.CUDA]
        names = [nm for nm in names if not nm.lower().startswith(("memcpy", "memset"))]
        return len(names), sorted(set(names))
    except Exception:  # noqa: BLE001
        return None, []


def _round(x, sig=4):
    if isinstance(x, float):
        return float(f"{x:.{sig}g}") if np.isfinite(x) else None
    if isinstance(x, dict):
        return {k: _round(v, sig) for k, v in x.items()}
    if isinstance(x, (list, tuple)):
        return [_round(v, sig) for v in x]
    return x


def emit_row(name, d):
    """One compact JSON line per secondary row, printed before the headline line."""
    print(json.dumps({"row": name, **_round(d)}, separators=(",", ":")), flush=True)


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


def _saveat_list(t0, tf, step):
    """t0, t0 + step, ..., tf (the saves of `saveat = step`)."""
    n = int(np.floor((tf - t0) / step + 1e-9))
    ts = [t0 + step * k for k in range(n + 1)]
    if ts[-1] < tf - 1e-12 * max(1.0, abs(tf)):
        ts.append(tf)
    return ts


def cpu_trbdf2_baseline(tri, u0, dconst, tf, saveat):
    """CPU baseline of an FVMProblem's TRBDF2 solve (zero Dirichlet, constant diffusivity): the
    oracle's TR-BDF2 (the same step control as the device) with exact sparse LU solves of
    W = I - d h J (scipy's SuperLU, the role KLU plays in the reference's tutorials) and the C
    restatement of fvm_eqs!, one host thread.  The Jacobian is formed once by coloured
    differences (the problem is affine), inside the timed region."""
    import build_oracle as B
    import fvm_oracle as O

    conds = O.Conditions(tri, [lambda x, y, t, u: 0.0 * x] * tri.num_ghost_vertices,
                         ["Dirichlet"] * tri.num_ghost_vertices)
    prob = O.Problem(tri, conds, D=lambda x, y, t, u: dconst + 0.0 * x, u0=u0, t0=0.0, tf=tf)
    cp = B.CProblem(prob.geo, tri, prob.code, B.D_CONST, (dconst,), prob.bnd_tri)
    f = lambda u, t: cp.rhs_serial(np.ascontiguousarray(u), t)  # noqa: E731
    cb = lambda u, t: O.update_dirichlet_nodes(prob, u, t)  # noqa: E731
    ent, n = O.jacobian_sparsity(tri)
    wall = float("inf")
    for _ in range(2):  # best of two: the first also loads the C library
        t0 = time.perf_counter()
        J = O.colored_jacobian(f, u0, 0.0, ent, n, affine=True)
        sol, st = O.trbdf2_solve(f, lambda u, t: J, u0, 0.0, tf, saveat, callback=cb, affine=True)
        wall = min(wall, time.perf_counter() - t0)
    return {"wall_ms": 1e3 * wall, "steps": st["naccept"], "rejected": st["nreject"], "kind": "port", "cores": 1,
            "sample": "the whole solve, best of two: oracle TR-BDF2 with SuperLU factorisations, C fvm_eqs!"}


def bench_config(tri, ws=1):
    """The `config` object both arms print (identical keys and values)."""
    return {"workload": WORKLOAD, "nv": tri.num_points, "nt": tri.num_triangles, "nbe": tri.num_boundary_edges,
            "flux_evals_per_step": flux_evals(tri),
            "l2": "GPU arm: L2 flushed between timed steps (256 MiB read); CPU arm: the 1M-vertex arrays exceed the "
                  "host caches",
            "parallelism": f"replicas x{ws}"}


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
            "config": bench_config(tri, args.gpus),
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
    t_mesh = time.perf_counter()
    mesh = F.FVMGeometry(tri)
    t_prob = time.perf_counter()
    prob = c2_problem(mesh)
    info = prob.info()
    setup = {"triangulate_rectangle_s": t_mesh - t_setup, "fvm_geometry_s": t_prob - t_mesh,
             "fvm_problem_s": time.perf_counter() - t_prob}
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
        ms_e2e = timed_steps(e2e_step, K, max(W, 3), flush, torch, device_only=False)
        torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    value, tmax = aggregate(dist, units * K, ms.sum() / 1e3)
    e2e_value, _ = aggregate(dist, units * K, ms_e2e.sum() / 1e3)
    peak, peak_kind = measured_peaks()
    alg_bytes = 12 * info["operator_nonzeros"] + 16 * n
    achieved = alg_bytes / (ms.mean() / 1e3) / 1e9
    stream = read_stream_reference(torch, flush, alg_bytes, K)
    traffic = profile_traffic("rhs_sell_stream_fp64_1000x1000")
    per_step, kernels = count_launches(step, torch)
    per_e2e, _ = count_launches(e2e_step, torch)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": max(W, 3),
        "ms_per_step": float(ms.mean()), "ms_per_step_median": float(np.median(ms)),
        "vertex_rhs_per_s": n * ws / tmax * K if tmax else None,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": bench_config(tri, ws),
        "layout": "device-resident u/du in the library's Hilbert numbering",
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "kernel": kernels[0] if len(kernels) == 1 else kernels,
                     "alg_bytes_per_launch": alg_bytes, "alg_bytes_per_flux_eval": alg_bytes / units,
                     "peak_source": f"{peak_kind} hbm_gbs (burst copy)",
                     "canonical": _round(canonical_roofline(tri, ms.mean(), peak)),
                     "read_stream": _round(stream)},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n,
                "ms_per_step": float(ms_e2e.mean()), "path": "fvm_rhs C ABI, pinned host buffers"},
        "clocks": clk.summary(),
        "setup": _round(setup),
    }
    if per_step is not None and per_e2e is not None:
        # value's K steps plus e2e's K steps, each counted by the activity profiler
        line["gpu_launches"] = int(K * (per_step + per_e2e))
        line["gpu_launches_per_step"] = {"device_resident": per_step, "e2e": per_e2e}
    if rank == 0 and ws == 1 and not args.no_extras:
        run_selected(args, F, torch, tri, mesh, prob, flush, u_int, peak)
    if rank == 0:
        if ws == 1 and not args.no_cpu_baseline:
            try:
                line["cpu_baseline"] = _round(cpu_baseline(tri))
            except Exception as e:  # noqa: BLE001
                line["cpu_baseline"] = {"value": None, "error": repr(e)}
        print(json.dumps(line), flush=True)


EXTRA_ROWS = ("rhs_fp32", "rhs_fp64_conservative", "rhs_triangle_fp64", "tsit5_1000_steps", "template_spmv",
              "c1_readme", "batched_c4", "multimesh_c4", "adjoint_c5", "system_gray_scott", "steady", "implicit")


def _kernel_row(F, torch, fn, K, flush, units, alg_bytes, peak, profile=None):
    ms = timed_steps(fn, K, 5, flush, torch)
    us = float(ms.mean()) * 1e3
    gbs = alg_bytes / (us * 1e-6) / 1e9
    nlaunch, kernels = count_launches(fn, torch)
    row = {"us": us, "flux_evals_per_s": units / (us * 1e-6), "alg_bytes": alg_bytes, "gbs": gbs,
           "frac": gbs / peak, "launches": nlaunch, "kernels": [k.split("(")[0][:60] for k in kernels]}
    if profile:
        row["traffic"] = profile_traffic(profile)
    return row


def run_selected(args, F, torch, tri, mesh, prob, flush, u_int, peak):
    """Secondary rows, each printed as its own compact JSON line: FP32 assembly, difference
    form, per-triangle kernel, Tsit5, template SpMV, C1, the batched, multi-mesh and adjoint
    rows, systems, steady solves.  `--rows` selects a subset."""
    want = set(args.rows.split(",")) if args.rows else set(EXTRA_ROWS)
    if args.no_batch:
        want -= {"batched_c4", "multimesh_c4", "adjoint_c5"}
    if args.no_steady:
        want.discard("steady")
    K = max(20, min(args.steps, 200))
    units = flux_evals(tri)
    n = tri.num_points
    du = torch.empty_like(u_int)
    nnz = prob.info()["operator_nonzeros"]

    def rhs_fp32():
        p32 = c2_problem(mesh, precision="fp32")
        # to_f32 pass (read u 8 B, write u32 4 B) + operator 8 B / entry + u32 4 B + rowscale 8 B + du 8 B
        b32 = 8 * p32.info()["operator_nonzeros"] + 32 * n
        return _kernel_row(F, torch, lambda: F.fvm_eqs(du, u_int, p32, 0.0, internal=True), K, flush, units, b32, peak)

    def rhs_fp64_conservative():
        bc = 12 * nnz - 12 * n + 24 * n
        return _kernel_row(F, torch, lambda: F.fvm_eqs(du, u_int, prob, 0.0, internal=True, conservative=True), K,
                           flush, units, bc, peak)

    def rhs_triangle_fp64():
        info = mesh.info()
        # per tile element: 3 vertex indices (12 B) + 6 coefficients with D(x, y) folded in
        # (48 B); per vertex u, du, 1 / V, code
        tb = 60 * info["ntile_elements"] + 25 * n
        row = _kernel_row(F, torch, lambda: F.fvm_eqs(du, u_int, prob, 0.0, internal=True, force_triangle=True), K,
                          flush, units, tb, peak, profile="rhs_triangle_fp64_1000x1000")
        row["tile_elements"] = info["ntile_elements"]
        return row

    def tsit5_1000_steps():
        torch.cuda.synchronize()
        sol = F.solve(prob, F.Tsit5(), dt=1e-7, adaptive=False, saveat=[prob.final_time])
        st = sol.stats
        us = 1e3 * st["elapsed_ms"] / max(1, st["naccept"])
        # 6 RHS launches per step, stage combinations in separate passes: stage s reads u and
        # s previous derivatives and writes one vector (33 vector passes per step)
        sb = 6 * (12 * nnz + 16 * n) + 33 * 8 * n
        return {"steps": st["naccept"], "rhs_evals": st["nrhs"], "elapsed_ms": st["elapsed_ms"], "us_per_step": us,
                "alg_bytes_per_step": sb, "gbs": sb / (us * 1e-6) / 1e9, "frac": sb / (us * 1e-6) / 1e9 / peak,
                "flux_evals_per_s": units * st["nrhs"] / (st["elapsed_ms"] / 1e3), "driver": st["driver"]}

    def template_spmv():
        BCs = F.BoundaryConditions(mesh, (zero_bc,) * 4, (F.Dirichlet,) * 4)
        tmpl = F.DiffusionEquation(mesh, BCs, diffusion_function=lambda x, y, p: sine_D(x, y, 0, 0, p),
                                   initial_condition=c2_u0(tri), final_time=1e-4)
        A = tmpl.A
        res = {}
        for prec in ("fp64", "fp32"):
            vb = 12 if prec == "fp64" else 8
            bb = vb * A.nnz + 4 * (n + 1) + 24 * n
            r = _kernel_row(F, torch, lambda: tmpl.apply(du, u_int, precision=prec, internal=True), K, flush, units,
                            bb, peak)
            res[prec] = {k: r[k] for k in ("us", "gbs", "frac", "alg_bytes", "launches")}
        return res

    rows = {"c1_readme": lambda: run_c1(F, torch, cpu=not args.no_cpu_baseline), "rhs_fp32": rhs_fp32, "rhs_fp64_conservative": rhs_fp64_conservative,
            "rhs_triangle_fp64": rhs_triangle_fp64, "tsit5_1000_steps": tsit5_1000_steps,
            "template_spmv": template_spmv, "batched_c4": lambda: run_batched(args, F, torch, flush, peak),
            "multimesh_c4": lambda: run_multimesh(args, F, torch), "adjoint_c5": lambda: run_adjoint(args, F, torch),
            "system_gray_scott": lambda: run_system(args, F, torch, flush, mesh),
            "steady": lambda: run_steady(args, F), "implicit": lambda: run_implicit(F, prob)}
    for name in EXTRA_ROWS:
        if name not in want:
            continue
        try:
            out = rows[name]()
        except Exception as e:  # noqa: BLE001
            out = {"error": repr(e)[:300]}
        log(f"[bench] {name}: {json.dumps(out)}")
        if name in ("system_gray_scott", "steady", "batched_c4", "implicit") and "error" not in out:
            for sub, d in out.items():
                emit_row(f"{name}.{sub}", d)
        else:
            emit_row(name, out)


def run_c1(F, torch, reps=5, cpu=True):
    """C1, the README problem (triangulate_rectangle(0, 2, 0, 2, 50, 50, single_boundary=true),
    zero Dirichlet, D = 1/9, u0 = 50 where y <= 1): adaptive Tsit5 to t = 0.5 as the reference's
    documentation times it - the DiffusionEquation template with saveat = 0.05 (published
    5.736 ms, hardware unstated) - and the FVMProblem with saveat = 0.001 (test/README.jl); the
    FVMProblem with TRBDF2 and saveat 0.05 (published 49.237 ms); the docs' 100 x 100 Poisson
    problem as a SteadyFVMProblem with DynamicSS(TRBDF2) (published 189.406 ms) and as the
    PoissonsEquation template (published 15.442 ms).  Wall time of the whole `solve` call, best
    of `reps` after one warm-up."""
    from fvmgpu.meshes import triangulate_rectangle

    tri = triangulate_rectangle(0.0, 2.0, 0.0, 2.0, 50, 50, single_boundary=True)
    mesh = F.FVMGeometry(tri)
    BCs = F.BoundaryConditions(mesh, zero_bc, F.Dirichlet)
    u0 = np.where(tri.points[:, 1] <= 1.0, 50.0, 0.0)
    tmpl = F.DiffusionEquation(mesh, BCs, diffusion_function=lambda x, y, p: 1 / 9 + 0.0 * x, initial_condition=u0,
                               final_time=0.5)
    prob = F.FVMProblem(mesh, BCs, diffusion_function=lambda x, y, t, u, p: 1 / 9 + 0.0 * x, initial_condition=u0,
                        final_time=0.5)
    out = {}
    for name, pr, saveat in (("template_saveat_0.05", tmpl, 0.05), ("fvmproblem_saveat_0.001", prob, 0.001)):
        F.solve(pr, F.Tsit5(), saveat=saveat)
        best, stats = float("inf"), None
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            sol = F.solve(pr, F.Tsit5(), saveat=saveat)
            best = min(best, time.perf_counter() - t0)
            stats = sol.stats
        out[name] = {"wall_ms": 1e3 * best, "device_ms": stats["elapsed_ms"], "steps": stats["naccept"],
                     "rejected": stats["nreject"], "saves": len(sol.u), "driver": stats["driver"]}
    out["template_saveat_0.05"]["published_reference_ms"] = 5.736
    # the same FVMProblem with TRBDF2 (published 49.237 ms with KLU factorisations)
    F.solve(prob, F.TRBDF2(), saveat=0.05)
    best, stats = float("inf"), None
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sol = F.solve(prob, F.TRBDF2(), saveat=0.05)
        best = min(best, time.perf_counter() - t0)
        stats = sol.stats
    out["fvmproblem_trbdf2_saveat_0.05"] = {"wall_ms": 1e3 * best, "device_ms": stats["elapsed_ms"],
                                            "steps": stats["naccept"], "rejected": stats["nreject"],
                                            "published_reference_ms": 49.237}
    if cpu:
        try:
            out["fvmproblem_trbdf2_saveat_0.05"]["cpu_baseline"] = cpu_trbdf2_baseline(
                tri, u0, 1 / 9, 0.5, _saveat_list(0.0, 0.5, 0.05))
        except Exception as e:  # noqa: BLE001
            out["fvmproblem_trbdf2_saveat_0.05"]["cpu_baseline"] = {"error": repr(e)[:200]}
    # docs/src/literate_wyos/poissons_equation.jl: the 100 x 100 Poisson problem as a
    # SteadyFVMProblem solved by DynamicSS(TRBDF2) (published 189.406 ms) and as the template
    # (published 15.442 ms with KLU); both against the exact solution at the docs' rtol 1e-4
    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, 100, 100, single_boundary=True)
    mesh = F.FVMGeometry(tri)
    BCs = F.BoundaryConditions(mesh, zero_bc, F.Dirichlet)
    P = tri.points
    exact = np.sin(np.pi * P[:, 0]) * np.sin(np.pi * P[:, 1]) / (2 * np.pi ** 2)
    rel = lambda u: float(np.linalg.norm(u - exact) / np.linalg.norm(exact))  # noqa: E731
    sprob = F.FVMProblem(mesh, BCs, diffusion_function=lambda x, y, t, u, p: 1.0 + 0.0 * x,
                         source_function=lambda x, y, t, u, p: np.sin(np.pi * x) * np.sin(np.pi * y),
                         initial_condition=np.zeros(tri.num_points), final_time=np.inf)
    steady = F.SteadyFVMProblem(sprob)
    F.solve(steady, F.DynamicSS(F.TRBDF2()))
    best, sol = float("inf"), None
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sol = F.solve(steady, F.DynamicSS(F.TRBDF2()))
        best = min(best, time.perf_counter() - t0)
    out["poisson_100x100_steady_dynamic_ss"] = {"wall_ms": 1e3 * best, "device_ms": sol.stats["elapsed_ms"],
                                                "steps": sol.stats["iterations"], "rel_err_vs_exact": rel(sol.u),
                                                "published_reference_ms": 189.406}
    pois = F.PoissonsEquation(mesh, BCs, source_function=lambda x, y, p: -np.sin(np.pi * x) * np.sin(np.pi * y))
    F.solve(pois)
    best, sol = float("inf"), None
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sol = F.solve(pois)
        best = min(best, time.perf_counter() - t0)
    out["poisson_100x100_template"] = {"wall_ms": 1e3 * best, "iterations": sol.stats["iterations"],
                                       "rel_err_vs_exact": rel(sol.u), "published_reference_ms": 15.442}
    return out


STEADY_FLOOR = {
    # ||b - A fl(x*)|| / ||b|| of the exactly solved disk system rounded to FP64 (x* by sparse LU
    # with two refinement steps, residuals in extended precision; oracle/steady_floor.py): no
    # FP64 vector does much better, so these bound the residual any FP64 solve can reach
    "c3_2M": 4.03e-10, "c3_500k": 7.52e-11}


def run_steady(args, F):
    """Steady Poisson on the unit disk (C3): Delaunay of N uniform random points (seed 0) plus
    4096 boundary points; D = 1 (r < 0.5), 10 otherwise (a non-symmetric operator: BiCGStab);
    f = -1; zero Dirichlet.  Plain FP64 Krylov against mixed precision, each pair with the same
    preconditioner, all stopped on the certified FP64 residual ||b - A x|| / ||b|| of the
    returned FP64 solution.  2M points run at rtol 5e-10, just above the 4.0e-10 that the exact
    solution rounded to FP64 attains; 500k points at 1e-10.  Also: the constant-D disk at 2M
    (symmetric: CG), and a CPU baseline (threaded C BiCGStab with Jacobi, FP64, to
    convergence) at 500k points."""
    res = {}
    cases = (("c3_2M", args.steady_points, "jump", 5e-10), ("c3_2M_constD", args.steady_points, "const", 5e-10),
             ("c3_500k", 500_000, "jump", 1e-10))
    meshes = {}
    for label, npts, dkind, rtol in cases:
        try:
            t0 = time.perf_counter()
            if npts not in meshes:
                meshes = {npts: F.triangulate_disk(npts, 4096, seed=0)}
            t1 = time.perf_counter()
            pois, A, b = c3_poisson(F, meshes[npts], dkind)
            # mesh_gen_s: the disk mesh generator standing in for DelaunayTriangulation;
            # setup_s: FVMGeometry, PoissonsEquation (conditions, sampling, assembly) and the host export
            r = {"nv": int(A.shape[0]), "nnz": int(A.nnz), "rtol": rtol, "mesh_gen_s": t1 - t0,
                 "setup_s": time.perf_counter() - t1}
            if label in STEADY_FLOOR:
                r["fl_xstar_residual"] = STEADY_FLOOR[label]
            modes = [("fp64", "chebyshev", 4), ("mixed", "chebyshev", 4), ("fp64", "chebyshev", 8),
                     ("mixed", "chebyshev", 8)]
            if dkind != "const":
                modes += [("fp64", "jacobi", 0)]
            for mode, precond, deg in modes:
                key = f"{mode}_{precond}{deg or ''}"
                try:
                    sol = F.solve(pois, F.KrylovSolver(mode=mode, rtol=rtol, precond=precond, cheb_degree=deg or 4))
                    conv = True
                except F.NotConvergedError as e:
                    sol, conv = e.solution, False
                st = sol.stats
                r[key] = {"ms": st["elapsed_ms"], "it": st["iterations"], "res": st["rel_residual"], "conv": conv,
                          "method": st["method"], **({"fallback_fp64": True} if st["fallback_fp64"] else {})}
            for deg in (4, 8):
                a_, b_ = r.get(f"fp64_chebyshev{deg}"), r.get(f"mixed_chebyshev{deg}")
                if a_ and b_ and a_["conv"] and b_["conv"]:
                    r[f"speedup_mixed_vs_fp64_chebyshev{deg}"] = a_["ms"] / b_["ms"]
            if label == "c3_500k" and not args.no_cpu_baseline:
                r["cpu_baseline"] = cpu_steady_baseline(A, b, rtol, pois.mesh.cv_volumes)
            res[label] = r
        except Exception as e:  # noqa: BLE001
            res[label] = {"error": repr(e)[:300]}
    return res


def c3_poisson(F, tri, dkind="jump"):
    """PoissonsEquation of C3 on the disk mesh `tri` and its operator (A, b) exported to the host."""
    mesh = F.FVMGeometry(tri)
    BCs = F.BoundaryConditions(mesh, zero_bc, F.Dirichlet)
    if dkind == "jump":
        D = lambda x, y, p: np.where(x * x + y * y < 0.25, 1.0, 10.0)  # noqa: E731
    else:
        D = lambda x, y, p: 1.0 + 0.0 * x  # noqa: E731
    pois = F.PoissonsEquation(mesh, BCs, diffusion_function=D, source_function=lambda x, y, p: -1.0 + 0.0 * x)
    return pois, pois.A, pois.b


def cpu_steady_baseline(A, b, rtol, V):
    """The steady solve on the host cores: threaded C BiCGStab with a Jacobi preconditioner,
    FP64, on every host thread, on the same reduced system as the GPU solver, run to
    ||b - A x|| / ||b|| <= rtol or 60 s (oracle/fvm_oracle_c.c)."""
    import build_oracle as B

    _, st = B.steady_bicgstab(A, b, rtol=rtol, maxit=400_000, max_seconds=60.0, V=V)
    return {"kind": "port", "method": "threaded C BiCGStab + Jacobi, FP64 (stopped at 60 s)", "cores": st["threads"],
            "ms": 1e3 * st["seconds"], "it": st["iterations"], "res": st["rel_residual"], "conv": st["converged"]}


def fourier_logfields(P, seeds, sigma, modes=16):
    """log-D fields sigma * sum_m a_m cos(2 pi k_m . x + phi_m) / sqrt(modes / 2) at the points
    P, one column per seed (a_m ~ N(0, 1), k_m integer in [1, 4]^2, phi_m ~ U[0, 2 pi), drawn in
    that order).  Evaluated through the 16 possible wave vectors: cos(a + phi) = cos a cos phi -
    sin a sin phi makes every field a column of one (npts x 32) x (32 x B) product."""
    ks = np.array([(i, j) for i in range(1, 5) for j in range(1, 5)], dtype=np.float64)
    ang = 2 * np.pi * (P[:, :1] * ks[:, 0] + P[:, 1:2] * ks[:, 1])
    CS = np.hstack([np.cos(ang), np.sin(ang)])
    W = np.zeros((32, len(seeds)))
    for c, seed in enumerate(seeds):
        rng = np.random.default_rng(seed)
        a = rng.standard_normal(modes)
        k = rng.integers(1, 5, size=(modes, 2))
        ph = rng.uniform(0, 2 * np.pi, modes)
        for m in range(modes):
            q = (k[m, 0] - 1) * 4 + (k[m, 1] - 1)
            W[q, c] += a[m] * np.cos(ph[m])
            W[16 + q, c] -= a[m] * np.sin(ph[m])
    return sigma * (CS @ W) / np.sqrt(modes / 2)


def run_batched(args, F, torch, flush, peak):
    """C4: 256 instances of LinearReactionDiffusionEquation (f = -1, zero Dirichlet) on the
    256 x 256 rectangle, log-normal D per instance (sigma = 0.5, 16 Fourier modes, seeds 0..255)
    sampled at every dual-edge midpoint and boundary quarter point; FP32 state, FP64 spot check.
    The per-instance loop is the same problem through the single-instance path (its cost does
    not depend on the D values): B x the time of one instance."""
    from fvmgpu.meshes import triangulate_rectangle

    out = {}
    B, dt, nsteps = 256, 1e-6, 100
    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, 256, 256, single_boundary=True)
    mesh = F.FVMGeometry(tri)
    BCs = F.BoundaryConditions(mesh, zero_bc, F.Dirichlet)
    u0 = c2_u0(tri)
    prob = F.FVMProblem(mesh, BCs, diffusion_function=lambda x, y, t, u, p: 1.0 + 0.0 * x,
                        source_function=lambda x, y, t, u, p: -1.0 * u, initial_condition=u0, final_time=nsteps * dt)
    dual, quarter = mesh.sample_points()
    Ps = np.vstack([dual.reshape(-1, 2), quarter.reshape(-1, 2)])
    Dall = np.ascontiguousarray(np.exp(fourier_logfields(Ps, range(B), 0.5)).T)
    b32 = F.BatchedProblem(prob, Dall, precision="fp32")
    n, units = tri.num_points, flux_evals(tri)
    K = max(20, min(args.steps, 100))
    U = torch.rand((n, B), dtype=torch.float32, device="cuda")
    dU = torch.empty_like(U)
    ms = timed_steps(lambda: b32.rhs(dU, U, internal=True), K, 5, flush, torch)
    nnz = mesh.info()["operator_nnz"]
    # per instance: values 4 B / entry, u gathered and du written 4 + 4 B / vertex; once: CSR
    bytes_ = B * (4 * nnz + 8 * n) + 4 * nnz + 8 * (n + 1)
    rhs = {"ms": float(ms.mean()), "instance_rhs_per_s": B / (ms.mean() / 1e3),
           "flux_evals_per_s": B * units / (ms.mean() / 1e3), "tuning": b32.tuning(), "alg_bytes": bytes_,
           "gbs": bytes_ / (ms.mean() / 1e3) / 1e9, "frac": bytes_ / (ms.mean() / 1e3) / 1e9 / peak}
    p1 = F.FVMProblem(mesh, BCs, diffusion_function=lambda x, y, t, u, p: 1.0 + 0.0 * x,
                      source_function=lambda x, y, t, u, p: -1.0 * u, initial_condition=u0, final_time=nsteps * dt,
                      precision="fp32")
    u1 = torch.rand(n, dtype=torch.float64, device="cuda")
    du1 = torch.empty_like(u1)
    ms1 = timed_steps(lambda: F.fvm_eqs(du1, u1, p1, 0.0, internal=True), K, 5, flush, torch)
    rhs["per_instance_loop_ms"] = float(B * ms1.mean())
    rhs["speedup_vs_per_instance_loop"] = float(B * ms1.mean() / ms.mean())
    out["batched_rhs_fp32"] = rhs
    # Tsit5: 100 fixed steps of the whole batch (graph-captured) vs the per-instance loop
    torch.cuda.synchronize()
    _, uT32, st = b32.solve(u0, dt=dt, saveat=[nsteps * dt])
    sol1 = F.solve(p1, F.Tsit5(), dt=dt, adaptive=False, saveat=[nsteps * dt])
    b64 = F.BatchedProblem(prob, Dall[:8].copy(), precision="fp64")
    _, uT64, _ = b64.solve(u0, dt=dt, saveat=[nsteps * dt])
    err = float(np.max(np.abs(uT32[0, :, :8] - uT64[0])) / np.max(np.abs(uT64[0])))
    out["batched_tsit5_fp32"] = {
        "steps": st["steps"], "elapsed_ms": st["elapsed_ms"],
        "instance_steps_per_s": B * st["steps"] / (st["elapsed_ms"] / 1e3),
        "per_instance_loop_ms": B * sol1.stats["elapsed_ms"],
        "speedup_vs_per_instance_loop": B * sol1.stats["elapsed_ms"] / st["elapsed_ms"],
        "fp32_vs_gpu_fp64_batch_max_rel_err_8_instances": err}
    return out


def gray_scott_system(F, mesh, centre, cross=False):
    """The Gray-Scott tutorial system (docs/src/literate_tutorials/
    gray_scott_model_turing_patterns_from_a_coupled_reaction_diffusion_system.jl): zero Neumann
    on the whole boundary, fluxes -eps_c grad u_c (eps = 2e-5, 1e-5), sources b (1 - u) - u v^2
    and -d v + u v^2 (b = 0.04, d = 0.1), initial bump exp(-80 r^2) about `centre`.  cross=True
    adds constant cross-diffusion (each flux also carries 0.3 eps_c times the other component's
    gradient), which the library stores as one operator shared by the four blocks."""
    bc = lambda x, y, t, uv, p: 0.0 * x  # noqa: E731
    P = mesh.triangulation.points
    r2 = (P[:, 0] - centre[0]) ** 2 + (P[:, 1] - centre[1]) ** 2
    u0, v0 = 1 - np.exp(-80 * r2), np.exp(-80 * r2)
    BCs = F.BoundaryConditions(mesh, (bc,) * mesh.triangulation.num_ghost_vertices,
                               (F.Neumann,) * mesh.triangulation.num_ghost_vertices)
    k = 0.3 if cross else 0.0
    up = F.FVMProblem(mesh, BCs, flux_function=lambda x, y, t, a, b, g, e: (-e * (a[0] + k * a[1]), -e * (b[0] + k * b[1])),
                      flux_parameters=2e-5,
                      source_function=lambda x, y, t, uv, b: b * (1 - uv[0]) - uv[0] * uv[1] ** 2,
                      source_parameters=0.04, initial_condition=u0, final_time=6000.0)
    vp = F.FVMProblem(mesh, BCs, flux_function=lambda x, y, t, a, b, g, e: (-e * (a[1] + k * a[0]), -e * (b[1] + k * b[0])),
                      flux_parameters=1e-5,
                      source_function=lambda x, y, t, uv, d: -d * uv[1] + uv[0] * uv[1] ** 2,
                      source_parameters=0.1, initial_condition=v0, final_time=6000.0)
    return F.FVMSystem(up, vp)


def system_cpu_baseline(n_side=1000, max_seconds=8.0, max_evals=50, nthreads=0):
    """CPU baseline of the system row: the C restatement of the reference's parallel fvm_eqs! on
    the Gray-Scott tutorial FVMSystem (oracle/fvm_oracle_c.c, per-thread duplicated du, all host
    threads) on the n_side x n_side mesh of [-1, 1]^2; a bounded sample of evaluations."""
    import build_oracle as B
    import fvm_oracle as O
    from fvmgpu.meshes import triangulate_rectangle

    tri = triangulate_rectangle(-1.0, 1.0, -1.0, 1.0, n_side, n_side, single_boundary=True)
    conds = O.Conditions(tri, [lambda x, y, t, u: 0.0 * x], ["Neumann"])
    geo = O.Geometry(tri.points, tri.triangles)
    be = tri.boundary_edges
    bnd_tri, _ = geo.find_triangle(be[:, 0], be[:, 1], tri.boundary_adjacent)
    code, _ = conds.vertex_tables(tri.num_points, tri.has_vertex())
    cp = B.CGrayScott(geo, tri, code, bnd_tri)
    P = tri.points
    r2 = P[:, 0] ** 2 + P[:, 1] ** 2
    u = np.stack([1 - np.exp(-80 * r2), np.exp(-80 * r2)])
    du = np.empty_like(u)
    nth = nthreads or B.max_threads()
    cp.rhs_threaded(u, 0.0, nth, du)  # warm-up
    t0 = time.perf_counter()
    k = 0
    while k < max_evals and time.perf_counter() - t0 < max_seconds:
        cp.rhs_threaded(u, 0.0, nth, du)
        k += 1
    dt = time.perf_counter() - t0
    return {"value": tri.num_points * k / dt, "unit": "point-RHS/s", "cores": nth, "kind": "port",
            "sample": f"{k} threaded evaluations of the {n_side}x{n_side} Gray-Scott system by the C restatement "
                      f"({dt:.2f} s)",
            "ms_per_eval": 1e3 * dt / k}


def run_system(args, F, torch, flush, c2_mesh):
    """FVMSystem: the Gray-Scott tutorial system on the tutorial's 200 x 200 mesh of [-1, 1]^2
    (RHS, and the tutorial's solve to t = 6000 with saveat 10 by adaptive Tsit5) and on the 1000 x 1000 mesh of
    the headline row (RHS: 2M state values).  Algorithmic bytes of one system RHS: per padded
    slot a 4-byte column and 8 bytes per coupled flux block, the state read and the result
    written (16 B per point and component), one mask byte per point; with constant diffusivities
    the blocks share one stored operator (8 bytes per slot in all)."""
    import time

    from fvmgpu.meshes import triangulate_rectangle

    out = {}
    K = max(20, min(args.steps, 200))
    peak = measured_peaks()[0]
    tri200 = triangulate_rectangle(-1.0, 1.0, -1.0, 1.0, 200, 200, single_boundary=True)
    for name, mesh, centre, cross in (("gray_scott_200x200", F.FVMGeometry(tri200), (0.0, 0.0), False),
                                      ("gray_scott_1000x1000", c2_mesh, (0.5, 0.5), False),
                                      ("gray_scott_cross_diffusion_1000x1000", c2_mesh, (0.5, 0.5), True)):
        t0 = time.perf_counter()
        sys = gray_scott_system(F, mesh, centre, cross)
        setup_s = time.perf_counter() - t0
        n, N = mesh.triangulation.num_points, sys.neqs
        info, minfo = sys.info(), mesh.info()
        U = torch.from_numpy(np.ascontiguousarray(sys.initial_condition.T)).cuda()
        dU = torch.empty_like(U)
        torch.cuda.nvtx.range_push(name)  # lets a profiler select this size's launches
        ms = timed_steps(lambda: sys.rhs(dU.T, U.T, internal=True), K, 5, flush, torch)
        torch.cuda.nvtx.range_pop()
        stored = 1 if info["shared_operator"] else info["flux_blocks"]
        alg = (4 + 8 * stored) * minfo["operator_slots"] + 16 * N * n + n
        row = {"points": n, "neqs": N, "setup_s": setup_s, "rhs_ms": float(ms.mean()),
               "point_rhs_per_s": n / (ms.mean() / 1e3), "alg_bytes": alg,
               "gbs": alg / (ms.mean() / 1e3) / 1e9, "frac": alg / (ms.mean() / 1e3) / 1e9 / peak,
               "flux_blocks": info["flux_blocks"], "shared_operator": info["shared_operator"]}
        if n <= 50_000:
            t1 = time.perf_counter()
            sol = F.solve(sys, F.Tsit5(), saveat=10.0)
            wall = time.perf_counter() - t1
            sol = F.solve(sys, F.Tsit5(), saveat=10.0)  # second solve: set-up paid
            row["tsit5_adaptive_to_t6000"] = {"first_wall_s": wall, "elapsed_ms": sol.stats["elapsed_ms"],
                                              "steps": sol.stats["naccept"], "rejects": sol.stats["nreject"],
                                              "driver": sol.stats["driver"], "saves": len(sol.u)}
        out[name] = row
    if not args.no_cpu_baseline:
        try:
            out["cpu_baseline"] = system_cpu_baseline()
        except Exception as e:  # noqa: BLE001  (the GPU rows above stand on their own)
            out["cpu_baseline"] = {"value": None, "error": repr(e)}
    return out


def run_multimesh(args, F, torch):
    """C4 second part: 64 rectangle meshes with log-uniform vertex counts in [1e3, 2e5]
    (nx = ny = round(sqrt(nv)), seed 0), D = 1 + 0.5 sin(2 pi x) sin(2 pi y), zero Dirichlet,
    u0 a Gaussian bump; 50 fixed Tsit5 steps of 1e-6.  One problem on the disjoint union (one
    operator launch per RHS, one captured graph per step) against the per-mesh loop."""
    from fvmgpu.meshes import triangulate_rectangle

    rng = np.random.default_rng(0)
    nvs = np.exp(rng.uniform(np.log(1e3), np.log(2e5), 64))
    tris = [triangulate_rectangle(0.0, 1.0, 0.0, 1.0, int(round(np.sqrt(v))), int(round(np.sqrt(v))),
                                  single_boundary=True) for v in nvs]
    dt, nsteps = 1e-6, 50
    U, poff, _ = F.disjoint_union(tris)
    mesh = F.FVMGeometry(U)
    BCs = F.BoundaryConditions(mesh, (zero_bc,) * U.num_ghost_vertices, (F.Dirichlet,) * U.num_ghost_vertices)
    prob = F.FVMProblem(mesh, BCs, diffusion_function=sine_D, initial_condition=c2_u0(U), final_time=nsteps * dt)
    torch.cuda.synchronize()
    F.solve(prob, F.Tsit5(), dt=dt, adaptive=False, saveat=[nsteps * dt])  # warm-up
    sol = F.solve(prob, F.Tsit5(), dt=dt, adaptive=False, saveat=[nsteps * dt])
    loop_ms = 0.0
    for t in tris:
        m = F.FVMGeometry(t)
        p = F.FVMProblem(m, F.BoundaryConditions(m, zero_bc, F.Dirichlet), diffusion_function=sine_D,
                         initial_condition=c2_u0(t), final_time=nsteps * dt)
        loop_ms += F.solve(p, F.Tsit5(), dt=dt, adaptive=False, saveat=[nsteps * dt]).stats["elapsed_ms"]
    nv = U.num_points
    return {"meshes": len(tris), "vertices": int(nv), "min_vertices": int(min(t.num_points for t in tris)),
            "max_vertices": int(max(t.num_points for t in tris)), "steps": nsteps,
            "elapsed_ms": sol.stats["elapsed_ms"], "vertex_steps_per_s": nv * nsteps / (sol.stats["elapsed_ms"] / 1e3),
            "per_mesh_loop_ms": loop_ms, "speedup_vs_per_mesh_loop": loop_ms / sol.stats["elapsed_ms"]}


def run_adjoint(args, F, torch):
    """C5: DiffusionEquation on the 512 x 512 rectangle, zero Dirichlet, u0 a Gaussian bump,
    200 Tsit5 steps of dt = 1e-6, loss = sum (u(T) - u_obs)^2, gradient with respect to the
    per-vertex log D by the discrete adjoint with checkpoints every 20 steps.  u_obs of each
    instance comes from a true log-D field log 0.4 + 16 Fourier modes of amplitude 0.3 (seeds
    100 + i; D stays below ~1, inside Tsit5's stability interval at this dt); the gradient is
    taken at log 0.4 + 16 modes of amplitude 0.1 (seeds 200 + i).  Batched forward+adjoint
    (B = 32 instances in one call) against the per-instance loop (the B = 1 path, 4 instances
    timed, scaled to 32)."""
    from fvmgpu.meshes import triangulate_rectangle

    N = getattr(args, "adjoint_steps", 200)
    B, dt, K = 32, 1e-6, 20 if N >= 20 else 5
    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, 512, 512, single_boundary=True)
    mesh = F.FVMGeometry(tri)
    BCs = F.BoundaryConditions(mesh, zero_bc, F.Dirichlet)
    tmpl = F.DiffusionEquation(mesh, BCs, diffusion_function=lambda x, y, p: 1.0 + 0.0 * x,
                               initial_condition=c2_u0(tri), final_time=N * dt)
    P = tri.points
    th_true = np.ascontiguousarray(np.log(0.4) + fourier_logfields(P, [100 + i for i in range(B)], 0.3))
    theta = np.ascontiguousarray(np.log(0.4) + fourier_logfields(P, [200 + i for i in range(B)], 0.1))
    u0 = np.ascontiguousarray(np.repeat(tmpl.u0[:, None], B, axis=1))
    adj = F.AdjointProblem(tmpl, batch=B)
    obs = adj.set_log_diffusion(th_true).forward(u0, dt, N)
    adj.set_log_diffusion(theta)
    adj.loss_and_grad(u0, obs, dt, N, checkpoint_every=K)  # warm-up (autotune, first-touch)
    torch.cuda.synchronize()
    with ClockSampler(torch.cuda.current_device()) as clk:
        t0 = time.perf_counter()
        _, _, _, st = adj.loss_and_grad(u0, obs, dt, N, checkpoint_every=K)
        wall_b = time.perf_counter() - t0
    clocks = clk.summary()
    dev_b = st["forward_ms"] + st["reverse_ms"]
    one = F.AdjointProblem(tmpl, batch=1)
    one.set_log_diffusion(theta[:, :1].copy())
    one.loss_and_grad(u0[:, :1].copy(), obs[:, :1].copy(), dt, N, checkpoint_every=K)  # warm-up
    dev_1, wall_1 = 0.0, 0.0
    for i in range(4):
        one.set_log_diffusion(theta[:, i:i + 1].copy())
        t0 = time.perf_counter()
        _, _, _, s1 = one.loss_and_grad(u0[:, i:i + 1].copy(), obs[:, i:i + 1].copy(), dt, N, checkpoint_every=K)
        wall_1 += time.perf_counter() - t0
        dev_1 += s1["forward_ms"] + s1["reverse_ms"]
    loop_dev = dev_1 / 4 * B
    nnz = mesh.info()["operator_nnz"]
    # FP64 issue ceiling: 2 DFMA per clock per SM at the sampled median SM clock
    mhz = clocks["sm_mhz"] or 2070.0
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    ceiling = 2.0 * sms * mhz * 1e6
    dfma_b = adjoint_dfma(tri.num_points, nnz, B, N, K)
    dfma_1 = adjoint_dfma(tri.num_points, nnz, 1, N, K)
    return {"instances": B, "steps": N, "checkpoint_every": K, "checkpoints": st["checkpoints"],
            "rhs_evals": st["rhs_evals"], "transpose_evals": st["transpose_evals"],
            "batched_device_ms": dev_b, "batched_wall_ms": 1e3 * wall_b,
            "gradients_per_s": B / (dev_b / 1e3),
            "per_instance_loop_device_ms": loop_dev, "per_instance_loop_wall_ms": 1e3 * wall_1 / 4 * B,
            "speedup_vs_per_instance_loop": loop_dev / dev_b,
            "fp64_roofline": {"dfma_per_gradient_batch": dfma_b, "batched_dfma_per_s": dfma_b / (dev_b / 1e3),
                              "batched_frac": dfma_b / (dev_b / 1e3) / ceiling,
                              "loop_dfma_per_s": dfma_1 * B / (loop_dev / 1e3),
                              "loop_frac": dfma_1 * B / (loop_dev / 1e3) / ceiling,
                              "ceiling_dfma_per_s": ceiling, "sm_mhz": mhz, "sms": sms,
                              "ceiling": "2 DFMA / clock / SM x SMs x median sampled SM clock"},
            "clocks": clocks}


def _brusselator_system(F, n=100, tf=5.0):
    """The Brusselator tutorial's system (unit square, fluxes -grad/4, sources Phi^2 Psi - 2 Phi
    and -Phi^2 Psi + Phi, boundary values with exp(-t/2), exp(t/2) factors); its exact solution
    is Phi = exp(-x - y - t/2), Psi = exp(x + y + t/2)."""
    tri = F.triangulate_rectangle(0.0, 1.0, 0.0, 1.0, n, n, single_boundary=False)
    mesh = F.FVMGeometry(tri)
    phi_bc = (lambda x, y, t, u, p: -1 / 4 * np.exp(-x - t / 2), lambda x, y, t, u, p: 1 / 4 * np.exp(-1 - y - t / 2),
              lambda x, y, t, u, p: np.exp(-1 - x - t / 2), lambda x, y, t, u, p: -1 / 4 * np.exp(-y - t / 2))
    psi_bc = (lambda x, y, t, u, p: np.exp(x + t / 2), lambda x, y, t, u, p: -1 / 4 * np.exp(1 + y + t / 2),
              lambda x, y, t, u, p: -1 / 4 * np.exp(1 + x + t / 2), lambda x, y, t, u, p: np.exp(y + t / 2))
    P = tri.points
    phi = F.FVMProblem(mesh, F.BoundaryConditions(mesh, phi_bc, (F.Neumann, F.Neumann, F.Dirichlet, F.Neumann)),
                       flux_function=lambda x, y, t, a, b, g, p: (-a[0] / 4, -b[0] / 4),
                       source_function=lambda x, y, t, u, p: u[0] ** 2 * u[1] - 2 * u[0],
                       initial_condition=np.exp(-P[:, 0] - P[:, 1]), final_time=tf)
    psi = F.FVMProblem(mesh, F.BoundaryConditions(mesh, psi_bc, (F.Dirichlet, F.Neumann, F.Neumann, F.Dirichlet)),
                       flux_function=lambda x, y, t, a, b, g, p: (-a[1] / 4, -b[1] / 4),
                       source_function=lambda x, y, t, u, p: -u[0] ** 2 * u[1] + u[0],
                       initial_condition=np.exp(P[:, 0] + P[:, 1]), final_time=tf)
    return tri, F.FVMSystem(phi, psi)


def _steady_rows(F):
    """SteadyFVMProblem: (1) the Laplace tutorial with an internal Dirichlet line (u = 0, 100y,
    100, 100y on the unit square's sides, u = 0 on x = 1/2, y <= 2/5; a 201 x 201 lattice with a
    column of points on the line), initial guess 100y, by NewtonRaphson and by DynamicSS;
    (2) the Helmholtz tutorial at its size (div grad u + u = 0 on [-1, 1]^2, q.n = -1, 125 x 125),
    NewtonRaphson from 0 and then DynamicSS from that solution, as the tutorial does."""
    out = {}
    tri = F.triangulate_rectangle(0.0, 1.0, 0.0, 1.0, 201, 201, single_boundary=False)
    P = tri.points
    on_line = (np.abs(P[:, 0] - 0.5) < 1e-12) & (P[:, 1] <= 0.4 + 1e-12)
    mesh = F.FVMGeometry(tri)
    BCs = F.BoundaryConditions(mesh, (lambda x, y, t, u, p: 0.0 * x, lambda x, y, t, u, p: 100 * y,
                                      lambda x, y, t, u, p: 100.0 + 0.0 * x, lambda x, y, t, u, p: 100 * y),
                               (F.Dirichlet,) * 4)
    ICs = F.InternalConditions((lambda x, y, t, u, p: 0.0 * x,),
                               dirichlet_nodes={int(i): 0 for i in np.nonzero(on_line)[0]})
    u0 = np.where(on_line, 0.0, 100 * P[:, 1])
    for name, alg in (("newton", F.NewtonRaphson()), ("dynamic_ss", F.DynamicSS(F.TRBDF2()))):
        prob = F.FVMProblem(mesh, BCs, ICs, diffusion_function=lambda x, y, t, u, p: 1.0 + 0.0 * x,
                            initial_condition=u0.copy(), final_time=np.inf)
        t0 = time.perf_counter()
        sol = F.solve(F.SteadyFVMProblem(prob), alg)
        wall = time.perf_counter() - t0
        out[f"laplace_internal_line_201x201_{name}"] = {
            "points": tri.num_points, "wall_ms": 1e3 * wall, "device_ms": sol.stats["elapsed_ms"],
            "iterations": sol.stats["iterations"], "krylov_iters": sol.stats["krylov_iters"],
            "residual": sol.stats["residual"]}
    tri = F.triangulate_rectangle(-1.0, 1.0, -1.0, 1.0, 125, 125, single_boundary=True)
    mesh = F.FVMGeometry(tri)
    prob = F.FVMProblem(mesh, F.BoundaryConditions(mesh, (lambda x, y, t, u, p: -1.0 + 0.0 * x,), (F.Neumann,)),
                        diffusion_function=lambda x, y, t, u, p: 1.0 + 0.0 * x, source_function=lambda x, y, t, u, p: u,
                        initial_condition=np.zeros(tri.num_points), final_time=np.inf)
    steady = F.SteadyFVMProblem(prob)
    t0 = time.perf_counter()
    sol = F.solve(steady, F.NewtonRaphson())
    wall_n = time.perf_counter() - t0
    prob.initial_condition[:] = sol.u
    t0 = time.perf_counter()
    sol2 = F.solve(steady, F.DynamicSS(F.TRBDF2()))
    wall_d = time.perf_counter() - t0
    out["helmholtz_125x125"] = {"newton_wall_ms": 1e3 * wall_n, "newton_iterations": sol.stats["iterations"],
                                "newton_krylov_iters": sol.stats["krylov_iters"], "newton_residual": sol.stats["residual"],
                                "then_dynamic_ss_wall_ms": 1e3 * wall_d, "dynamic_ss_steps": sol2.stats["iterations"],
                                "max_abs_change": float(np.max(np.abs(sol2.u - sol.u)))}
    return out


def run_implicit(F, c2_prob):
    """Implicit stepping (TR-BDF2 with the device JVP and matrix-free BiCGStab).  (1) The annulus
    tutorial (polar lattice stand-in, 2,304 vertices, time-dependent inner value, to t = 2,
    saveat 0.2) at the default tolerances: TR-BDF2 against Tsit5, which steps at its stability
    limit there.  (2) C2 (the 1M-vertex FVMProblem): 10 fixed TR-BDF2 steps of 1e-5, 100 times
    the 1000-step Tsit5 row's dt.  (3) The Brusselator tutorial's call, solve(system, TRBDF2(),
    saveat = 1) on its 100 x 100 mesh to t = 5, against Tsit5 and the exact solution.  (4) The
    steady-state tutorials' solves (SteadyFVMProblem with NewtonRaphson and DynamicSS)."""
    out = {}
    tri = F.triangulate_annulus(0.2, 1.0, 24, 96, nsegments=1)
    x, y = tri.points[:, 0], tri.points[:, 1]
    u0 = (10 * np.exp(-25 * ((x + 0.5) ** 2 + (y + 0.5) ** 2)) - 5 * np.exp(-50 * ((x + 0.3) ** 2 + (y + 0.5) ** 2))
          - 10 * np.exp(-45 * ((x - 0.5) ** 2 + (y - 0.5) ** 2)))
    mesh = F.FVMGeometry(tri)
    BCs = F.BoundaryConditions(mesh, (lambda x, y, t, u, p: 0.0 * x, lambda x, y, t, u, p: 50 * (1 - np.exp(-t / 2)) + 0.0 * x),
                               (F.Neumann, F.Dirichlet))
    prob = F.FVMProblem(mesh, BCs, diffusion_function=lambda x, y, t, u, p: 1.0 + 0.0 * x, initial_condition=u0,
                        final_time=2.0)
    F.solve(prob, F.TRBDF2(), saveat=0.2)  # warm-up
    t0 = time.perf_counter()
    imp = F.solve(prob, F.TRBDF2(), saveat=0.2)
    wall_i = time.perf_counter() - t0
    t0 = time.perf_counter()
    exp_ = F.solve(prob, F.Tsit5(), saveat=0.2)
    wall_e = time.perf_counter() - t0
    out["annulus_tutorial"] = {"vertices": tri.num_points, "trbdf2_steps": imp.stats["naccept"],
                               "trbdf2_rejected": imp.stats["nreject"], "newton_iters": imp.stats["newton_iters"],
                               "krylov_iters": imp.stats["krylov_iters"], "trbdf2_wall_ms": 1e3 * wall_i,
                               "trbdf2_device_ms": imp.stats["elapsed_ms"], "tsit5_steps": exp_.stats["naccept"],
                               "tsit5_wall_ms": 1e3 * wall_e, "tsit5_device_ms": exp_.stats["elapsed_ms"],
                               "max_rel_diff": float(np.max(np.abs(np.array(imp.u) - np.array(exp_.u)))
                                                     / np.max(np.abs(exp_.u)))}
    p = c2_prob  # final time 1e-4: ten steps of 1e-5
    sol = F.solve(p, F.TRBDF2(), dt=1e-5, adaptive=False, saveat=[p.final_time])
    out["c2_fixed_dt_1e-5"] = {"steps": sol.stats["naccept"], "device_ms": sol.stats["elapsed_ms"],
                               "ms_per_step": sol.stats["elapsed_ms"] / max(1, sol.stats["naccept"]),
                               "newton_iters": sol.stats["newton_iters"], "krylov_iters": sol.stats["krylov_iters"],
                               "jvps": sol.stats["jvps"],
                               "krylov_iters_per_stage": sol.stats["krylov_iters"] / max(1, sol.stats["newton_iters"])}
    try:
        out["brusselator_tutorial_100x100"] = _brusselator_row(F)
    except Exception as e:  # noqa: BLE001  (the rows above stand on their own)
        out["brusselator_tutorial_100x100"] = {"error": repr(e)[:300]}
    try:
        out["steady_states"] = _steady_rows(F)
    except Exception as e:  # noqa: BLE001
        out["steady_states"] = {"error": repr(e)[:300]}
    return out


def _brusselator_row(F):
    tri, system = _brusselator_system(F)
    P = tri.points
    saveat = np.arange(0.0, 5.0 + 1e-12, 1.0)
    row = {"points": tri.num_points, "unknowns": 2 * tri.num_points}
    for name, alg in (("trbdf2", F.TRBDF2()), ("tsit5", F.Tsit5())):
        t0 = time.perf_counter()
        sol = F.solve(system, alg, saveat=saveat)
        row[f"{name}_wall_ms"] = 1e3 * (time.perf_counter() - t0)
        row[f"{name}_steps"] = sol.stats["naccept"]
        if name == "trbdf2":
            row["krylov_iters_per_newton"] = sol.stats["krylov_iters"] / max(1, sol.stats["newton_iters"])
        ex = [np.stack([np.exp(-P[:, 0] - P[:, 1] - t / 2), np.exp(P[:, 0] + P[:, 1] + t / 2)]) for t in saveat]
        row[f"{name}_max_rel_err_vs_exact"] = float(max(np.max(np.abs(u[c] - e[c])) / np.max(e[c])
                                                        for u, e in zip(sol.u, ex) for c in range(2)))
    return row


def adjoint_dfma(npts, nnz, B, N, K):
    """FP64 fused multiply-adds of one loss-and-gradient call (forward, checkpointed reverse):
    one per operator entry and instance per product, one per term and element of each Tsit5
    stage, cotangent and lambda combination, six per entry and instance for the gradient
    accumulation G += sum_i kb_i (x) Y_i."""
    n, E = npts * B, nnz * B
    step_fwd = 6 * E + 21 * n  # six products; stage combinations 1 + 2 + 3 + 4 + 5 + 6 terms
    fwd = E + n + N * step_fwd
    recompute = sum(E + n + (min(N, s0 + K) - s0 - 1) * step_fwd for s0 in range(0, N, K) if min(N, s0 + K) - s0 > 1)
    # per reverse step: 5 stage products + 15 stage terms; kb_5 (1 term); 6 transpose products;
    # kb_4 .. kb_0 (2 + 3 + 4 + 5 + 6 terms); lambda (6 terms); gradient accumulation
    step_rev = 5 * E + 15 * n + n + 6 * E + 20 * n + 6 * n + 6 * E
    return int(fwd + recompute + N * step_rev)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--no-steady", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched, multi-mesh and adjoint rows")
    ap.add_argument("--rows", default="", help="comma-separated extra rows to run (default: all): " + ",".join(EXTRA_ROWS))
    ap.add_argument("--adjoint-steps", type=int, default=200, help="time steps of the adjoint row")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--steady-points", type=int, default=2_000_000)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
