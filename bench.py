"""Benchmark: solves/s of the global RBF collocation solve at N = 22,500 nodes.

Workload (the Poisson manufactured-solution configuration): SquareCloud
Nx = Ny = 150 (N = 22,500), interior nodes jittered by U(-0.2h, 0.2h) from a
seed, all facets Dirichlet u* = sin(pi x) sin(pi y), rhs -2 pi^2 u*,
polyharmonic r^3, max_degree = 2 (n = N + 6 = 22,506).  Synthetic, generated
here; no dataset exists for it.

A step is one complete solve of a fresh system: assemble the Kansa matrix,
equilibrate, factor, refine to the stopping test, evaluate vals.  `value` is
the FP32-LU + FP64-GMRES path with inputs resident in HBM; `fp64_lu` is the
plain FP64 LU path on the same GPU; `e2e` is the same metric through the
public API (`updes_gb300.pde_solver`: host capture of the operator, host
arrays copied in, vals and coeffs copied out).  The matrices (4-10 GB) are far
larger than L2, so no L2 flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "solves/s at N=22.5k: FP32-LU+FP64 IR vs FP64 LU, same GB300, rel err<=1e-8"
UNIT = "solves/s"


L2_BYTES = 129e6  # GB300's L2


def workload_spec(nx):
    n = nx * nx + 6
    planes = n * (-(-n // 32) * 32) * 8  # K as two FP32 planes, rows padded to 32 elements
    l2 = ("inputs larger than L2" if planes > L2_BYTES else "inputs smaller than L2") + \
        f" (K's double-float planes {planes / 1e9:.2f} GB, L2 {L2_BYTES / 1e6:.0f} MB)"
    return {"workload": f"poisson_manufactured_r3_deg2_jitter0.2_N{nx * nx}", "nodes": nx * nx,
            "n": n, "rbf": "polyharmonic r^3", "max_degree": 2, "jitter": "U(-0.2h,0.2h) seed 0",
            "facets": "all Dirichlet", "l2": l2}


def make_problem(nx, U):
    facets = {"South": "d", "West": "d", "North": "d", "East": "d"}
    cloud = U.SquareCloud(Nx=nx, Ny=nx, facet_types=facets, jitter=(0.2, 0))
    ustar = lambda c: np.sin(np.pi * c[0]) * np.sin(np.pi * c[1])
    op = lambda x, center, rbf, monomial, fields: U.nodal_laplacian(x, center, rbf, monomial)
    rhs = lambda x, centers, rbf, fields: -2 * np.pi ** 2 * np.sin(np.pi * x[0]) * np.sin(np.pi * x[1])
    bcs = {f: ustar for f in facets}
    return cloud, op, rhs, bcs, ustar


class ClockSampler:
    """nvidia-smi samples (200 ms) during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.proc, self.lines = index, None, []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def oracle_problem(nx):
    """The workload built by the oracle alone (its cloud, rows and weights): K, A and q of the N = nx^2 system."""
    from oracle import updes_np as O
    facets = {"South": "d", "West": "d", "North": "d", "East": "d"}
    cl = O.square_cloud(nx, nx, facets, coords=O.jitter_coords(nx, nx, facets, 0.2, 0))
    X = cl.sorted_nodes
    W = np.zeros((cl.Ni, 5))
    W[:, 3:] = 1.0
    K = O.assemble_K(cl, "polyharmonic", 1, 2, W, O.boundary_rows(cl, {}))
    A = O.assemble_A(cl, "polyharmonic", 1, 2)
    us = np.sin(np.pi * X[:, 0]) * np.sin(np.pi * X[:, 1])
    q = np.where(np.arange(cl.N) < cl.Ni, -2 * np.pi ** 2 * us, us)
    return K, A, q


def cpu_solve(nx, faithful):
    """One CPU solve of the full workload by the oracle on all host cores: assembly of K and A, then either the
    reference's own order of operations (inv -> GEMM -> QR -> inv, updes/operators.py:602-618) or one direct
    LU of K (a proxy with about 11x fewer flops).  Returns (seconds, assembly seconds, vals)."""
    from oracle import updes_np as O
    t0 = time.perf_counter()
    K, A, q = oracle_problem(nx)
    t1 = time.perf_counter()
    if faithful:
        u = O.solve_faithful(K, A, q)[0]
    else:
        u = O.solve_direct(K, A, q)[0]
    t2 = time.perf_counter()
    return t2 - t0, t1 - t0, u


def cpu_threads():
    try:
        from threadpoolctl import threadpool_info
        return max(int(i.get("num_threads", 1)) for i in threadpool_info()) or os.cpu_count()
    except Exception:
        return os.cpu_count()


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, world, rank):
    """The reference's CPU path, timed at the full configuration: the oracle's restatement of its solve
    (assembly, then inv -> GEMM -> QR -> inv, FP64 LAPACK on all host cores).  The reference itself needs JAX,
    which is not installed.  Warm-up steps run the 600-node README configuration (they load LAPACK and start
    its threads; a CPU path has nothing else to warm).  Timed steps run at full size until the time budget
    (--ref-budget-s) would be exceeded by another step; the line reports the steps actually timed."""
    if rank != 0:
        return
    from oracle import updes_np as O
    for _ in range(args.warmup):
        facets = {"South": "n", "West": "d", "North": "d", "East": "d"}
        cl = O.square_cloud(30, 20, facets)
        W = np.zeros((cl.Ni, 5)); W[:, 3:] = 1.0
        O.solve_faithful(O.assemble_K(cl, "polyharmonic", 1, 1, W, O.boundary_rows(cl, {})),
                         O.assemble_A(cl, "polyharmonic", 1, 1), np.ones(cl.N))
    times, asm = [], []
    t_start = time.perf_counter()
    for _ in range(args.steps):
        dt, ta, _ = cpu_solve(args.nx, faithful=True)
        times.append(dt)
        asm.append(ta)
        elapsed = time.perf_counter() - t_start
        if elapsed + statistics.mean(times) > args.ref_budget_s:
            break
    ms = 1000.0 * statistics.mean(times)
    value = 1000.0 / ms
    sample = (f"the full configuration (N={args.nx ** 2}, n={args.nx ** 2 + 6}) solved by the oracle's restatement "
              f"of the reference's order of operations (assembly {statistics.mean(asm):.1f} s, then "
              f"inv -> GEMM -> QR -> inv in FP64 LAPACK), {len(times)} of {args.steps} requested steps timed "
              f"(budget {args.ref_budget_s:.0f} s); JAX is not installed, so the reference itself cannot run")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": len(times),
            "steps_requested": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {**workload_spec(args.nx), "timed": "full size, no extrapolation",
                       "warmup_workload": "README Laplace N=600 (warms LAPACK's threads)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cpu_threads(), "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local):
    import torch

    import updes_gb300 as U
    from updes_gb300 import _lib
    from updes_gb300.operators import DeviceProblem, SolverOptions, prepare, solve_device

    torch.cuda.set_device(local)
    cloud, op, rhs, bcs, ustar = make_problem(args.nx, U)
    # every timed step is a fresh system: no reuse of earlier factors
    opts32 = SolverOptions(precision="fp32", reuse_factorization=False)
    opts64 = SolverOptions(precision="fp64", reuse_factorization=False)
    W, kind, bnodes, geom, q = prepare(op, rhs, cloud, bcs, U.polyharmonic, 2, options=opts32)
    dp = DeviceProblem(cloud, U.polyharmonic, 2, W, kind, bnodes, geom)
    qd = torch.as_tensor(q, device="cuda")
    stream = torch.cuda.current_stream()

    def timed(fn, steps, warmup, with_stats=False, clocks=None, nvtx=None):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        barrier(world)
        _lib.stats_reset(timing=with_stats)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ctx = clocks if clocks is not None else _Null()
        with ctx:
            if nvtx:  # lets a profiler select the timed launches (ncu --nvtx --nvtx-include "<name>/")
                torch.cuda.nvtx.range_push(nvtx)
            ev0.record(stream)
            for _ in range(steps):
                fn()
            ev1.record(stream)
            torch.cuda.synchronize()
            if nvtx:
                torch.cuda.nvtx.range_pop()
        barrier(world)
        ms = ev0.elapsed_time(ev1)
        return max_over_ranks(ms, world), _lib.stats_read()

    # accuracy references
    c64, v64, info64 = solve_device(dp, qd, opts64)
    c32, v32, info32 = solve_device(dp, qd, opts32)
    X = cloud.sorted_nodes
    us = ustar(X.T)
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    v32h, v64h = v32.cpu().numpy(), v64.cpu().numpy()

    # the timed region: K solves with no per-launch instrumentation (the library only counts launches)
    sampler = ClockSampler(local)
    steps = args.steps
    ms32, st32 = timed(lambda: solve_device(dp, qd, opts32), steps, args.warmup, clocks=sampler,
                       nvtx="mixed_solve_timed")
    clocks = sampler.summary()
    # the same K solves again with every launch bracketed by CUDA events on its stream: per-kernel times, the
    # roofline of the dominant kernel (its events run during these solves, so it is measured live)
    ms_prof, stp = timed(lambda: solve_device(dp, qd, opts32), steps, 0, with_stats=True)
    ms64, st64 = timed(lambda: solve_device(dp, qd, opts64), args.fp64_steps, 1)

    # end to end through the public API (host arrays in, vals/coeffs out), as many steps as the timed region
    def e2e_call():
        sol = U.pde_solver(op, rhs, cloud, bcs, U.polyharmonic, 2, options=opts32)
        return sol
    e2e_steps = args.e2e_steps or steps
    ms_e2e, _ = timed(e2e_call, e2e_steps, 1)
    h2d = (cloud.N * 2 * 8 + cloud.Ni * 5 * 8 + (cloud.N - cloud.Ni) * (4 * 2 + 4 + 8 * 8) + cloud.N * 8)
    d2h = cloud.N * 8 + (cloud.N + 6) * 8

    value = world * steps / (ms32 / 1000.0)
    per = {k: v for k, v in stp["by_class"].items() if v["count"]}
    dom = max(per, key=lambda k: per[k]["ms"])
    d = per[dom]
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    if dom == "trailing_update":
        # achieved counts the algorithmic flops of the updates, 2 m nc K per launch (the LU's (2/3) n^3 in
        # all), against the measured bf16 sustained peak of the tensor cores the update runs on (it runs
        # inside a seconds-long step).  Each FP32 operand is written as 3 bf16 integer digits and 8 of the
        # 3 x 3 digit products are exact tcgen05 MMAs (9 with UPDES_OZAKI=2): tensor_work_* count those.
        digit_products = 9 if os.environ.get("UPDES_OZAKI", "") == "2" else 8
        achieved = d["flops"] / (d["ms"] / 1000.0) / 1e12
        peak = peaks.get("bf16_tflops_sustained", 1700.0)
        roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "peak_source": "of measured bf16 sustained" if "bf16_tflops_sustained" in peaks else "of fallback",
                "work": "algorithmic 2*m*nc*K flops per update launch",
                "digit_products": digit_products, "tensor_work_tflops": digit_products * achieved,
                "tensor_work_frac": digit_products * achieved / peak}
    else:
        achieved = d["bytes"] / (d["ms"] / 1000.0) / 1e9
        peak = peaks.get("hbm_gbs", 6800.0)
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": "of measured" if "hbm_gbs" in peaks else "of fallback"}
    roof.update({"kernel": dom, "launches": d["count"] // steps, "avg_launch_ms": d["ms"] / d["count"],
                 "algorithmic_per_launch": (d["flops"] if roof["unit"] == "TFLOP/s" else d["bytes"]) / d["count"],
                 "algorithmic_bytes_per_launch": d["bytes"] / d["count"],
                 "measured_in": "a second pass of the same steps with per-launch CUDA events on each launch's "
                                "stream (the timed region itself runs without them)"})
    # DRAM bytes (read + write) of the update per algorithmic byte (the double-float C planes read and
    # written once plus the digit operands), from one ncu capture of the update kernel at this workload's size;
    # applied to this run's average launch.  An estimate, named with its source.
    dram_per_alg_byte = {"trailing_update": (8.3175e9 / 7.8752e9,
                                             "ncu dram__bytes_read.sum + dram__bytes_write.sum of the largest "
                                             "update launch at n = 22,506 (m = 22,250, nc = 21,994, K = 256; "
                                             "UPDES_LOOKAHEAD=0, launch 8): 4.458 + 3.859 GB against 7.875 GB "
                                             "algorithmic, scaled by this run's algorithmic bytes per launch")}
    if dom in dram_per_alg_byte:
        ratio, src = dram_per_alg_byte[dom]
        roof["traffic"] = ratio * d["bytes"] / d["count"]
        roof["traffic_source"] = src
    else:
        roof["traffic"] = None
    cpu = None
    if rank == 0 and not args.no_cpu:
        dt, ta, u_cpu = cpu_solve(args.nx, faithful=False)
        cpu = {"value": 1.0 / dt, "unit": UNIT, "cores": cpu_threads(), "kind": "port",
               "sample": f"one solve of the full configuration (N={args.nx ** 2}) on the host cores by the oracle, "
                         f"measured, not extrapolated: assembly {ta:.1f} s + a direct FP64 LU of K "
                         f"{dt - ta:.1f} s (a proxy: the reference's inv -> GEMM -> QR order, which "
                         f"`--impl reference` times, costs about 11x the flops); its vals agree with the GPU's "
                         f"mixed path to {rel(v32h, u_cpu):.1e}"}
    acc = {"rel_err_vals_vs_fp64_lu": rel(v32h, v64h), "rel_err_vals_vs_exact": rel(v32h, us),
           "fp64_rel_err_vs_exact": rel(v64h, us), "gmres_iters": info32["iters"],
           "fell_back": info32["fell_back"], "backward_error": info32["backward_error"],
           "fp64_backward_error": info64["backward_error"]}
    gold = os.path.join(ROOT, "tests", "golden", f"full_poisson_{args.nx}.npz")
    if os.path.exists(gold):
        g = np.load(gold)
        acc["rel_err_vals_vs_oracle"] = rel(v32h, g["vals"])
        acc["fp64_rel_err_vals_vs_oracle"] = rel(v64h, g["vals"])
        acc["oracle"] = "FP64 direct LU of K on the CPU (tests/golden/make_fullsize.py)"
        if "vals_faithful" in g.files:
            acc["rel_err_vals_vs_oracle_reference_order"] = rel(v32h, g["vals_faithful"])
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps, "warmup": args.warmup,
        "ms_per_step": ms32 / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32-lu+f64", "data": "synthetic",
        "config": {**workload_spec(args.nx), "parallelism": "replicas" if world > 1 else "single"},
        "fp64_lu": {"value": world * args.fp64_steps / (ms64 / 1000.0), "unit": UNIT,
                    "ms_per_step": ms64 / args.fp64_steps, "steps": args.fp64_steps},
        "speedup_vs_fp64_lu": (ms64 / args.fp64_steps) / (ms32 / steps),
        "accuracy": acc,
        "phases_ms": {k: info32[k] for k in ("t_assemble_ms", "t_factor_ms", "t_refine_ms", "t_eval_ms")},
        "e2e": {"value": world * e2e_steps / (ms_e2e / 1000.0), "unit": UNIT, "steps": e2e_steps,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": roof, "clocks": clocks, "gpu_launches": st32["launches"],
        "kernel_ms_per_step": {k: v["ms"] / steps for k, v in per.items()},
        "instrumented_ms_per_step": ms_prof / steps,
        "cpu_baseline": cpu,
    }
    if rank == 0 and not args.no_extra:
        line["configs"] = extra_configs(args, U, torch)
    if rank == 0:
        print(json.dumps(line), flush=True)


def profile_solve(args):
    """One mixed-precision solve of the workload and nothing else (no warm-up, no FP64 solve), so that a
    profiler sees the solve's launches first: ncu -k regex:<kernel> -c 1 then captures the kernel's first
    launch, e.g. the trailing update after the first 256-column block."""
    import torch

    import updes_gb300 as U
    from updes_gb300.operators import DeviceProblem, SolverOptions, prepare, solve_device
    cloud, op, rhs, bcs, _ = make_problem(args.nx, U)
    o = SolverOptions(precision="fp32", reuse_factorization=False)
    W, kind, bnodes, geom, q = prepare(op, rhs, cloud, bcs, U.polyharmonic, 2, options=o)
    dp = DeviceProblem(cloud, U.polyharmonic, 2, W, kind, bnodes, geom)
    _, _, info = solve_device(dp, torch.as_tensor(q, device="cuda"), o)
    torch.cuda.synchronize()
    print(json.dumps({"profile_solve": {"n": dp.n, **{k: info[k] for k in ("iters", "fell_back", "converged",
                                                                            "backward_error")}}}), flush=True)


def profile_batched(args):
    """One persistent launch (mixed precision, panel width 32, no autotuning) over the first
    ``--profile-batched`` systems of the uneven-cloud workload, and nothing else: the launch a profiler
    capture of batched_solve_kernel expects."""
    import torch

    import updes_gb300 as U
    from updes_gb300 import batched as B
    from updes_gb300 import workloads as WL
    systems = WL.uneven_clouds(args.batch_count)[:args.profile_batched]
    U.pde_solver_batched(systems, precision="fp32", tuner=B.PanelTuner(cache_path=None, candidates=(32,)))
    torch.cuda.synchronize()
    print(json.dumps({"profile_batched": {"systems": len(systems), **B.LAST_BATCHED_TIMING}}), flush=True)


def extra_configs(args, U, torch):
    """The other benchmark configurations, each bounded to seconds, measured with CUDA events (device work)
    on the current stream or the wall clock around a synchronised call (noted per entry).  A configuration
    that fails records its error and the others still run."""
    out = {}
    for fn in (_cfg_readme, _cfg_advection, _cfg_control, _cfg_uneven):
        try:
            out.update(fn(args, U, torch))
        except Exception as e:  # noqa: BLE001 - reported in the JSON line
            torch.cuda.synchronize()
            out[fn.__name__[5:]] = {"error": f"{type(e).__name__}: {e}"}
    return out


def _cfg_readme(args, U, torch):
    """README Laplace, N = 600: latency of one solve through the public API (host arrays in and out)."""
    from updes_gb300 import workloads as WL
    out = {}
    sysd = WL.readme_laplace()
    for prec in ("fp64", "fp32"):
        o = U.SolverOptions(precision=prec, reuse_factorization=False)
        for _ in range(3):
            U.pde_solver_jit(options=o, **sysd)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        reps = 20
        for _ in range(reps):
            U.pde_solver_jit(options=o, **sysd)
        torch.cuda.synchronize()
        ms = 1000 * (time.perf_counter() - t0) / reps
        out[f"readme_laplace_N600_{prec}"] = {"metric": "solves/s through pde_solver_jit (wall clock)",
                                              "value": 1000.0 / ms, "ms_per_solve": ms}
    return out


def _cfg_advection(args, U, torch):
    """Advection-diffusion, N = 6,400, 64 bumps, implicit steps replayed from a CUDA graph.  The factors are
    FP64 (computed once), applied in double-float with one refinement sweep: the configuration names FP32 LU
    factors, but classical refinement on FP32 factors diverges on this system (the first step's error
    against the oracle grows from 4e1 after 4 sweeps to 1e13 after 16, GPU measurement)."""
    from updes_gb300 import workloads as WL
    from updes_gb300.multirhs import MultiRHSSolver
    stream = torch.cuda.current_stream()
    sysd, U0, dt = WL.advection_bumps(80, 64)
    t0 = time.perf_counter()
    solver = MultiRHSSolver(sysd["diff_operator"], sysd["cloud"], sysd["boundary_conditions"], sysd["rbf"],
                            sysd["max_degree"], sweeps=1)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    Ud = torch.as_tensor(U0, device="cuda").contiguous()
    g = solver.make_graph(Ud, steps_per_graph=1, rhs_scale=1.0 / dt)
    for _ in range(3):
        g.replay()
    steps = args.adv_steps
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        g.replay()
    e1.record(stream)
    torch.cuda.synchronize()
    solver.check_status()
    ms = e0.elapsed_time(e1) / steps
    return {"advection_diffusion_N6400_R64_fp64_factors": {
        "metric": "column-solves/s (64 right-hand sides per implicit step, graph replay, CUDA events)",
        "value": 64 * 1000.0 / ms, "ms_per_step": ms, "steps": steps, "factor_setup_s": setup_s,
        "factors": "FP64 factors (not the FP32 LU the configuration names: classical refinement on FP32 factors "
                   "diverges on this system), applied in double-float, one refinement sweep per step; the first "
                   "step is within 1e-9 of the oracle (GPU test)"}}


def _cfg_control(args, U, torch):
    """Boundary control with adjoint, N = 10,000, r^5, FP64: forward and reverse through the solve."""
    from updes_gb300 import workloads as WL
    from updes_gb300.adjoint import pde_solver_torch
    sysd, F, controls, ut = WL.boundary_control(100, 32)
    cl = sysd["cloud"]
    Ni = cl.Ni
    utd = torch.as_tensor(ut, device="cuda")
    o = U.SolverOptions(precision="fp64")
    fwd_ms, bwd_ms = [], []
    for i in range(4):
        ctl = torch.tensor(controls[i], device="cuda", requires_grad=True)
        ft = [torch.tensor(f, device="cuda", requires_grad=True) for f in F]
        bcs = dict(sysd["boundary_conditions"])
        bcs["North"] = ctl
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        vals, _ = pde_solver_torch(sysd["diff_operator"], sysd["rhs_operator"], cl, bcs, sysd["rbf"],
                                   sysd["max_degree"], diff_args=ft, options=o)
        J = torch.mean((vals[:Ni] - utd[:Ni]) ** 2) + 1e-4 * torch.sum(ctl ** 2)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        J.backward()
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        if i > 0:  # the first pair warms up
            fwd_ms.append(1000 * (t1 - t0))
            bwd_ms.append(1000 * (t2 - t1))
    f, b = statistics.median(fwd_ms), statistics.median(bwd_ms)
    return {"boundary_control_adjoint_N10000": {
        "metric": "gradient evaluations/s (forward + reverse, wall clock, host capture included)",
        "value": 1000.0 / (f + b), "forward_ms": f, "backward_ms": b, "backward_over_forward": b / f}}


def _cfg_uneven(args, U, torch):
    """Batched uneven clouds: 512 independent systems of 100 to 2,025 nodes.  Per-problem FP64 (each system
    its own solve, 8 host-driven streams) against the persistent launch (one CTA per SM takes systems from a
    device queue), mixed ("auto": double-float LU on the FP32 pipes + FP64 refinement, FP64 relaunch of the
    systems that do not reach the FP64 floor) and FP64.  Wall clock includes host preparation; the
    persistent launch's own device time is reported beside it."""
    from updes_gb300 import batched as B
    from updes_gb300 import workloads as WL
    out = {}
    systems = WL.uneven_clouds(args.batch_count)
    o = U.SolverOptions(precision="fp64", reuse_factorization=False)
    U.pde_solver_many(systems[:16], options=o, streams=8)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    U.pde_solver_many(systems, options=o, streams=8)
    torch.cuda.synchronize()
    dt_s = time.perf_counter() - t0
    infos = U.operators.LAST_MANY_INFO
    out[f"uneven_clouds_{len(systems)}_per_problem_fp64"] = {
        "metric": "systems/s through pde_solver_many (wall clock, host preparation included)",
        "value": len(systems) / dt_s, "seconds": dt_s, "converged": int(sum(i["converged"] for i in infos))}
    for prec in ("auto", "fp64"):
        U.pde_solver_batched(systems, precision=prec)  # warm-up: the autotuner measures its panel widths here
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        U.pde_solver_batched(systems, precision=prec)
        torch.cuda.synchronize()
        dt_s = time.perf_counter() - t0
        tm = dict(B.LAST_BATCHED_TIMING)
        bi = B.LAST_BATCHED_INFO
        out[f"uneven_clouds_{len(systems)}_persistent_{'mixed' if prec == 'auto' else 'fp64'}"] = {
            "metric": "systems/s through pde_solver_batched (wall clock, host preparation included)",
            "value": len(systems) / dt_s, "seconds": dt_s,
            "device_systems_per_s": len(systems) / ((tm["launch_ms"] + tm["fp64_relaunch_ms"]) / 1000.0),
            "launch_ms": tm["launch_ms"], "fp64_relaunch_ms": tm["fp64_relaunch_ms"], "relaunched": tm["relaunched"],
            "host_prepare_s": tm["host_prepare_s"], "converged": int(sum(i["converged"] for i in bi)),
            "max_backward_error": float(max(i["backward_error"] for i in bi)),
            "panel_widths": sorted({int(i["panel_width"]) for i in bi})}
    return out


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--nx", type=int, default=150)
    ap.add_argument("--fp64-steps", type=int, default=1)
    ap.add_argument("--e2e-steps", type=int, default=0, help="end-to-end steps (default: --steps)")
    ap.add_argument("--ref-budget-s", type=float, default=240.0,
                    help="time budget of the reference arm's timed steps (at least one full-size step runs)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the other configurations")
    ap.add_argument("--adv-steps", type=int, default=500)
    ap.add_argument("--batch-count", type=int, default=512)
    ap.add_argument("--profile-solve", action="store_true",
                    help="run one mixed solve and exit (the launch order a profiler capture expects)")
    ap.add_argument("--profile-batched", type=int, default=0,
                    help="run one persistent launch over this many uneven clouds and exit")
    args = ap.parse_args()
    if args.profile_solve:
        profile_solve(args)
        return
    if args.profile_batched:
        profile_batched(args)
        return
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
