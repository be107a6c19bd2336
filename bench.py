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


def cpu_sample(nx_sample, n_full):
    """The oracle's restatement of the reference's solve (inv -> GEMM -> QR -> inv) at a bounded
    sample size, on all host cores; scaled to the full size by (n_full / n_sample)^3."""
    from oracle import updes_np as O
    facets = {"South": "d", "West": "d", "North": "d", "East": "d"}
    xs = np.linspace(0, 1, nx_sample)
    h = xs[1] - xs[0]
    coords = np.stack(np.meshgrid(xs, xs, indexing="ij"), -1).reshape(-1, 2)
    ii, jj = np.divmod(np.arange(nx_sample * nx_sample), nx_sample)
    inner = (ii > 0) & (ii < nx_sample - 1) & (jj > 0) & (jj < nx_sample - 1)
    coords[inner] += np.random.default_rng(0).uniform(-0.2 * h, 0.2 * h, size=(inner.sum(), 2))
    t0 = time.perf_counter()
    cl = O.square_cloud(nx_sample, nx_sample, facets, coords=coords)
    X = cl.sorted_nodes
    W = np.zeros((cl.Ni, 5)); W[:, 3:] = 1.0
    K = O.assemble_K(cl, "polyharmonic", 1, 2, W, O.boundary_rows(cl, {}))
    A = O.assemble_A(cl, "polyharmonic", 1, 2)
    us = np.sin(np.pi * X[:, 0]) * np.sin(np.pi * X[:, 1])
    q = np.where(np.arange(cl.N) < cl.Ni, -2 * np.pi ** 2 * us, us)
    t1 = time.perf_counter()
    O.solve_faithful(K, A, q)
    t2 = time.perf_counter()
    n_s = cl.N + 6
    r = n_full / n_s
    # assembly is O(n^2), the inverse / GEMM / QR O(n^3)
    return t2 - t0, (t1 - t0) * r ** 2 + (t2 - t1) * r ** 3, n_s


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
    """The reference's CPU path (the oracle port: the reference needs JAX, which is not installed)."""
    if rank != 0:
        return
    n_full = args.nx * args.nx + 6
    for _ in range(args.warmup):
        cpu_sample(args.sample_nx, n_full)
    times = []
    for _ in range(args.steps):
        dt, scaled, n_s = cpu_sample(args.sample_nx, n_full)
        times.append(scaled)
    ms = 1000.0 * statistics.mean(times)
    value = 1000.0 / ms
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": workload_spec(args.nx),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cpu_threads(), "kind": "port",
                             "sample": f"oracle restatement of the reference solve (inv->GEMM->QR->inv, FP64 "
                                       f"LAPACK) at N={args.sample_nx ** 2} (n={args.sample_nx ** 2 + 6}) per step; assembly "
                                       f"scaled by (n/n_sample)^2 and the solve by (n/n_sample)^3 to n={n_full}; "
                                       f"JAX is not installed, so the "
                                       f"reference itself cannot run"},
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

    sampler = ClockSampler(local)
    ms32, st32 = timed(lambda: solve_device(dp, qd, opts32), args.steps, args.warmup, with_stats=True, clocks=sampler,
                       nvtx="mixed_solve_timed")
    clocks = sampler.summary()
    ms64, st64 = timed(lambda: solve_device(dp, qd, opts64), args.fp64_steps, 1)

    # end to end through the public API (host arrays in, vals/coeffs out)
    def e2e_call():
        sol = U.pde_solver(op, rhs, cloud, bcs, U.polyharmonic, 2, options=opts32)
        return sol
    ms_e2e, _ = timed(e2e_call, max(1, args.e2e_steps), 1)
    h2d = (cloud.N * 2 * 8 + cloud.Ni * 5 * 8 + (cloud.N - cloud.Ni) * (4 * 2 + 4 + 8 * 8) + cloud.N * 8)
    d2h = cloud.N * 8 + (cloud.N + 6) * 8

    steps = args.steps
    value = world * steps / (ms32 / 1000.0)
    per = {k: v for k, v in st32["by_class"].items() if v["count"]}
    dom = max(per, key=lambda k: per[k]["ms"])
    d = per[dom]
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    if dom == "trailing_update":
        # The mixed path's trailing update runs on the tensor cores: each FP32 operand is written as 3 bf16
        # integer digits, and 8 of the 3 x 3 digit products of every 2 m n K update (all but the one below
        # the digit cut) are exact tcgen05 MMAs (9 with UPDES_OZAKI=2).
        # achieved = tensor flops of those products / kernel time, against the measured bf16 peak (the
        # kernel runs inside a seconds-long step: the sustained figure).
        digit_products = 9 if os.environ.get("UPDES_OZAKI", "") == "2" else 8
        achieved = digit_products * d["flops"] / (d["ms"] / 1000.0) / 1e12
        peak = peaks.get("bf16_tflops_sustained", 1700.0)
        roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "peak_source": "of measured bf16 sustained" if "bf16_tflops_sustained" in peaks else "of fallback",
                "digit_products": digit_products,
                "fp64_equivalent_tflops": d["flops"] / (d["ms"] / 1000.0) / 1e12}
        d = dict(d, flops=digit_products * d["flops"])
    else:
        achieved = d["bytes"] / (d["ms"] / 1000.0) / 1e9
        peak = peaks.get("hbm_gbs", 6800.0)
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": "of measured" if "hbm_gbs" in peaks else "of fallback"}
    roof.update({"kernel": dom, "launches": d["count"] // steps, "avg_launch_ms": d["ms"] / d["count"],
                 "algorithmic_per_launch": (d["flops"] if roof["unit"] == "TFLOP/s" else d["bytes"]) / d["count"]})
    # DRAM bytes (read + write) per algorithmic byte of the dominant kernel, from one ncu capture of the update
    # after the first block at n = 10,006 (m = 9,750, nc = 9,494, K = 256: 1.478 GB of DRAM traffic against
    # 1.501 GB algorithmic, current kernel), scaled to this run's average launch by its algorithmic bytes (the
    # traffic grows with the entries updated)
    dram_per_alg_byte = {"trailing_update": 1.4777e9 / 1.5008e9}
    roof["traffic"] = dram_per_alg_byte[dom] * d["bytes"] / d["count"] if dom in dram_per_alg_byte else None
    cpu = None
    if rank == 0 and not args.no_cpu:
        dt, scaled, n_s = cpu_sample(args.sample_nx, args.nx * args.nx + 6)
        cpu = {"value": 1000.0 / (scaled * 1000.0), "unit": UNIT, "cores": cpu_threads(), "kind": "port",
               "sample": f"oracle restatement of the reference solve (inv->GEMM->QR->inv) at N={args.sample_nx ** 2}: "
                         f"{dt:.2f} s; assembly scaled by (n/n_sample)^2, solve by (n/n_sample)^3 "
                         f"(n/n_sample = {(args.nx ** 2 + 6) / n_s:.2f})"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps, "warmup": args.warmup,
        "ms_per_step": ms32 / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32-lu+f64", "data": "synthetic",
        "config": {**workload_spec(args.nx), "parallelism": "replicas" if world > 1 else "single"},
        "fp64_lu": {"value": world * args.fp64_steps / (ms64 / 1000.0), "unit": UNIT,
                    "ms_per_step": ms64 / args.fp64_steps, "steps": args.fp64_steps},
        "speedup_vs_fp64_lu": (ms64 / args.fp64_steps) / (ms32 / steps),
        "accuracy": {"rel_err_vals_vs_fp64_lu": rel(v32h, v64h), "rel_err_vals_vs_exact": rel(v32h, us),
                     "fp64_rel_err_vs_exact": rel(v64h, us), "gmres_iters": info32["iters"],
                     "fell_back": info32["fell_back"], "backward_error": info32["backward_error"],
                     "fp64_backward_error": info64["backward_error"]},
        "phases_ms": {k: info32[k] for k in ("t_assemble_ms", "t_factor_ms", "t_refine_ms", "t_eval_ms")},
        "e2e": {"value": world * max(1, args.e2e_steps) / (ms_e2e / 1000.0), "unit": UNIT,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": roof, "clocks": clocks, "gpu_launches": st32["launches"],
        "kernel_ms_per_step": {k: v["ms"] / steps for k, v in per.items()},
        "cpu_baseline": cpu,
    }
    if rank == 0 and not args.no_extra:
        line["configs"] = extra_configs(args, U, torch)
    if rank == 0:
        print(json.dumps(line), flush=True)


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
    """Advection-diffusion, N = 6,400, 64 bumps, implicit steps replayed from a CUDA graph."""
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
    return {"advection_diffusion_N6400_R64": {
        "metric": "column-solves/s (64 right-hand sides per implicit step, graph replay, CUDA events)",
        "value": 64 * 1000.0 / ms, "ms_per_step": ms, "steps": steps, "factor_setup_s": setup_s,
        "factors": "FP64, applied as double-float planes, one refinement sweep"}}


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
    """Batched uneven clouds: independent systems of 100 to 2,025 nodes on 8 streams."""
    from updes_gb300 import workloads as WL
    out = {}
    systems = WL.uneven_clouds(args.batch_count)
    for prec in ("fp32", "fp64"):
        o = U.SolverOptions(precision=prec, reuse_factorization=False)
        U.pde_solver_many(systems[:16], options=o, streams=8)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        U.pde_solver_many(systems, options=o, streams=8)
        torch.cuda.synchronize()
        dt_s = time.perf_counter() - t0
        infos = U.operators.LAST_MANY_INFO
        out[f"uneven_clouds_{len(systems)}_{prec}"] = {
            "metric": "systems/s through pde_solver_many (wall clock, host preparation included)",
            "value": len(systems) / dt_s, "seconds": dt_s,
            "fell_back": int(sum(i["fell_back"] for i in infos)),
            "converged": int(sum(i["converged"] for i in infos))}
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
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--sample-nx", type=int, default=70)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the other configurations")
    ap.add_argument("--adv-steps", type=int, default=500)
    ap.add_argument("--batch-count", type=int, default=512)
    args = ap.parse_args()
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
