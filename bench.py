#!/usr/bin/env python
"""Headline benchmark: assembled-and-solved DoF/s for the 3D stationary heat equation
-div(kappa grad u) = 1 on the unit cube, 128^3 hex cells, continuous Q1 (2,146,689 DoF), kappa
piecewise constant and lognormal exp(N(0,1)) per cell (seeded), homogeneous Dirichlet boundary.

One step = assemble (stiffness + load + Dirichlet, one fused pass) + solve to 1e-8 relative error
(CG + Jacobi). `value` is the mixed-precision form (FP32 inner CG, FP64 iterative refinement),
inputs resident in HBM; the plain FP64 GPU path runs on the same inputs for comparison; `e2e` runs
the same step through the public API with kappa copied in from pinned host memory and the solution
copied back every step. Data: synthetic (seeded); the reference publishes no dataset for this path.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
Under torchrun (N > 1) every rank solves its own instance (weak scaling, no collective on the path).
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DoF/s assembled+solved at 1e-8 rel err: mixed/batched vs FP64 GPU; SpMV GB/s"
# kernel classes timed by gdt_context_kernel_timing, in GDT_TIMING_* order
KERNEL_CLASSES = ["spmv_fp64", "spmv_fp32", "cg_update", "cg_direction", "reliable_update"]
SEED = 20261205


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gdt", choices=["gdt", "reference"])
    p.add_argument("--n", type=int, default=128, help="cells per axis")
    p.add_argument("--tol", type=float, default=1e-11, help="relative residual stop of both solvers")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-iters", type=int, default=60, help="CG iterations timed in the CPU sample")
    p.add_argument("--config", default="heat3d", choices=["heat3d", "batched", "fv", "swipdg", "q2"],
                   help="heat3d: the headline 128^3 workload; batched: 512 parametric P1 problems of uneven "
                        "size in one persistent launch; fv: 2D Burgers FV, SSP-RK2; swipdg: SWIPDG P1 "
                        "forward solve + adjoint log-kappa gradient on 256^2 squares; q2: 3D Q2 assembly "
                        "(tensor-core local matrices, diffusion at quadrature points) + solve")
    p.add_argument("--problems", type=int, default=512, help="batched: number of problems")
    p.add_argument("--fv-n", type=int, default=4096, help="fv: cells per axis")
    p.add_argument("--fv-steps", type=int, default=500, help="fv: SSP-RK2 steps per bench step")
    p.add_argument("--fv-batch", type=int, default=1, help="fv: independent initial conditions")
    p.add_argument("--dg-n", type=int, default=256, help="swipdg: squares per axis (2 triangles each)")
    p.add_argument("--q2-n", type=int, default=64, help="q2: hexahedra per axis")
    p.add_argument("--dg-fd", type=int, default=64, help="swipdg: elements of the finite-difference check")
    return p.parse_args()


def kappa_field(n):
    rng = np.random.default_rng(SEED)
    return np.exp(rng.standard_normal(n ** 3))


# ------------------------------------------------------------------------------- clocks ---
class Clocks:
    """nvidia-smi samples (200 ms) during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if "Active" in r[5 + k] and "Not" not in r[5 + k]})
        loaded = [s for s in sm if mx and s > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------------------------- CPU legs ---
def cpu_sample(n, tol, iters, threads):
    """The oracle (CPU restatement of the reference path) on the same workload: full assembly +
    `iters` CG+Jacobi iterations, scaled to the iteration count the full solve needs."""
    import oracle

    oracle.build()
    oracle.set_threads(threads)
    og = oracle.grid(3, [n, n, n], 0.0, 1.0)
    kappa = kappa_field(n)
    t0 = time.perf_counter()
    A, b = oracle.assemble_cg(og, 1, kappa=kappa, force_const=1.0)
    t_asm = time.perf_counter() - t0
    t0 = time.perf_counter()
    _, it, rr, _ = oracle.solve(A, b, tol=1e-300, max_iter=iters)
    t_it = (time.perf_counter() - t0) / max(it, 1)
    return A.n, t_asm, t_it


# --------------------------------------------------------------------------------- GPU arm ---
def run_gdt(args):
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    gdt = importlib.import_module("dune-gdt_gb300")
    gdt._build.build()
    gdt._capi.load()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    n = args.n
    grid = gdt.make_cube_grid([0, 0, 0], [1, 1, 1], [n, n, n])
    space = gdt.ContinuousLagrangeSpace(grid, 1)
    op = gdt.MatrixOperator(grid, space)
    ctx = op.ctx
    ndof, nnz = space.num_DoFs, op.nnz
    kappa_host = kappa_field(n)
    kappa = torch.tensor(kappa_host, device="cuda")
    op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(kappa))
    rhs = torch.zeros(ndof, dtype=torch.float64, device="cuda")
    u = torch.zeros(ndof, dtype=torch.float64, device="cuda")
    # FP64 reference solution at a tight tolerance (untimed) for the error statement
    op.assemble(rhs=rhs, force=1.0, dirichlet=True)
    import ctypes as C

    sched = C.c_int()
    sched_ms = (C.c_double * 8)()
    ctx.call("gdt_matrix_tune", op.handle, C.byref(sched), sched_ms)
    u_ref = op.apply_inverse(rhs, opts={"tol": 1e-14, "max_iter": 200000}).clone()

    def step(precision):
        op.assemble(rhs=rhs, force=1.0, dirichlet=True)
        u.zero_()
        op.apply_inverse(rhs, u, opts={"tol": args.tol, "precision": precision, "max_iter": 200000})

    def timed(precision, steps, warmup, timing=False):
        for _ in range(warmup):
            step(precision)
        lib = gdt._capi.load()
        lib.gdt_context_set_timing(ctx.handle, int(timing))
        lib.gdt_context_spmv_timing(ctx.handle, None, None, None, None, 1)
        launches0 = ctx.kernel_launches
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            step(precision)
        e1.record()
        barrier()
        ms = e0.elapsed_time(e1) / steps
        launches = ctx.kernel_launches - launches0
        import ctypes as C

        kinds = {}
        for k, name in enumerate(KERNEL_CLASSES):
            t, c = C.c_double(), C.c_int64()
            lib.gdt_context_kernel_timing(ctx.handle, k, C.byref(t), C.byref(c), 1)
            if c.value:
                kinds[name] = (t.value, c.value)
        lib.gdt_context_set_timing(ctx.handle, 0)
        info = dict(op.last_solve_info)
        err = ((u - u_ref).abs().max() / u_ref.abs().max()).item()
        return ms, launches, info, err, kinds

    # inputs are larger than L2 (FP64 CSR 728 MB per SpMV), so no L2 flush is needed between steps.
    # The timed steps run the solvers as launched in production (iterations captured in CUDA graphs);
    # one further step per precision, outside the timed region, brackets every kernel class with
    # CUDA events (no graph capture) for the roofline and the per-kernel breakdown.
    clocks = Clocks(local)
    clocks.start()
    ms_mixed, launches, info_mixed, err_mixed, _ = timed("mixed", args.steps, args.warmup)
    clk = clocks.stop()
    ms_fp64, _, info_fp64, err_fp64, _ = timed("fp64", max(1, args.steps // 2), 1)
    _, _, _, _, kinds32 = timed("mixed", 1, 0, timing=True)
    _, _, _, _, kinds64 = timed("fp64", 1, 0, timing=True)
    # replicas: units of all ranks over the slowest rank's time (no collective on the data path)
    ms_mixed = gdt.replicas.max_over_ranks(ms_mixed, device="cuda")
    ms_fp64 = gdt.replicas.max_over_ranks(ms_fp64, device="cuda")

    # end to end through the public API: host kappa (pinned) -> device, assemble + solve, solution -> host
    kappa_pinned = torch.tensor(kappa_host).pin_memory()
    u_host = torch.empty(ndof, dtype=torch.float64).pin_memory()
    kappa_dev = torch.empty_like(kappa)
    op.forms = [gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(kappa_dev))]

    def e2e_step():
        kappa_dev.copy_(kappa_pinned, non_blocking=True)
        op.assemble(rhs=rhs, force=1.0, dirichlet=True)
        u.zero_()
        op.apply_inverse(rhs, u, opts={"tol": args.tol, "precision": "mixed", "max_iter": 200000})
        u_host.copy_(u, non_blocking=True)

    for _ in range(args.warmup):
        e2e_step()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        e2e_step()
    e1.record()
    barrier()
    ms_e2e = gdt.replicas.max_over_ranks(e0.elapsed_time(e1) / args.steps, device="cuda")

    value = world * ndof / (ms_mixed / 1e3)
    inner = info_mixed.get("inner_operator")
    # algorithmic bytes per launch of each kernel class of the mixed iteration (stencil path: 14 slot
    # arrays = diagonal + 13 upper neighbours of the 27-point stencil, p read, q written; update x32,
    # p, r32, q, 1/diag read, x32, r32 written; direction p, r32, 1/diag read, p written)
    if inner == "matrix_free":
        # Chronopoulos-Gear iteration: operator w = A z with r.z, z.w, r.r (coefficients, z, own r read,
        # w written); one vector update p, s, x, r, z (z, p, w, s, x, r, 1/diag read; p, s, x, r, z written)
        classes = {"spmv_fp32": ("k_mf_column: matrix-free FP32 Q1 operator from the element coefficients",
                                 4 * grid.num_elements + 12 * ndof),
                   "cg_update": ("k_cgcg_update: p, s, x, r, z", 48 * ndof)}
    else:
        classes = {"spmv_fp32": ("k_mx_spmv3d / k_mx_spmv: FP32 symmetric-stencil SpMV", (14 + 2) * 4 * ndof),
                   "cg_update": ("k_mx_update: x, r, r.z, r.r", 28 * ndof),
                   "cg_direction": ("k_mx_p: p = z + beta p", 16 * ndof)}
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    by_kernel = {}
    for cls, (kname, nbytes) in classes.items():
        t, c = kinds32.get(cls, (0.0, 0))
        if c:
            ms_l = t / c
            by_kernel[cls] = {"kernel": kname, "bytes_per_launch": nbytes, "avg_launch_ms": ms_l, "launches": c,
                              "total_ms": t, "achieved_gbs": nbytes / (ms_l / 1e3) / 1e9,
                              "frac": nbytes / (ms_l / 1e3) / 1e9 / hbm}
    dom = max(by_kernel, key=lambda k: by_kernel[k]["total_ms"])
    t64b, n64b = kinds64.get("spmv_fp64", (0.0, 0))
    spmv64_ms = t64b / max(n64b, 1)
    bytes64 = 12 * nnz + 4 * (ndof + 1) + 16 * ndof
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "DoF/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_mixed,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64 (FP32 inner CG values/vectors, FP64 assembly, residual and refinement)",
        "data": "synthetic (seeded lognormal kappa per cell)",
        "config": {"workload": f"3D heat equation, {n}^3 Q1 hexes, lognormal kappa, f=1, Dirichlet 0; "
                               "assemble + CG-Jacobi solve to 1e-8 rel error",
                   "dofs": ndof, "nnz": nnz, "precision": "mixed", "tol_rel_residual": args.tol,
                   "l2_flush": "not needed: every step assembles and streams the 685 MB FP64 CSR matrix (again "
                               "in each FP64 residual replacement), far more than the 129 MB L2; within a step "
                               "the inner FP32 iteration's ~52 MB working set stays L2-resident by design",
                   "parallelism": f"replicas x{world}"},
        "error_vs_fp64_reference": err_mixed,
        "solve": {"mixed": info_mixed, "fp64": info_fp64},
        "fp64_plain": {"ms_per_step": ms_fp64, "value": world * ndof / (ms_fp64 / 1e3), "error": err_fp64,
                       "launch": info_fp64.get("launch"),
                       "spmv_gbs": bytes64 / (spmv64_ms / 1e3) / 1e9 if n64b else None,
                       "spmv_frac_of_hbm": (bytes64 / (spmv64_ms / 1e3) / 1e9) / hbm if n64b else None,
                       "spmv_note": "spmv_gbs: the graph form's k_spmv, one CUDA-event pair per launch (timing mode "
                                    "runs the graph kernels); the timed FP64 solves run in the form named by launch"},
        "speedup_mixed_vs_fp64": ms_fp64 / ms_mixed,
        "spmv_autotuner": {"chosen_schedule": sched.value,
                           "ms_per_launch": {name: round(sched_ms[k], 4) for k, name in enumerate(
                               ["csr_vector_g4", "csr_vector_g8", "csr_vector_g16", "csr_vector_g32",
                                "warp_staged_pl8", "warp_staged_pl16", "warp_staged_pl32", "async_staged_28"]) if sched_ms[k] > 0}},
        "e2e": {"value": world * ndof / (ms_e2e / 1e3), "unit": "DoF/s", "h2d_bytes_per_step": 8 * grid.num_elements,
                "d2h_bytes_per_step": 8 * ndof},
        "gpu_launches": launches,
        "kernel_ms_per_launch": {
            "mixed": {k: round(t / c, 5) for k, (t, c) in kinds32.items()},
            "fp64": {k: round(t / c, 5) for k, (t, c) in kinds64.items()},
            "note": "CUDA events around each kernel class in one extra solve without graph capture"},
        "roofline": {"bound": "hbm", "kernel": by_kernel[dom]["kernel"],
                     "achieved": by_kernel[dom]["achieved_gbs"], "peak": hbm, "unit": "GB/s",
                     "frac": by_kernel[dom]["frac"], "bytes_per_launch": by_kernel[dom]["bytes_per_launch"],
                     "avg_launch_ms": by_kernel[dom]["avg_launch_ms"], "launches": by_kernel[dom]["launches"],
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)", "traffic": None,
                     "note": ("the inner iteration's working set stays L2-resident; the matrix-free operator is "
                              "bound by instruction issue and load latency, not HBM "
                              "(profiles/k_mf_column_128cube_ncu_full.md)") if inner == "matrix_free" else None},
        "roofline_by_kernel": by_kernel,
        "inner_operator": inner,
        "clocks": clk,
    }
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        nd, t_asm, t_it = cpu_sample(n, args.tol, args.cpu_iters, threads)
        iters = info_fp64["iterations"]
        t_total = t_asm + t_it * iters
        line["cpu_baseline"] = {"value": nd / t_total, "unit": "DoF/s", "cores": threads, "kind": "port",
                                "sample": f"oracle assembly of the full {n}^3 system + {args.cpu_iters} CG-Jacobi "
                                          f"iterations, scaled to the {iters} iterations the FP64 solve needs "
                                          f"(assembly {t_asm:.2f} s, {t_it * 1e3:.1f} ms/iteration)"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


# ------------------------------------------------------------------------- batched (config 3) ---
def quadrant_kappa(n, mu):
    cells = np.arange(n * n)
    cx, cy = cells % n, cells // n
    q = (cx >= n // 2).astype(int) + 2 * (cy >= n // 2).astype(int)
    return np.repeat(mu[q], 2)


def run_batched(args):
    """512 parametric diffusion problems on P1 triangle meshes of side n in {64,128,256,512}
    (uneven, seeded), kappa = mu_q per quadrant, mu ~ U[0.1, 10]: assemble + solve all in one
    persistent launch (FP64 and mixed), against the plain FP64 GPU path problem by problem."""
    import torch

    gdt = importlib.import_module("dune-gdt_gb300")
    gdt._build.build()
    rng = np.random.default_rng(SEED + 3)
    sides = rng.choice([64, 128, 256, 512], size=args.problems)
    mu = rng.uniform(0.1, 10.0, (args.problems, 4))
    mu_t = torch.tensor(mu, device="cuda")
    b = gdt.BatchedDiffusion(sides.tolist())
    ndof = b.total_dofs
    x_ref = b.solve(mu_t, precision="fp64", tol=1e-13, max_iter=200000).clone()
    x = torch.empty_like(x_ref)

    def err(xx):
        e = 0.0
        for i in range(args.problems):
            r = b.unpack(x_ref, i)
            e = max(e, ((b.unpack(xx, i) - r).abs().max() / r.abs().max()).item())
        return e

    def timed(precision):
        for _ in range(args.warmup):
            b.solve(mu_t, precision=precision, tol=args.tol, x=x, max_iter=200000)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            b.solve(mu_t, precision=precision, tol=args.tol, x=x, max_iter=200000, wait=False)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        b.solve(mu_t, precision=precision, tol=args.tol, x=x, max_iter=200000)  # waits, fills last_info
        return ms, dict(b.last_info), err(x)

    clocks = Clocks(0)
    clocks.start()
    ms_mixed, info_mixed, err_mixed = timed("mixed")
    clk = clocks.stop()
    ms_fp64, info_fp64, err_fp64 = timed("fp64")
    # plain FP64 GPU path, one problem after another (operators built beforehand, as a user would):
    # a stratified sample of `per_class` problems of every size, scaled by the class counts
    per_class = 4
    t_plain = 0.0
    sample = []
    for side in (64, 128, 256, 512):
        idx = np.nonzero(sides == side)[0]
        pick = idx[:per_class]
        probs = []
        for i in pick:
            g = gdt.make_cube_grid([0, 0], [1, 1], [side, side], simplex=True)
            pr = gdt.DiffusionProblem(g, solver_opts={"tol": args.tol, "max_iter": 200000})
            k = torch.tensor(quadrant_kappa(side, mu[i]), device="cuda")
            pr.solve(k)  # warm-up (pattern tuning, first use)
            probs.append((pr, k))
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for pr, k in probs:
            pr.solve(k)
        e1.record()
        torch.cuda.synchronize()
        t_class = e0.elapsed_time(e1) / len(probs) * len(idx)
        t_plain += t_class
        sample.append(f"{len(probs)} of {len(idx)} problems of side {side}")
    line = {
        "metric": "batched DoF/s assembled+solved (512 uneven P1 problems, one persistent launch)",
        "value": ndof / (ms_mixed / 1e3), "unit": "DoF/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_mixed, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 assembly + FP32 inner CG / FP64 refinement", "data": "synthetic (seeded sizes and mu)",
        "config": {"workload": f"{args.problems} problems, side n uniform in {{64,128,256,512}}, P1 Kuhn triangles, "
                               "kappa = mu_q per quadrant, mu ~ U[0.1,10], f=1, Dirichlet 0",
                   "dofs": ndof, "tol_rel_residual": args.tol},
        "batched_mixed": {"ms": ms_mixed, "error_vs_fp64_reference": err_mixed, **info_mixed},
        "batched_fp64": {"ms": ms_fp64, "value": ndof / (ms_fp64 / 1e3), "error_vs_fp64_reference": err_fp64,
                         **info_fp64},
        "plain_fp64_sequential": {"ms": t_plain, "value": ndof / (t_plain / 1e3),
                                  "sample": "; ".join(sample) + " (assemble + solve per problem, timed with CUDA "
                                                                "events, scaled by the class counts)"},
        "speedup_batched_mixed_vs_plain_fp64": t_plain / ms_mixed,
        "speedup_batched_fp64_vs_plain_fp64": t_plain / ms_fp64,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------- Q2 (next-1 row) ---
def run_q2(args):
    """-div(kappa grad u) = 1 on the unit cube, n^3 hexahedra, continuous Q2, Dirichlet 0; kappa at the
    quadrature points = exp(N(0,1)) per element x (1 + 0.5 sin(2 pi x) sin(2 pi y) sin(2 pi z)); one step =
    element-batched assembly (FP64 tensor cores) + load vector + Dirichlet + CG-Jacobi solve (FP64)."""
    import ctypes as C

    import torch

    gdt = importlib.import_module("dune-gdt_gb300")
    gdt._build.build()
    n = args.q2_n
    g = gdt.make_cube_grid([0, 0, 0], [1, 1, 1], [n, n, n])
    space = gdt.ContinuousLagrangeSpace(g, 2)
    ne, ndof = g.num_elements, space.num_DoFs
    xq, _ = space.quadrature()
    nq = xq.shape[0]
    rng = np.random.default_rng(SEED + 6)
    ke = torch.tensor(np.exp(rng.standard_normal(ne)), device="cuda")
    e = torch.arange(ne, device="cuda", dtype=torch.float64)
    ci = torch.stack([e % n, (e // n) % n, e // (n * n)], 1)  # [ne, 3]
    X = (ci[:, None, :] + torch.tensor(xq, device="cuda")[None, :, :]) / n  # physical points [ne, nq, 3]
    s2 = torch.sin(2 * np.pi * X)
    kappa_qp = (ke[:, None] * (1 + 0.5 * s2[..., 0] * s2[..., 1] * s2[..., 2])).contiguous()
    op = gdt.MatrixOperator(g, space)
    op += gdt.LocalElementIntegralBilinearForm(gdt.LocalLaplaceIntegrand(kappa_qp))
    rhs = torch.zeros(ndof, dtype=torch.float64, device="cuda")
    u = torch.zeros(ndof, dtype=torch.float64, device="cuda")
    tol = 1e-10

    def assemble():
        op.assemble(rhs=rhs, force=1.0, dirichlet=True)

    def step():
        assemble()
        u.zero_()
        op.apply_inverse(rhs, u, opts={"tol": tol, "max_iter": 200000})

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    clocks = Clocks(0)
    clocks.start()
    ev[0].record()
    for _ in range(args.steps):
        step()
    ev[1].record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = ev[0].elapsed_time(ev[1]) / args.steps
    info = dict(op.last_solve_info)
    ev[2].record()
    for _ in range(args.steps):
        assemble()
    ev[3].record()
    torch.cuda.synchronize()
    ms_asm = ev[2].elapsed_time(ev[3]) / args.steps
    # the contraction's arithmetic: 2 flops per (pair, quadrature point, element), pairs i <= j
    L = space.max_local_size
    flops = 2.0 * (L * (L + 1) // 2) * nq * ne
    r = (op.apply(u) - rhs).norm().item() / rhs.norm().item()
    line = {
        "metric": "Q2 DoF/s assembled+solved (3D, diffusion at quadrature points)",
        "value": ndof / (ms / 1e3), "unit": "DoF/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded lognormal kappa per element x smooth factor at quadrature points)",
        "config": {"workload": f"{n}^3 hexahedra, continuous Q2 ({ndof} DoF, {op.nnz} nnz), {nq} quadrature "
                               "points per element, f=1, Dirichlet 0, CG-Jacobi FP64 to 1e-10 rel. residual",
                   "dofs": ndof, "nnz": op.nnz},
        "assembly_ms": ms_asm,
        "assembly_contraction_flops": flops,
        "assembly_tflops_upper_bound": flops / (ms_asm / 1e3) / 1e12,
        "solve": info, "final_rel_residual": r,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------ SWIPDG (config 4) ---
def run_swipdg(args):
    """SWIPDG P1 on n^2 squares split into triangles (theta = 1, omega = kappa, sigma 8 / 14), log kappa
    ~ N(0,1) plus high-contrast horizontal channels (each band of 8 cell rows is a channel with
    probability 1/2, seeded; kappa x 1e4 there), f = 1; one step = forward assemble + solve,
    J = 0.5 ||u - u_d||^2 and its log-kappa gradient (adjoint solve + element kernel)."""
    import torch

    gdt = importlib.import_module("dune-gdt_gb300")
    gdt._build.build()
    n = args.dg_n
    g = gdt.make_cube_grid([0, 0], [1, 1], [n, n], simplex=True)
    ne = g.num_elements
    rng = np.random.default_rng(SEED + 4)
    channel = rng.random((n + 7) // 8) < 0.5  # random 8-cell-wide bands
    stripe = channel[((np.arange(ne) // 2) // n) // 8].astype(np.float64)
    logk_host = rng.standard_normal(ne) + stripe * np.log(1e4)
    tol = 1e-12
    prob = gdt.DiffusionProblem(g, dg=True, solver_opts={"tol": tol, "max_iter": 400000})
    ndof = prob.space.num_DoFs
    u_d = prob.solve(torch.exp(torch.tensor(rng.standard_normal(ne), device="cuda"))).clone()
    logk = torch.tensor(logk_host, device="cuda")

    def J(lk):
        u = gdt.DiffusionSolve.apply(lk, prob)
        return 0.5 * torch.sum((u - u_d) ** 2)

    def step():
        lk = logk.clone().requires_grad_(True)
        j = J(lk)
        j.backward()
        return j, lk.grad

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        j, grad = step()
    e1.record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    iters = prob.op.last_solve_info["iterations"]
    launch = prob.op.last_solve_info.get("launch")
    # The system (64 MB) stays in L2, so the solves run as one cooperative launch each (all CG
    # iterations, grid barriers between the steps). Per-iteration time of that launch: one more
    # forward solve bracketed by CUDA events on the context stream (setup kernels included, < 1 %),
    # and the same solve in the graph form (one kernel per step) for comparison.
    op = prob.op
    prob.assemble(torch.exp(logk))
    ctx = op.ctx

    def per_iteration(form):
        ctx.set_solver_launch(form)
        try:
            x = torch.zeros_like(prob.rhs)
            torch.cuda.synchronize()
            a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a0.record(ctx.stream)
            op.apply_inverse(prob.rhs, x, opts=prob.solver_opts)
            a1.record(ctx.stream)
            torch.cuda.synchronize()
            return a0.elapsed_time(a1) / max(op.last_solve_info["iterations"], 1), op.last_solve_info["iterations"]
        finally:
            ctx.set_solver_launch("auto")

    it_ms_persistent, it_persistent = per_iteration("persistent")
    it_ms_graph, it_graph = per_iteration("graph")
    nnz = prob.op.nnz
    # algorithmic bytes of one CG iteration: SpMV (values, columns, row pointers, p gathered once, q)
    # + x/r update (p, q, x, r, dinv read; x, r written) + direction (p, r, dinv read; p written)
    bytes_it = 12 * nnz + 4 * (ndof + 1) + 16 * ndof + 8 * ndof * (7 + 4)
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    # central differences on seeded elements, untimed: h = 1e-6 (the stated check) and h = 1e-4 (less
    # sensitive to the 1e-12 solver tolerance at this contrast); errors relative to max |gradient|
    grad_h = grad.detach().cpu().numpy()
    picks = rng.choice(ne, args.dg_fd, replace=False)
    fd_err = {1e-6: 0.0, 1e-4: 0.0}
    scale = max(np.abs(grad_h).max(), 1e-300)
    with torch.no_grad():
        for e in picks:
            for h in fd_err:
                lp = logk.clone()
                lp[e] += h
                lm = logk.clone()
                lm[e] -= h
                fd = (J(lp).item() - J(lm).item()) / (2 * h)
                fd_err[h] = max(fd_err[h], abs(fd - grad_h[e]) / scale)
    line = {
        "metric": "SWIPDG adjoint gradients: DoF/s (forward solve + adjoint solve + log-kappa gradient)",
        "value": ndof / (ms / 1e3), "unit": "DoF/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded log kappa: N(0,1) + random 8-cell-wide channels x1e4, seeded target field)",
        "config": {"workload": f"{n}^2 squares -> {ne} triangles, SWIPDG P1 ({ndof} DoF, {nnz} nnz), theta=1, "
                               "sigma 8/14, f=1; J = 0.5||u - u_d||^2, CG-Jacobi to 1e-12 rel. residual",
                   "dofs": ndof, "nnz": nnz},
        "cg_iterations_per_solve": iters,
        "solver_launch": launch,
        "ms_per_cg_iteration": {"persistent": it_ms_persistent, "graph": it_ms_graph,
                                "iterations": {"persistent": it_persistent, "graph": it_graph}},
        "gradient_vs_central_differences": {"max_rel_error_h1e-6": fd_err[1e-6], "max_rel_error_h1e-4": fd_err[1e-4],
                                            "elements": int(args.dg_fd), "relative_to": "max |gradient|"},
        "roofline": {"bound": "hbm", "kernel": "k_pcg_persistent: all CG iterations in one cooperative launch",
                     "achieved": bytes_it / (it_ms_persistent / 1e3) / 1e9, "peak": hbm, "unit": "GB/s",
                     "frac": bytes_it / (it_ms_persistent / 1e3) / 1e9 / hbm, "bytes_per_iteration": bytes_it,
                     "ms_per_iteration": it_ms_persistent, "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)",
                     "traffic": None,
                     "note": "the 64 MB system stays in the 129 MB L2 across iterations, so HBM is not the bound: "
                             "ncu shows the FP64 pipe active 64 % of cycles (about 21 FP64 operations per row and "
                             "iteration: 12 in the SpMV) and the rest in the three grid barriers and reductions of "
                             "an iteration (profiles/k_pcg_persistent_swipdg256_ncu_full.md)"},
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------- FV (config 5) ---
def bumps(n, seed, count=32):
    rng = np.random.default_rng(seed)
    xc = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(xc, xc, indexing="xy")  # X varies along axis 1 (x fastest in the flat index)
    u = np.zeros((n, n))
    for _ in range(count):
        a = rng.uniform(-1, 1)
        w = rng.uniform(0.01, 0.1)
        cx, cy = rng.uniform(0, 1, 2)
        dx = np.minimum(np.abs(X - cx), 1 - np.abs(X - cx))
        dy = np.minimum(np.abs(Y - cy), 1 - np.abs(Y - cy))
        u += a * np.exp(-(dx * dx + dy * dy) / (2 * w * w))
    return u.reshape(-1)


def run_fv(args):
    """2D inviscid Burgers on periodic n^2 cubes, FV P0, local LF flux, SSP-RK2 at CFL 0.5."""
    import torch

    gdt = importlib.import_module("dune-gdt_gb300")
    gdt._build.build()
    n, nb = args.fv_n, args.fv_batch
    g = gdt.make_cube_grid([0, 0], [1, 1], [n, n], periodic=True)
    space = gdt.FiniteVolumeSpace(g)
    op = gdt.AdvectionFvOperator(g, gdt.NumericalLaxFriedrichsFlux(gdt.BurgersFlux()), space)
    u0 = np.concatenate([bumps(n, SEED + 5 + b) for b in range(nb)])
    u0_t = torch.tensor(u0, device="cuda")
    dt = 0.5 * min(gdt.estimate_dt_for_hyperbolic_system(g, u0_t[b * n * n:(b + 1) * n * n].contiguous(), op)
                   for b in range(nb))
    u = u0_t.clone()
    stepper = gdt.ExplicitRungeKuttaTimeStepper(op, u, method="ssp2")
    for _ in range(args.warmup):
        u.copy_(u0_t)
        stepper.step(dt, args.fv_steps)
    torch.cuda.synchronize()
    ms = []
    clocks = Clocks(0)
    clocks.start()
    for _ in range(args.steps):
        u.copy_(u0_t)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        stepper.step(dt, args.fv_steps)
        e1.record()
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    clk = clocks.stop()
    t = sum(ms) / len(ms)
    cells = n * n * nb
    mass0 = u0_t.view(nb, -1).sum(1)
    mass_err = ((u.view(nb, -1).sum(1) - mass0).abs() / mass0.abs()).max().item()
    per_step_s = t / 1e3 / args.fv_steps
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    bytes_step = 40 * cells  # fused SSP-RK2: read u twice and k0, write k0 and the next state
    line = {
        "metric": "FV cell-updates/s (2D Burgers, LF flux, SSP-RK2)", "value": cells * args.fv_steps / (t / 1e3),
        "unit": "cell-updates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (32 seeded Gaussian bumps per state)",
        "config": {"workload": f"{nb} x {n}^2 periodic cells, {args.fv_steps} SSP-RK2 steps per bench step, "
                               "dt = 0.5 estimate_dt_for_hyperbolic_system", "dt": dt},
        "rel_mass_conservation_error": mass_err,
        "roofline": {"bound": "fp64 pipe (GB300 FP64 ~1.2 TFLOP/s); HBM fraction shown",
                     "achieved": bytes_step / per_step_s / 1e9, "peak": hbm, "unit": "GB/s",
                     "frac": bytes_step / per_step_s / 1e9 / hbm, "bytes_per_step": bytes_step},
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- reference arm ---
def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    n = args.n
    times = []
    nd = 0
    iters_needed = None
    for s in range(args.warmup + args.steps):
        nd, t_asm, t_it = cpu_sample(n, args.tol, args.cpu_iters, threads)
        if iters_needed is None:
            iters_needed = cg_iterations_needed(n, args.tol)
        if s >= args.warmup:
            times.append(t_asm + t_it * iters_needed)
    ms = 1e3 * sum(times) / len(times)
    value = nd / (ms / 1e3)
    line = {
        "metric": METRIC, "value": value, "unit": "DoF/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded lognormal kappa per cell)",
        "config": {"workload": f"3D heat equation, {n}^3 Q1 hexes, lognormal kappa, f=1, Dirichlet 0; "
                               "assemble + CG-Jacobi solve to 1e-8 rel error", "dofs": nd, "precision": "fp64",
                   "tol_rel_residual": args.tol, "parallelism": "host threads"},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "DoF/s", "cores": threads, "kind": "port",
                         "sample": f"per step: full assembly + {args.cpu_iters} CG-Jacobi iterations, scaled to "
                                   f"the {iters_needed} iterations of the full solve (the reference itself "
                                   "needs DUNE modules absent here; the oracle restates its CPU path)"},
        "e2e": {"value": value, "unit": "DoF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


_ITER_CACHE = {}


def cg_iterations_needed(n, tol):
    """CG+Jacobi iterations of the full solve, from a one-off oracle solve on a coarse proxy would be
    inexact; instead run the full oracle solve once (untimed) and reuse its count."""
    key = (n, tol)
    if key not in _ITER_CACHE:
        import oracle

        og = oracle.grid(3, [n, n, n], 0.0, 1.0)
        A, b = oracle.assemble_cg(og, 1, kappa=kappa_field(n), force_const=1.0)
        _, it, _, _ = oracle.solve(A, b, tol=tol, max_iter=100000)
        _ITER_CACHE[key] = it
    return _ITER_CACHE[key]


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif a.config == "batched":
        run_batched(a)
    elif a.config == "fv":
        run_fv(a)
    elif a.config == "swipdg":
        run_swipdg(a)
    elif a.config == "q2":
        run_q2(a)
    else:
        run_gdt(a)
