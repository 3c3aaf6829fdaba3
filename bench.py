#!/usr/bin/env python
"""Benchmark of the particle-in-cell Stokes hot path on one GB300 (replicas on N GPUs).

One step = one pass of the hot path over the resident material points:
    binning + integration-point mapping  ->  rheology + element assembly  ->  BSSCR Stokes
    solve (Schur-complement FGMRES, A11 FGMRES + geometric multigrid) to a relative residual
    of 1e-6.
Workload (default, --workload grf): 3D Q1-P0 Stokes, 128^3 elements, 30 seeded uniform-random
points per element, log10(viscosity) a seeded Gaussian random field (correlation length 0.1)
spanning [-3, 3] (1e6 contrast), density 0.5 * field + 0.5, free-slip walls, 5-level multigrid.
The timed form is the mixed-precision solve (--precision mixed: FP32 operators, smoothers and
inner solves inside FP64 refinement, FP64 Schur iteration); the FP64 solve of the same inputs is
timed beside it ("comparison", with the mixed solution's distance from it).
--workload spheres: 64^3 elements, 27 points per element on a jittered grid, 50 seeded spheres
(viscosity 10^U(-2,3), density U(0,1)), 4-level multigrid.

Arms:
  (default)          this library through its C ABI (ctypes)
  --impl reference   the reference algorithm restated in C (oracle/uwref.c), timed on the
                     host cores on a bounded sample of the same workload
Prints one JSON line (rank 0).
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Stokes solve s to 1e-6 rel. residual, mixed+learned vs FP64 GPU; particles/s"
# FP64 FMA throughput of this part (an FMA-chain micro-benchmark on the GB300), TFLOP/s
FP64_TFLOPS = 1.19
UNIT = "particles/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="grf", choices=["grf", "spheres"])
    ap.add_argument("--nel", type=int, default=None, help="elements per axis (grf: 128, spheres: 64)")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--no-compare", "--no-mixed", dest="no_compare", action="store_true",
                    help="skip the other precision form")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--mode", default="step", choices=["step", "kernels", "bfbt", "accuracy"],
                    help="step: the full hot-path step; kernels: operator apply and smoother only")
    ap.add_argument("--iters", type=int, default=20, help="launches per kernel in --mode kernels")
    ap.add_argument("--cpu-nel", type=int, default=20, help="mesh of the CPU baseline sample")
    ap.add_argument("--no-learned", action="store_true", help="skip the mixed+learned leg")
    ap.add_argument("--learn-nel", type=int, default=64, help="mesh the U-Net is trained on (then transferred)")
    ap.add_argument("--learn-rhs", type=int, default=40, help="multigrid solves that give the training pairs")
    ap.add_argument("--learn-epochs", type=int, default=12)
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    def __init__(self, world, local, use_cuda=True):
        self.world = world
        self.pg = None
        if world > 1:
            import torch
            import torch.distributed as dist
            backend = "nccl" if use_cuda and torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(local)
            dist.init_process_group(backend=backend)
            self.dist = dist
            self.torch = torch
            self.device = torch.device("cuda", local) if backend == "nccl" else torch.device("cpu")

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max(self, v):
        if self.world == 1:
            return v
        t = self.torch.tensor([float(v)], device=self.device, dtype=self.torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v):
        if self.world == 1:
            return v
        t = self.torch.tensor([float(v)], device=self.device, dtype=self.torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi sampled every 200 ms while running (SM clock, max clock, throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def default_nel(kind):
    return 128 if kind == "grf" else 64


def make_workload(kind, nel, shuffle=True):
    from earthbyte_underworld_gb300 import workloads as W
    if kind == "grf":
        return W.grf(nel=(nel, nel, nel), ppc=30, seed=11, grid=256, corr=0.1, shuffle=shuffle)
    return W.spheres(nel=(nel, nel, nel), nspheres=50, seed=2024, shuffle=shuffle)


def workload_name(kind, nel):
    if kind == "grf":
        return f"stokes3d_grf_{nel}cube_30ppc_1e6contrast"
    return f"stokes3d_spheres_{nel}cube_27ppc_50spheres"


def solve_kw(w):
    kw = dict(SOLVE_KW)
    kw["mg_levels"] = w.get("mg_levels", SOLVE_KW["mg_levels"])
    return kw


# BSSCR options: FGMRES Schur iteration (-scr_ksp_type fgmres) with the scaled BFBt Schur preconditioner
# (-Q22_pc_type gtkg, Solvers/KSPSolvers/src/BSSCR/pc_ScaledGtKG.c) and FGMRES velocity solves
# (-A11_ksp_type fgmres, Solvers/SysTest/ConvergenceTests/options-solv-mg.opt); tolerances chosen so
# that the full Stokes residual reaches 1e-6
SOLVE_KW = dict(mg_levels=4, smooth_down=2, smooth_up=2, smoother=1, schur_type=1, schur_pc=3, scr_rtol=1e-6, a11_rtol=5e-7,
                back_rtol=1e-7, restart=30, max_outer=500, max_inner=2000, bfbt_rtol=1e-2, bfbt_max_it=2000)


# ------------------------------------------------------------------------------------------
# CPU leg: the restated reference path on the host cores
# ------------------------------------------------------------------------------------------
def cpu_step(O, w, nthreads):
    import numpy as np
    m = O.make_mesh(3, w["nel"])
    xyz = np.stack([w["x"], w["y"], w["z"]], axis=1)
    t0 = time.perf_counter()
    _, off, perm, xi, _ = O.map_points(m, xyz)
    mats = [O.make_material([(mm.laws[i].law, list(mm.laws[i].p)) for i in range(mm.n_laws)], density=mm.density,
                            alpha=mm.alpha, ref_temp=mm.ref_temp) for mm in w["materials"]]
    f = O.make_fields(gravity=w["gravity"], vert_axis=w["vert_axis"])
    Ke, fe, Ge, Se, _ = O.assemble(m, off, perm, xi, w["material"], mats, f, point_eta=w.get("eta"),
                                   point_rho=w.get("rho"), nthreads=nthreads)
    t1 = time.perf_counter()
    levels = 3 if w["nel"][0] % 4 == 0 else 2
    u, p, rep = O.solve_bsscr(m, w["fixed"], Ke, Ge, fe, Se, mg_levels=levels, smooth=SOLVE_KW["smooth_down"],
                              schur_type=SOLVE_KW["schur_type"], schur_pc=SOLVE_KW["schur_pc"],
                              scr_rtol=SOLVE_KW["scr_rtol"], a11_rtol=SOLVE_KW["a11_rtol"],
                              back_rtol=SOLVE_KW["back_rtol"], bfbt_rtol=SOLVE_KW["bfbt_rtol"],
                              bfbt_max_it=SOLVE_KW["bfbt_max_it"], nthreads=nthreads)
    t2 = time.perf_counter()
    return t2 - t0, t1 - t0, rep


# what one profiled launch of each kernel family is, and what its algorithmic bytes count
FAMILY_NOTES = {
    "smooth": "one Chebyshev step (k_cheb_step): 27 stencil blocks of 3x3, the diagonal-block inverse, rhs "
              "and the iterate moved once per node; FP64 kernels on this part are also limited by its "
              "1.2 TFLOP/s FP64 rate (fp_tflops)",
    "apply": "one operator apply (k_apply): 27 stencil blocks of 3x3 per node, x read and y written once",
    "schur_pc": "one replay of the BFBt inner-CG graph = 12 iterations of k_cg_update + the direction kernel "
                "(k_cg_spmv_dir on the 27-point G^T W G stencil, or the matrix-free FP32 kernel k_cg_mf3_dir_tma, "
                "its element and weight planes staged by TMA, on meshes whose FP32 stencil would not fit in half "
                "of L2); the roofline line is the direction kernel",
    "learned": "U-Net corrections: tcgen05 implicit-GEMM convolutions (BF16, FP32 accumulate) and the head",
    "assembly": "rheology + moments per point, contraction of the moments into K_e (tensor core in the mixed forms)",
    "setup": "every launch of the solver's setup: node stencils from K_e, the Galerkin hierarchy and coarsest "
             "inverse, FP32 copies, Chebyshev bounds (power iterations), the right-hand side and the BFBt "
             "operator (weights, G^T W G stencil)",
}


def cpu_baseline(kind, nel, nthreads):
    from oracle import oracle as O
    O.lib()
    w = make_workload(kind, nel)
    dt, dt_asm, rep = cpu_step(O, w, nthreads)
    n = w["x"].shape[0]
    return {"value": n / dt, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"{kind} workload at {nel}^3 elements ({n} points), one full step: map + assemble + "
                      f"BSSCR to 1e-6 in FP64 (oracle/uwref.c, OpenMP); assembly part {n / dt_asm:.3e} points/s; "
                      f"solve residual {rep.rel_residual:.1e}",
            "step_s": dt}


def run_reference(args):
    rank, world, local = dist_info()
    if rank != 0:
        return 0
    from oracle import oracle as O
    O.lib()
    nthreads = os.cpu_count() or 1
    w = make_workload(args.workload, args.cpu_nel)
    n = w["x"].shape[0]
    for _ in range(args.warmup):
        cpu_step(O, w, nthreads)
    times = []
    res = None
    for _ in range(args.steps):
        dt, _, rep = cpu_step(O, w, nthreads)
        times.append(dt)
        res = rep.rel_residual
    tot = sum(times)
    value = n * args.steps / tot
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": f"{workload_name(args.workload, args.cpu_nel)} (bounded sample of the "
                                  f"{default_nel(args.workload)}^3 workload)",
                      "precision": "fp64", "solver": "BSSCR: Schur FGMRES(scaled BFBt) / A11 FGMRES + GMG (SOR 1+1)", "rel_residual": res},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                            "sample": f"{args.cpu_nel}^3 elements, {n} points, full step per iteration"},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)
    return 0


# ------------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------------
def train_learned(U, W, args, local, skw):
    """The U-Net of the mixed+learned form (4 levels, 16/32/64/128 channels), trained on the GPU with
    the library's own kernels on residual/error pairs of plain multigrid solves of the same workload
    family on a smaller mesh (args.learn_nel^3); its weights then serve the benchmark's mesh (the
    network is convolutional, so the same parameters apply on any grid).  Outside the timed region."""
    t0 = time.perf_counter()
    wt = make_workload(args.workload, args.learn_nel)
    with U.Context(local) as tctx:
        W.setup_context(tctx, wt)
        tctx.bin_and_map(want=False)
        tctx.assemble()
        kw = dict(skw)
        kw["mg_levels"] = max(2, kw["mg_levels"] - 1)
        opts = U.default_opts(precision=U.PREC_FP64, **kw)
        tctx.learned_create(levels=4, base=16, seed=1)
        t1 = time.perf_counter()
        tctx.learned_generate(opts, nsamples=12 * args.learn_rhs, seed=7)
        t2 = time.perf_counter()
        loss, hold = tctx.learned_train(epochs=args.learn_epochs, batch=8, lr=1e-3, seed=2)
        t3 = time.perf_counter()
        params = tctx.learned_params()
    return params, {"network": "3D U-Net, 4 levels, 16/32/64/128 channels", "parameters": int(params.size),
                    "trained_on": f"{workload_name(args.workload, args.learn_nel)}",
                    "pairs": 12 * args.learn_rhs, "multigrid_solves": args.learn_rhs, "epochs": args.learn_epochs,
                    "train_loss": loss, "holdout_error_ratio": hold,
                    "generate_s": t2 - t1, "train_s": t3 - t2, "total_s": time.perf_counter() - t0}


def run_ours(args):
    import numpy as np
    import torch

    from earthbyte_underworld_gb300 import uwgpu as U
    from earthbyte_underworld_gb300 import workloads as W

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    dist = Dist(world, local)
    nel = args.nel or default_nel(args.workload)
    w = make_workload(args.workload, nel)
    npts = w["x"].shape[0]
    skw = solve_kw(w)
    ctx = U.Context(local)
    W.setup_context(ctx, w)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", local))
    flush_buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")  # 256 MB > L2

    def opts_for(prec, learned=False):
        o = U.default_opts(precision=U.PREC_MIXED if prec != "fp64" else U.PREC_FP64, **skw)
        if learned:
            o.learned_pc = 1
            o.learned_stagnation = 2
        return o

    def use_assembly(prec):
        # the mixed forms contract the element moments on the tensor core (FP64-accurate FP16
        # slices); the FP64 drop-in keeps the FP64 contraction
        ctx.assembly_set(U.ASSEMBLY_TENSOR if prec != "fp64" else U.ASSEMBLY_FP64)

    def step(opts):
        ctx.bin_and_map(want=False)
        ctx.assemble()
        _, _, rep = ctx.solve_bsscr(opts, want=False)
        return rep

    def timed(opts, profile, warmup=None, steps=None):
        nsteps = args.steps if steps is None else steps
        for _ in range(args.warmup if warmup is None else warmup):
            step(opts)
        torch.cuda.synchronize()
        dist.barrier()
        torch.cuda.synchronize()
        if profile:
            ctx.profile_enable(True)
        launches0 = ctx.launch_count()
        clocks = ClockSampler(local)
        clocks.start()
        ev = []
        reps = []
        wall0 = time.perf_counter()
        for _ in range(nsteps):
            flush_buf.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            reps.append(step(opts))
            e1.record(stream)
            ev.append((e0, e1))
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
        clk = clocks.stop()
        dist.barrier()
        torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in ev)
        launches = ctx.launch_count() - launches0
        prof = {}
        if profile:
            for name, fam in (("assembly", U.KERNEL_ASSEMBLY), ("apply", U.KERNEL_APPLY),
                              ("smooth", U.KERNEL_SMOOTH), ("binning", U.KERNEL_BINNING),
                              ("schur_pc", U.KERNEL_SCHUR_PC), ("vector", U.KERNEL_VECTOR),
                              ("transfer", U.KERNEL_TRANSFER), ("learned", U.KERNEL_LEARNED),
                              ("setup", U.KERNEL_SETUP)):
                n, t = ctx.profile_read(fam)
                b, f = ctx.profile_work(fam)
                prof[name] = {"launches": n, "ms": t, "bytes": b, "flops": f}
            ctx.profile_enable(False)
        return ms, wall, launches, reps, clk, prof

    def leg_summary(name, ms, reps, clk, prof):
        r = reps[-1]
        return {"form": name, "value": dist.sum(npts) / (dist.max(ms) / 1e3 / args.steps),
                "ms_per_step": dist.max(ms) / args.steps, "stokes_solve_s": r.t_solve_ms / 1e3,
                "setup_ms": r.t_setup_ms, "rel_residual": r.rel_residual, "outer_its": r.outer_its,
                "inner_its": r.inner_its_total, "vcycles": r.vcycles, "pc_inner_its": r.pc_inner_its,
                "learned_applies": r.learned_applies, "learned_fallbacks": r.learned_fallbacks, "clocks": clk,
                "kernels": {k: {"launches": v["launches"], "ms": v["ms"]} for k, v in prof.items()}}

    prec = args.precision
    # The timed head is the precision form asked for (the mixed form by default).  The metric's
    # mixed+learned form (the U-Net correction inside the velocity solves) is timed beside it in
    # `comparison`, with the FP64 form; at this size the correction does not pay for itself (its
    # leg reports by how much), so the head stays the faster form without it.
    learned = prec == "mixed" and not args.no_learned
    learn_info = None
    if learned:
        params, learn_info = train_learned(U, W, args, local, skw)
        ctx.learned_create(levels=4, base=16, seed=1)
        ctx.learned_set_params(params)
    head = prec
    use_assembly(head)
    head_opts = opts_for(head)
    ms, wall, launches, reps, clk, _ = timed(head_opts, profile=False)
    # One more step of the same workload with every launch of the profiled kernel families
    # bracketed by CUDA events on the library stream: the per-family times and the roofline come
    # from it (the events add host work, so the timed steps above run without them).
    _, _, _, _, _, prof = timed(head_opts, profile=True, warmup=0, steps=1)
    ms_max = dist.max(ms)
    step_ms = ms_max / args.steps
    value = dist.sum(npts) / (ms_max / 1e3 / args.steps)
    rep = reps[-1]

    # the dominant kernel family of the step (profiled extra step); its roofline is given below
    # for the family's fine-level kernel timed alone (after the kernel rates are measured)
    peak, peak_kind = measured_peaks()
    dom = max((k for k in prof if prof[k]["bytes"] > 0), key=lambda k: prof[k]["ms"])
    d = prof[dom]
    family = {"name": dom, "share_of_step": d["ms"] / max(sum(v["ms"] for v in prof.values()), 1e-9),
              "launches": d["launches"], "ms": d["ms"],
              "achieved_GB_per_s": d["bytes"] / (d["ms"] / 1e3) / 1e9 if d["ms"] > 0 else 0.0,
              "fp_TFLOP_per_s": d["flops"] / (d["ms"] / 1e3) / 1e12 if d["ms"] > 0 else 0.0,
              "note": FAMILY_NOTES.get(dom, "")}
    kernels = {k: {"launches": v["launches"], "ms": v["ms"],
                   "GB_per_s": v["bytes"] / (v["ms"] / 1e3) / 1e9 if v["ms"] > 0 else None,
                   "TFLOP_per_s": v["flops"] / (v["ms"] / 1e3) / 1e12 if v["ms"] > 0 else None}
               for k, v in prof.items()}

    # assembly (rheology + moments + contraction into K_e, f_e, G_e, S_e) in both forms: points
    # assembled per second and the algorithmic bytes against HBM, with the FP64 rate beside it
    def assembly_rates(prec_form):
        use_assembly(prec_form)
        ctx.bin_and_map(want=False)
        for _ in range(2):
            ctx.assemble()
        ctx.profile_enable(True)
        for _ in range(3):
            ctx.assemble()
        n, t = ctx.profile_read(U.KERNEL_ASSEMBLY)
        b, f = ctx.profile_work(U.KERNEL_ASSEMBLY)
        ctx.profile_enable(False)
        ms_a = t / 3
        return {"contraction": "tensor core (tcgen05, FP16 slices, FP64-accurate)" if prec_form != "fp64" else
                "FP64 CUDA cores", "ms": ms_a, "points_per_s": npts / (ms_a / 1e3),
                "GB_per_s": b / 3 / (ms_a / 1e3) / 1e9, "frac_hbm": b / 3 / (ms_a / 1e3) / 1e9 / peak,
                "fp64_TFLOP_per_s": f / 3 / (ms_a / 1e3) / 1e12, "launches_per_assembly": n / 3}
    assembly = {"tensor": assembly_rates("mixed"), "fp64": assembly_rates("fp64"),
                "note": f"algorithmic bytes: points read (xi, material, inputs), viscosity written, packed K_e, "
                        f"f_e, G_e, S_e written (and the 27 moments written and read back in the tensor form); "
                        f"FP64 work is bounded by the {FP64_TFLOPS} TFLOP/s FP64 rate of this part"}

    # the other forms on the same inputs, and the distance between the solutions
    comparison = {}
    if not args.no_compare:
        others = ["mixed+learned", "fp64"] if learned else (["fp64"] if prec == "mixed" else ["mixed"])
        sols = {}
        for other in others:
            use_assembly(other)
            o_opts = opts_for(other, learned=other == "mixed+learned")
            ms2, wall2, l2, reps2, clk2, _ = timed(o_opts, profile=False, warmup=1)
            _, _, _, _, _, prof2 = timed(o_opts, profile=True, warmup=0, steps=1)
            comparison[other] = leg_summary(other, ms2, reps2, clk2, prof2)
            comparison[other][f"step_speedup_of_{head}"] = (dist.max(ms2) / args.steps) / step_ms
            comparison[other][f"solve_speedup_of_{head}"] = reps2[-1].t_solve_ms / rep.t_solve_ms
            sols[other] = ctx.solve_bsscr(o_opts, want=True)[:2]
        if "mixed+learned" in comparison and "fp64" in comparison:
            ml, f64 = comparison["mixed+learned"], comparison["fp64"]
            ml["step_speedup_vs_fp64"] = f64["ms_per_step"] / ml["ms_per_step"]
            ml["solve_speedup_vs_fp64"] = f64["stokes_solve_s"] / ml["stokes_solve_s"]
        use_assembly(head)
        ua, pa, _ = ctx.solve_bsscr(head_opts, want=True)
        for other, (ub, pb) in sols.items():
            comparison[other][f"{head}_u_rel_diff"] = float(np.linalg.norm(ua - ub) / np.linalg.norm(ub))
            comparison[other][f"{head}_p_rel_diff"] = float(np.linalg.norm(pa - pb) / np.linalg.norm(pb))

    # end to end through the public API with host buffers (pinned)
    use_assembly(head)
    xs = torch.from_numpy(w["x"]).pin_memory().numpy()
    ys = torch.from_numpy(w["y"]).pin_memory().numpy()
    zs = torch.from_numpy(w["z"]).pin_memory().numpy()
    ms_ = torch.from_numpy(w["material"]).pin_memory().numpy()
    pe = torch.from_numpy(w["eta"]).pin_memory().numpy() if w.get("eta") is not None else None
    pr = torch.from_numpy(w["rho"]).pin_memory().numpy() if w.get("rho") is not None else None
    nn = ctx.nnodes
    ne = ctx.nelements
    e2e_times = []
    e2e_warm = 1  # the context is warm from the legs above
    for it in range(0 if args.no_e2e else e2e_warm + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.particles_upload(xs, ys, zs, ms_, pe, pr)
        ctx.bin_and_map(want=False)
        ctx.assemble()
        u, p, _ = ctx.solve_bsscr(head_opts, want=True)
        torch.cuda.synchronize()
        if it >= e2e_warm:
            e2e_times.append(time.perf_counter() - t0)
    e2e_s = dist.max(sum(e2e_times)) if e2e_times else float("nan")
    e2e = {"value": dist.sum(npts) / (e2e_s / args.steps), "unit": UNIT,
           "h2d_bytes_per_step": int(npts * (3 * 8 + 4 + (8 if pe is not None else 0) + (8 if pr is not None else 0))),
           "d2h_bytes_per_step": int(nn * 3 * 8 + ne * 8)}

    operator_rates = kernel_rates(ctx, U, args.iters)
    roofline = fine_roofline(dom if dom in FINE_KERNEL else "schur_pc", "mixed" if prec != "fp64" else "fp64",
                             operator_rates, nel, peak, peak_kind, family)

    cpu = None
    same_size = None
    if rank == 0 and not args.no_cpu:
        try:
            cpu = cpu_baseline(args.workload, args.cpu_nel, os.cpu_count() or 1)
            cpu1 = cpu_baseline(args.workload, args.cpu_nel, 1)
            cpu["single_thread"] = {"value": cpu1["value"], "cores": 1, "step_s": cpu1["step_s"]}
        except Exception as ex:  # the baseline is reported, never required
            cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "sample": f"failed: {ex}"}
        same_size = gpu_at_cpu_size(U, W, args, local, skw)

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64" if prec == "fp64" else "f32/f64 (bf16/fp16 tensor-core parts)",
               "data": "synthetic",
               "config": {"workload": workload_name(args.workload, nel), "elements": ne,
                          "points": npts, "precision": head, "mg_levels": skw["mg_levels"],
                          "solver": "BSSCR: Schur FGMRES(scaled BFBt) / A11 FGMRES + GMG (Chebyshev block-Jacobi, degree 2+2)",
                          "target_rel_residual": 1e-6, "rel_residual": rep.rel_residual,
                          "outer_its": rep.outer_its, "inner_its": rep.inner_its_total, "vcycles": rep.vcycles,
                          "pc_inner_its": rep.pc_inner_its, "learned_applies": rep.learned_applies,
                          "learned_fallbacks": rep.learned_fallbacks,
                          "stokes_solve_s": rep.t_solve_ms / 1e3, "setup_ms": rep.t_setup_ms,
                          "l2": "256 MB buffer written between timed steps", "parallelism": f"replicas x{world}"},
               "roofline": roofline, "assembly": assembly, "kernels": kernels, "operator": operator_rates,
               "learned": learn_info, "cpu_baseline": cpu, "gpu_at_cpu_sample_size": same_size, "e2e": e2e,
               "gpu_launches": int(launches), "clocks": clk, "comparison": comparison,
               "wall_s_timed": wall}
        print(json.dumps(out), flush=True)
    ctx.close()
    dist.close()
    return 0


def gpu_at_cpu_size(U, W, args, local, skw):
    """This library on the CPU baseline's sample (same workload generator and mesh, FP64 and mixed,
    same solver options as the CPU leg): the same-configuration GPU/CPU comparison."""
    import torch
    w = make_workload(args.workload, args.cpu_nel)
    npts = w["x"].shape[0]
    out = {"workload": workload_name(args.workload, args.cpu_nel), "points": npts}
    kw = dict(SOLVE_KW)
    kw["mg_levels"] = 3 if args.cpu_nel % 4 == 0 else 2
    with U.Context(local) as c:
        W.setup_context(c, w)
        for prec in ("fp64", "mixed"):
            c.assembly_set(U.ASSEMBLY_TENSOR if prec == "mixed" else U.ASSEMBLY_FP64)
            opts = U.default_opts(precision=U.PREC_MIXED if prec == "mixed" else U.PREC_FP64, **kw)
            for _ in range(2):
                c.bin_and_map(want=False)
                c.assemble()
                c.solve_bsscr(opts, want=False)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            steps = 5
            for _ in range(steps):
                c.bin_and_map(want=False)
                c.assemble()
                c.solve_bsscr(opts, want=False)
            c.synchronize()
            dt = (time.perf_counter() - t0) / steps
            out[prec] = {"value": npts / dt, "unit": UNIT, "ms_per_step": 1e3 * dt}
    return out


# DRAM traffic (ncu dram__bytes_read.sum + dram__bytes_write.sum) of one fine-level launch, from the
# captures summarised in profiles/ (command lines there), with the node (or element) count of the
# captured mesh; scaled in proportion for other meshes, as the traffic of these kernels grows with it.
MEASURED_TRAFFIC = {
    ("cheb_step", "fp64"): (588.15e6, 65 ** 3),
    ("apply", "fp64"): (539.1e6, 65 ** 3),
    ("apply", "fp32"): (275.66e6, 65 ** 3),
    ("bfbt_dir", "fp32_matrix_free"): (34.80e6, 128 ** 3),   # k_cg_mf3_dir_tma, profiles/bfbt_mf_tma_fp32_grf128.md
}
FINE_KERNEL = {"smooth": ("cheb_step", "k_cheb_step<3,{t}> (one Chebyshev step, fine level)"),
               "apply": ("apply", "k_apply<3,{t}> (fine level)"),
               "schur_pc": ("bfbt_dir", "{bfbt} (BFBt inner-CG direction kernel, fine level)")}


def fine_roofline(dom, prec, rates, nel, peak, peak_kind, family):
    """Roofline of the dominant family's fine-level kernel, timed alone with CUDA events on the
    library stream (bench --mode kernels numbers): achieved = algorithmic bytes / launch time."""
    p = "fp64" if prec == "fp64" else "fp32"
    r = rates[p]
    key, label = FINE_KERNEL.get(dom, ("cheb_step", "k_cheb_step<3,{t}> (one Chebyshev step, fine level)"))
    ms = r[key + "_ms"]
    gbs = r[key + "_GB_per_s"]
    tkey = (key, r.get("bfbt_form", p)) if key == "bfbt_dir" else (key, p)
    traffic = MEASURED_TRAFFIC.get(tkey)
    if traffic is not None:
        count = nel ** 3 if key == "bfbt_dir" else (nel + 1) ** 3
        traffic = traffic[0] * count / traffic[1]
    return {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak if peak else None,
            "traffic": traffic, "kernel": label.format(t="double" if p == "fp64" else "float", bfbt=r.get("bfbt_kernel", "")),
            "avg_launch_us": 1e3 * ms, "algorithmic_bytes_per_launch": gbs * 1e6 * ms,
            "fp_tflops": r[key + "_fp_TFLOP_per_s"],
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback 6.8 TB/s",
            "traffic_source": "ncu capture (profiles/), scaled by nodes / elements" if traffic is not None else None,
            "note": ("the matrix-free kernel is bound by instruction issue and latency (ncu: 58% issue active at 24 warps "
                     "per SM, DRAM 20%); it "
                     "replaces an HBM-bound stencil kernel that moves five times the bytes"
                     if r.get("bfbt_form") == "fp32_matrix_free" and key == "bfbt_dir" else
                     "FP64 kernels on this part are also bounded by its 1.2 TFLOP/s FP64 rate (fp_tflops)"),
            "family": family}


def kernel_rates(ctx, U, iters):
    """Fine-level operator apply and smoother, timed back to back on resident vectors, with their
    algorithmic bytes (stencil 3^d blocks of d x d, diagonal inverse, right-hand side and the
    row vectors moved once per node)."""
    nn, dim = ctx.nnodes, ctx.dim
    nb = 27 if dim == 3 else 9
    peak, kind = measured_peaks()
    out = {}
    ctx.smoother_storage_set(32)
    for name, prec, size in (("fp64", U.PREC_FP64, 8), ("fp32", U.PREC_MIXED, 4)):
        ctx.time_apply(prec, 3)
        ms = ctx.time_apply(prec, iters) / iters
        apply_bytes = nn * (nb * dim * dim + 2 * dim) * size
        ctx.time_smooth(prec, 2, 2)
        sms = ctx.time_smooth(prec, 2, max(iters // 4, 2)) / max(iters // 4, 2)
        smooth_bytes = 2 * 2 * nn * (nb * dim * dim + dim * dim + 3 * dim) * size + nn * dim * size
        # Chebyshev steps (the benchmark's smoother), each a full pass from the current iterate:
        # stencil, diagonal-block inverse, rhs, iterate in / out and direction in / out once per node
        ctx.time_chebyshev(prec, 2, 2)
        nsteps = 2 * max(iters // 2, 2)
        cms = ctx.time_chebyshev(prec, 2, nsteps // 2) / nsteps
        cheb_bytes = nn * (nb * dim * dim + dim * dim + 6 * dim) * size
        out.setdefault(name, {})
        out[name].update({"cheb_step_ms": cms, "cheb_step_GB_per_s": cheb_bytes / cms / 1e6,
                          "cheb_step_frac_hbm": cheb_bytes / cms / 1e6 / peak,
                          "cheb_step_bytes": cheb_bytes,
                          "cheb_step_fp_TFLOP_per_s": 2.0 * nn * (nb + 1) * dim * dim / cms / 1e9})
        out[name].update({"apply_ms": ms, "applies_per_s": 1e3 / ms, "apply_GB_per_s": apply_bytes / ms / 1e6,
                     "apply_frac_hbm": apply_bytes / ms / 1e6 / peak,
                     "apply_fp_TFLOP_per_s": 2.0 * nn * nb * dim * dim / ms / 1e9,
                     "smooth2_ms": sms, "smooth2_GB_per_s": smooth_bytes / sms / 1e6,
                     "smooth2_frac_hbm": smooth_bytes / sms / 1e6 / peak,
                     "smooth2_fp_TFLOP_per_s": 2 * 2 * 2.0 * nn * (nb + 1) * dim * dim / sms / 1e9})
    # the mixed form's default smoother storage: FP16 row-scaled stencils, neighbour pairs packed in
    # 32-bit words (14 pair words per 3x3 block position in 3D), plus one FP32 row scale per row
    ctx.smoother_storage_set(16)
    ctx.time_chebyshev(U.PREC_MIXED, 2, 2)
    nsteps = 2 * max(iters // 2, 2)
    cms = ctx.time_chebyshev(U.PREC_MIXED, 2, nsteps // 2) / nsteps
    cheb_bytes = nn * (((nb + 1) // 2) * dim * dim * 4 + dim * dim * 4 + 7 * dim * 4)
    out["fp16_stencil"] = {"cheb_step_ms": cms, "cheb_step_GB_per_s": cheb_bytes / cms / 1e6,
                           "cheb_step_frac_hbm": cheb_bytes / cms / 1e6 / peak, "cheb_step_bytes": cheb_bytes,
                           "cheb_step_fp_TFLOP_per_s": 2.0 * nn * (nb + 1) * dim * dim / cms / 1e9}
    # the scaled BFBt inner operator (one value per element): the CG's direction kernel with p = z,
    # q = A z; algorithmic bytes: z read and p, q written, plus the 3^d stencil coefficients
    # (stencil forms) or the nodal W of about one node per element (matrix-free FP32 form).  The
    # "fp32" entry is the form the mixed solve uses on this mesh (the stencil while it and the CG
    # vectors fit in half of L2), the other FP32 form is listed beside it.
    import torch
    ne = ctx.nelements
    l2 = torch.cuda.get_device_properties(torch.cuda.current_device()).L2_cache_size
    mf = ne * 4.0 * (nb + 6) > 0.5 * l2
    mf3 = "k_cg_mf3_dir_tma (planes staged by TMA)" if ctx.nel[0] % 4 == 0 else "k_cg_mf3_dir"
    fp32_mf = ("fp32_matrix_free", 1, (dim + 3) * 4, mf3 if dim == 3 else "k_cg_mf2_dir")
    fp32_st = ("fp32_stencil", 2, (nb + 3) * 4, f"k_cg_spmv_dir<{dim},float>")
    forms = (("fp64", ("fp64_stencil", 0, (nb + 3) * 8, f"k_cg_spmv_dir<{dim},double>")),
             ("fp32", fp32_mf if mf else fp32_st), ("fp32_other", fp32_st if mf else fp32_mf))
    for name, (fname, form, per_elem, kname) in forms:
        ctx.time_bfbt_apply(form, 3)
        bms = ctx.time_bfbt_apply(form, iters) / iters
        gbs = ne * per_elem / bms / 1e6
        out.setdefault(name, {}).update({"bfbt_form": fname, "bfbt_kernel": kname, "bfbt_dir_ms": bms,
                                         "bfbt_dir_GB_per_s": gbs, "bfbt_dir_frac_hbm": gbs / peak,
                                         "bfbt_dir_bytes": ne * per_elem,
                                         "bfbt_dir_fp_TFLOP_per_s": ne * (45.0 if form == 1 else 2.0 * nb) / bms / 1e9})
    out["peak_GB_per_s"] = peak
    out["peak_source"] = kind
    return out


def run_kernels(args):
    import torch

    from earthbyte_underworld_gb300 import uwgpu as U
    from earthbyte_underworld_gb300 import workloads as W
    nel = args.nel or default_nel(args.workload)
    w = make_workload(args.workload, nel)
    with U.Context(0) as ctx:
        W.setup_context(ctx, w)
        ctx.bin_and_map(want=False)
        ctx.assemble()
        rates = kernel_rates(ctx, U, args.iters)
    torch.cuda.synchronize()
    print(json.dumps({"mode": "kernels", "workload": workload_name(args.workload, nel),
                      "nodes": (nel + 1) ** 3, **rates}), flush=True)
    return 0


def run_bfbt(args):
    """The scaled BFBt inner operator's kernel in its three forms (FP64 stencil, FP32 matrix-free,
    FP32 stencil) on a GRF-viscosity mesh of nel^3 elements (4 points per element: the operator
    depends on the viscosity field, not on the point count), timed back to back with CUDA events."""
    import numpy as np
    import torch

    from earthbyte_underworld_gb300 import uwgpu as U
    from earthbyte_underworld_gb300 import workloads as W
    n = args.nel or 128
    w = W.grf(nel=(n, n, n), ppc=4, grid=64, corr=0.1)
    out = {"mode": "bfbt", "workload": f"grf_{n}cube_4ppc", "elements": n ** 3}
    peak, kind = measured_peaks()
    with U.Context(0) as ctx:
        W.setup_context(ctx, w)
        ctx.bin_and_map(want=False)
        ctx.assemble()
        ctx.operator_apply(np.zeros(ctx.nnodes * 3))
        for name, form, per_elem in (("fp64_stencil", 0, 30 * 8), ("fp32_matrix_free", 1, 6 * 4),
                                     ("fp32_stencil", 2, 30 * 4)):
            ctx.time_bfbt_apply(form, 3)
            ms = ctx.time_bfbt_apply(form, args.iters) / args.iters
            gbs = n ** 3 * per_elem / ms / 1e6
            out[name] = {"us": 1e3 * ms, "algorithmic_bytes": n ** 3 * per_elem, "GB_per_s": gbs,
                         "frac_hbm": gbs / peak}
    torch.cuda.synchronize()
    out["peak_GB_per_s"] = peak
    out["peak_source"] = kind
    print(json.dumps(out), flush=True)
    return 0


def run_accuracy(args):
    """Accuracy at equal cost: a converged FP64 solve of the workload (Schur 1e-10, velocity 1e-11)
    is the reference; the mixed and FP64 forms are then solved on a ladder of tolerances (Schur,
    velocity), each timed once after a warm-up, with the relative L2 distance of u and p from the
    reference.  For each form the first rung whose velocity is within 1e-6 of the reference gives
    its time at that accuracy; the line states both and their ratio."""
    import numpy as np
    import torch

    from earthbyte_underworld_gb300 import uwgpu as U
    from earthbyte_underworld_gb300 import workloads as W
    nel = args.nel or default_nel(args.workload)
    w = make_workload(args.workload, nel)
    kw = solve_kw(w)
    ctx = U.Context(0)
    W.setup_context(ctx, w)
    ctx.bin_and_map(want=False)
    ctx.assemble()
    t0 = time.perf_counter()
    ref_opts = U.default_opts(precision=U.PREC_FP64, **dict(kw, scr_rtol=1e-10, a11_rtol=1e-11, back_rtol=1e-11,
                                                           max_outer=2000, max_inner=20000))
    ur, pr, rr = ctx.solve_bsscr(ref_opts)
    t_ref = time.perf_counter() - t0
    ladder = [(1e-6, 5e-7), (1e-7, 5e-8), (3e-8, 1.5e-8), (1e-8, 5e-9)]
    out = {"mode": "accuracy", "workload": workload_name(args.workload, nel), "target_u_rel": 1e-6,
           "reference": {"rel_residual": rr.rel_residual, "outer_its": rr.outer_its, "s": t_ref}, "forms": {}}
    ctx.solve_bsscr(U.default_opts(precision=U.PREC_MIXED, **kw))   # warm-up
    for name, prec in (("mixed", U.PREC_MIXED), ("fp64", U.PREC_FP64)):
        rows = []
        for scr, a11 in ladder:
            o = U.default_opts(precision=prec, **dict(kw, scr_rtol=scr, a11_rtol=a11, back_rtol=a11 / 5,
                                                      max_outer=2000, max_inner=20000))
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            u, p, r = ctx.solve_bsscr(o)
            dt = time.perf_counter() - t1
            rows.append({"scr_rtol": scr, "a11_rtol": a11, "s": dt, "rel_residual": r.rel_residual,
                         "outer_its": r.outer_its,
                         "u_rel": float(np.linalg.norm(u - ur) / np.linalg.norm(ur)),
                         "p_rel": float(np.linalg.norm(p - pr) / np.linalg.norm(pr))})
            if rows[-1]["u_rel"] <= 1e-6:
                break
        hit = [r for r in rows if r["u_rel"] <= 1e-6]
        out["forms"][name] = {"ladder": rows, "s_at_target": hit[0]["s"] if hit else None}
    m, f = out["forms"]["mixed"]["s_at_target"], out["forms"]["fp64"]["s_at_target"]
    out["speedup_at_equal_accuracy"] = f / m if m and f else None
    print(json.dumps(out), flush=True)
    ctx.close()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.mode == "bfbt":
        return run_bfbt(args)
    if args.mode == "kernels":
        return run_kernels(args)
    if args.mode == "accuracy":
        return run_accuracy(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
