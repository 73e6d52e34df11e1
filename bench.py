#!/usr/bin/env python
"""Benchmark: nonlinear P1-tet magnetostatic Newton solves/s at 96^3 cells.

Workload (one "step" = one full Newton solve from the initial guess to update norm
<= 1e-8): the Kuhn-tet box [-5,5]^3 with 96^3 cells (5,308,416 tets, 912,673 nodes),
interior nodes jittered +-0.1h (seeded), Froehlich plate [-1,1]x[-0.5,0.5]x[-0.25,0.25]
(Ms = 1.2e6 A/m, Hk = 500 A/m), air elsewhere, Dirichlet phi = -H0.x with
H0 = (8e4, 0, 0) A/m on the box surface.  Synthetic inputs; the reference publishes
no dataset for this path.

value: solves/s of the mixed path (FP32 operator and CG, FP64 residual/update/Newton),
timed with CUDA events on the library's stream, inputs resident in HBM.
fp64: the same solve with an FP64 inner CG (the plain FP64 GPU path).
e2e: the one-shot C-ABI call fg_scalar_potential_newton from pinned host buffers
(mesh upload, pattern build, solve, download of u/H/mu inside the timed region).
cpu_baseline / accuracy_vs_oracle: one full Newton solve of the CPU restatement of
the reference algorithm (oracle port, FP64, all host threads, the same Newton
settings), timed, and its u, H and magnetic energy as the FP64 reference for both
GPU solves.
--impl reference: the same full oracle solve(s), timed, as the reference arm.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import tempfile
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "femeko.jl_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "P1-tet magnetostatic solves/s @900k nodes, H err<=1e-8: mixed vs FP64 GPU"
UNIT = "solves/s"
SEED = 20261203
MS, HK = 1.2e6, 500.0
H0 = np.array([8e4, 0.0, 0.0])


def workload(cells: int):
    from femeko_gpu.mesh import MU0, box_tet_mesh
    mesh = box_tet_mesh(cells, seed=SEED)
    nl = (mesh.elementID == 2).astype(np.uint8)
    mu_lin = np.full(mesh.nt, MU0)
    u0 = -(H0[:, None] * mesh.p).sum(axis=0)
    return mesh, nl, mu_lin, u0


def config(cells, mesh):
    return {"workload": f"nonlinear Froehlich-plate magnetostatics, Kuhn tets {cells}^3 cells",
            "cells": cells, "tets": int(mesh.nt), "nodes": int(mesh.nv), "newton_tol_update": 1e-8,
            "inner_tolerance": "Eisenstat-Walker (choice 2, gamma 0.9) in [1e-2, 0.3], both precisions",
            "line_search": "alpha = 0.9^k backtracking on the nonlinear residual",
            "l2": "inputs larger than L2 (operator, records and element state ~2 GB)"}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def replica_seconds(local_sec: float, device: str = "cuda") -> float:
    """The job's timed seconds with one independent replica per GPU: the maximum over
    the ranks (the job ends with its slowest replica); the local value alone."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return local_sec
    import torch
    t = torch.tensor([local_sec], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world_size: int, steps: int, seconds: float) -> float:
    """Whole-job solves/s: every replica runs `steps` solves in at most `seconds`."""
    return world_size * steps / seconds


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, dev: int = 0):
        self.dev = dev
        self.proc = None
        # raw samples go to FG_CLOCKS_DIR (default: the system temporary folder); the
        # JSON line carries their summary
        self.path = os.path.join(os.environ.get("FG_CLOCKS_DIR", tempfile.gettempdir()),
                                 f"fg_clocks_{os.getpid()}.csv")

    def __enter__(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={q}", "--format=csv",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path).read().splitlines()[1:]:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1].split()[0]))
                mx.append(float(parts[2].split()[0]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        busy = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(busy), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the platform string)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


# The Newton settings both the GPU path and the oracle run: Eisenstat-Walker inner
# tolerances (choice 2, gamma 0.9) in [1e-2, 0.3], two Picard (secant) steps, alpha =
# 0.9^k backtracking on the true nonlinear residual, stop at |alpha du| <= 1e-8 |u|.
NEWTON_SETTINGS = dict(tol_update=1e-8, line_search="residual", forcing="ew", eta_min=1e-2, eta_max=0.3,
                       picard_steps=2)


def cpu_full_solve(mesh, nl, mu_lin, u0, threads):
    """One full FP64 Newton solve of the oracle port (the reference algorithm of
    Magnetostatics/NewtonRaphson.jl:109-214 with its per-iteration sparse assembly),
    wall-clock timed on `threads` OpenMP threads.  Returns (u, H, mu, stats, seconds)."""
    import oracle as O
    O.set_threads(threads)
    t0 = time.perf_counter()
    u, H, mu, st = O.newton(mesh, u0, nl, mu_lin, MS, HK, **NEWTON_SETTINGS)
    sec = time.perf_counter() - t0
    if not st["converged"]:
        raise RuntimeError(f"oracle Newton did not converge: {st}")
    return u, H, mu, st, sec


def oracle_energy(mesh, H, nl, mu_lin):
    import oracle as O
    return O.energy(mesh, H, nl, mu_lin, MS, HK)


def run_reference(args):
    ws, rank = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    mesh, nl, mu_lin, u0 = workload(args.cells)
    # warm-up: the same solve on the 24^3-cell plate (loads the library, starts the
    # OpenMP threads, faults in the allocator); a CPU solve keeps no other state
    wmesh, wnl, wmu, wu0 = workload(24)
    cpu_full_solve(wmesh, wnl, wmu, wu0, threads)
    # timed: full solves of the 96^3 workload; each takes about a minute on 16 cores,
    # so at most --ref-steps of the requested --steps are run (stated on the line)
    nsteps = max(1, min(args.steps, args.ref_steps))
    secs, st = [], None
    for _ in range(nsteps):
        _, _, _, st, sec = cpu_full_solve(mesh, nl, mu_lin, u0, threads)
        secs.append(sec)
    total = sum(secs)
    value = nsteps / total
    sample = (f"{nsteps} full FP64 Newton solve(s) of the oracle port (the reference algorithm, sparse assembly per "
              f"iteration) on the whole {args.cells}^3 workload, measured, not extrapolated: "
              f"{st['newton_iters']} Newton iterations, {st['cg_iters']} PCG iterations per solve")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": nsteps, "steps_requested": args.steps, "warmup": 1,
            "warmup_what": "one full solve of the 24^3-cell plate (same settings)",
            "ms_per_step": 1000.0 * total / nsteps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config(args.cells, mesh),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                             "cpu_model": cpu_model(), "measured": True},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def pinned(shape, dtype):
    import torch
    tdt = {np.float64: torch.float64, np.int32: torch.int32, np.uint8: torch.uint8}[dtype]
    t = torch.empty(shape, dtype=tdt, pin_memory=True)
    return t, t.numpy()


def run_ours(args):
    import torch
    import femeko_gpu as fg
    import femeko_gpu._lib as L

    ws, rank = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dev = torch.cuda.current_device()
    lib = L.lib()
    t0 = time.time()
    mesh, nl, mu_lin, u0 = workload(args.cells)
    t_gen = time.time() - t0
    t0 = time.time()
    g = fg.gpu_mesh(mesh)
    t_setup = time.time() - t0
    if args.cg_variant:
        L.check(lib.fg_set_cg_variant(g.h, L.FG_MIXED, args.cg_variant))
    if args.cg64_variant:
        L.check(lib.fg_set_cg_variant(g.h, L.FG_FP64, args.cg64_variant))

    # inputs uploaded once; each timed step is one Newton solve from them with the
    # results left on the device (downloaded once after the timed region)
    resident = fg.ResidentNewton(mesh, nl, mu_lin, u0)

    def solve(precision):
        st = resident.solve(precision=precision, check_every=args.check_every, use_graph=args.graph_mode)
        if not st["converged"]:
            raise RuntimeError(f"Newton did not converge: {st}")
        return st

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    res = {}
    launches0 = None
    for prec, steps in (("mixed", args.steps), ("fp64", args.fp64_steps)):
        for _ in range(args.warmup):
            solve(prec)
        barrier()
        if prec == "mixed":
            launches0 = lib.fg_kernel_launches()
        ms, stats = [], None
        with Clocks(dev) as clk:
            wall0 = time.time()
            for _ in range(steps):
                stats = solve(prec)
                ms.append(stats["ms"])
            barrier()
            wall = time.time() - wall0
        u, H, mu = resident.outputs()
        if prec == "mixed":
            launches = lib.fg_kernel_launches() - launches0
        tot = replica_seconds(sum(ms) / 1000.0)
        res[prec] = dict(u=u, H=H, mu=mu, stats=stats, sec=tot, wall=wall, steps=steps, clocks=clk.summary())

    Hm, Hd = res["mixed"]["H"], res["fp64"]["H"]
    herr = float(np.linalg.norm(Hm - Hd) / np.linalg.norm(Hd))
    uerr = float(np.linalg.norm(res["mixed"]["u"] - res["fp64"]["u"]) / np.linalg.norm(res["fp64"]["u"]))
    werr = abs(res["mixed"]["stats"]["energy"] - res["fp64"]["stats"]["energy"]) / abs(res["fp64"]["stats"]["energy"])
    value = job_rate(ws, args.steps, res["mixed"]["sec"])
    fp64_value = job_rate(ws, args.fp64_steps, res["fp64"]["sec"])

    # the CG variants the timed solves ran (autotuned at the first solve of the handle)
    used32, used64 = C.c_int32(), C.c_int32()
    L.check(lib.fg_get_cg_variant(g.h, L.FG_MIXED, C.byref(used32)))
    L.check(lib.fg_get_cg_variant(g.h, L.FG_FP64, C.byref(used64)))

    # roofline: dominant kernel = the FP32 CG SpMV on the converged tangent operator
    peak, peak_kind = measured_peaks()
    nsell, ninc, nsl = C.c_int64(), C.c_int64(), C.c_int32()
    lib.fg_mesh_layout(g.h, C.byref(nsell), C.byref(ninc), C.byref(nsl))
    fg.newton_magnetostatics(mesh, nl, mu_lin, u0, precision="mixed")   # leaves J32 on the handle
    chosen = C.c_int32()
    names = ["fused gather/256", "fused gather-hoist/256", "fused gather/128", "fused gather/512",
             "fused halo-smem", "fused halo-smem-pipelined", "split gather/256", "split halo-smem",
             "split gather persistent", "split gather persistent, programmatic launch",
             "split gather persistent 6/SM, values in L2 window", "split gather persistent 4/SM",
             "split gather persistent 3/SM", "split gather persistent 5/SM",
             "split gather persistent 6/SM", "split gather persistent 7/SM",
             "split, Jacobi-scaled system, persistent 6/SM",
             "split, bulk-staged entries, persistent 4/SM", "split, bulk-staged entries, persistent 3/SM",
             "split, bulk-staged entries, persistent 2/SM",
             "split, Jacobi-scaled system, persistent 6/SM, values in L2 window",
             "split, bulk-staged entries, persistent 4/SM, values in L2 window",
             "split, bulk-staged entries, persistent 4/SM, dots finished by a one-block kernel",
             "split, bulk-staged entries, persistent 3/SM, dots finished by a one-block kernel",
             "pipelined CG, bulk-staged SpMV 4/SM, dots finished by one SpMV block (forced only)",
             "pipelined CG, bulk-staged SpMV 3/SM, dots finished by one SpMV block (forced only)",
             "split iteration in one persistent cooperative launch, grid barriers, 4/SM",
             "split, bulk-staged entries, persistent 4/SM, dots finished by the last SpMV block",
             "split, bulk-staged entries, persistent 3/SM, dots finished by the last SpMV block"]
    variants_us = np.zeros(len(names))
    # the table of every variant on the converged operator (a second timing); the
    # per-kernel figures below are for the variant the timed solves used
    L.check(lib.fg_autotune(g.h, L.FG_MIXED, C.byref(chosen), L.ptr(variants_us), len(names)))
    L.check(lib.fg_set_cg_variant(g.h, L.FG_MIXED, used32.value))
    autotune = {"cg32_iteration_variants_us": [round(float(v), 2) for v in variants_us],
                "chosen_on_converged_operator": int(chosen.value), "used_by_timed_solves": int(used32.value) - 1,
                "used64_by_timed_solves": int(used64.value) - 1,
                "names": names}
    ms_spmv, ms_iter = C.c_double(), C.c_double()
    L.check(lib.fg_bench_kernel(g.h, 0, L.FG_MIXED, 200, C.byref(ms_spmv)))
    L.check(lib.fg_bench_kernel(g.h, 3, L.FG_MIXED, 200, C.byref(ms_iter)))
    ms_loop = C.c_double()
    L.check(lib.fg_bench_kernel(g.h, 6, L.FG_MIXED, 256, C.byref(ms_loop)))
    # cg32_iteration: direct launches; cg32_iteration_in_loop: the solver's graph loop
    kernels_us = {"cg32_spmv": ms_spmv.value * 1e3, "cg32_iteration": ms_iter.value * 1e3,
                  "cg32_iteration_in_loop": ms_loop.value * 1e3}
    if int(used32.value) - 1 in (22, 23):
        # the split-reduction variants: 0 timed the SpMV kernel alone; its dot products
        # are added by a one-block kernel launched after it
        ms_fin = C.c_double()
        L.check(lib.fg_bench_kernel(g.h, 9, L.FG_MIXED, 200, C.byref(ms_fin)))
        kernels_us["cg32_dots_finish"] = ms_fin.value * 1e3
    for name, which in (("newton_element_pass_all_f32", 2), ("newton_residual_split", 4),
                        ("newton_residual_jacobian_split_f32", 5)):
        t = C.c_double()
        L.check(lib.fg_bench_kernel(g.h, which, L.FG_MIXED, 20, C.byref(t)))
        kernels_us[name] = t.value * 1e3
    fg.newton_magnetostatics(mesh, nl, mu_lin, u0, precision="fp64")   # leaves J64 on the handle
    ch64, us64 = C.c_int32(), np.zeros(4)
    L.check(lib.fg_autotune(g.h, L.FG_FP64, C.byref(ch64), L.ptr(us64), 4))
    L.check(lib.fg_set_cg_variant(g.h, L.FG_FP64, used64.value))
    autotune["cg64_spmv_variants_us"] = [round(float(v), 2) for v in us64]
    autotune["chosen64_on_converged_operator"] = int(ch64.value)
    for name, which, reps in (("cg64_spmv", 0, 200), ("cg64_update", 1, 200), ("cg64_iteration_in_loop", 6, 256)):
        t = C.c_double()
        L.check(lib.fg_bench_kernel(g.h, which, L.FG_FP64, reps, C.byref(t)))
        kernels_us[name] = t.value * 1e3
    fg.newton_magnetostatics(mesh, nl, mu_lin, u0, precision="mixed")
    # P1 stiffness assembly K(mu) at the converged permeabilities into the FP64 and
    # FP32 operator: the one-pass row gather (7) and the two-pass record form (8)
    t_asm, t_asm2 = C.c_double(), C.c_double()
    L.check(lib.fg_bench_kernel(g.h, 7, L.FG_MIXED, 20, C.byref(t_asm)))
    L.check(lib.fg_bench_kernel(g.h, 8, L.FG_MIXED, 10, C.byref(t_asm2)))
    nt, nv_ = mesh.nt, mesh.nv
    # algorithmic bytes of the reference path's per-element model: per element
    # connectivity (16 B) and permeability (8 B), per node the coordinates (24 B), per
    # stored nonzero the FP64 value written (8 B)
    asm_alg = nt * 24 + nv_ * 24 + g.nnz * 8
    # bytes this design moves (gradients are not recomputed in FP64): per element the
    # 10-entry Gram matrix, volume and permeability (96 B), per incidence its element
    # code and slot bytes (8 B), per stored slot the FP64 and FP32 values (12 B), per
    # row the two Jacobi inverses (12 B)
    asm_design = nt * 96 + ninc.value * 8 + nsell.value * 12 + nv_ * 12
    asm_s = t_asm.value * 1e-3
    assembly = {"kernel": "k_asm_rows_tet4<ASM_STIFF>", "elements_per_s": nt / asm_s, "us": t_asm.value * 1e3,
                "alg_bytes": asm_alg, "achieved_GBs": asm_alg / asm_s / 1e9, "peak": peak,
                "frac": asm_alg / asm_s / 1e9 / peak,
                "design_bytes": asm_design, "design_GBs": asm_design / asm_s / 1e9,
                "design_frac": asm_design / asm_s / 1e9 / peak,
                "two_pass_us": t_asm2.value * 1e3, "speedup_vs_two_pass": t_asm2.value / t_asm.value}
    n = mesh.nv
    v = int(used32.value) - 1
    if v == 26:
        # one launch runs whole iterations: the vector pass (28 B read, 20 B written per
        # row) and w = A u with its dots (6 B per stored nonzero, u and r read, w
        # written: 12 B per row); timed per iteration inside the solver's loop
        alg_bytes = g.nnz * 6 + 60 * n
        kname = "k_cg32_coop"
    elif v in (24, 25):
        # pipelined CG, dominant kernel n = A m: FP32 value and 16-bit column per
        # stored nonzero; per row m read once and n written (8 B); no dot products
        alg_bytes = g.nnz * 6 + 8 * n
        kname = "k_pcg32_spmv_bulk"
    elif v in (16, 20):
        # scaled system: w = A' r with its dots; value + 16-bit column per stored
        # nonzero, r and the diagonal read and w written per row (12 B)
        alg_bytes = g.nnz * 6 + 12 * n
        kname = "k_cg32s_spmv"
    elif v >= 6:
        # split iteration, dominant kernel w = A u with its dots: FP32 value (4 B) and
        # 16-bit column (2 B) per stored nonzero; per row u and r read, w written
        # (12 B).  Neighbour gathers of u are re-reads.
        alg_bytes = g.nnz * 6 + 12 * n
        kname = {7: "k_cg32s_spmv_halo", 17: "k_cg32s_spmv_bulk", 18: "k_cg32s_spmv_bulk",
                 19: "k_cg32s_spmv_bulk", 21: "k_cg32s_spmv_bulk",
                 22: "k_cg32s_spmv_bulk<split>", 23: "k_cg32s_spmv_bulk<split>",
                 27: "k_cg32s_spmv_bulk<split, last-block finish>",
                 28: "k_cg32s_spmv_bulk<split, last-block finish>"}.get(v, "k_cg32s_spmv")
    else:
        # one fused iteration: matrix as above; per row the (r, w, s, dinv) state read
        # and written (16 + 16 B) and p, x read and written (8 + 8 B)
        alg_bytes = g.nnz * 6 + 48 * n
        kname = {4: "k_cg32_iter_halo", 5: "k_cg32_iter_pipe"}.get(v, "k_cg32_iter")
    t_dom = ms_loop.value if v == 26 else ms_spmv.value
    achieved = alg_bytes / (t_dom * 1e-3) / 1e9
    # DRAM bytes per launch of the same kernel from an ncu capture at 96^3: 10 and 20 =
    # the L2-window variants (warm L2), 14 = the grid of 10 without the window, 17 =
    # the bulk-staged SpMV, 22 = its split-reduction form and 27 = the split form whose
    # last block adds the partials (cold); other variants: none captured
    traffic, traffic_src = args.spmv_traffic, "--spmv-traffic" if args.spmv_traffic else None
    if traffic is None and args.cells == 96 and v in (10, 14, 17, 20, 22, 27):
        traffic = {10: 70.73e6, 14: 97.07e6, 17: 97.38e6, 20: 69.70e6, 22: 97.66e6, 27: 97.3e6}[v]
        traffic_src = "ncu dram__bytes_read.sum + dram__bytes_write.sum of this kernel at 96^3"
    # the whole CG iteration in the solver's loop (every kernel of it): the dominant
    # SpMV's bytes plus the vector pass's (split: 24 B read + 20 B written per row, u
    # formed again from r; Jacobi-scaled system: 20 + 16 B; fused: counted in the
    # kernel above)
    if v in (24, 25):
        it_bytes = None
    elif v in (16, 20):
        it_bytes = g.nnz * 6 + 12 * n + 36 * n
    elif v >= 6 and v != 26:
        it_bytes = g.nnz * 6 + 12 * n + 44 * n
    else:
        it_bytes = alg_bytes
    # the last-block-finish variants: their SpMV code without the finishing tail (the
    # split sibling, 22 or 23, whose kernel is the same up to the partials) timed alone
    spmv_part = None
    if v in (27, 28):
        ms_part = C.c_double()
        L.check(lib.fg_set_cg_variant(g.h, L.FG_MIXED, v - 5 + 1))
        L.check(lib.fg_bench_kernel(g.h, 0, L.FG_MIXED, 200, C.byref(ms_part)))
        L.check(lib.fg_set_cg_variant(g.h, L.FG_MIXED, v + 1))
        part_gbs = alg_bytes / (ms_part.value * 1e-3) / 1e9
        spmv_part = {"us_per_launch": ms_part.value * 1e3, "achieved": part_gbs, "frac": part_gbs / peak,
                     "finish_tail_us": (t_dom - ms_part.value) * 1e3,
                     "what": "the same SpMV without its last-block finish (the split variant's kernel), timed alone"}
    it_roof = None
    if it_bytes is not None:
        it_gbs = it_bytes / (ms_loop.value * 1e-3) / 1e9
        it_roof = {"algorithmic_bytes": it_bytes, "us_per_iteration": ms_loop.value * 1e3, "achieved": it_gbs,
                   "frac": it_gbs / peak, "timing": "CG iterations in the solver's graph loop, CUDA events"}
    roofline = {"bound": "hbm", "kernel": kname, "variant": autotune["names"][v],
                "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": traffic, "traffic_source": traffic_src, "algorithmic_bytes": alg_bytes,
                "us_per_launch": t_dom * 1e3,
                "timing": ("one CG iteration of the persistent launch, in the solver's loop" if v == 26
                           else "one launch, CUDA events on the library's stream"),
                "cg_iteration": it_roof, "spmv_without_finish": spmv_part}

    # e2e through the one-shot C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        p_t, p_np = pinned((mesh.nv, 3), np.float64)
        t_t, t_np = pinned((mesh.nt, 4), np.int32)
        p_np[:] = mesh.p.T
        t_np[:] = mesh.t.T
        fx_t, fx_np = pinned((mesh.nv,), np.uint8)
        fx_np[:] = mesh.dirichlet_mask()
        nl_t, nl_np = pinned((mesh.nt,), np.uint8)
        nl_np[:] = nl
        mu_t, mu_np = pinned((mesh.nt,), np.float64)
        mu_np[:] = mu_lin
        u0_t, u0_np = pinned((mesh.nv,), np.float64)
        u0_np[:] = u0
        uo_t, uo_np = pinned((mesh.nv,), np.float64)
        Ho_t, Ho_np = pinned((mesh.nt, 3), np.float64)
        muo_t, muo_np = pinned((mesh.nt,), np.float64)
        o = fg.newton_opts(precision="mixed")
        s = L.NewtonStats()

        def one():
            L.check(lib.fg_scalar_potential_newton(L.ptr(p_np), mesh.nv, L.ptr(t_np), mesh.nt, 0, L.ptr(fx_np),
                                                   L.ptr(nl_np), L.ptr(mu_np), L.ptr(u0_np), C.byref(o),
                                                   L.ptr(uo_np), L.ptr(Ho_np), L.ptr(muo_np), C.byref(s)))
        # at least three untimed calls: the first ones on a fresh process also grow the
        # device's memory pool and the recycled pinned read-back blocks
        for _ in range(max(3, args.warmup)):
            one()
        barrier()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        w0 = time.time()
        ev0.record()
        call_ms, solve_ms = [], []
        for _ in range(args.e2e_steps):
            c0 = time.perf_counter()
            one()
            call_ms.append(1e3 * (time.perf_counter() - c0))
            solve_ms.append(s.ms)
        ev1.record()
        barrier()
        e2e_sec = max(ev0.elapsed_time(ev1) / 1000.0, time.time() - w0)
        h2d = p_np.nbytes + t_np.nbytes + fx_np.nbytes + nl_np.nbytes + mu_np.nbytes + u0_np.nbytes
        d2h = uo_np.nbytes + Ho_np.nbytes + muo_np.nbytes
        # where an end-to-end call's time goes: the same four calls the one-shot entry
        # point makes, each timed on the host after the device is idle (untimed above)
        phases = {}
        hm = C.c_void_p()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        L.check(lib.fg_mesh_create(L.ptr(p_np), mesh.nv, L.ptr(t_np), mesh.nt, 4, 0, C.byref(hm)))
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        L.check(lib.fg_mesh_set_dirichlet(hm, L.ptr(fx_np)))
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        L.check(lib.fg_newton_magnetostatics(hm, L.ptr(nl_np), L.ptr(mu_np), L.ptr(u0_np), C.byref(o), L.ptr(uo_np),
                                             L.ptr(Ho_np), L.ptr(muo_np), C.byref(s)))
        torch.cuda.synchronize()
        t3 = time.perf_counter()
        L.check(lib.fg_mesh_destroy(hm))
        torch.cuda.synchronize()
        t4 = time.perf_counter()
        phases = {"mesh_create_upload_pattern": 1e3 * (t1 - t0), "set_dirichlet": 1e3 * (t2 - t1),
                  "newton_solve_with_io": 1e3 * (t3 - t2), "of_which_newton_device_ms": s.ms,
                  "of_which_newton_setup_ms": s.setup_ms, "destroy": 1e3 * (t4 - t3)}
        e2e = {"value": ws * args.e2e_steps / e2e_sec, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "steps": args.e2e_steps, "warmup": max(3, args.warmup),
               "call_ms": [round(c, 2) for c in call_ms],
               "newton_device_ms": [round(c, 2) for c in solve_ms],
               "what": "fg_scalar_potential_newton: upload + pattern build + solve + download per step",
               "phases_ms_one_call": {k: round(v, 3) for k, v in phases.items()}}

    cpu, acc_oracle = None, None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        uo, Ho, muo, so, sec = cpu_full_solve(mesh, nl, mu_lin, u0, threads)
        Wo = oracle_energy(mesh, Ho, nl, mu_lin)
        acc_oracle = {}
        for prec in ("mixed", "fp64"):
            r = res[prec]
            acc_oracle[prec] = {
                "H_rel": float(np.linalg.norm(r["H"] - Ho) / np.linalg.norm(Ho)),
                "u_rel": float(np.linalg.norm(r["u"] - uo) / np.linalg.norm(uo)),
                "mu_rel_max": float(np.abs(r["mu"] - muo).max() / np.abs(muo).max()),
                "energy_rel": float(abs(r["stats"]["energy"] - Wo) / abs(Wo))}
        acc_oracle["oracle"] = {"newton_iters": so["newton_iters"], "cg_iters": so["cg_iters"], "energy_J": Wo,
                                "settings": "FP64, the same Newton settings as the GPU solves"}
        acc_oracle["H_err_le_1e-8"] = all(acc_oracle[p]["H_rel"] <= 1e-8 for p in ("mixed", "fp64"))
        cpu = {"value": 1.0 / sec, "unit": UNIT, "cores": threads, "kind": "port", "measured": True,
               "cpu_model": cpu_model(),
               "sample": (f"one full FP64 Newton solve of the oracle port on the whole {args.cells}^3 workload "
                          f"({sec:.1f} s wall, {so['newton_iters']} Newton / {so['cg_iters']} PCG iterations, "
                          f"{threads} OpenMP threads), measured, not extrapolated")}

    sm = res["mixed"]["stats"]

    def phases(st):
        # one solve (the last timed one): set-up (linear elements' operator, first
        # residual), inner CG solves, the rest (residuals, line search, Jacobians)
        return {"setup": round(st["setup_ms"], 3), "cg": round(st["cg_ms"], 3),
                "newton_rest": round(st["ms"] - st["setup_ms"] - st["cg_ms"], 3)}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * res["mixed"]["sec"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 operator/CG, f64 residual/update",
            "data": "synthetic", "config": config(args.cells, mesh),
            "fp64": {"value": fp64_value, "unit": UNIT, "ms_per_step": 1000.0 * res["fp64"]["sec"] / args.fp64_steps,
                     "newton_iters": res["fp64"]["stats"]["newton_iters"], "cg_iters": res["fp64"]["stats"]["cg_iters"],
                     "phases_ms": phases(res["fp64"]["stats"])},
            "phases_ms": phases(sm),
            "mixed_over_fp64": value / fp64_value,
            "accuracy_vs_oracle": acc_oracle,
            "accuracy_vs_fp64_gpu": {"H_rel": herr, "u_rel": uerr, "energy_rel": werr},
            "newton_iters": sm["newton_iters"], "cg_iters": sm["cg_iters"], "trials": sm["trials"],
            "roofline": roofline, "assembly": assembly,
            "solved_dof_per_s": {"unknowns_per_s": mesh.nv * value,
                                 "interior_unknown_iterations_per_s":
                                     int((~mesh.dirichlet_mask().astype(bool)).sum()) * sm["cg_iters"] * value},
            "kernels_us": kernels_us, "autotune": autotune, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": int(launches), "cg_variant_fixed": {"mixed": args.cg_variant, "fp64": args.cg64_variant},
            "cg_loop": {"check_every": args.check_every, "graph_mode": args.graph_mode},
            "clocks": res["mixed"]["clocks"], "clocks_fp64": res["fp64"]["clocks"],
            "setup_s": {"mesh_generate": t_gen, "mesh_create_pattern": t_setup},
            "wall_s": {"mixed": res["mixed"]["wall"], "fp64": res["fp64"]["wall"]}}
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


# ---------------------------------------------------------------------------------
# Secondary workloads (--case): the other configurations of the path, each printing
# its own JSON line.  "cg-kernel" and "newton-kernels" are the small drivers the
# profiles under profiles/ were captured with.

def _line(metric, value, unit, higher, config, extra):
    d = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "higher_is_better": higher,
         "data": "synthetic", "config": config}
    d.update(extra)
    print(json.dumps(d))


def case_cg_kernel(args):
    """Forced FP32 CG kernel variant on K + M of the workload mesh, no graph:
    one launch per iteration (the ncu capture target)."""
    import femeko_gpu as fg
    mesh, nl, mu_lin, u0 = workload(args.cells)
    K = (fg.stiffnessMatrix(mesh) + fg.massMatrix(mesh)).tocsc()
    b = np.random.default_rng(1).normal(size=mesh.nv)
    x, st = fg.cg(K, b, reltol=1e-30, maxiter=args.iters, precision="mixed", spmv=args.variant, use_graph=False,
                  return_stats=True)
    _line("CG iteration time (FP32, forced variant)", 1e3 * st["ms"] / max(st["iterations"], 1), "us/iteration",
          False, {"workload": f"K+M of the Kuhn-tet box, {args.cells}^3 cells", "variant": args.variant,
                  "iterations": st["iterations"]}, {})


def case_cg_loop(args):
    """Forced FP32 CG kernel variant on K + M of the workload mesh run as the solver
    runs it (the whole solve in one graph launch): time per iteration including the
    loop's own costs, next to the autotuner's replayed-graph time."""
    import femeko_gpu as fg
    mesh, nl, mu_lin, u0 = workload(args.cells)
    K = (fg.stiffnessMatrix(mesh) + fg.massMatrix(mesh)).tocsc()
    b = np.random.default_rng(1).normal(size=mesh.nv) if args.rhs == "random" else np.ones(mesh.nv)
    out = {}
    for rep in range(2):   # the first run builds the handle and the graphs
        x, st = fg.cg(K, b, reltol=1e-30, maxiter=args.iters, precision="mixed", spmv=args.variant,
                      inner_rtol=1e-30, use_graph=args.graph_mode, check_every=args.check_every,
                      return_stats=True)
        out = {"us_per_iteration": 1e3 * st["ms"] / max(st["iterations"], 1), "iterations": st["iterations"]}
    _line("CG iteration time in the solve loop (FP32, forced variant)", out["us_per_iteration"], "us/iteration",
          False, {"workload": f"K+M of the Kuhn-tet box, {args.cells}^3 cells", "variant": args.variant,
                  "iterations": out["iterations"], "graph_mode": args.graph_mode, "check_every": args.check_every,
                  "rhs": args.rhs}, {})


def case_newton_kernels(args):
    """One mixed and one FP64 Newton solve, then the per-launch time of the hot
    kernels on each converged operator."""
    import femeko_gpu as fg
    import femeko_gpu._lib as L
    mesh, nl, mu_lin, u0 = workload(args.cells)
    g = fg.gpu_mesh(mesh)
    lib = L.lib()
    out = {}
    for prec in ("mixed", "fp64"):
        u, H, mu, st = fg.newton_magnetostatics(mesh, nl, mu_lin, u0, precision=prec)
        P = L.FG_MIXED if prec == "mixed" else L.FG_FP64
        for which, name in ((0, "cg_spmv"), (1, "cg_update"), (2, "newton_element_pass_all"),
                            (4, "newton_residual_split"), (5, "newton_residual_jacobian_split"),
                            (7, "stiffness_assembly_one_pass"), (8, "stiffness_assembly_two_pass")):
            t = C.c_double()
            L.check(lib.fg_bench_kernel(g.h, which, P, 5 if which < 2 else 3, C.byref(t)))
            out[f"{prec}_{name}_us"] = t.value * 1e3
    _line("Newton hot-kernel launch times", out["mixed_cg_spmv_us"], "us", False,
          {"workload": f"nonlinear Froehlich-plate magnetostatics, Kuhn tets {args.cells}^3 cells"}, {"kernels": out})


def case_heat(args):
    """Backward-Euler heat, 64^3 cells: lognormal(0,1) conductivity, rho_c = 1,
    dt = 1e-3, 100 steps, Gaussian bump of width 0.5 at a seeded interior point,
    T = 0 on the boundary; mixed (FP32 CG + FP64 refinement) vs FP64, the mixed
    snapshots compared with the FP64 ones every 10th step."""
    import femeko_gpu as fg
    from femeko_gpu.mesh import box_tet_mesh
    cells = args.cells if args.cells != 96 else 64
    mesh = box_tet_mesh(cells, seed=SEED)
    rng = np.random.default_rng(SEED)
    kappa = np.exp(rng.normal(size=mesh.nt))
    x0 = rng.uniform(-2.5, 2.5, 3)
    T0 = np.exp(-(((mesh.p - x0[:, None]) ** 2).sum(axis=0)) / 0.5 ** 2)
    res = {}
    variant = {}
    for prec in ("fp64", "mixed"):
        fg.heat_be(mesh, T0, kappa, nsteps=2, every=0, precision=prec, use_graph=args.graph_mode)   # warm-up
        T, snaps, st = fg.heat_be(mesh, T0, kappa, nsteps=100, every=10, precision=prec, use_graph=args.graph_mode)
        res[prec] = (snaps, st)
        import femeko_gpu._lib as L
        vv = C.c_int32(-1)
        L.check(L.lib().fg_get_cg_variant(fg.gpu_mesh(mesh).h, L.FG_MIXED if prec == "mixed" else L.FG_FP64,
                                          C.byref(vv)))
        variant[prec] = int(vv.value)
    err = [float(np.linalg.norm(a - b) / np.linalg.norm(b)) for a, b in zip(res["mixed"][0], res["fp64"][0])]
    ms_m, ms_d = res["mixed"][1]["ms"], res["fp64"][1]["ms"]
    # bandwidth per CG iteration with the whole step time charged to the iterations
    # (right-hand side, refinements and host checks included: a lower bound on the
    # iterations' own rate): FP32 split iteration 6 B per stored nonzero + 60 B per row,
    # FP64 iteration 10 B per stored nonzero + 24 B (SpMV) + 96 B (vector pass) per row
    peak, peak_kind = measured_peaks()
    nnz = int(fg.gpu_mesh(mesh).nnz)
    roof = {}
    for prec, per_nz, per_row in (("mixed", 6, 60), ("fp64", 10, 120)):
        its = max(res[prec][1]["iterations"], 1)
        gbs = (per_nz * nnz + per_row * mesh.nv) * its / (res[prec][1]["ms"] * 1e-3) / 1e9
        roof[prec] = {"bytes_per_iteration": per_nz * nnz + per_row * mesh.nv, "achieved_GBs": gbs,
                      "frac": gbs / peak, "us_per_iteration_with_step_overheads": 1e3 * res[prec][1]["ms"] / its}
    _line("heat BE steps/s (mixed FP32+FP64 refinement)", 100 / (ms_m * 1e-3), "steps/s", True,
          {"workload": f"backward-Euler heat, Kuhn tets {cells}^3 cells, 100 steps", "tets": int(mesh.nt),
           "nodes": int(mesh.nv)},
          {"fp64_steps_per_s": 100 / (ms_d * 1e-3), "mixed_over_fp64": ms_d / ms_m,
           "cg_iters": {"mixed": res["mixed"][1]["iterations"], "fp64": res["fp64"][1]["iterations"]},
           "rel_err_mixed_vs_fp64_every_10th_step": err, "cg_variant_forced_index": variant,
           "roofline": {"bound": "hbm", "peak": peak, "peak_source": peak_kind, **roof}})


def case_sweep(args):
    """256 applied fields h (cos t, sin t, 0), h ~ U[-1e5, 1e5], t ~ U[0, pi], on the
    48^3-cell linear plate mesh (mur 1000): the rank-revealing block CG (default
    method), the per-field multi-right-hand-side CG, and field-by-field solves."""
    import femeko_gpu as fg
    import femeko_gpu._lib as L
    from femeko_gpu.mesh import box_tet_mesh
    cells = args.cells if args.cells != 96 else 48
    mesh = box_tet_mesh(cells, seed=SEED)
    mu = np.where(mesh.elementID == 2, 1000.0, 1.0) * fg.MU0
    rng = np.random.default_rng(SEED)
    h, th = rng.uniform(-1e5, 1e5, 256), rng.uniform(0, np.pi, 256)
    H0 = np.stack([h * np.cos(th), h * np.sin(th), np.zeros(256)], axis=1)
    res = {}
    for method in ("block", "per_field"):
        fg.magnetostatics_sweep(mesh, mu, H0[:32], method=method)                # warm-up
        runs = [fg.magnetostatics_sweep(mesh, mu, H0, method=method)[1] for _ in range(3)]
        res[method] = min(runs, key=lambda st: st["ms"])
    singles = []
    for c in range(8):                                                           # field-by-field sample
        u0 = -(H0[c][:, None] * mesh.p).sum(axis=0)
        _, _, s1 = fg.magnetostatics_linear(mesh, mu, u0, precision="mixed")
        singles.append(s1["ms"])
    per_single = float(np.median(singles))
    # bytes per block-CG iteration (algorithmic): the SpMM reads the FP32 values and
    # int32 columns of every stored slot, the 4-wide z and p_old of each row once and
    # writes p_new and q; the update reads p, q, x, r and the diagonal and writes x, r, z
    g = fg.gpu_mesh(mesh)
    nsell = C.c_int64()
    L.check(L.lib().fg_mesh_layout(g.h, C.byref(nsell), None, None))
    n = mesh.nv
    spmm_bytes = nsell.value * 8 + n * (16 + 16 + 16 + 16)
    upd_bytes = n * (4 * 16 + 4 + 3 * 16)
    sb = res["block"]
    it_us = sb["ms"] * 1e3 / max(sb["iterations"], 1)
    peak = measured_peaks()[0]
    ach = (spmm_bytes + upd_bytes) / (it_us * 1e-6) / 1e9
    _line("field-sweep solves/s (256 fields, rank-revealing block CG)", 256 / (sb["ms"] * 1e-3), "solves/s", True,
          {"workload": f"linear plate magnetostatics, Kuhn tets {cells}^3 cells, 256 fields", "tets": int(mesh.nt),
           "nodes": int(mesh.nv)},
          {"ms": sb["ms"], "rank": sb["rank"], "block_iterations": sb["iterations"],
           "refinements": sb["refinements"], "relres_worst_field": sb["relres"],
           "us_per_block_iteration": it_us,
           "roofline": {"bound": "hbm", "alg_bytes_per_iteration": spmm_bytes + upd_bytes, "achieved_GBs": ach,
                        "peak": peak, "frac": ach / peak,
                        "note": "the 48^3 operator and block vectors (~40 MB) stay in L2 between iterations"},
           "per_field_cg": {"solves_per_s": 256 / (res["per_field"]["ms"] * 1e-3), "ms": res["per_field"]["ms"],
                            "iterations": res["per_field"]["iterations"]},
           "single_field_solves_per_s": 1e3 / per_single,
           "speedup_vs_single_field": (256 / sb["ms"]) / (1 / per_single),
           "speedup_vs_per_field_cg": res["per_field"]["ms"] / sb["ms"]})


def case_batch(args):
    """64 independent linear problems, cells per side ~ U{8..40}, mur ~ U[1,1000] per
    element, one graph launch (a thread-block cluster per problem, sized by its rows),
    in mixed precision (FP32 PCG inside FP64 refinement on each cluster) and in FP64."""
    import femeko_gpu as fg
    from femeko_gpu.mesh import box_tet_mesh
    rng = np.random.default_rng(SEED)
    ns = rng.integers(8, 41, 64)
    meshes = [box_tet_mesh(int(n), seed=SEED + k) for k, n in enumerate(ns)]
    mus = [rng.uniform(1, 1000, m.nt) * fg.MU0 for m in meshes]
    u0s = [-m.p[0].copy() for m in meshes]
    big = int(np.argmax(ns))
    nnz = np.array([fg.gpu_mesh(m).nnz for m in meshes], dtype=np.float64)
    nv = np.array([m.nv for m in meshes], dtype=np.float64)
    peak = measured_peaks()[0]
    res = {}
    for prec in ("mixed", "fp64"):
        fg.batch_magnetostatics_linear(meshes, mus, u0s, rtol=1e-10, precision=prec)   # warm-up (assembly)
        us, its, st = fg.batch_magnetostatics_linear(meshes, mus, u0s, rtol=1e-10, precision=prec)
        fg.batch_magnetostatics_linear([meshes[big]], [mus[big]], [u0s[big]], rtol=1e-10, precision=prec)
        _, its1, st1 = fg.batch_magnetostatics_linear([meshes[big]], [mus[big]], [u0s[big]], rtol=1e-10,
                                                      precision=prec)
        # algorithmic bytes per CG iteration of one problem: FP64, value and column of
        # each stored nonzero (12 B) and the vectors x, r, z, p, q, diagonal (80 B per
        # row); FP32 inner, 8 B per nonzero and 52 B per row
        per_nz, per_row = (12, 80) if prec == "fp64" else (8, 52)
        work = float((its * (per_nz * nnz + per_row * nv)).sum())
        ach = work / (st["ms"] * 1e-3) / 1e9
        res[prec] = {"ms": st["ms"], "solves_per_s": 64 / (st["ms"] * 1e-3), "max_iterations": st["max_iterations"],
                     "total_iterations": st["total_iterations"], "max_refinements": st["max_refinements"],
                     "converged": st["converged"], "largest_cluster_ctas": st["cluster_ctas"],
                     "largest_mesh_alone_ms": st1["ms"], "largest_mesh_alone_iterations": int(its1[0]),
                     "alg_bytes": work, "achieved_GBs": ach, "frac_of_measured_hbm": ach / peak}
    mx = res["mixed"]
    _line("batched independent solves/s (64 meshes, one graph launch)", mx["solves_per_s"], "solves/s",
          True, {"workload": "64 linear problems, Kuhn tets 8..40 cells per side", "cells": [int(n) for n in ns],
                 "total_nodes": int(sum(m.nv for m in meshes)), "precision": "mixed (FP32 PCG, FP64 refinement)",
                 "largest_mesh_cells": int(ns[big])},
          {**mx, "fp64": res["fp64"], "mixed_vs_fp64": res["fp64"]["ms"] / mx["ms"],
           "note": "the vectors and operators stay in L2; FP64 arithmetic issues at 1/64 of the FP32 rate"})


def case_batch_single(args):
    """One linear problem of --cells per side through the batch launch (one 16- or
    8-CTA cluster), mixed then FP64: per-iteration time of the cluster PCG (the ncu
    capture target of the batch kernels)."""
    import femeko_gpu as fg
    from femeko_gpu.mesh import box_tet_mesh
    rng = np.random.default_rng(SEED)
    m = box_tet_mesh(args.cells, seed=SEED)
    mu = rng.uniform(1, 1000, m.nt) * fg.MU0
    u0 = -m.p[0].copy()
    out = {}
    for prec in ("mixed", "fp64"):
        fg.batch_magnetostatics_linear([m], [mu], [u0], rtol=1e-10, precision=prec)
        _, its, st = fg.batch_magnetostatics_linear([m], [mu], [u0], rtol=1e-10, precision=prec)
        out[prec] = {"ms": st["ms"], "iterations": int(its[0]), "refinements": st["max_refinements"],
                     "us_per_iteration": st["ms"] * 1e3 / max(int(its[0]), 1), "cluster_ctas": st["cluster_ctas"]}
    _line("one problem through the batch launch, us per CG iteration (mixed)", out["mixed"]["us_per_iteration"],
          "us", False, {"workload": f"linear problem, Kuhn tets {args.cells} cells per side", "rows": int(m.nv)},
          out)


def _mean_hx(fg, mesh, target, u):
    """J = volume-weighted mean of H_x over the target elements (NewtonRaphson.jl:234-240)."""
    H = fg.hfield(mesh, u)
    sel = target.astype(bool)
    return float((mesh.VE[sel] * H[0, sel]).sum() / mesh.VE[sel].sum())


def case_adjoint(args):
    """dJ/dmur for J = mean Hx over elements with centroid in |x| < 0.5 on the 64^3
    mesh, mur ~ U[1,1000]: adjoint cost against the forward solve, and central
    differences (relative step 1e-6) on 32 elements.  --nonlinear: the same through
    the converged Newton Jacobian with the Froehlich plate of the 96^3 workload."""
    import femeko_gpu as fg
    from femeko_gpu.mesh import box_tet_mesh
    cells = args.cells if args.cells != 96 else 64
    mesh = box_tet_mesh(cells, seed=SEED)
    rng = np.random.default_rng(SEED)
    nl = (mesh.elementID == 2).astype(np.uint8) if args.nonlinear else None
    mur = rng.uniform(1, 1000, mesh.nt)
    if args.nonlinear:
        mur = np.where(nl == 1, 1.0, mur)
    c = mesh.centroids()
    target = (np.sqrt((c * c).sum(axis=0)) < 0.5).astype(np.uint8)
    u0 = -(H0[:, None] * mesh.p).sum(axis=0) if args.nonlinear else -mesh.p[0].copy()
    kw = dict(nl=nl, precision="mixed", rtol=1e-10)
    if args.nonlinear:
        kw.update(tol_update=1e-10)
    fg.adjoint_dJdmu(mesh, mur, u0, target, **kw)                           # warm-up
    J, grad, u, st = fg.adjoint_dJdmu(mesh, mur, u0, target, **kw)
    # central differences with relative step 1e-6 on 32 elements among those with at
    # least 1% of the largest sensitivity.  Linear: each perturbed solution is u + du
    # with A(mu +- d) du = -(+-d) dA/dmur_k u on the free nodes (a right-hand side
    # local to element k, free of the cancellation that forming b - A(mu +- d) u from
    # the whole field would bring); J is linear in u.  Nonlinear: perturbed Newton
    # solves (FP64, tight) from the converged u.
    rel_step = 1e-6
    pool = np.flatnonzero(np.abs(grad) >= 1e-2 * np.abs(grad).max())
    if args.nonlinear:
        pool = pool[nl[pool] == 0]
    picks = np.random.default_rng(11).choice(pool, min(32, pool.size), replace=False)
    errs = []
    if not args.nonlinear:
        import scipy.sparse as sp
        fixed = mesh.dirichlet_mask().astype(bool)
        free = np.flatnonzero(~fixed)
        Kff = fg.stiffnessMatrix(mesh, mur * fg.MU0).tocsr()[free][:, free].tocsc()
        pos = np.full(mesh.nv, -1)
        pos[free] = np.arange(free.size)
    for k in picks:
        d = rel_step * mur[k]
        us = []
        if not args.nonlinear:
            nodes = mesh.t[:4, k]
            Pm = np.vstack([np.ones(4), mesh.p[:, nodes]])
            Gk = np.linalg.inv(Pm)[:, 1:4]
            Ek = fg.MU0 * mesh.VE[k] * (Gk @ Gk.T)            # dA/dmur_k on the element
            gk = Ek @ u[nodes]
            keep = pos[nodes] >= 0
            fi = pos[nodes][keep]
            Pk = sp.csc_matrix((Ek[np.ix_(keep, keep)].ravel(), (np.repeat(fi, fi.size), np.tile(fi, fi.size))),
                               shape=Kff.shape)
        for sgn in (+1, -1):
            if args.nonlinear:
                mu2 = mur * fg.MU0
                mu2[k] = (mur[k] + sgn * d) * fg.MU0
                u2, _, _, s2 = fg.newton_magnetostatics(mesh, nl, mu2, u, precision="fp64", tol_update=1e-14,
                                                        forcing="fixed", inner_rtol=1e-14, picard_steps=0)
                us.append(u2)
            else:
                rhs = np.zeros(free.size)
                rhs[fi] = -sgn * d * gk[keep]
                du = np.zeros(mesh.nv)
                du[free] = fg.cg(Kff + sgn * d * Pk, rhs, reltol=1e-12, precision="fp64")
                us.append(du)
        fd = _mean_hx(fg, mesh, target, us[0] - us[1]) / (2 * d)
        errs.append(abs(fd - grad[k]) / abs(grad[k]))
    what = "Froehlich-plate Newton magnetostatics" if args.nonlinear else "linear magnetostatics"
    _line("adjoint dJ/dmur cost relative to the forward solve", st["adjoint_ms"] / st["forward_ms"], "x forward",
          False, {"workload": f"{what}, Kuhn tets {cells}^3 cells, mur ~ U[1,1000], |x| < 0.5 target",
                  "tets": int(mesh.nt), "nodes": int(mesh.nv), "target_elements": int(target.sum()),
                  "nonlinear": bool(args.nonlinear)},
          {"J": J, "forward_ms": st["forward_ms"], "adjoint_ms": st["adjoint_ms"],
           "forward_iters": st["forward_iters"], "adjoint_iters": st["adjoint_iters"],
           "newton_iters": st["newton_iters"],
           "central_differences": {"elements": int(len(picks)), "rel_step": rel_step,
                                   "max_rel_err": float(max(errs)), "median_rel_err": float(np.median(errs))}})


def case_transport(args):
    """P2 heat transport (backward Euler, LM = M + dt (A + R + C)) on the Kuhn box of
    48^3 cells, second order (912,673 nodes, the rows of the 96^3 linear workload):
    uniform flow along x with a swirl, rho_cp ~ U[0.8, 1.2], kappa = 0.05 lognormal(0,
    0.5), dt = 0.05, penalty intake (1e6) on the x = -5 faces, 20 steps; Jacobi-BiCGStab
    to 1e-10 per step (FP64)."""
    import femeko_gpu as fg
    from femeko_gpu.mesh import box_tet_mesh, surface_faces6
    cells = args.cells if args.cells != 96 else 48
    mesh = box_tet_mesh(cells, seed=SEED, order=2)
    rng = np.random.default_rng(SEED)
    x, y, z = mesh.p
    u = np.vstack([np.ones(mesh.nv), -0.2 * z, 0.2 * y])
    rho = rng.uniform(0.8, 1.2, mesh.nt)
    kap = 0.05 * np.exp(0.5 * rng.normal(size=mesh.nt))
    f6 = surface_faces6(mesh)
    F = np.where(np.all(np.isclose(x[f6[:3]], x.min()), axis=0), 1e6, 0.0)
    T0 = np.exp(-((x + 3.0) ** 2 + y ** 2 + z ** 2) / 1.0)
    nsteps = 20
    fg.transport_be(mesh, T0, rho, kap, u, 0.05, 2, face_F=F, faces=f6)                  # warm-up
    T, _, st = fg.transport_be(mesh, T0, rho, kap, u, 0.05, nsteps, face_F=F, faces=f6)
    g = fg.gpu_mesh(mesh)
    pat = g.csc(np.ones(g.nnz))
    rows_of = np.repeat(np.arange(mesh.nv), np.diff(pat.indptr))
    colb = 2 if np.abs(rows_of - pat.indices).max() < 32768 else 4
    # per BiCGStab iteration: two SpMVs (values + column offsets, x gathered once, y
    # written, the dot partner read) and the three vector passes (6 + 5 + 8 vectors)
    alg = 2 * g.nnz * (8 + colb) + 8 * mesh.nv * (2 * 3 + 6 + 5 + 8)
    it_us = st["ms"] * 1e3 / max(st["iterations"], 1)
    peak = measured_peaks()[0]
    _line("transport BE steps/s (P2, Jacobi-BiCGStab FP64)", nsteps / (st["ms"] * 1e-3), "steps/s", True,
          {"workload": f"P2 heat transport, Kuhn tets {cells}^3 cells, {nsteps} steps", "tets": int(mesh.nt),
           "nodes": int(mesh.nv), "nnz": int(g.nnz)},
          {"ms": st["ms"], "bicgstab_iterations": st["iterations"], "us_per_iteration": it_us,
           "alg_bytes_per_iteration": alg, "achieved_GBs": alg / (it_us * 1e-6) / 1e9,
           "frac_of_measured_hbm": alg / (it_us * 1e-6) / 1e9 / peak if peak else None,
           "converged": bool(st["converged"]), "relres_last": st["relres"],
           "note": "ms covers the operator assembly and all steps"})


def case_nedelec(args):
    """Nedelec Newton (vector potential, edge unknowns) on the Kuhn box of 32^3 cells,
    second order, with an iron cube |x|, |y|, |z| < 3 (relative reluctance 0.002 at low
    field, saturating towards 1 around 1.8 T, a 40-point table), Bext = 0.8 T along x,
    tol 1e-4 T on max |B - B_prev| (nedelec3D.jl:30), each correction by FP64 Jacobi-PCG
    to sqrt(eps) = 1.49e-8 relative, the default tolerance of the reference's
    IterativeSolvers.cg at nedelec3D.jl:185."""
    import femeko_gpu as fg
    from femeko_gpu.mesh import box_tet_mesh
    cells = args.cells if args.cells != 96 else 32
    mesh = box_tet_mesh(cells, seed=SEED, order=2, plate=((-3.0, 3.0), (-3.0, 3.0), (-3.0, 3.0)))
    b = np.linspace(0.0, 3.0, 40)
    q = (b / 1.8) ** 6
    nu_tab = 0.002 + 0.998 * q / (1.0 + q)
    nl = (mesh.elementID == 2).astype(np.uint8)
    Bext = np.array([0.8, 0.0, 0.0])
    rtol = float(np.sqrt(np.finfo(np.float64).eps))
    res = {}
    for prec in ("fp64", "mixed"):
        fg.nedelec_newton(mesh, Bext, b, nu_tab, nonlinear=nl, max_newton=2, precision=prec,
                          use_graph=args.graph_mode)                                              # warm-up
        res[prec] = fg.nedelec_newton(mesh, Bext, b, nu_tab, nonlinear=nl, tol=1e-4, rtol=rtol, precision=prec,
                                      use_graph=args.graph_mode)
    u, Bf, B, nu, steps, st = res["mixed"]
    _, Bf64, _, _, steps64, st64 = res["fp64"]
    g = fg.edge_mesh(mesh)
    _line("Nedelec Newton solves/s (edge elements, mixed FP32 CG + FP64 refinement)", 1e3 / st["ms"], "solves/s", True,
          {"workload": f"Nedelec vector-potential Newton, Kuhn tets {cells}^3 cells, iron cube", "tets": int(mesh.nt),
           "edges": int(g.ne), "nnz": int(g.nnz)},
          {"ms": st["ms"], "newton_steps": steps, "cg_iterations": st["iterations"],
           "short_inner_solves": st["short_inner_solves"],
           "us_per_cg_iteration": st["ms"] * 1e3 / max(st["iterations"], 1), "converged": bool(st["converged"]),
           "B_iron_max_T": float(B[nl == 1].max()),
           "fp64": {"solves_per_s": 1e3 / st64["ms"], "ms": st64["ms"], "newton_steps": steps64,
                    "cg_iterations": st64["iterations"]},
           "mixed_over_fp64": st64["ms"] / st["ms"],
           "B_rel_diff_mixed_vs_fp64": float(np.abs(Bf - Bf64).max() / np.abs(Bf64).max())})


CASES = {"cg-kernel": case_cg_kernel, "cg-loop": case_cg_loop, "newton-kernels": case_newton_kernels, "heat": case_heat,
         "sweep": case_sweep, "batch": case_batch, "batch-single": case_batch_single, "adjoint": case_adjoint, "transport": case_transport,
         "nedelec": case_nedelec}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--fp64-steps", type=int, default=None)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cells", type=int, default=96)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-steps", type=int, default=1,
                    help="--impl reference: full CPU solves timed (at most --steps; about a minute each at 96^3)")
    ap.add_argument("--spmv-traffic", type=float, default=None,
                    help="DRAM bytes per SpMV launch from an ncu capture (reported as roofline.traffic)")
    ap.add_argument("--check-every", type=int, default=32,
                    help="CG iterations between convergence tests (the body of the solve's graph loop)")
    ap.add_argument("--graph-mode", type=int, default=1, choices=[0, 1, 2],
                    help="1: whole CG in one graph launch (device-side loop); 2: host-checked graph blocks; 0: no graph")
    ap.add_argument("--cg-variant", type=int, default=0,
                    help="fix the FP32 CG kernel variant (1..29; 0: autotuned), e.g. for profiling runs")
    ap.add_argument("--cg64-variant", type=int, default=0, help="fix the FP64 CG SpMV variant (1..4; 0: autotuned)")
    ap.add_argument("--case", choices=sorted(CASES), default=None,
                    help="run a secondary workload instead of the headline benchmark")
    ap.add_argument("--variant", type=int, default=6, help="--case cg-kernel: forced CG kernel variant (1..6)")
    ap.add_argument("--iters", type=int, default=200, help="--case cg-kernel: CG iterations")
    ap.add_argument("--rhs", choices=["random", "ones"], default="random", help="--case cg-loop: right-hand side")
    ap.add_argument("--nonlinear", action="store_true", help="--case adjoint: through the Newton Jacobian")
    args = ap.parse_args()
    if args.fp64_steps is None:
        args.fp64_steps = args.steps
    if args.case:
        sys.path.insert(0, os.path.join(ROOT, "femeko.jl_gb300"))
        CASES[args.case](args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
