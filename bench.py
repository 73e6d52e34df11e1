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
--impl reference: the CPU restatement of the reference algorithm (oracle port, all
host threads) on a bounded sample, extrapolated to solves/s.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
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
            "inner_tolerance": "Eisenstat-Walker (choice 2, gamma 0.9) in [1e-6, 0.1], both precisions",
            "line_search": "alpha = 0.9^k backtracking on the nonlinear residual",
            "l2": "inputs larger than L2 (operator, records and element state ~2 GB)"}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, dev: int = 0):
        self.dev = dev
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_{os.getpid()}.csv")

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


def cpu_sample(mesh, nl, mu_lin, u0, counts, threads, cg_iters=100):
    """Bounded CPU sample of the oracle port, extrapolated to one full solve."""
    import oracle as O
    O.set_threads(threads)
    s = O.newton_sample(mesh, u0, nl, mu_lin, MS, HK, cg_iters)
    per_cg = s["cg_s"] / max(s["cg_iters"], 1)
    n_it, trials, cg_total = counts
    est = (1 + trials) * s["state_s"] + n_it * s["tangent_s"] + cg_total * per_cg
    return 1.0 / est, s, est


def run_reference(args):
    ws, rank = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    mesh, nl, mu_lin, u0 = workload(args.cells)
    # iteration counts of the same algorithm (FP64 Newton, inner rtol 1e-4, residual
    # backtracking) measured on this workload by the GPU FP64 path; stored so that the
    # reference arm needs no GPU.
    counts = tuple(args.ref_counts)
    vals = []
    for step in range(args.warmup + args.steps):
        v, s, est = cpu_sample(mesh, nl, mu_lin, u0, counts, threads, cg_iters=args.cpu_cg_iters)
        if step >= args.warmup:
            vals.append(v)
    value = statistics.median(vals)
    sample = (f"per step: one Newton state evaluation, one tangent assembly and {args.cpu_cg_iters} PCG iterations "
              f"of the oracle port on the 96^3 workload, extrapolated with the solve's counts "
              f"(newton, line-search trials, CG) = {counts}")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / value, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config(args.cells, mesh),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
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

    def solve(precision):
        u, H, mu, st = fg.newton_magnetostatics(mesh, nl, mu_lin, u0, precision=precision)
        if not st["converged"]:
            raise RuntimeError(f"Newton did not converge: {st}")
        return u, H, mu, st

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
                u, H, mu, stats = solve(prec)
                ms.append(stats["ms"])
            barrier()
            wall = time.time() - wall0
        if prec == "mixed":
            launches = lib.fg_kernel_launches() - launches0
        tot = sum(ms) / 1000.0
        if ws > 1:
            import torch.distributed as dist
            tt = torch.tensor([tot], device="cuda", dtype=torch.float64)
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            tot = float(tt.item())
        res[prec] = dict(u=u, H=H, mu=mu, stats=stats, sec=tot, wall=wall, steps=steps, clocks=clk.summary())

    Hm, Hd = res["mixed"]["H"], res["fp64"]["H"]
    herr = float(np.linalg.norm(Hm - Hd) / np.linalg.norm(Hd))
    uerr = float(np.linalg.norm(res["mixed"]["u"] - res["fp64"]["u"]) / np.linalg.norm(res["fp64"]["u"]))
    werr = abs(res["mixed"]["stats"]["energy"] - res["fp64"]["stats"]["energy"]) / abs(res["fp64"]["stats"]["energy"])
    value = ws * args.steps / res["mixed"]["sec"]
    fp64_value = ws * args.fp64_steps / res["fp64"]["sec"]

    # roofline: dominant kernel = the FP32 CG SpMV on the converged tangent operator
    peak, peak_kind = measured_peaks()
    nsell, ninc, nsl = C.c_int64(), C.c_int64(), C.c_int32()
    lib.fg_mesh_layout(g.h, C.byref(nsell), C.byref(ninc), C.byref(nsl))
    fg.newton_magnetostatics(mesh, nl, mu_lin, u0, precision="mixed")   # leaves J32 on the handle
    chosen = C.c_int32()
    variants_us = np.zeros(6)
    L.check(lib.fg_autotune(g.h, L.FG_MIXED, C.byref(chosen), L.ptr(variants_us), 6))
    autotune = {"cg32_iteration_variants_us": [round(float(v), 2) for v in variants_us], "chosen": int(chosen.value),
                "names": ["gather/256", "gather-hoist/256", "gather/128", "gather/512", "halo-smem",
                          "halo-smem-pipelined"]}
    ms_spmv = C.c_double()
    L.check(lib.fg_bench_kernel(g.h, 0, L.FG_MIXED, 200, C.byref(ms_spmv)))
    kernels_us = {"cg32_iteration": ms_spmv.value * 1e3}
    for name, which, prec in (("newton_assembly_f32", 2, L.FG_MIXED),):
        t = C.c_double()
        L.check(lib.fg_bench_kernel(g.h, which, prec, 20 if which == 2 else 200, C.byref(t)))
        kernels_us[name] = t.value * 1e3
    fg.newton_magnetostatics(mesh, nl, mu_lin, u0, precision="fp64")   # leaves J64 on the handle
    ch64, us64 = C.c_int32(), np.zeros(2)
    L.check(lib.fg_autotune(g.h, L.FG_FP64, C.byref(ch64), L.ptr(us64), 2))
    autotune["cg64_spmv_variants_us"] = [round(float(v), 2) for v in us64]
    autotune["chosen64"] = int(ch64.value)
    for name, which in (("cg64_spmv", 0), ("cg64_update", 1)):
        t = C.c_double()
        L.check(lib.fg_bench_kernel(g.h, which, L.FG_FP64, 200, C.byref(t)))
        kernels_us[name] = t.value * 1e3
    fg.newton_magnetostatics(mesh, nl, mu_lin, u0, precision="mixed")
    n = mesh.nv
    # one fused FP32 CG iteration: matrix value (4 B) + 16-bit column (2 B) per stored
    # nonzero; per row the (r, w, s, dinv) state read and written (16 + 16 B) and
    # p, x read and written (8 + 8 B).  Neighbour-state gathers are re-reads.
    alg_bytes = g.nnz * 6 + 48 * n
    achieved = alg_bytes / (ms_spmv.value * 1e-3) / 1e9
    kname = {4: "k_cg32_iter_halo", 5: "k_cg32_iter_pipe"}.get(int(chosen.value), "k_cg32_iter")
    roofline = {"bound": "hbm", "kernel": kname, "variant": autotune["names"][int(chosen.value)],
                "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": args.spmv_traffic, "algorithmic_bytes": alg_bytes, "us_per_launch": ms_spmv.value * 1e3}

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
        for _ in range(max(1, min(args.warmup, 2))):
            one()
        barrier()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        w0 = time.time()
        ev0.record()
        for _ in range(args.e2e_steps):
            one()
        ev1.record()
        barrier()
        e2e_sec = max(ev0.elapsed_time(ev1) / 1000.0, time.time() - w0)
        h2d = p_np.nbytes + t_np.nbytes + fx_np.nbytes + nl_np.nbytes + mu_np.nbytes + u0_np.nbytes
        d2h = uo_np.nbytes + Ho_np.nbytes + muo_np.nbytes
        e2e = {"value": ws * args.e2e_steps / e2e_sec, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "steps": args.e2e_steps,
               "what": "fg_scalar_potential_newton: upload + pattern build + solve + download per step"}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        st = res["fp64"]["stats"]
        counts = (st["newton_iters"], st["trials"], st["cg_iters"])
        threads = os.cpu_count() or 1
        v, s, est = cpu_sample(mesh, nl, mu_lin, u0, counts, threads, cg_iters=args.cpu_cg_iters)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": (f"one Newton state evaluation ({s['state_s']:.2f} s), one tangent assembly "
                          f"({s['tangent_s']:.2f} s) and {s['cg_iters']} PCG iterations ({s['cg_s']:.2f} s) of the "
                          f"oracle port on this workload, extrapolated with the FP64 solve's counts "
                          f"(newton, trials, cg) = {counts} to {est:.1f} s per solve")}

    sm = res["mixed"]["stats"]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * res["mixed"]["sec"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 operator/CG, f64 residual/update",
            "data": "synthetic", "config": config(args.cells, mesh),
            "fp64": {"value": fp64_value, "unit": UNIT, "ms_per_step": 1000.0 * res["fp64"]["sec"] / args.fp64_steps,
                     "newton_iters": res["fp64"]["stats"]["newton_iters"], "cg_iters": res["fp64"]["stats"]["cg_iters"]},
            "mixed_over_fp64": value / fp64_value,
            "accuracy_vs_fp64_gpu": {"H_rel": herr, "u_rel": uerr, "energy_rel": werr},
            "newton_iters": sm["newton_iters"], "cg_iters": sm["cg_iters"], "trials": sm["trials"],
            "roofline": roofline, "kernels_us": kernels_us, "autotune": autotune, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": int(launches),
            "clocks": res["mixed"]["clocks"], "clocks_fp64": res["fp64"]["clocks"],
            "setup_s": {"mesh_generate": t_gen, "mesh_create_pattern": t_setup},
            "wall_s": {"mixed": res["mixed"]["wall"], "fp64": res["fp64"]["wall"]}}
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--fp64-steps", type=int, default=None)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cells", type=int, default=96)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-cg-iters", type=int, default=100)
    ap.add_argument("--spmv-traffic", type=float, default=None,
                    help="DRAM bytes per SpMV launch from an ncu capture (reported as roofline.traffic)")
    ap.add_argument("--ref-counts", type=int, nargs=3, default=[11, 39, 1324],
                    help="(newton iterations, line-search trials, CG iterations) of the solve; default: the FP64 GPU solve at 96^3")
    args = ap.parse_args()
    if args.fp64_steps is None:
        args.fp64_steps = args.steps
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
