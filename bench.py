#!/usr/bin/env python
"""Benchmark of the HDG Poisson path on one GB300 (or N replicas, one per GPU).

Default workload (the plain-method scaled case): -Δu = f on the unit square, f = 2π² sin(πx)
sin(πy), homogeneous Dirichlet, structured right-diagonal mesh 2·256·256 = 131072 triangles,
p = 2, τ = 1, FP64: element assembly + condensation, trace-matrix gather, apply!, Jacobi-PCG to
1e-12 relative residual, recovery of u and q.  One step = one complete solve.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload c1|c2] [--precision fp64|mixed] [--no-cpu-baseline]

Prints one JSON line (rank 0).  `value` is solves/s with inputs resident on the device; `e2e`
is the same metric through the public API with host buffers (coordinates and source uploaded,
û, q, u downloaded every step).  With --impl reference the CPU oracle (a C++ restatement of the
reference's flow with a sparse direct solve) is timed on the host cores instead.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "HDG solves/s & p50/p99 latency, served vs plain GPU at ≤1e-8 rel L2 err"
WORKLOADS = {
    "c1": dict(n=32, p=1, qd=None, desc="2·32·32=2048 triangles, p=1, tau=1, FP64, manufactured sin·sin, "
                                       "homogeneous Dirichlet"),
    "c2": dict(n=256, p=2, qd=None, desc="2·256·256=131072 triangles, p=2, tau=1, FP64, manufactured sin·sin, "
                                        "homogeneous Dirichlet, Jacobi-PCG to 1e-12 relative residual"),
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--tol", type=float, default=1e-12)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


# ---------------------------------------------------------------- distributed helpers
def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v, ws):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- clocks
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in open(self.path):
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def profile_traffic(kernel: str):
    """dram bytes per launch of `kernel` from the committed ncu summary (profiles/), if present."""
    import re
    d = os.path.join(ROOT, "profiles")
    if not os.path.isdir(d):
        return None
    for fn in sorted(os.listdir(d)):
        if not fn.endswith((".md", ".txt")):
            continue
        for ln in open(os.path.join(d, fn)):
            m = re.match(r"\s*traffic_bytes_per_launch\[(\w+)\]\s*[:=]\s*([0-9.eE+]+)", ln)
            if m and m.group(1) == kernel:
                return float(m.group(2))
    return None


# ---------------------------------------------------------------- CPU oracle
def oracle_solve_once(n, p, qd, threads):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import hdgref
    t0 = time.perf_counter()
    r = hdgref.solve_poisson(hdgref.rectangle_mesh(n, n), p, qd=qd, f=hdgref.MANUFACTURED_F, threads=threads)
    return time.perf_counter() - t0, r


def cpu_baseline(w, threads):
    dt, _ = oracle_solve_once(w["n"], w["p"], w["qd"], threads)
    return {"value": 1.0 / dt, "unit": "solves/s", "cores": threads, "kind": "port",
            "sample": f"one complete solve of the same workload ({2 * w['n'] ** 2} cells, p={w['p']}) by the "
                      f"C++ oracle: OpenMP element loop on {threads} threads, COO->CSC, apply!, SuperLU "
                      f"(single-threaded, MMD on A'+A ordering), recovery; {dt:.2f} s"}


def run_reference(args, ws, rank):
    if rank != 0:
        return
    w = WORKLOADS[args.workload]
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        oracle_solve_once(w["n"], w["p"], w["qd"], threads)
    times = []
    for _ in range(args.steps):
        dt, _ = oracle_solve_once(w["n"], w["p"], w["qd"], threads)
        times.append(dt)
    tot = sum(times)
    value = args.steps / tot
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.workload}: {w['desc']}", "n": w["n"], "p": w["p"]},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port",
                         "sample": "each step is one complete solve of the workload by the C++ oracle (OpenMP element "
                                   "loop, COO->CSC, apply!, SuperLU direct solve, recovery); the reference itself is "
                                   "Julia, which is not installed on this machine"},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "p50_ms": 1e3 * statistics.median(times), "p99_ms": 1e3 * max(times),
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- our arm
def run_ours(args, ws, rank, local):
    import numpy as np
    import torch

    import __graft_entry__ as g
    g.build()
    H = g.import_package()
    w = WORKLOADS[args.workload]
    prec = H.PREC_FP64 if args.precision == "fp64" else H.PREC_MIXED
    torch.cuda.set_device(local)
    ctx = H.Context(local)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)

    n, p = w["n"], w["p"]
    mesh = H.rectangle_mesh(H.TriangleCell, (n, n), (0.0, 0.0), (1.0, 1.0), ctx=ctx)
    fe = H.GenericFiniteElement(H.Dubiner(2, H.RefTetrahedron, p))
    Wh = H.ScalarFunctionSpace(mesh, fe, quad_degree=w["qd"])
    Vh = H.VectorFunctionSpace(mesh, fe, quad_degree=w["qd"])
    Mh = H.ScalarTraceFunctionSpace(Wh, H.GenericFiniteElement(H.Legendre(1, H.RefTetrahedron, p)))
    f = H.MANUFACTURED_F
    K, b, K_e, b_e = H.doassemble(Vh, Wh, Mh, 1.0, f, precision=prec)
    dbc = H.Dirichlet(H.TrialFunction(Mh), mesh, "boundary")
    ndofs, ncells, nnz = K.ndofs, mesh.ncells, K.nnz

    def step():
        K.reassemble(1.0, f)
        K.apply_dirichlet(dbc.prescribed_dofs, dbc.values)
        K.solve(tol=args.tol, precision=prec, to_host=False)
        K.recover(to_host=False)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()

    # ---- timed region (device-resident inputs) ----
    ctx.set_profiling(True)
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = ctx.launches()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    tims = []
    iters = []
    barrier(ws)
    torch.cuda.synchronize()
    t_all0 = torch.cuda.Event(enable_timing=True)
    t_all1 = torch.cuda.Event(enable_timing=True)
    t_all0.record(stream)
    for k in range(args.steps):
        ev[k][0].record(stream)
        step()
        ev[k][1].record(stream)
        tims.append(K.timings())
        iters.append(K.stats.iterations)
    t_all1.record(stream)
    torch.cuda.synchronize()
    barrier(ws)
    launches = ctx.launches() - launches0
    ctx.set_profiling(False)
    clk = clocks.stop()
    elapsed_ms = max_over_ranks(t_all0.elapsed_time(t_all1), ws)
    step_ms = sorted(e0.elapsed_time(e1) for e0, e1 in ev)
    value = ws * args.steps / (elapsed_ms / 1e3)

    # accuracy of the timed solve: recovered u against the exact solution
    K.recover()
    err2 = K.errornorm(H.MANUFACTURED_U)

    # ---- roofline of the dominant kernel ----
    peaks, peak_kind = measured_peaks()
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    nt, nf = p + 1, mesh.nfaces
    nblocks = nnz // (nt * nt)
    s = 8 if prec == H.PREC_FP64 else 4
    bytes_a = nnz * s + nblocks * 4 + (nf + 1) * 4 + ndofs * (s + 4 * s)          # values, cols, rowptr, z, q r/w, p r/w
    bytes_b = ndofs * (8 * 2 + 3 * s + 2 * s + s)                                     # x r/w, p, q, dinv r; r r/w, z w
    nw_, m_ = (p + 1) * (p + 2) // 2, 3 * (p + 1)
    bytes_elem = ncells * (12 + 48 + 1 + 8 * (m_ * (m_ + 1) + 3 * nw_ * (m_ + 1)))
    avg = lambda key: statistics.mean(t[key] for t in tims)
    it_mean = statistics.mean(iters)
    kern = {
        "k_cg_a (q = A z + beta q, p update, p.q)": (avg("cg_a_ms"), bytes_a, it_mean),
        "k_cg_b (x, r, z update, r.z, r.r)": (avg("cg_b_ms"), bytes_b, it_mean),
        "k_element_condense": (avg("element_ms"), bytes_elem, 1),
    }
    dom = max(kern, key=lambda k: kern[k][0] * kern[k][2])
    dur, alg, cnt = kern[dom]
    achieved = alg / (dur / 1e3) / 1e9 if dur > 0 else None
    traffic = profile_traffic("k_cg_a" if dom.startswith("k_cg_a") else dom.split()[0])

    # ---- end-to-end through the public API with host buffers ----
    import numpy as np
    xy_host = H.get_vertices_matrix(mesh)
    xy_pinned = torch.from_numpy(xy_host).pin_memory().numpy()
    q_h = u_h = None

    def e2e_step():
        mesh.set_coordinates(xy_pinned)                       # H2D: node coordinates
        K.reassemble(1.0, f)                                  # H2D: source parameters
        K.apply_dirichlet(dbc.prescribed_dofs, dbc.values)    # H2D: prescribed dofs and values
        uh = K.solve(tol=args.tol, precision=prec, to_host=True)   # D2H: û
        return uh, K.recover(to_host=True)                    # D2H: q, u, û per cell

    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    barrier(ws)
    t0 = time.perf_counter()
    e2e_n = max(3, args.steps // 2)
    for _ in range(e2e_n):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, ws)
    nv_, nw2 = 2 * nw_, nw_
    h2d = xy_host.nbytes + len(f.params) * 8 + dbc.prescribed_dofs.nbytes + dbc.values.nbytes
    d2h = ndofs * 8 + ncells * (nv_ + nw2 + 3 * nt) * 8 + ncells * 3 * nt * 8

    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if prec == H.PREC_FP64 else "f32+f64",
        "data": "synthetic",
        "config": {"workload": f"{args.workload}: {w['desc']}", "n": n, "p": p, "cells": ncells, "trace_dofs": ndofs,
                   "nnz": nnz, "precision": args.precision, "tol": args.tol,
                   "l2": "inputs larger than L2: each step rewrites the per-cell condensed blocks "
                         f"({bytes_elem / 1e6:.0f} MB) before the solve",
                   "parallelism": f"{ws} independent replica(s), one per GPU"},
        "p50_ms": statistics.median(step_ms), "p99_ms": step_ms[min(len(step_ms) - 1, int(math.ceil(0.99 * len(step_ms))) - 1)],
        "cg_iterations": it_mean, "errornorm_sq": err2,
        "elements_per_s": ncells / (avg("element_ms") / 1e3) if avg("element_ms") > 0 else None,
        "trace_dof_iterations_per_s": ndofs * it_mean / (avg("cg_ms") / 1e3) if avg("cg_ms") > 0 else None,
        "phase_ms": {k: avg(k) for k in ("element_ms", "gather_ms", "apply_ms", "cg_ms", "cg_a_ms", "cg_b_ms",
                                          "recover_ms")},
        "gpu_launches": launches,
        "roofline": {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": (achieved / hbm) if achieved else None, "traffic": traffic,
                     "algorithmic_bytes_per_launch": alg, "avg_launch_ms": dur,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else
                     "fallback 6.8 TB/s"},
        "e2e": {"value": ws * e2e_n / e2e_s, "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "clocks": clk,
    }
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w, os.cpu_count() or 1)
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    ws, rank, local = dist_setup(args) if args.impl == "ours" else (int(os.environ.get("WORLD_SIZE", "1")),
                                                                    int(os.environ.get("RANK", "0")), 0)
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
