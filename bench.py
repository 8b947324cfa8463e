#!/usr/bin/env python
"""Benchmark of the HDG Poisson path on one GB300 (or N replicas, one per GPU).

Default workload (c4, the batching configuration the served-vs-plain metric is stated on): 256
independent Poisson problems, n log-uniform in [8, 128], p uniform in {1..4}, jittered meshes,
per-cell kappa log-uniform in [1e-2, 1e2], Gaussian-bump sources.  One step solves all 256 as
degree-binned batches (assemble + condense, apply!, multigrid-preconditioned CG to 1e-9 with an
FP32 V-cycle, recovery); the plain FP64 path that solves them one at a time with the same
preconditioner is timed beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload c1|c2|c3|c4|c5] [--precision fp64|mixed] [--no-cpu-baseline]

Prints one JSON line (rank 0).  `value` is solves/s with inputs resident on the device; `e2e`
is the same metric through the public API with host buffers.  With --impl reference the CPU
oracle (a C++ restatement of the reference's flow with a sparse direct solve) is timed on the
host cores instead.
"""
from __future__ import annotations

import argparse
import gc
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
                                        "homogeneous Dirichlet, PCG to 1e-12 relative residual"),
}


C4_SEED = 20240611


def c4_specs(count=256, seed=C4_SEED):
    """The batching workload as plain numbers (numpy only, so that the reference arm needs nothing
    of the library): `count` problems, n log-uniform in [8, 128], p uniform in {1,2,3,4}, interior
    nodes jittered by U(-0.2h, 0.2h) (splitmix64 stream seeded seed + k), per-cell kappa log-uniform
    in [1e-2, 1e2], f = 8 Gaussian bumps (centres uniform in the square, widths 0.03-0.15, amplitudes
    N(0, 10^2)).  Each spec: n, p, qd (the quadrature degree), bumps (the HDG_FIELD_BUMPS
    parameters {K, (cx, cy, s, a) x K}), kappa_cell, jitter, seed."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n = int(round(math.exp(rng.uniform(math.log(8), math.log(128)))))
        p = int(rng.integers(1, 5))
        centres, widths, amps = rng.random((8, 2)), 0.03 + 0.12 * rng.random(8), 10.0 * rng.standard_normal(8)
        bumps = np.concatenate([[8.0], np.column_stack([centres, widths, amps]).ravel()])
        kc = np.exp(rng.uniform(math.log(1e-2), math.log(1e2), 2 * n * n))
        out.append(dict(n=n, p=p, qd={1: 2, 2: 3, 3: 6, 4: 9}[p], bumps=bumps, kappa_cell=kc, jitter=0.2,
                        seed=seed + k))
    return out


def jitter_rect_xy(xy, n, a, seed):
    """Node coordinates of the n x n unit-square rectangle mesh (x fastest) with every interior
    node moved by U(-a, a) h per coordinate, in the order and from the splitmix64 stream that
    hdg_mesh_jitter uses (numpy uint64 arithmetic wraps as the C code does)."""
    import numpy as np
    G = np.uint64(0x9E3779B97F4A7C15)
    m = 2 * (n - 1) * (n - 1)
    with np.errstate(over="ignore"):
        z = (np.uint64(seed) ^ G) + np.arange(1, m + 1, dtype=np.uint64) * G
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    r = (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0) * 2.0 - 1.0
    h = 1.0 / n
    out = np.array(xy, dtype=np.float64, copy=True)
    jj, ii = np.meshgrid(np.arange(1, n), np.arange(1, n), indexing="ij")
    idx = (jj * (n + 1) + ii).ravel()
    out[idx, 0] = out[idx, 0] + (a * h) * r[0::2]
    out[idx, 1] = out[idx, 1] + (a * h) * r[1::2]
    return out


def c4_problems(H, count=256, seed=C4_SEED):
    """c4_specs as library Problem objects (the GPU arm)."""
    return [H.Problem(n=s["n"], p=s["p"], f=H.Field(H._lib.FIELD_BUMPS, tuple(float(v) for v in s["bumps"])),
                      kappa_cell=s["kappa_cell"], jitter=s["jitter"], seed=s["seed"]) for s in c4_specs(count, seed)]


def rel_l2(a, b):
    import numpy as np
    nb = float(np.linalg.norm(b))
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b))) / (nb if nb > 0 else 1.0)


C4_DESC = ("c4: 256 independent Poisson problems, n log-uniform [8,128], p uniform {1..4}, jitter 0.2h, "
           "per-cell kappa log-uniform [1e-2,1e2], 8 Gaussian bumps")


def _oracle_c4_solve(spec, keep=False):
    """One batching-workload problem solved completely by the CPU oracle on one thread (element loop,
    COO->CSC, apply!, SuperLU, recovery); returns (seconds, {"uhat", "u"} or None).  Runs in a pool
    worker; it imports only numpy and the oracle."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import hdgref
    n = spec["n"]
    om = hdgref.rectangle_mesh(n, n)
    om.set_xy(jitter_rect_xy(om.xy, n, spec["jitter"], spec["seed"]))
    t0 = time.perf_counter()
    r = hdgref.solve_poisson(om, spec["p"], qd=spec["qd"], f=(hdgref.F_BUMPS, spec["bumps"]),
                             kappa_cell=spec["kappa_cell"], threads=1)
    dt = time.perf_counter() - t0
    return dt, (dict(uhat=np.asarray(r["uhat"]), u=np.asarray(r["u"])) if keep else None)


def _pool_solve(args):
    spec, keep = args
    return _oracle_c4_solve(spec, keep)


def c4_cpu_sample_indices(specs, count=48):
    """A fixed stratified sample of the batch: the problems sorted by size (cells, then degree), cut
    into `count` equal strata, the middle problem of each.  The same sample in every step."""
    order = sorted(range(len(specs)), key=lambda k: (specs[k]["n"], specs[k]["p"], k))
    per = len(order) / count
    return [order[int(per * j + per / 2)] for j in range(count)]


class OraclePool:
    """Worker processes (started with spawn, one per host core) that solve batching-workload
    problems with the single-threaded oracle, largest problems first."""

    def __init__(self, workers=None):
        import multiprocessing as mp
        self.workers = workers or (os.cpu_count() or 1)
        self.pool = mp.get_context("spawn").Pool(self.workers)

    def run(self, specs, idx, keep=False):
        """Solves specs[idx]; returns (wall seconds, per-problem seconds, results) in idx order."""
        order = sorted(idx, key=lambda k: -(specs[k]["n"] ** 2) * (specs[k]["p"] + 1) ** 3)
        t0 = time.perf_counter()
        res = self.pool.map(_pool_solve, [(specs[k], keep) for k in order], chunksize=1)
        wall = time.perf_counter() - t0
        by = dict(zip(order, res))
        return wall, [by[k][0] for k in idx], [by[k][1] for k in idx]

    def close(self):
        self.pool.close()
        self.pool.join()


FP64_TFLOPS_MEASURED = 1.21  # FMA-loop probe on the GB300s (all lanes, FP64 pipe), TFLOP/s


def element_cost(p, schur):
    """Per-cell algorithmic bytes and FP64 FLOPs of the element kernel of degree p.  Bytes: read 3
    node ids, 6 coordinates, the orientation byte and kappa (69 B); write [Ate | bte] and the stored
    rows of [K_e | b_e] (all n rows on the full path, the nw u rows on the Cholesky-Schur path).
    FLOPs: the operations the kernel performs (2 per FMA); the count of a dense LU of the n x n local
    system with m+1 right-hand sides and the Ate product (2/3 n^3 + 2 n^2 (m+1) + 2 m^2 n) is the
    nominal work and is reported beside it."""
    nw, nt = (p + 1) * (p + 2) // 2, p + 1
    n, m = 3 * nw, 3 * nt
    rc = nw + m + 1
    rows = nw if schur else n
    nbytes = 69 + 8 * (m * (m + 1) + rows * (m + 1))
    if schur:
        chol = sum((rc - k - 1) + sum(rc - i for i in range(k + 1, nw)) for k in range(nw))
        fma = (7 * nw * (nw + 1) // 2 + 3 * nw * m + chol + (m * (m + 1) // 2 + m) * nw + 2 * (m * (m + 1) // 2)
               + nw * (nw - 1) // 2 * (m + 1) + nw * (m + 1))
    else:
        nc = n + m + 1
        fma = (sum((n - k - 1) * (nc - k - 1) for k in range(n)) + n * (n - 1) // 2 * (m + 1)
               + 3 * nw * (m + 1) * 3 + m * (m + 1) * nw)
    nominal = 2 * n ** 3 // 3 + 2 * n * n * (m + 1) + 2 * m * m * n
    return nbytes, 2 * fma, nominal


def c4_rooflines(H, B, tims, pc, hbm, peak_kind):
    """The dominant kernel of the timed batch step and the element kernels.  The dominant kernel is
    the instance that moves the most algorithmic bytes per step (bytes per launch x launches) in the
    kernel family with the most live time per step (mean event-timed launch x launches, summed over
    the bins): level-0 sweeps, first-coarse-level sweeps or FP64 products."""
    k = 2  # Chebyshev degree of the level-0 smoother: 2k sweeps per V-cycle
    chunk = 8
    cand = []
    for bn, t in zip(B.bins, tims):
        it = max(B.stats[i].iterations for i in bn.idx)
        it_launched = -(-it // chunk) * chunk
        nt = bn.p + 1
        if pc == H.PRECOND_AMG:
            smp = bn.kernel_sample(1)
            if smp["launches"]:
                cand.append(dict(kernel=f"k_amg_face_cheb<{nt}, __half> (level-0 Chebyshev sweep, p={bn.p} bin)",
                                 key=f"c4:k_amg_face_cheb<{nt}>", family="level-0 sweeps",
                                 mean_ms=smp["ms"] / smp["launches"],
                                 bytes_per_launch=smp["bytes"] / smp["launches"], launches=it_launched * 2 * k,
                                 full_launch_bytes=bn.ndofs * (5 * 2 * nt + 20 / nt + 20),
                                 sampled_launches=smp["launches"]))
                # the first coarse level's l1-Jacobi sweeps, timed in the same sampled chunks
                l1 = bn.kernel_sample(2)
                if l1["launches"]:
                    per_it = l1["launches"] / (smp["launches"] / (2 * k))  # sweeps per V-cycle
                    cand.append(dict(kernel=f"k_amg_l1_sweep<4> (first coarse level, p={bn.p} bin)",
                                     key="c4:k_amg_l1_sweep<4>", family="coarse sweeps",
                                     mean_ms=l1["ms"] / l1["launches"],
                                     bytes_per_launch=l1["bytes"] / l1["launches"], launches=it_launched * per_it,
                                     full_launch_bytes=None, sampled_launches=l1["launches"]))
        if t["cg_samples"]:
            cand.append(dict(kernel=f"k_cg_a<{nt}, double> (FP64 q = A z + beta q, p={bn.p} bin)", key=f"c4:k_cg_a<{nt}>",
                             family="FP64 products", mean_ms=t["cg_a_ms"], bytes_per_launch=t["cg_a_bytes"], launches=it_launched,
                             full_launch_bytes=bn.ndofs * (40 * nt + 20 / nt + 40), sampled_launches=t["cg_samples"]))
    for c in cand:
        c["est_ms_per_step"] = c["mean_ms"] * c["launches"]
        c["est_bytes_per_step"] = c["bytes_per_launch"] * c["launches"]
    # the family with the most live time per step (summed over the bins), then its instance that
    # moves the most bytes
    fam_ms = {}
    for c in cand:
        fam_ms[c["family"]] = fam_ms.get(c["family"], 0.0) + c["est_ms_per_step"]
    top = max(fam_ms, key=fam_ms.get) if fam_ms else None
    fam = [c for c in cand if c["family"] == top]
    dom = max(fam, key=lambda c: c["est_bytes_per_step"]) if fam else None
    rl = None
    if dom:
        ach = dom["bytes_per_launch"] / (dom["mean_ms"] / 1e3) / 1e9
        rl = {"kernel": dom["kernel"], "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
              "traffic": profile_traffic(dom["key"]), "algorithmic_bytes_per_launch": dom["bytes_per_launch"],
              "avg_launch_ms": dom["mean_ms"], "sampled_launches": dom["sampled_launches"],
              "algorithmic_bytes_per_full_launch": dom["full_launch_bytes"],
              "est_ms_per_step": dom["est_ms_per_step"],
              "family": dom["family"], "family_ms_per_step": fam_ms,
              "how": "CUDA events around each launch of the sampled (un-graphed) CG chunks of the timed step, on "
                     "the bin's stream while the other bins run; bytes = rows of the problems that iterated x "
                     "bytes per row; traffic: ncu dram read+write per launch of the same kernel in the same bench "
                     "command at the full row count (compare with algorithmic_bytes_per_full_launch)",
              "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else
              "fallback 6.8 TB/s",
              "others": [{kk: c[kk] for kk in ("kernel", "mean_ms", "bytes_per_launch", "launches", "est_ms_per_step")}
                         for c in sorted(cand, key=lambda c: -c["est_ms_per_step"])[:6]]}
    # the level-0 sweep, the largest HBM stream of the cycle, beside it (its traffic is captured)
    l0 = [c for c in cand if c["family"] == "level-0 sweeps"]
    if rl is not None and l0 and dom["family"] != "level-0 sweeps":
        c0 = max(l0, key=lambda c: c["est_bytes_per_step"])
        a0 = c0["bytes_per_launch"] / (c0["mean_ms"] / 1e3) / 1e9
        rl["level0_sweep"] = {"kernel": c0["kernel"], "achieved": a0, "frac": a0 / hbm,
                              "traffic": profile_traffic(c0["key"]),
                              "algorithmic_bytes_per_launch": c0["bytes_per_launch"], "avg_launch_ms": c0["mean_ms"],
                              "algorithmic_bytes_per_full_launch": c0["full_launch_bytes"]}
    el = []
    tot_b = tot_f = tot_nom = tot_ms = 0.0
    for bn, t in zip(B.bins, tims):
        schur = bn.p != 2
        nb, fl, nom = element_cost(bn.p, schur)
        cells = bn.mesh.ncells
        ms = t["element_ms"]
        el.append({"p": bn.p, "path": "cholesky-schur" if schur else "full LU", "cells": cells, "ms": ms,
                   "elements_per_s": cells / (ms / 1e3) if ms else None,
                   "gbs": cells * nb / (ms / 1e3) / 1e9 if ms else None,
                   "fp64_tflops": cells * fl / (ms / 1e3) / 1e12 if ms else None})
        tot_b += cells * nb
        tot_f += cells * fl
        tot_nom += cells * nom
        tot_ms += ms
    ach = tot_b / (tot_ms / 1e3) / 1e9 if tot_ms else None
    rl_el = {"kernel": "k_element_chol (p=1,3,4) + k_element_condense (p=2), all bins", "bound": "fp64 pipe",
             "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm if ach else None,
             "fp64_tflops": tot_f / (tot_ms / 1e3) / 1e12 if tot_ms else None,
             "fp64_peak_tflops": FP64_TFLOPS_MEASURED,
             "fp64_frac": tot_f / (tot_ms / 1e3) / 1e12 / FP64_TFLOPS_MEASURED if tot_ms else None,
             "nominal_dense_lu_tflops": tot_nom / (tot_ms / 1e3) / 1e12 if tot_ms else None,
             "ms_sum_of_bins": tot_ms, "bins": el,
             "elements_per_s": sum(b["cells"] for b in el) / (tot_ms / 1e3) if tot_ms else None,
             "how": "element kernel of each bin timed with CUDA events in the timed step (bins run concurrently, so "
                    "each kernel shares the GPU); HBM fraction of measured copy bandwidth and FP64 fraction of the "
                    "measured FMA rate"}
    return rl, rl_el


def run_c4(args, ws, rank, local):
    """Batched workload: the degree-binned batch (one launch sequence for all problems of a
    degree, interleaved CG) against the plain FP64 path that solves the problems one at a time."""
    import numpy as np
    import torch

    import __graft_entry__ as g
    g.build()
    H = g.import_package()
    torch.cuda.set_device(local)
    ctx = H.Context(local)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    probs = c4_problems(H)
    prec = H.PREC_FP64 if args.precision == "fp64" else H.PREC_MIXED
    pc = H.PRECOND_AMG if args.preconditioner == "amg" else H.PRECOND_JACOBI
    tol = args.tol if args.tol != 1e-12 else 1e-9
    ncells = sum(2 * pr.n * pr.n for pr in probs)

    # plain FP64 path: one resident system per problem, solved one after another
    plain = []
    for pr in probs:
        m = H.batch.host_mesh(pr)
        dm = H.rectangle_mesh(H.TriangleCell, (pr.n, pr.n), pr.LL, pr.UR, ctx=ctx)
        dm.set_coordinates(m._topology()[0])
        fe = H.GenericFiniteElement(H.Dubiner(2, H.RefTetrahedron, pr.p))
        Wh = H.ScalarFunctionSpace(dm, fe, quad_degree=pr.qd())
        Vh = H.VectorFunctionSpace(dm, fe, quad_degree=pr.qd())
        Mh = H.ScalarTraceFunctionSpace(Wh, H.GenericFiniteElement(H.Legendre(1, H.RefTetrahedron, pr.p)))
        K, b, _, _ = H.doassemble(Vh, Wh, Mh, pr.tau, pr.f, kappa_cell=pr.kappa_cell)
        dbc = H.Dirichlet(H.TrialFunction(Mh), dm, "boundary")
        plain.append((dm, K, dbc, pr))

    def plain_step(keep=False, tol_=tol, pc_=None):
        out = []
        for dm, K, dbc, pr in plain:
            K.reassemble(resident=True)
            K.apply_dirichlet(dbc.prescribed_dofs, dbc.values)
            uh = K.solve(tol=tol_, precision=H.PREC_FP64, to_host=keep, preconditioner=pc if pc_ is None else pc_)
            r = K.recover(to_host=keep)
            if keep:
                out.append((uh, r[0], r[1]))
        return out

    B = H.Batch(ctx, probs, precision=prec)
    for _ in range(max(args.warmup, 3)):
        B.solve(tol=tol, reassemble="resident", preconditioner=pc)
    plain_step()
    torch.cuda.synchronize()

    # ---- timed region: meshes, coefficients and Dirichlet data resident on the device ----
    ctx.set_profiling(True)
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = ctx.launches()
    barrier(ws)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    steps_ms = []
    e0.record(stream)
    for _ in range(args.steps):
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        B.solve(tol=tol, reassemble="resident", preconditioner=pc)
        s1.record(stream)
        s1.synchronize()
        steps_ms.append(s0.elapsed_time(s1))
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(ws)
    launches = ctx.launches() - launches0
    ctx.set_profiling(False)
    clk = clocks.stop()
    batch_ms = max_over_ranks(e0.elapsed_time(e1), ws) / args.steps
    value = ws * len(probs) / (batch_ms / 1e3)
    iters = [s.iterations for s in B.stats]

    # ---- rooflines, from the last timed step (profiling on: every 8th CG chunk of each bin runs
    # un-graphed with each kernel timed on its own, on the bin's stream, while the other bins run) ----
    peaks, peak_kind = measured_peaks()
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    tims = [bn.timings() for bn in B.bins]
    bins_detail = [{"p": bn.p, "problems": len(bn.problems), "cells": bn.mesh.ncells, "trace_dofs": bn.ndofs,
                    "element_ms": t["element_ms"], "cg_ms": t["cg_ms"],
                    "cg_iterations_max": max(B.stats[i].iterations for i in bn.idx)}
                   for bn, t in zip(B.bins, tims)]
    cg_ms = max(t["cg_ms"] for t in tims)
    cg_bytes = sum(t["cg_bytes"] for t in tims)
    el_ms = sum(t["element_ms"] for t in tims)
    rl, rl_element = c4_rooflines(H, B, tims, pc, hbm, peak_kind)
    # ---- plain path, one timed pass over the batch ----
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    plain_step()
    p1.record(stream)
    torch.cuda.synchronize()
    plain_ms = p0.elapsed_time(p1)

    # ---- accuracy against the plain FP64 path at tolerance 1e-12 ----
    ref = plain_step(keep=True, tol_=1e-12, pc_=H.PRECOND_JACOBI)
    sols = B.solutions()
    err = max(max(rel_l2(a[0], b[0]), rel_l2(a[1], b[1]), rel_l2(a[2], b[2])) for a, b in zip(sols, ref))

    # ---- end to end through the public API with host buffers ----
    def e2e_step():
        # H2D: kappa, sources, tau, Dirichlet data; D2H inside the step: uhat, q, u of every
        # problem into page-locked host arrays, each bin as soon as it is recovered
        res = B.solve(tol=tol, reassemble=True, preconditioner=pc, download=True)
        return res, B.solutions(downloaded=True)
    e2e_step()
    torch.cuda.synchronize()
    barrier(ws)
    t0 = time.perf_counter()
    e2e_n = max(2, args.steps // 3)
    for _ in range(e2e_n):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, ws)
    h2d = sum(bn.kc.nbytes if bn.kc is not None else 0 for bn in B.bins) + sum(
        8 * (len(pr.f.params) + 1) for pr in probs) + sum(bn.dofs.nbytes + bn.vals.nbytes for bn in B.bins)
    d2h = sum(8 * (bn.ndofs + bn.mesh.ncells * bn.n) for bn in B.bins)

    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": batch_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64" if prec == H.PREC_MIXED else "f64", "data": "synthetic",
        "config": {"workload": C4_DESC + f"; degree-binned batch, {args.precision}, {args.preconditioner}-preconditioned "
                               f"CG tol {tol:g}",
                   "problems": len(probs), "cells": ncells, "tol": tol,
                   "quadrature": "Strang(p+1) for p<=2, Strang(6) for p=3, Grundmann-Moeller(9) for p=4",
                   "step": "assemble+condense (coefficients resident) -> apply! -> CG -> recovery of all 256 problems",
                   "l2": "inputs larger than L2: every step rewrites the condensed blocks of 1.6M cells",
                   "parallelism": f"{ws} independent replica(s), one per GPU"},
        "p50_ms": statistics.median(steps_ms), "p99_ms": max(steps_ms),
        "plain_fp64_solves_per_s": len(probs) / (plain_ms / 1e3),
        "plain_path": f"one problem at a time: reassemble, apply!, FP64 {args.preconditioner}-preconditioned CG, recovery",
        "speedup_vs_plain": (len(probs) / (batch_ms / 1e3)) / (len(probs) / (plain_ms / 1e3)),
        "max_rel_l2_err_vs_fp64": err,
        "converged_fraction": float(np.mean([s.converged for s in B.stats])),
        "max_rel_residual": float(max(s.rel_residual for s in B.stats)),
        "cg_iterations_max": max(iters), "cg_iterations_mean": float(np.mean(iters)),
        "phase_ms": {"element_ms_sum_of_bins": el_ms, "cg_ms_longest_bin": cg_ms},
        "bins": bins_detail,
        "gpu_launches": launches,
        "roofline": rl, "roofline_element": rl_element,
        "cg_phase": {"algorithmic_bytes": cg_bytes, "wall_ms_longest_bin": cg_ms,
                     "achieved_gbs": cg_bytes / (cg_ms / 1e3) / 1e9 if cg_ms > 0 else None,
                     "note": "all CG iteration launches of all bins (concurrent streams) / the longest bin's CG wall time"},
        "e2e": {"value": ws * len(probs) * e2e_n / e2e_s, "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "clocks": clk,
    }
    # ---- the same kind of problems as a request stream through the serving engine: 2000 req/s for
    # the completed rate, 250 req/s (below saturation) for the service latency ----
    if not args.no_serving:
        del B
        plain.clear()
        gc.collect()
        torch.cuda.synchronize()
        kw = dict(tol=tol, precision=args.precision, preconditioner=args.preconditioner,
                  hbm_budget_gb=args.hbm_budget_gb, max_batch=args.max_batch, max_flights=args.max_flights,
                  seed=777 + rank, plain_sample=0)
        line["serving"] = {
            "workload": SERVE_DESC + f", {args.precision}, {args.preconditioner}-preconditioned CG tol {tol:g}; "
                                     "requests enter as host arrays and results are read back to host memory",
            "at_2000_req_per_s": serve_stream(H, ctx, local, 2000.0, 1000, **kw),
            "at_250_req_per_s": serve_stream(H, ctx, local, 250.0, 500, accuracy_sample=6, **kw)}

    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        specs = c4_specs()
        idx = c4_cpu_sample_indices(specs)
        pool = OraclePool()
        wall, per, res = pool.run(specs, idx, keep=True)
        pool.close()
        line["cpu_baseline"] = {
            "value": len(idx) / wall, "unit": "solves/s", "cores": pool.workers, "kind": "port",
            "single_thread_value": len(idx) / sum(per),
            "sample": f"a fixed stratified sample of {len(idx)} of the 256 problems (the middle problem of each "
                      f"1/{len(idx)} of the batch by size), each solved completely by the single-threaded C++ "
                      f"oracle (element loop, COO->CSC, apply!, SuperLU direct solve, recovery) on a pool of "
                      f"{pool.workers} worker processes, largest first: {wall:.1f} s wall; single_thread_value = "
                      f"problems / the sum of the per-problem times ({sum(per):.1f} s)"}
        line["max_rel_l2_err_vs_cpu_oracle"] = max(
            max(rel_l2(sols[k][0], r["uhat"]), rel_l2(sols[k][2].ravel(), r["u"].ravel())) for k, r in zip(idx, res))
    if rank == 0:
        print(json.dumps(line), flush=True)


C3_DESC = ("c3: 2·512·512=524288 triangles, interior nodes jittered U(-0.2h,0.2h) (seeded), p=3, "
           "kappa=exp(g) with g 64 random Fourier modes of wavelength >= 0.1 and RMS 1 (seeded), f a random smooth "
           "Fourier field; mixed CG against the FP64 run")


def c3_fields(H, seed=31337, modes=64):
    """kappa = exp(g) and f for the precision workload: g = sum a_k cos(2 pi k.x + phi_k) with
    integer-free wave vectors |k| <= 10 (wavelength >= 0.1) and a_k ~ N(0, 1/32) (RMS of g = 1);
    f is built the same way (no exponential) from another stream, scaled by 10."""
    import numpy as np
    rng = np.random.default_rng(seed)

    def draw(scale):
        ang = rng.uniform(0, 2 * math.pi, modes)
        rad = 10.0 * np.sqrt(rng.uniform(0, 1, modes))
        ph = rng.uniform(0, 2 * math.pi, modes)
        a = scale * rng.standard_normal(modes) / math.sqrt(32.0)
        return np.stack([rad * np.cos(ang), rad * np.sin(ang), ph, a], axis=1)
    kappa = H.Field.fourier(0.0, draw(1.0), exponential=True)
    f = H.Field.fourier(0.0, draw(10.0))
    return kappa, f


def run_c3(args, ws, rank, local):
    """Precision workload: the FP64 and the mixed trace solve of one large jittered, variable-kappa
    problem; reports the mixed run's solves/s and its relative L2 differences from the FP64 run."""
    import numpy as np
    import torch

    import __graft_entry__ as g
    g.build()
    H = g.import_package()
    torch.cuda.set_device(local)
    ctx = H.Context(local)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    n, p, qd = 512, 3, 6
    mesh = H.rectangle_mesh(H.TriangleCell, (n, n), (0.0, 0.0), (1.0, 1.0), ctx=ctx)
    mesh.jitter(0.2, 20240611)
    kappa, f = c3_fields(H)
    fe = H.GenericFiniteElement(H.Dubiner(2, H.RefTetrahedron, p))
    Wh = H.ScalarFunctionSpace(mesh, fe, quad_degree=qd)
    Vh = H.VectorFunctionSpace(mesh, fe, quad_degree=qd)
    Mh = H.ScalarTraceFunctionSpace(Wh, H.GenericFiniteElement(H.Legendre(1, H.RefTetrahedron, p)))
    K, b, _, _ = H.doassemble(Vh, Wh, Mh, 1.0, f, kappa=kappa)
    dbc = H.Dirichlet(H.TrialFunction(Mh), mesh, "boundary")
    tol = args.tol if args.tol != 1e-12 else 1e-10

    def run(prec, tol_, keep, pc=H.PRECOND_JACOBI):
        K.reassemble(resident=True)
        K.apply_dirichlet(dbc.prescribed_dofs, dbc.values)
        uh = K.solve(tol=tol_, precision=prec, to_host=keep, preconditioner=pc)
        r = K.recover(to_host=keep)
        return (uh, r[0], r[1]) if keep else None

    ref = run(H.PREC_FP64, 1e-12, True)
    it64 = K.stats.iterations
    for _ in range(max(args.warmup, 3) - 1):
        run(H.PREC_MIXED, tol, False)
    got = run(H.PREC_MIXED, tol, True)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = ctx.launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        run(H.PREC_MIXED, tol, False)
    e1.record(stream)
    torch.cuda.synchronize()
    launches = ctx.launches() - launches0
    clk = clocks.stop()
    ms = max_over_ranks(e0.elapsed_time(e1), ws) / args.steps
    itm = K.stats.iterations
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    run(H.PREC_FP64, tol, False)
    f1.record(stream)
    torch.cuda.synchronize()
    # the same solve with the multigrid preconditioner: FP64 CG around an FP32 V-cycle
    gmg = run(H.PREC_MIXED, tol, True, H.PRECOND_AMG)
    itg = K.stats.iterations
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0.record(stream)
    for _ in range(args.steps):
        run(H.PREC_MIXED, tol, False, H.PRECOND_AMG)
    g1.record(stream)
    torch.cuda.synchronize()
    line = {
        "metric": METRIC, "value": ws * 1e3 / ms, "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": C3_DESC, "n": n, "p": p, "quad_degree": qd, "cells": mesh.ncells,
                   "trace_dofs": K.ndofs, "nnz": K.nnz, "tol": tol,
                   "l2": "inputs larger than L2: the condensed blocks (2.3 GB) are rewritten every step"},
        "rel_l2_vs_fp64": {"uhat": rel_l2(got[0], ref[0]), "q": rel_l2(got[1].ravel(), ref[1].ravel()),
                           "u": rel_l2(got[2].ravel(), ref[2].ravel())},
        "fp64_solves_per_s": 1e3 / f0.elapsed_time(f1), "cg_iterations_mixed": itm, "cg_iterations_fp64": it64,
        "multigrid": {"solves_per_s": args.steps * 1e3 / g0.elapsed_time(g1), "cg_iterations": itg,
                      "what": "FP64 CG preconditioned by the FP32 smoothed-aggregation V-cycle, same tolerance",
                      "rel_l2_vs_fp64": {"uhat": rel_l2(gmg[0], ref[0]), "q": rel_l2(gmg[1].ravel(), ref[1].ravel()),
                                         "u": rel_l2(gmg[2].ravel(), ref[2].ravel())}},
        "gpu_launches": launches, "clocks": clk,
        "cpu_baseline": None,
        "cpu_baseline_note": "not measured for this workload: the oracle's sparse direct solve of 3.1 M trace dofs "
                             "does not fit a bounded CPU sample",
    }
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        # the FP64 device assembly of the full configuration against the oracle's (no direct solve:
        # the solution is compared on 2*128^2 cells in tests/test_gpu_parity.py)
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import hdgref
        K.reassemble(resident=True)
        K.apply_dirichlet(dbc.prescribed_dofs, dbc.values)
        t0 = time.perf_counter()
        om = hdgref.rectangle_mesh(n, n)
        om.set_xy(H.get_vertices_matrix(mesh))
        S = hdgref.System(om, p, qd, 1.0, f.as_oracle(), kappa.as_oracle(), None, threads=os.cpu_count() or 1)
        S.apply(*S.dirichlet())
        line["parity_vs_oracle"], _, _ = matrix_parity(K, S, dbc.prescribed_dofs)
        line["parity_vs_oracle"]["oracle_assembly_s"] = time.perf_counter() - t0
    if rank == 0:
        print(json.dumps(line), flush=True)


def draw_shape(rng):
    n = int(round(math.exp(rng.uniform(math.log(8), math.log(128)))))
    return n, int(rng.integers(1, 5))


def draw_coefficients(H, rng, n):
    import numpy as np
    f = H.Field.bumps(rng.random((8, 2)), 0.03 + 0.12 * rng.random(8), 10.0 * rng.standard_normal(8))
    kc = np.exp(rng.uniform(math.log(1e-2), math.log(1e2), 2 * n * n))
    return f, kc


def serve_stream(H, ctx, local, rate, nreq, *, tol, precision, preconditioner, hbm_budget_gb, max_batch,
                 max_flights, warmup=3, seed=777, plain_sample=48, accuracy_sample=12):
    """A Poisson stream of `nreq` solve requests at `rate` req/s (seeded) through the serving engine.
    Each request is drawn like the batching workload; 70 % reuse one of 32 resident meshes with a new
    source and coefficient, 30 % come with a new mesh.  Requests enter as host arrays and every result
    is read back to host memory, so the completed rate is an end-to-end figure.  Returns the measured
    figures; `plain_sample` requests are also solved one at a time by the plain FP64 path for the
    speed-up, and `accuracy_sample` completed requests are checked against FP64 solves at 1e-12."""
    import numpy as np
    import torch

    if not rate > 0:
        raise SystemExit("--rate must be positive")
    rng = np.random.default_rng(seed)
    resident = []
    for k in range(32):
        n, p = draw_shape(rng)
        resident.append(H.Problem(n=n, p=p, f=H.Field.const(1.0), jitter=0.2, seed=9000 + k))
    reqs = []
    t = 0.0
    for k in range(nreq):
        t += rng.exponential(1.0 / rate)
        if rng.random() < 0.7:
            mid = int(rng.integers(0, 32))
            pr = resident[mid]
            f, kc = draw_coefficients(H, rng, pr.n)
            reqs.append(dict(t=t, mid=mid, n=pr.n, p=pr.p, f=f, kc=kc, mesh=None, seed=pr.seed))
        else:
            n, p = draw_shape(rng)
            f, kc = draw_coefficients(H, rng, n)
            sd = 50000 + k
            reqs.append(dict(t=t, mid=-1, n=n, p=p, f=f, kc=kc, seed=sd,
                             mesh=H.batch.host_mesh(H.Problem(n=n, p=p, f=f, jitter=0.2, seed=sd))))
    for r in reqs:
        # bytes a request carries to the device: kappa per cell, the source's parameters and, for a new
        # mesh, its coordinates and connectivity
        r["h2d"] = np.asarray(r["kc"]).nbytes + 8 * (len(r["f"].params) + 1) + (
            sum(a.nbytes for a in r["mesh"]._topology()) if r["mesh"] is not None else 0)

    pc = H.PRECOND_AMG if preconditioner == "amg" else H.PRECOND_JACOBI
    eng = H.Engine(ctx, hbm_budget_gb=hbm_budget_gb, max_batch=max_batch, max_flights=max_flights,
                   tol=tol, precision=H.PREC_MIXED if precision == "mixed" else H.PREC_FP64, keep_results=True,
                   preconditioner=pc)
    host_res = [H.batch.host_mesh(pr) for pr in resident]
    mids = [eng.add_resident(hm, pr.p) for hm, pr in zip(host_res, resident)]

    def submit(r):
        if r["mid"] >= 0:
            return eng.submit(r["p"], r["f"], r["kc"], mesh_id=mids[r["mid"]])
        return eng.submit(r["p"], r["f"], r["kc"], mesh=r["mesh"])

    # warm-up: a short burst through the engine (compiles graphs, fills the memory pool)
    for w in range(max(warmup, 3)):
        for r in reqs[w * 16:(w + 1) * 16]:
            submit(r)
        for d in eng.run_until_idle():
            eng.result(d["id"])
    torch.cuda.synchronize()

    sample = set(range(0, nreq, max(1, nreq // max(1, accuracy_sample)))) if accuracy_sample else set()
    id2k, kept = {}, {}
    lat, its, res, conv = [], [], [], []
    h2d = d2h = 0
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = ctx.launches()
    t0 = time.perf_counter()
    i = ndone = 0
    t_last = 0.0
    while ndone < nreq:
        now = time.perf_counter() - t0
        while i < nreq and reqs[i]["t"] <= now:
            id2k[submit(reqs[i])] = i
            i += 1
        if i < nreq and eng.inflight == 0 and eng.pending == 0 and ndone == i:
            time.sleep(max(0.0, min(reqs[i]["t"] - now, 0.001)))
            continue
        eng.step()
        for d in eng.poll():
            k = id2k[d["id"]]
            uh, q, u = eng.result(d["id"])
            r = reqs[k]
            h2d += r["h2d"]
            d2h += uh.nbytes + q.nbytes + u.nbytes
            if k in sample:
                kept[k] = (uh, q, u)
            lat.append(d["latency"])
            its.append(d["iterations"])
            res.append(d["rel_residual"])
            conv.append(d["converged"])
            ndone += 1
            t_last = time.perf_counter() - t0
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    launches = ctx.launches() - launches0
    eng.close()
    first = reqs[0]["t"]
    served = nreq / (t_last - first)
    lat_ms = sorted(1e3 * x for x in lat)

    # plain FP64 path on a sample of the same requests, one at a time, and the accuracy check
    def plain_solve(r, tol_):
        pr = H.Problem(n=r["n"], p=r["p"], f=r["f"], kappa_cell=r["kc"], jitter=0.2, seed=r["seed"])
        hm = H.batch.host_mesh(pr)
        dm = H.rectangle_mesh(H.TriangleCell, (pr.n, pr.n), ctx=ctx)
        dm.set_coordinates(hm._topology()[0])
        fe = H.GenericFiniteElement(H.Dubiner(2, H.RefTetrahedron, pr.p))
        Wh = H.ScalarFunctionSpace(dm, fe, quad_degree=pr.qd())
        Vh = H.VectorFunctionSpace(dm, fe, quad_degree=pr.qd())
        Mh = H.ScalarTraceFunctionSpace(Wh, H.GenericFiniteElement(H.Legendre(1, H.RefTetrahedron, pr.p)))
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        K, b, _, _ = H.doassemble(Vh, Wh, Mh, 1.0, pr.f, kappa_cell=pr.kappa_cell)
        H.apply_(K, b, H.Dirichlet(H.TrialFunction(Mh), dm, "boundary"))
        uh = H.solve(K, b, tol=tol_, precision=H.PREC_FP64, preconditioner=pc)
        q, u, _ = K.recover()
        t2 = time.perf_counter()
        return t2 - t1, (uh, q, u)

    errs = []
    for k, got in kept.items():
        _, ref = plain_solve(reqs[k], 1e-12)
        errs.append(max(rel_l2(got[0], ref[0]), rel_l2(got[1].ravel(), ref[1].ravel()),
                        rel_l2(got[2].ravel(), ref[2].ravel())))
    out = {
        "rate_req_per_s": rate, "requests": nreq, "completed_per_s": served,
        "ms_per_request": 1e3 * (t_last - first) / nreq,
        "p50_ms": lat_ms[len(lat_ms) // 2], "p99_ms": lat_ms[min(len(lat_ms) - 1, int(0.99 * len(lat_ms)))],
        "h2d_bytes_per_request": h2d / nreq, "d2h_bytes_per_request": d2h / nreq,
        "max_rel_l2_err_vs_fp64": max(errs) if errs else None, "accuracy_sample": len(errs),
        "all_converged": bool(all(conv)), "max_rel_residual": float(max(res)),
        "cg_iterations_mean": float(np.mean(its)), "wall_s": wall, "gpu_launches": launches, "clocks": clk,
    }
    if plain_sample:
        plain_t = [plain_solve(reqs[k], tol)[0] for k in range(0, min(nreq, plain_sample))]
        out["plain_fp64_solves_per_s"] = len(plain_t) / sum(plain_t)
        out["plain_fp64_p50_ms"] = 1e3 * statistics.median(plain_t)
    return out


SERVE_DESC = ("c5: Poisson request stream (seeded), each request drawn like the batching workload; 70% on one of "
              "32 resident meshes with a new source and kappa, 30% new meshes; continuous batching")


def run_c5(args, ws, rank, local):
    """Serving workload: the request stream of serve_stream at --rate (2000 req/s by default)."""
    import torch

    import __graft_entry__ as g
    g.build()
    H = g.import_package()
    torch.cuda.set_device(local)
    ctx = H.Context(local)
    tol = args.tol if args.tol != 1e-12 else 1e-9
    s = serve_stream(H, ctx, local, args.rate, args.requests, tol=tol, precision=args.precision,
                     preconditioner=args.preconditioner, hbm_budget_gb=args.hbm_budget_gb, max_batch=args.max_batch,
                     max_flights=args.max_flights, warmup=args.warmup, seed=777 + rank)
    line = {
        "metric": METRIC, "value": s["completed_per_s"], "unit": "solves/s", "n_gpus": ws, "steps": s["requests"],
        "warmup": max(args.warmup, 3), "ms_per_step": s["ms_per_request"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if args.precision == "mixed" else "f64",
        "data": "synthetic",
        "config": {"workload": SERVE_DESC + f" at {args.rate:g} req/s, {args.precision}, {args.preconditioner}-"
                               f"preconditioned CG tol {tol:g}",
                   "requests": s["requests"], "hbm_budget_gb": args.hbm_budget_gb, "max_batch": args.max_batch,
                   "max_flights": args.max_flights, "step": "one request solved"},
        "p50_ms": s["p50_ms"], "p99_ms": s["p99_ms"],
        "plain_fp64_solves_per_s": s["plain_fp64_solves_per_s"],
        "plain_fp64_p50_ms": s["plain_fp64_p50_ms"],
        "speedup_vs_plain": s["completed_per_s"] / s["plain_fp64_solves_per_s"],
        "max_rel_l2_err_vs_fp64": s["max_rel_l2_err_vs_fp64"], "accuracy_sample": s["accuracy_sample"],
        "all_converged": s["all_converged"], "cg_iterations_mean": s["cg_iterations_mean"], "wall_s": s["wall_s"],
        "e2e": {"value": s["completed_per_s"], "unit": "solves/s",
                "h2d_bytes_per_step": int(s["h2d_bytes_per_request"]),
                "d2h_bytes_per_step": int(s["d2h_bytes_per_request"]),
                "note": "requests enter as host arrays and results are read back to host memory"},
        "gpu_launches": s["gpu_launches"], "clocks": s["clocks"],
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


CG_DESC = ("cg: examples/poisson2D_CG.jl scaled: -div grad u = 2 pi^2 sin(pi x) sin(pi y) on 2*n*n triangles, "
           "nodal ContinuousLagrange of order p, DofHandler numbering, homogeneous Dirichlet, Jacobi-PCG to 1e-12")


def run_cg(args, ws, rank, local):
    """The continuous-Galerkin Poisson path (examples/poisson2D_CG.jl): element loop and assemble!
    into the DofHandler's CSC pattern, apply!, Jacobi-PCG and errornorm, on the device."""
    import numpy as np
    import torch

    import __graft_entry__ as g
    g.build()
    H = g.import_package()
    torch.cuda.set_device(local)
    ctx = H.Context(local)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    n = args.n or 256
    order = args.p or 2
    mesh = H.rectangle_mesh(H.TriangleCell, (n, n), (0.0, 0.0), (1.0, 1.0), ctx=ctx)
    Wh = H.ScalarFunctionSpace(mesh, H.ContinuousLagrange(2, H.RefTetrahedron, order), update_face_data=False)
    u_h = H.TrialFunction(Wh)
    dh = H.DofHandler([u_h], mesh)
    K0 = H.create_sparsity_pattern(dh)
    dbc = H.Dirichlet(u_h, dh, "boundary", lambda x: 0.0)
    K = H.LagrangeSystem(Wh, K0, dh)
    dh._lagrange_system = K
    tol = args.tol

    def step():
        t = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        t[0].record(stream)
        K.assemble(H.MANUFACTURED_F)                         # element loop + assemble!
        t[1].record(stream)
        K.apply_dirichlet(dbc.prescribed_dofs, dbc.values)   # apply!
        t[2].record(stream)
        u = K.solve(tol=tol)                                 # K \ b, u to the host
        t[3].record(stream)
        return u, t

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = ctx.launches()
    barrier(ws)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    phases = []
    for _ in range(args.steps):
        u, t = step()
        phases.append(t)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(ws)
    launches = ctx.launches() - launches0
    clk = clocks.stop()
    ms = max_over_ranks(e0.elapsed_time(e1), ws) / args.steps
    value = ws * 1e3 / ms
    asm_ms = statistics.mean(a.elapsed_time(b) for a, b, _, _ in phases)
    apply_ms = statistics.mean(b.elapsed_time(c) for _, b, c, _ in phases)
    solve_ms = statistics.mean(c.elapsed_time(d) for _, _, c, d in phases)
    its = K.stats.iterations
    H.reconstruct_(u_h, u, dh)
    err = H.errornorm(u_h, H.MANUFACTURED_U)
    # roofline of the PCG (two kernels per iteration): the CSC values and row indices, the column
    # pointers, and the vectors (z, p_old gathered; p_new, q written; x, r read and written; z
    # written; D^-1 read) once each
    nd, nnz = K.ndofs, K.nnz
    it_bytes = nnz * (8 + 4) + (nd + 1) * 4 + nd * 8 * (2 + 2 + 4 + 1 + 1)
    peaks, peak_kind = measured_peaks()
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    achieved = it_bytes * its / (solve_ms / 1e3) / 1e9 if solve_ms > 0 else None
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": CG_DESC, "n": n, "order": order, "cells": mesh.ncells, "dofs": nd, "nnz": nnz,
                   "tol": tol, "step": "assemble (element loop + assemble!) -> apply! -> PCG -> u to the host",
                   "parallelism": f"{ws} independent replica(s), one per GPU"},
        "cg_iterations": its, "errornorm_sq": err,
        "phase_ms": {"assemble_ms": asm_ms, "apply_ms": apply_ms, "solve_ms": solve_ms},
        "gpu_launches": launches,
        "roofline": {"kernel": "k_lag_cg_a + k_lag_cg_b (one PCG iteration)", "bound": "hbm", "achieved": achieved,
                     "peak": hbm, "unit": "GB/s", "frac": (achieved / hbm) if achieved else None, "traffic": None,
                     "algorithmic_bytes_per_iteration": it_bytes, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": int(dbc.prescribed_dofs.nbytes + dbc.values.nbytes),
                "d2h_bytes_per_step": int(nd * 8)},
        "clocks": clk,
    }
    if rank == 0 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import cgref
        import hdgref
        ns = min(n, 48)
        om = hdgref.rectangle_mesh(ns, ns)
        t0 = time.perf_counter()
        r = cgref.solve_poisson_cg(om, order)
        dt = time.perf_counter() - t0
        scale = (ns * ns) / (n * n)
        line["cpu_baseline"] = {"value": scale / dt, "unit": "solves/s", "cores": 1, "kind": "port",
                                "sample": f"one complete solve of the {ns}x{ns} (2*{ns}^2 cells) order-{order} problem by "
                                          f"the numpy/SuperLU CG oracle in {dt:.2f} s, rate scaled by the cell ratio "
                                          f"{scale:.4f} (the direct solve grows faster than linearly, so this favours the CPU)"}
        line["cpu_oracle_errornorm_sq"] = r["err"]
    if rank == 0:
        print(json.dumps(line), flush=True)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c4", choices=sorted(WORKLOADS) + ["c3", "c4", "c5", "cg"])
    ap.add_argument("--requests", type=int, default=2000)
    ap.add_argument("--rate", type=float, default=2000.0,
                    help="c5 only: mean arrival rate in requests/s (2000 is the workload; lower rates show latency "
                         "without queueing)")
    ap.add_argument("--hbm-budget-gb", type=float, default=64.0)
    ap.add_argument("--max-batch", type=int, default=32,
                    help="serving: requests per flight (measured on the 2000 req/s stream: flights x batch 8x64 831, "
                         "12x64 901, 16x64 904, 16x32 964, 16x24 947, 24x32 915, 32x16 879 completed/s)")
    ap.add_argument("--max-flights", type=int, default=16, help="serving: flights in progress at once")
    ap.add_argument("--precision", default=None, choices=["fp64", "mixed"],
                    help="default: mixed for the batched and served workloads (c3, c4, c5), fp64 for c1, c2")
    ap.add_argument("--tol", type=float, default=1e-12)
    ap.add_argument("--preconditioner", default=None, choices=["jacobi", "amg"],
                    help="trace CG preconditioner (default: amg for the batch c4 and the stream c5, jacobi "
                         "otherwise); the plain FP64 paths of c4 and c5 use the same one")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serving", action="store_true",
                    help="c4 only: leave out the request-stream figures (the serving key)")
    ap.add_argument("--n", type=int, default=None, help="c1/c2 only: cells per side (a profiling case, not a bench line)")
    ap.add_argument("--p", type=int, default=None, help="c1/c2 only: polynomial degree (a profiling case)")
    args = ap.parse_args()
    if args.precision is None:
        args.precision = "mixed" if args.workload in ("c3", "c4", "c5") else "fp64"
    if args.preconditioner is None:
        args.preconditioner = "amg" if args.workload in ("c4", "c5") else "jacobi"
    return args


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
            m = re.match(r"\s*traffic_bytes_per_launch\[([^\]]+)\]\s*[:=]\s*([0-9.eE+]+)", ln)
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
    """One complete oracle solve of the workload, timed; returns (the cpu_baseline entry, the
    oracle's result, whose system the parity check reuses)."""
    dt, r = oracle_solve_once(w["n"], w["p"], w["qd"], threads)
    return {"value": 1.0 / dt, "unit": "solves/s", "cores": threads, "kind": "port",
            "sample": f"one complete solve of the same workload ({2 * w['n'] ** 2} cells, p={w['p']}) by the "
                      f"C++ oracle: OpenMP element loop on {threads} threads, COO->CSC, apply!, SuperLU "
                      f"(single-threaded; minimum degree on A'+A with diagonal-preferring pivots, as UMFPACK's "
                      f"symmetric strategy), recovery; {dt:.2f} s"}, r


def matrix_parity(K, S, dirichlet_dofs):
    """The device trace matrix and right-hand side (after apply!) against the oracle's: pattern
    bit-exact, entries relative to their row's largest entry, except the Dirichlet diagonal (mean
    |diag K|, summed in sequence by the reference and the oracle, in a tree on the device), and the
    rhs relative to its largest entry.  Returns (figures, oracle K, oracle b)."""
    import numpy as np
    colptr, rowval, nzval, rhs = K.csc(0)
    oK, ob = S.csc()
    out = {"csc_pattern_equal": bool(np.array_equal(colptr, oK.indptr) and np.array_equal(rowval, oK.indices))}
    if not out["csc_pattern_equal"]:
        return out, oK, ob
    rows = np.asarray(oK.indices)
    rowmax = np.zeros(oK.shape[0])
    np.maximum.at(rowmax, rows, np.abs(oK.data))
    dmask = np.zeros(oK.shape[0], bool)
    dmask[np.asarray(dirichlet_dofs) - 1] = True
    ddiag = np.zeros(len(rows), bool)
    for j in np.nonzero(dmask)[0]:  # the Dirichlet diagonal entries
        lo, hi = oK.indptr[j], oK.indptr[j + 1]
        ddiag[lo + np.searchsorted(rows[lo:hi], j)] = True
    d = np.abs(nzval - oK.data) / np.maximum(rowmax[rows], 1e-300)
    out["nzval_rel_rowmax"] = float(d[~ddiag].max())
    out["dirichlet_diag_rel"] = float(d[ddiag].max()) if ddiag.any() else 0.0
    out["rhs_rel_max"] = float(np.abs(rhs - ob).max() / max(np.abs(ob).max(), 1e-300))
    out["nnz"] = int(len(rows))
    return out, oK, ob


def parity_vs_oracle(H, K, S, pc, dirichlet_dofs):
    """The device system and solution against the oracle's on the same mesh (the oracle system S
    after apply!).  Sparsity pattern bit-exact; matrix entries relative to their row's largest
    entry, except the Dirichlet diagonal, which carries mean|diag K| summed in sequence as the
    reference does (src/boundary.jl:169-175; the device sums in a tree), reported on its own; the
    trace solution of the device (CG to 1e-12, then two double-double refinement steps) against the
    oracle's SuperLU solution refined the same way: relative L2 difference and componentwise
    backward error max_i |b - K x|_i / (|K| |x| + |b|)_i in the oracle's system."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import hdgref
    out, oK, ob = matrix_parity(K, S, dirichlet_dofs)
    if not out["csc_pattern_equal"]:
        return out
    x = K.solve(tol=1e-12, preconditioner=pc, refine=2)
    q, u, _ = K.recover()
    lu = S.solve()
    xr = S.solve(refine=3)
    oq, ou, _ = S.recover(xr)
    res = hdgref.csc_residual_dd(oK, x, ob)
    den = abs(oK) @ np.abs(x) + np.abs(ob)
    out.update({"uhat_rel_l2": rel_l2(x, xr), "uhat_backward_error": float((np.abs(res) / np.maximum(den, 1e-300)).max()),
                "q_rel_l2": rel_l2(q.ravel(), oq.ravel()), "u_rel_l2": rel_l2(u.ravel(), ou.ravel()),
                "oracle_direct_vs_refined_rel_l2": rel_l2(lu, xr)})
    return out


def run_reference(args, ws, rank):
    """The reference arm: the CPU oracle (the reference's flow restated in C++ with a sparse direct
    solve) on all host cores, on the same workload.  The reference itself is Julia, which is not
    installed here, so the restatement stands in for it."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    if args.workload == "c4":
        specs = c4_specs()
        idx = c4_cpu_sample_indices(specs)
        pool = OraclePool()
        threads = pool.workers
        for _ in range(args.warmup):
            pool.run(specs, idx)
        times, per_problem = [], []
        for _ in range(args.steps):
            wall, per, _ = pool.run(specs, idx)
            times.append(wall)
            per_problem += per
        pool.close()
        tot = sum(times)
        value = len(idx) * args.steps / tot
        cfg = {"workload": C4_DESC + f"; each step solves the same fixed stratified sample of {len(idx)} of the 256 "
                                     "problems (the middle problem of each equal slice of the batch sorted by size)",
               "problems": 256, "sample_problems": len(idx), "same_config": False,
               "scaling": f"the rate of the sample stands for the batch's rate: the sample spans the batch's size "
                          f"distribution (one problem per 1/{len(idx)} quantile of the size)"}
        sample = (f"each step is the fixed stratified sample of {len(idx)} problems, each solved completely by the "
                  f"single-threaded C++ oracle (element loop, COO->CSC, apply!, SuperLU direct solve, recovery) on a "
                  f"pool of {threads} worker processes, largest first; the reference itself is Julia, which is not "
                  "installed on this machine")
        step_times = [t / len(idx) for t in times]
        single = len(per_problem) / sum(per_problem)
    else:
        w = WORKLOADS[args.workload]
        for _ in range(args.warmup):
            oracle_solve_once(w["n"], w["p"], w["qd"], threads)
        times = [oracle_solve_once(w["n"], w["p"], w["qd"], threads)[0] for _ in range(args.steps)]
        tot = sum(times)
        value = args.steps / tot
        cfg = {"workload": f"{args.workload}: {w['desc']}", "n": w["n"], "p": w["p"]}
        sample = ("each step is one complete solve of the workload by the C++ oracle (OpenMP element loop, COO->CSC, "
                  "apply!, SuperLU direct solve, recovery); the reference itself is Julia, which is not installed on "
                  "this machine")
        step_times = times
        single = None
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port", "sample": sample,
                         "single_thread_value": single},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "p50_ms": 1e3 * statistics.median(step_times), "p99_ms": 1e3 * max(step_times),
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- our arm
def run_ours(args, ws, rank, local):
    import numpy as np
    import torch

    import __graft_entry__ as g
    g.build()
    H = g.import_package()
    w = dict(WORKLOADS[args.workload])
    if args.n or args.p:
        w["n"], w["p"] = args.n or w["n"], args.p or w["p"]
        w["qd"] = {3: 6, 4: 9}.get(w["p"], w["qd"])  # Strang(p+1) leaves M singular for p >= 3
        w["desc"] = (f"profiling case 2·{w['n']}·{w['n']} triangles, p={w['p']}, quadrature degree "
                     f"{w['qd'] or w['p'] + 1}, tau=1, manufactured sin·sin")
    prec = H.PREC_FP64 if args.precision == "fp64" else H.PREC_MIXED
    pc = H.PRECOND_AMG if args.preconditioner == "amg" else H.PRECOND_JACOBI
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
        K.solve(tol=args.tol, precision=prec, to_host=False, preconditioner=pc)
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
    # the CG kernels' algorithmic bytes come from the library's accounting of the sampled launches
    # (rows that iterated x per-row bytes; with the multigrid preconditioner the "update" sample
    # covers k_cg_b_mg, the V-cycle and k_cg_c)
    lib_a, lib_b = avg("cg_a_bytes"), avg("cg_b_bytes")
    name_a = "k_cg_a_fresh (q = A p_new, p.q)" if (prec == H.PREC_MIXED and pc != H.PRECOND_AMG) else \
        "k_cg_a (q = A z + beta q, p update, p.q)"
    name_b = ("k_cg_b_mg + multigrid V-cycle + k_cg_c" if pc == H.PRECOND_AMG else "k_cg_b (x, r, z update, r.z, r.r)")
    kern = {
        name_a: (avg("cg_a_ms"), lib_a if lib_a > 0 else bytes_a, it_mean),
        name_b: (avg("cg_b_ms"), lib_b if lib_b > 0 else bytes_b, it_mean),
        "k_element_condense": (avg("element_ms"), bytes_elem, 1),
    }
    dom = max(kern, key=lambda k: kern[k][0] * kern[k][2])
    dur, alg, cnt = kern[dom]
    achieved = alg / (dur / 1e3) / 1e9 if dur > 0 else None
    traffic = profile_traffic(dom.split()[0]) if not dom.startswith("k_cg_b_mg") else None

    # ---- end-to-end through the public API with host buffers ----
    import numpy as np
    xy_host = H.get_vertices_matrix(mesh)
    xy_pinned = torch.from_numpy(xy_host).pin_memory().numpy()
    q_h = u_h = None

    def e2e_step():
        mesh.set_coordinates(xy_pinned)                       # H2D: node coordinates
        K.reassemble(1.0, f)                                  # H2D: source parameters
        K.apply_dirichlet(dbc.prescribed_dofs, dbc.values)    # H2D: prescribed dofs and values
        uh = K.solve(tol=args.tol, precision=prec, to_host=True, preconditioner=pc)   # D2H: û
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
                   "nnz": nnz, "precision": args.precision, "preconditioner": args.preconditioner, "tol": args.tol,
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
        line["cpu_baseline"], r = cpu_baseline(w, os.cpu_count() or 1)
        line["parity_vs_oracle"] = parity_vs_oracle(H, K, r["system"], pc, dbc.prescribed_dofs)
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    ws, rank, local = dist_setup(args) if args.impl == "ours" else (int(os.environ.get("WORLD_SIZE", "1")),
                                                                    int(os.environ.get("RANK", "0")), 0)
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    if args.workload == "c4":
        run_c4(args, ws, rank, local)
    elif args.workload == "c3":
        run_c3(args, ws, rank, local)
    elif args.workload == "c5":
        run_c5(args, ws, rank, local)
    elif args.workload == "cg":
        run_cg(args, ws, rank, local)
    else:
        run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
