"""Study: can the element condensation run in FP32 with FP64 iterative refinement and still give
trace solutions within 1e-8 of FP64?

TEST INFRASTRUCTURE / ANALYSIS ONLY.  It uses the oracle's FP64 element blocks (the integrals of
examples/poisson2D_HDG.jl:88-153, through hdgref.element_blocks) on a batching-workload-like
problem (jittered mesh, kappa per cell log-uniform in [1e-2, 1e2], Gaussian-bump source) and
forms the condensed blocks Ate, bte in several arithmetics, emulated with numpy (float32 LAPACK
for the FP32 factorisations):

  fp64        S = C + B'A^-1 B, R' = F + B'A^-1 E, Ate = R'S^-1R' - E'A^-1E - He      (the reference)
  fp32        the same with every operand and operation in FP32
  fp32+k      S and R' formed in FP64, S factored in FP32, k refinement sweeps
              X <- X + S32^-1 (R' - S X) with the residual in FP64, then Ate from X in FP64

then assembles the global trace system from each, applies the homogeneous Dirichlet condition
and solves it with SuperLU, and reports the relative L2 difference of the trace solution from the
FP64 one, the largest relative Ate difference, and cond(Me), cond(S).

    python oracle/fp32_condensation_study.py [n] [p] [seed]
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import hdgref  # noqa: E402


def jitter(xy, n, a, rng):
    out = xy.copy()
    h = 1.0 / n
    for j in range(1, n):
        for i in range(1, n):
            k = j * (n + 1) + i
            out[k] += a * h * rng.uniform(-1, 1, 2)
    return out


def study(n=32, p=4, seed=5, refine=(1, 2, 3)):
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    qd = {1: 2, 2: 3, 3: 6, 4: 9}[p]
    rng = np.random.default_rng(seed)
    m = hdgref.rectangle_mesh(n, n)
    m.set_xy(jitter(m.xy, n, 0.2, rng))
    nc = m.ncells
    kappa = np.exp(rng.uniform(np.log(1e-2), np.log(1e2), nc))
    bumps = np.concatenate([[8.0], np.column_stack([rng.random((8, 2)), 0.03 + 0.12 * rng.random(8),
                                                    10 * rng.standard_normal(8)]).ravel()])
    f = (hdgref.F_BUMPS, bumps)
    nw, nt = (p + 1) * (p + 2) // 2, p + 1
    mm = 3 * nt
    variants = ["fp64", "fp32"] + [f"fp32+{k}" for k in refine]
    ate = {v: np.zeros((nc, mm, mm)) for v in variants}
    bte = {v: np.zeros((nc, mm)) for v in variants}
    cond_me, cond_s = np.zeros(nc), np.zeros(nc)
    for c in range(nc):
        b = hdgref.element_blocks(m, c, p, qd, 1.0, f)
        A = b["A"] / kappa[c]  # (kappa^-1 q, v): the mass block scales with 1/kappa on the cell
        B, C, E, F, H, be = b["B"], b["C"], b["E"], b["F"], b["H"], b["be"]
        Me = np.block([[A, -B], [B.T, C]])
        Ai = np.linalg.inv(A)
        S = C + B.T @ Ai @ B
        Rp = np.hstack([F + B.T @ Ai @ E, be[:, None]])
        P = E.T @ Ai @ E
        cond_me[c], cond_s[c] = np.linalg.cond(Me), np.linalg.cond(S)
        X = np.linalg.solve(S, Rp)
        G = Rp[:, :mm].T @ X
        ate["fp64"][c], bte["fp64"][c] = G[:, :mm] - P - H, -G[:, mm]
        # everything in FP32
        A32, B32, C32, E32, F32 = (x.astype(np.float32) for x in (A, B, C, E, F))
        Ai32 = np.linalg.inv(A32)
        S32 = C32 + B32.T @ Ai32 @ B32
        R32 = np.hstack([F32 + B32.T @ Ai32 @ E32, be.astype(np.float32)[:, None]])
        X32 = np.linalg.solve(S32, R32)
        G32 = R32[:, :mm].T @ X32
        ate["fp32"][c] = (G32[:, :mm] - E32.T @ Ai32 @ E32 - H.astype(np.float32)).astype(np.float64)
        bte["fp32"][c] = -G32[:, mm].astype(np.float64)
        # FP32 factorisation of the FP64 S, FP64 residuals, FP64 products
        S32b = S.astype(np.float32)
        Xk = np.linalg.solve(S32b, Rp.astype(np.float32)).astype(np.float64)
        for k in range(1, max(refine) + 1):
            Xk = Xk + np.linalg.solve(S32b, (Rp - S @ Xk).astype(np.float32)).astype(np.float64)
            if k in refine:
                Gk = Rp[:, :mm].T @ Xk
                ate[f"fp32+{k}"][c], bte[f"fp32+{k}"][c] = Gk[:, :mm] - P - H, -Gk[:, mm]
    # global trace system (face-major dofs) from each variant, homogeneous Dirichlet on the boundary
    nd = m.nfaces * nt
    gd = np.array([[(fc - 1) * nt + j for fc in m.cell_faces[c] for j in range(nt)] for c in range(nc)])
    I = np.repeat(gd, mm, axis=1).ravel()
    J = np.tile(gd, (1, mm)).ravel()
    bnd = np.zeros(nd, bool)
    for fc in m.faceset("boundary"):
        bnd[(fc - 1) * nt:fc * nt] = True
    sol = {}
    for v in variants:
        K = sp.csc_matrix((ate[v].ravel(), (I, J)), shape=(nd, nd))
        rhs = np.zeros(nd)
        np.add.at(rhs, gd.ravel(), bte[v].ravel())
        free = ~bnd
        Kf = K[free][:, free]
        x = np.zeros(nd)
        x[free] = spla.splu(Kf.tocsc()).solve(rhs[free])
        sol[v] = x
    ref = sol["fp64"]
    out = {"n": n, "p": p, "cells": nc, "kappa_range": [float(kappa.min()), float(kappa.max())],
           "cond_Me_median": float(np.median(cond_me)), "cond_Me_max": float(cond_me.max()),
           "cond_S_median": float(np.median(cond_s)), "cond_S_max": float(cond_s.max()), "variants": {}}
    for v in variants[1:]:
        da = np.abs(ate[v] - ate["fp64"]).max(axis=(1, 2)) / np.abs(ate["fp64"]).max(axis=(1, 2))
        out["variants"][v] = {"ate_rel_max": float(da.max()),
                              "uhat_rel_l2": float(np.linalg.norm(sol[v] - ref) / np.linalg.norm(ref))}
    return out


if __name__ == "__main__":
    a = [int(x) for x in sys.argv[1:]]
    print(json.dumps(study(*a), indent=1))
