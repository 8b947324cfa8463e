"""Serving: continuous batching of HDG solve requests (hdg_engine_* in libhdg).

    eng = Engine(ctx, hbm_budget_gb=32, max_batch=32, max_flights=16, tol=1e-10)
    mid = eng.add_resident(host_mesh, p)              # meshes kept on the engine
    rid = eng.submit(p, f, kappa_cell, mesh_id=mid)   # or mesh=<host mesh> for a new mesh
    while busy: eng.step(); done = eng.poll()          # admit / advance / complete
    uhat, q, u = eng.result(rid)

No reference counterpart: the reference is a one-problem script."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .fields import as_field


class Engine:
    def __init__(self, ctx, hbm_budget_gb=32.0, max_batch=32, max_flights=16, tol=1e-10,
                 precision=L.PREC_MIXED, chunk=32, maxit=100000, keep_results=True, preconditioner=L.PRECOND_JACOBI):
        self.ctx = ctx
        o = L.hdg_solver(float(tol), int(maxit), int(precision), int(chunk), 1e-5, int(preconditioner))
        h = C.c_void_p()
        L.check(L.load().hdg_engine_create(ctx.handle, float(hbm_budget_gb), int(max_batch), int(max_flights),
                                           C.byref(o), C.byref(h)), ctx.handle)
        self.h = h
        L.check(L.load().hdg_engine_set_keep_results(self.h, int(bool(keep_results))))
        self.inflight = 0
        self.pending = 0

    def close(self):
        """Release the engine (its flights, streams and results)."""
        if self.h:
            L.load().hdg_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_resident(self, host_mesh, p: int) -> int:
        mid = C.c_int()
        L.check(L.load().hdg_engine_add_resident_mesh(self.h, host_mesh.handle, int(p), C.byref(mid)))
        return mid.value

    def submit(self, p, f, kappa_cell=None, mesh_id=-1, mesh=None, quad_degree=None, tau=1.0) -> int:
        fc = as_field(f).as_c()
        kk = None if kappa_cell is None else L.f64(kappa_cell)
        qd = quad_degree if quad_degree is not None else {1: 2, 2: 3, 3: 6, 4: 9}[p]
        rid = C.c_int64()
        L.check(L.load().hdg_engine_submit(self.h, int(mesh_id), mesh.handle if mesh is not None else None, int(p),
                                           int(qd), C.byref(fc), L.dptr(kk), float(tau), C.byref(rid)),
                self.ctx.handle)
        return rid.value

    def step(self):
        a, b = C.c_int(), C.c_int()
        L.check(L.load().hdg_engine_step(self.h, C.byref(a), C.byref(b)), self.ctx.handle)
        self.inflight, self.pending = a.value, b.value
        return self.inflight, self.pending

    def poll(self, max_n=4096):
        ids = np.zeros(max_n, np.int64)
        lat = np.zeros(max_n)
        its = np.zeros(max_n, np.int32)
        res = np.zeros(max_n)
        conv = np.zeros(max_n, np.int32)
        n = C.c_int()
        L.check(L.load().hdg_engine_poll(self.h, max_n, L.i64ptr(ids), L.dptr(lat), its.ctypes.data_as(L.intp),
                                         L.dptr(res), conv.ctypes.data_as(L.intp), C.byref(n)))
        k = n.value
        return [dict(id=int(ids[i]), latency=float(lat[i]), iterations=int(its[i]), rel_residual=float(res[i]),
                     converged=bool(conv[i])) for i in range(k)]

    def result(self, rid: int):
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        L.check(L.load().hdg_engine_result(self.h, int(rid), None, None, None, C.byref(a), C.byref(b), C.byref(c)))
        uh, q, u = np.zeros(a.value), np.zeros(b.value), np.zeros(c.value)
        L.check(L.load().hdg_engine_result(self.h, int(rid), L.dptr(uh), L.dptr(q), L.dptr(u), C.byref(a), C.byref(b),
                                           C.byref(c)))
        return uh, q, u

    def run_until_idle(self, max_steps=10 ** 7):
        out = []
        for _ in range(max_steps):
            inflight, pending = self.step()
            out += self.poll()
            if inflight == 0 and pending == 0:
                break
        return out
