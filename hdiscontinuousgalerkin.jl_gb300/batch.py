"""Batches of independent HDG problems: many meshes of uneven size and several degrees solved
together.  Problems are grouped by degree ("bins"); each bin is one disjoint union mesh with one
space and one trace system, so a whole bin is assembled, condensed, gathered and solved by the
same launches, and the bins' CG iterations are interleaved by one host loop
(hdg_solve_batch).  No reference counterpart: the reference solves one problem per script."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from .fields import Field, as_field
from .mesh import PolygonalMesh, TriangleCell, rectangle_mesh
from .system import SolveStats


@dataclass
class Problem:
    """One Poisson problem: a rectangle mesh of n x n cells (jittered), degree p, source f,
    per-cell kappa (or None), tau."""
    n: int
    p: int
    f: Field
    kappa_cell: np.ndarray | None = None
    jitter: float = 0.0
    seed: int = 0
    tau: float = 1.0
    quad_degree: int | None = None
    LL: tuple = (0.0, 0.0)
    UR: tuple = (1.0, 1.0)

    def qd(self):
        # the default p+1 rule leaves the local systems singular for p >= 3: use an exact-enough rule
        if self.quad_degree is not None:
            return self.quad_degree
        return {1: 2, 2: 3, 3: 6, 4: 9}[self.p]


def host_mesh(pr: Problem) -> PolygonalMesh:
    m = rectangle_mesh(TriangleCell, (pr.n, pr.n), pr.LL, pr.UR, ctx=None)
    if pr.jitter > 0:
        m.jitter(pr.jitter, pr.seed)
    return m


def concat_meshes(ctx, meshes) -> PolygonalMesh:
    arr = (C.c_void_p * len(meshes))(*[m.handle for m in meshes])
    h = C.c_void_p()
    L.check(L.load().hdg_mesh_concat(ctx.handle if ctx else None, len(meshes), arr, C.byref(h)),
            ctx.handle if ctx else None)
    return PolygonalMesh(h, ctx.handle if ctx else None)


def problem_offsets(mesh: PolygonalMesh):
    n = C.c_int()
    L.check(L.load().hdg_mesh_problems(mesh.handle, C.byref(n), None, None, None))
    node0, cell0, face0 = (np.zeros(n.value + 1, np.int32) for _ in range(3))
    L.check(L.load().hdg_mesh_problems(mesh.handle, C.byref(n), L.i32ptr(node0), L.i32ptr(cell0), L.i32ptr(face0)))
    return node0, cell0, face0


class Bin:
    """All problems of one degree: a union mesh, one space, one trace system."""

    def __init__(self, ctx, problems, idx, precision):
        from .spaces import _SpaceHandle
        self.ctx, self.problems, self.idx = ctx, problems, idx
        self.p = problems[0].p
        self.hosts = [host_mesh(pr) for pr in problems]
        self.mesh = concat_meshes(ctx, self.hosts)
        self.node0, self.cell0, self.face0 = problem_offsets(self.mesh)
        self.sp = _SpaceHandle(self.mesh, self.p, problems[0].qd())
        self.nt, self.nw = self.sp.nt, self.sp.nw
        self.precision = precision
        self._coef_arrays()
        h = C.c_void_p()
        L.check(L.load().hdg_assemble_condense_batch(self.sp.h, L.dptr(self.taus), self.farr, None, L.dptr(self.kc),
                                                     int(precision), C.byref(h)), ctx.handle)
        self.h = h
        nd, nnz, n, m = C.c_int(), C.c_int64(), C.c_int(), C.c_int()
        L.check(L.load().hdg_system_sizes(self.h, C.byref(nd), C.byref(nnz), C.byref(n), C.byref(m)))
        self.ndofs, self.n = nd.value, n.value
        self._dirichlet()
        self._dir_set = False
        self._dl = None
        self._host_bufs = []

    def _coef_arrays(self):
        np_ = len(self.problems)
        self.taus = np.array([pr.tau for pr in self.problems], dtype=np.float64)
        self._fields = [pr.f.as_c() for pr in self.problems]
        self.farr = (L.hdg_field * np_)(*self._fields)
        if any(pr.kappa_cell is not None for pr in self.problems):
            self.kc = np.concatenate([pr.kappa_cell if pr.kappa_cell is not None else
                                      np.ones(2 * pr.n * pr.n) for pr in self.problems]).astype(np.float64)
        else:
            self.kc = None

    def _dirichlet(self):
        g = Field.const(0.0).as_c()
        n = C.c_int()
        L.check(L.load().hdg_dirichlet(self.sp.h, b"boundary", C.byref(g), None, None, C.byref(n)), self.ctx.handle)
        self.dofs = np.zeros(n.value, np.int32)
        self.vals = np.zeros(n.value)
        L.check(L.load().hdg_dirichlet(self.sp.h, b"boundary", C.byref(g), L.i32ptr(self.dofs), L.dptr(self.vals),
                                       C.byref(n)), self.ctx.handle)

    def reassemble(self, resident=False):
        """Element blocks and trace system again; with resident=True from the coefficients already
        on the device (no upload), else from the problems' host arrays."""
        if resident:
            L.check(L.load().hdg_system_reassemble_resident(self.h), self.ctx.handle)
            return
        L.check(L.load().hdg_system_reassemble_batch(self.h, L.dptr(self.taus), self.farr, None, L.dptr(self.kc)),
                self.ctx.handle)

    def apply(self):
        L.check(L.load().hdg_apply_dirichlet(self.h, L.i32ptr(self.dofs), L.dptr(self.vals), len(self.dofs)),
                self.ctx.handle)

    def set_coefficients(self):
        """Upload the problems' coefficients without assembling (the next step assembles)."""
        L.check(L.load().hdg_system_set_coefficients_batch(self.h, L.dptr(self.taus), self.farr, None,
                                                           L.dptr(self.kc)), self.ctx.handle)

    def set_dirichlet(self):
        """Record (upload and scatter) the Dirichlet set without applying it."""
        L.check(L.load().hdg_system_set_dirichlet(self.h, L.i32ptr(self.dofs), L.dptr(self.vals), len(self.dofs)),
                self.ctx.handle)

    def recover(self):
        L.check(L.load().hdg_recover(self.h, None, None, None), self.ctx.handle)

    def timings(self) -> dict:
        """Per-phase device times of this bin's system recorded while profiling was on (ms)."""
        t = L.hdg_timings()
        L.check(L.load().hdg_system_timings(self.h, C.byref(t)), self.ctx.handle)
        return {k: getattr(t, k) for k, _ in L.hdg_timings._fields_}

    def kernel_sample(self, which=1) -> dict:
        """One kernel family of the last solve's sampled chunks, timed launch by launch
        (hdg_system_kernel_sample): summed event ms, summed algorithmic bytes, launches."""
        ms, by, n = C.c_double(), C.c_double(), C.c_int()
        L.check(L.load().hdg_system_kernel_sample(self.h, int(which), C.byref(ms), C.byref(by), C.byref(n)),
                self.ctx.handle)
        return {"ms": ms.value, "bytes": by.value, "launches": n.value}

    def _pinned(self, count):
        ptr = C.c_void_p()
        L.check(L.load().hdg_host_alloc(C.c_size_t(8 * count), C.byref(ptr)), self.ctx.handle)
        self._host_bufs.append(ptr)
        return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_double)), shape=(count,))

    def enable_download(self):
        """Page-locked host arrays that each pipelined step fills with (uhat, [q; u])."""
        if self._dl is None:
            uh = self._pinned(self.ndofs)
            qu = self._pinned(self.mesh.ncells * self.n)
            L.check(L.load().hdg_system_set_download(self.h, L.dptr(uh), L.dptr(qu)), self.ctx.handle)
            self._dl = (uh, qu)
        return self._dl

    def solution(self, downloaded=False):
        """Per problem (uhat, q, u) on the host.  downloaded=True reads the page-locked arrays
        that the last step filled (views, valid until the next step) instead of copying."""
        if downloaded and self._dl is not None:
            uh, qu = self._dl
        else:
            uh = np.zeros(self.ndofs)
            qu = np.zeros(self.mesh.ncells * self.n)
            L.check(L.load().hdg_system_get_solution(self.h, L.dptr(uh), L.dptr(qu)), self.ctx.handle)
        qu = qu.reshape(self.mesh.ncells, self.n)
        out = []
        for k in range(len(self.problems)):
            f0, f1 = self.face0[k] * self.nt, self.face0[k + 1] * self.nt
            c0, c1 = self.cell0[k], self.cell0[k + 1]
            out.append((uh[f0:f1], qu[c0:c1, :2 * self.nw], qu[c0:c1, 2 * self.nw:]))
        return out

    def __del__(self):
        try:
            if self.h:
                L.load().hdg_system_destroy(self.h)
                self.h = None
            for ptr in self._host_bufs:
                L.load().hdg_host_free(ptr)
            self._host_bufs = []
        except Exception:
            pass


class Batch:
    """A batch of independent problems, binned by degree."""

    def __init__(self, ctx, problems, precision=L.PREC_MIXED):
        self.ctx, self.problems = ctx, list(problems)
        self.bins = []
        for p in sorted(set(pr.p for pr in self.problems)):
            idx = [i for i, pr in enumerate(self.problems) if pr.p == p]
            self.bins.append(Bin(ctx, [self.problems[i] for i in idx], idx, precision))
        self.stats = None

    def solve(self, tol=1e-10, maxit=100000, chunk=32, reassemble=True, preconditioner=L.PRECOND_JACOBI,
              download=False):
        """assemble + condense, apply!, CG and recovery of every problem, as one pipelined step
        (hdg_batch_step): each degree bin runs on a stream of its own, so one bin's assembly and
        recovery overlap the other bins' iterations.
        reassemble: True (upload the coefficients and Dirichlet data, then assemble), "resident"
        (assemble from the coefficients and Dirichlet data already on the device) or False (keep
        the assembled systems; they must not have been applied yet).
        download: copy every problem's solution to page-locked host arrays inside the step, each
        bin as soon as it is recovered (read them with solutions(downloaded=True))."""
        flags = L.STEP_APPLY | L.STEP_RECOVER
        if download:
            flags |= L.STEP_DOWNLOAD
            for b in self.bins:
                b.enable_download()
        for b in self.bins:
            if reassemble is True:
                b.set_coefficients()
            if reassemble is True or not b._dir_set:
                b.set_dirichlet()
                b._dir_set = True
        if reassemble:
            flags |= L.STEP_ASSEMBLE
        prec = self.bins[0].precision
        o = L.hdg_solver(float(tol), int(maxit), int(prec), int(chunk), 1e-5, int(preconditioner))
        n = len(self.problems)
        st = (L.hdg_stats * n)()
        arr = (C.c_void_p * len(self.bins))(*[b.h for b in self.bins])
        rc = L.load().hdg_batch_step(len(self.bins), arr, C.byref(o), flags, st)
        if rc not in (0, -5):  # a problem that misses the tolerance is reported in its stats
            L.check(rc, self.ctx.handle)
        stats = [None] * n
        k = 0
        for b in self.bins:
            for i in b.idx:
                stats[i] = SolveStats(st[k])
                k += 1
        self.stats = stats
        return stats

    def solutions(self, downloaded=False):
        """Per problem (uhat, q, u).  downloaded=True returns views of the page-locked arrays that
        the last solve(download=True) filled (valid until the next solve)."""
        out = [None] * len(self.problems)
        for b in self.bins:
            for i, sol in zip(b.idx, b.solution(downloaded)):
                out[i] = sol
        return out

    def ncells(self):
        return sum(2 * pr.n * pr.n for pr in self.problems)
