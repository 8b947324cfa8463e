"""Scalar fields passed across the C ABI (the reference passes Julia closures such as
``f(x) = 2π² sin(πx) sin(πy)``; a closure cannot cross a C boundary, so a field here is a kind
plus parameters, evaluated on the device)."""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L


@dataclass(frozen=True)
class Field:
    kind: int
    params: tuple = field(default=(0.0,))

    # ---- constructors -------------------------------------------------------------------
    @staticmethod
    def const(c: float) -> "Field":
        return Field(L.FIELD_CONST, (float(c),))

    @staticmethod
    def sinsin(a: float = 1.0, kx: float = 1.0, ky: float = 1.0) -> "Field":
        """a sin(kx π x) sin(ky π y)"""
        return Field(L.FIELD_SINSIN, (float(a), float(kx), float(ky)))

    @staticmethod
    def bumps(centers, sigmas, amps) -> "Field":
        """sum_k a_k exp(-|x - c_k|^2 / (2 s_k^2))"""
        c = np.asarray(centers, dtype=float).reshape(-1, 2)
        prm = [float(len(c))]
        for (cx, cy), s, a in zip(c, np.broadcast_to(sigmas, len(c)), np.broadcast_to(amps, len(c))):
            prm += [cx, cy, float(s), float(a)]
        return Field(L.FIELD_BUMPS, tuple(prm))

    @staticmethod
    def fourier(g0, modes, exponential: bool = False) -> "Field":
        """g = g0 + sum a cos(2π (kx x + ky y) + φ); modes rows (kx, ky, φ, a); exp(g) if exponential."""
        m = np.asarray(modes, dtype=float).reshape(-1, 4)
        prm = [float(len(m)), float(g0)] + m.ravel().tolist()
        return Field(L.FIELD_EXP_FOURIER if exponential else L.FIELD_FOURIER, tuple(prm))

    # ---- host evaluation (for tests and plotting-free post-processing) ------------------
    def __call__(self, x, y):
        p = self.params
        if self.kind == L.FIELD_CONST:
            return p[0] + 0.0 * np.asarray(x)
        if self.kind == L.FIELD_SINSIN:
            return p[0] * np.sin(p[1] * math.pi * np.asarray(x)) * np.sin(p[2] * math.pi * np.asarray(y))
        if self.kind == L.FIELD_BUMPS:
            s = 0.0
            for k in range(int(p[0])):
                cx, cy, sg, a = p[1 + 4 * k: 5 + 4 * k]
                s = s + a * np.exp(-((np.asarray(x) - cx) ** 2 + (np.asarray(y) - cy) ** 2) / (2 * sg * sg))
            return s
        g = p[1]
        for k in range(int(p[0])):
            kx, ky, ph, a = p[2 + 4 * k: 6 + 4 * k]
            g = g + a * np.cos(2 * math.pi * (kx * np.asarray(x) + ky * np.asarray(y)) + ph)
        return np.exp(g) if self.kind == L.FIELD_EXP_FOURIER else g

    def as_c(self):
        arr = np.ascontiguousarray(self.params, dtype=np.float64)
        f = L.hdg_field(self.kind, arr.size, arr.ctypes.data_as(C.POINTER(C.c_double)))
        f._keep = arr  # keep the parameter buffer alive with the struct
        return f

    def as_oracle(self):
        return (self.kind, list(self.params))


def as_field(f) -> Field | None:
    if f is None or isinstance(f, Field):
        return f
    if isinstance(f, (int, float)):
        return Field.const(f)
    raise TypeError("fields are hdiscontinuousgalerkin Field objects (kind + parameters); Julia-style "
                    "closures cannot cross the C ABI")


# The manufactured solution of examples/poisson2D_HDG.jl:55,216: f = 2π² sin(πx) sin(πy), u = sin(πx) sin(πy)
MANUFACTURED_F = Field.sinsin(2 * math.pi ** 2, 1.0, 1.0)
MANUFACTURED_U = Field.sinsin(1.0, 1.0, 1.0)
