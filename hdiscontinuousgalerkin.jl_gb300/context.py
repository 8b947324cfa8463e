"""Device context (one GPU, one CUDA stream) shared by the Python API objects."""
from __future__ import annotations

import ctypes as C
import threading

from . import _lib as L


class Context:
    def __init__(self, device: int = 0):
        h = C.c_void_p()
        L.check(L.load().hdg_ctx_create(int(device), C.byref(h)))
        self.handle = h
        self.device = device

    def launches(self) -> int:
        """Kernels launched by this context so far."""
        return int(L.load().hdg_ctx_launch_count(self.handle))

    def set_profiling(self, on: bool):
        L.check(L.load().hdg_ctx_set_profiling(self.handle, int(bool(on))), self.handle)

    def set_stream(self, stream_ptr: int | None):
        L.check(L.load().hdg_ctx_set_stream(self.handle, C.c_void_p(stream_ptr) if stream_ptr else None), self.handle)

    def close(self):
        if self.handle:
            L.load().hdg_ctx_destroy(self.handle)
            self.handle = None


_default = None
_lock = threading.Lock()


def default_context() -> Context:
    global _default
    with _lock:
        if _default is None:
            _default = Context(0)
        return _default
