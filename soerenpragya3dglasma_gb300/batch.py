"""Batches of independent events (lattices of uneven sizes) advanced together on one GPU."""
import ctypes

import numpy as np

from . import _lib
from .lattice import Lattice


class _EventView(Lattice):
    """A Lattice over an event handle owned by its batch (not destroyed on close)."""

    def __init__(self, lib, handle, N, a, precision):
        self.lib = lib
        self.h = handle
        self.N = tuple(N)
        self.a = tuple(a)
        self.precision = precision

    def close(self):
        self.h = None


def _bcheck(lib, st):
    if st != 0:
        raise _lib.GlasmaError(st, lib.glasma_batch_last_error().decode(errors="replace") or
                               lib.glasma_last_error().decode(errors="replace"))


class Batch:
    def __init__(self, extents, spacings=None, precision="fp32", reunitarize_every=16, stream=None):
        self.lib = _lib.load()
        n = len(extents)
        spacings = spacings or [(1.0, 1.0, 1.0)] * n
        ext = (ctypes.c_int * (3 * n))(*[int(v) for e in extents for v in e])
        sp = (ctypes.c_double * (3 * n))(*[float(v) for a in spacings for v in a])
        prec = {"fp64": _lib.FP64, "fp32": _lib.FP32}[precision]
        b = ctypes.c_void_p()
        _bcheck(self.lib, self.lib.glasma_batch_create(n, ext, sp, prec, int(reunitarize_every), ctypes.byref(b)))
        self.b = b
        self.events = []
        for i in range(n):
            h = ctypes.c_void_p()
            _bcheck(self.lib, self.lib.glasma_batch_event(self.b, i, ctypes.byref(h)))
            self.events.append(_EventView(self.lib, h, extents[i], spacings[i], precision))
        if stream is not None:
            ptr = getattr(stream, "cuda_stream", stream)
            _bcheck(self.lib, self.lib.glasma_batch_set_stream(self.b, ctypes.c_void_p(ptr) if ptr else None))

    def autotune(self, dt=0.1):
        t = (ctypes.c_int * len(self.events))()
        _bcheck(self.lib, self.lib.glasma_batch_autotune(self.b, float(dt), t))
        return list(t)

    def set_launch(self, mode):
        """"tile_grid" (default: one block per tile) or "persistent" (a device-filling grid walking the
        tile list); both cover all events in one launch per kernel and give the same fields."""
        _bcheck(self.lib, self.lib.glasma_batch_set_launch(self.b, {"persistent": 0, "tile_grid": 1}[mode]))

    def set_step_method(self, method):
        """"plaquette" (default: each event's force summed plaquette by plaquette into a
        48-real-per-site contribution buffer; two-pass when those cannot be allocated) or "two_pass"
        (the staple kernels); either gives each event the fields it would reach stepped alone with that
        method."""
        _bcheck(self.lib, self.lib.glasma_batch_set_step_method(self.b, Lattice.STEP_METHODS[method]))

    def step_method(self):
        m = ctypes.c_int()
        _bcheck(self.lib, self.lib.glasma_batch_get_step_method(self.b, ctypes.byref(m)))
        return {v: k for k, v in Lattice.STEP_METHODS.items()}[m.value]

    def set_link_reals(self, reals):
        """18 (default) or 12 reals per link in the batched step (FP32 batches; rows 0 and 1 of each
        link stored, row 2 formed as conj(row0 x row1)); every event follows the setting."""
        _bcheck(self.lib, self.lib.glasma_batch_set_link_storage(self.b, int(reals)))

    def step(self, dt, nsteps, use_graph=True):
        _bcheck(self.lib, self.lib.glasma_batch_step(self.b, float(dt), int(nsteps), int(bool(use_graph))))

    def energy(self):
        out = np.zeros(len(self.events))
        _bcheck(self.lib, self.lib.glasma_batch_energy(self.b, out.ctypes.data_as(_lib._D)))
        return out

    def synchronize(self):
        _bcheck(self.lib, self.lib.glasma_batch_synchronize(self.b))

    def close(self):
        if getattr(self, "b", None):
            for e in self.events:
                e.close()
            self.lib.glasma_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
