"""Configuration files: the reference's text format (IO::SaveConfiguration / SaveConfigurationJ /
LoadConfiguration, S/IO/SaveConfiguration.cpp, S/IO/LoadConfiguration.cpp) and a bit-exact binary
restart format.  The text functions here work on host arrays in the reference's layout and need no
GPU; Lattice.save_text / load_text / save_binary / load_binary do the same for a device lattice."""
import numpy as np

from . import _lib
from .lattice import empty_field

CURRENTS = ("JpStat", "Jp", "JmStat", "Jm")


def _path(p):
    return None if p is None else str(p).encode()


def _io_check(lib, status):
    if status != _lib.GLASMA_OK:
        raise _lib.GlasmaError(status, lib.glasma_io_last_error().decode(errors="replace"))


def _ptr(a):
    return None if a is None else a.ctypes.data


def write_text(N, fields, links=None, efield=None, currents=None):
    """Write fields (dict of host arrays: U, E, JpStat, Jp, JmStat, Jm) to the reference's text files."""
    lib = _lib.load()
    arrs = {k: (np.ascontiguousarray(fields[k]) if k in fields else None) for k in ("U", "E") + CURRENTS}
    _io_check(lib, lib.glasma_write_text_host(int(N[0]), int(N[1]), int(N[2]), _ptr(arrs["U"]), _ptr(arrs["E"]),
                                              *[_ptr(arrs[k]) for k in CURRENTS], _path(links), _path(efield),
                                              _path(currents)))


def read_text(N, links=None, efield=None, currents=None):
    """Read the reference's text files into host arrays; returns a dict of the fields read."""
    lib = _lib.load()
    out = {}
    if links is not None:
        out["U"] = empty_field("U", N)
    if efield is not None:
        out["E"] = empty_field("E", N)
    if currents is not None:
        for k in CURRENTS:
            out[k] = empty_field(k, N)
    _io_check(lib, lib.glasma_read_text_host(int(N[0]), int(N[1]), int(N[2]), _ptr(out.get("U")), _ptr(out.get("E")),
                                             *[_ptr(out.get(k)) for k in CURRENTS], _path(links), _path(efield),
                                             _path(currents)))
    return out
