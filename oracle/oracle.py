"""Python face of the oracle (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` use this module, always as the checker or as the timed CPU
baseline, never as part of the product path.

Fields are numpy arrays in the reference's host layout, ghost slices included
(site s = x + Nx*(y + Ny*(z+1)), z in [-1, Nz]; S/SUNcIndexing.cpp:82):

* links   U    complex128, shape (Nz+2, Ny, Nx, 3, 3, 3) = [z+1, y, x, mu, j, i]
               (flat 9*(mu+3*s) + i+3*j, S/LATTICE/GaugeLinks.cpp:38-41)
* E field E    float64,    shape (Nz+2, Ny, Nx, 3, 8)
* currents J   float64,    shape (Nz+2, Ny, Nx, 8)
* gauge G      complex128, shape (Nz+2, Ny, Nx, 3, 3)  = [z+1, y, x, j, i]

``Oracle`` wraps the CPU restatement (liboracle.so); ``Reference`` wraps the
reference's own code compiled by ``oracle/build.py`` (only where the reference
checkout exists).
"""
import ctypes
import os
import tempfile

import numpy as np

from . import build as _build

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)

FIELD_NAMES = ("U", "UOld", "E", "Jp", "Jm", "JpStat", "JmStat")


def _ptr(a):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def _ivec(v):
    return (ctypes.c_int * 3)(*[int(x) for x in v])


def _dvec(v):
    return (ctypes.c_double * 3)(*[float(x) for x in v])


# ----------------------------------------------------------------- field helpers
def shape_links(N):
    Nx, Ny, Nz = N
    return (Nz + 2, Ny, Nx, 3, 3, 3)


def identity_links(N):
    U = np.zeros(shape_links(N), dtype=np.complex128)
    for k in range(3):
        U[..., k, k] = 1.0
    return U


def zero_efield(N):
    Nx, Ny, Nz = N
    return np.zeros((Nz + 2, Ny, Nx, 3, 8))


def zero_current(N):
    Nx, Ny, Nz = N
    return np.zeros((Nz + 2, Ny, Nx, 8))


def identity_gauge(N):
    Nx, Ny, Nz = N
    G = np.zeros((Nz + 2, Ny, Nx, 3, 3), dtype=np.complex128)
    for k in range(3):
        G[..., k, k] = 1.0
    return G


def new_fields(N):
    return {
        "U": identity_links(N),
        "UOld": identity_links(N),
        "E": zero_efield(N),
        "Jp": zero_current(N),
        "Jm": zero_current(N),
        "JpStat": zero_current(N),
        "JmStat": zero_current(N),
    }


_SQ3 = np.sqrt(3.0)


def herm_from_algebra(al):
    """t^a al^a for an (..., 8) array -> (..., 3, 3) [i, j] Hermitian (S/SUNc/SU3/AlgebraOperations.cpp:31-45)."""
    al = np.asarray(al, dtype=np.float64)
    M = np.zeros(al.shape[:-1] + (3, 3), dtype=np.complex128)
    M[..., 0, 0] = 0.5 * (al[..., 2] + al[..., 7] / _SQ3)
    M[..., 1, 1] = -0.5 * (al[..., 2] - al[..., 7] / _SQ3)
    M[..., 2, 2] = -al[..., 7] / _SQ3
    M[..., 1, 0] = 0.5 * (al[..., 0] + 1j * al[..., 1])
    M[..., 2, 0] = 0.5 * (al[..., 3] + 1j * al[..., 4])
    M[..., 2, 1] = 0.5 * (al[..., 5] + 1j * al[..., 6])
    M[..., 0, 1] = np.conj(M[..., 1, 0])
    M[..., 0, 2] = np.conj(M[..., 2, 0])
    M[..., 1, 2] = np.conj(M[..., 2, 1])
    return M


def algebra_from_herm(W):
    """2 tr(t^a W) for Hermitian W (..., 3, 3) [i, j]."""
    out = np.empty(W.shape[:-2] + (8,))
    out[..., 0] = 2 * W[..., 0, 1].real
    out[..., 1] = -2 * W[..., 0, 1].imag
    out[..., 2] = W[..., 0, 0].real - W[..., 1, 1].real
    out[..., 3] = 2 * W[..., 0, 2].real
    out[..., 4] = -2 * W[..., 0, 2].imag
    out[..., 5] = 2 * W[..., 1, 2].real
    out[..., 6] = -2 * W[..., 1, 2].imag
    out[..., 7] = (W[..., 0, 0].real + W[..., 1, 1].real - 2 * W[..., 2, 2].real) / _SQ3
    return out


def expi_batched(c, al):
    """exp(i c t^a al^a) for (..., 8) -> (..., 3, 3) [i, j], by Hermitian eigen-decomposition."""
    H = c * herm_from_algebra(al)
    w, V = np.linalg.eigh(H)
    return np.einsum("...ik,...k,...jk->...ij", V, np.exp(1j * w), V.conj())


def links_as_matrices(U):
    """View [.., mu, j, i] storage as [.., mu, i, j] matrices (a transposed view, no copy)."""
    return np.swapaxes(U, -1, -2)


def matrices_to_links(M):
    return np.ascontiguousarray(np.swapaxes(M, -1, -2))


def sync_ghosts(F):
    """Open-z ghost sync (S/LATTICE/GaugeLinks.cpp:59-66): slice -1 <- 0, slice Nz <- Nz-1."""
    F[0] = F[1]
    F[-1] = F[-2]


def random_fields(N, seed, link_amp=0.35, e_amp=0.25, j_amp=0.08, sync=True):
    """Seeded random SU(3) links exp(i link_amp t.r), Gaussian E and currents; ghost slices synced."""
    rng = np.random.Generator(np.random.PCG64(seed))
    Nx, Ny, Nz = N
    f = new_fields(N)
    al = rng.standard_normal((Nz + 2, Ny, Nx, 3, 8))
    f["U"] = matrices_to_links(expi_batched(link_amp, al))
    f["UOld"] = f["U"].copy()
    f["E"] = e_amp * rng.standard_normal((Nz + 2, Ny, Nx, 3, 8))
    for k in ("Jp", "Jm", "JpStat", "JmStat"):
        f[k] = j_amp * rng.standard_normal((Nz + 2, Ny, Nx, 8))
    if sync:
        for k in FIELD_NAMES:
            sync_ghosts(f[k])
    return f


def copy_fields(f):
    return {k: v.copy() for k, v in f.items()}


# ----------------------------------------------------------------- the oracle
class Oracle:
    """CPU restatement of the reference path (liboracle.so)."""

    def __init__(self, threads=None):
        path = _build.build_oracle()
        self.lib = ctypes.CDLL(path)
        L = self.lib
        L.oracle_update.argtypes = [_ip, _dp, ctypes.c_double, ctypes.c_int] + [_dp] * 7
        L.oracle_update_efield.argtypes = [_ip, _dp, ctypes.c_double, _dp, _dp, _dp, _dp]
        L.oracle_update_links.argtypes = [_ip, _dp, ctypes.c_double, _dp, _dp]
        L.oracle_bulk.argtypes = [_ip, _dp, ctypes.c_double, _dp, _dp, _dp, _dp, _dp]
        L.oracle_gauss.argtypes = [_ip, _dp, ctypes.c_double, _dp, _dp, _dp, _dp, ctypes.c_int, _dp, _dp, _dp]
        L.oracle_unitarity.argtypes = [_ip, _dp, _dp, _dp]
        L.oracle_emt_map.argtypes = [_ip, _dp, ctypes.c_double, _dp, _dp, _dp, _dp]
        L.oracle_coulomb_fix.argtypes = [_ip, _dp, ctypes.c_double, _dp, _dp, _dp, _dp, _dp, ctypes.c_double,
                                         ctypes.c_int, ctypes.c_double, _dp, _ip, ctypes.c_uint]
        L.oracle_coulomb_fix.restype = ctypes.c_int
        L.oracle_coulomb_fix_local.argtypes = [_ip, _dp, ctypes.c_double, _dp, _dp, _dp, _dp, _dp, ctypes.c_int,
                                               ctypes.c_double, ctypes.c_ulonglong, ctypes.c_int, ctypes.c_double,
                                               _dp, ctypes.POINTER(ctypes.c_int)]
        L.oracle_coulomb_fix_local.restype = ctypes.c_int
        L.oracle_gf_uniform.argtypes = [ctypes.c_ulonglong, ctypes.c_long, ctypes.c_int, ctypes.c_long]
        L.oracle_gf_uniform.restype = ctypes.c_double
        L.oracle_expi.argtypes = [ctypes.c_double, _dp, _dp]
        L.oracle_adj_mul.argtypes = [_dp, _dp, _dp]
        L.oracle_inv_adj_mul.argtypes = [_dp, _dp, _dp]
        L.oracle_transform_charge.argtypes = [_ip, _dp, _dp, _dp]
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        L.oracle_get_threads.restype = ctypes.c_int
        if threads:
            L.oracle_set_threads(int(threads))

    def threads(self):
        return self.lib.oracle_get_threads()

    def expi(self, c, alpha):
        out = np.zeros(9, dtype=np.complex128)
        self.lib.oracle_expi(c, _ptr(np.ascontiguousarray(alpha, dtype=np.float64)), _ptr(out))
        return out.reshape(3, 3).T  # [i, j]

    def update(self, f, N, a, dt, nsteps=1, save_uold=True):
        """In place: nsteps x Dynamics::SUNc::Update."""
        uold = _ptr(f["UOld"]) if save_uold else None
        self.lib.oracle_update(_ivec(N), _dvec(a), dt, nsteps, _ptr(f["U"]), uold, _ptr(f["E"]), _ptr(f["Jp"]),
                               _ptr(f["Jm"]), _ptr(f["JpStat"]), _ptr(f["JmStat"]))

    def transform_charge(self, G, J, N):
        """jG(x) = G(x) j(x) G(x)^dagger on the interior, ghost slices copied from the edges."""
        out = np.zeros_like(J)
        self.lib.oracle_transform_charge(_ivec(N), _ptr(np.ascontiguousarray(G)), _ptr(np.ascontiguousarray(J)),
                                         _ptr(out))
        return out

    def bulk(self, f, N, a, a_scale=1.0):
        out = np.zeros(16)
        self.lib.oracle_bulk(_ivec(N), _dvec(a), a_scale, _ptr(f["U"]), _ptr(f["E"]), _ptr(f["Jp"]), _ptr(f["Jm"]),
                             _ptr(out))
        return out

    def gauss(self, f, N, a, a_scale=1.0, sync_first=False, profile=False):
        mx, avg = ctypes.c_double(), ctypes.c_double()
        zp = np.zeros(N[2]) if profile else None
        self.lib.oracle_gauss(_ivec(N), _dvec(a), a_scale, _ptr(f["U"]), _ptr(f["E"]), _ptr(f["JpStat"]),
                              _ptr(f["JmStat"]), int(sync_first), ctypes.byref(mx), ctypes.byref(avg),
                              _ptr(zp) if profile else None)
        return (mx.value, avg.value, zp) if profile else (mx.value, avg.value)

    def unitarity(self, f, N):
        mx, avg = ctypes.c_double(), ctypes.c_double()
        self.lib.oracle_unitarity(_ivec(N), _ptr(f["U"]), ctypes.byref(mx), ctypes.byref(avg))
        return mx.value, avg.value

    def emt_map(self, f, N, a, a_scale=1.0):
        out = np.zeros((N[2], 10))
        self.lib.oracle_emt_map(_ivec(N), _dvec(a), a_scale, _ptr(f["U"]), _ptr(f["UOld"]), _ptr(f["E"]), _ptr(out))
        return out

    def coulomb_fix(self, f, G, N, a, alpha, total_steps, tol=1e-15, a_scale=1.0, UG=None, EG=None, flags=0):
        """Returns (status, log[n,7], UG, EG); G is updated in place.  flags: 0 for the reference's
        iteration, GF_PROJECT_ZERO_MODE | GF_OPEN_Z for the converging open-z variant."""
        UG = identity_links(N) if UG is None else UG
        EG = zero_efield(N) if EG is None else EG
        log = np.zeros((max(total_steps, 1), 7))
        n = ctypes.c_int()
        st = self.lib.oracle_coulomb_fix(_ivec(N), _dvec(a), a_scale, _ptr(f["U"]), _ptr(f["E"]), _ptr(G), _ptr(UG),
                                         _ptr(EG), alpha, total_steps, tol, _ptr(log), ctypes.byref(n), flags)
        return st, log[: n.value], UG, EG

    def coulomb_fix_local(self, f, G, N, a, algorithm, param, total_steps, seed=0, tol=1e-15, a_scale=1.0,
                          UG=None, EG=None):
        """Los Alamos (algorithm "los_alamos", param = over-relaxation probability) or Jacobi
        ("jacobi", param = step size) gauge fixing; returns (status, log[n,7], UG, EG), G updated in place."""
        UG = identity_links(N) if UG is None else UG
        EG = zero_efield(N) if EG is None else EG
        log = np.zeros((max(total_steps, 1), 7))
        n = ctypes.c_int()
        st = self.lib.oracle_coulomb_fix_local(_ivec(N), _dvec(a), a_scale, _ptr(f["U"]), _ptr(f["E"]), _ptr(G),
                                               _ptr(UG), _ptr(EG), LOCAL_GAUGE_ALGORITHMS[algorithm], param, seed,
                                               total_steps, tol, _ptr(log), ctypes.byref(n))
        return st, log[: n.value], UG, EG

    def gf_uniforms_in_site_order(self, N, seed, iterations):
        """The over-relaxation draws of the Los Alamos update in the order a single-threaded sweep
        of the reference consumes them: per iteration the even sites, then the odd sites, z outer,
        x inner."""
        out = []
        for n in range(iterations):
            for parity in (0, 1):
                for z in range(N[2]):
                    for y in range(N[1]):
                        for x in range(N[0]):
                            if (x + y + z) % 2 == parity:
                                site = x + N[0] * (y + N[1] * z)
                                out.append(self.lib.oracle_gf_uniform(seed, n, parity, site))
        return np.array(out)


LOCAL_GAUGE_ALGORITHMS = {"los_alamos": 1, "jacobi": 2, "fourier": 0}
# coulomb_fix flags (the values of the library's GLASMA_GF_PROJECT_ZERO_MODE / GLASMA_GF_OPEN_Z)
GF_PROJECT_ZERO_MODE = 0x1
GF_OPEN_Z = 0x4


# ----------------------------------------------------------------- the reference itself
_FIELD_ID = {"U": 0, "UOld": 1, "E": 2, "Jp": 3, "Jm": 4, "JpStat": 5, "JmStat": 6, "G": 7, "UG": 8, "EG": 9,
             "rhoL": 10, "rhoR": 11, "CFL": 12, "CFR": 13, "RhoLT1": 14, "RhoRT1": 15, "VLeft": 16, "VRight": 17}


class Reference:
    """The reference's own code (oracle/_ref/libglasma_ref.so).  One lattice per process:
    the reference keeps its fields in global singletons."""

    def __init__(self, N, a, threads=None):
        path = _build.build_reference()
        if path is None:
            raise RuntimeError("reference sources not available on this machine")
        self.lib = ctypes.CDLL(path)
        L = self.lib
        L.ref_init.argtypes = [_ip, _dp]
        L.ref_set_field.argtypes = [ctypes.c_int, _dp]
        L.ref_get_field.argtypes = [ctypes.c_int, _dp]
        L.ref_update.argtypes = [ctypes.c_int, ctypes.c_double]
        L.ref_update.restype = ctypes.c_double
        L.ref_bulk.argtypes = [_dp]
        L.ref_gauss.argtypes = [_dp, _dp]
        L.ref_gauss_profile.argtypes = [_dp]
        L.ref_unitarity.argtypes = [_dp, _dp]
        L.ref_emt_map.argtypes = [_dp]
        L.ref_coulomb.argtypes = [ctypes.c_double, ctypes.c_int, _dp, ctypes.c_int]
        L.ref_coulomb.restype = ctypes.c_int
        L.ref_coulomb_local.argtypes = [ctypes.c_int, ctypes.c_double, _dp, ctypes.c_long, ctypes.c_int, _dp,
                                        ctypes.c_int]
        L.ref_coulomb_local.restype = ctypes.c_int
        L.ref_coulomb_profile.argtypes = [_dp, _dp]
        L.ref_expi.argtypes = [ctypes.c_double, _dp, _dp]
        L.ref_matrix_ilog.argtypes = [ctypes.c_double, _dp, _dp]
        L.ref_set_outdir.argtypes = [ctypes.c_char_p]
        L.ref_set_threads.argtypes = [ctypes.c_int]
        L.ref_save_configuration.argtypes = [ctypes.c_char_p] * 3
        L.ref_load_configuration.argtypes = [ctypes.c_char_p] * 3
        L.ref_tmd_init.argtypes = [_dp, ctypes.c_long, _dp, ctypes.c_long, ctypes.c_double, ctypes.c_int] + \
            [ctypes.c_double] * 6
        L.ref_uniforms_used.restype = ctypes.c_long
        L.ref_mv_init.argtypes = [_dp, ctypes.c_long, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                  ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int]
        self._tmp = tempfile.mkdtemp(prefix="glasma_ref_")
        L.ref_set_outdir(self._tmp.encode())
        if threads:
            L.ref_set_threads(int(threads))
        self.N = tuple(N)
        L.ref_init(_ivec(N), _dvec(a))

    def save_configuration(self):
        """IO::SaveConfiguration + SaveConfigurationJ of the current fields; returns the three paths
        (links, E, currents)."""
        self.lib.ref_save_configuration(b"U", b"E", b"J")
        return tuple(os.path.join(self._tmp, "%sID0.txt" % k) for k in ("U", "E", "J"))

    def load_configuration(self, links, efield, currents):
        """IO::LoadConfiguration into the reference's fields (it exits on malformed files)."""
        self.lib.ref_load_configuration(str(links).encode(), str(efield).encode(), str(currents).encode())

    def set_fields(self, f):
        for k, v in f.items():
            self.lib.ref_set_field(_FIELD_ID[k], _ptr(np.ascontiguousarray(v)))

    def get(self, name):
        N = self.N
        if name in ("U", "UOld", "UG"):
            out = np.zeros(shape_links(N), dtype=np.complex128)
        elif name in ("E", "EG"):
            out = zero_efield(N)
        elif name in ("G", "VLeft", "VRight"):
            out = identity_gauge(N)
        else:
            out = zero_current(N)
        self.lib.ref_get_field(_FIELD_ID[name], _ptr(out))
        return out

    def get_fields(self):
        return {k: self.get(k) for k in FIELD_NAMES}

    def update(self, nsteps, dt):
        return self.lib.ref_update(nsteps, dt)

    def bulk(self):
        out = np.zeros(16)
        self.lib.ref_bulk(_ptr(out))
        return out

    def gauss(self):
        mx, avg = ctypes.c_double(), ctypes.c_double()
        self.lib.ref_gauss(ctypes.byref(mx), ctypes.byref(avg))
        return mx.value, avg.value

    def gauss_profile(self):
        out = np.zeros(self.N[2])
        self.lib.ref_gauss_profile(_ptr(out))
        return out

    def unitarity(self):
        mx, avg = ctypes.c_double(), ctypes.c_double()
        self.lib.ref_unitarity(ctypes.byref(mx), ctypes.byref(avg))
        return mx.value, avg.value

    def emt_map(self):
        out = np.zeros((self.N[2], 10))
        self.lib.ref_emt_map(_ptr(out))
        return out

    def coulomb_fix(self, alpha, total_steps):
        log = np.zeros((max(total_steps, 1), 7))
        n = self.lib.ref_coulomb(alpha, total_steps, _ptr(log), total_steps)
        return log[:n]

    def coulomb_profile(self):
        """Per-slice (max |Delta|, sum Delta^2) of the reference's current gauge-fixed links, from its
        own deviation macro."""
        zmax, zsq = np.zeros(self.N[2]), np.zeros(self.N[2])
        self.lib.ref_coulomb_profile(_ptr(zmax), _ptr(zsq))
        return zmax, zsq

    def coulomb_fix_local(self, algorithm, param, total_steps, uniforms=()):
        """Los Alamos / Jacobi gauge fixing with the reference's own update functions; uniforms are
        what its rng() returns, in call order (construct with threads=1 for a fixed order)."""
        u = np.ascontiguousarray(uniforms, dtype=np.float64)
        log = np.zeros((max(total_steps, 1), 7))
        n = self.lib.ref_coulomb_local(LOCAL_GAUGE_ALGORITHMS[algorithm], param, _ptr(u), u.size, total_steps,
                                       _ptr(log), total_steps)
        return log[:n]

    def expi(self, c, alpha):
        out = np.zeros(9, dtype=np.complex128)
        self.lib.ref_expi(c, _ptr(np.ascontiguousarray(alpha, dtype=np.float64)), _ptr(out))
        return out.reshape(3, 3).T

    def tmd_init(self, gauss, uniforms, dt, A, qs0a, meff, ax_fm, ay_fm, az_fm, com_energy):
        """SimulationmitPC::Run's initial state; gauss / uniforms replay Gauss() / rng().  Returns the
        number of uniforms the nucleon sampling consumed."""
        g = np.ascontiguousarray(gauss, dtype=np.float64)
        u = np.ascontiguousarray(uniforms, dtype=np.float64)
        self.lib.ref_tmd_init(_ptr(g), g.size, _ptr(u), u.size, dt, int(A), qs0a, meff, ax_fm, ay_fm, az_fm, com_energy)
        return self.lib.ref_uniforms_used()

    def mv_init(self, gauss, dt, qs_left, qs_right, center_left, center_right, sigma, lam, meff, single_left=False):
        g = np.ascontiguousarray(gauss, dtype=np.float64)
        self.lib.ref_mv_init(_ptr(g), g.size, dt, qs_left, qs_right, int(center_left), int(center_right), sigma, lam,
                             meff, int(single_left))
