"""Host-side handle of one GPU-resident lattice, over the C ABI.

Fields cross the boundary as numpy arrays in the reference's host layout, FP64,
ghost slices included (site s = x + Nx*(y + Ny*(z+1)), z in [-1, Nz];
S/SUNcIndexing.cpp:82 with S/ the reference's SourceCode directory):

    U, UOld, UG   complex128 (Nz+2, Ny, Nx, 3, 3, 3)   [z+1, y, x, mu, j, i]
    E, EG         float64    (Nz+2, Ny, Nx, 3, 8)
    Jp, Jm, JpStat, JmStat   float64 (Nz+2, Ny, Nx, 8)
    G             complex128 (Nz+2, Ny, Nx, 3, 3)      [z+1, y, x, j, i]

Any C-contiguous array (or a pinned torch CPU tensor exposing the same bytes)
with that many doubles is accepted.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check

_SHAPES = {
    "U": lambda N: (N[2] + 2, N[1], N[0], 3, 3, 3),
    "UOld": lambda N: (N[2] + 2, N[1], N[0], 3, 3, 3),
    "UG": lambda N: (N[2] + 2, N[1], N[0], 3, 3, 3),
    "G": lambda N: (N[2] + 2, N[1], N[0], 3, 3),
    "E": lambda N: (N[2] + 2, N[1], N[0], 3, 8),
    "EG": lambda N: (N[2] + 2, N[1], N[0], 3, 8),
    "Jp": lambda N: (N[2] + 2, N[1], N[0], 8),
    "Jm": lambda N: (N[2] + 2, N[1], N[0], 8),
    "JpStat": lambda N: (N[2] + 2, N[1], N[0], 8),
    "JmStat": lambda N: (N[2] + 2, N[1], N[0], 8),
}
_COMPLEX = {"U", "UOld", "UG", "G"}

DYNAMICAL_FIELDS = ("U", "UOld", "E", "Jp", "Jm", "JpStat", "JmStat")


def field_shape(name, N):
    return _SHAPES[name](N)


def empty_field(name, N):
    return np.zeros(field_shape(name, N), dtype=np.complex128 if name in _COMPLEX else np.float64)


def _address(arr, n_doubles):
    """Host address of a C-contiguous buffer holding n_doubles doubles (numpy array or torch CPU tensor)."""
    if isinstance(arr, np.ndarray):
        if not arr.flags["C_CONTIGUOUS"]:
            raise ValueError("field array must be C-contiguous")
        if arr.nbytes != 8 * n_doubles:
            raise ValueError("field array has %d bytes, expected %d" % (arr.nbytes, 8 * n_doubles))
        return arr.ctypes.data
    # torch tensor
    if not arr.is_contiguous():
        raise ValueError("field tensor must be contiguous")
    if arr.numel() * arr.element_size() != 8 * n_doubles:
        raise ValueError("field tensor has the wrong number of bytes")
    return arr.data_ptr()


def tmd_default_params(dt=0.125):
    """The reference's TMD parameters for unit lattice spacing (glasma_tmd_default_params)."""
    lib = _lib.load()
    p = _lib.TmdParams()
    lib.glasma_tmd_default_params(ctypes.byref(p), float(dt))
    return p


def glauber_sample(A, uniforms):
    """Nucleon positions (A, 3) in fm from the reference's rng() draws, and the number of draws used
    (Nucleus::SetNucleonPositions; host only)."""
    lib = _lib.load()
    u = np.ascontiguousarray(uniforms, dtype=np.float64)
    pos = np.zeros((A, 3))
    used = ctypes.c_long()
    st = lib.glasma_glauber_sample(int(A), u.ctypes.data_as(_lib._D), u.size, pos.ctypes.data_as(_lib._D),
                                   ctypes.byref(used))
    if st:
        raise _lib.GlasmaError(st, lib.glasma_mv_last_error().decode(errors="replace"))
    return pos, used.value


class Lattice:
    """One lattice resident in GPU memory (the reference's global field singletons,
    S/LATTICE/SUNcVariables.cpp:4-90, become one handle)."""

    def __init__(self, N, a=(1.0, 1.0, 1.0), precision="fp64", reunitarize_every=0, stream=None):
        self.lib = _lib.load()
        self.N = tuple(int(n) for n in N)
        self.a = tuple(float(x) for x in a)
        self.precision = precision
        prec = {"fp64": _lib.FP64, "fp32": _lib.FP32}[precision]
        h = ctypes.c_void_p()
        check(self.lib.glasma_create(self.N[0], self.N[1], self.N[2], self.a[0], self.a[1], self.a[2], prec,
                                     int(reunitarize_every), ctypes.byref(h)))
        self.h = h
        if stream is not None:
            self.set_stream(stream)

    def close(self):
        if getattr(self, "h", None):
            self.lib.glasma_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- plumbing
    def set_stream(self, stream):
        """stream: a torch.cuda.Stream, an integer cudaStream_t, or None for the handle's own stream."""
        ptr = getattr(stream, "cuda_stream", stream)
        check(self.lib.glasma_set_stream(self.h, ctypes.c_void_p(ptr) if ptr else None))

    def set_scale(self, a_scale):
        check(self.lib.glasma_set_scale(self.h, float(a_scale)))

    def mv_init(self, zeta_left, zeta_right=None, qs=(0.5, 0.5), centers=None, sigma=4.0, lam=1.65, meff=0.2,
                dt=0.125):
        """MV collision (zeta_right given) or single left-moving nucleus (zeta_right None) on the GPU.
        zeta_*: 8*Nx*Ny N(0,1) charge fluctuations in the order a + 8*(x + Nx*y)."""
        zl = np.ascontiguousarray(zeta_left, dtype=np.float64)
        zr = None if zeta_right is None else np.ascontiguousarray(zeta_right, dtype=np.float64)
        nz = self.N[2]
        centers = centers or (nz // 2 - nz // 5, nz // 2 + nz // 5)
        st = self.lib.glasma_mv_init(self.h, int(zr is None), zl.ctypes.data_as(_lib._D),
                                     zr.ctypes.data_as(_lib._D) if zr is not None else None, float(qs[0]),
                                     float(qs[1]), int(centers[0]), int(centers[1]), float(sigma), float(lam),
                                     float(meff), float(dt))
        if st:
            raise _lib.GlasmaError(st, self.lib.glasma_mv_last_error().decode(errors="replace"))

    def tmd_init(self, noise_left, noise_right, nucleons_left, nucleons_right, dt=0.125, return_densities=False,
                 **params):
        """TMD / Glauber initial state on the GPU (SimulationmitPC::Run).  noise_*: 8*Nx*Ny*Nz N(0,1)
        numbers in the order a + 8*(x + Nx*(y + Ny*z)); nucleons_*: (A, 3) positions in fm (glauber_sample).
        params override tmd_default_params(dt) by field name.  With return_densities, returns the
        filtered densities (rhoL, rhoR) in the reference's ChargeDensity layout."""
        p = tmd_default_params(dt)
        for k, v in params.items():
            setattr(p, k, v)
        N = self.N
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (noise_left, noise_right, nucleons_left,
                                                                     nucleons_right)]
        assert arrs[0].size == arrs[1].size == 8 * N[0] * N[1] * N[2]
        assert arrs[2].size == arrs[3].size == 3 * p.atomic_number
        rho = [np.zeros((N[2] + 2, N[1], N[0], 8)) for _ in range(2)] if return_densities else [None, None]
        ptrs = [a.ctypes.data_as(_lib._D) for a in arrs]
        rptr = [r.ctypes.data_as(_lib._D) if r is not None else None for r in rho]
        st = self.lib.glasma_tmd_init(self.h, *ptrs, ctypes.byref(p), *rptr)
        if st:
            raise _lib.GlasmaError(st, self.lib.glasma_mv_last_error().decode(errors="replace"))
        return tuple(rho) if return_densities else None

    def fill_synthetic(self, seed, link_amp=0.3, e_amp=0.1, j_amp=0.02):
        """Seeded synthetic fields generated on the device (links exp(i link_amp t.r), Gaussian E, J)."""
        check(self.lib.glasma_fill_synthetic(self.h, int(seed), float(link_amp), float(e_amp), float(j_amp)))

    def autotune(self, dt=0.1):
        """Pick the electric-field kernel's block tile for this lattice; returns tile_x."""
        t = ctypes.c_int()
        check(self.lib.glasma_autotune(self.h, float(dt), ctypes.byref(t)))
        return t.value

    def set_tile(self, tile_x):
        check(self.lib.glasma_set_tile(self.h, int(tile_x)))

    def synchronize(self):
        check(self.lib.glasma_synchronize(self.h))

    def field_doubles(self, name):
        return self.lib.glasma_field_doubles(self.h, _lib.FIELDS[name])

    # -- field transfer
    def upload(self, name, arr):
        check(self.lib.glasma_upload(self.h, _lib.FIELDS[name], _address(arr, self.field_doubles(name))))

    def download(self, name, out=None):
        if out is None:
            out = empty_field(name, self.N)
        check(self.lib.glasma_download(self.h, _lib.FIELDS[name], _address(out, self.field_doubles(name))))
        return out

    def upload_begin(self, name, arr):
        """Start copying a host field on the handle's transfer stream (glasma_upload_begin); the array
        is kept alive here until upload_finish."""
        check(self.lib.glasma_upload_begin(self.h, _lib.FIELDS[name], _address(arr, self.field_doubles(name))))
        self._in_flight = getattr(self, "_in_flight", []) + [arr]

    def upload_finish(self):
        """Order the handle's stream after the begun copies and convert them into the fields.  The copies
        may still be reading the host arrays when this returns: they are kept alive until the next
        upload_finish (by then a synchronising call has passed in any sensible loop)."""
        check(self.lib.glasma_upload_finish(self.h))
        self._finished = getattr(self, "_in_flight", [])
        self._in_flight = []

    def upload_device(self, name, dev_ptr):
        check(self.lib.glasma_upload_device(self.h, _lib.FIELDS[name], ctypes.c_void_p(int(dev_ptr))))

    def download_device(self, name, dev_ptr):
        check(self.lib.glasma_download_device(self.h, _lib.FIELDS[name], ctypes.c_void_p(int(dev_ptr))))

    def upload_fields(self, fields):
        for k, v in fields.items():
            self.upload(k, v)

    def download_fields(self, names=DYNAMICAL_FIELDS):
        return {k: self.download(k) for k in names}

    # -- dynamics (Dynamics::SUNc, S/DYNAMICS/SUNcDynamics.cpp)
    def step(self, dt, nsteps=1, save_uold=True):
        check(self.lib.glasma_step(self.h, float(dt), int(nsteps), _lib.STEP_SAVE_UOLD if save_uold else 0))

    STEP_METHODS = {"one_pass": 0, "two_pass": 1, "plaquette": 2, "march": 3}

    def set_step_method(self, method):
        """"plaquette" (default: the electric force summed plaquette by plaquette, two kernels and a
        contribution buffer), "two_pass" (two kernels per step, in place, staple form) or "one_pass"
        (one kernel per step over two buffer sets; bit-identical to two_pass) or "march" (the plaquette
        method in one kernel per step, blocks marching along z; equal to plaquette up to rounding).  The
        plaquette methods equal the staple ones up to rounding."""
        check(self.lib.glasma_set_step_method(self.h, self.STEP_METHODS[method]))

    def set_march_chunk(self, slices):
        """z slices per block of the marching step (0: chosen from the lattice)."""
        check(self.lib.glasma_set_march_chunk(self.h, int(slices)))

    @property
    def last_step_method(self):
        """The method the last step() used."""
        m = ctypes.c_int()
        check(self.lib.glasma_get_step_method(self.h, ctypes.byref(m)))
        return {v: k for k, v in self.STEP_METHODS.items()}[m.value]

    FP64_ARITHMETIC = {"native": 0, "double_float": 1}

    @property
    def fp64_arithmetic(self):
        """"native" (default) or "double_float": the arithmetic of the plaquette force kernel on FP64
        handles (double-float = pairs of FP32 numbers on the FP32 pipe)."""
        m = ctypes.c_int()
        check(self.lib.glasma_get_fp64_arithmetic(self.h, ctypes.byref(m)))
        return {v: k for k, v in self.FP64_ARITHMETIC.items()}[m.value]

    @fp64_arithmetic.setter
    def fp64_arithmetic(self, mode):
        check(self.lib.glasma_set_fp64_arithmetic(self.h, self.FP64_ARITHMETIC[mode]))

    @property
    def link_reals(self):
        """Reals per link the leapfrog step reads and writes: 18, or 12 (rows 0 and 1 of each link,
        row 2 formed as conj(row0 x row1); FP32 handles only)."""
        m = ctypes.c_int()
        check(self.lib.glasma_get_link_storage(self.h, ctypes.byref(m)))
        return m.value

    @link_reals.setter
    def link_reals(self, reals):
        check(self.lib.glasma_set_link_storage(self.h, int(reals)))

    def step_profiled(self, dt, nsteps=1, save_uold=False):
        """Like step(); returns the summed CUDA-event milliseconds of (efield_jstat, links_j) for the
        two-pass method, (one-pass kernel, 0) for the one-pass method."""
        ms = np.zeros(2)
        check(self.lib.glasma_step_profiled(self.h, float(dt), int(nsteps), _lib.STEP_SAVE_UOLD if save_uold else 0,
                                            ms.ctypes.data_as(_lib._D)))
        return ms

    def update_efield(self, dt):
        check(self.lib.glasma_update_efield(self.h, float(dt)))

    def update_jstat(self, dt):
        check(self.lib.glasma_update_jstat(self.h, float(dt)))

    def update_links(self, dt_arg):
        check(self.lib.glasma_update_links(self.h, float(dt_arg)))

    def save_old_link(self):
        check(self.lib.glasma_save_old_link(self.h))

    def update_j(self, dt):
        check(self.lib.glasma_update_j(self.h, float(dt)))

    def reunitarize(self):
        check(self.lib.glasma_reunitarize(self.h))

    # -- observables (S/OBSERVABLES)
    def bulk(self):
        out = np.zeros(16)
        check(self.lib.glasma_bulk(self.h, out.ctypes.data_as(_lib._D)))
        return out

    def gauss(self, sync_first=False, profile=False):
        mx, avg = ctypes.c_double(), ctypes.c_double()
        zp = np.zeros(self.N[2]) if profile else None
        check(self.lib.glasma_gauss(self.h, int(sync_first), ctypes.byref(mx), ctypes.byref(avg),
                                    zp.ctypes.data_as(_lib._D) if profile else None))
        return (mx.value, avg.value, zp) if profile else (mx.value, avg.value)

    def unitarity(self):
        mx, avg = ctypes.c_double(), ctypes.c_double()
        check(self.lib.glasma_unitarity(self.h, ctypes.byref(mx), ctypes.byref(avg)))
        return mx.value, avg.value

    def emt_map(self):
        out = np.zeros((self.N[2], 10))
        check(self.lib.glasma_emt_map(self.h, out.ctypes.data_as(_lib._D)))
        return out

    def pressure_anisotropy(self, z_begin, z_end):
        """(P_L/P_T, P_L, P_T) over slices [z_begin, z_end) from the energy-momentum map."""
        r, pl, pt = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        check(self.lib.glasma_pressure_anisotropy(self.h, int(z_begin), int(z_end), ctypes.byref(r), ctypes.byref(pl),
                                                  ctypes.byref(pt)))
        return r.value, pl.value, pt.value

    # -- adjoint leapfrog
    PL_OVER_PT = ((1, 1, -1, 1, 1, -1), (0, 0, 1, 0, 0, 1))
    ENERGY = ((0.5,) * 6, (0,) * 6)

    def objective(self, z_begin, z_end, form=PL_OVER_PT):
        num = (ctypes.c_double * 6)(*form[0])
        den = (ctypes.c_double * 6)(*form[1])
        v = ctypes.c_double()
        st = self.lib.glasma_objective(self.h, int(z_begin), int(z_end), num, den, ctypes.byref(v))
        if st:
            raise _lib.GlasmaError(st, self.lib.glasma_adjoint_last_error().decode(errors="replace"))
        return v.value

    def adjoint(self, dt, nsteps, z_begin, z_end, form=PL_OVER_PT, checkpoint_every=50, grads=True):
        """Objective after nsteps and its gradient w.r.t. the initial E and currents (host layout;
        None with grads=False, which leaves the gradients on the device unread)."""
        num = (ctypes.c_double * 6)(*form[0])
        den = (ctypes.c_double * 6)(*form[1])
        v = ctypes.c_double()
        names = ("E", "Jp", "Jm", "JpStat", "JmStat")
        out = {k: empty_field(k, self.N) for k in names} if grads else None
        ptrs = [out[k].ctypes.data_as(_lib._D) for k in names] if grads else [None] * 5
        st = self.lib.glasma_adjoint(self.h, float(dt), int(nsteps), int(checkpoint_every), int(z_begin), int(z_end),
                                     num, den, ctypes.byref(v), *ptrs)
        if st:
            raise _lib.GlasmaError(st, self.lib.glasma_adjoint_last_error().decode(errors="replace"))
        return v.value, out

    # -- Coulomb gauge fixing (S/GAUGETRANSFORMATION)
    def coulomb_fix(self, alpha, max_iters, tol=1e-15, project_zero_mode=False, fft_fp32=False,
                    algorithm="fourier", seed=0, open_z=False, mixed=False):
        """Coulomb gauge fixing; returns the per-iteration log rows (n, max dev, avg dev, max step,
        avg step, min functional, functional / V).  algorithm: "fourier" (alpha = the step size of the
        Fourier-accelerated update), "los_alamos" (alpha = the over-relaxation probability; seed picks
        the draws) or "jacobi" (alpha = the step size).  open_z: the open-z functional
        (GLASMA_GF_OPEN_Z, Fourier only), which converges where the reference's iteration does not.
        mixed: FP32 sweeps first, FP64 for the final ones (GLASMA_GF_MIXED, FP64 handles).
        On failure the GlasmaError carries the rows of the iterations that ran (`log`)."""
        log = np.zeros((max(int(max_iters), 1), 7))
        n = ctypes.c_int()
        flags = (_lib.GF_PROJECT_ZERO_MODE if project_zero_mode else 0) | (_lib.GF_FFT_FP32 if fft_fp32 else 0) | \
            (_lib.GF_OPEN_Z if open_z else 0) | (_lib.GF_MIXED if mixed else 0)
        st = self.lib.glasma_coulomb_fix_algorithm(self.h, _lib.GF_ALGORITHMS[algorithm], float(alpha), int(seed),
                                                   int(max_iters), float(tol), flags, log.ctypes.data_as(_lib._D),
                                                   ctypes.byref(n))
        if st:
            e = _lib.GlasmaError(st, self.lib.glasma_last_error().decode(errors="replace"))
            e.log = log[: n.value]
            raise e
        return log[: n.value]

    def fft3d(self, X, inverse=False):
        """Batched 3D FFT of 8 colour planes: X complex128 of shape (8, Nz, Ny, Nx)."""
        X = np.ascontiguousarray(X, dtype=np.complex128)
        assert X.shape == (8, self.N[2], self.N[1], self.N[0])
        out = np.empty_like(X)
        check(self.lib.glasma_fft3d(self.h, X.ctypes.data, out.ctypes.data, int(inverse)))
        return out

    def fft3d_f32(self, X, inverse=False):
        """The same transform in FP32: X complex64 of shape (8, Nz, Ny, Nx)."""
        X = np.ascontiguousarray(X, dtype=np.complex64)
        assert X.shape == (8, self.N[2], self.N[1], self.N[0])
        out = np.empty_like(X)
        check(self.lib.glasma_fft3d_f32(self.h, X.ctypes.data, out.ctypes.data, int(inverse)))
        return out

    def fft3d_device(self, in_ptr, out_ptr, inverse=False, fp32=False):
        """Batched 3D FFT of 8 colour planes between device buffers (8*Nx*Ny*Nz complex doubles, or
        complex floats with fp32)."""
        fn = self.lib.glasma_fft3d_f32 if fp32 else self.lib.glasma_fft3d
        check(fn(self.h, ctypes.c_void_p(int(in_ptr)), ctypes.c_void_p(int(out_ptr)), int(inverse)))

    # -- configuration files
    def save_text(self, links=None, efield=None, currents=None):
        """The reference's text files (IO::SaveConfiguration / SaveConfigurationJ); any path may be None."""
        from .checkpoint import _io_check, _path

        _io_check(self.lib, self.lib.glasma_save_text(self.h, _path(links), _path(efield), _path(currents)))

    def load_text(self, links=None, efield=None, currents=None):
        """Read the reference's text files into the lattice (IO::LoadConfiguration)."""
        from .checkpoint import _io_check, _path

        _io_check(self.lib, self.lib.glasma_load_text(self.h, _path(links), _path(efield), _path(currents)))

    def save_binary(self, path):
        """Bit-exact restart file of U, UOld, E and the four currents."""
        from .checkpoint import _io_check, _path

        _io_check(self.lib, self.lib.glasma_save_binary(self.h, _path(path)))

    def load_binary(self, path):
        from .checkpoint import _io_check, _path

        _io_check(self.lib, self.lib.glasma_load_binary(self.h, _path(path)))

    def gauge_reset(self):
        check(self.lib.glasma_gauge_reset(self.h))

    def transform_charge(self, name, out=None):
        """G(x) j(x) G(x)^dagger of the colour-charge field `name` (Jp, Jm, JpStat, JmStat) with the
        handle's gauge transformation (glasma_transform_charge); the field itself is not changed."""
        if name not in ("Jp", "Jm", "JpStat", "JmStat"):
            raise ValueError("transform_charge takes Jp, Jm, JpStat or JmStat")
        if out is None:
            out = empty_field(name, self.N)
        check(self.lib.glasma_transform_charge(self.h, _lib.FIELDS[name], _address(out, self.field_doubles(name))))
        return out
