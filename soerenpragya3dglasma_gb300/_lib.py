"""ctypes binding of libglasma_gb300.so (the C ABI in include/glasma_gb300.h).

The library is the only compute path: if it is missing or cannot be loaded,
every entry point raises instead of falling back to anything else.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libglasma_gb300.so")

GLASMA_OK = 0
STATUS_NAMES = {
    0: "GLASMA_OK", 1: "GLASMA_ERR_INVALID_ARGUMENT", 2: "GLASMA_ERR_BAD_SHAPE", 3: "GLASMA_ERR_OUT_OF_MEMORY",
    4: "GLASMA_ERR_CUDA", 5: "GLASMA_ERR_NUMERICAL", 6: "GLASMA_ERR_TIMEOUT", 7: "GLASMA_ERR_UNSUPPORTED",
}
FP64, FP32 = 0, 1
FIELDS = {"U": 0, "UOld": 1, "E": 2, "Jp": 3, "Jm": 4, "JpStat": 5, "JmStat": 6, "G": 7, "UG": 8, "EG": 9}
STEP_SAVE_UOLD = 0x1
GF_PROJECT_ZERO_MODE = 0x1
GF_FFT_FP32 = 0x2
GF_OPEN_Z = 0x4
GF_MIXED = 0x8
GF_ALGORITHMS = {"fourier": 0, "los_alamos": 1, "jacobi": 2}



class TmdParams(ctypes.Structure):
    """glasma_tmd_params (include/glasma_gb300.h)."""
    _fields_ = [("atomic_number", ctypes.c_int), ("qs0a", ctypes.c_double), ("meff", ctypes.c_double),
                ("ax_fm", ctypes.c_double), ("ay_fm", ctypes.c_double), ("az_fm", ctypes.c_double),
                ("com_energy", ctypes.c_double), ("center_left", ctypes.c_int), ("center_right", ctypes.c_int),
                ("dt", ctypes.c_double)]


# (name, restype, argtypes) for every symbol declared in include/glasma_gb300.h
_H = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
SIGNATURES = [
    ("glasma_create", ctypes.c_int, [ctypes.c_int] * 3 + [ctypes.c_double] * 3 + [ctypes.c_int, ctypes.c_int,
                                                                                  ctypes.POINTER(ctypes.c_void_p)]),
    ("glasma_destroy", ctypes.c_int, [_H]),
    ("glasma_set_stream", ctypes.c_int, [_H, ctypes.c_void_p]),
    ("glasma_set_scale", ctypes.c_int, [_H, ctypes.c_double]),
    ("glasma_get_shape", ctypes.c_int, [_H, _I, _I, _I, _I]),
    ("glasma_field_doubles", ctypes.c_longlong, [_H, ctypes.c_int]),
    ("glasma_upload", ctypes.c_int, [_H, ctypes.c_int, ctypes.c_void_p]),
    ("glasma_download", ctypes.c_int, [_H, ctypes.c_int, ctypes.c_void_p]),
    ("glasma_upload_device", ctypes.c_int, [_H, ctypes.c_int, ctypes.c_void_p]),
    ("glasma_download_device", ctypes.c_int, [_H, ctypes.c_int, ctypes.c_void_p]),
    ("glasma_step", ctypes.c_int, [_H, ctypes.c_double, ctypes.c_int, ctypes.c_uint]),
    ("glasma_step_profiled", ctypes.c_int, [_H, ctypes.c_double, ctypes.c_int, ctypes.c_uint, _D]),
    ("glasma_set_step_method", ctypes.c_int, [_H, ctypes.c_int]),
    ("glasma_get_step_method", ctypes.c_int, [_H, _I]),
    ("glasma_set_march_chunk", ctypes.c_int, [_H, ctypes.c_int]),
    ("glasma_set_link_storage", ctypes.c_int, [_H, ctypes.c_int]),
    ("glasma_set_fp64_arithmetic", ctypes.c_int, [_H, ctypes.c_int]),
    ("glasma_get_fp64_arithmetic", ctypes.c_int, [_H, _I]),
    ("glasma_get_link_storage", ctypes.c_int, [_H, _I]),
    ("glasma_update_efield", ctypes.c_int, [_H, ctypes.c_double]),
    ("glasma_update_jstat", ctypes.c_int, [_H, ctypes.c_double]),
    ("glasma_update_links", ctypes.c_int, [_H, ctypes.c_double]),
    ("glasma_save_old_link", ctypes.c_int, [_H]),
    ("glasma_update_j", ctypes.c_int, [_H, ctypes.c_double]),
    ("glasma_bulk", ctypes.c_int, [_H, _D]),
    ("glasma_gauss", ctypes.c_int, [_H, ctypes.c_int, _D, _D, _D]),
    ("glasma_unitarity", ctypes.c_int, [_H, _D, _D]),
    ("glasma_emt_map", ctypes.c_int, [_H, _D]),
    ("glasma_pressure_anisotropy", ctypes.c_int, [_H, ctypes.c_int, ctypes.c_int, _D, _D, _D]),
    ("glasma_reunitarize", ctypes.c_int, [_H]),
    ("glasma_upload_begin", ctypes.c_int, [_H, ctypes.c_int, ctypes.c_void_p]),
    ("glasma_upload_finish", ctypes.c_int, [_H]),
    ("glasma_coulomb_fix", ctypes.c_int, [_H, ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_uint, _D, _I]),
    ("glasma_coulomb_fix_algorithm", ctypes.c_int, [_H, ctypes.c_int, ctypes.c_double, ctypes.c_ulonglong,
                                                    ctypes.c_int, ctypes.c_double, ctypes.c_uint, _D, _I]),
    ("glasma_gauge_reset", ctypes.c_int, [_H]),
    ("glasma_transform_charge", ctypes.c_int, [_H, ctypes.c_int, ctypes.c_void_p]),
    ("glasma_mv_init", ctypes.c_int, [_H, ctypes.c_int, _D, _D, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double]),
    ("glasma_mv_last_error", ctypes.c_char_p, []),
    ("glasma_tmd_default_params", None, [ctypes.POINTER(TmdParams), ctypes.c_double]),
    ("glasma_glauber_sample", ctypes.c_int, [ctypes.c_int, _D, ctypes.c_long, _D, ctypes.POINTER(ctypes.c_long)]),
    ("glasma_tmd_init", ctypes.c_int, [_H, _D, _D, _D, _D, ctypes.POINTER(TmdParams), _D, _D]),
    ("glasma_fill_synthetic", ctypes.c_int, [_H, ctypes.c_ulonglong, ctypes.c_double, ctypes.c_double,
                                             ctypes.c_double]),
    ("glasma_autotune", ctypes.c_int, [_H, ctypes.c_double, _I]),
    ("glasma_set_tile", ctypes.c_int, [_H, ctypes.c_int]),
    ("glasma_fft3d", ctypes.c_int, [_H, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    ("glasma_fft3d_f32", ctypes.c_int, [_H, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    ("glasma_save_text", ctypes.c_int, [_H, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p]),
    ("glasma_load_text", ctypes.c_int, [_H, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p]),
    ("glasma_write_text_host", ctypes.c_int, [ctypes.c_int] * 3 + [ctypes.c_void_p] * 6 + [ctypes.c_char_p] * 3),
    ("glasma_read_text_host", ctypes.c_int, [ctypes.c_int] * 3 + [ctypes.c_void_p] * 6 + [ctypes.c_char_p] * 3),
    ("glasma_save_binary", ctypes.c_int, [_H, ctypes.c_char_p]),
    ("glasma_load_binary", ctypes.c_int, [_H, ctypes.c_char_p]),
    ("glasma_io_last_error", ctypes.c_char_p, []),
    ("glasma_gauss_noalloc", ctypes.c_int, [ctypes.c_void_p] * 4 + [ctypes.c_int] * 3 + [ctypes.c_double] * 4 +
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    ("glasma_objective", ctypes.c_int, [_H, ctypes.c_int, ctypes.c_int, _D, _D, _D]),
    ("glasma_adjoint", ctypes.c_int, [_H, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      _D, _D, _D, _D, _D, _D, _D, _D]),
    ("glasma_adjoint_last_error", ctypes.c_char_p, []),
    ("glasma_batch_create", ctypes.c_int, [ctypes.c_int, _I, _D, ctypes.c_int, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_void_p)]),
    ("glasma_batch_destroy", ctypes.c_int, [_H]),
    ("glasma_batch_set_stream", ctypes.c_int, [_H, ctypes.c_void_p]),
    ("glasma_batch_event", ctypes.c_int, [_H, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    ("glasma_batch_autotune", ctypes.c_int, [_H, ctypes.c_double, _I]),
    ("glasma_batch_step", ctypes.c_int, [_H, ctypes.c_double, ctypes.c_int, ctypes.c_int]),
    ("glasma_batch_set_launch", ctypes.c_int, [_H, ctypes.c_int]),
    ("glasma_batch_set_step_method", ctypes.c_int, [_H, ctypes.c_int]),
    ("glasma_batch_get_step_method", ctypes.c_int, [_H, ctypes.POINTER(ctypes.c_int)]),
    ("glasma_batch_set_link_storage", ctypes.c_int, [_H, ctypes.c_int]),
    ("glasma_batch_energy", ctypes.c_int, [_H, _D]),
    ("glasma_batch_synchronize", ctypes.c_int, [_H]),
    ("glasma_batch_last_error", ctypes.c_char_p, []),
    ("glasma_synchronize", ctypes.c_int, [_H]),
    ("glasma_status_string", ctypes.c_char_p, [ctypes.c_int]),
    ("glasma_last_error", ctypes.c_char_p, []),
]

_lib = None


class GlasmaError(RuntimeError):
    def __init__(self, status, message):
        self.status = status
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), message))


def load(path=LIB_PATH):
    """Load (once) and return the CDLL with argtypes set.  Raises if the library is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libglasma_gb300.so is not built (%s); run soerenpragya3dglasma_gb300.build.build()" % path)
    lib = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status):
    if status != GLASMA_OK:
        msg = _lib.glasma_last_error().decode(errors="replace") if _lib is not None else ""
        raise GlasmaError(status, msg)
    return status
