"""ctypes binding of include/bcsim_gb300.h (libbcsim_gb300.so, built in-tree).

The library is required: importing this module without it raises, there is no
CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libbcsim_gb300.so")

OK = 0
E_INVALID, E_NOT_CONFIGURED, E_CUDA, E_CAPACITY, E_MEMORY, E_INTERNAL, E_PENDING = 1, 2, 3, 4, 5, 6, 7

# every symbol the header declares: (name, restype, argtypes)
_f32p = C.POINTER(C.c_float)
_i64p = C.POINTER(C.c_int64)
LOG_FN = C.CFUNCTYPE(None, C.c_int, C.c_char_p, C.c_void_p)
SIGNATURES = [
    ("bcsim_create", C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    ("bcsim_destroy", C.c_int, [C.c_void_p]),
    ("bcsim_last_error", C.c_char_p, [C.c_void_p]),
    ("bcsim_set_parameter", C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p]),
    ("bcsim_get_parameter", C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_int]),
    ("bcsim_set_excitation", C.c_int, [C.c_void_p, _f32p, C.c_int, C.c_int, C.c_float, C.c_float]),
    ("bcsim_set_scan_sequence", C.c_int, [C.c_void_p, _f32p, _f32p, _f32p, _f32p, C.c_int, C.c_float]),
    ("bcsim_set_analytical_profile", C.c_int, [C.c_void_p, C.c_float, C.c_float]),
    ("bcsim_set_lookup_profile", C.c_int, [C.c_void_p, _f32p, C.c_int, C.c_int, C.c_int,
                                           C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float]),
    ("bcsim_clear_fixed_scatterers", C.c_int, [C.c_void_p]),
    ("bcsim_add_fixed_scatterers", C.c_int, [C.c_void_p, _f32p, C.c_int64]),
    ("bcsim_set_fixed_scatterers", C.c_int, [C.c_void_p, _f32p, C.c_int64]),
    ("bcsim_clear_spline_scatterers", C.c_int, [C.c_void_p]),
    ("bcsim_add_spline_scatterers", C.c_int, [C.c_void_p, C.c_int, _f32p, C.c_int, _f32p, _f32p, C.c_int64, C.c_int]),
    ("bcsim_set_spline_scatterers", C.c_int, [C.c_void_p, C.c_int, _f32p, C.c_int, _f32p, _f32p, C.c_int64, C.c_int]),
    ("bcsim_get_total_num_scatterers", C.c_int, [C.c_void_p, _i64p]),
    ("bcsim_get_output_shape", C.c_int, [C.c_void_p, _i64p, _i64p]),
    ("bcsim_simulate_lines", C.c_int, [C.c_void_p, _f32p, C.c_int64, _i64p, _i64p]),
    ("bcsim_simulate_fixed_frames", C.c_int, [C.c_void_p, C.POINTER(_f32p), C.c_int64, C.c_int, C.POINTER(_f32p),
                                              C.c_int64]),
    ("bcsim_simulate_spline_frames", C.c_int, [C.c_void_p, C.c_int, _f32p, C.c_int, C.POINTER(_f32p),
                                               C.POINTER(_f32p), C.c_int64, C.c_int, C.c_int, C.POINTER(_f32p),
                                               C.c_int64]),
    ("bcsim_simulate_lines_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64]),
    ("bcsim_get_stream", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    ("bcsim_get_debug_data", C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_double), C.c_int64, _i64p]),
    ("bcsim_set_logger", C.c_int, [C.c_void_p, LOG_FN, C.c_void_p]),
    ("bcsim_debug_raise_wait_flag", C.c_int, [C.c_void_p]),
    ("bcsim_batch_create", C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    ("bcsim_batch_destroy", C.c_int, [C.c_void_p]),
    ("bcsim_batch_last_error", C.c_char_p, [C.c_void_p]),
    ("bcsim_batch_run", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), _i64p]),
    ("bcsim_batch_run_device", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), _i64p, C.POINTER(C.c_void_p)]),
    ("bcsim_server_create", C.c_int, [C.c_int64, C.c_int, C.POINTER(C.c_void_p)]),
    ("bcsim_server_destroy", C.c_int, [C.c_void_p]),
    ("bcsim_server_last_error", C.c_char_p, [C.c_void_p]),
    ("bcsim_server_set_max_in_flight", C.c_int, [C.c_void_p, C.c_int]),
    ("bcsim_server_add_phantom", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_int)]),
    ("bcsim_server_submit", C.c_int, [C.c_void_p, C.c_int, _f32p, _f32p, _f32p, _f32p, C.c_int, C.c_float, C.c_int,
                                      _i64p]),
    ("bcsim_server_wait", C.c_int, [C.c_void_p, C.c_int64, _f32p, C.c_int64, _i64p, _i64p,
                                    C.POINTER(C.c_double), C.c_int]),
    ("bcsim_server_stats", C.c_int, [C.c_void_p, _i64p, _i64p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                     _i64p, _i64p, _i64p]),
    ("bcsim_server_debug_inject", C.c_int, [C.c_void_p, C.c_int, C.c_int64]),
    ("bcsim_bmode_image", C.c_int, [C.c_void_p, _f32p, C.c_int64, C.c_int64, C.c_float, C.c_float, C.c_float,
                                    C.c_void_p, C.c_void_p, C.c_void_p, _f32p]),
    ("bcsim_simulate_bmode", C.c_int, [C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_void_p, C.c_void_p,
                                       C.c_void_p, _f32p]),
    ("bcsim_scan_convert", C.c_int, [C.c_void_p, _f32p, C.c_int64, C.c_int64, C.c_void_p, _f32p]),
    ("bcsim_simulate_packet", C.c_int, [C.c_void_p, C.c_int, C.c_float, _f32p, C.c_int64]),
    ("bcsim_color_doppler", C.c_int, [C.c_void_p, _f32p, C.c_int, C.c_int64, C.c_int64, _f32p, _f32p, C.c_void_p,
                                      C.c_void_p]),
    ("bcsim_simulate_color_doppler", C.c_int, [C.c_void_p, C.c_int, C.c_float, _f32p, _f32p, C.c_void_p,
                                               C.c_void_p]),
    ("bcsim_simulate_fixed_noalloc", C.c_int,
     [C.c_void_p, C.c_int64, _f32p, _f32p, _f32p, C.c_int, C.c_float, C.c_float, _f32p, C.c_int, C.c_int,
      C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int, C.c_int, C.c_float, C.c_void_p, C.c_int64,
      C.c_void_p, C.c_char_p, C.c_int]),
]



class ScanGeometryC(C.Structure):
    """bcsim_scan_geometry"""
    _fields_ = [("kind", C.c_int), ("width", C.c_float), ("depth", C.c_float), ("tilt", C.c_float),
                ("nx", C.c_int), ("ny", C.c_int)]


GEOMETRY_SECTOR, GEOMETRY_LINEAR = 0, 1

_lib = None


def load(path: str = LIB_PATH):
    """Load the engine library (once).  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -m openbcsim_gb300.build` "
                          "(there is no CPU fallback)")
    lib = C.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
