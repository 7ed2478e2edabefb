"""ctypes access to the CPU checkers of the image formation (TEST INFRASTRUCTURE ONLY).

* ``liboracle.so`` (oracle/imaging_oracle.c) -- restatement of the reference's
  B-mode and colour-Doppler steps after simulate_lines.
* ``_ref/libbcsim_ref.so`` -- the reference's own scan converter
  (CpuCartesianator, src/utils/cartesianator/Cartesianator.cpp) where the
  reference sources were available at build time.

Geometries are tuples (kind, width, depth, tilt, nx, ny) with kind 0 = sector,
1 = linear, or objects with those attributes (kind "sector" / "linear").
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .oracle import oracle_lib, ref_lib

_f32p = C.POINTER(C.c_float)
_u8p = C.POINTER(C.c_uint8)
_GEOM = [C.c_int, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int]
_configured = set()


def _lib():
    lib = oracle_lib()
    if "img" not in _configured:
        lib.oracle_max_value.argtypes = [_f32p, C.c_int64]
        lib.oracle_max_value.restype = C.c_float
        lib.oracle_envelope.argtypes = [_f32p, C.c_int64, _f32p]
        lib.oracle_log_compress.argtypes = [_f32p, C.c_int64, C.c_float, C.c_float, C.c_float, _f32p, _u8p]
        lib.oracle_scan_convert_f32.argtypes = [_f32p, C.c_int, C.c_int] + _GEOM + [_f32p]
        lib.oracle_scan_convert_u8.argtypes = [_u8p, C.c_int, C.c_int] + _GEOM + [_u8p]
        lib.oracle_color_doppler.argtypes = [_f32p, C.c_int, C.c_int64, _f32p, _f32p]
        lib.oracle_color_image.argtypes = [_f32p, _f32p, C.c_int, C.c_int] + _GEOM + [_f32p, _f32p, _f32p, _u8p]
        _configured.add("img")
    return lib


def _rlib():
    lib = ref_lib()
    if "ref" not in _configured:
        lib.ref_scan_convert_f32.argtypes = [_f32p, C.c_int, C.c_int] + _GEOM + [_f32p]
        lib.ref_scan_convert_f32.restype = C.c_int
        lib.ref_scan_convert_u8.argtypes = [_u8p, C.c_int, C.c_int] + _GEOM + [_u8p]
        lib.ref_scan_convert_u8.restype = C.c_int
        _configured.add("ref")
    return lib


def geom_tuple(g):
    if isinstance(g, tuple):
        return g
    return (0 if g.kind == "sector" else 1, float(g.width), float(g.depth), float(g.tilt), int(g.nx), int(g.ny))


def _f(a):
    return a.ctypes.data_as(_f32p)


def _u(a):
    return a.ctypes.data_as(_u8p)


def envelope(iq) -> np.ndarray:
    iq = np.ascontiguousarray(iq, np.complex64)
    out = np.empty(iq.shape, np.float32)
    _lib().oracle_envelope(_f(iq), iq.size, _f(out))
    return out


def max_value(v) -> float:
    v = np.ascontiguousarray(v, np.float32)
    return float(_lib().oracle_max_value(_f(v), v.size))


def log_compress(env, dyn_range, normalize, gain):
    env = np.ascontiguousarray(env, np.float32)
    f = np.empty(env.shape, np.float32)
    b = np.empty(env.shape, np.uint8)
    _lib().oracle_log_compress(_f(env), env.size, dyn_range, normalize, gain, _f(f), _u(b))
    return f, b


def scan_convert(beamspace, geometry) -> np.ndarray:
    g = geom_tuple(geometry)
    if beamspace.dtype == np.uint8:
        b = np.ascontiguousarray(beamspace)
        out = np.empty((g[5], g[4]), np.uint8)
        _lib().oracle_scan_convert_u8(_u(b), b.shape[0], b.shape[1], *g, _u(out))
    else:
        b = np.ascontiguousarray(beamspace, np.float32)
        out = np.empty((g[5], g[4]), np.float32)
        _lib().oracle_scan_convert_f32(_f(b), b.shape[0], b.shape[1], *g, _f(out))
    return out


def ref_scan_convert(beamspace, geometry) -> np.ndarray:
    """The reference's own CpuCartesianator (needs oracle/_ref)."""
    g = geom_tuple(geometry)
    lib = _rlib()
    if beamspace.dtype == np.uint8:
        b = np.ascontiguousarray(beamspace)
        out = np.empty((g[5], g[4]), np.uint8)
        rc = lib.ref_scan_convert_u8(_u(b), b.shape[0], b.shape[1], *g, _u(out))
    else:
        b = np.ascontiguousarray(beamspace, np.float32)
        out = np.empty((g[5], g[4]), np.float32)
        rc = lib.ref_scan_convert_f32(_f(b), b.shape[0], b.shape[1], *g, _f(out))
    if rc != 0:
        raise RuntimeError("reference scan conversion failed")
    return out


def bmode(iq, dyn_range, gain, normalize=0.0, geometry=None):
    """(image or None, beam-space bytes, normalize used) as the reference's
    worker computes them (RefreshWorker.hpp:179-246)."""
    env = envelope(iq)
    norm = max_value(env) if normalize <= 0 else float(normalize)
    _, b = log_compress(env, dyn_range, norm, gain)
    img = scan_convert(b, geometry) if geometry is not None else None
    return img, b, norm


def color_doppler(packet):
    """R0 and arg R1 [lines, samples] of a packet [P, lines, samples]."""
    p = np.ascontiguousarray(packet, np.complex64)
    P = p.shape[0]
    n = p[0].size
    r0 = np.empty(p.shape[1:], np.float32)
    vel = np.empty(p.shape[1:], np.float32)
    _lib().oracle_color_doppler(_f(p), P, n, _f(r0), _f(vel))
    return r0, vel


def color_image(r0, vel, geometry) -> np.ndarray:
    g = geom_tuple(geometry)
    r0 = np.ascontiguousarray(r0, np.float32)
    vel = np.ascontiguousarray(vel, np.float32)
    wp = np.empty((g[5], g[4]), np.float32)
    wv = np.empty((g[5], g[4]), np.float32)
    wb = np.empty(r0.shape, np.float32)
    out = np.empty((g[5], g[4], 4), np.uint8)
    _lib().oracle_color_image(_f(r0), _f(vel), r0.shape[0], r0.shape[1], *g, _f(wp), _f(wv), _f(wb), _u(out))
    return out
