"""ctypes access to the CPU checkers (TEST INFRASTRUCTURE ONLY).

* ``liboracle.so``            -- the C restatement of the reference CPU algorithm
                                (oracle/cole_oracle.c), modes FP64 and REF32.
* ``_ref/libbcsim_ref.so``    -- the reference's own CPU algorithm compiled from its
                                sources (oracle/Makefile), present only where the
                                reference sources were available at build time.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, and only as the checker or the timed CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libbcsim_ref.so")

MODE_FP64 = 0
MODE_REF32 = 1
BEAM_GAUSSIAN = 1
BEAM_LUT = 2

_f32p = C.POINTER(C.c_float)


class SplineSetC(C.Structure):
    _fields_ = [("degree", C.c_int), ("num_knots", C.c_int), ("knots", _f32p),
                ("num_scatterers", C.c_int64), ("num_cs", C.c_int),
                ("control_points", _f32p), ("amplitudes", _f32p)]


class CaseC(C.Structure):
    _fields_ = [("taps", _f32p), ("num_taps", C.c_int), ("center_index", C.c_int),
                ("fs", C.c_float), ("demod_freq", C.c_float),
                ("sound_speed", C.c_float), ("use_arc_projection", C.c_int),
                ("phase_delay", C.c_int), ("radial_decimation", C.c_int),
                ("beam", C.c_int), ("sigma_lateral", C.c_float), ("sigma_elevational", C.c_float),
                ("lut", _f32p), ("lut_nr", C.c_int), ("lut_nl", C.c_int), ("lut_ne", C.c_int),
                ("lut_r", C.c_float * 2), ("lut_l", C.c_float * 2), ("lut_e", C.c_float * 2),
                ("num_lines", C.c_int), ("line_length", C.c_float),
                ("origins", _f32p), ("directions", _f32p), ("lateral_dirs", _f32p), ("timestamps", _f32p),
                ("num_fixed_sets", C.c_int), ("fixed_counts", C.POINTER(C.c_int64)),
                ("fixed_xyza", C.POINTER(_f32p)),
                ("num_spline_sets", C.c_int), ("spline_sets", C.POINTER(SplineSetC)),
                ("noise_sigma", C.c_float), ("noise_seed", C.c_uint64), ("noise_frame", C.c_uint32)]


def reference_sources() -> str:
    """Where the reference's source tree is read from: $BCSIM_REF_SRC, else the
    default of oracle/Makefile (the recipe that compiles it).  The directory may
    be absent (then the reference-backed checks are skipped)."""
    env = os.environ.get("BCSIM_REF_SRC")
    if env:
        return env
    out = subprocess.run(["make", "-s", "-C", HERE, "print-ref-src"], capture_output=True, text=True)
    return out.stdout.strip()


def build(quiet: bool = True) -> None:
    """Build liboracle.so (and _ref/ when the reference sources are present)."""
    out = subprocess.run(["make", "-C", HERE, "all"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)


_lib_cache = {}


def _load(path: str):
    if path not in _lib_cache:
        if not os.path.exists(path):
            if path == ORACLE_SO:
                build()
            else:
                raise FileNotFoundError(path)
        lib = C.CDLL(path)
        _lib_cache[path] = lib
    return _lib_cache[path]


def oracle_lib():
    lib = _load(ORACLE_SO)
    lib.oracle_simulate.argtypes = [C.POINTER(CaseC), C.c_int, C.c_int, C.c_int, C.c_int, _f32p, C.c_int64, C.c_char_p, C.c_int]
    lib.oracle_simulate.restype = C.c_int
    lib.oracle_num_rf_samples.argtypes = [C.c_float, C.c_float, C.c_float]
    lib.oracle_num_rf_samples.restype = C.c_int64
    lib.oracle_next_pow2.argtypes = [C.c_int64]
    lib.oracle_next_pow2.restype = C.c_int64
    lib.oracle_hilbert_mask.argtypes = [C.c_int64, C.POINTER(C.c_double)]
    lib.oracle_fft_conv.argtypes = [C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_double)]
    lib.oracle_fft_conv.restype = C.c_int
    lib.oracle_direct_conv_i64.argtypes = [C.POINTER(C.c_int64), C.c_int, C.POINTER(C.c_int64), C.c_int, C.POINTER(C.c_int64)]
    lib.oracle_direct_conv_i64.restype = C.c_int
    lib.oracle_gaussian_excitation.argtypes = [C.c_float, C.c_float, C.c_float, _f32p, C.c_int, C.POINTER(C.c_int)]
    lib.oracle_gaussian_excitation.restype = C.c_int
    lib.oracle_bspline_basis_d.argtypes = [C.c_int, C.c_int, C.c_double, _f32p]
    lib.oracle_bspline_basis_d.restype = C.c_double
    lib.oracle_bspline_basis_f.argtypes = [C.c_int, C.c_int, C.c_float, _f32p]
    lib.oracle_bspline_basis_f.restype = C.c_float
    lib.oracle_knot_interval.argtypes = [_f32p, C.c_int, C.c_float]
    lib.oracle_knot_interval.restype = C.c_int
    lib.oracle_uniform_regular_knots.argtypes = [C.c_int, C.c_int, C.c_float, C.c_float, _f32p, C.c_int]
    lib.oracle_uniform_regular_knots.restype = C.c_int
    lib.oracle_project_bins.argtypes = [C.POINTER(CaseC), C.c_int, C.c_int, C.POINTER(C.c_double), C.c_int64, C.c_char_p, C.c_int]
    lib.oracle_project_bins.restype = C.c_int
    lib.oracle_analytic_spectrum.argtypes = [_f32p, C.c_int, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.oracle_bin_noise.argtypes = [C.c_uint64, C.c_uint32, C.c_int, C.c_int64, C.POINTER(C.c_double),
                                     C.POINTER(C.c_double)]
    lib.oracle_bin_noise.restype = None
    lib.oracle_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.c_uint32, C.c_uint32]
    lib.oracle_philox4x32_10.restype = None
    return lib


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref_lib():
    lib = _load(REF_SO)
    lib.ref_simulate.argtypes = [C.POINTER(CaseC), C.c_int, _f32p, C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.c_char_p, C.c_int]
    lib.ref_simulate.restype = C.c_int
    lib.ref_project_bins.argtypes = [C.POINTER(CaseC), C.c_int, _f32p, C.c_int64, C.POINTER(C.c_int64), C.c_char_p, C.c_int]
    lib.ref_project_bins.restype = C.c_int
    lib.ref_fft_conv.argtypes = [_f32p, C.c_int, _f32p, C.c_int, _f32p]
    lib.ref_fft_conv.restype = C.c_int
    lib.ref_next_power_of_two.argtypes = [C.c_int64]
    lib.ref_next_power_of_two.restype = C.c_int64
    lib.ref_hilbert_mask.argtypes = [C.c_int, C.POINTER(C.c_int)]
    lib.ref_gaussian_excitation.argtypes = [C.c_float, C.c_float, C.c_float, _f32p, C.c_int, C.POINTER(C.c_int)]
    lib.ref_gaussian_excitation.restype = C.c_int
    lib.ref_bspline_basis.argtypes = [C.c_int, C.c_int, C.c_float, _f32p, C.c_int]
    lib.ref_bspline_basis.restype = C.c_float
    lib.ref_knot_interval.argtypes = [_f32p, C.c_int, C.c_float]
    lib.ref_knot_interval.restype = C.c_int
    lib.ref_uniform_regular_knots.argtypes = [C.c_int, C.c_int, C.c_float, C.c_float, _f32p, C.c_int]
    lib.ref_uniform_regular_knots.restype = C.c_int
    return lib


def fptr(a: np.ndarray):
    return a.ctypes.data_as(_f32p)


class Case:
    """Holds the numpy arrays of one job alive while a CaseC points at them."""

    def __init__(self, job, lines: Optional[slice] = None):
        self.keep = []
        c = CaseC()
        taps = np.ascontiguousarray(job.taps, np.float32)
        self.keep.append(taps)
        c.taps, c.num_taps, c.center_index = fptr(taps), len(taps), int(job.center_index)
        c.fs, c.demod_freq = job.fs, job.demod_freq
        c.sound_speed, c.use_arc_projection = job.sound_speed, int(job.arc)
        c.phase_delay, c.radial_decimation = int(job.phase_delay), int(job.decimation)
        beam = job.beam
        if hasattr(beam, "sigma_lateral"):
            c.beam, c.sigma_lateral, c.sigma_elevational = BEAM_GAUSSIAN, beam.sigma_lateral, beam.sigma_elevational
        else:
            lut = np.ascontiguousarray(beam.samples, np.float32)
            self.keep.append(lut)
            c.beam, c.lut = BEAM_LUT, fptr(lut)
            c.lut_nr, c.lut_nl, c.lut_ne = lut.shape
            c.lut_r[0], c.lut_r[1] = beam.r_range
            c.lut_l[0], c.lut_l[1] = beam.l_range
            c.lut_e[0], c.lut_e[1] = beam.e_range
        scan = job.scan
        arrs = [np.ascontiguousarray(a, np.float32) for a in (scan.origins, scan.directions, scan.lateral_dirs, scan.timestamps)]
        self.keep += arrs
        c.num_lines, c.line_length = scan.num_lines, scan.line_length
        c.origins, c.directions, c.lateral_dirs, c.timestamps = [fptr(a) for a in arrs]
        nf = len(job.fixed)
        counts = (C.c_int64 * max(1, nf))(*[f.xyza.shape[0] for f in job.fixed])
        ptrs = (_f32p * max(1, nf))()
        for i, f in enumerate(job.fixed):
            a = np.ascontiguousarray(f.xyza, np.float32)
            self.keep.append(a)
            ptrs[i] = fptr(a)
        self.keep += [counts, ptrs]
        c.num_fixed_sets, c.fixed_counts, c.fixed_xyza = nf, counts, ptrs
        ns = len(job.splines)
        sets = (SplineSetC * max(1, ns))()
        for i, s in enumerate(job.splines):
            k = np.ascontiguousarray(s.knots, np.float32)
            cp = np.ascontiguousarray(s.control_points, np.float32)
            am = np.ascontiguousarray(s.amplitudes, np.float32)
            self.keep += [k, cp, am]
            sets[i].degree, sets[i].num_knots, sets[i].knots = s.degree, len(k), fptr(k)
            sets[i].num_scatterers, sets[i].num_cs = cp.shape[0], cp.shape[1]
            sets[i].control_points, sets[i].amplitudes = fptr(cp), fptr(am)
        self.keep.append(sets)
        c.num_spline_sets, c.spline_sets = ns, sets
        c.noise_sigma = float(getattr(job, "noise_amplitude", 0.0))
        c.noise_seed = int(getattr(job, "noise_seed", 0))
        c.noise_frame = int(getattr(job, "noise_frame", 0))
        self.c = c


def simulate(job, mode: int = MODE_FP64, threads: int = 0, line_begin: int = 0, line_end: int = -1) -> np.ndarray:
    """Run the oracle; returns complex64 [L, nd] (rows line_begin..line_end)."""
    lib = oracle_lib()
    case = Case(job)
    L = job.scan.num_lines
    if line_end < 0:
        line_end = L
    nd = job.num_out
    out = np.zeros((line_end - line_begin, nd), np.complex64)
    err = C.create_string_buffer(512)
    rc = lib.oracle_simulate(C.byref(case.c), mode, threads, line_begin, line_end,
                             out.ctypes.data_as(_f32p), out.size * 2, err, 512)
    if rc != 0:
        raise RuntimeError(err.value.decode())
    return out


def ref_simulate(job, threads: int = 0) -> np.ndarray:
    """Run the compiled reference CPU algorithm; returns complex64 [L, nd]."""
    lib = ref_lib()
    case = Case(job)
    L, nd = job.scan.num_lines, job.num_out
    out = np.zeros((L, nd), np.complex64)
    nl, nsmp = C.c_int64(), C.c_int64()
    err = C.create_string_buffer(512)
    rc = lib.ref_simulate(C.byref(case.c), threads, out.ctypes.data_as(_f32p), out.size * 2,
                          C.byref(nl), C.byref(nsmp), err, 512)
    if rc != 0:
        raise RuntimeError(err.value.decode())
    return out


def bin_noise(seed: int, frame: int, line: int, count: int) -> np.ndarray:
    """Unit-variance seeded noise of samples 0..count-1 of one line: complex128 [count]."""
    lib = oracle_lib()
    out = np.empty(count, np.complex128)
    re, im = C.c_double(), C.c_double()
    for j in range(count):
        lib.oracle_bin_noise(seed, frame, line, j, C.byref(re), C.byref(im))
        out[j] = complex(re.value, im.value)
    return out


def rel_rms(a: np.ndarray, b: np.ndarray) -> float:
    """||a - b||_2 / ||b||_2 over all lines and samples (complex)."""
    a = a.astype(np.complex128)
    b = b.astype(np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def project_bins(job, line: int, mode: int = MODE_FP64) -> np.ndarray:
    """Oracle time-projection bins of one line: complex128 [ns]."""
    lib = oracle_lib()
    case = Case(job)
    ns = job.num_samples
    out = np.zeros(ns, np.complex128)
    err = C.create_string_buffer(512)
    rc = lib.oracle_project_bins(C.byref(case.c), mode, line, out.ctypes.data_as(C.POINTER(C.c_double)), ns, err, 512)
    if rc != 0:
        raise RuntimeError(err.value.decode())
    return out


def ref_project_bins(job, line: int) -> np.ndarray:
    """Reference (compiled) time-projection bins of one line: complex64 [ns]."""
    lib = ref_lib()
    case = Case(job)
    ns = job.num_samples
    out = np.zeros(ns, np.complex64)
    n = C.c_int64()
    err = C.create_string_buffer(512)
    rc = lib.ref_project_bins(C.byref(case.c), line, out.ctypes.data_as(_f32p), ns, C.byref(n), err, 512)
    if rc != 0:
        raise RuntimeError(err.value.decode())
    assert n.value == ns, (n.value, ns)
    return out
