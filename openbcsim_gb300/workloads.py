"""Seeded synthetic inputs for the COLE simulator: excitation pulses, scan
geometries, beam lookup tables and phantoms.

The reference builds its inputs with `MakeGaussianExcitation`
(src/utils/GaussPulse.cpp:33-70), sector/volume scan builders
(python/benchmark_paper.py:27-38, src/utils/BCSimConvenience.cpp), Field II
lookup tables (utilities/make_lut.py:134-143) and HDF5 phantoms written by
phantom_scripts/.  HDF5 is not available here, so every workload below is a
seeded synthetic stand-in with the shapes, sizes and value distributions of the
reference's own inputs.

Workloads (numpy ``default_rng(1000 * workload + job)``):

* ``sector_2d_fixed``   -- 100k fixed scatterers in x in [-3,3] cm, y = 0, z in [1,12] cm,
  128 lines over +-35 deg, 2.5 MHz / bw 0.1 / 50 MHz, Gaussian beam 1 mm, decimation 10.
* ``volume_3d_lut``     -- 2M fixed scatterers in a 6x6x11 cm box from z = 1 cm,
  64x64 lines over +-30 deg azimuth and elevation, 256x64x64 float32 beam LUT,
  3.5 MHz / bw 0.15 / 50 MHz, decimation 8, line length 13 cm.
* ``sector_spline``     -- 500k cubic B-spline scatterers with 16 control points,
  1024 sector lines with their own timestamps over [0, 1) s, Gaussian beam,
  2.5 MHz / 50 MHz, decimation 10.
* ``batch_uneven``      -- 64 independent jobs with uneven scatterer counts, line
  counts, depths and pulses, half of them spline phantoms.
* ``served_stream``     -- a Poisson request stream over 8 resident phantoms.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

SOUND_SPEED = 1540.0
FS = 50e6


# ---------------------------------------------------------------------------
# excitation (src/utils/GaussPulse.cpp:33-70)
# ---------------------------------------------------------------------------
def gaussian_pulse_time_limit(fc: float, bw: float, bwr: float = -6.0, tpr: float = -60.0) -> float:
    """GaussianPulseTimeLimits (GaussPulse.cpp:33-38), in double."""
    pi = 4.0 * math.atan(1.0)
    f_cutoff = bw * fc
    return math.sqrt(-tpr / (20.0 * (-pi * pi * f_cutoff * f_cutoff /
                                      math.log(10.0 ** (bwr / 20.0))) * math.log10(math.e)))


_LIBM = None


def _libm():
    """The C library's math (cosf, exp): the functions the reference's float
    template calls, so that the taps come out bit for bit as its own."""
    global _LIBM
    if _LIBM is None:
        import ctypes
        import ctypes.util

        try:
            lib = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
            lib.cosf.restype, lib.cosf.argtypes = ctypes.c_float, [ctypes.c_float]
            lib.exp.restype, lib.exp.argtypes = ctypes.c_double, [ctypes.c_double]
            _LIBM = lib
        except (OSError, AttributeError):
            _LIBM = False
    return _LIBM


def gaussian_excitation(fc: float, bw: float, fs: float):
    """MakeGaussianExcitation<float> (GaussPulse.cpp:52-70).

    Returns (taps float32 [n], center_index).  The arithmetic follows the
    reference's float/double mix: the time, the envelope's exponent numerator
    and the cosine's argument in float, the exponent divided by a double
    log(10^(-6/20)) and exponentiated in double, the cosine in float (the
    float overload, the C library's cosf), their product rounded to float.
    With the C library's cosf and exp the taps equal the reference's bit for
    bit; without them (numpy's own functions) they may differ by an ulp.
    """
    fc32, bw32, fs32 = np.float32(fc), np.float32(bw), np.float32(fs)
    lim = gaussian_pulse_time_limit(float(fc32), float(bw32))
    n = int(2 * lim * float(fs32))
    i = np.arange(n)
    t = ((i - n // 2).astype(np.float32) / fs32).astype(np.float32)
    pi32 = np.float32(4.0 * math.atan(1.0))
    f_cutoff = np.float32(bw32 * fc32)
    ftp = (f_cutoff * t).astype(np.float32)
    ppf = (((pi32 * pi32) * ftp).astype(np.float32) * ftp).astype(np.float32)
    den = math.log(10.0 ** (-6.0 / 20.0))
    arg = (((np.float32(2) * pi32) * fc32).astype(np.float32) * t).astype(np.float32)
    lib = _libm()
    if lib:
        env = np.array([lib.exp(float(v) / den) for v in ppf], np.float64)
        cos32 = np.array([lib.cosf(float(v)) for v in arg], np.float32)
    else:
        env = np.exp(ppf.astype(np.float64) / den)
        cos32 = np.cos(arg.astype(np.float64)).astype(np.float32)
    taps = (env * cos32.astype(np.float64)).astype(np.float32)
    return taps, n // 2


def num_rf_samples(sound_speed: float, line_length: float, fs: float) -> int:
    """compute_num_rf_samples<float> (src/core/algorithm/common_utils.hpp:38-41)."""
    max_time = np.float32(2.0 * float(np.float32(line_length)) / float(np.float32(sound_speed)))
    prod = np.float32(np.float32(fs) * max_time)
    return int(math.floor(float(prod) + 0.5))


# ---------------------------------------------------------------------------
# scan geometry
# ---------------------------------------------------------------------------
def _rot_y(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])


def _rot_x(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[1, 0, 0], [0, c, -s], [0, s, c]])


@dataclass
class ScanSequence:
    origins: np.ndarray        # [L,3] float32
    directions: np.ndarray     # [L,3] float32
    lateral_dirs: np.ndarray   # [L,3] float32
    timestamps: np.ndarray     # [L]   float32
    line_length: float

    @property
    def num_lines(self) -> int:
        return int(self.origins.shape[0])


def sector_scan(num_lines: int, half_angle_deg: float, line_length: float,
                timestamps: Optional[np.ndarray] = None, angles_deg: Optional[np.ndarray] = None) -> ScanSequence:
    """2-D sector from the origin in the xz-plane: direction R_y(theta) z, lateral
    R_y(theta) x (the convention of python/benchmark_paper.py:32-38)."""
    if angles_deg is None:
        angles_deg = np.linspace(-half_angle_deg, half_angle_deg, num_lines)
    dirs = np.empty((num_lines, 3))
    lats = np.empty((num_lines, 3))
    for i, a in enumerate(np.radians(angles_deg)):
        m = _rot_y(a)
        dirs[i] = m @ np.array([0.0, 0.0, 1.0])
        lats[i] = m @ np.array([1.0, 0.0, 0.0])
    ts = np.zeros(num_lines, np.float32) if timestamps is None else np.asarray(timestamps, np.float32)
    return ScanSequence(np.zeros((num_lines, 3), np.float32), dirs.astype(np.float32),
                        lats.astype(np.float32), ts, float(line_length))


def volume_scan(n_az: int, n_el: int, half_az_deg: float, half_el_deg: float, line_length: float) -> ScanSequence:
    """3-D pyramid from the origin: direction R_x(phi) R_y(theta) z, lateral
    R_x(phi) R_y(theta) x; azimuth theta is the fast index."""
    dirs, lats = [], []
    for phi in np.radians(np.linspace(-half_el_deg, half_el_deg, n_el)):
        for theta in np.radians(np.linspace(-half_az_deg, half_az_deg, n_az)):
            m = _rot_x(phi) @ _rot_y(theta)
            dirs.append(m @ np.array([0.0, 0.0, 1.0]))
            lats.append(m @ np.array([1.0, 0.0, 0.0]))
    n = n_az * n_el
    return ScanSequence(np.zeros((n, 3), np.float32), np.asarray(dirs, np.float32),
                        np.asarray(lats, np.float32), np.zeros(n, np.float32), float(line_length))


def linear_scan(num_lines: int, width: float, line_length: float, timestamps=None) -> ScanSequence:
    """Linear array: origins spread along x, all lines along +z."""
    xs = np.linspace(-width / 2, width / 2, num_lines)
    origins = np.stack([xs, np.zeros_like(xs), np.zeros_like(xs)], 1).astype(np.float32)
    dirs = np.tile(np.array([0, 0, 1], np.float32), (num_lines, 1))
    lats = np.tile(np.array([1, 0, 0], np.float32), (num_lines, 1))
    ts = np.zeros(num_lines, np.float32) if timestamps is None else np.asarray(timestamps, np.float32)
    return ScanSequence(origins, dirs, lats, ts, float(line_length))


# ---------------------------------------------------------------------------
# beam profiles
# ---------------------------------------------------------------------------
@dataclass
class GaussianBeam:
    sigma_lateral: float
    sigma_elevational: float


@dataclass
class LutBeam:
    samples: np.ndarray   # float32 [rad][lat][ele]
    r_range: tuple
    l_range: tuple
    e_range: tuple


def synthetic_lut(seed: int, nr=256, nl=64, ne=64, r_range=(0.0, 0.13), l_range=(-0.01, 0.01),
                  e_range=(-0.01, 0.01), w0=1e-3, w1=4e-3, perturb=0.05) -> LutBeam:
    """A smooth Gaussian beam whose width grows linearly with depth, with a seeded
    smooth perturbation of at most `perturb` (the layout of utilities/make_lut.py:134-143:
    samples[rad, lat, ele])."""
    rng = np.random.default_rng(seed)
    r = np.linspace(*r_range, nr)
    l = np.linspace(*l_range, nl)
    e = np.linspace(*e_range, ne)
    w = w0 + (w1 - w0) * (r - r_range[0]) / (r_range[1] - r_range[0])
    # smooth perturbation: a few low-order cosines in each axis
    pr = sum(rng.uniform(-1, 1) * np.cos(k * np.pi * (r - r[0]) / (r[-1] - r[0]) + rng.uniform(0, 2 * np.pi)) for k in range(1, 4))
    pl = sum(rng.uniform(-1, 1) * np.cos(k * np.pi * (l - l[0]) / (l[-1] - l[0]) + rng.uniform(0, 2 * np.pi)) for k in range(1, 4))
    pe = sum(rng.uniform(-1, 1) * np.cos(k * np.pi * (e - e[0]) / (e[-1] - e[0]) + rng.uniform(0, 2 * np.pi)) for k in range(1, 4))
    pert = pr[:, None, None] + pl[None, :, None] + pe[None, None, :]
    pert = perturb * pert / max(1e-12, np.abs(pert).max())
    vals = np.exp(-(l[None, :, None] ** 2 + e[None, None, :] ** 2) / w[:, None, None] ** 2) * (1.0 + pert)
    return LutBeam(vals.astype(np.float32), tuple(map(float, r_range)), tuple(map(float, l_range)), tuple(map(float, e_range)))


# ---------------------------------------------------------------------------
# phantoms
# ---------------------------------------------------------------------------
@dataclass
class FixedSet:
    xyza: np.ndarray    # float32 [N,4]


@dataclass
class SplineSet:
    degree: int
    knots: np.ndarray           # float32 [K+p+1]
    control_points: np.ndarray  # float32 [N,K,3]
    amplitudes: np.ndarray      # float32 [N]


def uniform_regular_knots(n: int, p: int, t0: float, t1: float) -> np.ndarray:
    """uniform_regular_knot_vector<float> (src/core/bspline.hpp:95-112)."""
    if n < p + 1:
        raise ValueError("Too small n for a uniform regular knot vector")
    t0, t1 = np.float32(t0), np.float32(t1)
    mid = n + 1 - p
    middle = [np.float32(t0 + np.float32(i) * (t1 - t0) / np.float32(mid - 1)) for i in range(mid)]
    return np.array([t0] * p + middle + [t1] * p, np.float32)


def end_hack_knots(n: int, p: int) -> np.ndarray:
    """Clamped uniform knots on [0, 1] with the reference's "end-hack": the last
    knot moved to 2 so that the support is closed (src/examples/gpu_example2.cpp:130-142)."""
    k = uniform_regular_knots(n, p, 0.0, 1.0)
    k[-1] += np.float32(1.0)
    return k


def greville(p: int, knots: np.ndarray) -> np.ndarray:
    """control_points (src/core/bspline.hpp:116-126): knot averages."""
    k = knots.astype(np.float64)
    return np.array([k[i + 1:i + 1 + p].mean() for i in range(len(k) - p - 1)])


def spline_time_limits(degree: int, knots: np.ndarray, num_cs: int):
    """SplineScatterers::get_time_limits (src/core/BCSimConfig.hpp:145-154)."""
    return float(knots[degree]), float(knots[num_cs]) - 1e-5


def random_fixed(rng, n, xr, yr, zr) -> FixedSet:
    x = rng.uniform(*xr, n)
    y = np.zeros(n) if yr is None else rng.uniform(*yr, n)
    z = rng.uniform(*zr, n)
    a = rng.standard_normal(n)
    return FixedSet(np.stack([x, y, z, a], 1).astype(np.float32))


def random_spline(rng, n, num_cs, degree=3, box=((-0.02, 0.02), (-0.02, 0.02), (0.01, 0.11)),
                  amp=(0.0, 3e-3), freq=(1.0, 2.0)) -> SplineSet:
    knots = end_hack_knots(num_cs, degree)
    tk = greville(degree, knots)                                       # [K]
    base = np.stack([rng.uniform(*box[a], n) for a in range(3)], 1)    # [N,3]
    A = rng.uniform(*amp, (n, 3))
    f = rng.uniform(*freq, (n, 3))
    ph = rng.uniform(0, 2 * np.pi, (n, 3))
    cps = base[:, None, :] + A[:, None, :] * np.sin(2 * np.pi * f[:, None, :] * tk[None, :, None] + ph[:, None, :])
    amps = rng.standard_normal(n)
    return SplineSet(degree, knots, cps.astype(np.float32), amps.astype(np.float32))


# ---------------------------------------------------------------------------
# complete simulation jobs
# ---------------------------------------------------------------------------
@dataclass
class Job:
    name: str
    scan: ScanSequence
    taps: np.ndarray
    center_index: int
    fs: float
    demod_freq: float
    beam: object
    fixed: List[FixedSet] = field(default_factory=list)
    splines: List[SplineSet] = field(default_factory=list)
    decimation: int = 1
    sound_speed: float = SOUND_SPEED
    phase_delay: bool = True
    arc: bool = True
    noise_amplitude: float = 0.0   # sigma of the seeded complex noise on the time projection (0: off)
    noise_seed: int = 0
    noise_frame: int = 0           # the frame number the noise is drawn for

    @property
    def num_scatterers(self) -> int:
        return sum(f.xyza.shape[0] for f in self.fixed) + sum(s.amplitudes.shape[0] for s in self.splines)

    @property
    def projections(self) -> int:
        return self.num_scatterers * self.scan.num_lines

    @property
    def num_samples(self) -> int:
        return num_rf_samples(self.sound_speed, self.scan.line_length, self.fs)

    @property
    def num_out(self) -> int:
        return -(-self.num_samples // self.decimation)


def _excitation_job(name, scan, fc, bw, beam, fixed=(), splines=(), decimation=1, phase_delay=True):
    taps, ci = gaussian_excitation(fc, bw, FS)
    return Job(name, scan, taps, ci, FS, float(np.float32(fc)), beam, list(fixed), list(splines),
               decimation, SOUND_SPEED, phase_delay)


def sector_2d_fixed(num_scatterers=100_000, num_lines=128, phase_delay=True, seed=1000) -> Job:
    rng = np.random.default_rng(seed)
    fixed = random_fixed(rng, num_scatterers, (-0.03, 0.03), None, (0.01, 0.12))
    scan = sector_scan(num_lines, 35.0, 0.12)
    return _excitation_job("sector_2d_fixed", scan, 2.5e6, 0.1, GaussianBeam(1e-3, 1e-3), [fixed], [], 10, phase_delay)


def volume_3d_lut(num_scatterers=2_000_000, n_az=64, n_el=64, phase_delay=True, seed=2000,
                  lut_shape=(256, 64, 64)) -> Job:
    rng = np.random.default_rng(seed)
    fixed = random_fixed(rng, num_scatterers, (-0.03, 0.03), (-0.03, 0.03), (0.01, 0.12))
    scan = volume_scan(n_az, n_el, 30.0, 30.0, 0.13)
    lut = synthetic_lut(seed + 1, *lut_shape)
    return _excitation_job("volume_3d_lut", scan, 3.5e6, 0.15, lut, [fixed], [], 8, phase_delay)


def sector_spline(num_scatterers=500_000, num_lines=1024, num_cs=16, phase_delay=True, seed=3000) -> Job:
    rng = np.random.default_rng(seed)
    sp = random_spline(rng, num_scatterers, num_cs)
    t0, t1 = spline_time_limits(sp.degree, sp.knots, num_cs)
    ts = np.linspace(t0, t1, num_lines).astype(np.float32)
    scan = sector_scan(num_lines, 35.0, 0.12, timestamps=ts)
    return _excitation_job("sector_spline", scan, 2.5e6, 0.1, GaussianBeam(1e-3, 1e-3), [], [sp], 10, phase_delay)


def batch_uneven(num_jobs=64, seed=4000, scale=1.0) -> List[Job]:
    """64 independent jobs: N log-uniform in [1e4, 2e6], L uniform in 32..1024,
    depth uniform in [5, 15] cm, fc in [2, 7] MHz, bw in [0.1, 0.3], decimation
    4..16, fixed or spline (p = 3, K in 8..24) with probability 1/2.  `scale`
    shrinks N and L for quick tests."""
    jobs = []
    for j in range(num_jobs):
        rng = np.random.default_rng(seed + j)
        n = int(round(10 ** rng.uniform(4, math.log10(2e6)) * scale))
        n = max(n, 16)
        L = max(2, int(round(rng.integers(32, 1025) * scale)))
        depth = rng.uniform(0.05, 0.15)
        fc = rng.uniform(2e6, 7e6)
        bw = rng.uniform(0.1, 0.3)
        dec = int(rng.integers(4, 17))
        if rng.uniform() < 0.5:
            fixed = [random_fixed(rng, n, (-0.03, 0.03), None, (0.01, depth))]
            scan = sector_scan(L, 35.0, depth)
            jobs.append(_excitation_job(f"job{j}_fixed", scan, fc, bw, GaussianBeam(1e-3, 1e-3), fixed, [], dec))
        else:
            K = int(rng.integers(8, 25))
            sp = random_spline(rng, n, K, box=((-0.02, 0.02), (-0.02, 0.02), (0.01, max(0.02, depth - 0.01))))
            t0, t1 = spline_time_limits(sp.degree, sp.knots, K)
            ts = np.sort(rng.uniform(t0, t1, L)).astype(np.float32)
            scan = sector_scan(L, 35.0, depth, timestamps=ts)
            jobs.append(_excitation_job(f"job{j}_spline", scan, fc, bw, GaussianBeam(1e-3, 1e-3), [], [sp], dec))
    return jobs


# ---------------------------------------------------------------------------
# served request stream
# ---------------------------------------------------------------------------
def served_phantoms(seed=5000, scale=1.0) -> List[Job]:
    """Eight resident phantoms: fixed 100k, 500k, 1M, 2M scatterers and spline
    50k, 100k, 250k, 500k scatterers with 8, 12, 16, 24 control points; Gaussian
    beam 1 mm, 2.5 MHz / bw 0.1 / 50 MHz, 12 cm lines.  The scan lines of a job
    are placeholders: every request brings its own."""
    out = []
    for i, n in enumerate([100_000, 500_000, 1_000_000, 2_000_000]):
        rng = np.random.default_rng(seed + i)
        fixed = random_fixed(rng, max(16, int(n * scale)), (-0.03, 0.03), None, (0.01, 0.12))
        out.append(_excitation_job(f"fixed{n}", sector_scan(2, 35.0, 0.12), 2.5e6, 0.1,
                                   GaussianBeam(1e-3, 1e-3), [fixed], [], 8))
    for i, (n, K) in enumerate([(50_000, 8), (100_000, 12), (250_000, 16), (500_000, 24)]):
        rng = np.random.default_rng(seed + 10 + i)
        sp = random_spline(rng, max(16, int(n * scale)), K)
        out.append(_excitation_job(f"spline{n}", sector_scan(2, 35.0, 0.12, timestamps=[0.0, 0.5]), 2.5e6, 0.1,
                                   GaussianBeam(1e-3, 1e-3), [], [sp], 8))
    return out


@dataclass
class Request:
    arrival: float          # seconds from the start of the stream
    phantom: int
    scan: ScanSequence
    decimation: int


def request_stream(phantoms: List[Job], rate_hz=200.0, seconds=60.0, seed=5100, max_lines=256) -> List[Request]:
    """Poisson arrivals at rate_hz; each request: 1..max_lines lines at random
    angles in +-35 degrees and random timestamps in the phantom's time range,
    decimation 4..16."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate_hz)
        if t >= seconds:
            break
        k = int(rng.integers(0, len(phantoms)))
        L = int(rng.integers(1, max_lines + 1))
        job = phantoms[k]
        if job.splines:
            sp = job.splines[0]
            t0, t1 = spline_time_limits(sp.degree, sp.knots, sp.control_points.shape[1])
            ts = rng.uniform(t0, t1, L)
        else:
            ts = rng.uniform(0.0, 1.0, L)
        scan = sector_scan(L, 35.0, 0.12, timestamps=ts.astype(np.float32), angles_deg=rng.uniform(-35.0, 35.0, L))
        out.append(Request(t, k, scan, int(rng.integers(4, 17))))
    return out
