"""Phantom, scan-sequence, excitation and beam-profile files.

The reference stores these as HDF5 datasets (src/utils/HDFConvenience.cpp:44-196);
this module reads and writes the same datasets, under the same names and with
the same validation, as NumPy ``.npz`` archives (HDF5 is not available to this
package).  A file written by h5py from one of the reference's HDF5 files with
``np.savez(path, **{k: f[k][()] for k in f})`` loads unchanged.

    fixed scatterers   data [N, 4] (x, y, z, amplitude)            loadFixedScatterersFromHdf   :44-67
    spline scatterers  control_points [N, K, 3], amplitudes [N],   loadSplineScatterersFromHdf  :69-106
                       spline_degree, knot_vector [K + p + 1]
    scan sequence      origins, directions, lateral_dirs [L, 3],   loadScanSequenceFromHdf      :108-135
                       timestamps [L], lengths (line length)
    excitation         samples, center_index, sampling_frequency,  loadExcitationFromHdf        :137-145
                       demod_freq
    beam profile       beam_profile [nr, nl, ne] (normalised to a  loadBeamProfileFromHdf       :147-196
                       maximum of 1), rad_extent, lat_extent,
                       ele_extent (each [min, max])
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


class FormatError(RuntimeError):
    pass


def _load(path):
    try:
        return np.load(path, allow_pickle=False)
    except (OSError, ValueError) as e:
        raise FormatError(f"cannot read {path}: {e}") from e


def _get(z, key):
    if key not in z:
        raise FormatError(f"missing dataset '{key}'")
    return z[key]


# --- fixed scatterers ------------------------------------------------------
def load_fixed_scatterers(path) -> np.ndarray:
    """[N, 4] float32 (x, y, z, amplitude)."""
    z = _load(path)
    data = np.asarray(_get(z, "data"), np.float32)
    if data.ndim != 2:
        raise FormatError("failed to load fixed scatterers")
    if data.shape[1] != 4:
        raise FormatError("Second dimension must have length four")
    return np.ascontiguousarray(data)


def save_fixed_scatterers(path, data) -> None:
    data = np.asarray(data, np.float32)
    if data.ndim != 2 or data.shape[1] != 4:
        raise FormatError("Second dimension must have length four")
    np.savez(path, data=data)


# --- spline scatterers -----------------------------------------------------
@dataclass
class SplineScatterers:
    spline_degree: int
    knot_vector: np.ndarray      # [K + p + 1] float32
    control_points: np.ndarray   # [N, K, 3] float32
    amplitudes: np.ndarray       # [N] float32


def load_spline_scatterers(path) -> SplineScatterers:
    z = _load(path)
    cps = np.asarray(_get(z, "control_points"), np.float32)
    amps = np.asarray(_get(z, "amplitudes"), np.float32).reshape(-1)
    degree = int(np.asarray(_get(z, "spline_degree")).reshape(()))
    knots = np.asarray(_get(z, "knot_vector"), np.float32).reshape(-1)
    if cps.ndim != 3:
        raise FormatError("failed to load spline scatterers")
    if cps.shape[2] != 3:
        raise FormatError("SplineScatterer illegal number of components (should be 3)")
    if amps.shape[0] < cps.shape[0]:
        raise FormatError("failed to load spline scatterers")
    return SplineScatterers(degree, knots, np.ascontiguousarray(cps), np.ascontiguousarray(amps[: cps.shape[0]]))


def save_spline_scatterers(path, s: SplineScatterers) -> None:
    cps = np.asarray(s.control_points, np.float32)
    if cps.ndim != 3 or cps.shape[2] != 3:
        raise FormatError("SplineScatterer illegal number of components (should be 3)")
    np.savez(path, control_points=cps, amplitudes=np.asarray(s.amplitudes, np.float32),
             spline_degree=np.int32(s.spline_degree), knot_vector=np.asarray(s.knot_vector, np.float32))


# --- scan sequence ---------------------------------------------------------
@dataclass
class ScanSequence:
    origins: np.ndarray        # [L, 3]
    directions: np.ndarray     # [L, 3]
    lateral_dirs: np.ndarray   # [L, 3]
    timestamps: np.ndarray     # [L]
    line_length: float


def load_scan_sequence(path) -> ScanSequence:
    z = _load(path)
    d = np.asarray(_get(z, "directions"), np.float32)
    o = np.asarray(_get(z, "origins"), np.float32)
    length = float(np.asarray(_get(z, "lengths"), np.float32).reshape(-1)[0])
    lat = np.asarray(_get(z, "lateral_dirs"), np.float32)
    t = np.asarray(_get(z, "timestamps"), np.float32).reshape(-1)
    if d.ndim != 2 or o.ndim != 2 or lat.ndim != 2 or d.shape[1] != 3 or o.shape[1] != 3 or lat.shape[1] != 3:
        raise FormatError("ScanSequence::size error")
    if d.shape[0] != o.shape[0] or d.shape[0] != t.shape[0] or lat.shape[0] < d.shape[0]:
        raise FormatError("ScanSequence::size error")
    L = d.shape[0]
    return ScanSequence(np.ascontiguousarray(o), np.ascontiguousarray(d), np.ascontiguousarray(lat[:L]),
                        np.ascontiguousarray(t), length)


def save_scan_sequence(path, s: ScanSequence) -> None:
    np.savez(path, origins=np.asarray(s.origins, np.float32), directions=np.asarray(s.directions, np.float32),
             lateral_dirs=np.asarray(s.lateral_dirs, np.float32), timestamps=np.asarray(s.timestamps, np.float32),
             lengths=np.float32(s.line_length))


# --- excitation ------------------------------------------------------------
@dataclass
class Excitation:
    samples: np.ndarray
    center_index: int
    sampling_frequency: float
    demod_freq: float


def load_excitation(path) -> Excitation:
    """The reference's loader stops at the missing demodulation frequency
    (HDFConvenience.cpp:143); files that carry ``demod_freq`` load."""
    z = _load(path)
    ci = int(np.asarray(_get(z, "center_index")).reshape(()))
    fs = float(np.asarray(_get(z, "sampling_frequency"), np.float32).reshape(()))
    samples = np.asarray(_get(z, "samples"), np.float32).reshape(-1)
    if "demod_freq" not in z:
        raise FormatError("TODO: Must read and set demodulation frequency")
    fd = float(np.asarray(z["demod_freq"], np.float32).reshape(()))
    return Excitation(samples, ci, fs, fd)


def save_excitation(path, e: Excitation) -> None:
    np.savez(path, samples=np.asarray(e.samples, np.float32), center_index=np.int32(e.center_index),
             sampling_frequency=np.float32(e.sampling_frequency), demod_freq=np.float32(e.demod_freq))


# --- beam profile ----------------------------------------------------------
@dataclass
class BeamProfile:
    samples: np.ndarray   # [nr, nl, ne] float32, maximum 1
    rad_extent: tuple
    lat_extent: tuple
    ele_extent: tuple


def load_beam_profile(path) -> BeamProfile:
    z = _load(path)
    lut = np.asarray(_get(z, "beam_profile"), np.float32)
    ext = {}
    for key in ("rad_extent", "lat_extent", "ele_extent"):
        v = np.asarray(_get(z, key), np.float32).reshape(-1)
        if v.shape[0] != 2:
            raise FormatError(f"{key} must contain two elements: [min, max]")
        ext[key] = (float(v[0]), float(v[1]))
    if lut.ndim != 3:
        raise FormatError("beam_profile data must be a 3D array")
    # normalise so that the maximum is one, in float as the reference divides
    mx = np.float32(lut.max())
    return BeamProfile((lut / mx).astype(np.float32), ext["rad_extent"], ext["lat_extent"], ext["ele_extent"])


def save_beam_profile(path, b: BeamProfile) -> None:
    np.savez(path, beam_profile=np.asarray(b.samples, np.float32), rad_extent=np.float32(b.rad_extent),
             lat_extent=np.float32(b.lat_extent), ele_extent=np.float32(b.ele_extent))


# --- configuring a simulator from files -------------------------------------
def add_fixed_scatterers_from_file(sim, path) -> None:
    sim.add_fixed_scatterers(load_fixed_scatterers(path))


def add_spline_scatterers_from_file(sim, path) -> None:
    s = load_spline_scatterers(path)
    sim.add_spline_scatterers(s.spline_degree, s.knot_vector, s.control_points, s.amplitudes)


def set_scan_sequence_from_file(sim, path) -> None:
    s = load_scan_sequence(path)
    sim.set_scan_sequence(s.origins, s.directions, s.line_length, s.lateral_dirs, s.timestamps)


def set_excitation_from_file(sim, path) -> None:
    e = load_excitation(path)
    sim.set_excitation(e.samples, e.center_index, e.sampling_frequency, e.demod_freq)


def set_beam_profile_from_file(sim, path) -> None:
    b = load_beam_profile(path)
    sim.set_lut_beam_profile(b.rad_extent[0], b.rad_extent[1], b.lat_extent[0], b.lat_extent[1], b.ele_extent[0],
                             b.ele_extent[1], b.samples)
