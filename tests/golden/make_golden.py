"""Regenerates the golden fixtures of this directory.

* reference_kats.json -- the known-answer vectors of the reference's own unit
  tests, restated with their source lines:
    src/core/unittest/test_fft.cpp:55-90          (fft_conv, next_power_of_two)
    src/core/unittest/test_hilbert_mask.cpp:14-34 (discrete_hilbert_mask)
    src/utils/unittest/test_SignalProcessing.cpp:6-27 (direct_conv)
* ref_imaging.npz -- seeded float and byte beam spaces, three scan geometries
  (sector, tilted sector, linear) and what the reference's own scan converter
  (CpuCartesianator, src/utils/cartesianator/Cartesianator.cpp:107-205)
  returns for them.
* ref_excitation.npz -- the taps and centre index that the reference's own
  MakeGaussianExcitation<float> (src/utils/GaussPulse.cpp:52-70) returns for
  the pulses of the benchmark workloads and a spread of others
  (`python tests/golden/make_golden.py excitation`).
* ref_full_<workload>.npz -- the reference's own IQ for 32 lines spread over
  each full-size benchmark workload (2-D sector, 3-D LUT volume, spline
  sector; their inputs are regenerated from the workloads' seeds), with the
  line indices (`python tests/golden/make_golden.py full`).
* ref_<case>.npz -- inputs of a small seeded case, the IQ that the reference's
  own CPU algorithm returns for them (bcsim::Create("cpu")->simulate_lines), and
  the time-projection bins of a few lines from its projection loops
  (CpuAlgorithm::projection_loop).  Produced by oracle/_ref/libbcsim_ref.so,
  which oracle/Makefile compiles from the reference sources; run this script
  where those sources exist:

    make -C oracle all && python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from openbcsim_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402

KATS = {
    "fft_conv": [
        {"source": "src/core/unittest/test_fft.cpp:55-63", "x": [1.0, 2.0, 3.0], "h": [1.0],
         "expected": [1.0, 2.0, 3.0], "rel_tol_percent": 0.01},
        {"source": "src/core/unittest/test_fft.cpp:65-75",
         "x": [1.0, 2.0, 3.0, -0.23, 0.001, 32.3, 4.0], "h": [-0.33, 0.9, -0.002, 1.1, 2.3],
         "expected": [-0.33, 0.24, 0.808, 3.8719, 4.28667, -2.75764, 34.396998, 3.0075, 35.5243, 78.69, 9.2],
         "rel_tol_percent": 0.01},
    ],
    "next_power_of_two": {"source": "src/core/unittest/test_fft.cpp:77-90",
                          "table": [[1, 1], [2, 2], [3, 4], [4, 4], [5, 8], [7, 8], [8, 8], [15, 16], [16, 16],
                                    [32767, 32768], [65535, 65536], [65536, 65536]]},
    "hilbert_mask": {"source": "src/core/unittest/test_hilbert_mask.cpp:14-34",
                     "masks": {"7": [1, 2, 2, 2, 0, 0, 0], "8": [1, 2, 2, 2, 1, 0, 0, 0],
                               "11": [1, 2, 2, 2, 2, 2, 0, 0, 0, 0, 0],
                               "18": [1, 2, 2, 2, 2, 2, 2, 2, 2, 1, 0, 0, 0, 0, 0, 0, 0, 0]}},
    "direct_conv": [
        {"source": "src/utils/unittest/test_SignalProcessing.cpp:6-14", "x": [1, 2, 3], "h": [1], "expected": [1, 2, 3]},
        {"source": "src/utils/unittest/test_SignalProcessing.cpp:16-27", "x": [1, -1, 0, 10, 3], "h": [3, 9, -2],
         "expected": [3, 6, -11, 32, 99, 7, -6]},
    ],
}


def edge_case_job() -> W.Job:
    """Scatterers on the awkward spots: at and next to the origin, behind the
    probe, perpendicular to a line, beyond the line end, exactly on bin
    boundaries, zero amplitude."""
    job = W.sector_2d_fixed(num_scatterers=2000, num_lines=8, phase_delay=True, seed=7001)
    rng = np.random.default_rng(7002)
    k = 2.0 * job.fs / job.sound_speed            # bins per metre
    extra = [
        [0.0, 0.0, 0.0, 1.0],                      # at the origin
        [0.0, 0.0, 0.3 / k, 1.0],                  # within half a sample
        [0.0, 0.0, 0.5 / k, -1.0],                 # on the first rounding boundary
        [0.0, 0.0, -2e-3, 2.0],                    # behind the probe
        [2e-4, 0.0, 0.0, 1.5],                     # perpendicular to the centre line
        [0.0, 0.0, 0.119999, 1.0],                 # at the line end
        [0.0, 0.0, 0.2, 1.0],                      # beyond the line end
        [0.01, 0.0, 0.05, 0.0],                    # zero amplitude
    ]
    for i in range(64):                            # exactly on .5 boundaries of r*2fs/c along the centre line
        extra.append([0.0, 0.0, (100 + 37 * i + 0.5) / k, float(rng.standard_normal())])
    job.fixed[0].xyza = np.concatenate([job.fixed[0].xyza, np.asarray(extra, np.float32)], 0)
    job.name = "edge"
    return job


def linear_job() -> W.Job:
    job = W.sector_2d_fixed(num_scatterers=3000, num_lines=12, phase_delay=True, seed=7101)
    job.scan = W.linear_scan(12, 0.03, 0.12)
    job.name = "linear"
    return job


def cases():
    yield "sector_pd", W.sector_2d_fixed(num_scatterers=4000, num_lines=16, phase_delay=True, seed=7201)
    yield "sector_nopd", W.sector_2d_fixed(num_scatterers=4000, num_lines=16, phase_delay=False, seed=7202)
    yield "lut3d", W.volume_3d_lut(num_scatterers=20000, n_az=4, n_el=4, seed=7301, lut_shape=(32, 16, 16))
    yield "spline", W.sector_spline(num_scatterers=1000, num_lines=8, seed=7401)
    yield "linear", linear_job()
    yield "edge", edge_case_job()


def job_to_arrays(job: W.Job) -> dict:
    d = {
        "taps": job.taps, "center_index": job.center_index, "fs": job.fs, "demod_freq": job.demod_freq,
        "sound_speed": job.sound_speed, "phase_delay": int(job.phase_delay), "arc": int(job.arc),
        "decimation": job.decimation, "origins": job.scan.origins, "directions": job.scan.directions,
        "lateral_dirs": job.scan.lateral_dirs, "timestamps": job.scan.timestamps, "line_length": job.scan.line_length,
    }
    b = job.beam
    if hasattr(b, "sigma_lateral"):
        d["beam"] = "gaussian"
        d["sigma"] = np.array([b.sigma_lateral, b.sigma_elevational])
    else:
        d["beam"] = "lut"
        d["lut"] = b.samples
        d["lut_extent"] = np.array(list(b.r_range) + list(b.l_range) + list(b.e_range))
    for i, f in enumerate(job.fixed):
        d[f"fixed{i}"] = f.xyza
    for i, s in enumerate(job.splines):
        d[f"spline{i}_degree"] = s.degree
        d[f"spline{i}_knots"] = s.knots
        d[f"spline{i}_cps"] = s.control_points
        d[f"spline{i}_amps"] = s.amplitudes
    return d


def arrays_to_job(z) -> W.Job:
    scan = W.ScanSequence(z["origins"], z["directions"], z["lateral_dirs"], z["timestamps"], float(z["line_length"]))
    if str(z["beam"]) == "gaussian":
        beam = W.GaussianBeam(float(z["sigma"][0]), float(z["sigma"][1]))
    else:
        e = z["lut_extent"]
        beam = W.LutBeam(z["lut"], (float(e[0]), float(e[1])), (float(e[2]), float(e[3])), (float(e[4]), float(e[5])))
    fixed, splines = [], []
    i = 0
    while f"fixed{i}" in z:
        fixed.append(W.FixedSet(z[f"fixed{i}"]))
        i += 1
    i = 0
    while f"spline{i}_knots" in z:
        splines.append(W.SplineSet(int(z[f"spline{i}_degree"]), z[f"spline{i}_knots"], z[f"spline{i}_cps"],
                                   z[f"spline{i}_amps"]))
        i += 1
    return W.Job("golden", scan, z["taps"], int(z["center_index"]), float(z["fs"]), float(z["demod_freq"]), beam,
                 fixed, splines, int(z["decimation"]), float(z["sound_speed"]), bool(int(z["phase_delay"])),
                 bool(int(z["arc"])))


BIN_LINES = (0, 3)


IMAGING_GEOMETRIES = [
    (0, float(np.float32(np.deg2rad(70.0))), 0.12, 0.0, 161, 139),   # sector, 70 degrees, 12 cm
    (0, 1.0, 0.1, 0.2, 120, 101),                                     # tilted sector
    (1, 0.04, 0.06, 0.0, 97, 140),                                    # linear, 4 cm x 6 cm
]


def make_imaging():
    from oracle import imaging as OI

    rng = np.random.default_rng(4242)
    bf = rng.random((48, 200), dtype=np.float32)
    bu = (rng.random((48, 200)) * 256).astype(np.uint8)
    d = {"beamspace_f32": bf, "beamspace_u8": bu, "geometries": np.array(IMAGING_GEOMETRIES, np.float64)}
    for k, g in enumerate(IMAGING_GEOMETRIES):
        g = (int(g[0]), g[1], g[2], g[3], int(g[4]), int(g[5]))
        d[f"ref_f32_{k}"] = OI.ref_scan_convert(bf, g)
        d[f"ref_u8_{k}"] = OI.ref_scan_convert(bu, g)
    np.savez_compressed(os.path.join(HERE, "ref_imaging.npz"), **d)
    print("imaging", os.path.getsize(os.path.join(HERE, "ref_imaging.npz")))


# (centre frequency, fractional bandwidth, sampling frequency): the workloads'
# pulses (2.5 MHz / 0.1, 3.5 MHz / 0.15 at 50 MHz), the batch range's corners
# (2-7 MHz, 0.1-0.3) and other sampling rates
EXCITATIONS = [(2.5e6, 0.1, 50e6), (3.5e6, 0.15, 50e6), (2e6, 0.1, 50e6), (7e6, 0.3, 50e6), (2e6, 0.3, 50e6),
               (7e6, 0.1, 50e6), (4.37e6, 0.213, 50e6), (5e6, 0.5, 100e6), (1e6, 0.05, 20e6), (10e6, 0.6, 80e6)]


def make_excitation():
    lib = O.ref_lib()
    d = {"params": np.array(EXCITATIONS, np.float64)}
    for k, (fc, bw, fs) in enumerate(EXCITATIONS):
        buf = np.zeros(1 << 16, np.float32)
        ci = O.C.c_int()
        n = lib.ref_gaussian_excitation(fc, bw, fs, O.fptr(buf), buf.size, O.C.byref(ci))
        d[f"taps_{k}"] = buf[:n].copy()
        d[f"center_{k}"] = np.array(ci.value)
    np.savez_compressed(os.path.join(HERE, "ref_excitation.npz"), **d)
    print("excitation", os.path.getsize(os.path.join(HERE, "ref_excitation.npz")))


FULL_WORKLOADS = ["sector_2d_fixed", "volume_3d_lut", "sector_spline"]


def full_lines(L: int) -> np.ndarray:
    return np.unique(np.linspace(0, L - 1, 32).round().astype(int))


def make_full():
    import copy

    for name in FULL_WORKLOADS:
        job = getattr(W, name)()
        idx = full_lines(job.scan.num_lines)
        sub = copy.copy(job)
        s = job.scan
        sub.scan = W.ScanSequence(s.origins[idx], s.directions[idx], s.lateral_dirs[idx], s.timestamps[idx],
                                  s.line_length)
        iq = O.ref_simulate(sub, threads=0)
        np.savez_compressed(os.path.join(HERE, f"ref_full_{name}.npz"), lines=idx, ref_iq=iq)
        print(name, iq.shape, os.path.getsize(os.path.join(HERE, f"ref_full_{name}.npz")))


def main():
    if not O.ref_available():
        raise SystemExit("oracle/_ref/libbcsim_ref.so is missing: run `make -C oracle all` where the reference sources are")
    with open(os.path.join(HERE, "reference_kats.json"), "w") as f:
        json.dump(KATS, f, indent=1)
    for name, job in cases():
        iq = O.ref_simulate(job, threads=1)
        bins = np.stack([O.ref_project_bins(job, ln) for ln in BIN_LINES])
        d = job_to_arrays(job)
        d["ref_iq"] = iq
        d["ref_bins"] = bins
        d["ref_bins_lines"] = np.array(BIN_LINES)
        np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **d)
        print(name, iq.shape, os.path.getsize(os.path.join(HERE, f"ref_{name}.npz")))


if __name__ == "__main__":
    if sys.argv[1:] == ["imaging"]:
        make_imaging()
    elif sys.argv[1:] == ["excitation"]:
        make_excitation()
    elif sys.argv[1:] == ["full"]:
        make_full()
    else:
        main()
        make_imaging()
        make_excitation()
        make_full()
