"""Phantom / scan / excitation / beam-profile files (openbcsim_gb300.formats):
the reference's HDF5 dataset names and checks (src/utils/HDFConvenience.cpp:44-196)
over .npz archives.  CPU tests: round trips, validation messages,
normalisation.  GPU test: a simulator configured from files equals one
configured from the same arrays."""
import numpy as np
import pytest

from conftest import load_golden


def test_round_trips(tmp_path):
    from openbcsim_gb300 import formats as F
    from openbcsim_gb300 import workloads as W

    job, _ = load_golden("spline")
    xyza = np.random.default_rng(1).standard_normal((50, 4)).astype(np.float32)
    F.save_fixed_scatterers(tmp_path / "fixed.npz", xyza)
    assert np.array_equal(F.load_fixed_scatterers(tmp_path / "fixed.npz"), xyza)

    sp = job.splines[0]
    F.save_spline_scatterers(tmp_path / "spline.npz",
                             F.SplineScatterers(sp.degree, sp.knots, sp.control_points, sp.amplitudes))
    s2 = F.load_spline_scatterers(tmp_path / "spline.npz")
    assert s2.spline_degree == sp.degree and np.array_equal(s2.knot_vector, sp.knots)
    assert np.array_equal(s2.control_points, sp.control_points) and np.array_equal(s2.amplitudes, sp.amplitudes)

    s = job.scan
    F.save_scan_sequence(tmp_path / "scan.npz",
                         F.ScanSequence(s.origins, s.directions, s.lateral_dirs, s.timestamps, s.line_length))
    s3 = F.load_scan_sequence(tmp_path / "scan.npz")
    assert np.array_equal(s3.origins, s.origins) and np.array_equal(s3.timestamps, s.timestamps)
    assert s3.line_length == pytest.approx(s.line_length)

    F.save_excitation(tmp_path / "ex.npz", F.Excitation(job.taps, job.center_index, job.fs, job.demod_freq))
    e = F.load_excitation(tmp_path / "ex.npz")
    assert np.array_equal(e.samples, job.taps) and e.center_index == job.center_index

    lut = W.volume_3d_lut(num_scatterers=10, n_az=2, n_el=2, lut_shape=(8, 6, 5)).beam
    F.save_beam_profile(tmp_path / "beam.npz", F.BeamProfile(3.0 * lut.samples, lut.r_range, lut.l_range, lut.e_range))
    b = F.load_beam_profile(tmp_path / "beam.npz")
    # normalised to a maximum of one (HDFConvenience.cpp:181-192)
    assert b.samples.max() == 1.0
    assert np.array_equal(b.samples, (np.float32(3.0) * lut.samples) / np.float32((3.0 * lut.samples).max()))


def test_validation_messages(tmp_path):
    from openbcsim_gb300 import formats as F

    np.savez(tmp_path / "f.npz", data=np.zeros((4, 3), np.float32))
    with pytest.raises(F.FormatError, match="Second dimension must have length four"):
        F.load_fixed_scatterers(tmp_path / "f.npz")
    np.savez(tmp_path / "s.npz", control_points=np.zeros((2, 5, 2), np.float32), amplitudes=np.zeros(2, np.float32),
             spline_degree=np.int32(3), knot_vector=np.zeros(9, np.float32))
    with pytest.raises(F.FormatError, match="illegal number of components"):
        F.load_spline_scatterers(tmp_path / "s.npz")
    np.savez(tmp_path / "q.npz", directions=np.zeros((3, 3), np.float32), origins=np.zeros((2, 3), np.float32),
             lateral_dirs=np.zeros((3, 3), np.float32), timestamps=np.zeros(3, np.float32), lengths=np.float32(0.1))
    with pytest.raises(F.FormatError, match="ScanSequence::size error"):
        F.load_scan_sequence(tmp_path / "q.npz")
    np.savez(tmp_path / "e.npz", samples=np.ones(4, np.float32), center_index=np.int32(2),
             sampling_frequency=np.float32(50e6))
    with pytest.raises(F.FormatError, match="demodulation frequency"):
        F.load_excitation(tmp_path / "e.npz")
    np.savez(tmp_path / "b.npz", beam_profile=np.ones((2, 2, 2), np.float32), rad_extent=np.float32([0, 1, 2]),
             lat_extent=np.float32([0, 1]), ele_extent=np.float32([0, 1]))
    with pytest.raises(F.FormatError, match="rad_extent must contain two elements"):
        F.load_beam_profile(tmp_path / "b.npz")
    np.savez(tmp_path / "b2.npz", beam_profile=np.ones((2, 2), np.float32), rad_extent=np.float32([0, 1]),
             lat_extent=np.float32([0, 1]), ele_extent=np.float32([0, 1]))
    with pytest.raises(F.FormatError, match="must be a 3D array"):
        F.load_beam_profile(tmp_path / "b2.npz")
    with pytest.raises(F.FormatError, match="missing dataset 'data'"):
        np.savez(tmp_path / "x.npz", other=np.zeros(1))
        F.load_fixed_scatterers(tmp_path / "x.npz")


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["lut3d", "spline"])
def test_simulator_from_files(tmp_path, name):
    import openbcsim_gb300 as gb
    from openbcsim_gb300 import formats as F

    job, _ = load_golden(name)
    b = job.beam
    if hasattr(b, "samples"):   # files hold the normalised table: configure the reference run the same way
        b.samples = (b.samples / np.float32(b.samples.max())).astype(np.float32)
        F.save_beam_profile(tmp_path / "beam.npz", F.BeamProfile(b.samples, b.r_range, b.l_range, b.e_range))
    s = job.scan
    F.save_scan_sequence(tmp_path / "scan.npz",
                         F.ScanSequence(s.origins, s.directions, s.lateral_dirs, s.timestamps, s.line_length))
    F.save_excitation(tmp_path / "ex.npz", F.Excitation(job.taps, job.center_index, job.fs, job.demod_freq))
    for k, f in enumerate(job.fixed):
        F.save_fixed_scatterers(tmp_path / f"fixed{k}.npz", f.xyza)
    for k, sp in enumerate(job.splines):
        F.save_spline_scatterers(tmp_path / f"spline{k}.npz",
                                 F.SplineScatterers(sp.degree, sp.knots, sp.control_points, sp.amplitudes))

    ref = gb.configure_job(gb.RfSimulator("gpu"), job).simulate_lines_line_major()
    sim = gb.RfSimulator("gpu")
    sim.set_parameter("sound_speed", repr(float(np.float32(job.sound_speed))))
    sim.set_parameter("use_arc_projection", "on" if job.arc else "off")
    sim.set_parameter("phase_delay", "on" if job.phase_delay else "off")
    sim.set_parameter("radial_decimation", str(job.decimation))
    F.set_excitation_from_file(sim, tmp_path / "ex.npz")
    F.set_scan_sequence_from_file(sim, tmp_path / "scan.npz")
    if hasattr(b, "samples"):
        F.set_beam_profile_from_file(sim, tmp_path / "beam.npz")
    else:
        sim.set_analytical_beam_profile(b.sigma_lateral, b.sigma_elevational)
    for k in range(len(job.fixed)):
        F.add_fixed_scatterers_from_file(sim, tmp_path / f"fixed{k}.npz")
    for k in range(len(job.splines)):
        F.add_spline_scatterers_from_file(sim, tmp_path / f"spline{k}.npz")
    assert np.array_equal(sim.simulate_lines_line_major(), ref)
