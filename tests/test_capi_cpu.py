"""The C ABI without a GPU: the library loads, exports every function that
include/bcsim_gb300.h declares, and the host-side logic (factory, parameters,
scan-sequence validation, configuration order, error messages) behaves as the
reference's IAlgorithm does.  No call here launches device work."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "bcsim_gb300.h")


@pytest.fixture(scope="module")
def lib():
    from openbcsim_gb300 import build, _capi

    build.build()
    return _capi.load()


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(bcsim_\w+)\s*\(", text, re.M)))


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    # and the Python binding covers them all
    from openbcsim_gb300 import _capi

    bound = {s[0] for s in _capi.SIGNATURES}
    assert set(names) <= bound


def test_factory_rejects_other_types(lib):
    import openbcsim_gb300 as gb

    with pytest.raises(RuntimeError, match="Illegal algorithm type: cpu"):
        gb.RfSimulator("cpu")
    with pytest.raises(RuntimeError, match="Illegal algorithm type: gpu_fixed"):
        gb.RfSimulator("gpu_fixed")


def test_parameters(lib):
    import openbcsim_gb300 as gb

    s = gb.RfSimulator("gpu")
    for key, bad, msg in [("sound_speed", "-1", "illegal sound speed"),
                          ("radial_decimation", "0", "illegal radial decimation value"),
                          ("use_arc_projection", "maybe", "invalid boolean value"),
                          ("phase_delay", "yes", "invalid boolean value"),
                          ("cuda_streams", "3", "exceeds MAX_NUM_CUDA_STREAMS"),
                          ("cuda_streams", "0", "must be more than zero"),
                          ("threads_per_block", "0", "invalid number of threads per block"),
                          ("store_kernel_details", "x", "invalid value"),
                          ("precision_mode", "fp16", "precision_mode"),
                          ("no_such_key", "1", "illegal parameter name: 'no_such_key'")]:
        with pytest.raises(RuntimeError, match=msg):
            s.set_parameter(key, bad)
    s.set_parameter("sound_speed", "1480.5")
    assert float(s.get_parameter("sound_speed")) == pytest.approx(1480.5)
    s.set_parameter("phase_delay", "true")
    assert s.get_parameter("phase_delay") == "on"
    s.set_parameter("radial_decimation", "7")
    assert s.get_parameter("radial_decimation") == "7"
    s.set_parameter("precision_mode", "reference")
    assert s.get_parameter("precision_mode") == "reference"
    with pytest.raises(RuntimeError, match="Illegal key: nope"):
        s.get_parameter("nope")
    with pytest.raises(RuntimeError):     # std::stoi failure, as in the reference
        s.set_parameter("radial_decimation", "ten")


def test_configuration_order_and_checks(lib):
    import openbcsim_gb300 as gb
    from openbcsim_gb300 import workloads as W

    s = gb.RfSimulator("gpu")
    scan = W.sector_scan(4, 30.0, 0.05)
    # CpuAlgorithm.cpp:258-260
    with pytest.raises(RuntimeError, match="Excitation must be configured before scan sequence"):
        s.set_scan_sequence(scan.origins, scan.directions, scan.line_length, scan.lateral_dirs, scan.timestamps)
    taps, ci = W.gaussian_excitation(2.5e6, 0.1, 50e6)
    s.set_excitation(taps, ci, 50e6, 2.5e6)
    # ScanSequence.cpp:37-70
    bad = scan.lateral_dirs.copy()
    bad[1] = scan.directions[1]
    with pytest.raises(RuntimeError, match="Not orthogonal unit vectors"):
        s.set_scan_sequence(scan.origins, scan.directions, scan.line_length, bad, scan.timestamps)
    with pytest.raises(RuntimeError, match="Not unit length vectors"):
        s.set_scan_sequence(scan.origins, scan.directions * 1.01, scan.line_length, scan.lateral_dirs * 1.01,
                            scan.timestamps)
    with pytest.raises(RuntimeError, match="Scan sequence not configured."):
        s.simulate_lines()
    s.set_scan_sequence(scan.origins, scan.directions, scan.line_length, scan.lateral_dirs, scan.timestamps)
    assert s.output_shape() == (4, -(-W.num_rf_samples(1540.0, 0.05, 50e6) // 1))
    with pytest.raises(RuntimeError, match="Beam profile not configured."):
        s.simulate_lines()
    s.set_analytical_beam_profile(1e-3, 1e-3)
    with pytest.raises(RuntimeError, match="no scatterers are configured"):
        s.simulate_lines()
    assert s.get_total_num_scatterers() == 0
    with pytest.raises(RuntimeError, match="Too few radial samples"):
        s.set_lut_beam_profile(0, 1, -1, 1, -1, 1, np.zeros((1, 4, 4), np.float32))
    with pytest.raises(RuntimeError, match="Too few lateral samples"):
        s.set_lut_beam_profile(0, 1, -1, 1, -1, 1, np.zeros((4, 1, 4), np.float32))
    with pytest.raises(RuntimeError, match="Number of columns must be four"):
        s.add_fixed_scatterers(np.zeros((3, 3), np.float32))
    with pytest.raises(RuntimeError, match="mismatch in number of nodes"):
        s.add_spline_scatterers(3, np.zeros(5, np.float32), np.zeros((2, 4, 3), np.float32), np.zeros(2, np.float32))


def test_output_shape_follows_reference_sample_count(lib):
    """ns = floor(fs*2L/c + 0.5) in float (common_utils.hpp:38-41) for the
    workloads' line lengths; the output keeps every D-th sample."""
    import openbcsim_gb300 as gb
    from openbcsim_gb300 import workloads as W
    from oracle import oracle as O

    olib = O.oracle_lib()
    for L, D in [(0.12, 10), (0.13, 8), (0.05, 4), (0.15, 16), (0.0731, 3)]:
        s = gb.RfSimulator("gpu")
        taps, ci = W.gaussian_excitation(3e6, 0.2, 50e6)
        s.set_excitation(taps, ci, 50e6, 3e6)
        s.set_parameter("radial_decimation", str(D))
        scan = W.sector_scan(3, 10.0, L)
        s.set_scan_sequence(scan.origins, scan.directions, scan.line_length, scan.lateral_dirs, scan.timestamps)
        ns = olib.oracle_num_rf_samples(1540.0, L, 50e6)
        assert W.num_rf_samples(1540.0, L, 50e6) == ns
        assert s.output_shape() == (3, -(-ns // D))
    assert olib.oracle_num_rf_samples(1540.0, 0.12, 50e6) == 7792


def test_null_and_capacity_errors(lib):
    h = C.c_void_p()
    assert lib.bcsim_create(b"gpu", C.byref(h)) == 0
    buf = C.create_string_buffer(2)
    assert lib.bcsim_get_parameter(h, b"precision_mode", buf, 2) == 4      # BCSIM_E_CAPACITY
    assert lib.bcsim_simulate_lines(h, None, 0, None, None) == 2            # not configured
    assert b"Scan sequence not configured." in lib.bcsim_last_error(h)
    assert lib.bcsim_destroy(h) == 0
    assert lib.bcsim_set_parameter(None, b"verbose", b"1") == 1


def test_logger_receives_messages(lib):
    import openbcsim_gb300 as gb

    got = []
    s = gb.RfSimulator("gpu")
    s.set_logger(lambda level, msg: got.append((level, msg)))
    s.set_analytical_beam_profile(1e-3, 1e-3)
    assert any("analytical beam profile" in m for _, m in got)
    s.set_logger(None)


def test_frame_stream_argument_errors(lib):
    """bcsim_simulate_fixed_frames / bcsim_simulate_spline_frames check their
    arguments before any device work: missing data, a knot vector that does not
    match degree and control points (the reference's message), a degree out of
    range, null frames; zero frames is a no-op."""
    h = C.c_void_p()
    assert lib.bcsim_create(b"gpu", C.byref(h)) == 0
    f = C.POINTER(C.c_float)
    knots = np.zeros(8, np.float32)
    cps = np.zeros((4, 4, 3), np.float32)
    amps = np.zeros(4, np.float32)
    out = np.zeros(8, np.complex64)
    one = lambda a: (f * 1)(a.ctypes.data_as(f))   # noqa: E731
    kp = knots.ctypes.data_as(f)

    def spline(degree, num_knots, n, num_cs, frames, cps_arr=None, amps_arr=None, out_arr=None):
        return lib.bcsim_simulate_spline_frames(h, degree, kp, num_knots, cps_arr, amps_arr, n, num_cs, frames,
                                                out_arr, 8)

    assert spline(3, 8, 4, 4, 0) == 0                                       # no frames: nothing to do
    assert spline(3, 8, 4, 4, 1) == 1                                       # no frame pointers
    assert b"simulate_spline_frames: invalid data" in lib.bcsim_last_error(h)
    assert spline(3, 7, 4, 4, 1, one(cps), one(amps), one(out)) == 1
    assert b"mismatch in number of nodes, degree and control points" in lib.bcsim_last_error(h)
    assert spline(9, 14, 4, 4, 1, one(cps), one(amps), one(out)) == 1
    assert b"spline degree must be in [0, 7]" in lib.bcsim_last_error(h)
    nulls = (f * 1)()
    assert spline(3, 8, 4, 4, 1, nulls, one(amps), one(out)) == 1
    assert b"null frame or output" in lib.bcsim_last_error(h)
    xyza = np.zeros((4, 4), np.float32)
    assert lib.bcsim_simulate_fixed_frames(h, one(xyza), 0, 1, one(out), 8) == 1
    assert b"simulate_fixed_frames: invalid data" in lib.bcsim_last_error(h)
    assert lib.bcsim_simulate_fixed_frames(h, nulls, 4, 1, one(out), 8) == 1
    assert b"null frame or output" in lib.bcsim_last_error(h)
    assert lib.bcsim_destroy(h) == 0
