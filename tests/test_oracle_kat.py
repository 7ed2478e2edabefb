"""The CPU oracle against the known answers of the reference's own unit tests
(tests/golden/reference_kats.json, restated from src/core/unittest/test_fft.cpp,
test_hilbert_mask.cpp and src/utils/unittest/test_SignalProcessing.cpp)."""
import ctypes as C
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN


@pytest.fixture(scope="module")
def kats():
    with open(os.path.join(GOLDEN, "reference_kats.json")) as f:
        return json.load(f)


def test_fft_conv(oracle, kats):
    lib = oracle.oracle_lib()
    for case in kats["fft_conv"]:
        x = np.array(case["x"], np.float64)
        h = np.array(case["h"], np.float64)
        out = np.zeros(len(x) + len(h) - 1)
        n = lib.oracle_fft_conv(x.ctypes.data_as(C.POINTER(C.c_double)), len(x), h.ctypes.data_as(C.POINTER(C.c_double)),
                                len(h), out.ctypes.data_as(C.POINTER(C.c_double)))
        assert n == len(case["expected"])
        # BOOST_CHECK_CLOSE(x, y, 0.01): relative difference within 0.01 percent
        np.testing.assert_allclose(out, case["expected"], rtol=case["rel_tol_percent"] / 100.0)


def test_next_power_of_two(oracle, kats):
    lib = oracle.oracle_lib()
    for n, expected in kats["next_power_of_two"]["table"]:
        assert lib.oracle_next_pow2(n) == expected


def test_hilbert_mask(oracle, kats):
    lib = oracle.oracle_lib()
    for n, expected in kats["hilbert_mask"]["masks"].items():
        out = np.zeros(int(n))
        lib.oracle_hilbert_mask(int(n), out.ctypes.data_as(C.POINTER(C.c_double)))
        assert out.astype(int).tolist() == expected


def test_direct_conv(oracle, kats):
    lib = oracle.oracle_lib()
    for case in kats["direct_conv"]:
        x = np.array(case["x"], np.int64)
        h = np.array(case["h"], np.int64)
        out = np.zeros(len(x) + len(h) - 1, np.int64)
        lib.oracle_direct_conv_i64(x.ctypes.data_as(C.POINTER(C.c_int64)), len(x),
                                   h.ctypes.data_as(C.POINTER(C.c_int64)), len(h),
                                   out.ctypes.data_as(C.POINTER(C.c_int64)))
        assert out.tolist() == case["expected"]


def test_bspline_partition_of_unity(oracle):
    """Clamped uniform knots: the basis sums to one inside the support, the
    non-zero basis functions are mu-p..mu (src/core/bspline.hpp:74-91)."""
    from openbcsim_gb300 import workloads as W

    lib = oracle.oracle_lib()
    knots = W.end_hack_knots(16, 3)
    kp = knots.ctypes.data_as(C.POINTER(C.c_float))
    for t in np.linspace(0.0, 1.0 - 1e-5, 57).astype(np.float32):
        mu = lib.oracle_knot_interval(kp, len(knots), float(t))
        vals = [lib.oracle_bspline_basis_d(j, 3, float(t), kp) for j in range(16)]
        assert abs(sum(vals) - 1.0) < 1e-12
        nz = [j for j, v in enumerate(vals) if abs(v) > 1e-12]
        assert min(nz) >= mu - 3 and max(nz) <= mu
    # t at the end-hacked last knot interval is outside the usable range
    assert lib.oracle_knot_interval(kp, len(knots), 2.0) == -1


def test_gaussian_excitation_matches_restatement(oracle):
    """MakeGaussianExcitation (src/utils/GaussPulse.cpp:52-70): the C oracle and
    the package's numpy generator give the same taps and centre index."""
    from openbcsim_gb300 import workloads as W

    lib = oracle.oracle_lib()
    for fc, bw in [(2.5e6, 0.1), (3.5e6, 0.15), (7e6, 0.3), (2e6, 0.25)]:
        buf = np.zeros(4096, np.float32)
        ci = C.c_int()
        n = lib.oracle_gaussian_excitation(fc, bw, 50e6, buf.ctypes.data_as(C.POINTER(C.c_float)), 4096, C.byref(ci))
        taps, c = W.gaussian_excitation(fc, bw, 50e6)
        assert n == len(taps) and ci.value == c
        np.testing.assert_allclose(buf[:n], taps, rtol=0, atol=2e-7)


def _excitation_fixture():
    import os

    from conftest import GOLDEN

    z = np.load(os.path.join(GOLDEN, "ref_excitation.npz"))
    return [(tuple(p), z[f"taps_{k}"], int(z[f"center_{k}"])) for k, p in enumerate(z["params"])]


def test_gaussian_excitation_pinned_to_reference():
    """The package's pulse generator against the taps that the reference's own
    MakeGaussianExcitation<float> (src/utils/GaussPulse.cpp:52-70, compiled by
    oracle/Makefile) returned for ten pulses (tests/golden/ref_excitation.npz):
    the same length and centre index and the same taps, bit for bit (the
    generator calls the C library's cosf and exp, as the reference does)."""
    from openbcsim_gb300 import workloads as W

    for (fc, bw, fs), ref_taps, ref_center in _excitation_fixture():
        taps, center = W.gaussian_excitation(fc, bw, fs)
        assert len(taps) == len(ref_taps) and center == ref_center, (fc, bw, fs)
        assert np.array_equal(taps, ref_taps), (fc, bw, fs)


def test_gaussian_excitation_live_reference(oracle):
    """Where the reference is compiled here, it still gives the fixture's taps."""
    if not oracle.ref_available():
        pytest.skip("reference not compiled on this machine")
    lib = oracle.ref_lib()
    for (fc, bw, fs), ref_taps, ref_center in _excitation_fixture():
        buf = np.zeros(1 << 16, np.float32)
        ci = C.c_int()
        n = lib.ref_gaussian_excitation(fc, bw, fs, buf.ctypes.data_as(C.POINTER(C.c_float)), buf.size, C.byref(ci))
        assert n == len(ref_taps) and ci.value == ref_center
        assert np.array_equal(buf[:n], ref_taps)
