"""Pins the CPU oracle against the reference's own CPU algorithm.

The golden fixtures hold the output of the compiled reference (bcsim CPU
algorithm) for small seeded cases.  The oracle's REF32 mode restates the
reference's float arithmetic and must reproduce its time-projection bins bit
for bit; its IQ differs only by the reference's float FFT rounding.  The FP64
mode is the tolerance reference for the GPU engine.
"""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden

# the reference convolves with a recursive float FFT whose twiddle factors are
# built by repeated multiplication; its rounding bounds the IQ agreement
REF_FFT_TOL = 3e-4
# FP32 (reference) versus FP64 (oracle) arithmetic on the same inputs
REF_VS_FP64_TOL = 3e-3


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_ref32_bins_bit_exact(oracle, name):
    job, z = load_golden(name)
    for row, line in enumerate(z["ref_bins_lines"]):
        ob = oracle.project_bins(job, int(line), oracle.MODE_REF32)
        rb = z["ref_bins"][row].astype(np.complex128)
        assert np.array_equal(ob, rb), f"{name} line {line}: max |diff| {np.abs(ob - rb).max()}"


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_ref32_iq_matches_reference(oracle, name):
    job, z = load_golden(name)
    iq = oracle.simulate(job, oracle.MODE_REF32)
    assert iq.shape == z["ref_iq"].shape
    assert oracle.rel_rms(iq, z["ref_iq"]) <= REF_FFT_TOL


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_fp64_close_to_reference(oracle, name):
    job, z = load_golden(name)
    iq = oracle.simulate(job, oracle.MODE_FP64)
    assert oracle.rel_rms(iq, z["ref_iq"]) <= REF_VS_FP64_TOL


def test_live_reference_when_available(oracle):
    """Where the reference sources were compiled (oracle/_ref), the fixtures are
    reproduced by the live reference."""
    if not oracle.ref_available():
        pytest.skip("reference not compiled on this machine")
    job, z = load_golden("sector_pd")
    iq = oracle.ref_simulate(job, threads=1)
    assert np.array_equal(iq, z["ref_iq"])


def test_oracle_errors_match_reference_messages(oracle):
    from openbcsim_gb300 import workloads as W

    job = W.sector_spline(num_scatterers=10, num_lines=2, seed=1)
    job.scan.timestamps[:] = 5.0        # outside every knot interval
    # the reference throws this from inside its OpenMP line loop
    # (CpuAlgorithm.cpp:289-299), which terminates the process instead of
    # reaching the caller; the oracle and the engine report it as an error
    with pytest.raises(RuntimeError, match="could not determine knot interval"):
        oracle.simulate(job)


def _full_subset(name):
    import copy
    import os

    from conftest import GOLDEN
    from openbcsim_gb300 import workloads as W

    z = np.load(os.path.join(GOLDEN, f"ref_full_{name}.npz"))
    job = getattr(W, name)()
    idx = z["lines"]
    sub = copy.copy(job)
    s = job.scan
    sub.scan = W.ScanSequence(s.origins[idx], s.directions[idx], s.lateral_dirs[idx], s.timestamps[idx],
                              s.line_length)
    return sub, z["ref_iq"]


@pytest.mark.parametrize("name", ["sector_2d_fixed", "volume_3d_lut", "sector_spline"])
def test_full_size_workloads_pinned(oracle, name):
    """The full-size benchmark workloads (inputs from their seeds): 32 lines
    spread over each, against the IQ that the reference's own CPU algorithm
    returned for them (tests/golden/ref_full_*.npz).  The REF32 restatement
    differs only by the reference's float FFT; the FP64 oracle by the
    reference's FP32 arithmetic."""
    sub, ref_iq = _full_subset(name)
    assert oracle.rel_rms(oracle.simulate(sub, oracle.MODE_REF32), ref_iq) <= 1e-4
    assert oracle.rel_rms(oracle.simulate(sub, oracle.MODE_FP64), ref_iq) <= REF_VS_FP64_TOL
