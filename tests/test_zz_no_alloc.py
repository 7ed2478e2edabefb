"""The allocation-free entry point, bcsim_simulate_fixed_noalloc, against the
allocating one and against the FP64 oracle.

Callers that cannot allocate GPU memory -- imaging pipelines that reserve all
device memory at start-up, processes whose device memory is owned by another
framework's pool -- pass their own device buffers for the scatterers and the IQ,
and the engine keeps every intermediate in one static device array.  These
tests drive it through the C ABI twice in a row (the static array keeps the
previous call's contents, so the second call checks that it is cleared) and
compare each result with bcsim_simulate_lines on the same inputs and with the
FP64 oracle, over arc projection on and off, a decimation that divides the
sample count and one that does not, and a long and a short pulse.  Invalid
amplitudes, bounds, beam widths and pointers are rejected before anything runs.
The file sits apart so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# the tolerance of the GPU parity tests (relative RMS of the complex IQ)
TOL = 1e-4


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _call(lib, job, xyza_dev, n, out_dev, cap, bound, num_lines=None):
    s = job.scan
    L = s.num_lines if num_lines is None else num_lines
    origins = np.ascontiguousarray(np.resize(s.origins, (L, 3)), np.float32)
    dirs = np.ascontiguousarray(np.resize(s.directions, (L, 3)), np.float32)
    lats = np.ascontiguousarray(np.resize(s.lateral_dirs, (L, 3)), np.float32)
    taps = np.ascontiguousarray(job.taps, np.float32)
    err = C.create_string_buffer(512)
    rc = lib.bcsim_simulate_fixed_noalloc(
        C.c_void_p(xyza_dev), n, _fptr(origins), _fptr(dirs), _fptr(lats), L, s.line_length, job.sound_speed,
        _fptr(taps), len(taps), job.center_index, job.fs, job.demod_freq, job.beam.sigma_lateral,
        job.beam.sigma_elevational, int(job.arc), int(job.phase_delay), job.decimation, bound,
        C.c_void_p(out_dev), cap, None, err, 512)
    return rc, err.value.decode()


def _job(phase_delay=True, arc=True, decimation=10, short_pulse=False, seed=9101):
    from openbcsim_gb300 import workloads as W

    job = W.sector_2d_fixed(num_scatterers=20000, num_lines=48, phase_delay=phase_delay, seed=seed)
    job.arc = arc
    job.decimation = decimation
    if short_pulse:
        # the 3.5 MHz / bandwidth 0.15 pulse (132 taps) instead of 2.5 MHz / 0.1 (278)
        job.taps, job.center_index = W.gaussian_excitation(3.5e6, 0.15, job.fs)
        job.demod_freq = float(np.float32(3.5e6))
    return job


# ns = 7792 samples per line: decimation 8 divides it, 10 does not
CASES = [dict(phase_delay=True), dict(phase_delay=False), dict(arc=False), dict(decimation=8),
         dict(short_pulse=True, decimation=8), dict(arc=False, phase_delay=False, short_pulse=True)]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "-".join(f"{k}={v}" for k, v in c.items()))
def test_noalloc_matches_allocating_entry_point_and_oracle(case):
    import torch

    import openbcsim_gb300 as gb
    from openbcsim_gb300 import _capi
    from oracle import oracle as O
    from oracle.oracle import rel_rms

    job = _job(**case)
    sim = gb.RfSimulator("gpu")
    gb.configure_job(sim, job)
    ref = sim.simulate_lines_line_major().copy()
    fp64 = O.simulate(job, O.MODE_FP64)
    assert fp64.shape == ref.shape

    lib = _capi.load()
    xyza = torch.from_numpy(job.fixed[0].xyza).cuda()
    n = xyza.shape[0]
    out = torch.empty(ref.shape, dtype=torch.complex64, device="cuda")
    bound = float(np.abs(job.fixed[0].xyza[:, 3].astype(np.float64)).sum())
    for _ in range(2):
        out.fill_(complex(1e30, -1e30))
        torch.cuda.synchronize()
        rc, msg = _call(lib, job, xyza.data_ptr(), n, out.data_ptr(), out.numel(), bound)
        assert rc == 0, msg
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel_rms(got, ref) <= TOL
        assert rel_rms(got, fp64) <= TOL


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import torch

    from openbcsim_gb300 import _capi
    from openbcsim_gb300 import workloads as W

    job = W.sector_2d_fixed(num_scatterers=100, num_lines=4, phase_delay=True, seed=9102)
    lib = _capi.load()
    xyza = torch.from_numpy(job.fixed[0].xyza).cuda()
    out = torch.empty(16, dtype=torch.complex64, device="cuda")
    rc, msg = _call(lib, job, xyza.data_ptr(), 100, out.data_ptr(), out.numel(), 100.0, num_lines=5000)
    assert rc == 4 and "4096" in msg
    # 600 lines x 7792 samples x 2 exceed the 30 MiB of bins
    rc, msg = _call(lib, job, xyza.data_ptr(), 100, out.data_ptr(), out.numel(), 100.0, num_lines=600)
    assert rc == 4 and "scratch" in msg
    # too small an output buffer
    rc, msg = _call(lib, job, xyza.data_ptr(), 100, out.data_ptr(), out.numel(), 100.0)
    assert rc == 4 and "output buffer too small" in msg


def test_noalloc_rejects_invalid_amplitudes_bounds_and_pointers():
    import torch

    from openbcsim_gb300 import _capi

    job = _job(seed=9103)
    lib = _capi.load()
    xyza_host = job.fixed[0].xyza.copy()
    n = xyza_host.shape[0]
    L, nd = job.scan.num_lines, job.num_out
    out = torch.empty((L, nd), dtype=torch.complex64, device="cuda")
    bound = float(np.abs(xyza_host[:, 3].astype(np.float64)).sum())
    xyza = torch.from_numpy(xyza_host).cuda()
    # an understated amplitude bound would overflow the fixed-point bins
    rc, msg = _call(lib, job, xyza.data_ptr(), n, out.data_ptr(), out.numel(), bound * 0.5)
    assert rc == 1 and "amplitude_sum_bound" in msg
    # a NaN amplitude: the allocating path's message
    bad = xyza_host.copy()
    bad[17, 3] = np.nan
    bad_dev = torch.from_numpy(bad).cuda()
    rc, msg = _call(lib, job, bad_dev.data_ptr(), n, out.data_ptr(), out.numel(), bound)
    assert rc == 1 and msg == "Nan in scatterer projection."
    # a zero beam width
    job0 = _job(seed=9103)
    job0.beam.sigma_lateral = 0.0
    rc, msg = _call(lib, job0, xyza.data_ptr(), n, out.data_ptr(), out.numel(), bound)
    assert rc == 1 and "sigma" in msg
    # host memory where device memory is required (checked, never dereferenced)
    host_out = np.empty((L, nd), np.complex64)
    rc, msg = _call(lib, job, xyza.data_ptr(), n, host_out.ctypes.data, host_out.size, bound)
    assert rc == 1 and "d_out" in msg
    rc, msg = _call(lib, job, xyza_host.ctypes.data, n, out.data_ptr(), out.numel(), bound)
    assert rc == 1 and "d_xyza" in msg
    # and a valid call still succeeds afterwards
    rc, msg = _call(lib, job, xyza.data_ptr(), n, out.data_ptr(), out.numel(), bound)
    assert rc == 0, msg
    assert np.isfinite(out.cpu().numpy()).all()
