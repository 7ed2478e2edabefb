"""The allocation-free entry point, bcsim_simulate_fixed_noalloc, against the
allocating one.

Callers that cannot allocate GPU memory -- imaging pipelines that reserve all
device memory at start-up, processes whose device memory is owned by another
framework's pool -- pass their own device buffers for the scatterers and the IQ,
and the engine keeps every intermediate in one static device array.  This test
drives it through the C ABI twice in a row (the static array keeps the previous
call's contents, so the second call checks that it is cleared) and compares
each result with bcsim_simulate_lines on the same inputs.  It sits in a file of
its own that pytest collects last.
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


@pytest.mark.parametrize("phase_delay", [True, False])
def test_noalloc_matches_allocating_entry_point(phase_delay):
    import torch

    import openbcsim_gb300 as gb
    from openbcsim_gb300 import _capi
    from openbcsim_gb300 import workloads as W
    from oracle.oracle import rel_rms

    job = W.sector_2d_fixed(num_scatterers=20000, num_lines=48, phase_delay=phase_delay, seed=9101)
    sim = gb.RfSimulator("gpu")
    gb.configure_job(sim, job)
    ref = sim.simulate_lines_line_major().copy()

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
