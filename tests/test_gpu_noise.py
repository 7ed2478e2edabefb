"""Seeded noise on the GPU against the oracle.

noise_amplitude > 0 adds complex Gaussian noise N(0, noise_amplitude) to every
time-projection sample j < ns before the convolution, as the reference does
(CpuAlgorithm.cpp:340-347); here it is keyed by (noise_seed, frame, line, j), so
it is reproducible and independent of how the lines are tiled or convolved.
The GPU's FP32 Box-Muller values differ from the oracle's double ones only by
rounding, so the noisy frames meet the same 1e-4 relative-RMS tolerance as the
noiseless ones.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-4


def sim_for(job, **params):
    import openbcsim_gb300 as gb

    s = gb.RfSimulator("gpu")
    gb.configure_job(s, job)
    for k, v in params.items():
        s.set_parameter(k, v)
    return s


@pytest.mark.parametrize("phase_delay", [True, False])
@pytest.mark.parametrize("conv", ["fir", "fft"])
def test_noise_matches_oracle(oracle, phase_delay, conv):
    from openbcsim_gb300 import workloads as W

    job = W.sector_2d_fixed(num_scatterers=5000, num_lines=24, phase_delay=phase_delay, seed=71)
    job.noise_amplitude, job.noise_seed = 0.2, 2024
    s = sim_for(job, convolution=conv)
    assert s.get_parameter("noise_frame") == "0"
    f0 = s.simulate_lines_line_major().copy()
    f1 = s.simulate_lines_line_major().copy()      # the next frame: fresh noise
    assert s.get_parameter("noise_frame") == "2"
    assert oracle.rel_rms(f0, oracle.simulate(job)) <= FP64_TOL
    job.noise_frame = 1
    assert oracle.rel_rms(f1, oracle.simulate(job)) <= FP64_TOL
    assert oracle.rel_rms(f0, f1) > 1e-2
    # the noise is a visible part of the frame
    job.noise_amplitude = 0.0
    assert oracle.rel_rms(f0, oracle.simulate(job)) > 1e-2


def test_noise_is_reproducible_and_tiling_independent():
    """The same seed gives the same bits: in another simulator, after the seed
    is set again, and whether the frame is convolved in one launch (device
    output) or in four line blocks (host output, 1024 lines)."""
    import torch

    from openbcsim_gb300 import workloads as W

    job = W.sector_2d_fixed(num_scatterers=3000, num_lines=1024, phase_delay=True, seed=72)
    job.noise_amplitude, job.noise_seed = 0.1, 7
    a = sim_for(job)
    host = a.simulate_lines_line_major().copy()     # four line blocks, each copied out
    b = sim_for(job)
    L, nd = b.output_shape()
    dev = torch.empty((L, nd), dtype=torch.complex64, device="cuda")
    b.simulate_lines_device(dev.data_ptr(), dev.numel())
    torch.cuda.synchronize()
    assert np.array_equal(dev.cpu().numpy(), host)
    a.set_parameter("noise_seed", "7")              # restarts the frame counter
    assert np.array_equal(a.simulate_lines_line_major(), host)
    a.set_parameter("noise_seed", "8")
    assert not np.array_equal(a.simulate_lines_line_major(), host)


def test_noise_in_batches_and_frames(oracle):
    """A batch with a noisy simulator draws a new frame every run (no graph
    replay of one frame); a stream of fixed-scatterer frames draws one frame
    of noise per frame."""
    import openbcsim_gb300 as gb
    from openbcsim_gb300 import workloads as W

    job = W.sector_2d_fixed(num_scatterers=4000, num_lines=16, phase_delay=True, seed=73)
    job.noise_amplitude, job.noise_seed = 0.3, 11
    batch = gb.Batch([sim_for(job), sim_for(W.sector_2d_fixed(num_scatterers=4000, num_lines=8, seed=74))])
    for frame in range(3):
        out = batch.run()[0]
        job.noise_frame = frame
        assert oracle.rel_rms(out, oracle.simulate(job)) <= FP64_TOL, frame
    s = sim_for(job)
    outs = s.simulate_fixed_frames([job.fixed[0].xyza] * 3)
    for frame, out in enumerate(outs):
        job.noise_frame = frame
        assert oracle.rel_rms(out, oracle.simulate(job)) <= FP64_TOL, frame
