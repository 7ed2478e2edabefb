"""Streams of fixed-scatterer frames through bcsim_simulate_fixed_frames (the
next frame's upload overlapping the current frame's simulation) give, bit for
bit, what clear + add_fixed_scatterers + simulate_lines per frame give, on the
shared-origin path and on the per-pair path; the last frame stays the fixed
dataset; a non-finite amplitude stops the stream with the reference's message."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def engine(job):
    import openbcsim_gb300 as gb

    sim = gb.RfSimulator("gpu")
    gb.configure_job(sim, job)
    return sim


def frames_of(job, count, seed):
    rng = np.random.default_rng(seed)
    base = np.concatenate([f.xyza for f in job.fixed])
    out = []
    for _ in range(count):
        f = base.copy()
        f[:, :3] += rng.normal(0.0, 2e-4, f[:, :3].shape).astype(np.float32)
        f[:, 3] *= np.float32(rng.uniform(0.5, 2.0))
        out.append(np.ascontiguousarray(f, np.float32))
    return out


@pytest.mark.parametrize("name", ["lut3d", "sector_pd", "linear"])
def test_frames_equal_per_frame_calls(name):
    job, _ = load_golden(name)
    frames = frames_of(job, 5, 31)
    sim = engine(job)
    outs = sim.simulate_fixed_frames(frames)
    assert len(outs) == len(frames)
    for k, f in enumerate(frames):
        ref = engine(job)
        ref.clear_fixed_scatterers()
        ref.add_fixed_scatterers(f)
        assert np.array_equal(outs[k], ref.simulate_lines_line_major()), (name, k)
    assert not np.array_equal(outs[0], outs[1])
    # the last frame is the fixed dataset afterwards
    assert np.array_equal(sim.simulate_lines_line_major(), outs[-1])
    assert sim.get_total_num_scatterers() == frames[0].shape[0]


def test_frames_from_pinned_memory_and_reused_outputs():
    import torch

    job, _ = load_golden("lut3d")
    frames = frames_of(job, 3, 7)
    pinned = []
    for f in frames:
        t = torch.empty(f.shape, dtype=torch.float32, pin_memory=True)
        t.numpy()[:] = f
        pinned.append(t.numpy())
    sim = engine(job)
    L, nd = sim.output_shape()
    outs = [torch.empty((L, nd), dtype=torch.complex64, pin_memory=True).numpy() for _ in frames]
    a = [o.copy() for o in sim.simulate_fixed_frames(pinned, outs)]
    b = sim.simulate_fixed_frames(frames)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_frames_stop_at_a_non_finite_amplitude():
    job, _ = load_golden("sector_pd")
    frames = frames_of(job, 3, 5)
    frames[1][17, 3] = np.nan
    sim = engine(job)
    with pytest.raises(RuntimeError, match="Nan in scatterer projection."):
        sim.simulate_fixed_frames(frames)
    with pytest.raises(RuntimeError, match="Nan in scatterer projection."):
        sim.simulate_lines_line_major()
    # a clean stream afterwards works
    good = frames_of(job, 2, 6)
    outs = sim.simulate_fixed_frames(good)
    ref = engine(job)
    ref.clear_fixed_scatterers()
    ref.add_fixed_scatterers(good[1])
    assert np.array_equal(outs[1], ref.simulate_lines_line_major())


def test_frames_argument_errors():
    job, _ = load_golden("sector_pd")
    sim = engine(job)
    f = frames_of(job, 2, 1)
    with pytest.raises(ValueError):
        sim.simulate_fixed_frames([f[0], f[1][:-1]])
    with pytest.raises(RuntimeError):
        sim.simulate_fixed_frames([f[0][:, :3]])


def spline_frames_of(sp, count, seed):
    rng = np.random.default_rng(seed)
    cps, amps = [], []
    for _ in range(count):
        c = sp.control_points + rng.normal(0.0, 2e-4, sp.control_points.shape).astype(np.float32)
        cps.append(np.ascontiguousarray(c, np.float32))
        amps.append(np.ascontiguousarray(sp.amplitudes * np.float32(rng.uniform(0.5, 2.0)), np.float32))
    return cps, amps


@pytest.mark.parametrize("shared_time", [False, True])
def test_spline_frames_equal_per_frame_calls(shared_time):
    """Streams of spline frames (bcsim_simulate_spline_frames): lines at their
    own times (the per-pair path) and at one shared time (rendered once into
    shared-origin records) give, bit for bit, clear_spline_scatterers +
    add_spline_scatterers + simulate_lines per frame; the last frame stays the
    spline dataset."""
    from openbcsim_gb300 import workloads as W

    rng = np.random.default_rng(41)
    sp = W.random_spline(rng, 30_000, 12)
    t0, t1 = W.spline_time_limits(sp.degree, sp.knots, 12)
    ts = np.full(96, 0.5 * (t0 + t1), np.float32) if shared_time else np.linspace(t0, t1, 96).astype(np.float32)
    scan = W.sector_scan(96, 35.0, 0.12, timestamps=ts)
    job = W._excitation_job("spline_frames", scan, 2.5e6, 0.1, W.GaussianBeam(1e-3, 1e-3), [], [sp], 10)
    cps, amps = spline_frames_of(sp, 4, 43)
    sim = engine(job)
    outs = sim.simulate_spline_frames(sp.degree, sp.knots, cps, amps)
    assert len(outs) == len(cps)
    for k in range(len(cps)):
        ref = engine(job)
        ref.clear_spline_scatterers()
        ref.add_spline_scatterers(sp.degree, sp.knots, cps[k], amps[k])
        assert np.array_equal(outs[k], ref.simulate_lines_line_major()), k
    assert not np.array_equal(outs[0], outs[1])
    assert np.array_equal(sim.simulate_lines_line_major(), outs[-1])
    assert sim.get_total_num_scatterers() == cps[0].shape[0]


def test_spline_frames_stop_at_a_non_finite_amplitude():
    import openbcsim_gb300 as gb
    from openbcsim_gb300 import workloads as W

    job = W.sector_spline(num_scatterers=8_000, num_lines=32)
    sp = job.splines[0]
    cps, amps = spline_frames_of(sp, 3, 47)
    amps[1] = amps[1].copy()
    amps[1][5] = np.nan
    sim = engine(job)
    outs = [np.zeros(sim.output_shape(), np.complex64) for _ in cps]
    with pytest.raises(gb.SimulatorError) as ei:
        sim.simulate_spline_frames(sp.degree, sp.knots, cps, amps, outs)
    assert "Nan in scatterer projection." in str(ei.value)
    ref = engine(job)
    ref.clear_spline_scatterers()
    ref.add_spline_scatterers(sp.degree, sp.knots, cps[0], amps[0])
    assert np.array_equal(outs[0], ref.simulate_lines_line_major())
    with pytest.raises(ValueError):
        sim.simulate_spline_frames(sp.degree, sp.knots, cps, amps[:2])
