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
