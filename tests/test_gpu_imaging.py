"""GPU post-processing (B-mode, scan conversion, colour Doppler, packets)
through the C ABI, against the CPU restatement (oracle/imaging_oracle.c) and the
reference's own scan converter (tests/golden/ref_imaging.npz).

Tolerances: where the kernels call a libm function that CUDA rounds
differently (log10f of the log compression, atan2f of the sector transform and
of arg R1), a byte may differ by 1 on at most 0.1 % of the pixels, a float by
1e-4 (absolute, values of order 1), an angle by 1e-6 rad.  Everything else is
bit-exact: R0, the linear scan conversion, and every engine entry point against
the equivalent sequence of calls."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden

pytestmark = pytest.mark.gpu

BYTE_FRAC = 1e-3


def engine(job):
    import openbcsim_gb300 as gb

    sim = gb.RfSimulator("gpu")
    gb.configure_job(sim, job)
    return sim


def bytes_close(a, b):
    d = np.abs(a.astype(np.int32) - b.astype(np.int32))
    return d.max() <= 1 and np.mean(d > 0) <= BYTE_FRAC


def sector_geometry(job, nx=300, ny=260):
    import openbcsim_gb300 as gb

    return gb.ScanGeometry("sector", float(np.float32(np.deg2rad(70.0))), job.scan.line_length, nx, ny)


@pytest.fixture(scope="module")
def oi():
    from oracle import imaging as OI

    return OI


def test_scan_conversion_vs_reference_fixture():
    import openbcsim_gb300 as gb

    z = np.load(os.path.join(GOLDEN, "ref_imaging.npz"))
    sim = gb.RfSimulator("gpu")
    for k, g in enumerate(z["geometries"]):
        geo = gb.ScanGeometry("sector" if g[0] == 0 else "linear", float(g[1]), float(g[2]), int(g[4]), int(g[5]),
                              tilt=float(g[3]))
        out = sim.scan_convert(z["beamspace_f32"], geo)
        ref = z[f"ref_f32_{k}"]
        if g[0] == 1:
            assert np.array_equal(out, ref), k      # no libm call on the linear path
        else:
            assert np.max(np.abs(out - ref)) <= 1e-4, k


@pytest.mark.parametrize("name", ["sector_pd", "sector_nopd", "lut3d"])
def test_bmode_vs_oracle(oi, name):
    job, _ = load_golden(name)
    sim = engine(job)
    iq = sim.simulate_lines_line_major()
    geo = sector_geometry(job)
    for normalize in (0.0, float(np.abs(iq).max()) * 0.5):
        img, bs, used = sim.bmode_image(iq, dyn_range=45.0, gain=1.2, normalize=normalize, geometry=geo,
                                        beamspace=True)
        oimg, obs, oused = oi.bmode(iq, 45.0, 1.2, normalize, geo)
        assert used == pytest.approx(oused, rel=1e-6)
        assert bytes_close(bs, obs)
        assert bytes_close(img, oimg)


def test_simulate_bmode_equals_the_two_calls():
    job, _ = load_golden("sector_pd")
    sim = engine(job)
    geo = sector_geometry(job, 200, 180)
    img, bs, used = sim.simulate_bmode(dyn_range=50.0, geometry=geo, beamspace=True)
    iq = sim.simulate_lines_line_major()
    img2, bs2, used2 = sim.bmode_image(iq, dyn_range=50.0, geometry=geo, beamspace=True)
    assert used == used2 and np.array_equal(bs, bs2) and np.array_equal(img, img2)


def test_doppler_vs_oracle(oi):
    rng = np.random.default_rng(21)
    P, L, nd = 10, 24, 300
    w = rng.uniform(-3.0, 3.0, (L, nd))
    amp = rng.uniform(0.1, 2.0, (L, nd))
    k = np.arange(P)[:, None, None]
    packet = (amp * np.exp(1j * (w * k + rng.uniform(0, 6.28, (L, nd)))) +
              0.05 * (rng.standard_normal((P, L, nd)) + 1j * rng.standard_normal((P, L, nd)))).astype(np.complex64)
    import openbcsim_gb300 as gb

    sim = gb.RfSimulator("gpu")
    geo = gb.ScanGeometry("linear", 0.03, 0.05, 120, 150)
    r0, vel, img = sim.color_doppler(packet, geometry=geo)
    or0, ovel = oi.color_doppler(packet)
    assert np.array_equal(r0, or0)
    assert np.max(np.abs(vel - ovel)) <= 1e-6
    oimg = oi.color_image(or0, ovel, geo)
    assert bytes_close(img, oimg)


def test_packet_of_fixed_scatterers_repeats_the_frame():
    job, _ = load_golden("sector_pd")
    sim = engine(job)
    one = sim.simulate_lines_line_major().copy()
    packet = sim.simulate_packet(4, 1.0 / 2500)
    assert packet.shape == (4,) + one.shape
    for f in packet:
        assert np.array_equal(f, one)


def test_packet_of_moving_scatterers():
    """Frame k equals a simulation with every timestamp advanced by k * prt;
    the configured scan sequence is unchanged afterwards."""
    job, _ = load_golden("spline")
    s0 = job.scan   # timestamps kept below the last knot interval for every frame
    job.scan = type(s0)(s0.origins, s0.directions, s0.lateral_dirs, (0.5 * s0.timestamps).astype(np.float32),
                        s0.line_length)
    sim = engine(job)
    before = sim.simulate_lines_line_major().copy()
    prt = 1.0 / 2500
    P = 3
    packet = sim.simulate_packet(P, prt)
    s = job.scan
    for k in range(P):
        ts = (s.timestamps.astype(np.float32) + np.float32(k) * np.float32(prt)).astype(np.float32)
        other = engine(job)
        other.set_scan_sequence(s.origins, s.directions, s.line_length, s.lateral_dirs, ts)
        assert np.array_equal(packet[k], other.simulate_lines_line_major()), k
    assert not np.array_equal(packet[0], packet[P - 1])
    assert np.array_equal(sim.simulate_lines_line_major(), before)


def test_simulate_color_doppler_equals_the_two_calls():
    import openbcsim_gb300 as gb

    job, _ = load_golden("spline")
    s0 = job.scan
    job.scan = type(s0)(s0.origins, s0.directions, s0.lateral_dirs, (0.5 * s0.timestamps).astype(np.float32),
                        s0.line_length)
    sim = engine(job)
    geo = gb.ScanGeometry("sector", 1.2, job.scan.line_length, 90, 80)
    r0, vel, img = sim.simulate_color_doppler(4, 1.0 / 2000, geometry=geo)
    packet = sim.simulate_packet(4, 1.0 / 2000)
    r0b, velb, imgb = sim.color_doppler(packet, geometry=geo)
    assert np.array_equal(r0, r0b) and np.array_equal(vel, velb) and np.array_equal(img, imgb)


def test_imaging_argument_errors():
    import openbcsim_gb300 as gb

    sim = gb.RfSimulator("gpu")
    iq = np.ones((4, 10), np.complex64)
    with pytest.raises(RuntimeError, match="at least 2 x 2"):
        sim.bmode_image(iq, geometry=gb.ScanGeometry("sector", 1.0, 0.1, 1, 50))
    with pytest.raises(RuntimeError, match="dynamic range"):
        sim.bmode_image(iq, dyn_range=0.0)
    with pytest.raises(RuntimeError, match="at least 2 frames"):
        sim.color_doppler(np.ones((1, 4, 10), np.complex64))
    with pytest.raises(RuntimeError, match="at least 2 beams"):
        sim.scan_convert(np.ones((1, 10), np.float32), gb.ScanGeometry("linear", 0.02, 0.05, 10, 10))
