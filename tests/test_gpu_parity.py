"""GPU parity: the engine (through the C ABI) against the CPU oracle and the
reference's own outputs.

Tolerances (relative RMS over all lines and samples of the complex IQ):
  * fp64 mode vs the FP64 oracle:             1e-4 (the stated accuracy target)
  * reference mode vs the reference's IQ:      3e-4 (the reference's float FFT)
  * reference mode vs the oracle's REF32 mode: 2e-5 (same bins; double-precision
    convolution on both sides, FIR truncation 1e-10 of the pulse energy)
"""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-4
REF_IQ_TOL = 3e-4
REF32_TOL = 2e-5


def engine(job, mode="fp64", **params):
    import openbcsim_gb300 as gb

    sim = gb.RfSimulator("gpu")
    gb.configure_job(sim, job, mode)
    for k, v in params.items():
        sim.set_parameter(k, v)
    return sim


def run(job, mode="fp64", **params):
    return engine(job, mode, **params).simulate_lines_line_major()


@pytest.mark.parametrize("conv", ["fir", "fft"])
@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_fp64_vs_oracle(oracle, name, conv):
    job, _ = load_golden(name)
    iq = run(job, convolution=conv)
    ref = oracle.simulate(job, oracle.MODE_FP64)
    assert iq.shape == ref.shape
    assert oracle.rel_rms(iq, ref) <= FP64_TOL


@pytest.mark.parametrize("conv", ["fir", "fft"])
@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_reference_mode_vs_reference(oracle, name, conv):
    job, z = load_golden(name)
    iq = run(job, "reference", convolution=conv)
    assert oracle.rel_rms(iq, z["ref_iq"]) <= REF_IQ_TOL
    assert oracle.rel_rms(iq, oracle.simulate(job, oracle.MODE_REF32)) <= REF32_TOL


def test_convolution_routes():
    """The FFT route (the exact circular convolution) and the direct FIR (the
    window of the analytic pulse holding all but 1e-10 of its energy) agree to
    the window's truncation, about 1e-5.  The automatic choice weighs the two
    routes' times for the line count: the FFT (one CTA per line) for many lines
    with the long 2.5 MHz / bw 0.1 pulse (a 1960-tap window), the FIR for few
    lines and for the short 3.5 MHz / bw 0.15 pulse with decimation 8."""
    from oracle.oracle import rel_rms
    from openbcsim_gb300 import workloads as W

    many = W.sector_2d_fixed(num_scatterers=2000, num_lines=256, phase_delay=True, seed=17)
    cases = [(load_golden("sector_pd")[0], "fir"), (load_golden("lut3d")[0], "fir"), (many, "fft")]
    for job, route in cases:
        sim = engine(job)
        assert sim.get_parameter("convolution_route") == ""
        auto = sim.simulate_lines_line_major().copy()
        assert sim.get_parameter("convolution_route") == route, job.name
        fir = run(job, convolution="fir")
        fft = run(job, convolution="fft")
        assert np.array_equal(auto, fft if route == "fft" else fir)
        assert rel_rms(fft, fir) <= 3e-5, job.name


def test_fft_route_decimation_folds(oracle):
    """Every decimation folds a different power of two into the spectrum
    (F = 1, 2, 4, 8, 16; D = 48 folds 16 and keeps every third sample)."""
    from openbcsim_gb300 import workloads as W

    for D in (1, 2, 5, 12, 24, 32, 48):
        job = W.sector_2d_fixed(num_scatterers=2000, num_lines=3, phase_delay=True, seed=40 + D)
        job.decimation = D
        iq = run(job, convolution="fft")
        assert iq.shape == (3, -(-job.num_samples // D))
        assert oracle.rel_rms(iq, oracle.simulate(job)) <= FP64_TOL, D


@pytest.mark.parametrize("line_length,fc,bw,D", [(0.0019, 3.5e6, 0.15, 8), (0.0036, 2.5e6, 0.1, 10),
                                                (0.006, 2.5e6, 0.1, 10), (0.012, 2.5e6, 0.1, 5),
                                                (0.05, 2.5e6, 0.1, 16)])
def test_fft_route_transform_lengths(oracle, line_length, fc, bw, D):
    """Transform lengths M = 256, 512, 1024, 2048, 4096: every radix plan of the
    FFT route (16 x 16, 16 x 2 x 16, 16 x 4 x 16, 16 x 8 x 16, 16 x 16 x 16)
    against the FP64 oracle, scatterers within the short lines."""
    from openbcsim_gb300 import workloads as W

    rng = np.random.default_rng(int(line_length * 1e5))
    n = 3000
    xyza = np.stack([rng.uniform(-0.3, 0.3, n) * line_length, np.zeros(n),
                     rng.uniform(0.1, 0.95, n) * line_length, rng.standard_normal(n)], axis=1).astype(np.float32)
    scan = W.sector_scan(4, 20.0, line_length)
    job = W._excitation_job("short_lines", scan, fc, bw, W.GaussianBeam(1e-3, 1e-3), [W.FixedSet(xyza)], [], D)
    iq = run(job, convolution="fft")
    M = 1 << int(np.ceil(np.log2(job.num_samples + len(job.taps) - 1)))
    assert M <= 4096 and np.abs(iq).max() > 0
    assert oracle.rel_rms(iq, oracle.simulate(job)) <= FP64_TOL, M


def test_fft_route_rejects_long_lines():
    """M beyond one CTA's shared memory: convolution=fft is refused, auto takes the FIR."""
    from openbcsim_gb300 import workloads as W

    job = W.sector_2d_fixed(num_scatterers=500, num_lines=2, phase_delay=True, seed=3)
    s = job.scan
    job.scan = type(s)(s.origins, s.directions, s.lateral_dirs, s.timestamps, 0.3)   # ns ~ 19.5k: M = 32768
    with pytest.raises(RuntimeError, match="convolution=fft"):
        run(job, convolution="fft")
    sim = engine(job)
    sim.simulate_lines_line_major()
    assert sim.get_parameter("convolution_route") == "fir"


@pytest.mark.parametrize("name", ["sector_pd", "lut3d", "spline", "linear"])
def test_deterministic(name):
    job, _ = load_golden(name)
    sim = engine(job)
    a = sim.simulate_lines_line_major().copy()
    b = sim.simulate_lines_line_major().copy()
    c = run(job)
    assert np.array_equal(a, b) and np.array_equal(a, c)


def test_pyrfsim_layout():
    """simulate_lines returns [samples, lines] like pyrfsim (PythonInterface.cpp:299-318)."""
    job, _ = load_golden("sector_pd")
    sim = engine(job)
    a = sim.simulate_lines()
    b = sim.simulate_lines_line_major()
    assert a.shape == (b.shape[1], b.shape[0]) and np.array_equal(a, b.T) and a.dtype == np.complex64


def test_amplitude_scaling_is_exact():
    """Doubling every amplitude doubles the IQ bit for bit: the fixed-point scale
    follows the amplitude bound by a power of two."""
    job, _ = load_golden("lut3d")
    a = run(job)
    job.fixed[0].xyza = job.fixed[0].xyza.copy()
    job.fixed[0].xyza[:, 3] *= 2
    b = run(job)
    assert np.array_equal(b, 2 * a)


def test_line_permutation_and_split_datasets():
    job, _ = load_golden("sector_pd")
    a = run(job)
    perm = np.random.default_rng(5).permutation(job.scan.num_lines)
    s = job.scan
    job.scan = type(s)(s.origins[perm], s.directions[perm], s.lateral_dirs[perm], s.timestamps[perm], s.line_length)
    b = run(job)
    assert np.array_equal(b, a[perm])
    job.scan = s
    xyza = job.fixed[0].xyza
    from openbcsim_gb300 import workloads as W

    job.fixed = [W.FixedSet(xyza[:1234]), W.FixedSet(xyza[1234:])]
    c = run(job)
    assert np.array_equal(c, a)


def test_superposition():
    """The simulation is linear in the scatterers."""
    from openbcsim_gb300 import workloads as W
    from oracle.oracle import rel_rms

    job, _ = load_golden("linear")
    xyza = job.fixed[0].xyza
    a = run(job)
    job.fixed = [W.FixedSet(xyza[:1500])]
    b = run(job)
    job.fixed = [W.FixedSet(xyza[1500:])]
    c = run(job)
    assert rel_rms(b + c, a) <= 1e-6


def test_empty_and_out_of_range_scatterers():
    from openbcsim_gb300 import workloads as W

    job, _ = load_golden("sector_pd")
    far = np.array([[0.0, 0.0, 1.0, 1.0], [0.0, 0.0, -1.0, 1.0]], np.float32)   # beyond the line end / behind
    job.fixed = [W.FixedSet(np.zeros((0, 4), np.float32)), W.FixedSet(far)]
    iq = run(job)
    assert np.all(iq == 0)


def test_single_line_decimations(oracle):
    from openbcsim_gb300 import workloads as W

    for D in (1, 3, 16):
        job = W.sector_2d_fixed(num_scatterers=3000, num_lines=1, phase_delay=True, seed=11 + D)
        job.decimation = D
        iq = run(job)
        assert iq.shape == (1, -(-job.num_samples // D))
        assert oracle.rel_rms(iq, oracle.simulate(job)) <= FP64_TOL


def test_nan_amplitude_reports_reference_message():
    from openbcsim_gb300 import workloads as W

    job, _ = load_golden("sector_pd")
    bad = job.fixed[0].xyza.copy()
    bad[10, 3] = np.nan
    job.fixed = [W.FixedSet(bad)]
    with pytest.raises(RuntimeError, match="Nan in scatterer projection."):
        run(job)


def test_spline_time_outside_knots():
    job, _ = load_golden("spline")
    job.scan.timestamps = np.full_like(job.scan.timestamps, 3.0)
    with pytest.raises(RuntimeError, match="could not determine knot interval"):
        run(job)


def _line_subset(job, idx):
    """The job restricted to scan lines idx (lines are independent)."""
    import copy

    from openbcsim_gb300 import workloads as W

    sub = copy.copy(job)
    s = job.scan
    sub.scan = W.ScanSequence(s.origins[idx], s.directions[idx], s.lateral_dirs[idx], s.timestamps[idx],
                              s.line_length)
    return sub


def _spread_lines(which, L):
    if which == "sector_2d_fixed":
        return np.arange(L)                                   # the whole frame
    if which == "sector_spline":
        return np.unique(np.linspace(0, L - 1, 128).round().astype(int))
    # 64 x 64 volume: a spread of 256 lines over the grid (its stride is not a
    # multiple of the row length, so azimuths vary), the four corners, the
    # middles of the four edges and the centre lines
    n = int(round(np.sqrt(L)))
    extra = [0, n - 1, L - n, L - 1, n // 2, L - n + n // 2, (n // 2) * n, (n // 2) * n + n - 1,
             (n // 2) * n + n // 2 - 1, (n // 2) * n + n // 2]
    return np.unique(np.concatenate([np.linspace(0, L - 1, 256).round().astype(int), extra]))


@pytest.mark.parametrize("which", ["sector_2d_fixed", "volume_3d_lut", "sector_spline"])
def test_full_size_frames_vs_oracle(oracle, which):
    """The workloads at full size against the FP64 oracle: every line of the
    2-D sector frame (128), 128 lines spread over the spline frame's 1024, and
    256 spread lines of the 64 x 64 volume plus its corners, edge middles and
    centre; each over all its samples."""
    from openbcsim_gb300 import workloads as W

    job = getattr(W, which)()
    iq = run(job)
    assert np.isfinite(iq).all()
    idx = _spread_lines(which, job.scan.num_lines)
    ref = oracle.simulate(_line_subset(job, idx), oracle.MODE_FP64)
    assert oracle.rel_rms(iq[idx], ref) <= FP64_TOL, which
    # and no line is off on its own: the worst line's relative RMS
    worst = max(oracle.rel_rms(iq[i], ref[k]) for k, i in enumerate(idx) if np.abs(ref[k]).max() > 0)
    assert worst <= 10 * FP64_TOL, (which, worst)


@pytest.mark.parametrize("which", ["sector_2d_fixed", "volume_3d_lut", "sector_spline"])
def test_full_size_vs_reference_iq(oracle, which):
    """The full-size workloads on the GPU against the IQ that the reference's
    own CPU algorithm returned for 32 spread lines of each
    (tests/golden/ref_full_*.npz): the reference-arithmetic mode within the
    reference's float FFT, the fp64 mode within the reference's own FP32
    error against FP64."""
    import os

    from conftest import GOLDEN
    from openbcsim_gb300 import workloads as W

    z = np.load(os.path.join(GOLDEN, f"ref_full_{which}.npz"))
    job = getattr(W, which)()
    idx = z["lines"]
    assert oracle.rel_rms(run(job, "reference")[idx], z["ref_iq"]) <= REF_IQ_TOL
    assert oracle.rel_rms(run(job)[idx], z["ref_iq"]) <= 3e-3


def test_render_once_at_shared_timestamp(oracle):
    """Splines that every line sees at one timestamp from one origin are
    rendered once into shared-origin records (the reference renders them to
    fixed scatterers first, GpuAlgorithm.cpp:181-187 and
    GpuScatterers.cpp:48-123), alone and mixed with fixed scatterers: the frame
    matches the FP64 oracle, the per-pair evaluation of the same splines
    (render_once=off) and, in reference arithmetic, the oracle's REF32 mode."""
    from openbcsim_gb300 import workloads as W

    rng = np.random.default_rng(81)
    sp = W.random_spline(rng, 40_000, 16)
    fixed = W.random_fixed(rng, 20_000, (-0.03, 0.03), None, (0.01, 0.12))
    scan = W.sector_scan(96, 35.0, 0.12, timestamps=np.full(96, 0.37, np.float32))
    for fixed_sets in ([], [fixed]):
        job = W._excitation_job("render_once", scan, 2.5e6, 0.1, W.GaussianBeam(1e-3, 1e-3), fixed_sets, [sp], 10)
        sim = engine(job, store_kernel_details="on")
        once = sim.simulate_lines_line_major().copy()
        # the shared-origin path ran (its record preparation was timed)
        assert len(sim.get_debug_data("prep_sort_ms")) == 1
        per_pair_sim = engine(job, store_kernel_details="on", render_once="off")
        per_pair = per_pair_sim.simulate_lines_line_major().copy()
        if not fixed_sets:
            with pytest.raises(RuntimeError):
                per_pair_sim.get_debug_data("prep_sort_ms")   # no shared-origin records at all
        ref = oracle.simulate(job, oracle.MODE_FP64)
        assert oracle.rel_rms(once, ref) <= FP64_TOL
        assert oracle.rel_rms(per_pair, ref) <= FP64_TOL
        assert oracle.rel_rms(once, per_pair) <= 3e-5
        # deterministic, and bit-identical when simulated again
        assert np.array_equal(once, sim.simulate_lines_line_major())
        ref32 = oracle.simulate(job, oracle.MODE_REF32)
        assert oracle.rel_rms(run(job, "reference"), ref32) <= REF32_TOL


def test_large_phantom_few_lines(oracle):
    """30 million fixed scatterers (0.5 GB of phantom, 1 GB of sorted records)
    on 8 lines of the 3-D LUT volume: every record chunk, sort key and count
    stays in range; the IQ matches the FP64 oracle."""
    from openbcsim_gb300 import workloads as W

    job = W.volume_3d_lut(num_scatterers=30_000_000, n_az=4, n_el=2)
    iq = run(job)
    assert np.isfinite(iq).all()
    assert oracle.rel_rms(iq, oracle.simulate(job, oracle.MODE_FP64)) <= FP64_TOL


def test_many_lines(oracle):
    """128 x 128 = 16384 lines (sixteen 1024-line groups per record chunk):
    lines from the first, a middle and the last group match the FP64 oracle."""
    from openbcsim_gb300 import workloads as W

    job = W.volume_3d_lut(num_scatterers=200_000, n_az=128, n_el=128)
    iq = run(job)
    assert iq.shape[0] == 16384 and np.isfinite(iq).all()
    for lo in (0, 8190, 16380):
        ref = oracle.simulate(job, oracle.MODE_FP64, line_begin=lo, line_end=lo + 4)
        assert oracle.rel_rms(iq[lo:lo + 4], ref) <= FP64_TOL, lo


@pytest.mark.parametrize("name", ["sector_pd", "sector_nopd", "lut3d", "edge", "spline", "linear"])
def test_culling_is_exact(name):
    """Skipping (scatterer, line-slot) pairs whose weight is provably zero
    changes no bit of the output."""
    job, _ = load_golden(name)
    a = run(job, cull="on")
    b = run(job, cull="off")
    assert np.array_equal(a, b)


def test_culling_is_exact_full_volume():
    from openbcsim_gb300 import workloads as W

    job = W.volume_3d_lut(num_scatterers=300_000, n_az=48, n_el=40)
    assert np.array_equal(run(job, cull="on"), run(job, cull="off"))


@pytest.mark.parametrize("beam", ["lut", "gaussian"])
def test_word_test_is_exact(oracle, beam):
    """Dense phantoms (at least 64 records per bin): the records of a bin are
    ordered by the angular cell of their direction, and each slot first tests
    whole 32-record words by their bounding spheres.  A word the test skips
    holds no pair of non-zero weight: culling on and off are bit-identical,
    and the IQ matches the FP64 oracle."""
    from openbcsim_gb300 import workloads as W

    if beam == "lut":
        job = W.volume_3d_lut(num_scatterers=700_000, n_az=40, n_el=24)
    else:
        job = W.sector_2d_fixed(num_scatterers=600_000, num_lines=128)
    assert job.num_scatterers >= 64 * job.num_samples   # the angular order and the word test are on
    on = run(job, cull="on")
    assert np.array_equal(on, run(job, cull="off"))
    L = job.scan.num_lines
    for lo in (0, L // 2, L - 3):
        ref = oracle.simulate(job, oracle.MODE_FP64, line_begin=lo, line_end=lo + 3)
        assert oracle.rel_rms(on[lo:lo + 3], ref) <= FP64_TOL


@pytest.mark.parametrize("num_scatterers,lut_shape", [(300_000, (256, 64, 64)),   # dense: chunks within 1-2 planes
                                                      (20_000, (256, 64, 64)),    # sparse: chunks span many planes
                                                      (100_000, (64, 96, 80))])   # one staged plane fits
def test_lut_planes_in_shared_memory_are_exact(oracle, num_scatterers, lut_shape):
    """The wide shared-origin kernel reads the chunk's lookup-table planes from
    shared memory (records beyond them from the cache): the output is
    bit-identical to reading every corner through the cache, and to the
    256-thread kernel."""
    from openbcsim_gb300 import workloads as W

    job = W.volume_3d_lut(num_scatterers=num_scatterers, n_az=40, n_el=32, lut_shape=lut_shape)
    staged = run(job, lut_smem="on")
    assert np.array_equal(staged, run(job, lut_smem="off"))
    assert np.array_equal(staged, run(job, wide_cta="off"))
    ref = oracle.simulate(job, oracle.MODE_FP64, line_begin=600, line_end=604)
    assert oracle.rel_rms(staged[600:604], ref) <= FP64_TOL


def test_spline_lines_at_random_times(oracle):
    """Lines with their own random timestamps over every knot interval: a tile of
    lines spans several intervals (the control-point window of the tile); each
    line's IQ matches the FP64 oracle and does not depend on how the lines are
    ordered (tiles differ, results are bit-identical)."""
    from openbcsim_gb300 import workloads as W

    rng = np.random.default_rng(77)
    sp = W.random_spline(rng, 20_000, 24)
    t0, t1 = W.spline_time_limits(sp.degree, sp.knots, 24)
    L = 200
    ts = rng.uniform(t0, t1, L).astype(np.float32)
    scan = W.sector_scan(L, 35.0, 0.12, timestamps=ts, angles_deg=rng.uniform(-35.0, 35.0, L))
    job = W._excitation_job("spline_random_times", scan, 2.5e6, 0.1, W.GaussianBeam(1e-3, 1e-3), [], [sp], 8)
    iq = run(job)
    for lo in (0, 97, 196):
        ref = oracle.simulate(job, oracle.MODE_FP64, line_begin=lo, line_end=lo + 4)
        assert oracle.rel_rms(iq[lo:lo + 4], ref) <= FP64_TOL
    perm = rng.permutation(L)
    s = job.scan
    job.scan = type(s)(s.origins[perm], s.directions[perm], s.lateral_dirs[perm], s.timestamps[perm], s.line_length)
    assert np.array_equal(run(job), iq[perm])
    # the per-tile culling (control-point boxes) changes no bit
    assert np.array_equal(run(job, cull="off"), iq[perm])


def test_new_frame_same_shape_matches_fresh_simulator():
    """Replacing the scatterers by others of the same count (a new frame) reuses
    the simulator's plan but for the fixed-point scale and the records: the IQ
    equals that of a simulator configured from scratch with the new frame."""
    from openbcsim_gb300 import workloads as W

    job = W.volume_3d_lut(num_scatterers=50_000, n_az=32, n_el=24)
    sim = engine(job)
    sim.simulate_lines_line_major()
    rng = np.random.default_rng(9)
    for frame in (job.fixed[0].xyza * np.array([1, 1, 1, 2], np.float32),          # scale changes
                  W.random_fixed(rng, 50_000, (-0.03, 0.03), (-0.03, 0.03), (0.01, 0.12)).xyza):
        sim.clear_fixed_scatterers()
        sim.add_fixed_scatterers(frame)
        a = sim.simulate_lines_line_major().copy()
        job.fixed = [W.FixedSet(frame)]
        assert np.array_equal(a, run(job))


def test_pair_counting_run():
    """The instrumented shared-origin kernel gives the same IQ and counts
    0 < non-zero-weight pairs <= visited pairs <= N x L; kernel launches are
    reported per simulation."""
    from openbcsim_gb300 import workloads as W

    job = W.volume_3d_lut(num_scatterers=100_000, n_az=40, n_el=32)
    sim = engine(job)
    a = sim.simulate_lines_line_major().copy()
    assert sim.get_debug_data("kernel_launches")[0] >= 7
    sim.set_parameter("count_pairs", "on")
    b = sim.simulate_lines_line_major().copy()
    visited = sim.get_debug_data("evaluated_pairs")[0]
    nonzero = sim.get_debug_data("weighted_pairs")[0]
    assert np.array_equal(a, b)
    assert 0 < nonzero <= visited <= job.num_scatterers * job.scan.num_lines
