"""Batched and served simulation give the same IQ as plain simulate_lines,
bit for bit (deterministic fixed-point accumulation; per-job configuration)."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def sim_for(job, **params):
    import openbcsim_gb300 as gb

    s = gb.RfSimulator("gpu")
    gb.configure_job(s, job)
    for k, v in params.items():
        s.set_parameter(k, v)
    return s


def test_batch_equals_plain():
    import openbcsim_gb300 as gb

    jobs = [load_golden(n)[0] for n in ["sector_pd", "lut3d", "spline", "linear", "edge"]]
    plain = [sim_for(j).simulate_lines_line_major().copy() for j in jobs]
    sims = [sim_for(j) for j in jobs]
    for use_graph in (False, True):
        batch = gb.Batch(sims, use_graph=use_graph)
        for _ in range(3):                     # first run direct, then captured graph replays
            outs = batch.run()
            for a, b in zip(outs, plain):
                assert np.array_equal(a, b)


def test_batch_uneven_workload_vs_oracle(oracle):
    import openbcsim_gb300 as gb
    from openbcsim_gb300 import workloads as W

    jobs = W.batch_uneven(num_jobs=12, scale=0.02)
    sims = [sim_for(j) for j in jobs]
    outs = gb.Batch(sims).run()
    for j, o in zip(jobs, outs):
        ref = oracle.simulate(j, oracle.MODE_FP64, line_begin=0, line_end=j.scan.num_lines)
        assert oracle.rel_rms(o, ref) <= 1e-4, j.name


def test_autotune_changes_time_not_results():
    from openbcsim_gb300 import workloads as W

    job = W.volume_3d_lut(num_scatterers=200_000, n_az=24, n_el=16)
    a = sim_for(job).simulate_lines_line_major()
    b = sim_for(job, autotune="on").simulate_lines_line_major()
    c = sim_for(job, tile_lines="4096").simulate_lines_line_major()
    assert np.array_equal(a, b) and np.array_equal(a, c)


def test_record_cache_reuse_and_invalidation():
    job, _ = load_golden("lut3d")
    s = sim_for(job)
    a = s.simulate_lines_line_major().copy()
    b = s.simulate_lines_line_major().copy()         # records reused
    assert np.array_equal(a, b)
    xyza = job.fixed[0].xyza.copy()
    xyza[:, 3] *= -1
    s.clear_fixed_scatterers()
    s.add_fixed_scatterers(xyza)                     # records rebuilt
    c = s.simulate_lines_line_major()
    assert np.array_equal(c, -a)


def test_server_same_alone_and_in_the_mix():
    import openbcsim_gb300 as gb
    from openbcsim_gb300 import workloads as W

    fixed = W.sector_2d_fixed(num_scatterers=50_000, num_lines=8, seed=77)
    spline = W.sector_spline(num_scatterers=20_000, num_lines=8, seed=78)
    lut = W.volume_3d_lut(num_scatterers=100_000, n_az=4, n_el=2, seed=79, lut_shape=(64, 32, 32))
    server = gb.Server(hbm_budget_bytes=8 << 30, max_slots_per_phantom=3)
    jobs = [fixed, spline, lut]
    pids = [server.add_phantom(sim_for(j)) for j in jobs]
    rng = np.random.default_rng(5)
    reqs = []
    for i in range(30):
        k = int(rng.integers(0, 3))
        j = jobs[k]
        L = int(rng.integers(1, 48))
        if k == 2:
            scan = W.volume_scan(L, 1, 30.0, 30.0, j.scan.line_length)
        else:
            ts = np.sort(rng.uniform(0.0, 0.99, L)).astype(np.float32)
            scan = W.sector_scan(L, 35.0, j.scan.line_length, timestamps=ts,
                                 angles_deg=rng.uniform(-35, 35, L))
        D = int(rng.integers(4, 17))
        rid = server.submit(pids[k], scan.origins, scan.directions, scan.line_length, scan.lateral_dirs,
                            scan.timestamps, D)
        reqs.append((rid, k, scan, D))
    results = {rid: server.wait(rid)[0] for rid, *_ in reqs}
    st = server.stats()
    assert st["completed"] == 30 and st["failed"] == 0 and st["p99_ms"] >= st["p50_ms"] > 0
    server.close()
    for rid, k, scan, D in reqs:
        alone = sim_for(jobs[k], radial_decimation=str(D))
        alone.set_scan_sequence(scan.origins, scan.directions, scan.line_length, scan.lateral_dirs, scan.timestamps)
        assert np.array_equal(results[rid], alone.simulate_lines_line_major()), (rid, k)
