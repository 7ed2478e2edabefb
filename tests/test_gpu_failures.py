"""Failure detection without a device fault.

The engine's kernels wait for their asynchronous copies with bounded waits; a
wait that gives up sets the simulator's device error flag and returns, and the
host turns the flag into an error at its next synchronisation.  These tests
raise that flag from the host (bcsim_debug_raise_wait_flag, as such a wait
would) and check that every synchronising entry point reports it, clears it and
works again, bit for bit.  The request server is driven through malformed
requests, an injected worker exception, an injected wait failure and refusals
by its device-memory admission; the other requests of the stream must complete
unchanged and `failed` must count the bad ones.  Nothing here faults, traps or
hangs a GPU.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

E_INVALID, E_MEMORY, E_INTERNAL = 1, 5, 6
WAIT_MSG = "a bounded device wait gave up; results are incomplete"


def sim_for(job, **params):
    import openbcsim_gb300 as gb

    s = gb.RfSimulator("gpu")
    gb.configure_job(s, job)
    for k, v in params.items():
        s.set_parameter(k, v)
    return s


def _expect(code, msg, fn):
    import openbcsim_gb300 as gb

    with pytest.raises(gb.SimulatorError) as ei:
        fn()
    assert ei.value.code == code, ei.value
    assert msg in str(ei.value)


def test_wait_failure_fails_simulate_lines_and_clears():
    from openbcsim_gb300 import workloads as W

    # the shared-origin kernel (the one with the bounded wait) runs on this workload
    job = W.volume_3d_lut(num_scatterers=30_000, n_az=8, n_el=8, seed=31, lut_shape=(64, 32, 32))
    s = sim_for(job)
    a = s.simulate_lines_line_major().copy()
    s.debug_raise_wait_flag()
    _expect(E_INTERNAL, WAIT_MSG, s.simulate_lines_line_major)
    # the flag was cleared by the report: the next call succeeds, unchanged
    assert np.array_equal(s.simulate_lines_line_major(), a)


def test_wait_failure_fails_frames_batch_and_packet():
    import openbcsim_gb300 as gb
    from openbcsim_gb300 import workloads as W

    job = W.sector_2d_fixed(num_scatterers=20_000, num_lines=16, seed=32)
    s = sim_for(job)
    a = s.simulate_lines_line_major().copy()
    frames = [job.fixed[0].xyza, job.fixed[0].xyza]
    s.debug_raise_wait_flag()
    _expect(E_INTERNAL, WAIT_MSG, lambda: s.simulate_fixed_frames(frames))
    outs = s.simulate_fixed_frames(frames)
    assert all(np.array_equal(o, a) for o in outs)

    other = sim_for(W.sector_spline(num_scatterers=5_000, num_lines=8, seed=33))
    b = other.simulate_lines_line_major().copy()
    batch = gb.Batch([s, other])
    other.debug_raise_wait_flag()
    _expect(E_INTERNAL, WAIT_MSG, batch.run)
    for _ in range(2):
        o1, o2 = batch.run()
        assert np.array_equal(o1, a) and np.array_equal(o2, b)

    s.debug_raise_wait_flag()
    _expect(E_INTERNAL, WAIT_MSG, lambda: s.simulate_packet(2, 1e-4))
    p = s.simulate_packet(2, 1e-4)
    assert np.array_equal(p[0], a) and np.array_equal(p[1], a)


def _requests(W, rng, jobs, n):
    reqs = []
    for _ in range(n):
        k = int(rng.integers(0, len(jobs)))
        L = int(rng.integers(1, 24))
        ts = np.sort(rng.uniform(0.0, 0.99, L)).astype(np.float32)
        scan = W.sector_scan(L, 35.0, jobs[k].scan.line_length, timestamps=ts, angles_deg=rng.uniform(-35, 35, L))
        reqs.append((k, scan, int(rng.integers(4, 17))))
    return reqs


def _submit(server, pids, k, scan, D):
    return server.submit(pids[k], scan.origins, scan.directions, scan.line_length, scan.lateral_dirs,
                         scan.timestamps, D)


def _alone(job, scan, D):
    s = sim_for(job, radial_decimation=str(D))
    s.set_scan_sequence(scan.origins, scan.directions, scan.line_length, scan.lateral_dirs, scan.timestamps)
    return s.simulate_lines_line_major()


def test_server_isolates_failed_requests():
    import openbcsim_gb300 as gb
    from openbcsim_gb300 import workloads as W

    jobs = [W.sector_2d_fixed(num_scatterers=30_000, num_lines=8, seed=34),
            W.sector_spline(num_scatterers=10_000, num_lines=8, seed=35)]
    server = gb.Server(hbm_budget_bytes=8 << 30, max_slots_per_phantom=2)
    pids = [server.add_phantom(sim_for(j)) for j in jobs]
    rng = np.random.default_rng(36)
    good = _requests(W, rng, jobs, 12)
    ids, results = [], {}
    expect_fail = {}

    def drain():
        # the injections act on the worker's next dispatch: let every earlier
        # request finish first, so that the next one dispatched is the target
        for r in ids:
            if r not in results:
                results[r] = server.wait(r)[0]

    for i, (k, scan, D) in enumerate(good):
        ids.append(_submit(server, pids, k, scan, D))
        if i == 2:
            # not orthonormal: the reference's Scanline check (ScanSequence.cpp:37-70)
            bad = W.sector_scan(3, 35.0, 0.12)
            rid = server.submit(pids[0], bad.origins, bad.directions * 1.5, 0.12, bad.lateral_dirs,
                                bad.timestamps, 8)
            expect_fail[rid] = (E_INVALID, "Invalid Scanline")
        if i == 5:
            # a spline timestamp past the knot vector (bspline.hpp:74-82)
            bad = W.sector_scan(2, 35.0, 0.12, timestamps=np.array([0.5, 7.0], np.float32))
            rid = server.submit(pids[1], bad.origins, bad.directions, 0.12, bad.lateral_dirs, bad.timestamps, 8)
            expect_fail[rid] = (E_INVALID, "knot interval")
        if i == 7:
            drain()
            server.debug_inject(server.INJECT_WORKER_THROW)
            rid = _submit(server, pids, k, scan, D)
            expect_fail[rid] = (E_INTERNAL, "injected worker failure")
        if i == 9:
            drain()
            server.debug_inject(server.INJECT_WAIT_FLAG)
            rid = _submit(server, pids, k, scan, D)
            expect_fail[rid] = (E_INTERNAL, WAIT_MSG)
    for rid, (code, msg) in expect_fail.items():
        with pytest.raises(gb.SimulatorError) as ei:
            server.wait(rid)
        assert ei.value.code == code and msg in str(ei.value), ei.value
    drain()
    results = [results[r] for r in ids]
    st = server.stats()
    assert st["completed"] == len(good) and st["failed"] == len(expect_fail)
    server.close()
    for (k, scan, D), got in zip(good, results):
        assert np.array_equal(got, _alone(jobs[k], scan, D))


def test_server_admission_by_device_memory():
    import openbcsim_gb300 as gb
    from openbcsim_gb300 import workloads as W

    job = W.sector_2d_fixed(num_scatterers=30_000, num_lines=8, seed=37)
    scan = W.sector_scan(64, 35.0, 0.12)
    # a request whose footprint exceeds the whole budget is refused
    small = gb.Server(hbm_budget_bytes=1 << 20, max_slots_per_phantom=1)
    pid = small.add_phantom(sim_for(job))
    rid = small.submit(pid, scan.origins, scan.directions, 0.12, scan.lateral_dirs, scan.timestamps, 8)
    with pytest.raises(gb.SimulatorError) as ei:
        small.wait(rid)
    assert ei.value.code == E_MEMORY and "budget" in str(ei.value)
    small.close()

    server = gb.Server(hbm_budget_bytes=8 << 30, max_slots_per_phantom=1)
    pid = server.add_phantom(sim_for(job))
    # no device memory available to grow the slot, nothing in flight: refused
    server.debug_inject(server.INJECT_FREE_MEMORY_CAP, 0)
    rid = server.submit(pid, scan.origins, scan.directions, 0.12, scan.lateral_dirs, scan.timestamps, 8)
    with pytest.raises(gb.SimulatorError) as ei:
        server.wait(rid)
    assert ei.value.code == E_MEMORY and "available" in str(ei.value)
    # with the memory back, the same request is served, as alone
    server.debug_inject(server.INJECT_FREE_MEMORY_CAP, -1)
    rid = server.submit(pid, scan.origins, scan.directions, 0.12, scan.lateral_dirs, scan.timestamps, 8)
    got = server.wait(rid)[0]
    # a request that fits the slot as it has grown needs no more memory: served under a zero cap
    server.debug_inject(server.INJECT_FREE_MEMORY_CAP, 0)
    rid = server.submit(pid, scan.origins[:16], scan.directions[:16], 0.12, scan.lateral_dirs[:16],
                        scan.timestamps[:16], 8)
    got16 = server.wait(rid)[0]
    st = server.stats()
    assert st["completed"] == 2 and st["failed"] == 1
    server.close()
    assert np.array_equal(got, _alone(job, scan, 8))
    sub = W.ScanSequence(scan.origins[:16], scan.directions[:16], scan.lateral_dirs[:16], scan.timestamps[:16], 0.12)
    assert np.array_equal(got16, _alone(job, sub, 8))
