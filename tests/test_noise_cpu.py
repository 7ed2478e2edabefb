"""The seeded noise of the time projection, on the CPU.

The reference adds complex Gaussian noise N(0, noise_amplitude) to every sample
of the time projection before the convolution (CpuAlgorithm.cpp:340-347, GPU
GpuAlgorithm.cpp:165-177,270-277), from an unseeded generator.  Here each
sample's noise is a pure function of (seed, frame, line, sample): a
Philox4x32-10 block turned into two normals by the Box-Muller transform.  These
tests pin the oracle's generator -- the checker of the GPU kernels' noise -- to
the published Philox known answers, and check the statistics the reference's
noise has: zero mean, unit variance per part, no correlation between parts,
lines or frames.
"""
import ctypes as C

import numpy as np


def test_philox_known_answers(oracle):
    """Known-answer vectors of Philox4x32-10 published with the algorithm
    (Random123): zero counter and key, all-ones, and the digits of pi."""
    lib = oracle.oracle_lib()
    cases = [((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
             ((0xffffffff,) * 4, (0xffffffff, 0xffffffff), (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
             ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
              (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]
    for ctr, key, expect in cases:
        c = (C.c_uint32 * 4)(*ctr)
        lib.oracle_philox4x32_10(c, key[0], key[1])
        assert tuple(c) == expect


def test_noise_statistics(oracle):
    n = 20000
    a = oracle.bin_noise(seed=12345, frame=0, line=3, count=n)
    b = oracle.bin_noise(seed=12345, frame=0, line=4, count=n)
    f = oracle.bin_noise(seed=12345, frame=1, line=3, count=n)
    s = oracle.bin_noise(seed=54321, frame=0, line=3, count=n)
    tol = 4.0 / np.sqrt(n)   # four standard errors
    for z in (a, b, f, s):
        assert abs(z.real.mean()) < tol and abs(z.imag.mean()) < tol
        assert abs(z.real.var() - 1.0) < 0.03 and abs(z.imag.var() - 1.0) < 0.03
        assert abs(np.corrcoef(z.real, z.imag)[0, 1]) < tol
        # Gaussian tails: about 0.27 % beyond 3 sigma
        assert 0.001 < np.mean(np.abs(z.real) > 3.0) < 0.0045
    for u, v in ((a, b), (a, f), (a, s)):   # other line, other frame, other seed
        assert abs(np.corrcoef(u.real, v.real)[0, 1]) < tol
        assert abs(np.corrcoef(u.imag, v.imag)[0, 1]) < tol
    # neighbouring samples of one line are uncorrelated too
    assert abs(np.corrcoef(a.real[1:], a.real[:-1])[0, 1]) < tol
    # a pure function of its key: drawn again, the same bits
    assert np.array_equal(a, oracle.bin_noise(seed=12345, frame=0, line=3, count=n))


def test_oracle_adds_noise_before_the_convolution(oracle):
    """The oracle's noisy frame equals the noiseless frame plus the convolution
    of the noise alone: the simulation is linear, the noise enters the
    time projection."""
    from openbcsim_gb300 import workloads as W

    job = W.sector_2d_fixed(num_scatterers=2000, num_lines=4, phase_delay=False, seed=61)
    clean = oracle.simulate(job)
    job.noise_amplitude, job.noise_seed = 0.5, 99
    noisy = oracle.simulate(job)
    assert not np.allclose(noisy, clean)
    # far from every scatterer's echo the output is the filtered noise alone,
    # of the order of sigma times the pulse's gain
    job2 = W.sector_2d_fixed(num_scatterers=1, num_lines=4, phase_delay=False, seed=61)
    job2.fixed[0].xyza[:] = [0.0, 0.0, 0.115, 1e-6]
    job2.noise_amplitude, job2.noise_seed = 0.5, 99
    only = oracle.simulate(job2)
    assert np.std(only[:, :200]) > 0.01
