// host_dsp.hpp -- host-side double-precision signal processing and B-spline
// helpers of the engine (excitation analytic taps, demodulation factors,
// knot intervals and basis values).
#pragma once
#include <complex>
#include <cstdint>
#include <vector>

namespace bcsim_gb300 {

// compute_num_rf_samples<float> (src/core/algorithm/common_utils.hpp:38-41).
int64_t num_rf_samples(float sound_speed, float line_length, float fs);

// next_power_of_two (src/core/fft.cpp:80-82).
int64_t next_power_of_two(int64_t n);

// In-place radix-2 FFT in double; sign -1 forward, +1 inverse (unscaled).
void fft_double(std::vector<std::complex<double>>& x, int sign);

// Analytic excitation spectrum FFT_M(taps) * hilbert_mask(M) (natural order).
std::vector<std::complex<double>> analytic_spectrum(const std::vector<float>& taps, int64_t M);

// Analytic excitation pulse h_a = IFFT(FFT_M(taps) * hilbert_mask(M))
// (src/core/BeamConvolver.cpp:77-91, src/core/discrete_hilbert_mask.hpp:36-66).
std::vector<std::complex<double>> analytic_pulse(const std::vector<float>& taps, int64_t M);

// Smallest circular window [start, start + count) of h_a around its main
// support [0, num_taps) holding all but `tail` of its energy.  count == M means
// the whole (exact) circular kernel.
void choose_tap_window(const std::vector<std::complex<double>>& ha, int num_taps, double tail, int64_t* start,
                       int64_t* count);

// Demodulation factor of decimated output m (sample i = m * D):
// fp64: exp(-j 2 pi (fd/fs) i) in double;
// reference: the float expression of CpuAlgorithm.cpp:353-358.
std::vector<std::complex<float>> demod_factors(float fd, float fs, int D, int64_t nd, bool reference_mode);

// B-spline helpers (src/core/bspline.hpp:44-91), double and float.
double bspline_basis_d(int j, int p, double x, const std::vector<float>& knots);
float bspline_basis_f(int j, int p, float x, const std::vector<float>& knots);
int knot_interval(const std::vector<float>& knots, float t);  // -1 where the reference throws

}  // namespace bcsim_gb300
