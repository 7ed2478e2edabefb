// host_dsp.cpp -- see host_dsp.hpp.
#include "host_dsp.hpp"

#include <cmath>

namespace bcsim_gb300 {

static const double kTwoPi = 6.283185307179586;

int64_t num_rf_samples(float sound_speed, float line_length, float fs) {
    // max_time is rounded to float and multiplied by fs in float, as the template
    // is instantiated with T = float by CpuAlgorithm::set_scan_sequence
    const float max_time = static_cast<float>(2.0 * line_length / sound_speed);
    const float prod = fs * max_time;
    return static_cast<int64_t>(std::floor(prod + 0.5));
}

int64_t next_power_of_two(int64_t n) {
    return static_cast<int64_t>(std::pow(2.0, std::ceil(std::log(static_cast<double>(n)) / std::log(2.0))));
}

void fft_double(std::vector<std::complex<double>>& x, int sign) {
    const size_t n = x.size();
    for (size_t i = 1, j = 0; i < n; i++) {
        size_t bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(x[i], x[j]);
    }
    for (size_t len = 2; len <= n; len <<= 1) {
        const size_t half = len >> 1;
        const double ang = sign * kTwoPi / static_cast<double>(len);
        for (size_t k = 0; k < half; k++) {
            const std::complex<double> w(std::cos(ang * k), std::sin(ang * k));
            for (size_t s = 0; s < n; s += len) {
                const std::complex<double> v = x[s + k + half] * w;
                x[s + k + half] = x[s + k] - v;
                x[s + k] += v;
            }
        }
    }
}

std::vector<std::complex<double>> analytic_spectrum(const std::vector<float>& taps, int64_t M) {
    std::vector<std::complex<double>> h(static_cast<size_t>(M), 0.0);
    for (size_t i = 0; i < taps.size() && static_cast<int64_t>(i) < M; i++) h[i] = taps[i];
    fft_double(h, -1);
    // discrete Hilbert mask: 1, 2 ... 2, (1), 0 ... 0
    for (int64_t i = 0; i < M; i++) {
        double k = 0.0;
        if (M % 2 == 0) {
            if (i == 0 || i == M / 2) k = 1.0;
            else if (i >= 1 && i <= M / 2 - 1) k = 2.0;
        } else {
            if (i == 0) k = 1.0;
            else if (i >= 1 && i < (M + 1) / 2) k = 2.0;
        }
        h[i] *= k;
    }
    return h;
}

std::vector<std::complex<double>> analytic_pulse(const std::vector<float>& taps, int64_t M) {
    std::vector<std::complex<double>> h = analytic_spectrum(taps, M);
    fft_double(h, +1);
    for (auto& v : h) v /= static_cast<double>(M);
    return h;
}

void choose_tap_window(const std::vector<std::complex<double>>& ha, int num_taps, double tail, int64_t* start,
                       int64_t* count) {
    const int64_t M = static_cast<int64_t>(ha.size());
    std::vector<double> e(static_cast<size_t>(M));
    double total = 0.0;
    for (int64_t i = 0; i < M; i++) {
        e[i] = std::norm(ha[i]);
        total += e[i];
    }
    const int64_t base = std::min<int64_t>(std::max(num_taps, 1), M);
    double inside = 0.0;
    for (int64_t i = 0; i < base; i++) inside += e[i];
    int64_t a = 0, b = base;  // window [a, b), circular; a may go negative
    // grow by one tap at a time on the side holding more energy
    while (b - a < M && (total - inside) > tail * total) {
        const double left = e[static_cast<size_t>(((a - 1) % M + M) % M)];
        const double right = e[static_cast<size_t>(b % M)];
        if (left >= right) {
            a -= 1;
            inside += left;
        } else {
            inside += right;
            b += 1;
        }
    }
    if (b - a >= M) {
        a = 0;
        b = M;
    }
    *start = a;
    *count = b - a;
}

std::vector<std::complex<float>> demod_factors(float fd, float fs, int D, int64_t nd, bool reference_mode) {
    std::vector<std::complex<float>> out(static_cast<size_t>(nd));
    if (!reference_mode) {
        const double nf = static_cast<double>(fd) / static_cast<double>(fs);
        for (int64_t m = 0; m < nd; m++) {
            const double ph = -kTwoPi * nf * static_cast<double>(m * D);
            out[m] = std::complex<float>(static_cast<float>(std::cos(ph)), static_cast<float>(std::sin(ph)));
        }
    } else {
        const float two_pi = static_cast<float>(2.0 * 4.0 * std::atan(1.0));
        const float nf = fd / fs;
        const float a = -two_pi * nf;
        for (int64_t m = 0; m < nd; m++) {
            const float arg = a * static_cast<float>(m * D);
            out[m] = std::complex<float>(std::cos(arg), std::sin(arg));
        }
    }
    return out;
}

static double special_div_d(double num, double den) {
    if (std::fabs(num) < 1e-6 && std::fabs(den) < 1e-6) return 0.0;
    return num / den;
}

static float special_div_f(float num, float den) {
    if (std::fabs(static_cast<double>(num)) < 1e-6 && std::fabs(static_cast<double>(den)) < 1e-6) return 0.0f;
    return num / den;
}

double bspline_basis_d(int j, int p, double x, const std::vector<float>& k) {
    if (p == 0) return (x >= static_cast<double>(k[j]) && x < static_cast<double>(k[j + 1])) ? 1.0 : 0.0;
    const double left = special_div_d((x - k[j]) * bspline_basis_d(j, p - 1, x, k),
                                      static_cast<double>(k[j + p]) - static_cast<double>(k[j]));
    const double right = special_div_d((static_cast<double>(k[j + 1 + p]) - x) * bspline_basis_d(j + 1, p - 1, x, k),
                                       static_cast<double>(k[j + 1 + p]) - static_cast<double>(k[j + 1]));
    return left + right;
}

float bspline_basis_f(int j, int p, float x, const std::vector<float>& k) {
    if (p == 0) return (x >= k[j] && x < k[j + 1]) ? 1.0f : 0.0f;
    const float left = special_div_f((x - k[j]) * bspline_basis_f(j, p - 1, x, k), k[j + p] - k[j]);
    const float right = special_div_f((k[j + 1 + p] - x) * bspline_basis_f(j + 1, p - 1, x, k), k[j + 1 + p] - k[j + 1]);
    return left + right;
}

int knot_interval(const std::vector<float>& knots, float t) {
    for (int i = 0; i + 1 < static_cast<int>(knots.size()); i++)
        if (t >= knots[i] && t < knots[i + 1]) return i;
    return -1;
}

}  // namespace bcsim_gb300
