// noalloc.cu -- an allocation-free simulation entry point.
//
// Some callers cannot call cudaMalloc at all: real-time imaging pipelines that
// reserve every byte of device memory once at start-up and forbid allocation
// afterwards, processes whose device memory is owned by another framework's
// pool, and code that runs where a driver allocation would stall or fail (for
// example inside a tightly budgeted streaming loop).  bcsim_simulate_fixed_noalloc
// serves them: the caller passes its scatterers and its output buffer in device
// memory, and every intermediate (the time-projection bins, the line table, the
// FIR taps and the demodulation factors) lives in one file-scope static device
// array of fixed size, g_noalloc_scratch below.  Nothing is allocated on the
// device, and the host side uses only static buffers.
//
// Rules that come with a shared static array:
//  * every GPU that loads this library holds the array (NA_TOTAL bytes, about 31.3 MiB)
//    until the process exits;
//  * the first call on each device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call before
//    any stream capture;
//  * all calls share the array and it keeps the last call's contents: the bins
//    are cleared at the start of every call, and calls whose work overlaps on the
//    GPU (different streams, or different host threads) race on it -- serialise
//    them on one stream;
//  * sizes beyond the stated maxima are rejected with an error message;
//  * the call is synchronous: it returns once the IQ is in the caller's buffer.
//
// The amplitudes are checked on the device before anything is projected: a
// non-finite amplitude fails the call with the allocating path's message
// ("Nan in scatterer projection."), and so does an amplitude_sum_bound below
// the measured sum of |a| (the bound sets the fixed-point scale of the bins; an
// understated one could overflow them).  That reduction keeps its partial sums
// in its own region of the static array.
#include <cuda_runtime.h>

#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/bcsim_gb300.h"
#include "host_dsp.hpp"
#include "kernels.hpp"

namespace bcsim_gb300 {

// Layout of the static scratch (byte offsets).
constexpr size_t NA_BINS_BYTES = (size_t)30 << 20;              // int64 bins
constexpr size_t NA_LINES_OFF = NA_BINS_BYTES;                   // LineGeom [4096]
constexpr int NA_MAX_LINES = 4096;
constexpr size_t NA_IDS_OFF = NA_LINES_OFF + NA_MAX_LINES * sizeof(LineGeom);
constexpr size_t NA_TILES_OFF = NA_IDS_OFF + NA_MAX_LINES * sizeof(int);
constexpr size_t NA_TAPS_OFF = NA_TILES_OFF + NA_MAX_LINES * sizeof(LineTile);
constexpr int NA_MAX_TAPS = 32768;
constexpr int NA_MAX_DEC = 1024;                                 // radial decimation
constexpr size_t NA_PM_OFF = NA_TAPS_OFF + NA_MAX_TAPS * sizeof(float2);              // phase-major taps
constexpr size_t NA_PHOFF_OFF = NA_PM_OFF + (NA_MAX_TAPS + 4 * NA_MAX_DEC) * sizeof(float2);  // phase offsets
constexpr size_t NA_DEMOD_OFF = NA_PHOFF_OFF + 4096 * sizeof(int);
static_assert(3 * NA_MAX_DEC + 1 <= 4096, "phase table fits its region");
constexpr int NA_MAX_OUT = 65536;                                // decimated samples per line
constexpr size_t NA_SUM_OFF = NA_DEMOD_OFF + NA_MAX_OUT * sizeof(float2);   // amplitude reduction
constexpr size_t NA_SUM_BYTES = 8192;
constexpr size_t NA_TOTAL = NA_SUM_OFF + NA_SUM_BYTES;
constexpr int NA_MAX_FFT = 65536;                                // convolution length M

static_assert(NA_TOTAL % 256 == 0, "scratch regions stay 256-byte aligned");

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_TOTAL];

namespace {

std::mutex g_na_mutex;
void* g_na_ptr[64];          // device address of the scratch, per device (set-up once)

// host-side static buffers (no heap allocation per call)
std::complex<double> g_fft[NA_MAX_FFT];
double g_energy[NA_MAX_FFT];
float2 g_taps[NA_MAX_TAPS];
float2 g_taps_pm[NA_MAX_TAPS + 4 * NA_MAX_DEC];
int g_ph_off[3 * NA_MAX_DEC + 1];
float2 g_demod[NA_MAX_OUT];
LineGeom g_lines[NA_MAX_LINES];
int g_ids[NA_MAX_LINES];
LineTile g_tiles[NA_MAX_LINES];
double g_amp_sum;
int g_amp_nonfinite;

void fft_inplace(std::complex<double>* x, int64_t n, int sign) {
    for (int64_t i = 1, j = 0; i < n; i++) {
        int64_t bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(x[i], x[j]);
    }
    for (int64_t len = 2; len <= n; len <<= 1) {
        const int64_t half = len >> 1;
        const double ang = sign * 6.283185307179586 / (double)len;
        for (int64_t k = 0; k < half; k++) {
            const std::complex<double> w(std::cos(ang * k), std::sin(ang * k));
            for (int64_t s = 0; s < n; s += len) {
                const std::complex<double> v = x[s + k + half] * w;
                x[s + k + half] = x[s + k] - v;
                x[s + k] += v;
            }
        }
    }
}

int fail(char* err, int cap, int code, const char* msg) {
    if (err && cap > 0) std::snprintf(err, (size_t)cap, "%s", msg);
    return code;
}

}  // namespace
}  // namespace bcsim_gb300

using namespace bcsim_gb300;

extern "C" int bcsim_simulate_fixed_noalloc(const void* d_xyza, int64_t n, const float* origins,
                                            const float* directions, const float* lateral_dirs, int num_lines,
                                            float line_length, float sound_speed, const float* taps, int num_taps,
                                            int center_index, float fs, float demod_freq, float sigma_lateral,
                                            float sigma_elevational, int use_arc_projection, int phase_delay,
                                            int radial_decimation, float amplitude_sum_bound, void* d_out,
                                            int64_t cap_complex, void* stream, char* err, int err_cap) {
    if (err && err_cap > 0) err[0] = 0;
    if ((n > 0 && !d_xyza) || n < 0 || !origins || !directions || !lateral_dirs || !taps || !d_out)
        return fail(err, err_cap, BCSIM_E_INVALID, "null or negative argument");
    if (num_lines < 1 || num_lines > NA_MAX_LINES)
        return fail(err, err_cap, BCSIM_E_CAPACITY, "num_lines must be in [1, 4096] for the allocation-free entry point");
    if (radial_decimation < 1) return fail(err, err_cap, BCSIM_E_INVALID, "illegal radial decimation value");
    if (radial_decimation > NA_MAX_DEC)
        return fail(err, err_cap, BCSIM_E_CAPACITY, "radial decimation above 1024 for the allocation-free entry point");
    if (!(sound_speed > 0) || !std::isfinite(sound_speed)) return fail(err, err_cap, BCSIM_E_INVALID, "illegal sound speed");
    if (!(fs > 0) || !std::isfinite(fs)) return fail(err, err_cap, BCSIM_E_INVALID, "sampling frequency must be positive and finite");
    if (!std::isfinite(line_length)) return fail(err, err_cap, BCSIM_E_INVALID, "line length must be finite");
    if (!std::isfinite(demod_freq)) return fail(err, err_cap, BCSIM_E_INVALID, "demodulation frequency must be finite");
    if (!(sigma_lateral > 0) || !std::isfinite(sigma_lateral) || !(sigma_elevational > 0) ||
        !std::isfinite(sigma_elevational))
        return fail(err, err_cap, BCSIM_E_INVALID, "beam sigmas must be positive and finite");
    if (num_taps < 1) return fail(err, err_cap, BCSIM_E_INVALID, "excitation has no samples");
    if (!(amplitude_sum_bound >= 0.0f) || !std::isfinite(amplitude_sum_bound))
        return fail(err, err_cap, BCSIM_E_INVALID, "amplitude_sum_bound must be a finite upper bound of sum |a|");
    const int64_t ns = num_rf_samples(sound_speed, line_length, fs);
    if (ns <= 0) return fail(err, err_cap, BCSIM_E_INVALID, "line length gives no RF samples");
    const int stride = phase_delay ? 2 : 1;
    if ((size_t)num_lines * (size_t)ns * stride * sizeof(unsigned long long) > NA_BINS_BYTES)
        return fail(err, err_cap, BCSIM_E_CAPACITY,
                    "num_lines x samples per line exceeds the allocation-free scratch "
                    "(30 MiB of bins: lines * ns * (phase_delay ? 2 : 1) <= 3932160)");
    const int64_t M = next_power_of_two(ns + num_taps - 1);
    if (M > NA_MAX_FFT) return fail(err, err_cap, BCSIM_E_CAPACITY, "samples + excitation length exceed 65536");
    const int64_t nd = (ns + radial_decimation - 1) / radial_decimation;
    if (nd > NA_MAX_OUT) return fail(err, err_cap, BCSIM_E_CAPACITY, "more than 65536 output samples per line");
    if (cap_complex < (int64_t)num_lines * nd) return fail(err, err_cap, BCSIM_E_CAPACITY, "output buffer too small");
    if (center_index < 0 || (int64_t)center_index + (nd - 1) * radial_decimation >= M)
        return fail(err, err_cap, BCSIM_E_INVALID, "excitation center index outside the convolution buffer");

    std::lock_guard<std::mutex> lock(g_na_mutex);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
        return fail(err, err_cap, BCSIM_E_CUDA, "no current CUDA device");
    if (!g_na_ptr[dev]) {
        // one-time set-up on this device: the device address of the static array
        void* ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) return fail(err, err_cap, BCSIM_E_CUDA, cudaGetErrorString(e));
        g_na_ptr[dev] = ptr;
    }
    unsigned char* base = static_cast<unsigned char*>(g_na_ptr[dev]);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the scatterers and the output must be device (or managed) memory of this
    // device: a host pointer would fault inside the kernels
    {
        const void* ptrs[2] = {n > 0 ? d_xyza : nullptr, d_out};
        const char* names[2] = {"d_xyza", "d_out"};
        for (int k = 0; k < 2; k++) {
            if (!ptrs[k]) continue;
            cudaPointerAttributes at;
            const cudaError_t pe = cudaPointerGetAttributes(&at, ptrs[k]);
            if (pe != cudaSuccess) {
                cudaGetLastError();
                return fail(err, err_cap, BCSIM_E_INVALID, k == 0 ? "d_xyza is not a device pointer" : "d_out is not a device pointer");
            }
            const bool ok = at.type == cudaMemoryTypeManaged || (at.type == cudaMemoryTypeDevice && at.device == dev);
            if (!ok) {
                char msg[128];
                std::snprintf(msg, sizeof msg, "%s is not device memory of the current device", names[k]);
                return fail(err, err_cap, BCSIM_E_INVALID, msg);
            }
        }
    }
    // amplitudes: finite, and their sum of |a| within the caller's bound (the
    // 0.1 % margin of the fixed-point scale below covers the bound's rounding
    // to float); checked before anything is written
    if (n > 0) {
        if (abs_sum_scratch_bytes() > NA_SUM_BYTES)
            return fail(err, err_cap, BCSIM_E_INTERNAL, "amplitude reduction scratch too small");
        cudaError_t se = abs_sum_enqueue(static_cast<const float*>(d_xyza) + 3, 4, n, base + NA_SUM_OFF, &g_amp_sum,
                                         &g_amp_nonfinite, st);
        if (se == cudaSuccess) se = cudaStreamSynchronize(st);
        if (se != cudaSuccess) return fail(err, err_cap, BCSIM_E_CUDA, cudaGetErrorString(se));
        if (g_amp_nonfinite) return fail(err, err_cap, BCSIM_E_INVALID, "Nan in scatterer projection.");
        if (g_amp_sum > (double)amplitude_sum_bound * 1.001)
            return fail(err, err_cap, BCSIM_E_INVALID, "amplitude_sum_bound is below the sum of |amplitude| of the scatterers");
    }

    // line table (elevational = lateral x direction, ScanSequence.cpp:40), identity order, tiles
    for (int i = 0; i < num_lines; i++) {
        LineGeom& g = g_lines[i];
        for (int k = 0; k < 3; k++) {
            g.o[k] = origins[3 * i + k];
            g.d[k] = directions[3 * i + k];
            g.l[k] = lateral_dirs[3 * i + k];
        }
        g.e[0] = g.l[1] * g.d[2] - g.d[1] * g.l[2];
        g.e[1] = g.d[0] * g.l[2] - g.l[0] * g.d[2];
        g.e[2] = g.l[0] * g.d[1] - g.d[0] * g.l[1];
        g_ids[i] = i;
    }
    int num_tiles = 0;
    for (int i = 0; i < num_lines; i += PAIR_THREADS) {
        LineTile t;
        t.first = i;
        t.count = num_lines - i < PAIR_THREADS ? num_lines - i : PAIR_THREADS;
        t.mu = 0;
        t.span = 1;
        g_tiles[num_tiles++] = t;
    }

    // analytic pulse, FIR window (all but 1e-10 of the energy), demodulation
    for (int64_t i = 0; i < M; i++) g_fft[i] = i < num_taps ? std::complex<double>(taps[i], 0.0) : 0.0;
    fft_inplace(g_fft, M, -1);
    for (int64_t i = 0; i < M; i++) {
        const double k = (i == 0 || i == M / 2) ? 1.0 : (i < M / 2 ? 2.0 : 0.0);
        g_fft[i] *= k;
    }
    fft_inplace(g_fft, M, +1);
    double total = 0.0;
    for (int64_t i = 0; i < M; i++) {
        g_fft[i] /= (double)M;
        g_energy[i] = std::norm(g_fft[i]);
        total += g_energy[i];
    }
    int64_t a = 0, bnd = num_taps < M ? num_taps : M;
    double inside = 0.0;
    for (int64_t i = 0; i < bnd; i++) inside += g_energy[i];
    while (bnd - a < M && (total - inside) > 1e-10 * total) {
        const double left = g_energy[((a - 1) % M + M) % M], right = g_energy[bnd % M];
        if (left >= right) { a--; inside += left; } else { inside += right; bnd++; }
    }
    if (bnd - a >= M) { a = 0; bnd = M; }
    const int64_t W = bnd - a;
    if (W > NA_MAX_TAPS) return fail(err, err_cap, BCSIM_E_CAPACITY, "FIR window longer than 32768 taps");
    for (int64_t w = 0; w < W; w++) {
        const std::complex<double> h = g_fft[((a + w) % M + M) % M];
        g_taps[w] = make_float2((float)h.real(), (float)h.imag());
    }
    int max_ph = 0;
    const int n_pm = make_phase_major_taps(g_taps, (int)W, radial_decimation, g_taps_pm, g_ph_off, &max_ph);
    const double nf = (double)demod_freq / (double)fs;
    for (int64_t m = 0; m < nd; m++) {
        const double ph = -6.283185307179586 * nf * (double)(m * radial_decimation);
        g_demod[m] = make_float2((float)std::cos(ph), (float)std::sin(ph));
    }

    // parameters
    SimParams p;
    std::memset(&p, 0, sizeof(p));
    p.ns = (int)ns;
    p.num_lines = num_lines;
    p.phase_delay = phase_delay ? 1 : 0;
    p.arc = use_arc_projection ? 1 : 0;
    p.mode = MODE_FP64;
    p.fs = fs; p.c = sound_speed; p.fd = demod_freq;
    p.fs_d = fs; p.c_d = sound_speed; p.fd_d = demod_freq;
    const double kk = 2.0 * (double)fs / (double)sound_speed;
    p.k_hi = (float)kk;
    p.k_lo = (float)(kk - (double)p.k_hi);
    p.two_pi_fd_over_fs = (float)(6.283185307179586 * (double)demod_freq / (double)fs);
    int S = 0;
    if (amplitude_sum_bound > 0.0f) S = (int)std::floor(61.0 - std::log2((double)amplitude_sum_bound * 1.001));
    S = S < -100 ? -100 : (S > 100 ? 100 : S);
    p.log2scale = S;
    p.scale = std::ldexp(1.0f, S);
    BeamDev b;
    std::memset(&b, 0, sizeof(b));
    b.type = BEAM_GAUSSIAN;
    const double log2e = 1.4426950408889634;
    b.gl = (float)(log2e / (2.0 * (double)sigma_lateral * (double)sigma_lateral));
    b.ge = (float)(log2e / (2.0 * (double)sigma_elevational * (double)sigma_elevational));
    b.two_sl2 = 2 * sigma_lateral * sigma_lateral;
    b.two_se2 = 2 * sigma_elevational * sigma_elevational;

    // upload the tables into the scratch, clear the bins, run projection + FIR
    unsigned long long* bins = reinterpret_cast<unsigned long long*>(base);
    LineGeom* dl = reinterpret_cast<LineGeom*>(base + NA_LINES_OFF);
    int* dids = reinterpret_cast<int*>(base + NA_IDS_OFF);
    LineTile* dtiles = reinterpret_cast<LineTile*>(base + NA_TILES_OFF);
    float2* ddemod = reinterpret_cast<float2*>(base + NA_DEMOD_OFF);
    float2* dpm = reinterpret_cast<float2*>(base + NA_PM_OFF);
    int* dphoff = reinterpret_cast<int*>(base + NA_PHOFF_OFF);
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = cudaMemcpyAsync(dl, g_lines, num_lines * sizeof(LineGeom), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dids, g_ids, num_lines * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dtiles, g_tiles, num_tiles * sizeof(LineTile), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ddemod, g_demod, nd * sizeof(float2), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dpm, g_taps_pm, n_pm * sizeof(float2), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dphoff, g_ph_off, (3 * radial_decimation + 1) * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(bins, 0, (size_t)num_lines * ns * stride * sizeof(unsigned long long), st);
    if (e == cudaSuccess)
        e = launch_project_generic(static_cast<const float4*>(d_xyza), nullptr, nullptr, n, 0, 0, nullptr, nullptr, 0,
                                   dl, dids, dtiles, num_tiles, nullptr, p, b, bins, st);
    if (e == cudaSuccess)
        e = launch_convolve_demodulate(bins, num_lines, (int)ns, p.phase_delay, std::ldexp(1.0f, -S), dpm, dphoff,
                                       n_pm, max_ph, (int)W, (int)a, M, center_index, radial_decimation, (int)nd,
                                       ddemod, static_cast<float2*>(d_out), st);
    // the host tables above are reused by the next call: make sure they were consumed
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(err, err_cap, BCSIM_E_CUDA, cudaGetErrorString(e));
    return BCSIM_OK;
}
