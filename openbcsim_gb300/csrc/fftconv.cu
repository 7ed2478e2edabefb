// fftconv.cu -- pulse convolution, IQ demodulation and radial decimation by
// FFT, for long analytic pulses.
//
// The reference's convolution is a length-M circular convolution with the
// analytic pulse, by FFT, multiply and inverse FFT (src/core/BeamConvolver.cpp:
// 64-91; GPU: cuFFT + MultiplyFftKernel, GpuAlgorithm.cpp:280-325), followed by
// the demodulation of every sample and the decimation (CpuAlgorithm.cpp:353-365):
//     out[m] = y[center + m D] * exp(-j 2 pi fd/fs m D),
//     y = IFFT_M(FFT_M(bins) * H),  H = FFT_M(h) * hilbert_mask.
// The direct FIR (conv.cu) costs one complex MAC per tap and output, which for
// long pulses (the Hilbert part of h_a decays slowly: windows of ~2000 taps)
// exceeds the FFT's O(log M) per sample.  This kernel runs the FFT route for
// one line per CTA, entirely in shared memory (M <= 16384):
//
//   1. forward transform, decimation in frequency, in place: radix-R passes
//      (R = 16, the second pass 2, 4 or 8 to make up log2 M); a pass treats
//      the array as blocks of length L, and for each offset n1 < L/R transforms
//      the R elements n1 + j L/R in registers and multiplies output q by the
//      twiddle W_L^(n1 q).  The first pass reads the fixed-point bins straight
//      from global memory, sixteen independent loads per thread.  The spectrum
//      ends in digit-reversed order, which the host's copy of H matches (so no
//      reordering pass is needed);
//   2. the last forward pass, the multiply by H (pre-scaled by 1/M and by the
//      phase ramp exp(+j 2 pi center k / M), so that the result starts at
//      sample `center`), the decimation fold and the first inverse pass run in
//      registers: with F the largest power of two dividing D (F <= 16), the
//      samples y[F n'] are the length-M/F inverse transform of the spectrum
//      folded onto k mod M/F, and the F terms of a fold lie in one thread's
//      block of 16 (the M/F results are written in place, after a barrier);
//   3. inverse transform of length M/F, decimation in time: the exact inverse
//      passes in reverse order, the last one writing out[m] = y[F n'] times
//      the demodulation factor for the n' = m D / F.
//
// Shared memory holds the array padded by one float2 per 16 (element i at
// i + i/16): every pass then reads and writes its data without bank conflicts
// (two wavefronts per warp access of 8 bytes).  It also holds a quarter-wave
// table of twiddles W_M^y, y < M/4, copied from a host-made table (double
// precision rounded once); a task reads four of them (at strided exponents,
// so these reads do conflict) and multiplies out the rest; the first pass
// reads its four from the host-made table while the copy proceeds.  M = 8192
// then takes 87 KB, two CTAs per SM; M = 16384 one.  FP32 throughout: the
// relative RMS error is ~2e-7 of the IQ.
#include <cmath>
#include <complex>
#include <cstdint>
#include <cuda_runtime.h>
#include <type_traits>
#include <vector>
#include "fixedpoint.cuh"
#include "noise.cuh"
#include "kernels.hpp"

namespace bcsim_gb300 {

namespace {

constexpr int FFT_THREADS = 512;

// cos(2 pi k / 16) and sin(2 pi k / 16) for 0 <= k < 8
__host__ __device__ constexpr float cos16(int k) {
    return k == 0   ? 1.0f
           : k == 1 ? 0.92387953251128674f
           : k == 2 ? 0.70710678118654752f
           : k == 3 ? 0.38268343236508977f
           : k == 4 ? 0.0f
           : k == 5 ? -0.38268343236508977f
           : k == 6 ? -0.70710678118654752f
                    : -0.92387953251128674f;
}
__host__ __device__ constexpr float sin16(int k) { return cos16(4 - k < 0 ? k - 4 : 4 - k); }

__host__ __device__ constexpr int bit_reverse(int q, int R) {
    int r = 0;
    for (int b = 1; b < R; b <<= 1) r = (r << 1) | ((q & b) ? 1 : 0);
    return r;
}

__device__ __forceinline__ int fpad(int i) { return i + (i >> 4); }

__device__ __forceinline__ float2 cmul(float2 a, float2 w) {
    return make_float2(a.x * w.x - a.y * w.y, a.x * w.y + a.y * w.x);
}
__device__ __forceinline__ float2 cmul_conj(float2 a, float2 w) {   // a * conj(w)
    return make_float2(a.x * w.x + a.y * w.y, a.y * w.x - a.x * w.y);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

// a * W_16^e (forward: W = exp(-j 2 pi / 16); inverse: its conjugate), 0 <= e < 8
template <bool INV>
__device__ __forceinline__ float2 mul_w16(float2 a, int e) {
    if (e == 0) return a;
    if (e == 4) return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
    const float c = cos16(e), s = INV ? sin16(e) : -sin16(e);
    return make_float2(a.x * c - a.y * s, a.x * s + a.y * c);
}

// In-register DFT of R <= 16 points (natural order in), radix-2 decimation in
// frequency: output q lands in v[bit_reverse(q, R)].
template <int R, bool INV>
__device__ __forceinline__ void dft(float2 (&v)[R]) {
#pragma unroll
    for (int half = R / 2; half >= 1; half >>= 1) {
#pragma unroll
        for (int b = 0; b < R; b += 2 * half) {
#pragma unroll
            for (int j = 0; j < half; j++) {
                const float2 a = v[b + j], c = v[b + j + half];
                v[b + j] = cadd(a, c);
                v[b + j + half] = mul_w16<INV>(csub(a, c), j * (16 / (2 * half)));
            }
        }
    }
}

// W_M^x for 0 <= x < M/2 from the shared quarter-wave table tq (W_M^y, y < M/4,
// padded like the data): W^(y + M/4) = -j W^y.
__device__ __forceinline__ float2 twid(const float2* tq, int x, int q4) {
    if (x < q4) return tq[fpad(x)];
    const float2 a = tq[fpad(x - q4)];
    return make_float2(a.y, -a.x);
}

// Twiddles W^(e q), 0 < q < R, of one task, held as six factors: W^e, W^2e,
// W^3e = W^e W^2e for the two low bits of q, W^4e, W^8e, W^12e = W^4e W^8e for
// the two high bits; W^(eq) is one factor or the product of one of each (at
// most two roundings deep: ~2e-7 relative).  Twelve registers, not thirty.
struct TaskTw {
    float2 b1, b2, b3, b4, b8, b12;
};
template <int R>
__device__ __forceinline__ TaskTw task_twiddles(const float2* tq, int q4, int e) {
    TaskTw t;
    t.b1 = twid(tq, e, q4);
    if (R > 2) { t.b2 = twid(tq, 2 * e, q4); t.b3 = cmul(t.b1, t.b2); }
    if (R > 4) t.b4 = twid(tq, 4 * e, q4);
    if (R > 8) { t.b8 = twid(tq, 8 * e, q4); t.b12 = cmul(t.b4, t.b8); }
    return t;
}
// the same from the global table (tw[x] = W_M^x, x < M)
__device__ __forceinline__ TaskTw task_twiddles_global(const float2* __restrict__ tw, int e) {
    TaskTw t;
    t.b1 = __ldg(tw + e);
    t.b2 = __ldg(tw + 2 * e);
    t.b4 = __ldg(tw + 4 * e);
    t.b8 = __ldg(tw + 8 * e);
    t.b3 = cmul(t.b1, t.b2);
    t.b12 = cmul(t.b4, t.b8);
    return t;
}
// y * W^(eq) (or y * conj W^(eq)), q a compile-time constant 0 < q < 16
template <bool CONJ>
__device__ __forceinline__ float2 twiddle_q(float2 y, int q, const TaskTw& t) {
    const int lo = q & 3, hi = q >> 2;
    const float2 wl = lo == 1 ? t.b1 : lo == 2 ? t.b2 : t.b3;
    const float2 wh = hi == 1 ? t.b4 : hi == 2 ? t.b8 : t.b12;
    const float2 w = lo == 0 ? wh : hi == 0 ? wl : cmul(wl, wh);
    return CONJ ? cmul_conj(y, w) : cmul(y, w);
}

// One in-place pass of radix R over an array of Mc elements in blocks of
// length L: forward (output q of offset n1 times W_L^(n1 q)) or its exact
// inverse (input q times conj W_L^(n1 q), inverse DFT).  The twiddle W_L^x is
// W_M^(x ts), ts = M / L.  A thread takes 16 / R tasks at a time for R >= 8,
// 8 / R below (eight or sixteen loads in flight per thread).
template <int R, bool INV>
__device__ __forceinline__ void fft_pass(float2* s, int Mc, int L, int ts, const float2* tq, int q4) {
    constexpr int G = R >= 8 ? 16 / R : 8 / R;
    const int S = L / R;
    const int T = Mc / R;
    for (int t0 = threadIdx.x; t0 < T; t0 += blockDim.x * G) {
        float2 v[G][R];
        TaskTw w[G];
        int base[G];
#pragma unroll
        for (int g = 0; g < G; g++) {
            const int t = min(t0 + g * (int)blockDim.x, T - 1);   // (a clamped task is recomputed, not stored)
            const int n1 = t & (S - 1);
            base[g] = (t - n1) * R + n1;
            w[g] = task_twiddles<R>(tq, q4, n1 * ts);
#pragma unroll
            for (int j = 0; j < R; j++) v[g][j] = s[fpad(base[g] + j * S)];
        }
#pragma unroll
        for (int g = 0; g < G; g++) {
            if (INV) {
#pragma unroll
                for (int q = 1; q < R; q++) v[g][q] = twiddle_q<true>(v[g][q], q, w[g]);
            }
            dft<R, INV>(v[g]);
        }
#pragma unroll
        for (int g = 0; g < G; g++) {
            if (t0 + g * (int)blockDim.x >= T) continue;
#pragma unroll
            for (int q = 0; q < R; q++) {
                float2 y = v[g][bit_reverse(q, R)];
                if (!INV && q > 0) y = twiddle_q<false>(y, q, w[g]);
                s[fpad(base[g] + q * S)] = y;
            }
        }
    }
}

// The fused middle: last forward pass (blocks of 16, no twiddles), multiply by
// the spectrum, fold by F = 16 / RF, first inverse pass (radix RF, blocks of
// RF, no twiddles), in place: block b's RF results go to b*RF .. b*RF+RF-1
// after every thread has read its blocks (at most two per thread).
template <int RF, int NB>
__device__ __forceinline__ void fft_middle(float2* s, int M, const float4* __restrict__ spec4) {
    float2 f[NB][RF];
#pragma unroll
    for (int i = 0; i < NB; i++) {
        const int b = threadIdx.x + i * blockDim.x;
        if (b >= M / 16) break;
        float2 v[16];
#pragma unroll
        for (int j = 0; j < 16; j++) v[j] = s[fpad(b * 16 + j)];
        dft<16, false>(v);
#pragma unroll
        for (int r = 0; r < RF; r++) f[i][r] = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int q = 0; q < 16; q += 2) {
            const float4 h = __ldg(spec4 + b * 8 + q / 2);   // spectrum entries q, q + 1
            f[i][q % RF] = cadd(f[i][q % RF], cmul(v[bit_reverse(q, 16)], make_float2(h.x, h.y)));
            f[i][(q + 1) % RF] = cadd(f[i][(q + 1) % RF], cmul(v[bit_reverse(q + 1, 16)], make_float2(h.z, h.w)));
        }
        if (RF > 1) dft<RF, true>(f[i]);
        if (RF == 16) {   // no fold: the block's own positions
#pragma unroll
            for (int k = 0; k < RF; k++) s[fpad(b * RF + k)] = f[i][bit_reverse(k, RF)];
        }
    }
    if (RF == 16) return;
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NB; i++) {
        const int b = threadIdx.x + i * blockDim.x;
        if (b >= M / 16) break;
#pragma unroll
        for (int k = 0; k < RF; k++) s[fpad(b * RF + k)] = f[i][bit_reverse(k, RF)];
    }
}

// Bin n of a line as float, plus its seeded noise (noise.cuh) when nz.sigma > 0.
template <bool PD>
__device__ __forceinline__ float2 load_bin(const long long* __restrict__ lb, int n, int ns, float inv_scale,
                                           const NoiseParams& nz, int line) {
    if (n >= ns) return make_float2(0.0f, 0.0f);
    float2 v;
    if (PD) {
        const longlong2 q = __ldg(reinterpret_cast<const longlong2*>(lb) + n);
        v = make_float2(fix2f(q.x, inv_scale), fix2f(q.y, inv_scale));
    } else {
        v = make_float2(fix2f(__ldg(lb + n), inv_scale), 0.0f);
    }
    if (nz.sigma > 0.0f) {   // uniform over the CTA
        const float2 e = bin_noise(nz, nz.line0 + line, n);
        v.x += e.x;
        v.y += e.y;
    }
    return v;
}

// One line per CTA.  Passes: forward radix 16 at L = M (from the bins), radix
// RS (1 = none) at L = M/16, radix 16 down to L = 256, the middle at L = 16;
// inverse (length M' = M/F) radix 16 from L' = 16 (16/F) up to M'/(16 RS),
// radix RS at L' = M'/16, the output pass radix 16 at L' = M'.  MINB: CTAs per
// SM the register allocation leaves room for.
template <int RS, bool PD, int MINB>
__global__ void __launch_bounds__(FFT_THREADS, MINB)
    fft_convolve_demodulate_kernel(const unsigned long long* __restrict__ bins, int ns, float inv_scale, int M,
                                   int F, const float4* __restrict__ spec4, const float2* __restrict__ tw, int D,
                                   int nd, const float2* __restrict__ demod, float2* __restrict__ out,
                                   NoiseParams nz) {
    extern __shared__ __align__(16) float2 s[];
    const int Mp = M / F;
    float2* tq = s + fpad(M);   // W_M^y, y < M/4 (complete at the barrier after pass 0)
    const int q4 = M / 4;
    for (int y = threadIdx.x; y < q4; y += blockDim.x) tq[fpad(y)] = __ldg(tw + y);
    const int line = blockIdx.x;
    const long long* lb = reinterpret_cast<const long long*>(bins) + (int64_t)line * ns * (PD ? 2 : 1);

    // forward pass 0 (radix 16, L = M), from the bins: sixteen independent
    // loads per task, its twiddles from the global table meanwhile
    {
        const int S = M / 16;
        for (int t = threadIdx.x; t < S; t += blockDim.x) {
            float2 v[16];
            const TaskTw w = task_twiddles_global(tw, t);
#pragma unroll
            for (int j = 0; j < 16; j++) v[j] = load_bin<PD>(lb, t + j * S, ns, inv_scale, nz, line);
            dft<16, false>(v);
#pragma unroll
            for (int q = 0; q < 16; q++) {
                float2 y = v[bit_reverse(q, 16)];
                if (q > 0) y = twiddle_q<false>(y, q, w);
                s[fpad(t + q * S)] = y;
            }
        }
    }
    __syncthreads();
    int L = M / 16;
    if (RS > 1) {
        fft_pass<RS, false>(s, M, L, M / L, tq, q4);
        __syncthreads();
        L /= RS;
    }
    for (; L > 16; L /= 16) {
        fft_pass<16, false>(s, M, L, M / L, tq, q4);
        __syncthreads();
    }
    switch (F) {
        case 1: fft_middle<16, MINB == 2 ? 1 : 2>(s, M, spec4); break;
        case 2: fft_middle<8, MINB == 2 ? 1 : 2>(s, M, spec4); break;
        case 4: fft_middle<4, MINB == 2 ? 1 : 2>(s, M, spec4); break;
        case 8: fft_middle<2, MINB == 2 ? 1 : 2>(s, M, spec4); break;
        default: fft_middle<1, MINB == 2 ? 1 : 2>(s, M, spec4); break;
    }
    __syncthreads();
    for (L = (16 / F) * 16; L <= Mp / (16 * RS); L *= 16) {
        fft_pass<16, true>(s, Mp, L, M / L, tq, q4);
        __syncthreads();
    }
    if (RS > 1) {
        fft_pass<RS, true>(s, Mp, Mp / 16, M / (Mp / 16), tq, q4);
        __syncthreads();
    }
    // output pass (radix 16, L' = M'): samples y[F n'], n' = k1 + k2 M'/16;
    // output m takes n' = m D / F
    {
        const int S = Mp / 16;
        const int DF = D / F;
        for (int k1 = threadIdx.x; k1 < S; k1 += blockDim.x) {
            float2 v[16];
            const TaskTw w = task_twiddles<16>(tq, q4, k1 * F);
#pragma unroll
            for (int q = 0; q < 16; q++) v[q] = s[fpad(k1 + q * S)];
#pragma unroll
            for (int q = 1; q < 16; q++) v[q] = twiddle_q<true>(v[q], q, w);
            dft<16, true>(v);
#pragma unroll
            for (int k = 0; k < 16; k++) {
                const int n = k1 + k * S;
                const int m = n / DF;
                if (m * DF == n && m < nd) out[(int64_t)line * nd + m] = cmul(v[bit_reverse(k, 16)], __ldg(demod + m));
            }
        }
    }
}

// the radix between the first pass and the radix-16 passes: M = 16 RS 16^k
int fft_mid_radix(int64_t M) {
    int n = 0;
    while ((int64_t(1) << n) < M) n++;
    return n % 4 ? 1 << (n % 4) : 1;
}

}  // namespace

bool fft_convolution_supported(int64_t M) { return M >= 256 && M <= FFT_MAX_M && (M & (M - 1)) == 0; }

int fft_fold(int D) {
    int F = 1;
    while (F < 16 && D % (2 * F) == 0) F *= 2;
    return F;
}

size_t fft_convolution_smem(int64_t M) {
    const int64_t words = (M + M / 16) + (M / 4 + M / 64);
    return (size_t)words * sizeof(float2);
}

void make_fft_tables(const std::complex<double>* H, int64_t M, int center, float2* spec, float2* tw) {
    // position p of the forward transform's output holds frequency
    // k = q_0 + R_0 (q_1 + R_1 (q_2 + ...)), p = q_0 M/R_0 + q_1 M/(R_0 R_1) + ...
    std::vector<int> radices{16};
    if (fft_mid_radix(M) > 1) radices.push_back(fft_mid_radix(M));
    int64_t rest = M / 16 / fft_mid_radix(M);
    for (; rest > 1; rest /= 16) radices.push_back(16);
    const double two_pi = 6.283185307179586;
    for (int64_t p = 0; p < M; p++) {
        int64_t rem = p, Lc = M, mult = 1, k = 0;
        for (int R : radices) {
            Lc /= R;
            const int64_t q = rem / Lc;
            rem -= q * Lc;
            k += mult * q;
            mult *= R;
        }
        // H(k) exp(+j 2 pi center k / M) / M: the inverse transform then starts at `center`
        const double ph = two_pi * (double)((int64_t)center * k % M) / (double)M;
        const std::complex<double> v = H[k] * std::complex<double>(std::cos(ph), std::sin(ph)) / (double)M;
        spec[p] = make_float2((float)v.real(), (float)v.imag());
    }
    for (int64_t e = 0; e < M; e++) {
        const double ph = -two_pi * (double)e / (double)M;
        tw[e] = make_float2((float)std::cos(ph), (float)std::sin(ph));
    }
}

cudaError_t launch_fft_convolve_demodulate(const unsigned long long* bins, int num_lines, int ns, int phase_delay,
                                           float inv_scale, const float2* spec, const float2* tw, int64_t M,
                                           int decimation, int nd, const float2* demod, float2* out,
                                           cudaStream_t stream, const NoiseParams* noise) {
    if (num_lines <= 0 || nd <= 0) return cudaSuccess;
    NoiseParams nz{};
    if (noise && noise->sigma > 0.0f) nz = *noise;
    if (!fft_convolution_supported(M) || ns > M) return cudaErrorInvalidValue;
    const int F = fft_fold(decimation);
    const size_t smem = fft_convolution_smem(M);
    const int RS = fft_mid_radix(M);
    const bool two = 2 * smem <= 227 * 1024;   // two CTAs per SM fit: leave them the registers
    auto launch = [&](auto k) -> cudaError_t {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k<<<num_lines, FFT_THREADS, smem, stream>>>(bins, ns, inv_scale, (int)M, F,
                                                   reinterpret_cast<const float4*>(spec), tw, decimation, nd, demod,
                                                   out, nz);
        return cudaGetLastError();
    };
    auto pick = [&](auto pd) -> cudaError_t {
        constexpr bool PD = decltype(pd)::value;
        if (two) {
            switch (RS) {
                case 2: return launch(fft_convolve_demodulate_kernel<2, PD, 2>);
                case 4: return launch(fft_convolve_demodulate_kernel<4, PD, 2>);
                case 8: return launch(fft_convolve_demodulate_kernel<8, PD, 2>);
                default: return launch(fft_convolve_demodulate_kernel<1, PD, 2>);
            }
        }
        switch (RS) {
            case 2: return launch(fft_convolve_demodulate_kernel<2, PD, 1>);
            case 4: return launch(fft_convolve_demodulate_kernel<4, PD, 1>);
            case 8: return launch(fft_convolve_demodulate_kernel<8, PD, 1>);
            default: return launch(fft_convolve_demodulate_kernel<1, PD, 1>);
        }
    };
    return phase_delay ? pick(std::true_type{}) : pick(std::false_type{});
}

}  // namespace bcsim_gb300
