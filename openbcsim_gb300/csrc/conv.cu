// conv.cu -- fused pulse convolution, IQ demodulation and radial decimation.
//
// The reference convolves every line's time-projection bins with the analytic
// (Hilbert-masked) excitation by a length-M FFT, multiply and inverse FFT
// (src/core/BeamConvolver.cpp:64-91, GPU: cuFFT + MultiplyFftKernel,
// GpuAlgorithm.cpp:280-325), keeps samples center .. center+ns-1, demodulates
// every sample (CpuAlgorithm.cpp:353-358) and then keeps every D-th
// (CpuAlgorithm.cpp:362-365).  That is a circular convolution
//     y[k] = sum_n h_a[n] * bins[(k - n) mod M],  h_a = IFFT(FFT_M(h) * mask),
// and only k = center + m*D, m < ceil(ns/D), is ever used.  This kernel
// evaluates exactly those outputs as a direct FIR over the window of h_a taps
// that holds all but a stated fraction of its energy (chosen on the host), then
// applies the demodulation factor of output m.
//
// Layout: one CTA per (line, block of OUT_PER_CTA outputs).  The bins the block
// needs are converted from fixed point and staged in shared memory split into D
// polyphase rows, so that for every tap the threads of a warp read consecutive
// words (tap w of output m reads row (W-1-w) mod D, column m + (W-1-w) div D).
#include <cstdint>
#include <cuda_runtime.h>
#include "kernels.hpp"

namespace bcsim_gb300 {

constexpr int OUT_PER_CTA = 256;

template <bool PD>
__global__ void __launch_bounds__(OUT_PER_CTA)
    convolve_demodulate_kernel(const unsigned long long* __restrict__ bins, int ns, float inv_scale,
                               const float2* __restrict__ taps, int W, int tap_start, int64_t M, int center, int D,
                               int nd, const float2* __restrict__ demod, float2* __restrict__ out) {
    extern __shared__ float2 seg[];
    const int line = blockIdx.y;
    const int m0 = blockIdx.x * OUT_PER_CTA;
    const int tid = threadIdx.x;
    // bins index of segment element q:  j = jbase + q
    const int64_t k0 = (int64_t)center + (int64_t)m0 * D;
    const int64_t jbase = k0 - tap_start - (W - 1);
    const int seg_len = (OUT_PER_CTA - 1) * D + W;
    const int row = (seg_len + D - 1) / D;   // polyphase row length
    const int stride = PD ? 2 : 1;
    const long long* lb = (const long long*)bins + (int64_t)line * ns * stride;
    for (int q = tid; q < seg_len; q += OUT_PER_CTA) {
        int64_t j = (jbase + q) % M;
        if (j < 0) j += M;
        float2 v = make_float2(0.0f, 0.0f);
        if (j < ns) {
            v.x = __ll2float_rn(__ldg(lb + j * stride)) * inv_scale;
            if (PD) v.y = __ll2float_rn(__ldg(lb + j * stride + 1)) * inv_scale;
        }
        seg[(q % D) * row + q / D] = v;
    }
    __syncthreads();
    const int m = m0 + tid;
    if (m >= nd) return;
    float yr = 0.0f, yi = 0.0f;
    // output m uses segment elements q = (m - m0) * D + (W - 1 - w), w = 0 .. W-1
    int ph = (W - 1) % D, col = tid + (W - 1) / D;
    for (int w = 0; w < W; w++) {
        const float2 h = __ldg(taps + w);
        const float2 v = seg[ph * row + col];
        if (PD) {
            yr = fmaf(v.x, h.x, fmaf(-v.y, h.y, yr));
            yi = fmaf(v.x, h.y, fmaf(v.y, h.x, yi));
        } else {
            yr = fmaf(v.x, h.x, yr);
            yi = fmaf(v.x, h.y, yi);
        }
        // next tap: q decreases by one
        if (ph == 0) { ph = D - 1; col -= 1; } else { ph -= 1; }
    }
    const float2 dm = __ldg(demod + m);
    out[(int64_t)line * nd + m] = make_float2(yr * dm.x - yi * dm.y, yr * dm.y + yi * dm.x);
}

cudaError_t launch_convolve_demodulate(const unsigned long long* bins, int num_lines, int ns, int phase_delay,
                                       float inv_scale, const float2* taps, int num_taps, int tap_start, int64_t M,
                                       int center, int decimation, int nd, const float2* demod, float2* out,
                                       cudaStream_t stream) {
    if (num_lines <= 0 || nd <= 0) return cudaSuccess;
    const int seg_len = (OUT_PER_CTA - 1) * decimation + num_taps;
    const int row = (seg_len + decimation - 1) / decimation;
    const size_t smem = (size_t)row * decimation * sizeof(float2);
    dim3 grid((unsigned)((nd + OUT_PER_CTA - 1) / OUT_PER_CTA), (unsigned)num_lines);
    if (phase_delay) {
        auto k = convolve_demodulate_kernel<true>;
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k<<<grid, OUT_PER_CTA, smem, stream>>>(bins, ns, inv_scale, taps, num_taps, tap_start, M, center,
                                               decimation, nd, demod, out);
    } else {
        auto k = convolve_demodulate_kernel<false>;
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k<<<grid, OUT_PER_CTA, smem, stream>>>(bins, ns, inv_scale, taps, num_taps, tap_start, M, center,
                                               decimation, nd, demod, out);
    }
    return cudaGetLastError();
}

}  // namespace bcsim_gb300
