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
// Layout: one CTA per (line, block of THREADS*4 outputs).  The bins the block
// needs are converted from fixed point and staged in shared memory split into D
// polyphase rows: with q = (m - m0) * D + (W - 1 - w) the segment index of tap w
// of output m, row q mod D holds the elements of one phase, so that a phase's
// taps walk along one row.  Each thread computes 4 consecutive outputs; along a
// row they need consecutive elements, held in a rotating window of 4 registers:
// one shared-memory load and one (broadcast) tap load per 16 complex MACs.  A
// row is stored as 4 sub-rows by element index mod 4 (element e at sub-row e&3,
// position e>>2), so that the 32 threads of a warp, whose windows start 4
// elements apart, read 32 consecutive elements of one sub-row (no bank
// conflicts); sub-rows are padded to 4 mod 16 elements so that the staging
// stores, which cover all four sub-rows, do not conflict either.  The taps are
// stored phase-major on the host, zero-padded to a multiple of 4 per phase.
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>
#include "kernels.hpp"
#include "fixedpoint.cuh"

namespace bcsim_gb300 {

constexpr int CONV_K = 4;   // outputs per thread

// Complex multiply-accumulate y += v h with paired FP32 FMAs (two per
// instruction): the tap is held as (h.re, h.im, -h.im, h.re), so that
//     y += (v.im, v.im) * (-h.im, h.re),   y += (v.re, v.re) * (h.re, h.im)
// are two FFMA2 -- per component the same two fused operations, in the same
// order, as fma(v.re, h.re, fma(-v.im, h.im, y.re)) and its imaginary twin.
__device__ __forceinline__ void cmac(float2& y, float2 v, float4 h) {
    y = __ffma2_rn(make_float2(v.y, v.y), make_float2(h.z, h.w), y);
    y = __ffma2_rn(make_float2(v.x, v.x), make_float2(h.x, h.y), y);
}
// real bins (no phase delay): y += v.re h
__device__ __forceinline__ void rmac(float2& y, float2 v, float4 h) {
    y = __ffma2_rn(make_float2(v.x, v.x), make_float2(h.x, h.y), y);
}
__device__ __forceinline__ float4 tap4(float2 h) { return make_float4(h.x, h.y, -h.y, h.x); }

template <bool PD, bool TAPS_SMEM>
__global__ void __launch_bounds__(128)
    convolve_demodulate_kernel(const unsigned long long* __restrict__ bins, int ns, float inv_scale,
                               const float2* __restrict__ taps_pm, const int* __restrict__ ph_off, int W,
                               int tap_start, int64_t M, int center, int D, int nd, int sub, int cols,
                               const float2* __restrict__ demod, float2* __restrict__ out) {
    extern __shared__ float4 smem4[];
    float2* seg = reinterpret_cast<float2*>(smem4);   // [D][4][sub]
    const int row = 4 * sub;
    // phase-major taps as (h.re, h.im, -h.im, h.re), in shared memory when they fit
    float4* tp4 = reinterpret_cast<float4*>(seg + (size_t)D * row);
    const int line = blockIdx.y;
    const int per_cta = blockDim.x * CONV_K;
    const int m0 = blockIdx.x * per_cta;
    const int tid = threadIdx.x;
    if (TAPS_SMEM) {
        const int ntaps_pm = __ldg(ph_off + D);
        for (int i = tid; i < ntaps_pm; i += blockDim.x) tp4[i] = tap4(__ldg(taps_pm + i));
    }
    // bins index of segment element q = col * D + ph: j = (jbase + q) mod M, M a
    // power of two (next_power_of_two, fft.cpp:80-82), so the wrap is a mask
    const int64_t k0 = (int64_t)center + (int64_t)m0 * D;
    const int64_t jbase = k0 - tap_start - (W - 1);
    const long long mmask = (long long)M - 1;
    const int stride = PD ? 2 : 1;
    const long long* lb = (const long long*)bins + (int64_t)line * ns * stride;
    // the last block of a line may hold fewer than per_cta outputs: stage only
    // the columns its threads read
    const int valid = min(per_cta, nd - m0);
    const int cols_used = min(cols, ((valid + CONV_K - 1) / CONV_K) * CONV_K + (cols - CONV_K * (int)blockDim.x));
    // each thread stages the D consecutive bins of a column (one or two cache
    // lines, read once), writing one element of every phase row
    for (int col = tid; col < cols_used; col += blockDim.x) {
        const long long j0 = jbase + (long long)col * D;
        float2* dst = seg + (col & 3) * sub + (col >> 2);
        for (int ph = 0; ph < D; ph++) {
            const long long j = (j0 + ph) & mmask;
            float2 v = make_float2(0.0f, 0.0f);
            if (j < ns) {
                if (PD) {
                    const longlong2 q = __ldg(reinterpret_cast<const longlong2*>(lb) + j);
                    v.x = ll2f_rn(q.x) * inv_scale;
                    v.y = ll2f_rn(q.y) * inv_scale;
                } else {
                    v.x = ll2f_rn(__ldg(lb + j)) * inv_scale;
                }
            }
            dst[ph * row] = v;
        }
    }
    __syncthreads();
    if (tid * CONV_K >= valid) return;   // no output of this thread (no barrier follows)
    float2 y0 = make_float2(0.f, 0.f), y1 = y0, y2 = y0, y3 = y0;
    for (int ph = 0; ph < D; ph++) {
        // element tid*4 + t + j of the phase row: sub-row j & 3, position tid + t/4 + j/4
        const float2* r0 = seg + ph * row + tid;
        const float2* r1 = r0 + sub;
        const float2* r2 = r1 + sub;
        const float2* r3 = r2 + sub;
        const int t_beg = __ldg(ph_off + ph), t_end = __ldg(ph_off + ph + 1);
        float2 w0 = r0[0], w1 = r1[0], w2 = r2[0], w3;
        const float4* hp = tp4 + t_beg;
        const float2* hg = taps_pm + t_beg;
        for (int t = 0, i = 0; t < t_end - t_beg; t += 4, i++) {
            float4 h;
            w3 = r3[i]; h = TAPS_SMEM ? hp[t] : tap4(__ldg(hg + t));
            if (PD) { cmac(y0, w0, h); cmac(y1, w1, h); cmac(y2, w2, h); cmac(y3, w3, h); }
            else { rmac(y0, w0, h); rmac(y1, w1, h); rmac(y2, w2, h); rmac(y3, w3, h); }
            w0 = r0[i + 1]; h = TAPS_SMEM ? hp[t + 1] : tap4(__ldg(hg + t + 1));
            if (PD) { cmac(y0, w1, h); cmac(y1, w2, h); cmac(y2, w3, h); cmac(y3, w0, h); }
            else { rmac(y0, w1, h); rmac(y1, w2, h); rmac(y2, w3, h); rmac(y3, w0, h); }
            w1 = r1[i + 1]; h = TAPS_SMEM ? hp[t + 2] : tap4(__ldg(hg + t + 2));
            if (PD) { cmac(y0, w2, h); cmac(y1, w3, h); cmac(y2, w0, h); cmac(y3, w1, h); }
            else { rmac(y0, w2, h); rmac(y1, w3, h); rmac(y2, w0, h); rmac(y3, w1, h); }
            w2 = r2[i + 1]; h = TAPS_SMEM ? hp[t + 3] : tap4(__ldg(hg + t + 3));
            if (PD) { cmac(y0, w3, h); cmac(y1, w0, h); cmac(y2, w1, h); cmac(y3, w2, h); }
            else { rmac(y0, w3, h); rmac(y1, w0, h); rmac(y2, w1, h); rmac(y3, w2, h); }
        }
    }
    const float2 ys[CONV_K] = {y0, y1, y2, y3};
    const int base = tid * CONV_K;
#pragma unroll
    for (int k = 0; k < CONV_K; k++) {
        const int m = m0 + base + k;
        if (m < nd) {
            const float2 dm = __ldg(demod + m);
            out[(int64_t)line * nd + m] = make_float2(ys[k].x * dm.x - ys[k].y * dm.y, ys[k].x * dm.y + ys[k].y * dm.x);
        }
    }
}

// Staged elements per phase row for a block of `threads` threads: thread T's
// window reaches element 4T + max_ph_taps + 2, so 4*threads + max_ph_taps
// elements (max_ph_taps is a multiple of 4) cover every read.
static int conv_cols(int threads, int max_ph_taps) { return threads * CONV_K + max_ph_taps; }
// Sub-row length: cols/4 positions, padded to 4 mod 16.
static int conv_sub(int threads, int max_ph_taps) {
    const int need = conv_cols(threads, max_ph_taps) / 4;
    return need + ((4 - need) % 16 + 16) % 16;
}

cudaError_t launch_convolve_demodulate(const unsigned long long* bins, int num_lines, int ns, int phase_delay,
                                       float inv_scale, const float2* taps_pm, const int* ph_off, int ntaps_pm,
                                       int max_ph_taps, int W, int tap_start, int64_t M, int center, int decimation,
                                       int nd, const float2* demod, float2* out, cudaStream_t stream) {
    if (num_lines <= 0 || nd <= 0) return cudaSuccess;
    if (max_ph_taps % 4) return cudaErrorInvalidValue;
    // a line's outputs split evenly over its blocks of at most 128 threads
    // (4 outputs each; no block left nearly empty), and more blocks per line
    // for few lines so that the grid still fills the GPU
    auto threads_for = [&](int64_t blocks) {
        const int64_t per = (nd + blocks - 1) / blocks;
        return (int)std::max<int64_t>(32, ((per + CONV_K - 1) / CONV_K + 31) / 32 * 32);
    };
    int64_t nblk = (nd + 128 * CONV_K - 1) / (128 * CONV_K);
    int threads = threads_for(nblk);
    while (threads > 32 && (int64_t)num_lines * nblk < 2 * 152) threads = threads_for(++nblk);
    nblk = (nd + threads * CONV_K - 1) / (threads * CONV_K);
    auto smem_for = [&](int th, int taps_smem) {
        return (size_t)4 * conv_sub(th, max_ph_taps) * decimation * sizeof(float2) +
               (taps_smem ? (size_t)ntaps_pm * sizeof(float4) : 0);
    };
    int taps_in_smem = 1;
    const size_t limit = 200 * 1024;
    if (smem_for(threads, 1) > limit) taps_in_smem = 0;   // very long windows: taps from global memory (broadcast loads)
    while (smem_for(threads, taps_in_smem) > limit && threads > 32) threads -= 32;
    const size_t smem = smem_for(threads, taps_in_smem);
    if (smem > limit) return cudaErrorInvalidValue;
    const int sub = conv_sub(threads, max_ph_taps), cols = conv_cols(threads, max_ph_taps);
    nblk = (nd + threads * CONV_K - 1) / (threads * CONV_K);
    const dim3 grid((unsigned)nblk, (unsigned)num_lines);
    auto launch = [&](auto k) -> cudaError_t {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k<<<grid, threads, smem, stream>>>(bins, ns, inv_scale, taps_pm, ph_off, W, tap_start, M, center, decimation,
                                           nd, sub, cols, demod, out);
        return cudaGetLastError();
    };
    if (phase_delay) return taps_in_smem ? launch(convolve_demodulate_kernel<true, true>)
                                         : launch(convolve_demodulate_kernel<true, false>);
    return taps_in_smem ? launch(convolve_demodulate_kernel<false, true>) : launch(convolve_demodulate_kernel<false, false>);
}

int make_phase_major_taps(const float2* taps, int W, int D, float2* out, int* off, int* max_ph) {
    int n = 0, mx = 0;
    for (int ph = 0; ph < D; ph++) {
        off[ph] = n;
        const int cnt = ph <= W - 1 ? (W - 1 - ph) / D + 1 : 0;
        const int pad = (cnt + 3) / 4 * 4;
        for (int t = 0; t < pad; t++) out[n + t] = t < cnt ? taps[W - 1 - (ph + t * D)] : make_float2(0.0f, 0.0f);
        n += pad;
        mx = pad > mx ? pad : mx;
    }
    off[D] = n;
    *max_ph = mx;
    return n;
}

}  // namespace bcsim_gb300
