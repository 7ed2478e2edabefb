// conv.cu -- fused pulse convolution, IQ demodulation and radial decimation.
//
// The reference convolves every line's time-projection bins with the analytic
// (Hilbert-masked) excitation by a length-M FFT, multiply and inverse FFT
// (src/core/BeamConvolver.cpp:64-91, GPU: cuFFT + MultiplyFftKernel,
// GpuAlgorithm.cpp:280-325), keeps samples center .. center+ns-1, demodulates
// every sample (CpuAlgorithm.cpp:353-358) and then keeps every D-th
// (CpuAlgorithm.cpp:362-365).  That is a circular convolution
//     y[k] = sum_n h_a[n] * bins[(k - n) mod M],  h_a = IFFT(FFT_M(h) * mask),
// and only k = center + m*D, m < ceil(ns/D), is ever used.  These kernels
// evaluate exactly those outputs as a direct FIR over the window of h_a taps
// that holds all but a stated fraction of its energy (chosen on the host), then
// apply the demodulation factor of output m.
//
// Work item: one line and a block of consecutive outputs m0 .. m0+P-1.  The
// bins the item needs (its segment: columns of D consecutive bins) are
// converted from fixed point and staged in shared memory split into D
// polyphase rows: with q = (m - m0) * D + (W - 1 - w) the segment index of tap
// w of output m, row q mod D holds the elements of one phase, so that a phase's
// taps walk along one row.  Each thread computes 4 consecutive outputs; along a
// row they need consecutive elements, held in a rotating window of 4 registers:
// one shared-memory load and one (broadcast) tap load per 4 complex MACs per
// output.  A row is stored as 4 sub-rows by element index mod 4 (element e at
// sub-row e&3, position e>>2), so that the 32 threads of a warp, whose windows
// start 4 elements apart, read 32 consecutive elements of one sub-row (no bank
// conflicts).  The staging writes element q (column q / D, phase q % D) for
// consecutive q from consecutive threads; sub-rows of odd length and rows of
// length 2 mod 16 (in float2) keep those stores free of bank conflicts for
// D = 8.  The taps are stored phase-major on the host, zero-padded to a
// multiple of 4 per phase.
//
// One CTA per work item (blockIdx.y = line, blockIdx.x = output block): the
// threads load the segment's bins with coalesced 16-byte loads (eight in
// flight per thread), convert them and store the phase rows; while one CTA
// convolves, the SM's other resident CTAs load theirs.
//
// Complex MACs split the analytic pulse h_a = h + i g by parts.  Its real part
// is the excitation itself (Re IFFT(FFT(h) mask) = h for the Hilbert mask), so
// h is non-zero only on the excitation's short support, while g (the Hilbert
// transform) fills the window.  For bin a + ib,
//     G += (a, b) g  over every tap,  H += (a, b) h  over the support only,
//     y = (H.re - G.im, H.im + G.re),
// each a paired FP32 FMA (FFMA2) per tap and output: one per complex MAC
// outside the support, two inside it.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>
#include "kernels.hpp"
#include "fixedpoint.cuh"
#include "noise.cuh"

namespace bcsim_gb300 {

constexpr int CONV_K = 4;   // outputs per thread

// real bins (no phase delay): y += v.re h with h = (c, d)
__device__ __forceinline__ void rmac(float2& y, float2 v, float4 h) {
    y = __ffma2_rn(make_float2(v.x, v.x), make_float2(h.x, h.y), y);
}
// tap h + ig in the form the MAC loop reads: (g, g, h, h) for complex bins,
// (h, g, 0, 0) for real bins
__device__ __forceinline__ float4 tap_split(float2 t) { return make_float4(t.y, t.y, t.x, t.x); }
__device__ __forceinline__ float4 tap_real(float2 t) { return make_float4(t.x, t.y, 0.0f, 0.0f); }

// Row padding (in float2) that makes a row 2 mod 16 long: consecutive phases of
// one column then fall on different bank pairs.
__host__ __device__ __forceinline__ int conv_rowpad(int sub) { return ((2 - 4 * sub) % 16 + 16) % 16; }

// The MAC loop of one thread: outputs 4*tid .. 4*tid+3 of the staged item, over
// all D phases.  seg: [D][row] with 4 sub-rows of `sub` positions per row;
// tp4: taps in shared memory (TAPS_SMEM) else taps_pm in global memory;
// ph: phase offsets into the phase-major taps (D + 1 entries), then per phase
// the range [lo, hi) of 4-tap iterations that hold the excitation's support.
//
// Iteration i of a phase covers taps 4i .. 4i+3: it needs row elements
// r0[i], r1[i], r2[i] (from iteration i-1), r3[i], r0[i+1], r1[i+1], r2[i+1]
// and four taps.  Three register sets rotate: iteration i computes from set
// i mod 3 (loaded during iteration i-1) and the carried elements of set
// (i-1) mod 3, and loads set (i+1) mod 3 for the next iteration -- every
// shared-memory load has a whole iteration to land, with no register moves.
struct FirSet {
    float2 a, b, c, d;        // r3[i], r0[i+1], r1[i+1], r2[i+1]
    float4 h0, h1, h2, h3;    // taps 4i .. 4i+3
};

template <bool PD, bool TAPS_SMEM>
__device__ __forceinline__ void fir_mac(const float2* seg, int row, int sub, int tid, const float4* tp4,
                                        const float2* __restrict__ taps_pm, const int* ph, int D, float2 out[4]) {
    // PD: G (every tap) and H (support taps); real bins: y in G
    float2 G0 = make_float2(0.f, 0.f), G1 = G0, G2 = G0, G3 = G0;
    float2 H0 = G0, H1 = G0, H2 = G0, H3 = G0;
    for (int p = 0; p < D; p++) {
        // element tid*4 + t + j of the phase row: sub-row j & 3, position tid + t/4 + j/4
        const float2* r0 = seg + p * row + tid;
        const float2* r1 = r0 + sub;
        const float2* r2 = r1 + sub;
        const float2* r3 = r2 + sub;
        const int t_beg = ph[p];
        const int n4 = (ph[p + 1] - t_beg) >> 2;
        if (n4 == 0) continue;
        const int h_lo = ph[D + 1 + 2 * p], h_hi = ph[D + 2 + 2 * p];
        const float4* hp = tp4 + t_beg;
        const float2* hg = taps_pm + t_beg;
        auto tap = [&](int t) -> float4 {
            return TAPS_SMEM ? hp[t] : (PD ? tap_split(__ldg(hg + t)) : tap_real(__ldg(hg + t)));
        };
        FirSet S0, S1, S2;
#define BCSIM_LOAD(S, I)                                                            \
    {                                                                               \
        S.a = r3[I]; S.b = r0[(I) + 1]; S.c = r1[(I) + 1]; S.d = r2[(I) + 1];       \
        S.h0 = tap(4 * (I)); S.h1 = tap(4 * (I) + 1); S.h2 = tap(4 * (I) + 2); S.h3 = tap(4 * (I) + 3); \
    }
#define BCSIM_G(Y, W, H)                                                            \
    { if (PD) Y = __ffma2_rn(W, make_float2(H.x, H.y), Y); else rmac(Y, W, H); }
#define BCSIM_H(Y, W, H) { Y = __ffma2_rn(W, make_float2(H.z, H.w), Y); }
#define BCSIM_ITER(C, P, N, I)                                                      \
    {                                                                               \
        if ((I) + 1 < n4) BCSIM_LOAD(N, (I) + 1)                                    \
        BCSIM_G(G0, P.b, C.h0) BCSIM_G(G1, P.c, C.h0) BCSIM_G(G2, P.d, C.h0) BCSIM_G(G3, C.a, C.h0) \
        BCSIM_G(G0, P.c, C.h1) BCSIM_G(G1, P.d, C.h1) BCSIM_G(G2, C.a, C.h1) BCSIM_G(G3, C.b, C.h1) \
        BCSIM_G(G0, P.d, C.h2) BCSIM_G(G1, C.a, C.h2) BCSIM_G(G2, C.b, C.h2) BCSIM_G(G3, C.c, C.h2) \
        BCSIM_G(G0, C.a, C.h3) BCSIM_G(G1, C.b, C.h3) BCSIM_G(G2, C.c, C.h3) BCSIM_G(G3, C.d, C.h3) \
        if (PD && (I) >= h_lo && (I) < h_hi) {   /* warp-uniform */                 \
            BCSIM_H(H0, P.b, C.h0) BCSIM_H(H1, P.c, C.h0) BCSIM_H(H2, P.d, C.h0) BCSIM_H(H3, C.a, C.h0) \
            BCSIM_H(H0, P.c, C.h1) BCSIM_H(H1, P.d, C.h1) BCSIM_H(H2, C.a, C.h1) BCSIM_H(H3, C.b, C.h1) \
            BCSIM_H(H0, P.d, C.h2) BCSIM_H(H1, C.a, C.h2) BCSIM_H(H2, C.b, C.h2) BCSIM_H(H3, C.c, C.h2) \
            BCSIM_H(H0, C.a, C.h3) BCSIM_H(H1, C.b, C.h3) BCSIM_H(H2, C.c, C.h3) BCSIM_H(H3, C.d, C.h3) \
        }                                                                           \
    }
        // the elements carried into iteration 0: r0[0], r1[0], r2[0]
        S2.b = r0[0]; S2.c = r1[0]; S2.d = r2[0];
        BCSIM_LOAD(S0, 0)
        for (int i = 0;; i += 3) {
            BCSIM_ITER(S0, S2, S1, i)
            if (i + 1 >= n4) break;
            BCSIM_ITER(S1, S0, S2, i + 1)
            if (i + 2 >= n4) break;
            BCSIM_ITER(S2, S1, S0, i + 2)
            if (i + 3 >= n4) break;
        }
#undef BCSIM_ITER
#undef BCSIM_H
#undef BCSIM_G
#undef BCSIM_LOAD
    }
    if (PD) {   // y = (H.re - G.im, H.im + G.re)
        out[0] = make_float2(H0.x - G0.y, H0.y + G0.x); out[1] = make_float2(H1.x - G1.y, H1.y + G1.x);
        out[2] = make_float2(H2.x - G2.y, H2.y + G2.x); out[3] = make_float2(H3.x - G3.y, H3.y + G3.x);
    } else {
        out[0] = G0; out[1] = G1; out[2] = G2; out[3] = G3;
    }
}

// Demodulated outputs m0 + 4*tid + k (k < 4, m < nd) of one line.
__device__ __forceinline__ void fir_store(const float2 ys[4], int64_t line, int m0, int tid, int nd,
                                          const float2* __restrict__ demod, float2* __restrict__ out) {
#pragma unroll
    for (int k = 0; k < CONV_K; k++) {
        const int m = m0 + tid * CONV_K + k;
        if (m < nd) {
            const float2 dm = __ldg(demod + m);
            out[line * nd + m] = make_float2(ys[k].x * dm.x - ys[k].y * dm.y, ys[k].x * dm.y + ys[k].y * dm.x);
        }
    }
}

// One work item per CTA: line blockIdx.y, outputs blockIdx.x * blockDim.x * 4 ...
// (at most 102 registers: 96 in the complex-bin kernel, so that an SM holds 20
// warps -- six 96-thread CTAs, their shared memory permitting -- not 16).
// PD: the bins are complex (phase delay); NZ: seeded noise is added to every
// staged bin j < ns (noise.cuh), which makes real bins complex too.
template <bool PD, bool TAPS_SMEM, bool NZ>
__global__ void __launch_bounds__(128, 5)
    convolve_demodulate_kernel(const unsigned long long* __restrict__ bins, int ns, float inv_scale,
                               const float2* __restrict__ taps_pm, const int* __restrict__ ph_off, int W,
                               int tap_start, int64_t M, int center, int D, int nd, int sub, int row, int cols,
                               const float2* __restrict__ demod, float2* __restrict__ out, NoiseParams nz) {
    constexpr bool CX = PD || NZ;   // complex arithmetic
    extern __shared__ __align__(16) float4 smem4[];
    float2* seg = reinterpret_cast<float2*>(smem4);   // [D][row]
    // phase-major taps, in shared memory when they fit
    float4* tp4 = reinterpret_cast<float4*>(seg + (size_t)D * row);
    const int line = blockIdx.y;
    const int per_cta = blockDim.x * CONV_K;
    const int m0 = blockIdx.x * per_cta;
    const int tid = threadIdx.x;
    if (TAPS_SMEM) {
        const int ntaps_pm = __ldg(ph_off + D);
        for (int i = tid; i < ntaps_pm; i += blockDim.x)
            tp4[i] = CX ? tap_split(__ldg(taps_pm + i)) : tap_real(__ldg(taps_pm + i));
    }
    const long long jbase = (long long)center + (long long)m0 * D - tap_start - (W - 1);
    const long long mmask = (long long)M - 1;
    const int stride = PD ? 2 : 1;
    const long long* lb = (const long long*)bins + (int64_t)line * ns * stride;
    // the last block of a line may hold fewer than per_cta outputs: stage only
    // the columns its threads read
    const int valid = min(per_cta, nd - m0);
    const int cols_used = min(cols, ((valid + CONV_K - 1) / CONV_K) * CONV_K + (cols - CONV_K * (int)blockDim.x));
    // element q of the segment (column q / D, phase q % D) is bin jbase + q:
    // consecutive threads read consecutive bins, 8 loads in flight per thread
    const int nelem = cols_used * D;
    const int step_c = blockDim.x / D, step_p = blockDim.x - step_c * D;
    const int big_c = (8 * blockDim.x) / D, big_p = 8 * blockDim.x - big_c * D;
    int col_t = tid / D, ph_t = tid - col_t * D;   // (column, phase) of element q0
    for (int q0 = tid; q0 < nelem; q0 += 8 * blockDim.x) {
        longlong2 v[8];
        int jj[NZ ? 8 : 1];
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const int q = q0 + u * (int)blockDim.x;
            const long long j = (jbase + q) & mmask;
            v[u] = make_longlong2(0, 0);
            if (NZ) jj[u] = (q < nelem && j < ns) ? (int)j : -1;
            if (q < nelem && j < ns) {
                if (PD) v[u] = __ldg(reinterpret_cast<const longlong2*>(lb) + j);
                else v[u].x = __ldg(lb + j);
            }
        }
        int c = col_t, p = ph_t;
#pragma unroll
        for (int u = 0; u < 8; u++) {
            if (q0 + u * (int)blockDim.x < nelem) {
                float2 val = make_float2(fix2f(v[u].x, inv_scale), PD ? fix2f(v[u].y, inv_scale) : 0.0f);
                if (NZ && jj[u] >= 0) {
                    const float2 n = bin_noise(nz, nz.line0 + line, jj[u]);
                    val.x += n.x;
                    val.y += n.y;
                }
                seg[p * row + (c & 3) * sub + (c >> 2)] = val;
            }
            c += step_c;
            p += step_p;
            if (p >= D) { p -= D; c++; }
        }
        col_t += big_c;
        ph_t += big_p;
        if (ph_t >= D) { ph_t -= D; col_t++; }
    }
    __syncthreads();
    if (tid * CONV_K >= valid) return;   // no output of this thread (no barrier follows)
    float2 ys[CONV_K];
    fir_mac<CX, TAPS_SMEM>(seg, row, sub, tid, tp4, taps_pm, ph_off, D, ys);
    fir_store(ys, line, m0, tid, nd, demod, out);
}

// Staged elements per phase row for `outputs` outputs: thread T's window reaches
// element 4T + max_ph_taps + 2, so 4*ceil(outputs/4) + max_ph_taps elements
// (max_ph_taps is a multiple of 4) cover every read.
static int conv_cols(int outputs, int max_ph_taps) {
    return (outputs + CONV_K - 1) / CONV_K * CONV_K + max_ph_taps;
}
// Sub-row length: cols/4 positions, odd.
static int conv_sub(int cols) { return (cols / 4) | 1; }
static int conv_row(int cols) {
    const int sub = conv_sub(cols);
    return 4 * sub + conv_rowpad(sub);
}

cudaError_t launch_convolve_demodulate(const unsigned long long* bins, int num_lines, int ns, int phase_delay,
                                       float inv_scale, const float2* taps_pm, const int* ph_off, int ntaps_pm,
                                       int max_ph_taps, int W, int tap_start, int64_t M, int center, int decimation,
                                       int nd, const float2* demod, float2* out, cudaStream_t stream,
                                       const NoiseParams* noise) {
    if (num_lines <= 0 || nd <= 0) return cudaSuccess;
    if (max_ph_taps % 4) return cudaErrorInvalidValue;
    NoiseParams nz{};
    const bool noisy = noise && noise->sigma > 0.0f;
    if (noisy) nz = *noise;
    const int D = decimation;
    int dev = 0, sms = 0, smem_optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return e;
    const size_t limit = std::min<size_t>(200 * 1024, (size_t)smem_optin);

    // a line's outputs split evenly over blocks of at most 128 threads (4
    // outputs each; no block left nearly empty), more blocks per line only
    // while the grid has fewer CTAs than SMs (more, smaller blocks per line
    // measured slower: more halo per output, and a second partial wave where
    // the first would have held the grid)
    auto threads_for = [&](int64_t blocks) {
        const int64_t per = (nd + blocks - 1) / blocks;
        return (int)std::max<int64_t>(32, ((per + CONV_K - 1) / CONV_K + 31) / 32 * 32);
    };

    int64_t nblk = (nd + 128 * CONV_K - 1) / (128 * CONV_K);
    int threads = threads_for(nblk);
    while (threads > 32 && (int64_t)num_lines * nblk < sms) threads = threads_for(++nblk);
    auto smem_for = [&](int th, int taps_smem) {
        return (size_t)D * conv_row(conv_cols(th * CONV_K, max_ph_taps)) * sizeof(float2) +
               (taps_smem ? (size_t)ntaps_pm * sizeof(float4) : 0);
    };
    int taps_in_smem = 1;
    if (smem_for(threads, 1) > limit) taps_in_smem = 0;   // very long windows: taps from global memory (broadcast loads)
    while (smem_for(threads, taps_in_smem) > limit && threads > 32) threads -= 32;
    const size_t smem = smem_for(threads, taps_in_smem);
    if (smem > limit) return cudaErrorInvalidValue;
    const int cols = conv_cols(threads * CONV_K, max_ph_taps);
    const int sub = conv_sub(cols), row = conv_row(cols);
    nblk = (nd + threads * CONV_K - 1) / (threads * CONV_K);
    const dim3 grid((unsigned)nblk, (unsigned)num_lines);
    auto launch = [&](auto k) -> cudaError_t {
        cudaError_t e2 = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e2 != cudaSuccess) return e2;
        k<<<grid, threads, smem, stream>>>(bins, ns, inv_scale, taps_pm, ph_off, W, tap_start, M, center, D, nd, sub,
                                           row, cols, demod, out, nz);
        return cudaGetLastError();
    };
    if (noisy) {
        if (phase_delay) return taps_in_smem ? launch(convolve_demodulate_kernel<true, true, true>)
                                             : launch(convolve_demodulate_kernel<true, false, true>);
        return taps_in_smem ? launch(convolve_demodulate_kernel<false, true, true>)
                            : launch(convolve_demodulate_kernel<false, false, true>);
    }
    if (phase_delay) return taps_in_smem ? launch(convolve_demodulate_kernel<true, true, false>)
                                         : launch(convolve_demodulate_kernel<true, false, false>);
    return taps_in_smem ? launch(convolve_demodulate_kernel<false, true, false>)
                        : launch(convolve_demodulate_kernel<false, false, false>);
}

int make_phase_major_taps(const float2* taps, int W, int D, float2* out, int* off, int* max_ph) {
    // the excitation's support: real parts above 1e-9 of the largest (outside
    // it the FP64 analytic pulse's real part is rounding residue, set to 0)
    float re_max = 0.0f;
    for (int w = 0; w < W; w++) re_max = std::max(re_max, std::fabs(taps[w].x));
    const float thr = 1e-9f * re_max;
    int n = 0, mx = 0;
    for (int ph = 0; ph < D; ph++) {
        off[ph] = n;
        const int cnt = ph <= W - 1 ? (W - 1 - ph) / D + 1 : 0;
        const int pad = (cnt + 3) / 4 * 4;
        int lo = pad / 4, hi = 0;   // 4-tap iterations holding support taps
        for (int t = 0; t < pad; t++) {
            float2 v = make_float2(0.0f, 0.0f);
            if (t < cnt) {
                v = taps[W - 1 - (ph + t * D)];
                if (std::fabs(v.x) <= thr) v.x = 0.0f;
            }
            out[n + t] = v;
            if (v.x != 0.0f) {
                lo = std::min(lo, t / 4);
                hi = std::max(hi, t / 4 + 1);
            }
        }
        if (hi <= lo) lo = hi = 0;
        off[D + 1 + 2 * ph] = lo;
        off[D + 2 + 2 * ph] = hi;
        n += pad;
        mx = pad > mx ? pad : mx;
    }
    off[D] = n;
    *max_ph = mx;
    return n;
}

}  // namespace bcsim_gb300
