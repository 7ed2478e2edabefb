// imaging.cu -- device post-processing of simulated IQ: B-mode (envelope, log
// compression, scan conversion) and colour Doppler (autocorrelation estimates
// of a packet, power threshold, colour map).
//
// The reference does this on the host, after simulate_lines, in its GUI's
// refresh worker (src/qt5gui/RefreshWorker.hpp:179-395) with the helpers of
// src/utils/BCSimConvenience.cpp:57-83 and the polar/linear-to-Cartesian
// resampler src/utils/cartesianator/Cartesianator.cpp:107-205.  Here each step
// is one kernel over device-resident IQ; every float expression follows the
// reference's operation order with explicitly rounded (unfused) operations, so
// that results agree with it to the last bit except where a libm function
// (log10f, atan2f) rounds differently from CUDA's -- the tests state those
// tolerances.
//
// Layouts (as the reference's): IQ frames complex64 [line][sample]; packets
// [frame][line][sample]; beam space [beam][range] (range fastest); images
// [y][x] with x fastest, colour images 4 bytes per pixel (B, G, R, A).
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>
#include "imaging.hpp"

namespace bcsim_gb300 {

// ---------------------------------------------------------------------------
// deterministic maxima (max is exact and order-independent; two passes)
// ---------------------------------------------------------------------------
constexpr int MAX_BLOCKS = 256;
constexpr int MAX_THREADS = 256;

__device__ __forceinline__ float envelope(float2 z) {
    // |z| = sqrt(re^2 + im^2) (std::abs of std::complex<float>), unfused
    return __fsqrt_rn(__fadd_rn(__fmul_rn(z.x, z.x), __fmul_rn(z.y, z.y)));
}

template <bool ENVELOPE>
__global__ void __launch_bounds__(MAX_THREADS) max_partial_kernel(const void* __restrict__ data, int64_t n,
                                                                  float* __restrict__ partial) {
    __shared__ float s[MAX_THREADS / 32];
    float m = -INFINITY;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float v = ENVELOPE ? envelope(__ldg(static_cast<const float2*>(data) + i))
                                 : __ldg(static_cast<const float*>(data) + i);
        m = fmaxf(m, v);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = s[0];
        for (int k = 1; k < (int)(blockDim.x >> 5); k++) t = fmaxf(t, s[k]);
        partial[blockIdx.x] = t;
    }
}

__global__ void max_final_kernel(const float* __restrict__ partial, int count, float* __restrict__ out) {
    float m = -INFINITY;
    for (int i = threadIdx.x; i < count; i += 32) m = fmaxf(m, partial[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) *out = m;
}

static cudaError_t launch_max(bool env, const void* data, int64_t n, float* scratch, float* out, cudaStream_t st) {
    if (n <= 0) return cudaErrorInvalidValue;
    const int blocks = (int)std::min<int64_t>(MAX_BLOCKS, (n + MAX_THREADS - 1) / MAX_THREADS);
    if (env) max_partial_kernel<true><<<blocks, MAX_THREADS, 0, st>>>(data, n, scratch);
    else max_partial_kernel<false><<<blocks, MAX_THREADS, 0, st>>>(data, n, scratch);
    max_final_kernel<<<1, 32, 0, st>>>(scratch, blocks, out);
    return cudaGetLastError();
}

size_t imaging_max_scratch_floats() { return MAX_BLOCKS; }

cudaError_t launch_envelope_max(const float2* iq, int64_t n, float* scratch, float* out, cudaStream_t st) {
    return launch_max(true, iq, n, scratch, out, st);
}

cudaError_t launch_value_max(const float* v, int64_t n, float* scratch, float* out, cudaStream_t st) {
    return launch_max(false, v, n, scratch, out, st);
}

// ---------------------------------------------------------------------------
// B-mode beam space: envelope, log compression, bytes
// ---------------------------------------------------------------------------
// One sample (BCSimConvenience.cpp:65-83 and the byte conversion of
// RefreshWorker.hpp:226-236):
//   p = (float)(20.0 * log10f(gain * env / normalize))
//   p = (float)((255.0 / dyn_range) * (p + dyn_range)), clamped to [0, 255]
//   byte = (unsigned char)p (truncation)
// 20.0 * (float) is exact in double, so the first line is one float rounding;
// the second is evaluated in double as the reference does.
__global__ void log_compress_kernel(const float2* __restrict__ iq, int64_t n, double k255, float dyn_range,
                                    float gain, const float* __restrict__ normalize, uint8_t* __restrict__ out) {
    const float norm = *normalize;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float env = envelope(__ldg(iq + i));
        float p = __fmul_rn(20.0f, log10f(__fdiv_rn(__fmul_rn(gain, env), norm)));
        p = (float)(k255 * ((double)p + (double)dyn_range));
        if (p < 0.0f) p = 0.0f;
        if (p >= 255.0f) p = 255.0f;
        out[i] = (uint8_t)(unsigned)p;   // p in [0, 255] (NaN compares false: -> 0 below)
    }
}

cudaError_t launch_log_compress(const float2* iq, int64_t n, float dyn_range, float gain, const float* normalize_dev,
                                uint8_t* out, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int threads = 256;
    const int blocks = (int)std::min<int64_t>(4096, (n + threads - 1) / threads);
    log_compress_kernel<<<blocks, threads, 0, st>>>(iq, n, 255.0 / (double)dyn_range, dyn_range, gain, normalize_dev,
                                                    out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// scan conversion (CpuCartesianator<T>::DoSectorTransform / DoLinearTransform)
// ---------------------------------------------------------------------------
// Constants the host derives from the geometry exactly as the reference's
// SetGeometry / get_xy_extent / get_angle_limits do (float arithmetic).
struct ScanConst {
    int kind;
    int nx, ny, beams, range;
    float x_min, y_min, dx, dy;   // output grid
    float a_min, da;              // beam axis: theta (sector) or x (linear)
    float r_min, dr;              // range axis: r (sector) or y (linear)
    float half_pi;                // (float)(atan(1) * 2), the sector's theta where |x| <= 1e-6
};

template <typename T>
__device__ __forceinline__ float sample_at(const T* __restrict__ in, int range, int beams, int ri, int bi) {
    return (ri >= 0 && ri < range && bi >= 0 && bi < beams) ? (float)__ldg(in + (int64_t)range * bi + ri) : 0.0f;
}

// The interpolation of both transforms: value at (r, a) from the four samples
// around it, "Wikipedia formula" (Cartesianator.cpp:150-154 and 197-200).
template <typename T>
__device__ __forceinline__ float bilinear(const T* __restrict__ in, const ScanConst& c, float r, float a) {
    const int ri0 = (int)floorf(__fdiv_rn(__fsub_rn(r, c.r_min), c.dr));
    const int ai0 = (int)floorf(__fdiv_rn(__fsub_rn(a, c.a_min), c.da));
    const int ri1 = ri0 + 1, ai1 = ai0 + 1;
    const float s00 = sample_at(in, c.range, c.beams, ri0, ai0);
    const float s01 = sample_at(in, c.range, c.beams, ri0, ai1);
    const float s10 = sample_at(in, c.range, c.beams, ri1, ai0);
    const float s11 = sample_at(in, c.range, c.beams, ri1, ai1);
    const float r0 = __fadd_rn(c.r_min, __fmul_rn((float)ri0, c.dr));
    const float r1 = __fadd_rn(r0, c.dr);
    const float a0 = __fadd_rn(c.a_min, __fmul_rn((float)ai0, c.da));
    const float a1 = __fadd_rn(a0, c.da);
    const float w = __fdiv_rn(1.0f, __fmul_rn(__fsub_rn(r1, r0), __fsub_rn(a1, a0)));
    float acc = __fmul_rn(__fmul_rn(s00, __fsub_rn(r1, r)), __fsub_rn(a1, a));
    acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(s10, __fsub_rn(r, r0)), __fsub_rn(a1, a)));
    acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(s01, __fsub_rn(r1, r)), __fsub_rn(a, a0)));
    acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(s11, __fsub_rn(r, r0)), __fsub_rn(a, a0)));
    return __fmul_rn(w, acc);
}

// Output pixel (xi, yi) -> its (range, beam-axis) coordinates.
__device__ __forceinline__ void pixel_coords(const ScanConst& c, int xi, int yi, float* r, float* a) {
    const float x = __fadd_rn(c.x_min, __fmul_rn((float)xi, c.dx));
    const float y = __fadd_rn(c.y_min, __fmul_rn((float)yi, c.dy));
    if (c.kind == SCAN_SECTOR) {
        *r = __fsqrt_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)));
        // std::abs(x) > 1e-6 compares in double (Cartesianator.cpp:128)
        *a = (double)fabsf(x) > 1e-6 ? atan2f(y, x) : c.half_pi;
    } else {
        *r = y;
        *a = x;
    }
}

// (unsigned char)(float) as the reference's x86 build performs it: truncation
// to a 32-bit integer, then its low byte.
__device__ __forceinline__ uint8_t to_byte(float v) { return (uint8_t)(unsigned)__float2int_rz(v); }

template <typename T>
__global__ void scan_convert_kernel(const T* __restrict__ in, ScanConst c, T* __restrict__ out) {
    const int xi = blockIdx.x * blockDim.x + threadIdx.x;
    const int yi = blockIdx.y;
    if (xi >= c.nx) return;
    float r, a;
    pixel_coords(c, xi, yi, &r, &a);
    const float v = bilinear(in, c, r, a);
    T o;
    if constexpr (sizeof(T) == 1) o = to_byte(v);
    else o = v;
    out[(int64_t)c.nx * yi + xi] = o;
}

static ScanConst scan_const(const ScanGeometry2D& g, int beams, int range) {
    ScanConst c{};
    c.kind = g.kind;
    c.nx = g.nx;
    c.ny = g.ny;
    c.beams = beams;
    c.range = range;
    float x_max, y_max;
    if (g.kind == SCAN_SECTOR) {
        // SectorScanGeometry::get_angle_limits / get_xy_extent (ScanGeometry.hpp:49-63)
        const float pi = static_cast<float>(4.0 * std::atan(1.0f));
        const float min_angle = 0.5f * pi - 0.5f * g.width + g.tilt;
        const float max_angle = 0.5f * pi + 0.5f * g.width + g.tilt;
        c.x_min = static_cast<float>(g.depth * std::cos(max_angle));
        x_max = static_cast<float>(g.depth * std::cos(min_angle));
        c.y_min = 0.0f;
        y_max = g.depth;
        c.r_min = 0.0f;
        c.dr = (g.depth - c.r_min) / (range - 1);
        c.a_min = min_angle;
        c.da = (max_angle - min_angle) / (beams - 1);
    } else {
        // LinearScanGeometry::get_xy_extent (ScanGeometry.hpp:72-77), beam-space
        // limits of DoLinearTransform (Cartesianator.cpp:168-176)
        c.x_min = -0.5f * g.width;
        x_max = 0.5f * g.width;
        c.y_min = 0.0f;
        y_max = g.depth;
        c.a_min = c.x_min;
        c.da = (x_max - c.x_min) / (beams - 1);
        c.r_min = 0.0f;
        c.dr = (y_max - c.r_min) / (range - 1);
    }
    c.dx = (x_max - c.x_min) / (float)(g.nx - 1);
    c.dy = (y_max - c.y_min) / (float)(g.ny - 1);
    c.half_pi = static_cast<float>(std::atan(1.0) * 2);
    return c;
}

template <typename T>
static cudaError_t launch_scan(const T* in, int beams, int range, const ScanGeometry2D& g, T* out, cudaStream_t st) {
    const ScanConst c = scan_const(g, beams, range);
    const dim3 grid((unsigned)((g.nx + 127) / 128), (unsigned)g.ny);
    scan_convert_kernel<T><<<grid, 128, 0, st>>>(in, c, out);
    return cudaGetLastError();
}

cudaError_t launch_scan_convert_u8(const uint8_t* in, int beams, int range, const ScanGeometry2D& g, uint8_t* out,
                                   cudaStream_t st) {
    return launch_scan(in, beams, range, g, out, st);
}

cudaError_t launch_scan_convert_f32(const float* in, int beams, int range, const ScanGeometry2D& g, float* out,
                                    cudaStream_t st) {
    return launch_scan(in, beams, range, g, out, st);
}

// ---------------------------------------------------------------------------
// colour Doppler
// ---------------------------------------------------------------------------
// Per (line, sample) over a packet of P frames (RefreshWorker.hpp:268-300):
//   mean = sum_k x_k / P                      (clutter filter)
//   R0   = sum_k |x_k - mean|^2
//   R1   = sum_{k<P-1} conj(x_k) x_{k+1}      (of the unfiltered samples)
//   velocity = arg(R1)
// with std::complex<float> arithmetic unfused, in the reference's order.
__global__ void doppler_kernel(const float2* __restrict__ packet, int P, int64_t n, float* __restrict__ r0_out,
                               float* __restrict__ vel_out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float mr = 0.0f, mi = 0.0f;
        for (int k = 0; k < P; k++) {
            const float2 z = __ldg(packet + (int64_t)k * n + i);
            mr = __fadd_rn(mr, z.x);
            mi = __fadd_rn(mi, z.y);
        }
        const float fp = (float)P;
        mr = __fdiv_rn(mr, fp);
        mi = __fdiv_rn(mi, fp);
        float r0 = 0.0f, r1r = 0.0f, r1i = 0.0f;
        float2 prev = make_float2(0.0f, 0.0f);
        for (int k = 0; k < P; k++) {
            const float2 x = __ldg(packet + (int64_t)k * n + i);
            const float a = __fsub_rn(x.x, mr), b = __fsub_rn(x.y, mi);
            // (z * conj(z)).real() = a*a - b*(-b)
            r0 = __fadd_rn(r0, __fsub_rn(__fmul_rn(a, a), __fmul_rn(b, -b)));
            if (k > 0) {
                // conj(prev) * x = (p.re, -p.im) * (x.re, x.im)
                const float re = __fsub_rn(__fmul_rn(prev.x, x.x), __fmul_rn(-prev.y, x.y));
                const float im = __fadd_rn(__fmul_rn(prev.x, x.y), __fmul_rn(-prev.y, x.x));
                r1r = __fadd_rn(r1r, re);
                r1i = __fadd_rn(r1i, im);
            }
            prev = x;
        }
        if (r0_out) r0_out[i] = r0;
        if (vel_out) vel_out[i] = atan2f(r1i, r1r);
    }
}

cudaError_t launch_doppler(const float2* packet, int P, int64_t n, float* r0, float* vel, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int threads = 256;
    const int blocks = (int)std::min<int64_t>(8192, (n + threads - 1) / threads);
    doppler_kernel<<<blocks, threads, 0, st>>>(packet, P, n, r0, vel);
    return cudaGetLastError();
}

// Colour image (RefreshWorker.hpp:326-395): power R0 / max R0 scan converted
// and thresholded at 0.001; velocity scan converted; a thresholded pixel gets
// alpha 255 and 255 |v| / 3.14159 in red (v >= 0) or blue (v < 0).  Pixels
// below the threshold are (0, 0, 0, 0) (the reference leaves their red and
// blue bytes uninitialised).  Normalising the beam-space power sample by
// sample before the interpolation, as the reference's buffer does.
__global__ void color_image_kernel(const float* __restrict__ r0, const float* __restrict__ vel,
                                   const float* __restrict__ r0_max, ScanConst c, uchar4* __restrict__ out) {
    const int xi = blockIdx.x * blockDim.x + threadIdx.x;
    const int yi = blockIdx.y;
    if (xi >= c.nx) return;
    const float mx = *r0_max;
    float r, a;
    pixel_coords(c, xi, yi, &r, &a);
    // power: the same interpolation over normalised samples
    const int ri0 = (int)floorf(__fdiv_rn(__fsub_rn(r, c.r_min), c.dr));
    const int ai0 = (int)floorf(__fdiv_rn(__fsub_rn(a, c.a_min), c.da));
    auto pw = [&](int ri, int ai) {
        return (ri >= 0 && ri < c.range && ai >= 0 && ai < c.beams)
                   ? __fdiv_rn(__ldg(r0 + (int64_t)c.range * ai + ri), mx)
                   : 0.0f;
    };
    const float s00 = pw(ri0, ai0), s01 = pw(ri0, ai0 + 1), s10 = pw(ri0 + 1, ai0), s11 = pw(ri0 + 1, ai0 + 1);
    const float rr0 = __fadd_rn(c.r_min, __fmul_rn((float)ri0, c.dr));
    const float rr1 = __fadd_rn(rr0, c.dr);
    const float aa0 = __fadd_rn(c.a_min, __fmul_rn((float)ai0, c.da));
    const float aa1 = __fadd_rn(aa0, c.da);
    const float w = __fdiv_rn(1.0f, __fmul_rn(__fsub_rn(rr1, rr0), __fsub_rn(aa1, aa0)));
    float acc = __fmul_rn(__fmul_rn(s00, __fsub_rn(rr1, r)), __fsub_rn(aa1, a));
    acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(s10, __fsub_rn(r, rr0)), __fsub_rn(aa1, a)));
    acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(s01, __fsub_rn(rr1, r)), __fsub_rn(a, aa0)));
    acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(s11, __fsub_rn(r, rr0)), __fsub_rn(a, aa0)));
    const float power = __fmul_rn(w, acc);
    uchar4 px = make_uchar4(0, 0, 0, 0);   // (B, G, R, A)
    if (power >= 0.001f) {
        const float v = bilinear(vel, c, r, a);
        const uint8_t cv = to_byte(__fdiv_rn(__fmul_rn(255.0f, fabsf(v)), 3.14159f));
        px.w = 255;
        if (v >= 0.0f) px.z = cv;
        else px.x = cv;
    }
    out[(int64_t)c.nx * yi + xi] = px;
}

cudaError_t launch_color_image(const float* r0, const float* vel, const float* r0_max_dev, int beams, int range,
                               const ScanGeometry2D& g, uint8_t* bgra, cudaStream_t st) {
    const ScanConst c = scan_const(g, beams, range);
    const dim3 grid((unsigned)((g.nx + 127) / 128), (unsigned)g.ny);
    color_image_kernel<<<grid, 128, 0, st>>>(r0, vel, r0_max_dev, c, reinterpret_cast<uchar4*>(bgra));
    return cudaGetLastError();
}

}  // namespace bcsim_gb300
