// project.cu -- scatterer -> scan-line time projection on sm_103a.
//
// Semantics follow the reference CPU projection loops
// (src/core/algorithm/CpuAlgorithm.cpp:50-183): for every (scatterer, line)
// pair the scatterer is expressed in the line's frame (r, l, e), the radial
// coordinate is replaced by the signed distance to the origin when arc
// projection is on, the bin index is floor(r * 2 fs / c + 0.5), the beam weight
// is the Gaussian of src/core/BeamProfile.cpp:49-51 or the trilinear lookup of
// src/core/BeamProfile.cpp:79-130, and (optionally) the sub-sample delay is
// applied as a phase (CpuAlgorithm.cpp:85-95).
//
// Two paths:
//  * shared origin (every line starts at the same point, arc projection on):
//    the distance to the origin -- and therefore the bin index and the phase --
//    does not depend on the line.  prep computes them once per scatterer in FP64
//    (bit-identical to the FP64 oracle's expression), the records are radix
//    sorted by bin, and the projection kernel walks runs of equal bins with the
//    line frame in registers, summing in FP32 registers and flushing each run
//    once per line into fixed-point bins.
//  * per pair (any geometry, splines): the time of flight is computed per pair
//    with float-pair arithmetic, each non-zero contribution goes to the bins.
//
// Bins are signed 64-bit fixed point (value * 2^S); integer addition is
// associative, so the result does not depend on the order in which CTAs,
// warps or atomics land: the accumulation is deterministic by construction,
// where the reference's GPU path (cuda_kernels_fixed.cuh:59-62) uses float
// atomics whose order varies from run to run.
#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>
#include <cub/device/device_radix_sort.cuh>
#include "kernels.hpp"
#include "dfloat.cuh"
#include "fixedpoint.cuh"
#include "async_copy.cuh"

namespace bcsim_gb300 {

static constexpr double TWO_PI_LITERAL = 6.283185307179586;  // CpuAlgorithm.cpp:89,175

// ---------------------------------------------------------------------------
// fixed-point accumulation
// ---------------------------------------------------------------------------
__device__ __forceinline__ void bin_add(unsigned long long* addr, float v, float scale) {
    if (v != 0.0f) {
        const long long q = f2ll_rn_bounded(v * scale);
        if (q != 0) atomicAdd(addr, (unsigned long long)q);
    }
}

// ---------------------------------------------------------------------------
// Lookup-table weight shared by both paths, float arithmetic, given the radial
// table coordinate (r0, fr) and the lateral/elevational positions.
// The packed table holds, at (r, l, e), the corners
// (c[r][l][e], c[r][l][e+1], c[r+1][l][e], c[r+1][l][e+1]).
// Valid coordinate range per axis is -1 < t < n-1 (the reference's index test
// for trunc-toward-zero indices, BeamProfile.cpp:94-103); for -1 < t < 0 both
// indices are 0 and the fraction is dropped.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float lut_weight_packed(const BeamDev& b, int r0, float fr, float tl, float te) {
    if (!(tl > -1.0f && tl < (float)(b.nl - 1) && te > -1.0f && te < (float)(b.ne - 1))) return 0.0f;
    const int l0 = (int)tl, e0 = (int)te;
    const float fl = tl < 0.0f ? 0.0f : tl - (float)l0;
    const float fe = te < 0.0f ? 0.0f : te - (float)e0;
    const int base = (r0 * b.nl + l0) * b.ne + e0;
    // (r0,l0,e0) (r0,l0,e1) and the radial differences to r1 at both, then the same at l1
    const float4 P = __ldg(b.lut4 + base);
    const float4 Q = __ldg(b.lut4 + base + b.ne);
    // radial, then lateral, then elevational interpolation (BeamProfile.cpp:116-127)
    const float c00 = __fmaf_rn(fr, P.z, P.x);
    const float c01 = __fmaf_rn(fr, P.w, P.y);
    const float c10 = __fmaf_rn(fr, Q.z, Q.x);
    const float c11 = __fmaf_rn(fr, Q.w, Q.y);
    const float c0 = __fmaf_rn(fl, c10 - c00, c00);
    const float c1 = __fmaf_rn(fl, c11 - c01, c01);
    return __fmaf_rn(fe, c1 - c0, c0);
}

// Lookup-table weight in the reference's own arithmetic (reference mode,
// BeamProfile.cpp:79-130): float differences divided by double spacings,
// trunc indices, float interpolation weights.
__device__ float lut_weight_ref(const BeamDev& b, float r, float l, float e) {
    const double tr = (double)__fsub_rn(r, b.rf) / b.dr;
    const double tl = (double)__fsub_rn(l, b.lf) / b.dl;
    const double te = (double)__fsub_rn(e, b.ef) / b.de;
    if (!(tr > -1.0 && tr < (double)(b.nr - 1))) return 0.0f;
    if (!(tl > -1.0 && tl < (double)(b.nl - 1))) return 0.0f;
    if (!(te > -1.0 && te < (double)(b.ne - 1))) return 0.0f;
    const int r0 = (int)tr, l0 = (int)tl, e0 = (int)te;
    const float fr = tr < 0.0 ? 0.0f : (float)(tr - r0);
    const float fl = tl < 0.0 ? 0.0f : (float)(tl - l0);
    const float fe = te < 0.0 ? 0.0f : (float)(te - e0);
    const int base = (r0 * b.nl + l0) * b.ne + e0;
    const float4 P = __ldg(b.lut4 + base);
    const float4 Q = __ldg(b.lut4 + base + b.ne);
    const float omr = __fsub_rn(1.0f, fr), oml = __fsub_rn(1.0f, fl), ome = __fsub_rn(1.0f, fe);
    const float c00 = __fadd_rn(__fmul_rn(omr, P.x), __fmul_rn(fr, P.z));
    const float c10 = __fadd_rn(__fmul_rn(omr, Q.x), __fmul_rn(fr, Q.z));
    const float c01 = __fadd_rn(__fmul_rn(omr, P.y), __fmul_rn(fr, P.w));
    const float c11 = __fadd_rn(__fmul_rn(omr, Q.y), __fmul_rn(fr, Q.w));
    const float c0 = __fadd_rn(__fmul_rn(oml, c00), __fmul_rn(fl, c10));
    const float c1 = __fadd_rn(__fmul_rn(oml, c01), __fmul_rn(fl, c11));
    return __fadd_rn(__fmul_rn(ome, c0), __fmul_rn(fe, c1));
}

// Gaussian weight in the reference's arithmetic (BeamProfile.cpp:49-56).
__device__ __forceinline__ float gauss_weight_ref(const BeamDev& b, float l, float e) {
    const float q = __fadd_rn(__fdiv_rn(__fmul_rn(l, l), b.two_sl2), __fdiv_rn(__fmul_rn(e, e), b.two_se2));
    return expf(-q);
}

// ---------------------------------------------------------------------------
// shared-origin prep
// ---------------------------------------------------------------------------
struct PrepOut {
    uint32_t key;
    float4 A, B;
};

// fp64 mode.  (dx, dy, dz): the scatterer relative to the origin in double
// and (px, py, pz) the same as float pairs; a: amplitude.  The distance and the
// time of flight t = |d| 2 fs / c are evaluated in float-pair arithmetic (about
// 2^-44 relative error); the bin index floor(t + 1/2) is taken from it unless t
// lies within 2^-36 t of a rounding boundary, where the FP64 oracle's own
// expression decides (fixed loop r*2*fs/c, CpuAlgorithm.cpp:75; spline loop
// r*2/(c*dt), :161-162) -- so the index is the oracle's for every scatterer.
// The sub-sample phase (CpuAlgorithm.cpp:85-92, |argument| <= pi fd/fs) and the
// lookup-table radial coordinate are FP32 / float-pair.
__device__ __forceinline__ PrepOut prep_fp64(double dx, double dy, double dz, df px, df py, df pz, float fdx,
                                             float fdy, float fdz, float a, const SimParams& p, const BeamDev& b,
                                             bool spline) {
    PrepOut o;
    // |d|^2 = sum hi^2 (exact products) + 2 hi lo, then its square root
    const df x2 = two_prod(px.hi, px.hi), y2 = two_prod(py.hi, py.hi), z2 = two_prod(pz.hi, pz.hi);
    const df s1 = two_sum(x2.hi, y2.hi);
    const df s2 = two_sum(s1.hi, z2.hi);
    float lo = s1.lo + s2.lo + x2.lo + y2.lo + z2.lo;
    lo = fmaf(2.0f * px.hi, px.lo, lo);
    lo = fmaf(2.0f * py.hi, py.lo, lo);
    lo = fmaf(2.0f * pz.hi, pz.lo, lo);
    const df rho = df_sqrt(fast_two_sum(s2.hi, lo));
    const df t = df_mul(rho, df_make(p.k_hi, p.k_lo));
    uint32_t key;
    int idx = 0;
    float delay = 0.0f;   // idx - t, samples
    if (!(t.hi < (float)p.ns + 1.0f)) {
        key = (uint32_t)p.ns + 1u;                // beyond the line end for every line (or NaN)
    } else {
        const float f = floorf(t.hi);
        const float g = (t.hi - f - 0.5f) + t.lo;   // t + 1/2 - (f + 1); t.hi - f and its difference with 1/2 are exact
        if (fabsf(g) <= fmaf(fabsf(t.hi), 0x1p-36f, 0x1p-60f)) {
            double t64;
            const double rho64 = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
            if (!spline) t64 = __ddiv_rn(__dmul_rn(__dmul_rn(rho64, 2.0), p.fs_d), p.c_d);
            else t64 = __ddiv_rn(__dmul_rn(rho64, 2.0), __dmul_rn(p.c_d, __ddiv_rn(1.0, p.fs_d)));
            const double fidx = floor(t64 + 0.5);
            idx = (int)fidx;
            delay = (float)(fidx - t64);
            if (!(fidx < (double)p.ns)) key = (uint32_t)p.ns + 1u;
            else if (t64 <= 0.5) key = (uint32_t)p.ns;
            else key = (uint32_t)idx;
        } else {
            idx = (int)f + (g >= 0.0f ? 1 : 0);
            delay = ((float)idx - t.hi) - t.lo;
            if (idx >= p.ns) key = (uint32_t)p.ns + 1u;
            else if ((t.hi - 0.5f) + t.lo <= 0.0f) key = (uint32_t)p.ns;   // near origin: a line behind may still hit bin 0
            else key = (uint32_t)idx;
        }
    }
    float Ar = a, Ai = 0.0f;
    if (p.phase_delay && key < (uint32_t)p.ns) {
        float sn, cs;
        sincosf(p.two_pi_fd_over_fs * delay, &sn, &cs);
        Ar = a * cs;
        Ai = a * sn;
    }
    int r0 = 0;
    float fr = 0.0f;
    if (b.type == BEAM_LUT && key < (uint32_t)p.ns) {
        // (|d| - r_first) / dr as a pair; valid for -1 < tr < nr-1 (BeamProfile.cpp:94-103)
        df q = two_sum(rho.hi, -b.rf);
        q = fast_two_sum(q.hi, q.lo + rho.lo);
        const df tr = df_mul(q, df_make(b.inv_dr, b.inv_dr_lo));
        if (!((tr.hi + 1.0f) + tr.lo > 0.0f && (tr.hi - (float)(b.nr - 1)) + tr.lo < 0.0f)) {
            key = (uint32_t)p.ns + 1u;            // radial coordinate outside the table: weight 0
        } else if (tr.hi + tr.lo > 0.0f) {
            float f = floorf(tr.hi);
            float rem = tr.hi - f;
            if (rem + tr.lo < 0.0f) { f -= 1.0f; rem += 1.0f; }
            r0 = (int)f;
            fr = rem + tr.lo;
        }                                          // -1 < tr <= 0: index 0, fraction dropped
    }
    o.key = key;
    o.A = make_float4(fdx, fdy, fdz, Ar);
    o.B = make_float4(Ai, fr, __int_as_float(r0), __int_as_float(idx));
    return o;
}

// Reference mode: the reference's float distance and its double index
// expression (fixed r*2*fs/c, CpuAlgorithm.cpp:75; spline r*2/(c*dt) with
// dt = float(1/fs), :161-162), float phase from a double delay (:85-92), and
// the lookup-table coordinate of BeamProfile.cpp:94-103.
__device__ __forceinline__ PrepOut prep_ref(float fdx, float fdy, float fdz, float a, const SimParams& p,
                                            const BeamDev& b, bool spline) {
    PrepOut o;
    const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(fdx, fdx), __fmul_rn(fdy, fdy)), __fmul_rn(fdz, fdz));
    const double rho = (double)__fsqrt_rn(r2);
    double t;
    if (!spline) {
        t = __ddiv_rn(__dmul_rn(__dmul_rn(rho, 2.0), p.fs_d), p.c_d);
    } else {
        const float dt = (float)(1.0 / p.fs_d);
        t = __ddiv_rn(__dmul_rn(rho, 2.0), (double)__fmul_rn(p.c, dt));
    }
    const double fidx = floor(t + 0.5);
    uint32_t key;
    if (!(t == t) || !(fidx < (double)p.ns)) {
        key = (uint32_t)p.ns + 1u;               // beyond the line end for every line
    } else if (t <= 0.5) {
        key = (uint32_t)p.ns;                    // near origin: a line behind may still hit bin 0
    } else {
        key = (uint32_t)fidx;
    }
    const int idx = (int)fidx;
    float Ar = a, Ai = 0.0f;
    if (p.phase_delay && key < (uint32_t)p.ns) {
        const float ss_delay = (float)(((double)idx - t) / p.fs_d);
        const float ph = (float)(TWO_PI_LITERAL * p.fd_d * (double)ss_delay);
        float sn, cs;
        sincosf(ph, &sn, &cs);
        Ar = __fmul_rn(a, cs);
        Ai = __fmul_rn(a, sn);
    }
    int r0 = 0;
    float fr = 0.0f;
    if (b.type == BEAM_LUT && key < (uint32_t)p.ns) {
        const double tr = (double)__fsub_rn((float)rho, b.rf) / b.dr;
        if (!(tr > -1.0 && tr < (double)(b.nr - 1))) {
            key = (uint32_t)p.ns + 1u;           // radial coordinate outside the table: weight 0
        } else {
            r0 = (int)tr;
            fr = tr < 0.0 ? 0.0f : (float)(tr - (double)r0);
        }
    }
    o.key = key;
    o.A = make_float4(fdx, fdy, fdz, Ar);
    o.B = make_float4(Ai, fr, __int_as_float(r0), __int_as_float(idx));
    return o;
}

// Angular cell of the direction (x, y, z) from the origin: the octahedral map
// of the unit sphere onto [-1, 1]^2, 2^(bits/2) cells per axis, numbered in
// Morton order.  Records of one bin sorted by it form compact patches of
// directions, so that 32 consecutive records share a small bounding sphere.
__device__ __forceinline__ uint32_t dir_cell(float x, float y, float z, int bits) {
    const int h = bits >> 1;
    const float s = fabsf(x) + fabsf(y) + fabsf(z);
    if (h <= 0 || !(s > 0.0f)) return 0u;
    float px = x / s, py = y / s;
    if (z < 0.0f) {   // the lower hemisphere folded onto the corners
        const float qx = copysignf(1.0f - fabsf(py), px);
        const float qy = copysignf(1.0f - fabsf(px), py);
        px = qx;
        py = qy;
    }
    const int m = (1 << h) - 1;
    const float half_n = 0.5f * (float)(1 << h);
    const uint32_t ix = (uint32_t)min(max((int)((px + 1.0f) * half_n), 0), m);
    const uint32_t iy = (uint32_t)min(max((int)((py + 1.0f) * half_n), 0), m);
    uint32_t c = 0;
    for (int k = 0; k < h; k++) c |= (((ix >> k) & 1u) << (2 * k)) | (((iy >> k) & 1u) << (2 * k + 1));
    return c;
}

// The sort key of a record: its bin (or ns / ns + 1 for the near-origin and the
// out-of-range ones) above its angular cell.
__device__ __forceinline__ uint32_t record_key(const PrepOut& o, const SimParams& p) {
    const uint32_t cell = o.key < (uint32_t)p.ns ? dir_cell(o.A.x, o.A.y, o.A.z, p.cell_bits) : 0u;
    return (o.key << p.cell_bits) | cell;
}

__global__ void prep_shared_kernel(const float4* __restrict__ xyza, int64_t n, int64_t off, double ox, double oy,
                                   double oz, float ofx, float ofy, float ofz, SimParams p, BeamDev b,
                                   uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                   float4* __restrict__ recA, float4* __restrict__ recB) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 q = __ldg(xyza + i);
    PrepOut o;
    if (p.mode == MODE_FP64) {
        // q - origin: exact as float pairs and in double
        const df px = two_sum(q.x, -ofx), py = two_sum(q.y, -ofy), pz = two_sum(q.z, -ofz);
        const double dx = __dsub_rn((double)q.x, ox), dy = __dsub_rn((double)q.y, oy), dz = __dsub_rn((double)q.z, oz);
        o = prep_fp64(dx, dy, dz, px, py, pz, px.hi, py.hi, pz.hi, q.w, p, b, false);
    } else {
        o = prep_ref(__fsub_rn(q.x, ofx), __fsub_rn(q.y, ofy), __fsub_rn(q.z, ofz), q.w, p, b, false);
    }
    keys[off + i] = record_key(o, p);
    vals[off + i] = (uint32_t)(off + i);
    recA[off + i] = o.A;
    recB[off + i] = o.B;
}

// Spline scatterers at one common timestamp: position = sum_i B_i * C_i over the
// degree+1 non-zero basis functions, in double (fp64 mode) or in the reference's
// float accumulation (reference mode, CpuAlgorithm.cpp:137-140).
__global__ void prep_shared_spline_kernel(const float4* __restrict__ cps, const float* __restrict__ amps, int64_t n,
                                          int first_cs, int degree, const double* __restrict__ bd,
                                          const float* __restrict__ bf, int64_t off, double ox, double oy,
                                          double oz, float ofx, float ofy, float ofz, SimParams p, BeamDev b,
                                          uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                          float4* __restrict__ recA, float4* __restrict__ recB) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double px = 0.0, py = 0.0, pz = 0.0;
    float fx = 0.0f, fy = 0.0f, fz = 0.0f;
    for (int k = 0; k <= degree; k++) {
        const float4 c = __ldg(cps + (int64_t)(first_cs + k) * n + i);
        if (p.mode == MODE_FP64) {
            px = __dadd_rn(px, __dmul_rn((double)c.x, bd[k]));
            py = __dadd_rn(py, __dmul_rn((double)c.y, bd[k]));
            pz = __dadd_rn(pz, __dmul_rn((double)c.z, bd[k]));
        } else {
            fx = __fadd_rn(fx, __fmul_rn(c.x, bf[k]));
            fy = __fadd_rn(fy, __fmul_rn(c.y, bf[k]));
            fz = __fadd_rn(fz, __fmul_rn(c.z, bf[k]));
        }
    }
    PrepOut o;
    if (p.mode == MODE_FP64) {
        const double dx = __dsub_rn(px, ox), dy = __dsub_rn(py, oy), dz = __dsub_rn(pz, oz);
        // the double offsets as float pairs (48 of their 53 bits)
        const float hx = __double2float_rn(dx), hy = __double2float_rn(dy), hz = __double2float_rn(dz);
        const df qx = fast_two_sum(hx, __double2float_rn(__dsub_rn(dx, (double)hx)));
        const df qy = fast_two_sum(hy, __double2float_rn(__dsub_rn(dy, (double)hy)));
        const df qz = fast_two_sum(hz, __double2float_rn(__dsub_rn(dz, (double)hz)));
        o = prep_fp64(dx, dy, dz, qx, qy, qz, hx, hy, hz, __ldg(amps + i), p, b, true);
    } else {
        o = prep_ref(__fsub_rn(fx, ofx), __fsub_rn(fy, ofy), __fsub_rn(fz, ofz), __ldg(amps + i), p, b, true);
    }
    keys[off + i] = record_key(o, p);
    vals[off + i] = (uint32_t)(off + i);
    recA[off + i] = o.A;
    recB[off + i] = o.B;
}

// Boundaries of the sorted keys (bin = key >> cell_bits): counts[2] = first
// index with bin >= ns, counts[3] = first index with bin > ns (both n if absent).
__global__ void init_counts_kernel(int* counts, int64_t n) {
    counts[0] = 0;
    counts[1] = 0;
    counts[2] = (int)n;
    counts[3] = (int)n;
}

__global__ void count_keys_kernel(const uint32_t* __restrict__ keys, int64_t n, int ns, int cell_bits, int* counts) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t k = keys[i] >> cell_bits;
    const bool first = i == 0;
    const uint32_t prev = first ? 0u : keys[i - 1] >> cell_bits;
    if (k >= (uint32_t)ns && (first || prev < (uint32_t)ns)) counts[2] = (int)i;
    if (k > (uint32_t)ns && (first || prev <= (uint32_t)ns)) counts[3] = (int)i;
}

// counts[0] = #keys < ns (records for the shared-origin kernel),
// counts[1] = #keys == ns (near-origin scatterers for the per-pair kernel).
__global__ void finish_counts_kernel(int* counts) {
    counts[0] = counts[2];
    counts[1] = counts[3] - counts[2];
}

// Sorted values -> the two record planes in bin order (plane B at out + plane).
__global__ void gather_records_kernel(const uint32_t* __restrict__ svals, const int* __restrict__ counts,
                                      int64_t n, const float4* __restrict__ recA, const float4* __restrict__ recB,
                                      float4* __restrict__ out, int64_t plane) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n || s >= (int64_t)__ldg(counts)) return;
    const uint32_t src = svals[s];
    out[s] = recA[src];
    out[plane + s] = recB[src];
}

// ---------------------------------------------------------------------------
// shared-origin projection
// ---------------------------------------------------------------------------
// The FP32 run sum of a line is folded into its integer bin total at absolute
// record indices k * p.fold (128 or 512, fixed per configuration; chunks are
// multiples of it), which bounds any FP32 summation to p.fold terms and keeps
// the result independent of the chunk size.

// Per-line constants of the shared-origin kernel (fp64 mode):
//   Gaussian: u = lateral * sqrt(gl), v = elevational * sqrt(ge), so that the
//             weight is exp2(-((d.u)^2 + (d.v)^2));
//   LUT:      u = lateral / dl, v = elevational / de, ou = -l_first / dl,
//             ov = -e_first / de: table coordinates tl = d.u + ou, te = d.v + ov.
struct LineK {
    float rx, ry, rz, ux, uy, uz, vx, vy, vz, ou, ov;
};

template <int BEAM, bool REF>
__device__ __forceinline__ LineK load_line(const LineGeom* g, const BeamDev& b) {
    LineK k;
    k.rx = __ldg(&g->d[0]); k.ry = __ldg(&g->d[1]); k.rz = __ldg(&g->d[2]);
    const float lx = __ldg(&g->l[0]), ly = __ldg(&g->l[1]), lz = __ldg(&g->l[2]);
    const float ex = __ldg(&g->e[0]), ey = __ldg(&g->e[1]), ez = __ldg(&g->e[2]);
    float su = 1.0f, sv = 1.0f;
    k.ou = 0.0f; k.ov = 0.0f;
    if (!REF) {
        if (BEAM == BEAM_GAUSSIAN) {
            su = sqrtf(b.gl); sv = sqrtf(b.ge);
        } else {
            su = b.inv_dl; sv = b.inv_de;
            k.ou = -b.lf * b.inv_dl; k.ov = -b.ef * b.inv_de;
        }
    }
    k.ux = lx * su; k.uy = ly * su; k.uz = lz * su;
    k.vx = ex * sv; k.vy = ey * sv; k.vz = ez * sv;
    return k;
}

// One CTA: a chunk of `chunk` (<= 1024) consecutive records, sorted by bin
// (and within a bin by the angular cell of their direction where bins are
// dense), staged once in shared memory by a TMA bulk copy; then the lines, in
// slots of 32 (one line per lane, in direction order so that a slot's lines
// point in nearby directions), are handed to the warps one slot at a time as
// the warps finish the previous one (walk lengths differ between slots), two
// phases per slot:
//   A. mask: where the records carry angular cells, one lane per 32-record
//      word first tests the word's bounding sphere against the slot box and
//      whole words are skipped; then each lane tests one record of the words
//      left against the warp's "slot box": the
//      lateral/elevational ranges outside which every line of the slot has
//      weight exactly 0 (the lookup table's extent, or where exp2 underflows),
//      widened by the spread of the slot's line frames (along the slot's
//      radial direction times the record's radial coordinate, normal to it times
//      the record's distance from the axis).  32 records per instruction; the
//      selection kept transposed (lane l, bit w: record 32 w + l).
//   B. walk: only the selected records, in bin order.  A line's
//      contributions to one bin are summed in FP32, folded into an int64 total
//      at absolute record indices k*p.fold, and written when the bin changes: a
//      plain store for bins strictly inside the chunk (no other CTA holds
//      records there), an integer atomic for the chunk's first and last bin.
// Skipped records contribute exactly 0, so the result is bit-identical to
// walking every record (cull=off), and does not depend on the chunk size.
template <bool PD, int BEAM, bool REF, int THREADS, bool COUNT>
__global__ void __launch_bounds__(THREADS, THREADS >= 1024 ? 1 : (THREADS >= 512 ? 2 : 3))
    project_shared_kernel(const float4* __restrict__ records, int64_t plane, const int* __restrict__ counts, int chunk,
                          const LineGeom* __restrict__ lines, const int* __restrict__ line_order,
                          const SlotCone* __restrict__ cones, int L, unsigned long long* __restrict__ bins,
                          SimParams p, BeamDev b, int lut_planes, unsigned long long* __restrict__ pair_counts) {
    extern __shared__ __align__(128) float4 sm[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ int s_lut_base, s_lut_planes, s_next_slot;
    // segments of the chunk: record index ranges [s_seg[k], s_seg[k+1]) within
    // one bin and one fold group (the walk folds and stores only at their ends)
    __shared__ int s_seg[1024 + 2];
    __shared__ unsigned short s_seg_of[1024];   // segment of each record
    __shared__ int s_seg_warp[32];
    const int n_valid = __ldg(counts);
    const int64_t start = (int64_t)blockIdx.x * chunk;
    if (start >= n_valid) return;
    const int cnt = (int)min((int64_t)chunk, (int64_t)n_valid - start);
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    float4* smA = sm;
    float4* smB = sm + chunk;
    // lut_planes radial planes of the packed table, rows padded to an odd number
    // of float4 so that the lanes' corner gathers spread over the banks
    float4* smL = sm + 2 * chunk;
    const int lut_plane_size = b.nl * b.ne;
    const int lut_row = b.ne | 1, lut_splane = b.nl * lut_row;

    if (tid == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // records are in bin order, so their radial table index r0 does not
        // decrease within the chunk: stage the planes from the first record's on
        int base = 0, planes = 0;
        if (BEAM == BEAM_LUT && !REF && lut_planes > 0) {
            base = __float_as_int(__ldg(&records[plane + start].z));
            base = min(max(base, 0), b.nr - 1);
            planes = min(lut_planes, b.nr - base);
        }
        s_lut_base = base;
        s_lut_planes = planes;
        s_next_slot = blockDim.x >> 5;
    }
    __syncthreads();
    const int lut_base = s_lut_base, lut_staged = s_lut_planes;
    if (tid == 0) {
        const unsigned bytes = (unsigned)cnt * sizeof(float4);
        mbar_expect_tx(&bar, 2 * bytes);
        bulk_load(smA, records + start, bytes, &bar);
        bulk_load(smB, records + plane + start, bytes, &bar);
    }
    if (lut_staged > 0) {   // (BEAM == BEAM_LUT only) while the records arrive
        const float4* src = b.lut4 + (int64_t)lut_base * lut_plane_size;
        for (int k = tid; k < lut_staged * lut_plane_size; k += blockDim.x) {
            const int pl = k / lut_plane_size, rem = k - pl * lut_plane_size;
            const int l = rem / b.ne, e = rem - l * b.ne;
            smL[pl * lut_splane + l * lut_row + e] = __ldg(src + k);
        }
        __syncthreads();
    }
    // bounded wait for the records, decided once for the whole CTA: thread 0
    // waits and publishes the outcome; if it gave up, the CTA sets the
    // simulator's error flag and leaves together (thread 0 first waits once
    // more, bounded, for the copy in flight).  Otherwise every thread observes
    // the completed phase itself (at once), which orders the bulk copy's
    // shared-memory writes before its reads.
    __shared__ int s_gave_up;
    if (tid == 0) s_gave_up = mbar_wait(&bar, 0, 1u << 26) ? 0 : 1;
    __syncthreads();
    if (s_gave_up) {
        if (tid == 0) {
            if (p.err_flag) atomicExch(p.err_flag, 1);
            mbar_wait(&bar, 0, 1u << 26);
        }
        return;
    }
    mbar_wait(&bar, 0, 1u << 26);

    const int stride = PD ? 2 : 1;
    const float scale = p.scale;
    // Do the staged planes hold every record's radial plane?  Then the walk
    // reads the table from shared memory without a per-record check, and each
    // record carries its plane's offset in shared memory (in B.z).
    __shared__ int s_r0_min, s_r0_max;
    bool all_staged = false;
    // 0x4B000000 = bits(2^23): the table indices' float bit patterns carry it
    const unsigned lut_addr0 = (unsigned)__cvta_generic_to_shared(smL) - 0x4B000000u * 16u * (unsigned)(lut_row + 1);
    if (BEAM == BEAM_LUT && !REF && lut_staged > 0) {
        if (tid == 0) {
            s_r0_min = 0x7fffffff;
            s_r0_max = -0x7fffffff;
        }
        __syncthreads();
        int mn = 0x7fffffff, mx = -0x7fffffff;
        for (int r = tid; r < cnt; r += blockDim.x) {
            const int r0 = __float_as_int(smB[r].z);
            mn = min(mn, r0);
            mx = max(mx, r0);
        }
        mn = __reduce_min_sync(0xffffffffu, mn);
        mx = __reduce_max_sync(0xffffffffu, mx);
        if (lane == 0) {
            atomicMin(&s_r0_min, mn);
            atomicMax(&s_r0_max, mx);
        }
        __syncthreads();
        all_staged = s_r0_min >= lut_base && s_r0_max < lut_base + lut_staged;
        if (all_staged) {
            for (int r = tid; r < cnt; r += blockDim.x)
                // the shared byte address of the record's plane, less the table
                // index bias: corner (l0, e0) of a pair then lies at
                // B.z + bits(l0 + 2^23) * 16 lut_row + bits(e0 + 2^23) * 16 (mod 2^32)
                smB[r].z = __uint_as_float(lut_addr0 + (unsigned)((__float_as_int(smB[r].z) - lut_base) * lut_splane) * 16u);
            __syncthreads();
        }
    }
    const int first_bin = __float_as_int(smB[0].w);
    const int last_bin = __float_as_int(smB[cnt - 1].w);
    // lookup-table coordinate ranges -1 < t < n-1 as |t - c| < h
    const float cl = 0.5f * (float)(b.nl - 2), hl = 0.5f * (float)b.nl;
    const float ce = 0.5f * (float)(b.ne - 2), he = 0.5f * (float)b.ne;
    const bool cull = !REF && p.cull;
    const int nwords = (cnt + 31) >> 5;
    // bounding sphere (centre, radius) of each word of 32 records, for the
    // slots' word test; records of one bin are sorted by the angular cell of
    // their direction, so a word covers a compact patch of directions
    __shared__ float4 s_sph[32];
    const bool word_test = cull && p.cell_bits > 0;
    if (word_test) {
        const int nwarps = blockDim.x >> 5, wid = tid >> 5;
        for (int w = wid; w < nwords; w += nwarps) {
            // the last word's missing lanes repeat the chunk's last record
            const float4 A = smA[min((w << 5) + lane, cnt - 1)];
            float x0 = A.x, x1 = A.x, y0 = A.y, y1 = A.y, z0 = A.z, z1 = A.z;
            for (int o = 16; o > 0; o >>= 1) {
                x0 = fminf(x0, __shfl_xor_sync(0xffffffffu, x0, o));
                x1 = fmaxf(x1, __shfl_xor_sync(0xffffffffu, x1, o));
                y0 = fminf(y0, __shfl_xor_sync(0xffffffffu, y0, o));
                y1 = fmaxf(y1, __shfl_xor_sync(0xffffffffu, y1, o));
                z0 = fminf(z0, __shfl_xor_sync(0xffffffffu, z0, o));
                z1 = fmaxf(z1, __shfl_xor_sync(0xffffffffu, z1, o));
            }
            const float cx = 0.5f * (x0 + x1), cy = 0.5f * (y0 + y1), cz = 0.5f * (z0 + z1);
            const float dx = A.x - cx, dy = A.y - cy, dz = A.z - cz;
            float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            for (int o = 16; o > 0; o >>= 1) d2 = fmaxf(d2, __shfl_xor_sync(0xffffffffu, d2, o));
            // radius widened past the rounding of the differences and the square root
            if (lane == 0) s_sph[w] = make_float4(cx, cy, cz, fmaf(sqrtf(d2), 1.0001f, 1e-9f));
        }
    }
    {
        // a record starts a segment where its bin differs from its predecessor's
        // or at a fold-group start; ordered compaction: a ballot per warp, then a
        // scan of the warps' counts
        const int nwarps = blockDim.x >> 5, wid = tid >> 5;
        int total = 0;
        for (int base = 0; base < cnt; base += blockDim.x) {
            const int r = base + tid;
            const bool start = r < cnt && (r == 0 || (r & (p.fold - 1)) == 0 ||
                                           __float_as_int(smB[r].w) != __float_as_int(smB[r - 1].w));
            const unsigned bal = __ballot_sync(0xffffffffu, start);
            if (lane == 0) s_seg_warp[wid] = __popc(bal);
            __syncthreads();
            int off = total;
            for (int k = 0; k < wid; k++) off += s_seg_warp[k];
            if (start) s_seg[off + __popc(bal & ((1u << lane) - 1u))] = r;
            if (r < cnt) s_seg_of[r] = (unsigned short)(off + __popc(bal & ((2u << lane) - 1u)) - 1);
            for (int k = 0; k < nwarps; k++) total += s_seg_warp[k];
            __syncthreads();
        }
        if (tid == 0) {
            s_seg[total] = cnt;
        }
        __syncthreads();
    }

    // slots of 32 lines are handed out to the warps as they finish the previous
    // one, so that warps with short walks take more slots
    const int nslots = (L + 31) >> 5;
    for (int slot = tid >> 5; slot < nslots;) {
        const int slot_pos = (slot << 5) + lane;
        const bool active = slot_pos < L;
        const int line = __ldg(line_order + (active ? slot_pos : L - 1));
        const LineK q = load_line<BEAM, REF>(lines + line, b);
        unsigned long long* lb = bins + (int64_t)line * p.ns * stride;

        // ---- phase A: records this warp's lines can see ----
        // sel, transposed: bit w of lane l's word <=> record 32 w + l selected
        unsigned sel;
        bool front_certain = false;
        if (cull) {
            const SlotCone* c = cones + slot;   // warp-uniform
            const float lx = __ldg(&c->lx), ly = __ldg(&c->ly), lz = __ldg(&c->lz);
            const float ex = __ldg(&c->ex), ey = __ldg(&c->ey), ez = __ldg(&c->ez);
            const float rx = __ldg(&c->rx), ry = __ldg(&c->ry), rz = __ldg(&c->rz);
            const float du_par = __ldg(&c->du_par), du_perp = __ldg(&c->du_perp);
            const float dv_par = __ldg(&c->dv_par), dv_perp = __ldg(&c->dv_perp), dd = __ldg(&c->dd);
            const float dd2 = dd * dd * 1.0001f + 1e-12f;
            const float ddm2 = (dd + 1e-5f) * (dd + 1e-5f) * 1.0001f;
            const float cl_c = 0.5f * (p.cull_l_lo + p.cull_l_hi), ce_c = 0.5f * (p.cull_e_lo + p.cull_e_hi);
            const float cl_h = 0.5f * (p.cull_l_hi - p.cull_l_lo) + 1e-6f * (fabsf(p.cull_l_lo) + fabsf(p.cull_l_hi));
            const float ce_h = 0.5f * (p.cull_e_hi - p.cull_e_lo) + 1e-6f * (fabsf(p.cull_e_lo) + fabsf(p.cull_e_hi));
            // word test, lane w for word w: a record A of the word lies within R
            // of its centre C, so |A.l - C.l| <= R, |A.r| <= |C.r| + R, the part of A
            // normal to r is at most |C_perp| + R and |A| <= |C| + R.  A word
            // that fails with these bounds (and tol, past their float rounding)
            // holds no record that passes the record test below in exact
            // arithmetic: no line of the slot gives any of its records a weight.
            bool word_pass = lane < nwords;
            if (word_test && word_pass) {
                const float4 S = s_sph[lane];
                const float uC = fmaf(S.z, lz, fmaf(S.y, ly, S.x * lx));
                const float vC = fmaf(S.z, ez, fmaf(S.y, ey, S.x * ex));
                const float dtC = fmaf(S.z, rz, fmaf(S.y, ry, S.x * rx));
                const float c2 = fmaf(S.z, S.z, fmaf(S.y, S.y, S.x * S.x));
                const float cn = sqrtf(c2);
                const float apC = sqrtf(fmaf(c2, 4e-6f, fmaxf(fmaf(-dtC, dtC, c2), 0.0f))) * 1.00001f;
                const float adt = fabsf(dtC) + S.w, apm = apC + S.w;
                const float su = fmaf(adt, du_par, fmaf(apm, du_perp, S.w));
                const float sv = fmaf(adt, dv_par, fmaf(apm, dv_perp, S.w));
                const float tol = 1e-5f * (cn + S.w + su + sv + fabsf(cl_c) + cl_h + fabsf(ce_c) + ce_h);
                const bool front = fmaf(cn + S.w, sqrtf(dd2), dtC + S.w + tol) >= 0.0f;
                word_pass = fabsf(uC - cl_c) < cl_h + su + tol && fabsf(vC - ce_c) < ce_h + sv + tol && front;
            }
            const unsigned words = __ballot_sync(0xffffffffu, word_pass);
            sel = 0;
            bool certain = true;   // every selected record in front of every line of the slot
            for (int w = 0; w < nwords; w++) {
                if (!((words >> w) & 1u)) continue;   // warp-uniform
                const int r = (w << 5) + lane;
                bool pass = false, sure = true;
                if (r < cnt) {
                    const float4 A = smA[r];
                    const float2 uv = __ffma2_rn(make_float2(A.z, A.z), make_float2(lz, ez),
                                      __ffma2_rn(make_float2(A.y, A.y), make_float2(ly, ey),
                                      __fmul2_rn(make_float2(A.x, A.x), make_float2(lx, ex))));
                    const float u = uv.x, v = uv.y;
                    const float dt = fmaf(A.z, rz, fmaf(A.y, ry, A.x * rx));
                    // |A|^2, and |A_perp|^2 = |A|^2 - dt^2 bounded from above: the
                    // margin 4e-6 |A|^2 exceeds the rounding of both terms and of the
                    // slot axis' length (rsqrt's error is far below 1e-5)
                    const float a2 = fmaf(A.z, A.z, fmaf(A.y, A.y, A.x * A.x));
                    const float ap2 = fmaf(a2, 4e-6f, fmaxf(fmaf(-dt, dt, a2), 0.0f));
                    const float ap = ap2 * rsqrtf(fmaxf(ap2, 1e-30f)) * 1.00001f;
                    const float adt = fabsf(dt);
                    const float su = fmaf(adt, du_par, ap * du_perp), sv = fmaf(adt, dv_par, ap * dv_perp);
                    // some line may have the record in front: A.r_k >= dt - |A| dd
                    const bool front = dt >= 0.0f || a2 * dd2 >= dt * dt;
                    // lo - s < u < hi + s as |u - c| < h + s (h widened past the roundings)
                    pass = fabsf(u - cl_c) < cl_h + su && fabsf(v - ce_c) < ce_h + sv && front;
                    // every line's A.r_k >= dt - |A| dd: in front of all of them, with a
                    // margin of 1e-5 |A| for the rounding of the per-pair dot product
                    sure = !pass || (dt > 0.0f && dt * dt > a2 * ddm2);
                }
                sel |= (unsigned)pass << w;
                certain = certain && sure;
            }
            front_certain = __all_sync(0xffffffffu, certain);
        } else {
            // every record of the chunk: words 0 .. cnt/32 - 1 full, then cnt % 32 lanes
            const int full = cnt >> 5;
            sel = (full >= 32 ? 0xffffffffu : (1u << full) - 1u) | (lane < (cnt & 31) ? 1u << full : 0u);
        }

        // ---- phase B: walk the selected records in order ----
        // Segment by segment (one FP32 run each): from the next selected record,
        // the segment's words with a selected record and their bits in order,
        // then on to the next selected record past the segment (segments without
        // one are never visited).  All of this control is warp-uniform (segment
        // bounds through redux, words through ballot).  A segment's run is
        // folded into the integer total at its end, and at a bin change the total
        // is stored (a plain store inside the chunk, an atomic at its edge bins:
        // other CTAs hold records there).
        // COUNT: pairs visited, pairs with a non-zero weight, walk steps in which
        // no lane of the warp had a non-zero weight
        unsigned walked = 0, weighted = 0, idle_steps = 0;
        const unsigned nzw = __reduce_or_sync(0xffffffffu, sel);   // bit w: word w has a selected record
        int cur = first_bin;
        long long tr = 0, ti = 0;
        float ar = 0.0f, ai = 0.0f;
        auto store_bin = [&]() {
            if (active) {
                unsigned long long* dst = lb + (int64_t)cur * stride;
                if (cur == first_bin || cur == last_bin) {
                    if (tr) atomicAdd(dst, (unsigned long long)tr);
                    if (PD && ti) atomicAdd(dst + 1, (unsigned long long)ti);
                } else {
                    if (tr) dst[0] = (unsigned long long)tr;
                    if (PD && ti) dst[1] = (unsigned long long)ti;
                }
            }
        };
        // the first selected record at or after record s (cnt if none)
        auto next_selected = [&](int s) -> int {
            if (s >= cnt) return cnt;
            const int w = s >> 5;
            const unsigned word = __ballot_sync(0xffffffffu, (sel >> w) & 1u) & (0xffffffffu << (s & 31));
            if (word) return (w << 5) + __ffs(word) - 1;
            const unsigned rest = w >= 31 ? 0u : nzw & (0xfffffffeu << w);
            if (!rest) return cnt;
            const int w2 = __ffs(rest) - 1;
            return (w2 << 5) + __ffs(__ballot_sync(0xffffffffu, (sel >> w2) & 1u)) - 1;
        };
        auto walk = [&](auto nodot_tag, auto staged_tag) {
            constexpr bool NODOT = decltype(nodot_tag)::value;
            constexpr bool STAGED = decltype(staged_tag)::value;
            // from the first selected record on, segment by segment: the segment
            // of the next selected record, its selected records from there to
            // its end, then the next selected record past it
            for (int s0 = next_selected(0); s0 < cnt;) {
                const int sg = __reduce_max_sync(0xffffffffu, (int)s_seg_of[s0]);
                const int s1 = __reduce_max_sync(0xffffffffu, s_seg[sg + 1]);
                const int w0 = s0 >> 5, w1 = (s1 - 1) >> 5;
                unsigned wm = nzw & (0xffffffffu << w0) & (0xffffffffu >> (31 - w1));
                const int nb = __reduce_max_sync(0xffffffffu, __float_as_int(smB[s0].w));
                if (nb != cur) {
                    store_bin();
                    tr = 0;
                    ti = 0;
                    cur = nb;
                }
                ar = 0.0f;
                ai = 0.0f;
                do {
                    const int w = __ffs(wm) - 1;
                    wm &= wm - 1u;
                    unsigned word = __ballot_sync(0xffffffffu, (sel >> w) & 1u);
                    if (w == w0) word &= 0xffffffffu << (s0 & 31);
                    if (w == w1) word &= 0xffffffffu >> (31 - ((s1 - 1) & 31));
                    while (word) {
                    const int i = (w << 5) + __ffs(word) - 1;
                    word &= word - 1u;
                    const float4 B = smB[i];
                    const float4 A = smA[i];
                    float w8;
                    if (REF) {
                        // vector3::dot, x*rx + y*ry + z*rz left to right (vector3.hpp:87-89)
                        const float dot = __fadd_rn(__fadd_rn(__fmul_rn(A.x, q.rx), __fmul_rn(A.y, q.ry)), __fmul_rn(A.z, q.rz));
                        const float l = __fadd_rn(__fadd_rn(__fmul_rn(A.x, q.ux), __fmul_rn(A.y, q.uy)), __fmul_rn(A.z, q.uz));
                        const float e = __fadd_rn(__fadd_rn(__fmul_rn(A.x, q.vx), __fmul_rn(A.y, q.vy)), __fmul_rn(A.z, q.vz));
                        if (BEAM == BEAM_GAUSSIAN) {
                            w8 = gauss_weight_ref(b, l, e);
                        } else {
                            // the reference recomputes the radial table coordinate per pair from r
                            w8 = lut_weight_ref(b, __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(A.x, A.x), __fmul_rn(A.y, A.y)),
                                                                       __fmul_rn(A.z, A.z))),
                                                l, e);
                        }
                        w8 = signbit(dot) ? 0.0f : w8;
                    } else {
                        const float dot = NODOT ? 1.0f : fmaf(A.z, q.rz, fmaf(A.y, q.ry, A.x * q.rx));
                        const float2 uv = __ffma2_rn(make_float2(A.z, A.z), make_float2(q.uz, q.vz),
                                          __ffma2_rn(make_float2(A.y, A.y), make_float2(q.uy, q.vy),
                                          __ffma2_rn(make_float2(A.x, A.x), make_float2(q.ux, q.vx), make_float2(q.ou, q.ov))));
                        const float u = uv.x, v = uv.y;
                        if (BEAM == BEAM_GAUSSIAN) {
                            w8 = exp2f(-fmaf(u, u, v * v));
                            // arc projection: a line for which the scatterer lies behind the
                            // origin sees it at -rho, outside [0, ns) for every record
                            // (near-origin scatterers take the per-pair path)
                            if (!NODOT) w8 = signbit(dot) ? 0.0f : w8;
                        } else {
                            w8 = 0.0f;
                            // (a warp whose lanes all miss the table skips the lookup)
                            if (fabsf(u - cl) < hl && fabsf(v - ce) < he && (NODOT || !signbit(dot))) {
                                // -1 < t < n-1: the reference's trunc-toward-zero index
                                // with the fraction dropped for -1 < t < 0
                                // (BeamProfile.cpp:94-103) is floor(max(t, 0)), the
                                // integer part of max(t, 0) + 2^23 rounded down
                                // (paired FP32 operations, two per instruction; the same
                                // rounding per component as the scalar forms)
                                const float2 ucv = make_float2(fmaxf(u, 0.0f), fmaxf(v, 0.0f));
                                const float2 t2 = __fadd2_rd(ucv, make_float2(8388608.0f, 8388608.0f));
                                const int l0 = __float_as_int(t2.x) - 0x4B000000, e0 = __float_as_int(t2.y) - 0x4B000000;
                                // fraction = t - floor(t): uc - (tu - 2^23), both differences exact
                                const float2 fle = __ffma2_rn(__fadd2_rn(t2, make_float2(-8388608.0f, -8388608.0f)),
                                                              make_float2(-1.0f, -1.0f), ucv);
                                const float fl = fle.x, fe = fle.y;
                                const int r0 = __float_as_int(B.z);
                                float4 P, Q;
                                if (STAGED) {   // B.z: the record's plane address, see above
                                    const unsigned a = __float_as_uint(B.z) +
                                                       __float_as_uint(t2.x) * (16u * (unsigned)lut_row) +
                                                       __float_as_uint(t2.y) * 16u;
                                    asm("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                                        : "=f"(P.x), "=f"(P.y), "=f"(P.z), "=f"(P.w) : "r"(a));
                                    asm("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                                        : "=f"(Q.x), "=f"(Q.y), "=f"(Q.z), "=f"(Q.w) : "r"(a + 16u * (unsigned)lut_row));
                                } else if ((unsigned)(r0 - lut_base) < (unsigned)lut_staged) {   // warp-uniform
                                    const float4* pl = smL + (r0 - lut_base) * lut_splane + l0 * lut_row + e0;
                                    P = pl[0];
                                    Q = pl[lut_row];
                                } else {
                                    const int base = r0 * lut_plane_size + l0 * b.ne + e0;
                                    P = __ldg(b.lut4 + base);
                                    Q = __ldg(b.lut4 + base + b.ne);
                                }
                                const float fr = B.y;
                                // radial (the table holds the radial differences),
                                // lateral, elevational (BeamProfile.cpp:116-127)
                                // (c00, c01) and (c10, c11), then (c0, c1) = c.0 + fl (c.1 - c.0)
                                const float2 frr = make_float2(fr, fr);
                                const float2 cl0 = __ffma2_rn(frr, make_float2(P.z, P.w), make_float2(P.x, P.y));
                                const float2 cl1 = __ffma2_rn(frr, make_float2(Q.z, Q.w), make_float2(Q.x, Q.y));
                                const float2 dl = __ffma2_rn(cl0, make_float2(-1.0f, -1.0f), cl1);
                                const float2 ce2 = __ffma2_rn(make_float2(fl, fl), dl, cl0);
                                w8 = fmaf(fe, ce2.y - ce2.x, ce2.x);
                            }
                        }
                    }
                    ar = fmaf(w8, A.w, ar);
                    if (PD) ai = fmaf(w8, B.x, ai);
                    if (COUNT) {
                        walked += active ? 1u : 0u;
                        weighted += (active && w8 != 0.0f) ? 1u : 0u;
                        idle_steps += __ballot_sync(0xffffffffu, active && w8 != 0.0f) == 0u ? 1u : 0u;
                    }
                    }
                } while (wm);
                tr += f2ll_rn(ar * scale);
                if (PD) ti += f2ll_rn(ai * scale);
                s0 = next_selected(s1);
            }
        };
        using T_ = std::true_type;
        using F_ = std::false_type;
        if (!REF && front_certain) {
            if (BEAM == BEAM_LUT && all_staged) walk(T_{}, T_{});
            else walk(T_{}, F_{});
        } else {
            if (BEAM == BEAM_LUT && !REF && all_staged) walk(F_{}, T_{});
            else walk(F_{}, F_{});
        }
        store_bin();
        if (COUNT) {
            walked = __reduce_add_sync(0xffffffffu, walked);
            weighted = __reduce_add_sync(0xffffffffu, weighted);
            if (lane == 0) {
                atomicAdd(pair_counts, (unsigned long long)walked);
                atomicAdd(pair_counts + 1, (unsigned long long)weighted);
                atomicAdd(pair_counts + 2, (unsigned long long)idle_steps);
            }
        }
        int next = 0;
        if (lane == 0) next = atomicAdd(&s_next_slot, 1);
        slot = __shfl_sync(0xffffffffu, next, 0);
    }
}

// Scatterers per staged chunk of the per-pair kernel (lines per CTA:
// PAIR_THREADS in kernels.hpp).
constexpr int PAIR_CHUNK = 256;
// Control points staged per scatterer at the full chunk size (a cubic spline's
// tile window: 4 plus one per extra knot interval); wider windows stage fewer
// scatterers per chunk.  30 KB of shared memory per CTA: seven fit an SM.
constexpr int PAIR_SPAN = 6;

// Exact arc-projection time of flight of one pair in float-pair arithmetic (fp64 mode).
// (dx, dy, dz): the scatterer relative to the line origin as pairs.  Returns
// false if the bin is outside [0, ns); otherwise the bin and the sub-sample
// delay idx - t in samples.
__device__ __forceinline__ bool pair_bin(df dx, df dy, df dz, float dot, const SimParams& p, int* idx_out,
                                         float* delay_out, float* r_out, float* tie_out = nullptr) {
    df r;
    {
        // arc projection: r = +-|d|, |d|^2 = sum hi^2 (exact products) + 2 hi lo
        const df x2 = two_prod(dx.hi, dx.hi), y2 = two_prod(dy.hi, dy.hi), z2 = two_prod(dz.hi, dz.hi);
        df s = two_sum(x2.hi, y2.hi);
        const df s2 = two_sum(s.hi, z2.hi);
        float lo = s.lo + s2.lo + x2.lo + y2.lo + z2.lo;
        lo = fmaf(2.0f * dx.hi, dx.lo, lo);
        lo = fmaf(2.0f * dy.hi, dy.lo, lo);
        lo = fmaf(2.0f * dz.hi, dz.lo, lo);
        r = df_sqrt(fast_two_sum(s2.hi, lo));
        if (signbit(dot)) { r.hi = -r.hi; r.lo = -r.lo; }
    }
    *r_out = r.hi + r.lo;
    const df t = df_mul(r, df_make(p.k_hi, p.k_lo));
    // idx = floor(t + 0.5) decided on the pair: with f = floor(hi) the remainder
    // hi - f is exact, so compare (hi - f - 0.5) with -lo.
    float f = floorf(t.hi);
    float rem = t.hi - f;
    if (rem + t.lo < 0.0f) { f -= 1.0f; rem += 1.0f; }
    const bool up = (rem - 0.5f) >= -t.lo;
    // distance (in samples) of t from the rounding boundary
    if (tie_out) *tie_out = fabsf((rem - 0.5f) + t.lo);
    const float fidx = up ? f + 1.0f : f;
    if (!(fidx >= 0.0f && fidx < (float)p.ns)) return false;
    *idx_out = (int)fidx;
    *delay_out = (up ? 1.0f : 0.0f) - rem - t.lo;
    return true;
}

// Per (scatterer, line) pair projection for any line geometry and for splines.
// CTA = a tile of up to PAIR_THREADS lines (one per thread; for splines sorted
// by knot interval) x a chunk of scatterers staged in shared memory and
// broadcast to the threads (for splines the tile's window of control points per
// scatterer, each line reading its own p+1 of them).  Each pair first gets an FP32 position
// and weight; a pair whose contribution rounds to zero in the fixed-point bins
// (or lies outside the lookup table by a margin) is skipped -- exactly, since it
// would add 0 -- and only the remaining pairs compute the float-pair time of
// flight and add their contribution with integer atomics.
template <int BEAM, bool SPLINE, bool REF, int DEG>
__global__ void __launch_bounds__(PAIR_THREADS, (SPLINE && DEG >= 0) ? 6 : 0)
    project_generic_kernel(const float4* __restrict__ xyza, const float4* __restrict__ cps,
                           const float* __restrict__ amps, int64_t n, int degree,
                           const uint32_t* __restrict__ index_list, const int* __restrict__ counts,
                           int64_t list_lo, const LineGeom* __restrict__ lines, const int* __restrict__ line_ids,
                           const LineTile* __restrict__ tiles, const LineBasis* __restrict__ basis,
                           unsigned long long* __restrict__ bins, SimParams p, BeamDev b,
                           const TileBox* __restrict__ boxes, unsigned long long* __restrict__ pair_counts) {
    // staged scatterers: fixed (x, y, z, a); splines (fp64 mode) the window's
    // control points relative to its first one (R, in sr), the global index for
    // the exact re-evaluation at rounding ties; splines (reference mode) the
    // control points themselves
    __shared__ float4 sp[PAIR_CHUNK * (SPLINE ? PAIR_SPAN : 1)];
    __shared__ float sa[PAIR_CHUNK];
    __shared__ float4 sr[SPLINE && !REF ? PAIR_CHUNK : 1];
    __shared__ int sidx[SPLINE && !REF ? PAIR_CHUNK : 1];
    __shared__ int s_kept;   // scatterers of the chunk kept for the tile
    const LineTile tile = tiles[blockIdx.y];
    int64_t count = n, list_off = 0;
    if (index_list) {
        list_off = __ldg(counts);
        count = __ldg(counts + 1);
    }
    const int tid = threadIdx.x;
    // non-zero basis functions per line: DEG + 1 for a spline degree fixed at
    // compile time (the cubic case: fewer registers, six CTAs per SM), else the
    // runtime degree's
    constexpr int NB = DEG >= 0 ? DEG + 1 : MAX_SPLINE_DEGREE + 1;
    const int np = DEG >= 0 ? DEG + 1 : degree + 1;
    // control points staged per scatterer, and scatterers per chunk so that
    // they fit the shared array
    const int span = SPLINE ? tile.span : 1;
    const int chunk = SPLINE ? min(PAIR_CHUNK, PAIR_CHUNK * PAIR_SPAN / span) : PAIR_CHUNK;
    const bool active = tid < tile.count;
    const int line = __ldg(line_ids + tile.first + (active ? tid : 0));
    const LineGeom* g = lines + line;
    const float ox = __ldg(&g->o[0]), oy = __ldg(&g->o[1]), oz = __ldg(&g->o[2]);
    const float rx = __ldg(&g->d[0]), ry = __ldg(&g->d[1]), rz = __ldg(&g->d[2]);
    const float lx = __ldg(&g->l[0]), ly = __ldg(&g->l[1]), lz = __ldg(&g->l[2]);
    const float ex = __ldg(&g->e[0]), ey = __ldg(&g->e[1]), ez = __ldg(&g->e[2]);
    float bh[NB];   // the line's basis (high parts; the low parts are read at rounding ties only)
    int win = 0;   // this line's first control point within the staged window
    if (SPLINE) {
        const LineBasis* lb = basis + line;
        win = __ldg(&lb->mu) - tile.mu;
#pragma unroll
        for (int k = 0; k < NB; k++) bh[k] = k < np ? __ldg(&lb->hi[k]) : 0.0f;
    }
    const int stride = p.phase_delay ? 2 : 1;
    unsigned long long* lbins = bins + (int64_t)line * p.ns * stride;
    // a contribution below half a fixed-point unit rounds to 0
    const float skip_below = 0.499f / p.scale;
    const float gl = b.gl, ge = b.ge;

    // tile culling: the tile's reference frame and spreads
    const bool tcull = boxes != nullptr;
    TileBox bx;
    if (tcull) bx = boxes[blockIdx.y];
    const int lane = tid & 31;

    for (int64_t c0 = (int64_t)blockIdx.x * chunk; c0 < count; c0 += (int64_t)gridDim.x * chunk) {
    const int cand = (int)min((int64_t)chunk, count - c0);
    __syncthreads();   // the previous chunk is consumed
    if (tid == 0) s_kept = 0;
    __syncthreads();
    // stage the chunk's scatterers that the tile may see (gathering through the
    // index list for the near-origin residue), compacted: the order does not
    // matter, every contribution is an integer atomic
    for (int i0 = 0; i0 < cand; i0 += blockDim.x) {
        const int ci = i0 + tid;
        int64_t s = c0 + ci;
        bool ok = ci < cand;
        if (ok && index_list) {
            s = (int64_t)__ldg(index_list + list_off + s) - list_lo;
            ok = s >= 0 && s < n;
        }
        float a = 0.0f;
        float lo_x = 0.f, lo_y = 0.f, lo_z = 0.f, hi_x = 0.f, hi_y = 0.f, hi_z = 0.f;
        if (ok) {
            if (SPLINE) {
                a = __ldg(amps + s);
                // convex hull: the curve over the tile's knot intervals lies in the
                // box of the window's control points
                lo_x = lo_y = lo_z = INFINITY;
                hi_x = hi_y = hi_z = -INFINITY;
                for (int k = 0; k < span; k++) {
                    const float4 c = __ldg(cps + (int64_t)(tile.mu - degree + k) * n + s);
                    lo_x = fminf(lo_x, c.x); lo_y = fminf(lo_y, c.y); lo_z = fminf(lo_z, c.z);
                    hi_x = fmaxf(hi_x, c.x); hi_y = fmaxf(hi_y, c.y); hi_z = fmaxf(hi_z, c.z);
                }
            } else {
                const float4 q = __ldg(xyza + s);
                a = q.w;
                lo_x = hi_x = q.x; lo_y = hi_y = q.y; lo_z = hi_z = q.z;
            }
            ok = a != 0.0f;
        }
        if (ok && tcull) {
            // lateral / elevational ranges outside which no contribution survives:
            // the lookup table's extent, or (Gaussian) where w |a| <= 1/4 of a
            // fixed-point unit, i.e. l^2 gl + e^2 ge >= log2(scale |a|) + 2
            float llo = p.cull_l_lo, lhi = p.cull_l_hi, elo = p.cull_e_lo, ehi = p.cull_e_hi;
            if (BEAM == BEAM_GAUSSIAN) {
                const float Q = log2f(p.scale * fabsf(a)) + 2.01f;
                const float rl = Q > 0.0f ? sqrtf(Q / gl) : 0.0f, re = Q > 0.0f ? sqrtf(Q / ge) : 0.0f;
                llo = -rl; lhi = rl; elo = -re; ehi = re;
                ok = Q > 0.0f;
            }
            const float cx = 0.5f * (lo_x + hi_x) - bx.ox, cy = 0.5f * (lo_y + hi_y) - bx.oy;
            const float cz = 0.5f * (lo_z + hi_z) - bx.oz;
            const float hx = 0.5f * (hi_x - lo_x) * 1.0001f, hy = 0.5f * (hi_y - lo_y) * 1.0001f;
            const float hz = 0.5f * (hi_z - lo_z) * 1.0001f;
            const float uc = fmaf(cz, bx.lz, fmaf(cy, bx.ly, cx * bx.lx));
            const float uh = fmaf(hz, fabsf(bx.lz), fmaf(hy, fabsf(bx.ly), hx * fabsf(bx.lx))) + 1e-6f;
            const float vc = fmaf(cz, bx.ez, fmaf(cy, bx.ey, cx * bx.ex));
            const float vh = fmaf(hz, fabsf(bx.ez), fmaf(hy, fabsf(bx.ey), hx * fabsf(bx.ex))) + 1e-6f;
            const float dc = fmaf(cz, bx.rz, fmaf(cy, bx.ry, cx * bx.rx));
            const float dh = fmaf(hz, fabsf(bx.rz), fmaf(hy, fabsf(bx.ry), hx * fabsf(bx.rx))) + 1e-6f;
            const float amax = fabsf(cx) + fabsf(cy) + fabsf(cz) + hx + hy + hz;   // >= |A - o|
            const float adt = fabsf(dc) + dh;
            // a tile line's coordinates differ from the reference's by the frame
            // spread times the offset, plus its origin's distance from o
            const float su = (fmaf(adt, bx.du_par, amax * bx.du_perp) + bx.d_orig) * 1.001f + 1e-6f;
            const float sv = (fmaf(adt, bx.dv_par, amax * bx.dv_perp) + bx.d_orig) * 1.001f + 1e-6f;
            ok = ok && (uc + uh + su > llo) && (uc - uh - su < lhi) && (vc + vh + sv > elo) && (vc - vh - sv < ehi);
        }
        const unsigned bal = __ballot_sync(0xffffffffu, ok);
        int base = 0;
        if (lane == 0 && bal) base = atomicAdd(&s_kept, __popc(bal));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (ok) {
            const int d = base + __popc(bal & ((1u << lane) - 1u));
            if (SPLINE) {
                if (REF) {
                    for (int k = 0; k < span; k++) sp[d * span + k] = __ldg(cps + (int64_t)(tile.mu - degree + k) * n + s);
                } else {
                    const float4 R = __ldg(cps + (int64_t)(tile.mu - degree) * n + s);
                    for (int k = 0; k < span; k++) {
                        const float4 c = __ldg(cps + (int64_t)(tile.mu - degree + k) * n + s);
                        sp[d * span + k] = make_float4(c.x - R.x, c.y - R.y, c.z - R.z, 0.0f);
                    }
                    sr[d] = R;
                    sidx[d] = (int)s;
                }
            } else {
                sp[d] = make_float4(lo_x, lo_y, lo_z, a);
            }
            sa[d] = a;
        }
    }
    __syncthreads();
    const int cnt = s_kept;
    // instrumented run: the (scatterer, line) pairs this tile evaluates
    if (pair_counts && tid == 0 && cnt > 0) atomicAdd(pair_counts + 3, (unsigned long long)cnt * tile.count);
    if (!active) continue;
    for (int i = 0; i < cnt; i++) {
        const float a = sa[i];
        if (a == 0.0f) continue;
        float w, cph = 1.0f, sph = 0.0f;
        int idx;
        if (!REF) {
            // FP32 position relative to the origin
            float fx, fy, fz;
            float Sx = 0.f, Sy = 0.f, Sz = 0.f;   // sum_k B_k (C_k - R)
            float4 R = make_float4(0.f, 0.f, 0.f, 0.f);
            if (SPLINE) {
                // the basis sums to one: P = R + sum_k B_k (C_k - R)
                R = sr[i];
#pragma unroll
                for (int k = 0; k < NB; k++) {
                    if (k < np) {
                        const float4 c = sp[i * span + win + k];
                        Sx = fmaf(bh[k], c.x, Sx); Sy = fmaf(bh[k], c.y, Sy); Sz = fmaf(bh[k], c.z, Sz);
                    }
                }
                fx = (R.x - ox) + Sx; fy = (R.y - oy) + Sy; fz = (R.z - oz) + Sz;
            } else {
                const float4 c = sp[i];
                fx = c.x - ox; fy = c.y - oy; fz = c.z - oz;
            }
            const float l = fmaf(fz, lz, fmaf(fy, ly, fx * lx));
            const float e = fmaf(fz, ez, fmaf(fy, ey, fx * ex));
            float tl = 0.f, te = 0.f;
            if (BEAM == BEAM_GAUSSIAN) {
                w = exp2f(-fmaf(l * l, gl, e * e * ge));
                if (fabsf(w * a) < skip_below) continue;
            } else {
                tl = (l - b.lf) * b.inv_dl;
                te = (e - b.ef) * b.inv_de;
                // outside the table by more than rounding can explain: weight 0
                if (!(tl > -1.001f && tl < (float)(b.nl - 1) + 0.001f && te > -1.001f && te < (float)(b.ne - 1) + 0.001f))
                    continue;
            }
            // position relative to the origin as float pairs: R - o exactly, plus
            // the FP32 sum S (its error, ~1e-8 of the control points' spread, is
            // ~2e-5 of a sample; bins within 1e-3 of a sample of a rounding tie
            // are decided again from the exact float-pair spline sum below)
            df dx, dy, dz;
            if (SPLINE) {
                auto near = [](float r, float o, float sum) {
                    const df a = two_sum(r, -o);
                    const df b = two_sum(a.hi, sum);
                    return fast_two_sum(b.hi, b.lo + a.lo);
                };
                dx = near(R.x, ox, Sx);
                dy = near(R.y, oy, Sy);
                dz = near(R.z, oz, Sz);
            } else {
                const float4 c = sp[i];
                dx = two_sum(c.x, -ox);
                dy = two_sum(c.y, -oy);
                dz = two_sum(c.z, -oz);
            }
            // the exact float-pair sum sum_k (bh_k + bl_k) C_k - o, control points from global memory
            auto exact_position = [&]() {
                df sx = df_make(0.f, 0.f), sy = df_make(0.f, 0.f), sz = df_make(0.f, 0.f);
                float ex_ = 0.f, ey_ = 0.f, ez_ = 0.f;   // accumulated low parts
                const int gs = sidx[i];
                const LineBasis* lbs = basis + line;
#pragma unroll
                for (int k = 0; k < NB; k++) {
                    if (k < np) {
                        const float4 c = __ldg(cps + (int64_t)(tile.mu - degree + win + k) * n + gs);
                        const float blk = __ldg(&lbs->lo[k]);
                        const df px = two_prod(bh[k], c.x), py = two_prod(bh[k], c.y), pz = two_prod(bh[k], c.z);
                        const df tx = two_sum(sx.hi, px.hi), ty = two_sum(sy.hi, py.hi), tz = two_sum(sz.hi, pz.hi);
                        sx.hi = tx.hi; sy.hi = ty.hi; sz.hi = tz.hi;
                        ex_ += tx.lo + fmaf(blk, c.x, px.lo);
                        ey_ += ty.lo + fmaf(blk, c.y, py.lo);
                        ez_ += tz.lo + fmaf(blk, c.z, pz.lo);
                    }
                }
                const df ux = two_sum(sx.hi, -ox), uy = two_sum(sy.hi, -oy), uz = two_sum(sz.hi, -oz);
                dx = fast_two_sum(ux.hi, ux.lo + ex_);
                dy = fast_two_sum(uy.hi, uy.lo + ey_);
                dz = fast_two_sum(uz.hi, uz.lo + ez_);
            };
            const float fdx = dx.hi + dx.lo, fdy = dy.hi + dy.lo, fdz = dz.hi + dz.lo;
            const float dot = fmaf(fdz, rz, fmaf(fdy, ry, fdx * rx));
            float delay, rr;
            if (p.arc) {
                if (SPLINE) {
                    float tie = 1.0f;
                    const bool in = pair_bin(dx, dy, dz, dot, p, &idx, &delay, &rr, &tie);
                    if (tie < 1e-3f) {   // near a rounding tie: decide from the exact sum
                        exact_position();
                        const float xd = dx.hi + dx.lo, yd = dy.hi + dy.lo, zd = dz.hi + dz.lo;
                        if (!pair_bin(dx, dy, dz, fmaf(zd, rz, fmaf(yd, ry, xd * rx)), p, &idx, &delay, &rr)) continue;
                    } else if (!in) {
                        continue;
                    }
                } else {
                    if (!pair_bin(dx, dy, dz, dot, p, &idx, &delay, &rr)) continue;
                }
            } else {
                // radial coordinate = projection on the line direction
                auto linear_bin = [&](float* tie) {
                    const df r = df_add(df_add(df_mul_f(dx, rx), df_mul_f(dy, ry)), df_mul_f(dz, rz));
                    rr = r.hi + r.lo;
                    const df t = df_mul(r, df_make(p.k_hi, p.k_lo));
                    float f = floorf(t.hi);
                    float rem = t.hi - f;
                    if (rem + t.lo < 0.0f) { f -= 1.0f; rem += 1.0f; }
                    const bool up = (rem - 0.5f) >= -t.lo;
                    *tie = fabsf((rem - 0.5f) + t.lo);
                    const float fidx = up ? f + 1.0f : f;
                    if (!(fidx >= 0.0f && fidx < (float)p.ns)) return false;
                    idx = (int)fidx;
                    delay = (up ? 1.0f : 0.0f) - rem - t.lo;
                    return true;
                };
                float tie = 1.0f;
                bool in = linear_bin(&tie);
                if (SPLINE && tie < 1e-3f) {   // near a rounding tie: decide from the exact sum
                    exact_position();
                    in = linear_bin(&tie);
                }
                if (!in) continue;
            }
            if (BEAM == BEAM_LUT) {
                const float tr = (rr - b.rf) * b.inv_dr;
                if (!(tr > -1.0f && tr < (float)(b.nr - 1))) continue;
                const int r0 = (int)tr;
                const float frr = tr < 0.0f ? 0.0f : tr - (float)r0;
                w = lut_weight_packed(b, r0, frr, tl, te);
            }
            if (p.phase_delay) {
                // sub-sample delay (idx - t) in samples as a phase (CpuAlgorithm.cpp:85-92);
                // |argument| < pi fd/fs, where the fast sine/cosine is accurate to ~4e-7
                __sincosf(p.two_pi_fd_over_fs * delay, &sph, &cph);
            }
        } else {
            // the reference's float expressions (CpuAlgorithm.cpp:58-95 and 137-181)
            float fx, fy, fz;
            if (SPLINE) {
                float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
                for (int k = 0; k < NB; k++) {
                    if (k < np) {
                        const float4 c = sp[i * span + win + k];
                        sx = __fadd_rn(sx, __fmul_rn(c.x, bh[k]));
                        sy = __fadd_rn(sy, __fmul_rn(c.y, bh[k]));
                        sz = __fadd_rn(sz, __fmul_rn(c.z, bh[k]));
                    }
                }
                fx = __fsub_rn(sx, ox); fy = __fsub_rn(sy, oy); fz = __fsub_rn(sz, oz);
            } else {
                const float4 c = sp[i];
                fx = __fsub_rn(c.x, ox); fy = __fsub_rn(c.y, oy); fz = __fsub_rn(c.z, oz);
            }
            float r = __fadd_rn(__fadd_rn(__fmul_rn(fx, rx), __fmul_rn(fy, ry)), __fmul_rn(fz, rz));
            const float l = __fadd_rn(__fadd_rn(__fmul_rn(fx, lx), __fmul_rn(fy, ly)), __fmul_rn(fz, lz));
            const float e = __fadd_rn(__fadd_rn(__fmul_rn(fx, ex), __fmul_rn(fy, ey)), __fmul_rn(fz, ez));
            if (p.arc)
                r = copysignf(__fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(fx, fx), __fmul_rn(fy, fy)), __fmul_rn(fz, fz))), r);
            double t;
            if (SPLINE) {
                // r*2.0/(c*dt) with dt = float(1/fs) (CpuAlgorithm.cpp:161-162)
                const float dt = (float)(1.0 / p.fs_d);
                t = __ddiv_rn(__dmul_rn((double)r, 2.0), (double)__fmul_rn(p.c, dt));
            } else {
                t = __ddiv_rn(__dmul_rn(__dmul_rn((double)r, 2.0), p.fs_d), p.c_d);
            }
            const double fidx = floor(t + 0.5);
            if (!(fidx >= 0.0 && fidx < (double)p.ns)) continue;
            idx = (int)fidx;
            if (BEAM == BEAM_GAUSSIAN) w = gauss_weight_ref(b, l, e);
            else w = lut_weight_ref(b, r, l, e);
            if (p.phase_delay) {
                const float ss_delay = (float)(((double)idx - t) / p.fs_d);
                const float ph = (float)(TWO_PI_LITERAL * p.fd_d * (double)ss_delay);
                sincosf(ph, &sph, &cph);
            }
        }
        const float amp = w * a;
        unsigned long long* dst = lbins + (int64_t)idx * stride;
        if (p.phase_delay) {
            bin_add(dst, amp * cph, p.scale);
            bin_add(dst + 1, amp * sph, p.scale);
        } else {
            bin_add(dst, amp, p.scale);
        }
    }
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
cudaError_t launch_prep_shared(const float4* xyza, int64_t n, int64_t off, const float origin[3], const SimParams& p,
                               const BeamDev& b, uint32_t* keys, uint32_t* vals, float4* recA, float4* recB,
                               cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    const int threads = 256;
    const int64_t blocks = (n + threads - 1) / threads;
    prep_shared_kernel<<<(unsigned)blocks, threads, 0, stream>>>(xyza, n, off, (double)origin[0], (double)origin[1],
                                                                 (double)origin[2], origin[0], origin[1], origin[2],
                                                                 p, b, keys, vals, recA, recB);
    return cudaGetLastError();
}

cudaError_t launch_prep_shared_spline(const float4* cps, const float* amps, int64_t n, int num_cs, int first_cs,
                                      int degree, const double* basis_d, const float* basis_f, int64_t off,
                                      const float origin[3], const SimParams& p, const BeamDev& b, uint32_t* keys,
                                      uint32_t* vals, float4* recA, float4* recB, cudaStream_t stream) {
    (void)num_cs;
    if (n <= 0) return cudaSuccess;
    const int threads = 256;
    const int64_t blocks = (n + threads - 1) / threads;
    prep_shared_spline_kernel<<<(unsigned)blocks, threads, 0, stream>>>(
        cps, amps, n, first_cs, degree, basis_d, basis_f, off, (double)origin[0], (double)origin[1],
        (double)origin[2], origin[0], origin[1], origin[2], p, b, keys, vals, recA, recB);
    return cudaGetLastError();
}

cudaError_t launch_count_keys(const uint32_t* sorted_keys, int64_t n, int ns, int cell_bits, int* counts,
                              cudaStream_t stream) {
    init_counts_kernel<<<1, 1, 0, stream>>>(counts, n);
    if (n > 0) {
        const int threads = 256;
        count_keys_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, stream>>>(sorted_keys, n, ns,
                                                                                        cell_bits, counts);
    }
    finish_counts_kernel<<<1, 1, 0, stream>>>(counts);
    return cudaGetLastError();
}

cudaError_t launch_gather_records(const uint32_t* sorted_vals, const int* counts, int64_t n, const float4* recA,
                                  const float4* recB, float4* out, int64_t plane, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    const int threads = 256;
    gather_records_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, stream>>>(sorted_vals, counts, n,
                                                                                        recA, recB, out, plane);
    return cudaGetLastError();
}

template <bool PD, int BEAM, bool REF, bool COUNT>
static cudaError_t launch_shared_t(const float4* records, int64_t plane, const int* counts, int64_t n, int chunk,
                                   const LineGeom* lines, const int* line_order, const SlotCone* cones, int L,
                                   const SimParams& p, const BeamDev& b, unsigned long long* bins,
                                   unsigned long long* pair_counts, cudaStream_t stream) {
    if (chunk > 1024 || p.fold < 1 || (p.fold & (p.fold - 1)) || chunk % p.fold) return cudaErrorInvalidValue;
    size_t smem = 2 * (size_t)chunk * sizeof(float4);
    const int64_t chunks = (n + chunk - 1) / chunk;
    if (p.wide_cta && L >= 512) {
        // large CTAs (one per SM with lookup-table planes): all warps of an SM
        // share one record chunk and the lookup-table planes it touches, staged
        // in shared memory (up to two planes: a chunk of <= 1024 records spans
        // far less than a table cell radially in any dense phantom; records
        // beyond them read the table through the cache).  1024 threads: the
        // warps take the slots of 32 lines one after another as they finish
        // (measured: 512-thread CTAs, one or two per SM, and a single staged
        // plane are all slower on the 3-D table workload).
        int lut_planes = 0;
        if (BEAM == BEAM_LUT && !REF && p.lut_smem) {
            const size_t plane_bytes = (size_t)b.nl * (b.ne | 1) * sizeof(float4);
            const size_t budget = 200 * 1024;
            if (smem + plane_bytes <= budget) lut_planes = (budget - smem) / plane_bytes >= 2 ? 2 : 1;
            smem += (size_t)lut_planes * plane_bytes;
        }
        auto k = project_shared_kernel<PD, BEAM, REF, 1024, COUNT>;
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k<<<(unsigned)chunks, 1024, smem, stream>>>(records, plane, counts, chunk, lines, line_order, cones, L, bins,
                                                    p, b, lut_planes, pair_counts);
        return cudaGetLastError();
    }
    auto k = project_shared_kernel<PD, BEAM, REF, 256, COUNT>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int threads = L >= 256 ? 256 : ((L + 31) / 32) * 32;
    k<<<(unsigned)chunks, threads, smem, stream>>>(records, plane, counts, chunk, lines, line_order, cones, L, bins,
                                                   p, b, 0, pair_counts);
    return cudaGetLastError();
}

cudaError_t launch_project_shared(const float4* records, int64_t plane, const int* counts, int64_t n, int chunk,
                                  const LineGeom* lines, const int* line_order, const SlotCone* cones, int L,
                                  const SimParams& p, const BeamDev& b, unsigned long long* bins,
                                  unsigned long long* pair_counts, cudaStream_t stream) {
    if (n <= 0 || L <= 0) return cudaSuccess;
    const bool pd = p.phase_delay != 0;
    const bool ref = p.mode == MODE_REFERENCE;
    if (pair_counts && ref) return cudaErrorInvalidValue;   // counting instruments the fp64-mode kernel only
#define BCSIM_SH(PDV, BM, R, C) \
    launch_shared_t<PDV, BM, R, C>(records, plane, counts, n, chunk, lines, line_order, cones, L, p, b, bins, pair_counts, stream)
    if (pair_counts) {
        if (b.type == BEAM_GAUSSIAN) return pd ? BCSIM_SH(true, BEAM_GAUSSIAN, false, true) : BCSIM_SH(false, BEAM_GAUSSIAN, false, true);
        return pd ? BCSIM_SH(true, BEAM_LUT, false, true) : BCSIM_SH(false, BEAM_LUT, false, true);
    }
    if (b.type == BEAM_GAUSSIAN) {
        if (pd) return ref ? BCSIM_SH(true, BEAM_GAUSSIAN, true, false) : BCSIM_SH(true, BEAM_GAUSSIAN, false, false);
        return ref ? BCSIM_SH(false, BEAM_GAUSSIAN, true, false) : BCSIM_SH(false, BEAM_GAUSSIAN, false, false);
    }
    if (pd) return ref ? BCSIM_SH(true, BEAM_LUT, true, false) : BCSIM_SH(true, BEAM_LUT, false, false);
    return ref ? BCSIM_SH(false, BEAM_LUT, true, false) : BCSIM_SH(false, BEAM_LUT, false, false);
#undef BCSIM_SH
}

template <int BEAM, bool SPLINE, bool REF, int DEG>
static cudaError_t launch_generic_t(const float4* xyza, const float4* cps, const float* amps, int64_t n, int degree,
                                    const uint32_t* index_list, const int* counts, int64_t list_lo,
                                    const LineGeom* lines, const int* line_ids, const LineTile* tiles,
                                    int num_tiles, const LineBasis* basis, const SimParams& p, const BeamDev& b,
                                    unsigned long long* bins, cudaStream_t stream, const TileBox* boxes,
                                    unsigned long long* pair_counts, int threads) {
    if (threads < 32 || threads > PAIR_THREADS || threads % 32) return cudaErrorInvalidValue;
    // chunks over all scatterers (for the residue list: over n, the kernel
    // returns early past the list length, which is a handful)
    int64_t chunks = (n + PAIR_CHUNK - 1) / PAIR_CHUNK;
    if (index_list) chunks = 8;
    if (chunks < 1) chunks = 1;
    dim3 grid((unsigned)chunks, (unsigned)num_tiles);
    project_generic_kernel<BEAM, SPLINE, REF, DEG><<<grid, threads, 0, stream>>>(
        xyza, cps, amps, n, degree, index_list, counts, list_lo, lines, line_ids, tiles, basis, bins, p, b,
        REF ? nullptr : boxes, pair_counts);
    return cudaGetLastError();
}

cudaError_t launch_project_generic(const float4* xyza, const float4* cps, const float* amps, int64_t n, int num_cs,
                                   int degree, const uint32_t* index_list, const int* counts, int64_t list_lo,
                                   const LineGeom* lines, const int* line_ids, const LineTile* tiles, int num_tiles,
                                   const LineBasis* basis, const SimParams& p, const BeamDev& b,
                                   unsigned long long* bins, cudaStream_t stream, const TileBox* boxes,
                                   unsigned long long* pair_counts, int threads) {
    (void)num_cs;
    if (n <= 0 || num_tiles <= 0) return cudaSuccess;
    const bool spline = cps != nullptr;
    const bool ref = p.mode == MODE_REFERENCE;
#define BCSIM_GEN(B, S, R, G) launch_generic_t<B, S, R, G>(xyza, cps, amps, n, degree, index_list, counts, list_lo, lines, line_ids, tiles, num_tiles, basis, p, b, bins, stream, boxes, pair_counts, threads)
    // cubic splines (the reference's and the workloads' degree) get a kernel
    // with the degree fixed at compile time
    const bool cubic = spline && degree == 3;
    if (b.type == BEAM_GAUSSIAN) {
        if (spline) {
            if (ref) return cubic ? BCSIM_GEN(BEAM_GAUSSIAN, true, true, 3) : BCSIM_GEN(BEAM_GAUSSIAN, true, true, -1);
            return cubic ? BCSIM_GEN(BEAM_GAUSSIAN, true, false, 3) : BCSIM_GEN(BEAM_GAUSSIAN, true, false, -1);
        }
        return ref ? BCSIM_GEN(BEAM_GAUSSIAN, false, true, -1) : BCSIM_GEN(BEAM_GAUSSIAN, false, false, -1);
    }
    if (spline) {
        if (ref) return cubic ? BCSIM_GEN(BEAM_LUT, true, true, 3) : BCSIM_GEN(BEAM_LUT, true, true, -1);
        return cubic ? BCSIM_GEN(BEAM_LUT, true, false, 3) : BCSIM_GEN(BEAM_LUT, true, false, -1);
    }
    return ref ? BCSIM_GEN(BEAM_LUT, false, true, -1) : BCSIM_GEN(BEAM_LUT, false, false, -1);
#undef BCSIM_GEN
}

cudaError_t enqueue_error_flag_read(const int* dev_flag, int* host_flag, cudaStream_t stream) {
    return cudaMemcpyAsync(host_flag, dev_flag, sizeof(int), cudaMemcpyDeviceToHost, stream);
}

cudaError_t read_and_clear_error_flag(int* dev_flag, int* flag, cudaStream_t stream) {
    cudaError_t e = cudaMemcpyAsync(flag, dev_flag, sizeof(int), cudaMemcpyDeviceToHost, stream);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(dev_flag, 0, sizeof(int), stream);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(stream);
}

cudaError_t radix_sort_pairs(void* temp, size_t* temp_bytes, const uint32_t* keys_in, uint32_t* keys_out,
                             const uint32_t* vals_in, uint32_t* vals_out, int64_t n, int end_bit,
                             cudaStream_t stream) {
    return cub::DeviceRadixSort::SortPairs(temp, *temp_bytes, keys_in, keys_out, vals_in, vals_out, (int)n, 0,
                                           end_bit, stream);
}

}  // namespace bcsim_gb300
