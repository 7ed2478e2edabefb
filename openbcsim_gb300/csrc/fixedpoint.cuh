// fixedpoint.cuh -- exact conversions between FP32 and the int64 fixed-point
// bins, in integer arithmetic.
//
// The CUDA conversion instructions between 64-bit integers and floats issue on
// the FP64 pipe, which GB300 has only a sliver of; the projection folds and the
// FIR staging convert once per bin touched, enough to make that pipe a
// bottleneck.  These functions compute the same IEEE round-to-nearest-even
// results from the bit patterns with 32/64-bit integer operations only.  They
// are plain C++ (host and device), so the host test suite checks them against
// the C library's conversions.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define BCSIM_HD __host__ __device__ __forceinline__
#else
#define BCSIM_HD inline
#endif

namespace bcsim_gb300 {

BCSIM_HD unsigned fp_bits(float x) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x);
#else
    unsigned u;
    std::memcpy(&u, &x, sizeof u);
    return u;
#endif
}

BCSIM_HD float fp_from_bits(unsigned u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float x;
    std::memcpy(&x, &u, sizeof x);
    return x;
#endif
}

BCSIM_HD int clz64(unsigned long long a) {   // a != 0
#if defined(__CUDA_ARCH__)
    return __clzll((long long)a);
#else
    return __builtin_clzll(a);
#endif
}

// float -> int64, rounding to nearest even; |x| >= 2^63 saturates, NaN gives 0
// (the result of cvt.rni.s64.f32).
BCSIM_HD long long f2ll_rn(float x) {
    const unsigned u = fp_bits(x);
    const int ex = (int)((u >> 23) & 0xffu);
    if (ex >= 190) {   // |x| >= 2^63, infinities and NaN
        if (ex == 255 && (u & 0x7fffffu)) return 0;
        return (u >> 31) ? (long long)0x8000000000000000ull : 0x7fffffffffffffffll;
    }
    const unsigned m = ex ? ((u & 0x7fffffu) | 0x800000u) : 0u;   // subnormals round to 0
    const int sh = ex - 150;                                      // |x| = m * 2^sh
    unsigned long long mag;
    if (sh >= 0) {
        mag = (unsigned long long)m << sh;   // sh <= 39
    } else {
        const int rs = -sh < 25 ? -sh : 25;   // m < 2^24: 2^-25 m < 1/2 rounds to 0
        const unsigned q = m >> rs;
        const unsigned rem = m & ((1u << rs) - 1u);
        const unsigned half = 1u << (rs - 1);
        mag = q + ((rem > half || (rem == half && (q & 1u))) ? 1u : 0u);
    }
    return (u >> 31) ? -(long long)mag : (long long)mag;
}

// float -> int64, rounding to nearest even, for |x| < 2^62 (a bin
// contribution: the fixed-point scale keeps every sum below 2^61); other
// values take f2ll_rn.  Below 2^31 one FP32 -> int32 conversion; above, x is
// an integer: x = h 2^32 + l with h = floor(x / 2^32) and l = x - h 2^32 both
// exact in FP32 (l < 2^32 has at most 24 significant bits), each converted
// exactly.  Three to five instructions instead of the integer code's ~18.
BCSIM_HD long long f2ll_rn_bounded(float x) {
#if defined(__CUDA_ARCH__)
    const float ax = fabsf(x);
    if (ax < 2147483648.0f) return (long long)__float2int_rn(x);
    if (!(ax < 4.611686e18f)) return f2ll_rn(x);
    const float h = floorf(x * 2.3283064365386963e-10f);
    const float l = fmaf(-h, 4294967296.0f, x);
    return (long long)__float2int_rn(h) * 4294967296ll + (long long)__float2uint_rn(l);
#else
    const float ax = std::fabs(x);
    if (ax < 2147483648.0f) return (long long)std::nearbyint(x);
    if (!(ax < 4.611686e18f)) return f2ll_rn(x);
    const float h = std::floor(x * 2.3283064365386963e-10f);
    const float l = std::fma(-h, 4294967296.0f, x);
    return (long long)h * 4294967296ll + (long long)l;
#endif
}

// int64 -> float, rounding to nearest even.
BCSIM_HD float ll2f_rn(long long v) {
    const unsigned long long a = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
    if (a == 0) return 0.0f;
    const int lz = clz64(a);
    const unsigned long long nrm = a << lz;   // leading one at bit 63
    unsigned mant = (unsigned)(nrm >> 40);     // 24 significant bits
    const unsigned long long rem = nrm & 0xffffffffffull;
    const unsigned long long half = 0x8000000000ull;
    mant += (rem > half || (rem == half && (mant & 1u))) ? 1u : 0u;
    // biased exponent 127 + 63 - lz; the hidden bit of mant adds one to the
    // exponent field, and a mantissa rounded up to 2^24 carries into it
    const unsigned bits = ((unsigned)(126 + 63 - lz) << 23) + mant;
    return fp_from_bits(bits | (v < 0 ? 0x80000000u : 0u));
}

#if defined(__CUDACC__)
// Fixed-point bin -> float (times inv_scale = 2^-S).  The magnitude is split
// as hi * 2^32 + lo; hi * 2^32 + float(lo) is rounded once by the FMA and
// float(lo) once before it, so the error is at most 2^7 units of the
// fixed-point scale plus half an FP32 ulp of the result -- 2^-54 of the scale's
// range bound 2^61, far below the FP32 resolution of any bin that matters --
// and conversion is odd (-v converts to exactly minus v's value).  No FP64 or
// 64-bit multiply instruction is involved.
__device__ __forceinline__ float fix2f(long long v, float inv_scale) {
    const unsigned long long a = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
    const float r = fmaf(__uint2float_rn((unsigned)(a >> 32)), 4294967296.0f, __uint2float_rn((unsigned)a)) * inv_scale;
    return v < 0 ? -r : r;
}
#endif

}  // namespace bcsim_gb300
