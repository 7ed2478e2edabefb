// noise.cuh -- seeded Gaussian noise on the time-projection bins.
//
// The reference adds complex noise N(0, sigma) to every sample of a line's
// time-projection buffer before the convolution (CPU: two draws per sample
// from an unseeded std::default_random_engine, CpuAlgorithm.cpp:340-347; GPU:
// cuRAND normals added by AddNoiseKernel, GpuAlgorithm.cpp:165-177,270-277 and
// cuda_kernels_common.cu:67-72), so its noise cannot be reproduced.  Here the
// noise of sample j of line l in frame f is a pure function of (seed, f, l, j):
// one Philox4x32-10 block (Salmon, Moraes, Dror and Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC 2011) with key = the 64-bit seed and counter
// = (j, l, f, 0x6e6f6973), whose first two words become two independent
// normals by the Box-Muller transform.  The noise therefore does not depend on
// how lines are tiled, ordered or convolved, and a frame can be reproduced by
// its seed and frame number.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace bcsim_gb300 {

// Noise of one simulation: sigma = 0 turns it off.  line0: the absolute index
// of the first line a launch sees (launches may cover a block of lines).
struct NoiseParams {
    float sigma;
    uint32_t key0, key1;   // the seed, low and high words
    uint32_t frame;        // frame counter of the simulator
    int line0;
};

constexpr uint32_t PHILOX_M0 = 0xD2511F53u, PHILOX_M1 = 0xCD9E8D57u;   // round multipliers
constexpr uint32_t PHILOX_W0 = 0x9E3779B9u, PHILOX_W1 = 0xBB67AE85u;   // key schedule (Weyl) increments
constexpr uint32_t NOISE_TAG = 0x6e6f6973u;                              // fourth counter word

__host__ __device__ __forceinline__ uint32_t mulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
#endif
}

// Philox4x32 with 10 rounds: c (counter) -> c, key (k0, k1).
__host__ __device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        if (r > 0) {
            k0 += PHILOX_W0;
            k1 += PHILOX_W1;
        }
        const uint32_t hi0 = mulhi32(PHILOX_M0, c[0]), lo0 = PHILOX_M0 * c[0];
        const uint32_t hi1 = mulhi32(PHILOX_M1, c[2]), lo1 = PHILOX_M1 * c[2];
        const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
    }
}

#ifdef __CUDACC__
// The noise (re, im) of sample j of absolute line `line`, in FP32: u1 in (0, 1)
// from the top 24 bits of word 0 (offset by half a step), u2 in [0, 1) from
// word 1; radius sqrt(-2 ln u1), angle 2 pi u2.
__device__ __forceinline__ float2 bin_noise(const NoiseParams& nz, int line, int j) {
    uint32_t c[4] = {(uint32_t)j, (uint32_t)line, nz.frame, NOISE_TAG};
    philox4x32_10(c, nz.key0, nz.key1);
    const float u1 = ((float)(c[0] >> 8) + 0.5f) * 0x1p-24f;
    const float u2 = (float)(c[1] >> 8) * 0x1p-24f;
    const float rad = nz.sigma * sqrtf(-2.0f * logf(u1));
    float s, co;
    sincospif(2.0f * u2, &s, &co);
    return make_float2(rad * co, rad * s);
}
#endif

}  // namespace bcsim_gb300
