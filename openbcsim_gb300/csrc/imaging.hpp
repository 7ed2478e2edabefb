// imaging.hpp -- device post-processing of simulated IQ (imaging.cu): B-mode
// beam space and scan conversion, colour-Doppler estimates and image.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace bcsim_gb300 {

enum ScanKind : int { SCAN_SECTOR = 0, SCAN_LINEAR = 1 };

// The reference's scan geometries (src/utils/ScanGeometry.hpp:44-78) and the
// output image size of its Cartesianator (Cartesianator.hpp:67-104).
struct ScanGeometry2D {
    int kind;      // ScanKind
    float width;   // sector: opening angle [rad]; linear: scan width [m]
    float depth;   // sector: depth [m]; linear: maximum range [m]
    float tilt;    // sector tilt [rad]
    int nx, ny;    // output pixels (>= 2 each)
};

// Scratch floats the maximum reductions need.
size_t imaging_max_scratch_floats();
// *out = max over i < n of |iq[i]| / of v[i] (device scalar; deterministic).
cudaError_t launch_envelope_max(const float2* iq, int64_t n, float* scratch, float* out, cudaStream_t st);
cudaError_t launch_value_max(const float* v, int64_t n, float* scratch, float* out, cudaStream_t st);
// B-mode beam-space bytes of n IQ samples (normalize_dev: device scalar).
cudaError_t launch_log_compress(const float2* iq, int64_t n, float dyn_range, float gain, const float* normalize_dev,
                                uint8_t* out, cudaStream_t st);
// Beam space [beams][range] -> image [ny][nx].
cudaError_t launch_scan_convert_u8(const uint8_t* in, int beams, int range, const ScanGeometry2D& g, uint8_t* out,
                                   cudaStream_t st);
cudaError_t launch_scan_convert_f32(const float* in, int beams, int range, const ScanGeometry2D& g, float* out,
                                    cudaStream_t st);
// Packet [P][n] complex -> R0 [n], arg R1 [n] (either may be null).
cudaError_t launch_doppler(const float2* packet, int P, int64_t n, float* r0, float* vel, cudaStream_t st);
// Colour image [ny][nx] of (B, G, R, A) bytes from R0 / velocity beam space.
cudaError_t launch_color_image(const float* r0, const float* vel, const float* r0_max_dev, int beams, int range,
                               const ScanGeometry2D& g, uint8_t* bgra, cudaStream_t st);

}  // namespace bcsim_gb300
