// imaging_host.hpp -- host orchestration of the device post-processing.
#pragma once
#include <cstdint>

#include "engine.hpp"
#include "imaging.hpp"

namespace bcsim_gb300 {

// Device scratch of the post-processing, owned by one handle (stream-ordered
// on that handle's stream).
struct ImagingBuffers {
    DeviceBuffer in;        // host inputs uploaded (IQ frame or packet)
    DeviceBuffer bytes;     // B-mode beam space
    DeviceBuffer image;     // scan-converted image
    DeviceBuffer r0, vel;   // Doppler estimates (r0: also float beam space input)
    DeviceBuffer scratch;   // maximum reduction partials
    DeviceBuffer scalar;    // normalisation constant / maximum
};

void check_scan_geometry(const ScanGeometry2D& g, int64_t beams, int64_t range);

// B-mode from a device IQ frame [L][nd]: normalisation (normalize <= 0: the
// frame's largest envelope), log compression to beam-space bytes, and (with g)
// scan conversion.  image ([ny][nx]), beamspace ([L][nd]) and normalize_used
// are host pointers (beamspace and normalize_used may be null).  Synchronises.
void bmode_from_device(cudaStream_t st, ImagingBuffers& b, const float2* d_iq, int64_t L, int64_t nd,
                       float dyn_range, float gain, float normalize, const ScanGeometry2D* g, uint8_t* image,
                       uint8_t* beamspace, float* normalize_used);

// Colour Doppler from a device packet [P][L][nd]: R0 and arg R1 per sample
// (host r0 / velocity [L][nd], either may be null) and (with g) the colour
// image (host bgra [ny][nx][4]).  Synchronises.
void doppler_from_device(cudaStream_t st, ImagingBuffers& b, const float2* d_packet, int P, int64_t L, int64_t nd,
                         float* r0, float* velocity, const ScanGeometry2D* g, uint8_t* bgra);

// Scan conversion of a host float beam space [beams][range] into host image [ny][nx].
void scan_convert_host(cudaStream_t st, ImagingBuffers& b, const float* beamspace, int64_t beams, int64_t range,
                       const ScanGeometry2D& g, float* image);

}  // namespace bcsim_gb300
