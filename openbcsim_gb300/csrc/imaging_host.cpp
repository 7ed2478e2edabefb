// imaging_host.cpp -- host side of the device post-processing (imaging.cu):
// argument checks, device scratch on the simulator's stream, transfers.
#include <cmath>
#include <string>

#include "../../include/bcsim_gb300.h"
#include "imaging_host.hpp"

namespace bcsim_gb300 {

#define BCSIM_IMG_CUDA(call)                                                                                \
    do {                                                                                                    \
        cudaError_t e_ = (call);                                                                            \
        if (e_ != cudaSuccess)                                                                              \
            throw SimError(BCSIM_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));               \
    } while (0)

void check_scan_geometry(const ScanGeometry2D& g, int64_t beams, int64_t range) {
    if (g.kind != SCAN_SECTOR && g.kind != SCAN_LINEAR) throw SimError(BCSIM_E_INVALID, "unknown geometry");
    if (g.nx < 2 || g.ny < 2) throw SimError(BCSIM_E_INVALID, "output image must be at least 2 x 2 pixels");
    // the interpolation grid divides by (beams - 1) and (range - 1) (Cartesianator.cpp:119-120, 175-176)
    if (beams < 2 || range < 2) throw SimError(BCSIM_E_INVALID, "scan conversion needs at least 2 beams and 2 samples");
    if (beams > (1 << 30) || range > (1 << 30)) throw SimError(BCSIM_E_INVALID, "beam space too large");
    if (!(g.depth > 0.0f) || !std::isfinite(g.width) || !std::isfinite(g.tilt) || !(g.width > 0.0f))
        throw SimError(BCSIM_E_INVALID, "invalid scan geometry");
}

void bmode_from_device(cudaStream_t st, ImagingBuffers& b, const float2* d_iq, int64_t L, int64_t nd,
                       float dyn_range, float gain, float normalize, const ScanGeometry2D* g, uint8_t* image,
                       uint8_t* beamspace, float* normalize_used) {
    const int64_t n = L * nd;
    if (n <= 0) throw SimError(BCSIM_E_INVALID, "No lines returned");
    if (!(dyn_range > 0.0f)) throw SimError(BCSIM_E_INVALID, "dynamic range must be positive");
    if (g) check_scan_geometry(*g, L, nd);
    b.scalar.reserve(2 * sizeof(float), st);
    b.scratch.reserve(imaging_max_scratch_floats() * sizeof(float), st);
    b.bytes.reserve((size_t)n, st);
    float* d_norm = b.scalar.as<float>();
    if (normalize > 0.0f) {
        BCSIM_IMG_CUDA(cudaMemcpyAsync(d_norm, &normalize, sizeof(float), cudaMemcpyHostToDevice, st));
    } else {   // bcsim::get_max_value of the envelope (BCSimConvenience.cpp:57-63)
        BCSIM_IMG_CUDA(launch_envelope_max(d_iq, n, b.scratch.as<float>(), d_norm, st));
    }
    BCSIM_IMG_CUDA(launch_log_compress(d_iq, n, dyn_range, gain, d_norm, b.bytes.as<uint8_t>(), st));
    if (g) {
        b.image.reserve((size_t)g->nx * g->ny, st);
        BCSIM_IMG_CUDA(launch_scan_convert_u8(b.bytes.as<uint8_t>(), (int)L, (int)nd, *g, b.image.as<uint8_t>(), st));
        BCSIM_IMG_CUDA(cudaMemcpyAsync(image, b.image.get(), (size_t)g->nx * g->ny, cudaMemcpyDeviceToHost, st));
    }
    if (beamspace) BCSIM_IMG_CUDA(cudaMemcpyAsync(beamspace, b.bytes.get(), (size_t)n, cudaMemcpyDeviceToHost, st));
    float used = normalize;
    BCSIM_IMG_CUDA(cudaMemcpyAsync(&used, d_norm, sizeof(float), cudaMemcpyDeviceToHost, st));
    BCSIM_IMG_CUDA(cudaStreamSynchronize(st));
    if (normalize_used) *normalize_used = used;
}

void doppler_from_device(cudaStream_t st, ImagingBuffers& b, const float2* d_packet, int P, int64_t L, int64_t nd,
                         float* r0, float* velocity, const ScanGeometry2D* g, uint8_t* bgra) {
    const int64_t n = L * nd;
    if (P < 2) throw SimError(BCSIM_E_INVALID, "a colour-Doppler packet needs at least 2 frames");
    if (n <= 0) throw SimError(BCSIM_E_INVALID, "No lines returned");
    if (g) check_scan_geometry(*g, L, nd);
    b.r0.reserve((size_t)n * sizeof(float), st);
    b.vel.reserve((size_t)n * sizeof(float), st);
    BCSIM_IMG_CUDA(launch_doppler(d_packet, P, n, b.r0.as<float>(), b.vel.as<float>(), st));
    if (g) {
        // max R0 over the frame (RefreshWorker.hpp:309), then the colour image
        b.scalar.reserve(2 * sizeof(float), st);
        b.scratch.reserve(imaging_max_scratch_floats() * sizeof(float), st);
        BCSIM_IMG_CUDA(launch_value_max(b.r0.as<float>(), n, b.scratch.as<float>(), b.scalar.as<float>(), st));
        b.image.reserve((size_t)g->nx * g->ny * 4, st);
        BCSIM_IMG_CUDA(launch_color_image(b.r0.as<float>(), b.vel.as<float>(), b.scalar.as<float>(), (int)L, (int)nd,
                                          *g, b.image.as<uint8_t>(), st));
        BCSIM_IMG_CUDA(cudaMemcpyAsync(bgra, b.image.get(), (size_t)g->nx * g->ny * 4, cudaMemcpyDeviceToHost, st));
    }
    if (r0) BCSIM_IMG_CUDA(cudaMemcpyAsync(r0, b.r0.get(), (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, st));
    if (velocity)
        BCSIM_IMG_CUDA(cudaMemcpyAsync(velocity, b.vel.get(), (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, st));
    BCSIM_IMG_CUDA(cudaStreamSynchronize(st));
}

void scan_convert_host(cudaStream_t st, ImagingBuffers& b, const float* beamspace, int64_t beams, int64_t range,
                       const ScanGeometry2D& g, float* image) {
    check_scan_geometry(g, beams, range);
    const size_t in_bytes = (size_t)beams * range * sizeof(float), out_bytes = (size_t)g.nx * g.ny * sizeof(float);
    b.r0.reserve(in_bytes, st);
    b.image.reserve(out_bytes, st);
    BCSIM_IMG_CUDA(cudaMemcpyAsync(b.r0.get(), beamspace, in_bytes, cudaMemcpyHostToDevice, st));
    BCSIM_IMG_CUDA(launch_scan_convert_f32(b.r0.as<float>(), (int)beams, (int)range, g, b.image.as<float>(), st));
    BCSIM_IMG_CUDA(cudaMemcpyAsync(image, b.image.get(), out_bytes, cudaMemcpyDeviceToHost, st));
    BCSIM_IMG_CUDA(cudaStreamSynchronize(st));
}

}  // namespace bcsim_gb300
