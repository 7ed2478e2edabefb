// capi.cpp -- the extern "C" boundary declared in include/bcsim_gb300.h.
// Every entry point catches all C++ exceptions and turns them into a status
// code plus the handle's last-error message.
#include <cstring>
#include <exception>
#include <new>
#include <stdexcept>
#include <string>

#include "../../include/bcsim_gb300.h"
#include "engine.hpp"
#include "imaging_host.hpp"

// Message of the last bcsim_create failure on this thread (no handle exists to hold it).
static thread_local std::string g_create_error;

struct bcsim_handle {
    bcsim_gb300::Simulator sim;
    bcsim_gb300::ImagingBuffers imaging;
    bcsim_gb300::DeviceBuffer packet;   // device IQ of the imaging entry points
    std::string last_error;
};

namespace bcsim_gb300 {
Simulator& simulator_of(bcsim_handle* h) { return h->sim; }
}  // namespace bcsim_gb300

namespace {
template <typename F>
int guarded(bcsim_handle* h, F&& f) {
    if (!h) return BCSIM_E_INVALID;
    try {
        f();
        h->last_error.clear();
        return BCSIM_OK;
    } catch (const bcsim_gb300::SimError& e) {
        h->last_error = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        h->last_error = "host allocation failed";
        return BCSIM_E_MEMORY;
    } catch (const std::logic_error& e) {
        // std::stoi / std::stof failures (std::invalid_argument, std::out_of_range)
        // are logic_errors, as in the reference's set_parameter
        h->last_error = e.what();
        return BCSIM_E_INVALID;
    } catch (const std::exception& e) {
        h->last_error = e.what();
        return BCSIM_E_INTERNAL;
    } catch (...) {
        h->last_error = "unknown error";
        return BCSIM_E_INTERNAL;
    }
}
}  // namespace

extern "C" {

int bcsim_create(const char* sim_type, bcsim_handle** out) {
    if (!out) return BCSIM_E_INVALID;
    *out = nullptr;
    const std::string t = sim_type ? sim_type : "";
    // LibBCSim.cpp:39-49
    if (t != "gpu") {
        g_create_error = "Illegal algorithm type: " + t;
        return BCSIM_E_INVALID;
    }
    try {
        *out = new bcsim_handle();
    } catch (...) {
        g_create_error = "host allocation failed";
        return BCSIM_E_MEMORY;
    }
    g_create_error.clear();
    return BCSIM_OK;
}

int bcsim_destroy(bcsim_handle* h) {
    delete h;
    return BCSIM_OK;
}

const char* bcsim_last_error(const bcsim_handle* h) { return h ? h->last_error.c_str() : g_create_error.c_str(); }

int bcsim_set_parameter(bcsim_handle* h, const char* key, const char* value) {
    return guarded(h, [&] { h->sim.set_parameter(key ? key : "", value ? value : ""); });
}

int bcsim_get_parameter(const bcsim_handle* hc, const char* key, char* buf, int cap) {
    bcsim_handle* h = const_cast<bcsim_handle*>(hc);
    return guarded(h, [&] {
        const std::string v = h->sim.get_parameter(key ? key : "");
        if (!buf || cap <= (int)v.size()) throw bcsim_gb300::SimError(BCSIM_E_CAPACITY, "buffer too small");
        std::memcpy(buf, v.c_str(), v.size() + 1);
    });
}

int bcsim_set_excitation(bcsim_handle* h, const float* samples, int n, int center_index, float fs, float fd) {
    return guarded(h, [&] { h->sim.set_excitation(samples, n, center_index, fs, fd); });
}

int bcsim_set_scan_sequence(bcsim_handle* h, const float* origins, const float* directions, const float* lateral_dirs,
                            const float* timestamps, int num_lines, float line_length) {
    return guarded(h, [&] {
        h->sim.set_scan_sequence(origins, directions, lateral_dirs, timestamps, num_lines, line_length);
    });
}

int bcsim_set_analytical_profile(bcsim_handle* h, float sl, float se) {
    return guarded(h, [&] { h->sim.set_analytical_profile(sl, se); });
}

int bcsim_set_lookup_profile(bcsim_handle* h, const float* samples, int nr, int nl, int ne, float r0, float r1,
                             float l0, float l1, float e0, float e1) {
    return guarded(h, [&] { h->sim.set_lookup_profile(samples, nr, nl, ne, r0, r1, l0, l1, e0, e1); });
}

int bcsim_clear_fixed_scatterers(bcsim_handle* h) {
    return guarded(h, [&] { h->sim.clear_fixed_scatterers(); });
}

int bcsim_add_fixed_scatterers(bcsim_handle* h, const float* xyza, int64_t n) {
    return guarded(h, [&] { h->sim.add_fixed_scatterers(xyza, n); });
}

int bcsim_set_fixed_scatterers(bcsim_handle* h, const float* xyza, int64_t n) {
    return guarded(h, [&] {
        h->sim.clear_fixed_scatterers();
        h->sim.add_fixed_scatterers(xyza, n);
    });
}

int bcsim_clear_spline_scatterers(bcsim_handle* h) {
    return guarded(h, [&] { h->sim.clear_spline_scatterers(); });
}

int bcsim_add_spline_scatterers(bcsim_handle* h, int degree, const float* knots, int num_knots,
                                const float* control_points, const float* amplitudes, int64_t n, int num_cs) {
    return guarded(h, [&] {
        h->sim.add_spline_scatterers(degree, knots, num_knots, control_points, amplitudes, n, num_cs);
    });
}

int bcsim_set_spline_scatterers(bcsim_handle* h, int degree, const float* knots, int num_knots,
                                const float* control_points, const float* amplitudes, int64_t n, int num_cs) {
    return guarded(h, [&] {
        h->sim.clear_spline_scatterers();
        h->sim.add_spline_scatterers(degree, knots, num_knots, control_points, amplitudes, n, num_cs);
    });
}

int bcsim_get_total_num_scatterers(const bcsim_handle* hc, int64_t* out) {
    bcsim_handle* h = const_cast<bcsim_handle*>(hc);
    return guarded(h, [&] {
        if (!out) throw bcsim_gb300::SimError(BCSIM_E_INVALID, "null output pointer");
        *out = h->sim.total_num_scatterers();
    });
}

int bcsim_get_output_shape(const bcsim_handle* hc, int64_t* num_lines, int64_t* num_samples) {
    bcsim_handle* h = const_cast<bcsim_handle*>(hc);
    return guarded(h, [&] { h->sim.output_shape(num_lines, num_samples); });
}

int bcsim_simulate_lines(bcsim_handle* h, float* out, int64_t cap_complex, int64_t* num_lines, int64_t* num_samples) {
    return guarded(h, [&] { h->sim.simulate_host(out, cap_complex, num_lines, num_samples); });
}

int bcsim_simulate_fixed_frames(bcsim_handle* h, const float* const* xyza_frames, int64_t n, int num_frames,
                                float* const* iq_out_frames, int64_t cap_complex) {
    return guarded(h, [&] { h->sim.simulate_fixed_frames(xyza_frames, n, num_frames, iq_out_frames, cap_complex); });
}

int bcsim_simulate_spline_frames(bcsim_handle* h, int degree, const float* knots, int num_knots,
                                 const float* const* cps_frames, const float* const* amps_frames, int64_t n,
                                 int num_cs, int num_frames, float* const* iq_out_frames, int64_t cap_complex) {
    return guarded(h, [&] {
        h->sim.simulate_spline_frames(degree, knots, num_knots, cps_frames, amps_frames, n, num_cs, num_frames,
                                      iq_out_frames, cap_complex);
    });
}

int bcsim_simulate_lines_device(bcsim_handle* h, void* device_out, int64_t cap_complex) {
    return guarded(h, [&] { h->sim.simulate_device(device_out, cap_complex); });
}

int bcsim_get_stream(const bcsim_handle* hc, void** stream) {
    bcsim_handle* h = const_cast<bcsim_handle*>(hc);
    return guarded(h, [&] {
        if (!stream) throw bcsim_gb300::SimError(BCSIM_E_INVALID, "null output pointer");
        *stream = (void*)h->sim.stream();
    });
}

int bcsim_get_debug_data(const bcsim_handle* hc, const char* key, double* out, int64_t cap, int64_t* n) {
    bcsim_handle* h = const_cast<bcsim_handle*>(hc);
    return guarded(h, [&] {
        const auto v = h->sim.get_debug_data(key ? key : "");
        if (n) *n = (int64_t)v.size();
        if ((int64_t)v.size() > cap || (!out && !v.empty()))
            throw bcsim_gb300::SimError(BCSIM_E_CAPACITY, "buffer too small");
        for (size_t i = 0; i < v.size(); i++) out[i] = v[i];
    });
}

namespace {
bcsim_gb300::ScanGeometry2D to_geometry(const bcsim_scan_geometry* g) {
    return bcsim_gb300::ScanGeometry2D{g->kind, g->width, g->depth, g->tilt, g->nx, g->ny};
}
}  // namespace

int bcsim_bmode_image(bcsim_handle* h, const float* iq, int64_t num_lines, int64_t num_samples, float dyn_range,
                      float gain, float normalize, const bcsim_scan_geometry* geometry, uint8_t* image,
                      uint8_t* beamspace, float* normalize_used) {
    return guarded(h, [&] {
        using bcsim_gb300::SimError;
        if (!iq || num_lines <= 0 || num_samples <= 0) throw SimError(BCSIM_E_INVALID, "No lines returned");
        if (geometry && !image) throw SimError(BCSIM_E_INVALID, "null image pointer");
        const cudaStream_t st = h->sim.stream();
        const size_t bytes = (size_t)num_lines * num_samples * sizeof(float2);
        h->packet.reserve(bytes, st);
        if (cudaMemcpyAsync(h->packet.get(), iq, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess)
            throw SimError(BCSIM_E_CUDA, "IQ upload failed");
        bcsim_gb300::ScanGeometry2D g{};
        if (geometry) g = to_geometry(geometry);
        bcsim_gb300::bmode_from_device(st, h->imaging, h->packet.as<float2>(), num_lines, num_samples, dyn_range, gain,
                                       normalize, geometry ? &g : nullptr, image, beamspace, normalize_used);
    });
}

int bcsim_simulate_bmode(bcsim_handle* h, float dyn_range, float gain, float normalize,
                         const bcsim_scan_geometry* geometry, uint8_t* image, uint8_t* beamspace,
                         float* normalize_used) {
    return guarded(h, [&] {
        using bcsim_gb300::SimError;
        if (geometry && !image) throw SimError(BCSIM_E_INVALID, "null image pointer");
        int64_t L = 0, nd = 0;
        h->sim.output_shape(&L, &nd);
        const cudaStream_t st = h->sim.stream();
        h->packet.reserve((size_t)L * nd * sizeof(float2), st);
        h->sim.simulate_device(h->packet.get(), L * nd);
        bcsim_gb300::ScanGeometry2D g{};
        if (geometry) g = to_geometry(geometry);
        bcsim_gb300::bmode_from_device(st, h->imaging, h->packet.as<float2>(), L, nd, dyn_range, gain, normalize,
                                       geometry ? &g : nullptr, image, beamspace, normalize_used);
        h->sim.check_device_flag();
    });
}

int bcsim_scan_convert(bcsim_handle* h, const float* beamspace, int64_t num_beams, int64_t num_range,
                       const bcsim_scan_geometry* geometry, float* image) {
    return guarded(h, [&] {
        if (!beamspace || !geometry || !image) throw bcsim_gb300::SimError(BCSIM_E_INVALID, "null pointer");
        bcsim_gb300::scan_convert_host(h->sim.stream(), h->imaging, beamspace, num_beams, num_range,
                                       to_geometry(geometry), image);
    });
}

int bcsim_simulate_packet(bcsim_handle* h, int packet_size, float prt, float* out, int64_t cap_complex) {
    return guarded(h, [&] {
        using bcsim_gb300::SimError;
        int64_t L = 0, nd = 0;
        h->sim.output_shape(&L, &nd);
        if (packet_size < 1) throw SimError(BCSIM_E_INVALID, "packet size must be at least 1");
        const int64_t total = (int64_t)packet_size * L * nd;
        if (!out || cap_complex < total)
            throw SimError(BCSIM_E_CAPACITY, "output buffer too small: need " + std::to_string(total) + " complex values");
        const cudaStream_t st = h->sim.stream();
        h->packet.reserve((size_t)total * sizeof(float2), st);
        h->sim.simulate_packet(packet_size, prt, h->packet.as<float2>(), total);
        if (cudaMemcpyAsync(out, h->packet.get(), (size_t)total * sizeof(float2), cudaMemcpyDeviceToHost, st) !=
                cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            throw SimError(BCSIM_E_CUDA, "packet download failed");
    });
}

int bcsim_color_doppler(bcsim_handle* h, const float* iq_packet, int packet_size, int64_t num_lines,
                        int64_t num_samples, float* r0, float* velocity, const bcsim_scan_geometry* geometry,
                        uint8_t* bgra) {
    return guarded(h, [&] {
        using bcsim_gb300::SimError;
        if (!iq_packet || num_lines <= 0 || num_samples <= 0) throw SimError(BCSIM_E_INVALID, "No lines returned");
        if (packet_size < 2) throw SimError(BCSIM_E_INVALID, "a colour-Doppler packet needs at least 2 frames");
        if (geometry && !bgra) throw SimError(BCSIM_E_INVALID, "null image pointer");
        const cudaStream_t st = h->sim.stream();
        const size_t bytes = (size_t)packet_size * num_lines * num_samples * sizeof(float2);
        h->packet.reserve(bytes, st);
        if (cudaMemcpyAsync(h->packet.get(), iq_packet, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess)
            throw SimError(BCSIM_E_CUDA, "IQ upload failed");
        bcsim_gb300::ScanGeometry2D g{};
        if (geometry) g = to_geometry(geometry);
        bcsim_gb300::doppler_from_device(st, h->imaging, h->packet.as<float2>(), packet_size, num_lines, num_samples,
                                         r0, velocity, geometry ? &g : nullptr, bgra);
    });
}

int bcsim_simulate_color_doppler(bcsim_handle* h, int packet_size, float prt, float* r0, float* velocity,
                                 const bcsim_scan_geometry* geometry, uint8_t* bgra) {
    return guarded(h, [&] {
        using bcsim_gb300::SimError;
        if (packet_size < 2) throw SimError(BCSIM_E_INVALID, "a colour-Doppler packet needs at least 2 frames");
        if (geometry && !bgra) throw SimError(BCSIM_E_INVALID, "null image pointer");
        int64_t L = 0, nd = 0;
        h->sim.output_shape(&L, &nd);
        const int64_t total = (int64_t)packet_size * L * nd;
        const cudaStream_t st = h->sim.stream();
        h->packet.reserve((size_t)total * sizeof(float2), st);
        h->sim.simulate_packet(packet_size, prt, h->packet.as<float2>(), total);
        bcsim_gb300::ScanGeometry2D g{};
        if (geometry) g = to_geometry(geometry);
        bcsim_gb300::doppler_from_device(st, h->imaging, h->packet.as<float2>(), packet_size, L, nd, r0, velocity,
                                         geometry ? &g : nullptr, bgra);
    });
}

int bcsim_debug_raise_wait_flag(bcsim_handle* h) {
    return guarded(h, [&] { h->sim.raise_device_flag(); });
}

int bcsim_set_logger(bcsim_handle* h, bcsim_log_fn fn, void* user) {
    return guarded(h, [&] { h->sim.set_logger(fn, user); });
}

}  // extern "C"
