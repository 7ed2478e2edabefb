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

// Message of the last bcsim_create failure on this thread (no handle exists to hold it).
static thread_local std::string g_create_error;

struct bcsim_handle {
    bcsim_gb300::Simulator sim;
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

int bcsim_set_logger(bcsim_handle* h, bcsim_log_fn fn, void* user) {
    return guarded(h, [&] { h->sim.set_logger(fn, user); });
}

}  // extern "C"
