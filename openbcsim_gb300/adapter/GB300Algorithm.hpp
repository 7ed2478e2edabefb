// GB300Algorithm.hpp -- bcsim::IAlgorithm implemented by the GB300 engine.
//
// The C++ binding a maintainer adds to the reference, next to its own
// algorithms in src/core/algorithm/, so that bcsim::Create("gpu")
// (src/core/LibBCSim.cpp:39-49) returns this engine and every IAlgorithm
// caller (the Qt GUI, the examples, the Python binding) runs unchanged.  Each
// override forwards to the C ABI function of include/bcsim_gb300.h that
// replaces the reference member (src/core/LibBCSim.hpp:42-91); a failed call
// becomes the std::runtime_error the reference would throw, with its message.
#pragma once
#include <complex>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>
#include "../LibBCSim.hpp"
#include "../BeamProfile.hpp"
#include "bcsim_gb300.h"

namespace bcsim {

class GB300Algorithm : public IAlgorithm {
public:
    GB300Algorithm() {
        if (bcsim_create("gpu", &m_h) != BCSIM_OK) throw std::runtime_error(bcsim_last_error(nullptr));
    }
    ~GB300Algorithm() override { bcsim_destroy(m_h); }

    void set_parameter(const std::string& key, const std::string& value) override {
        check(bcsim_set_parameter(m_h, key.c_str(), value.c_str()));
    }
    std::string get_parameter(const std::string& key) const override {
        char buf[1024];
        check(bcsim_get_parameter(m_h, key.c_str(), buf, sizeof(buf)));
        return buf;
    }
    void clear_fixed_scatterers() override { check(bcsim_clear_fixed_scatterers(m_h)); }
    void add_fixed_scatterers(FixedScatterers::s_ptr fs) override {
        std::vector<float> xyza;
        xyza.reserve(4 * fs->scatterers.size());
        for (const auto& s : fs->scatterers) {
            xyza.push_back(s.pos.x); xyza.push_back(s.pos.y); xyza.push_back(s.pos.z); xyza.push_back(s.amplitude);
        }
        check(bcsim_add_fixed_scatterers(m_h, xyza.data(), (int64_t)fs->scatterers.size()));
    }
    void clear_spline_scatterers() override { check(bcsim_clear_spline_scatterers(m_h)); }
    void add_spline_scatterers(SplineScatterers::s_ptr ss) override {
        const int64_t n = ss->num_scatterers();
        const int k = n ? (int)ss->get_num_control_points() : 0;
        std::vector<float> cps;
        cps.reserve(3 * n * k);
        for (const auto& row : ss->control_points)
            for (const auto& p : row) { cps.push_back(p.x); cps.push_back(p.y); cps.push_back(p.z); }
        check(bcsim_add_spline_scatterers(m_h, ss->spline_degree, ss->knot_vector.data(),
                                          (int)ss->knot_vector.size(), cps.data(), ss->amplitudes.data(), n, k));
    }
    void set_scan_sequence(ScanSequence::s_ptr seq) override {
        const int n = seq->get_num_lines();
        std::vector<float> o(3 * n), d(3 * n), l(3 * n), t(n);
        for (int i = 0; i < n; i++) {
            const auto& s = seq->get_scanline(i);
            const auto a = s.get_origin(), b = s.get_direction(), c = s.get_lateral_dir();
            o[3*i] = a.x; o[3*i+1] = a.y; o[3*i+2] = a.z;
            d[3*i] = b.x; d[3*i+1] = b.y; d[3*i+2] = b.z;
            l[3*i] = c.x; l[3*i+1] = c.y; l[3*i+2] = c.z;
            t[i] = s.get_timestamp();
        }
        check(bcsim_set_scan_sequence(m_h, o.data(), d.data(), l.data(), t.data(), n, seq->line_length));
    }
    void set_excitation(const ExcitationSignal& ex) override {
        check(bcsim_set_excitation(m_h, ex.samples.data(), (int)ex.samples.size(), ex.center_index,
                                   ex.sampling_frequency, ex.demod_freq));
    }
    void set_analytical_profile(IBeamProfile::s_ptr bp) override {
        auto g = std::dynamic_pointer_cast<GaussianBeamProfile>(bp);
        if (!g) throw std::runtime_error("GB300Algorithm: failed to cast beam profile");
        check(bcsim_set_analytical_profile(m_h, g->getSigmaLateral(), g->getSigmaElevational()));
    }
    void set_lookup_profile(IBeamProfile::s_ptr bp) override {
        auto lut = std::dynamic_pointer_cast<LUTBeamProfile>(bp);
        if (!lut) throw std::runtime_error("GB300Algorithm: failed to cast beam profile");
        const auto r = lut->getRangeRange(), l = lut->getLateralRange(), e = lut->getElevationalRange();
        const std::vector<float>& s = LutSamples::of(*lut);   // [rad][lat][ele], BeamProfile.hpp:127-129
        check(bcsim_set_lookup_profile(m_h, s.data(), lut->getNumSamplesRadial(), lut->getNumSamplesLateral(),
                                       lut->getNumSamplesElevational(), r.first, r.last, l.first, l.last,
                                       e.first, e.last));
    }
    void simulate_lines(std::vector<std::vector<std::complex<float>>>& out) override {
        int64_t nl = 0, ns = 0;
        check(bcsim_get_output_shape(m_h, &nl, &ns));
        std::vector<std::complex<float>> flat((size_t)(nl * ns));
        check(bcsim_simulate_lines(m_h, reinterpret_cast<float*>(flat.data()), nl * ns, &nl, &ns));
        out.assign((size_t)nl, std::vector<std::complex<float>>());
        for (int64_t i = 0; i < nl; i++) out[i].assign(flat.begin() + i * ns, flat.begin() + (i + 1) * ns);
    }
    std::vector<double> get_debug_data(const std::string& key) const override {
        int64_t n = 0;
        bcsim_get_debug_data(m_h, key.c_str(), nullptr, 0, &n);
        std::vector<double> v((size_t)n);
        check(bcsim_get_debug_data(m_h, key.c_str(), v.data(), n, &n));
        return v;
    }
    size_t get_total_num_scatterers() const override {
        int64_t n = 0;
        check(bcsim_get_total_num_scatterers(m_h, &n));
        return (size_t)n;
    }
    void set_logger(ILog::ptr log) override {
        m_log = log;
        check(bcsim_set_logger(m_h, log ? &GB300Algorithm::forward : nullptr, this));
    }

private:
    // LUTBeamProfile keeps its samples in a protected member; naming it through a
    // derived class yields a member pointer that reads it from any LUTBeamProfile.
    struct LutSamples : public LUTBeamProfile {
        static const std::vector<float>& of(const LUTBeamProfile& p) { return p.*(&LutSamples::m_samples); }
    };
    static void forward(int level, const char* msg, void* user) {
        auto self = static_cast<GB300Algorithm*>(user);
        if (self->m_log) self->m_log->write(static_cast<ILog::LogType>(level), msg);
    }
    void check(int rc) const {
        if (rc != BCSIM_OK) throw std::runtime_error(bcsim_last_error(m_h));
    }
    bcsim_handle* m_h = nullptr;
    ILog::ptr m_log;
};

}  // namespace bcsim
