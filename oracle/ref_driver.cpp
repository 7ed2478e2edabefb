// ref_driver.cpp -- C entry points around the reference's own CPU algorithm.
//
// TEST INFRASTRUCTURE ONLY.  This file is compiled together with the reference
// sources where they lie (see oracle/Makefile) into oracle/_ref/libbcsim_ref.so.
// It drives the UNMODIFIED reference through its public factory and interface:
//   bcsim::Create("cpu")                      src/core/LibBCSim.cpp:39-49
//   IAlgorithm::set_parameter / set_excitation / set_scan_sequence /
//   set_analytical_profile / set_lookup_profile / add_fixed_scatterers /
//   add_spline_scatterers / simulate_lines   src/core/LibBCSim.hpp:42-91
// and exposes the reference helpers that its own unit tests pin
// (fft_conv, next_power_of_two: src/core/fft.cpp; discrete_hilbert_mask:
// src/core/discrete_hilbert_mask.hpp; MakeGaussianExcitation:
// src/utils/GaussPulse.cpp:52-70; bsplineBasis & friends: src/core/bspline.hpp).
#include <cstring>
#include <cstdio>
#include <string>
#include <vector>
#include <complex>
#ifdef _OPENMP
#include <omp.h>
#endif
#include <stdexcept>
#include "cole_case.h"
#include "LibBCSim.hpp"
#include "BeamProfile.hpp"
#include "ScanSequence.hpp"
#include "fft.hpp"
#include "discrete_hilbert_mask.hpp"
#include "bspline.hpp"
#include "utils/GaussPulse.hpp"
#include "algorithm/CpuAlgorithm.hpp"
#include "algorithm/common_utils.hpp"
#include "utils/ScanGeometry.hpp"
#include "utils/cartesianator/Cartesianator.hpp"

static void copy_err(const char* msg, char* err, int errcap) {
    if (err && errcap > 0) {
        std::snprintf(err, (size_t)errcap, "%s", msg);
    }
}

// Exposes the reference's own per-line projection loops
// (CpuAlgorithm::projection_loop, src/core/algorithm/CpuAlgorithm.cpp:50-183),
// which are protected members, so that the time-projection bins can be compared
// before any convolution.
class BinsProbe : public bcsim::CpuAlgorithm {
public:
    void project(const bcsim::Scanline& line, std::complex<float>* bins, size_t ns) {
        for (auto& f : m_scatterers_collection.fixed_collections) projection_loop(f, line, bins, ns);
        for (auto& s : m_scatterers_collection.spline_collections) projection_loop(s, line, bins, ns);
    }
    size_t num_samples() const { return m_rf_line_num_samples; }
};

static void configure(bcsim::IAlgorithm* sim, const cole_case* c, int num_threads);

// float -> string that parses back to the same float
static std::string fstr(float v) {
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%.9g", (double)v);
    return buf;
}

// The reference's scan converter (CpuCartesianator<T>, src/utils/cartesianator/
// Cartesianator.cpp:32-205) for a sector (kind 0: width, depth, tilt) or linear
// (kind 1: width, range_max = depth) geometry; in: [beams][range]; out: [ny][nx].
template <typename T>
static int ref_scan_convert_t(const T* in, int beams, int range, int kind, float width, float depth, float tilt,
                              int nx, int ny, T* out) {
    try {
        bcsim::ScanGeometry::ptr g;
        if (kind == 0) {
            auto s = std::make_shared<bcsim::SectorScanGeometry>();
            s->width = width;
            s->depth = depth;
            s->tilt = tilt;
            g = s;
        } else {
            auto l = std::make_shared<bcsim::LinearScanGeometry>();
            l->width = width;
            l->range_max = depth;
            g = l;
        }
        CpuCartesianator<T> cart;
        cart.SetGeometry(g);
        cart.SetOutputSize((size_t)nx, (size_t)ny);
        std::vector<T> buf(in, in + (size_t)beams * range);
        cart.Process(buf.data(), beams, range);
        const T* o = cart.GetOutputBuffer();
        std::memcpy(out, o, sizeof(T) * (size_t)nx * ny);
        return 0;
    } catch (const std::exception&) {
        return 1;
    }
}

extern "C" {

// Time-projection bins of one line from the reference's own projection loops.
// out: float [ns][2].  Returns 0 on success, 1 if the reference threw.
int ref_project_bins(const cole_case* c, int line_no, float* out, int64_t cap_pairs, int64_t* out_ns,
                     char* err, int errcap) {
    try {
        BinsProbe probe;
        configure(&probe, c, 1);
        const size_t ns = probe.num_samples();
        if (out_ns) *out_ns = (int64_t)ns;
        if ((int64_t)ns > cap_pairs) { copy_err("output buffer too small", err, errcap); return 2; }
        std::vector<std::complex<float>> bins(ns, std::complex<float>(0.0f, 0.0f));
        const float* o = c->origins + 3 * line_no;
        const float* d = c->directions + 3 * line_no;
        const float* l = c->lateral_dirs + 3 * line_no;
        bcsim::Scanline line(bcsim::vector3(o[0], o[1], o[2]), bcsim::vector3(d[0], d[1], d[2]),
                             bcsim::vector3(l[0], l[1], l[2]), c->timestamps[line_no]);
        probe.project(line, bins.data(), ns);
        std::memcpy(out, bins.data(), sizeof(float) * 2 * ns);
        return 0;
    } catch (const std::exception& e) {
        copy_err(e.what(), err, errcap);
        return 1;
    }
}

// Run simulate_lines of the reference CPU algorithm on one case.
// out: float [L][nd][2] (complex64).  Returns 0 on success, 1 if the reference
// threw (message copied to err), 2 if out is too small.
int ref_simulate(const cole_case* c, int num_threads, float* out, int64_t out_cap_floats,
                 int64_t* out_lines, int64_t* out_samples, char* err, int errcap) {
    try {
        auto sim = bcsim::Create("cpu");
        configure(sim.get(), c, num_threads);
        std::vector<std::vector<std::complex<float>>> lines;
        sim->simulate_lines(lines);
        const int64_t L = (int64_t)lines.size();
        const int64_t nd = L ? (int64_t)lines[0].size() : 0;
        if (out_lines) *out_lines = L;
        if (out_samples) *out_samples = nd;
        if (L * nd * 2 > out_cap_floats) {
            copy_err("output buffer too small", err, errcap);
            return 2;
        }
        for (int64_t i = 0; i < L; i++)
            std::memcpy(out + i * nd * 2, lines[i].data(), sizeof(float) * 2 * nd);
        return 0;
    } catch (const std::exception& e) {
        copy_err(e.what(), err, errcap);
        return 1;
    }
}

// The reference's fft_conv (src/core/fft.cpp:94-120), for its known-answer tests.
int ref_fft_conv(const float* x, int nx, const float* h, int nh, float* out) {
    std::vector<float> xv(x, x + nx), hv(h, h + nh);
    auto r = fft_conv(xv, hv);
    std::memcpy(out, r.data(), sizeof(float) * r.size());
    return (int)r.size();
}

int64_t ref_next_power_of_two(int64_t n) { return (int64_t)next_power_of_two((size_t)n); }

void ref_hilbert_mask(int n, int* out) {
    auto m = discrete_hilbert_mask<int>((size_t)n);
    for (int i = 0; i < n; i++) out[i] = m[i];
}

// MakeGaussianExcitation (src/utils/GaussPulse.cpp:52-70).  Returns the number of
// taps (and writes at most cap of them).
int ref_gaussian_excitation(float fc, float bw, float fs, float* out, int cap, int* center_index) {
    std::vector<float> times, samples;
    int ci = 0;
    bcsim::MakeGaussianExcitation<float>(fc, bw, fs, times, samples, ci);
    for (int i = 0; i < (int)samples.size() && i < cap; i++) out[i] = samples[i];
    if (center_index) *center_index = ci;
    return (int)samples.size();
}

float ref_bspline_basis(int j, int p, float x, const float* knots, int nk) {
    std::vector<float> k(knots, knots + nk);
    return bspline_storve::bsplineBasis<float>(j, p, x, k);
}

int ref_knot_interval(const float* knots, int nk, float t) {
    std::vector<float> k(knots, knots + nk);
    try {
        return bspline_storve::compute_knot_interval<float>(k, t);
    } catch (...) {
        return -1;
    }
}

int ref_uniform_regular_knots(int n, int p, float t0, float t1, float* out, int cap) {
    auto v = bspline_storve::uniform_regular_knot_vector<float>(n, p, t0, t1);
    for (int i = 0; i < (int)v.size() && i < cap; i++) out[i] = v[i];
    return (int)v.size();
}

int ref_scan_convert_f32(const float* in, int beams, int range, int kind, float width, float depth, float tilt, int nx,
                         int ny, float* out) {
    return ref_scan_convert_t(in, beams, range, kind, width, depth, tilt, nx, ny, out);
}

int ref_scan_convert_u8(const unsigned char* in, int beams, int range, int kind, float width, float depth, float tilt,
                        int nx, int ny, unsigned char* out) {
    return ref_scan_convert_t(in, beams, range, kind, width, depth, tilt, nx, ny, out);
}

}  // extern "C"

static void configure(bcsim::IAlgorithm* sim, const cole_case* c, int num_threads) {
        if (num_threads > 0) {
#ifdef _OPENMP
            // the reference accepts at most omp_get_max_threads() cores
            // (CpuAlgorithm.cpp:203-215): raise this thread's OpenMP limit to the
            // requested count first, as process launchers (torchrun) start their
            // workers with OMP_NUM_THREADS=1
            if (num_threads > omp_get_max_threads()) omp_set_num_threads(num_threads);
#endif
            sim->set_parameter("num_cpu_cores", std::to_string(num_threads));
        }
        sim->set_parameter("sound_speed", fstr(c->sound_speed));
        sim->set_parameter("use_arc_projection", c->use_arc_projection ? "on" : "off");
        sim->set_parameter("phase_delay", c->phase_delay ? "on" : "off");
        sim->set_parameter("radial_decimation", std::to_string(c->radial_decimation));

        bcsim::ExcitationSignal ex;
        ex.samples.assign(c->taps, c->taps + c->num_taps);
        ex.center_index = c->center_index;
        ex.sampling_frequency = c->fs;
        ex.demod_freq = c->demod_freq;
        sim->set_excitation(ex);

        auto seq = std::make_shared<bcsim::ScanSequence>(c->line_length);
        for (int i = 0; i < c->num_lines; i++) {
            const float* o = c->origins + 3 * i;
            const float* d = c->directions + 3 * i;
            const float* l = c->lateral_dirs + 3 * i;
            seq->add_scanline(bcsim::Scanline(bcsim::vector3(o[0], o[1], o[2]),
                                              bcsim::vector3(d[0], d[1], d[2]),
                                              bcsim::vector3(l[0], l[1], l[2]),
                                              c->timestamps[i]));
        }
        sim->set_scan_sequence(seq);

        if (c->beam == COLE_BEAM_GAUSSIAN) {
            sim->set_analytical_profile(std::make_shared<bcsim::GaussianBeamProfile>(c->sigma_lateral, c->sigma_elevational));
        } else if (c->beam == COLE_BEAM_LUT) {
            auto lut = std::make_shared<bcsim::LUTBeamProfile>(
                c->lut_nr, c->lut_nl, c->lut_ne,
                bcsim::Interval(c->lut_r[0], c->lut_r[1]),
                bcsim::Interval(c->lut_l[0], c->lut_l[1]),
                bcsim::Interval(c->lut_e[0], c->lut_e[1]));
            for (int ir = 0; ir < c->lut_nr; ir++)
                for (int il = 0; il < c->lut_nl; il++)
                    for (int ie = 0; ie < c->lut_ne; ie++)
                        lut->setDiscreteSample(ir, il, ie, c->lut[((int64_t)ir * c->lut_nl + il) * c->lut_ne + ie]);
            sim->set_lookup_profile(lut);
        }

        for (int s = 0; s < c->num_fixed_sets; s++) {
            auto fs = std::make_shared<bcsim::FixedScatterers>();
            const float* p = c->fixed_xyza[s];
            fs->scatterers.resize((size_t)c->fixed_counts[s]);
            for (int64_t i = 0; i < c->fixed_counts[s]; i++) {
                fs->scatterers[i].pos = bcsim::vector3(p[4 * i], p[4 * i + 1], p[4 * i + 2]);
                fs->scatterers[i].amplitude = p[4 * i + 3];
            }
            sim->add_fixed_scatterers(fs);
        }
        for (int s = 0; s < c->num_spline_sets; s++) {
            const cole_spline_set& ss = c->spline_sets[s];
            auto sp = std::make_shared<bcsim::SplineScatterers>();
            sp->spline_degree = ss.degree;
            sp->knot_vector.assign(ss.knots, ss.knots + ss.num_knots);
            sp->control_points.resize((size_t)ss.num_scatterers);
            sp->amplitudes.assign(ss.amplitudes, ss.amplitudes + ss.num_scatterers);
            for (int64_t i = 0; i < ss.num_scatterers; i++) {
                sp->control_points[i].resize(ss.num_cs);
                for (int k = 0; k < ss.num_cs; k++) {
                    const float* q = ss.control_points + (i * ss.num_cs + k) * 3;
                    sp->control_points[i][k] = bcsim::vector3(q[0], q[1], q[2]);
                }
            }
            sim->add_spline_scatterers(sp);
        }

}
