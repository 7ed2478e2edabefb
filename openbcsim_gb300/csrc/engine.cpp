// engine.cpp -- host side of the GB300 COLE simulator (see engine.hpp).
#include "engine.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <map>
#include <mutex>
#include <sstream>

#include "../../include/bcsim_gb300.h"
#include "host_dsp.hpp"

namespace bcsim_gb300 {

#define BCSIM_CUDA(call)                                                                                    \
    do {                                                                                                    \
        cudaError_t e_ = (call);                                                                            \
        if (e_ != cudaSuccess) {                                                                            \
            throw SimError(BCSIM_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_) + " (" __FILE__ \
                                             ":" + std::to_string(__LINE__) + ")");                          \
        }                                                                                                   \
    } while (0)

// ---------------------------------------------------------------------------
// DeviceBuffer
// ---------------------------------------------------------------------------
DeviceBuffer& DeviceBuffer::operator=(DeviceBuffer&& o) noexcept {
    if (this != &o) {
        release();
        ptr_ = o.ptr_;
        bytes_ = o.bytes_;
        stream_ = o.stream_;
        o.ptr_ = nullptr;
        o.bytes_ = 0;
    }
    return *this;
}

DeviceBuffer::~DeviceBuffer() { release(); }

void DeviceBuffer::release() {
    if (ptr_) {
        if (stream_) cudaFreeAsync(ptr_, stream_);
        else cudaFree(ptr_);
    }
    ptr_ = nullptr;
    bytes_ = 0;
}

void DeviceBuffer::reserve(size_t bytes, cudaStream_t stream) {
    if (bytes <= bytes_ && ptr_) return;
    // a buffer that has to grow grows by at least half, so that a sequence of
    // slowly growing requests reallocates only a few times
    if (ptr_) bytes = std::max(bytes, bytes_ + bytes_ / 2);
    release();
    if (bytes == 0) bytes = 16;
    bytes = (bytes + 255) & ~(size_t)255;
    const cudaError_t e = stream ? cudaMallocAsync(&ptr_, bytes, stream) : cudaMalloc(&ptr_, bytes);
    if (e != cudaSuccess) {
        ptr_ = nullptr;
        cudaGetLastError();
        throw SimError(BCSIM_E_MEMORY, std::string("device allocation of ") + std::to_string(bytes) +
                                           " bytes failed: " + cudaGetErrorString(e));
    }
    stream_ = stream;
    bytes_ = bytes;
}

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
static bool parse_bool(const std::string& v, bool* out) {
    if (v == "on" || v == "true") { *out = true; return true; }
    if (v == "off" || v == "false") { *out = false; return true; }
    return false;
}

static float fdot(const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

static std::string fmt_double(double v) {
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%.17g", v);
    return buf;
}

Simulator::Simulator() = default;

Simulator::~Simulator() {   // buffers freed in stream order, then the streams (OwnedStream)
    for (cudaEvent_t e : ev_blocks_) cudaEventDestroy(e);
    drop_timings();
}

// Stage intervals of a timed call that did not finish (an error on the way).
void Simulator::drop_timings() {
    for (PendingTiming& t : pending_timings_) {
        cudaEventDestroy(t.a);
        cudaEventDestroy(t.b);
    }
    pending_timings_.clear();
}

void Simulator::log(int level, const std::string& msg) const {
    if (log_fn_) log_fn_(level, msg.c_str(), log_user_);
}

void Simulator::ensure_device() {
    if (device_ready_) return;
    int count = 0;
    BCSIM_CUDA(cudaGetDeviceCount(&count));
    if (device_ < 0 || device_ >= count) throw SimError(BCSIM_E_INVALID, "illegal CUDA device number");
    BCSIM_CUDA(cudaSetDevice(device_));
    BCSIM_CUDA(cudaStreamCreateWithFlags(&owned_stream_.s, cudaStreamNonBlocking));
    BCSIM_CUDA(cudaStreamCreateWithFlags(&side_stream_.s, cudaStreamNonBlocking));
    BCSIM_CUDA(cudaStreamCreateWithFlags(&copy_stream_.s, cudaStreamNonBlocking));
    BCSIM_CUDA(cudaStreamCreateWithFlags(&upload_stream_.s, cudaStreamNonBlocking));
    BCSIM_CUDA(cudaStreamCreateWithFlags(&prep_stream_.s, cudaStreamNonBlocking));
    for (int k = 0; k < 2; k++) {
        BCSIM_CUDA(cudaEventCreateWithFlags(&ev_staged_[k].e, cudaEventDisableTiming));
        BCSIM_CUDA(cudaEventCreateWithFlags(&ev_uploaded_[k].e, cudaEventDisableTiming));
        BCSIM_CUDA(cudaEventCreateWithFlags(&ev_consumed_[k].e, cudaEventDisableTiming));
        BCSIM_CUDA(cudaEventCreateWithFlags(&ev_out_free_[k].e, cudaEventDisableTiming));
    }
    BCSIM_CUDA(cudaEventCreateWithFlags(&ev_fork_.e, cudaEventDisableTiming));
    BCSIM_CUDA(cudaEventCreateWithFlags(&ev_join_.e, cudaEventDisableTiming));
    BCSIM_CUDA(cudaEventCreateWithFlags(&ev_copied_.e, cudaEventDisableTiming));
    stream_ = owned_stream_.s;
    err_flag_dev_.reserve(sizeof(int));
    BCSIM_CUDA(cudaMemset(err_flag_dev_.get(), 0, sizeof(int)));
    device_ready_ = true;
    {
        // the device pool behind the stream-ordered buffers keeps freed memory
        // for reuse instead of returning it at every synchronisation
        static std::mutex pool_mu;
        static bool pool_set[64] = {};
        std::lock_guard<std::mutex> lock(pool_mu);
        if (device_ < 64 && !pool_set[device_]) {
            cudaMemPool_t pool;
            if (cudaDeviceGetDefaultMemPool(&pool, device_) == cudaSuccess) {
                uint64_t keep = UINT64_MAX;
                cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
            }
            pool_set[device_] = true;
        }
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device_) == cudaSuccess) {
        std::ostringstream ss;
        ss << "=== CUDA Device " << device_ << ": " << prop.name << " (compute capability " << prop.major << "."
           << prop.minor << ", " << prop.multiProcessorCount << " SMs)";
        log(1, ss.str());
    }
}

cudaStream_t Simulator::stream() {
    ensure_device();
    return stream_;
}

// ---------------------------------------------------------------------------
// parameters (BaseAlgorithm.cpp:48-87, GpuAlgorithm.cpp:68-107)
// ---------------------------------------------------------------------------
void Simulator::set_parameter(const std::string& key, const std::string& value) {
    bool b = false;
    cfg_version_++;
    static_version_++;
    if (key == "verbose") {
        verbose_ = std::stoi(value);
    } else if (key == "sound_speed") {
        const float v = std::stof(value);
        if (v <= 0) throw SimError(BCSIM_E_INVALID, "illegal sound speed");
        sound_speed_ = v;
    } else if (key == "noise_amplitude") {
        // BaseAlgorithm.cpp:58-60: any float; noise is added when it is > 0
        const float v = std::stof(value);
        if (!std::isfinite(v)) throw SimError(BCSIM_E_INVALID, "noise_amplitude must be finite");
        noise_amplitude_ = v;
    } else if (key == "noise_seed") {
        // the seed of the counter-based noise; setting it restarts the frame counter
        noise_seed_ = std::stoull(value);
        noise_frame_ = 0;
    } else if (key == "use_arc_projection") {
        if (!parse_bool(value, &b)) throw SimError(BCSIM_E_INVALID, "invalid boolean value");
        arc_ = b;
    } else if (key == "radial_decimation") {
        const int v = std::stoi(value);
        if (v <= 0) throw SimError(BCSIM_E_INVALID, "illegal radial decimation value");
        if (v != decimation_) tables_valid_ = false;
        decimation_ = v;
    } else if (key == "phase_delay") {
        if (!parse_bool(value, &b)) throw SimError(BCSIM_E_INVALID, "invalid boolean value");
        phase_delay_ = b;
    } else if (key == "gpu_device") {
        if (device_ready_) throw SimError(BCSIM_E_INVALID, "cannot change CUDA device now");
        int count = 0;
        BCSIM_CUDA(cudaGetDeviceCount(&count));
        const int v = std::stoi(value);
        if (v < 0 || v >= count) throw SimError(BCSIM_E_INVALID, "illegal device number");
        device_ = v;
    } else if (key == "cuda_streams") {
        const int v = std::stoi(value);
        if (v > 2) throw SimError(BCSIM_E_INVALID, "number of CUDA streams exceeds MAX_NUM_CUDA_STREAMS");
        if (v <= 0) throw SimError(BCSIM_E_INVALID, "number of CUDA streams must be more than zero");
        cuda_streams_ = v;
    } else if (key == "threads_per_block") {
        const int v = std::stoi(value);
        if (v <= 0) throw SimError(BCSIM_E_INVALID, "invalid number of threads per block");
        threads_per_block_ = v;
    } else if (key == "store_kernel_details") {
        if (!parse_bool(value, &b)) throw SimError(BCSIM_E_INVALID, "invalid value");
        store_details_ = b;
    } else if (key == "precision_mode") {
        int m;
        if (value == "fp64") m = MODE_FP64;
        else if (value == "reference") m = MODE_REFERENCE;
        else throw SimError(BCSIM_E_INVALID, "invalid value for precision_mode (fp64 | reference)");
        if (m != mode_) tables_valid_ = false;
        mode_ = m;
    } else if (key == "fir_tail_energy") {
        const double v = std::stod(value);
        if (!(v >= 0.0 && v < 1.0)) throw SimError(BCSIM_E_INVALID, "fir_tail_energy must be in [0, 1)");
        if (v != fir_tail_) tables_valid_ = false;
        fir_tail_ = v;
    } else if (key == "convolution") {
        int v;
        if (value == "auto") v = 0;
        else if (value == "fir") v = 1;
        else if (value == "fft") v = 2;
        else throw SimError(BCSIM_E_INVALID, "invalid value for convolution (auto | fir | fft)");
        if (v != convolution_) tables_valid_ = false;
        convolution_ = v;
    } else if (key == "wide_cta") {
        if (!parse_bool(value, &b)) throw SimError(BCSIM_E_INVALID, "invalid boolean value");
        wide_cta_ = b;
    } else if (key == "count_pairs") {
        if (!parse_bool(value, &b)) throw SimError(BCSIM_E_INVALID, "invalid boolean value");
        count_pairs_ = b;
    } else if (key == "lut_smem") {
        if (!parse_bool(value, &b)) throw SimError(BCSIM_E_INVALID, "invalid boolean value");
        lut_smem_ = b;
    } else if (key == "record_cache") {
        if (!parse_bool(value, &b)) throw SimError(BCSIM_E_INVALID, "invalid boolean value");
        record_cache_ = b;
    } else if (key == "autotune") {
        if (!parse_bool(value, &b)) throw SimError(BCSIM_E_INVALID, "invalid boolean value");
        autotune_ = b;
    } else if (key == "cull") {
        if (!parse_bool(value, &b)) throw SimError(BCSIM_E_INVALID, "invalid boolean value");
        cull_ = b;
    } else if (key == "render_once") {
        if (!parse_bool(value, &b)) throw SimError(BCSIM_E_INVALID, "invalid boolean value");
        render_once_ = b;
    } else if (key == "tile_lines") {
        const int v = std::stoi(value);
        if (v < 0) throw SimError(BCSIM_E_INVALID, "tile_lines must be >= 0");
        tile_lines_ = v;
    } else {
        throw SimError(BCSIM_E_INVALID, std::string("illegal parameter name: '") + key + "'");
    }
}

std::string Simulator::get_parameter(const std::string& key) const {
    if (key == "num_cuda_devices") {
        int count = 0;
        BCSIM_CUDA(cudaGetDeviceCount(&count));
        return std::to_string(count);
    }
    if (key == "cur_device_name") {
        cudaDeviceProp prop;
        BCSIM_CUDA(cudaGetDeviceProperties(&prop, device_));
        return prop.name;
    }
    if (key == "verbose") return std::to_string(verbose_);
    if (key == "sound_speed") return fmt_double(sound_speed_);
    if (key == "noise_amplitude") return fmt_double(noise_amplitude_);
    if (key == "noise_seed") return std::to_string(noise_seed_);
    // the frame number the next simulation draws its noise for
    if (key == "noise_frame") return std::to_string(noise_frame_);
    if (key == "use_arc_projection") return arc_ ? "on" : "off";
    if (key == "radial_decimation") return std::to_string(decimation_);
    if (key == "phase_delay") return phase_delay_ ? "on" : "off";
    if (key == "gpu_device") return std::to_string(device_);
    if (key == "cuda_streams") return std::to_string(cuda_streams_);
    if (key == "threads_per_block") return std::to_string(threads_per_block_);
    if (key == "store_kernel_details") return store_details_ ? "on" : "off";
    if (key == "precision_mode") return mode_ == MODE_FP64 ? "fp64" : "reference";
    if (key == "fir_tail_energy") return fmt_double(fir_tail_);
    if (key == "convolution") return convolution_ == 0 ? "auto" : convolution_ == 1 ? "fir" : "fft";
    // the route the last prepared configuration took ("" before the first simulation)
    if (key == "convolution_route") return route_known_ ? (last_route_fft_ ? "fft" : "fir") : "";
    if (key == "tile_lines") return std::to_string(tile_lines_);
    if (key == "cull") return cull_ ? "on" : "off";
    if (key == "render_once") return render_once_ ? "on" : "off";
    if (key == "record_cache") return record_cache_ ? "on" : "off";
    if (key == "wide_cta") return wide_cta_ ? "on" : "off";
    if (key == "lut_smem") return lut_smem_ ? "on" : "off";
    if (key == "count_pairs") return count_pairs_ ? "on" : "off";
    if (key == "autotune") return autotune_ ? "on" : "off";
    if (key == "fir_taps") return std::to_string(tap_count_);
    throw SimError(BCSIM_E_INVALID, "Illegal key: " + key);
}

// ---------------------------------------------------------------------------
// configuration
// ---------------------------------------------------------------------------
void Simulator::set_excitation(const float* samples, int n, int center_index, float fs, float demod_freq) {
    cfg_version_++;
    static_version_++;
    if (n < 0 || (n > 0 && !samples)) throw SimError(BCSIM_E_INVALID, "set_excitation: invalid samples");
    taps_.assign(samples, samples + n);
    center_ = center_index;
    fs_ = fs;
    fd_ = demod_freq;
    excitation_set_ = true;
    tables_valid_ = false;
    log(1, "Number of excitation samples: " + std::to_string(n));
}

void Simulator::set_scan_sequence(const float* origins, const float* dirs, const float* lats, const float* timestamps,
                                  int num_lines, float line_length) {
    if (num_lines < 0 || (num_lines > 0 && (!origins || !dirs || !lats || !timestamps)))
        throw SimError(BCSIM_E_INVALID, "set_scan_sequence(): Invalid rank.");
    // Scanline construction and validation (ScanSequence.cpp:37-70)
    std::vector<LineGeom> lines(static_cast<size_t>(num_lines));
    for (int i = 0; i < num_lines; i++) {
        LineGeom& g = lines[i];
        for (int k = 0; k < 3; k++) {
            g.o[k] = origins[3 * i + k];
            g.d[k] = dirs[3 * i + k];
            g.l[k] = lats[3 * i + k];
        }
        // elevational = lateral x direction (vector3.hpp:97-103)
        g.e[0] = g.l[1] * g.d[2] - g.d[1] * g.l[2];
        g.e[1] = g.d[0] * g.l[2] - g.l[0] * g.d[2];
        g.e[2] = g.l[0] * g.d[1] - g.d[0] * g.l[1];
        const float thr = 1e-4f;
        if (std::abs(fdot(g.d, g.l)) >= thr || std::abs(fdot(g.l, g.e)) >= thr || std::abs(fdot(g.e, g.d)) >= thr)
            throw SimError(BCSIM_E_INVALID, "Invalid Scanline: Not orthogonal unit vectors");
        const float nd = std::sqrt(fdot(g.d, g.d)), nl = std::sqrt(fdot(g.l, g.l)), ne = std::sqrt(fdot(g.e, g.e));
        if (std::abs(nd - 1.0) >= thr || std::abs(nl - 1.0) >= thr || std::abs(ne - 1.0) >= thr)
            throw SimError(BCSIM_E_INVALID, "Invalid Scanline: Not unit length vectors");
    }
    // CpuAlgorithm.cpp:258-260
    if (!excitation_set_) throw SimError(BCSIM_E_INVALID, "Excitation must be configured before scan sequence");
    lines_ = std::move(lines);
    timestamps_.assign(timestamps, timestamps + num_lines);
    num_lines_ = num_lines;
    line_length_ = line_length;
    ns_ = num_rf_samples(sound_speed_, line_length, fs_);
    shared_origin_ = true;
    timestamps_equal_ = true;
    for (int i = 1; i < num_lines; i++) {
        if (std::memcmp(lines_[i].o, lines_[0].o, sizeof(lines_[0].o)) != 0) shared_origin_ = false;
        if (std::memcmp(&timestamps_[i], &timestamps_[0], sizeof(float)) != 0) timestamps_equal_ = false;
    }
    scan_set_ = true;
    lines_valid_ = false;
    tables_valid_ = false;
    cfg_version_++;
    static_version_++;
}

void Simulator::copy_scan_from(const Simulator& o) {
    if (!o.scan_set_) return;
    lines_ = o.lines_;
    timestamps_ = o.timestamps_;
    num_lines_ = o.num_lines_;
    line_length_ = o.line_length_;
    ns_ = num_rf_samples(sound_speed_, line_length_, fs_);
    shared_origin_ = o.shared_origin_;
    timestamps_equal_ = o.timestamps_equal_;
    scan_set_ = true;
    lines_valid_ = false;
    tables_valid_ = false;
    cfg_version_++;
    static_version_++;
}

void Simulator::set_analytical_profile(float sigma_lateral, float sigma_elevational) {
    cfg_version_++;
    static_version_++;
    log(1, "Setting analytical beam profile for GPU algorithm");
    beam_type_ = BEAM_GAUSSIAN;
    sigma_l_ = sigma_lateral;
    sigma_e_ = sigma_elevational;
}

void Simulator::set_lookup_profile(const float* samples, int nr, int nl, int ne, float r0, float r1, float l0,
                                   float l1, float e0, float e1) {
    log(1, "Setting LUT profile for GPU algorithm");
    // LUTBeamProfile constructor checks (BeamProfile.cpp:64-66)
    if (nr <= 1) throw SimError(BCSIM_E_INVALID, "Too few radial samples");
    if (nl <= 1) throw SimError(BCSIM_E_INVALID, "Too few lateral samples");
    if (ne <= 1) throw SimError(BCSIM_E_INVALID, "Too few elevational samples");
    if (!samples) throw SimError(BCSIM_E_INVALID, "set_lookup_profile: samples is null");
    const size_t total = (size_t)nr * nl * ne;
    lut_.assign(samples, samples + total);
    lut_nr_ = nr; lut_nl_ = nl; lut_ne_ = ne;
    lut_ext_[0] = r0; lut_ext_[1] = r1; lut_ext_[2] = l0; lut_ext_[3] = l1; lut_ext_[4] = e0; lut_ext_[5] = e1;
    lut_absmax_ = 0.0;
    for (float v : lut_) lut_absmax_ = std::max(lut_absmax_, (double)std::fabs(v));
    beam_type_ = BEAM_LUT;
    lut_uploaded_ = false;
    cfg_version_++;
    static_version_++;
}

void Simulator::clear_fixed_scatterers() {
    fixed_src_ = nullptr;
    cfg_version_++;
    data_version_++;
    fixed_n_ = 0;
    num_fixed_sets_ = 0;
    fixed_sum_abs_ = 0.0;
    amplitude_nonfinite_ = false;
    for (const auto& s : splines_) (void)s;
}

void Simulator::add_fixed_scatterers(const float* xyza, int64_t n) {
    if (n < 0 || (n > 0 && !xyza)) throw SimError(BCSIM_E_INVALID, "add_fixed_scatterers: invalid data");
    ensure_device();
    if (n > 0) {
        const size_t need = (size_t)(fixed_n_ + n) * sizeof(float4);
        if (need > fixed_xyza_.bytes()) {
            DeviceBuffer grown;
            grown.reserve(std::max(need, fixed_xyza_.bytes() * 3 / 2), stream_);
            if (fixed_n_ > 0)
                BCSIM_CUDA(cudaMemcpyAsync(grown.get(), fixed_xyza_.get(), (size_t)fixed_n_ * sizeof(float4),
                                           cudaMemcpyDeviceToDevice, stream_));
            BCSIM_CUDA(cudaStreamSynchronize(stream_));
            fixed_xyza_ = std::move(grown);
        }
        BCSIM_CUDA(cudaMemcpyAsync(fixed_xyza_.as<float4>() + fixed_n_, xyza, (size_t)n * sizeof(float4),
                                   cudaMemcpyHostToDevice, stream_));
        // amplitude bound and finiteness on the device (the amplitude is the
        // 4th float of every scatterer)
        double s = 0.0;
        int bad = 0;
        ingest_scratch_.reserve(abs_sum_scratch_bytes(), stream_);
        BCSIM_CUDA(abs_sum(reinterpret_cast<const float*>(fixed_xyza_.as<float4>() + fixed_n_) + 3, 4, n,
                           ingest_scratch_.get(), &s, &bad, stream_));
        if (bad) amplitude_nonfinite_ = true;
        fixed_sum_abs_ += s;
    }
    fixed_n_ += n;
    num_fixed_sets_ += 1;
    cfg_version_++;
    data_version_++;
    if (verbose_) log(1, "Number of fixed scatterers: " + std::to_string(fixed_n_));
}

void Simulator::clear_spline_scatterers() {
    splines_.clear();
    cfg_version_++;
    data_version_++;
}

void Simulator::add_spline_scatterers(int degree, const float* knots, int num_knots, const float* cps,
                                      const float* amps, int64_t n, int num_cs) {
    if (n < 0 || num_cs < 0 || num_knots < 0 || (n > 0 && (!cps || !amps)) || (num_knots > 0 && !knots))
        throw SimError(BCSIM_E_INVALID, "add_spline_scatterers: invalid data");
    // src/python/PythonInterface.cpp:150-153
    if (num_knots != num_cs + degree + 1)
        throw SimError(BCSIM_E_INVALID, "add_spline_scatterers : mismatch in number of nodes, degree and control points");
    if (degree < 0 || degree > MAX_SPLINE_DEGREE)
        throw SimError(BCSIM_E_INVALID, "add_spline_scatterers : spline degree must be in [0, " +
                                            std::to_string(MAX_SPLINE_DEGREE) + "]");
    ensure_device();
    SplineDataset ds;
    ds.degree = degree;
    ds.num_cs = num_cs;
    ds.knots.assign(knots, knots + num_knots);
    ds.n = n;
    if (n > 0 && num_cs > 0) {
        // the caller's [n][K][3] as it is, laid out [K][n] float4 on the device
        DeviceBuffer raw;
        raw.reserve((size_t)n * num_cs * 3 * sizeof(float), stream_);
        BCSIM_CUDA(cudaMemcpyAsync(raw.get(), cps, (size_t)n * num_cs * 3 * sizeof(float), cudaMemcpyHostToDevice,
                                   stream_));
        ds.cps.reserve((size_t)num_cs * n * sizeof(float4), stream_);
        BCSIM_CUDA(launch_spline_transpose(raw.as<float>(), n, num_cs, ds.cps.as<float4>(), stream_));
    }
    if (n > 0) {
        ds.amps.reserve((size_t)n * sizeof(float), stream_);
        BCSIM_CUDA(cudaMemcpyAsync(ds.amps.get(), amps, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, stream_));
        int bad = 0;
        ingest_scratch_.reserve(abs_sum_scratch_bytes(), stream_);
        BCSIM_CUDA(abs_sum(ds.amps.as<float>(), 1, n, ingest_scratch_.get(), &ds.sum_abs_amp, &bad, stream_));
        if (bad) amplitude_nonfinite_ = true;
    }
    BCSIM_CUDA(cudaStreamSynchronize(stream_));
    splines_.push_back(std::move(ds));
    cfg_version_++;
    data_version_++;
    if (verbose_) log(1, "Number of spline datasets: " + std::to_string(splines_.size()));
}

int64_t Simulator::total_num_scatterers() const {
    int64_t t = fixed_n_;
    for (const auto& s : splines_) t += s.n;
    return t;
}

void Simulator::output_shape(int64_t* lines, int64_t* samples) const {
    if (!scan_set_) throw SimError(BCSIM_E_NOT_CONFIGURED, "Scan sequence not configured.");
    if (lines) *lines = num_lines_;
    if (samples) *samples = (ns_ + decimation_ - 1) / decimation_;
}

// CpuAlgorithm.cpp:385-398 and GpuAlgorithm.cpp:157-163
void Simulator::throw_if_not_configured() const {
    if (!scan_set_) throw SimError(BCSIM_E_NOT_CONFIGURED, "Scan sequence not configured.");
    if (!excitation_set_) throw SimError(BCSIM_E_NOT_CONFIGURED, "Excitation not configured.");
    if (beam_type_ == 0) throw SimError(BCSIM_E_NOT_CONFIGURED, "Beam profile not configured.");
    if (total_num_scatterers() == 0) throw SimError(BCSIM_E_NOT_CONFIGURED, "no scatterers are configured");
    if (num_lines_ < 1) throw SimError(BCSIM_E_NOT_CONFIGURED, "No scanlines in scansequence");
}

std::vector<double> Simulator::get_debug_data(const std::string& key) const {
    if (key == "kernel_launches") return {(double)last_launches_};
    auto it = debug_.find(key);
    if (it == debug_.end()) throw SimError(BCSIM_E_INVALID, "invalid debug data key: " + key);
    return it->second;
}

// ---------------------------------------------------------------------------
// derived tables
// ---------------------------------------------------------------------------

// Automatic convolution route, from the time each takes on GB300 for L lines:
// the direct FIR ~0.23 ps per line, output and tap plus ~8 us, filling the GPU
// at any line count (a line's outputs split over more CTAs when lines are
// few); the FFT route one CTA per line, a wave of 2 CTAs per SM (M <= 8192,
// ~30 us at M = 8192, scaling with M log2 M) or 1 (M = 16384, ~25 us).  Few
// lines or short windows favour the FIR.
static bool fft_faster(int64_t L, int64_t nd, int64_t window, int64_t M, int sms) {
    int lg = 0;
    while ((int64_t(1) << lg) < M) lg++;
    const double t_fir = (double)L * (double)nd * (double)window * 0.23e-12 + 8e-6;
    const int64_t slots = (M <= 8192 ? 2 : 1) * (int64_t)std::max(sms, 1);
    const double t_wave = M <= 8192 ? 30e-6 * (double)M * lg / (8192.0 * 13.0) : 25e-6;
    const double t_fft = (double)((L + slots - 1) / slots) * t_wave;
    return t_fft < t_fir;
}

void Simulator::prepare_excitation_tables() {
    if (tables_valid_) return;
    const int64_t ntaps = (int64_t)taps_.size();
    M_ = next_power_of_two(ns_ + ntaps - 1);
    nd_ = (ns_ + decimation_ - 1) / decimation_;
    if (center_ < 0 || (int64_t)center_ + (nd_ - 1) * decimation_ >= M_)
        throw SimError(BCSIM_E_INVALID, "excitation center index outside the convolution buffer");
    // the FIR window depends on the excitation, M and the tail energy only:
    // recompute it (an M-point FFT in double) only when one of them changed
    if (!(fir_key_taps_ == taps_ && fir_key_M_ == M_ && fir_key_tail_ == fir_tail_)) {
        analytic_spec_ = analytic_spectrum(taps_, M_);
        std::vector<std::complex<double>> ha = analytic_spec_;
        fft_double(ha, +1);
        for (auto& v : ha) v /= (double)M_;
        choose_tap_window(ha, (int)ntaps, fir_tail_, &tap_start_, &tap_count_);
        std::vector<float2> taps((size_t)tap_count_);
        for (int64_t w = 0; w < tap_count_; w++) {
            const int64_t n = ((tap_start_ + w) % M_ + M_) % M_;
            taps[w] = make_float2((float)ha[n].real(), (float)ha[n].imag());
        }
        fir_taps_host_ = taps;
        fir_key_taps_ = taps_;
        fir_key_M_ = M_;
        fir_key_tail_ = fir_tail_;
        log(0, "FIR window: start " + std::to_string(tap_start_) + ", taps " + std::to_string(tap_count_) + ", M " +
                   std::to_string(M_));
    }
    const auto dm = demod_factors(fd_, fs_, decimation_, nd_, mode_ == MODE_REFERENCE);
    demod_dev_.reserve(dm.size() * sizeof(float2), stream_);
    BCSIM_CUDA(cudaMemcpyAsync(demod_dev_.get(), dm.data(), dm.size() * sizeof(float2), cudaMemcpyHostToDevice, stream_));
    // the window's taps in the kernel's phase-major order for this decimation
    std::vector<float2> pm((size_t)tap_count_ + 4 * decimation_);
    std::vector<int> off((size_t)3 * decimation_ + 1);
    ntaps_pm_ = make_phase_major_taps(fir_taps_host_.data(), (int)tap_count_, decimation_, pm.data(), off.data(),
                                      &max_ph_taps_);
    taps_pm_dev_.reserve(std::max<size_t>(1, (size_t)ntaps_pm_) * sizeof(float2), stream_);
    ph_off_dev_.reserve(off.size() * sizeof(int), stream_);
    BCSIM_CUDA(cudaMemcpyAsync(taps_pm_dev_.get(), pm.data(), (size_t)ntaps_pm_ * sizeof(float2), cudaMemcpyHostToDevice, stream_));
    BCSIM_CUDA(cudaMemcpyAsync(ph_off_dev_.get(), off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice, stream_));
    // the FFT route, where a line fits one CTA's shared memory; its tables
    // depend on the excitation, M and the center only (not on the decimation)
    int smem_optin = 0;
    BCSIM_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device_));
    BCSIM_CUDA(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, device_));
    fft_ok_ = fft_convolution_supported(M_) && ns_ <= M_ && fft_convolution_smem(M_) <= (size_t)smem_optin;
    if (convolution_ == 2 && !fft_ok_)
        throw SimError(BCSIM_E_INVALID, "convolution=fft needs a power-of-two convolution length M in [256, 16384] "
                                        "(this configuration has M = " + std::to_string(M_) + ")");
    std::vector<float2> hold_spec, hold_tw;
    if (convolution_ != 1 && fft_ok_ && !(fft_key_taps_ == taps_ && fft_key_M_ == M_ && fft_key_center_ == center_)) {
        hold_spec.resize((size_t)M_);
        hold_tw.resize((size_t)M_);
        make_fft_tables(analytic_spec_.data(), M_, center_, hold_spec.data(), hold_tw.data());
        fft_spec_dev_.reserve((size_t)M_ * sizeof(float2), stream_);
        fft_tw_dev_.reserve((size_t)M_ * sizeof(float2), stream_);
        BCSIM_CUDA(cudaMemcpyAsync(fft_spec_dev_.get(), hold_spec.data(), (size_t)M_ * sizeof(float2),
                                   cudaMemcpyHostToDevice, stream_));
        BCSIM_CUDA(cudaMemcpyAsync(fft_tw_dev_.get(), hold_tw.data(), (size_t)M_ * sizeof(float2),
                                   cudaMemcpyHostToDevice, stream_));
        fft_key_taps_ = taps_;
        fft_key_M_ = M_;
        fft_key_center_ = center_;
    }
    BCSIM_CUDA(cudaStreamSynchronize(stream_));
    tables_valid_ = true;
}

// Kernel line order for the shared-origin kernel: recursive bisection of the
// lines by direction into slots of 32 -- each set is sorted along the major
// principal axis of its directions (projected on the plane normal to their mean)
// and cut at the multiple of 32 nearest its middle -- so that the 32 lines of a
// slot point in a compact patch of directions (a 4 x 8 block of a regular
// azimuth/elevation grid); then the frame spread of each slot about its line
// nearest the slot's mean direction.
namespace {
struct Dir3 {
    double x, y, z;
};
Dir3 unit_mean(const std::vector<LineGeom>& lines, const int* idx, int n) {
    double m[3] = {0, 0, 0};
    for (int i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) m[k] += lines[idx[i]].d[k];
    double mn = std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
    if (mn < 1e-12) return Dir3{0, 0, 1};
    return Dir3{m[0] / mn, m[1] / mn, m[2] / mn};
}
void bisect_lines(const std::vector<LineGeom>& lines, int* idx, int n) {
    if (n <= 32) return;
    const Dir3 m = unit_mean(lines, idx, n);
    // tangent basis (t1, t2) normal to m
    double a[3] = {1, 0, 0};
    if (std::fabs(m.x) > 0.9) { a[0] = 0; a[1] = 1; }
    double t1[3] = {a[1] * m.z - a[2] * m.y, a[2] * m.x - a[0] * m.z, a[0] * m.y - a[1] * m.x};
    const double n1 = std::sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
    for (double& v : t1) v /= n1;
    const double t2[3] = {m.y * t1[2] - m.z * t1[1], m.z * t1[0] - m.x * t1[2], m.x * t1[1] - m.y * t1[0]};
    std::vector<double> pu(n), pv(n);
    double su = 0, sv = 0;
    for (int i = 0; i < n; i++) {
        const float* d = lines[idx[i]].d;
        pu[i] = d[0] * t1[0] + d[1] * t1[1] + d[2] * t1[2];
        pv[i] = d[0] * t2[0] + d[1] * t2[1] + d[2] * t2[2];
        su += pu[i];
        sv += pv[i];
    }
    su /= n;
    sv /= n;
    double cuu = 0, cuv = 0, cvv = 0;
    for (int i = 0; i < n; i++) {
        const double du = pu[i] - su, dv = pv[i] - sv;
        cuu += du * du; cuv += du * dv; cvv += dv * dv;
    }
    // major axis of the 2 x 2 covariance
    const double ang = 0.5 * std::atan2(2.0 * cuv, cuu - cvv);
    const double ax = std::cos(ang), ay = std::sin(ang);
    std::vector<std::pair<double, int>> key(n);
    for (int i = 0; i < n; i++) key[i] = {(pu[i] - su) * ax + (pv[i] - sv) * ay, idx[i]};
    std::stable_sort(key.begin(), key.end(),
                     [](const std::pair<double, int>& x, const std::pair<double, int>& y) { return x.first < y.first; });
    for (int i = 0; i < n; i++) idx[i] = key[i].second;
    int half = (int)std::lround(n / 64.0) * 32;
    half = std::max(32, std::min(half, n - 32 > 32 ? n - 32 : 32));
    bisect_lines(lines, idx, half);
    bisect_lines(lines, idx + half, n - half);
}
}  // namespace

// Culling extent of a per-pair tile (lines ids[0 .. count)): its line nearest
// the tiles' mean direction as reference, the frame spread about it (split along
// and across its direction, as for the shared-origin slots) and the largest
// origin offset, with margins for the float arithmetic of the test.
static TileBox make_tile_box(const std::vector<LineGeom>& lines, const int* ids, int count) {
    double m[3] = {0, 0, 0};
    for (int i = 0; i < count; i++)
        for (int k = 0; k < 3; k++) m[k] += lines[ids[i]].d[k];
    const double mn = std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
    int best = ids[0];
    double best_dot = -2.0;
    for (int i = 0; i < count; i++) {
        const float* d = lines[ids[i]].d;
        const double dot = mn > 0 ? (d[0] * m[0] + d[1] * m[1] + d[2] * m[2]) / mn : 0.0;
        if (dot > best_dot) { best_dot = dot; best = ids[i]; }
    }
    const LineGeom& ref = lines[best];
    double upar = 0, uperp = 0, vpar = 0, vperp = 0, dorig = 0;
    for (int i = 0; i < count; i++) {
        const LineGeom& g = lines[ids[i]];
        double dl[3], de[3], pl = 0, pe = 0, oo = 0;
        for (int k = 0; k < 3; k++) {
            dl[k] = (double)g.l[k] - ref.l[k];
            de[k] = (double)g.e[k] - ref.e[k];
            pl += dl[k] * ref.d[k];
            pe += de[k] * ref.d[k];
            oo += ((double)g.o[k] - ref.o[k]) * ((double)g.o[k] - ref.o[k]);
        }
        double ql = 0, qe = 0;
        for (int k = 0; k < 3; k++) {
            const double xl = dl[k] - pl * ref.d[k], xe = de[k] - pe * ref.d[k];
            ql += xl * xl;
            qe += xe * xe;
        }
        upar = std::max(upar, std::fabs(pl));
        uperp = std::max(uperp, std::sqrt(ql));
        vpar = std::max(vpar, std::fabs(pe));
        vperp = std::max(vperp, std::sqrt(qe));
        dorig = std::max(dorig, std::sqrt(oo));
    }
    TileBox t;
    t.ox = ref.o[0]; t.oy = ref.o[1]; t.oz = ref.o[2];
    t.lx = ref.l[0]; t.ly = ref.l[1]; t.lz = ref.l[2];
    t.ex = ref.e[0]; t.ey = ref.e[1]; t.ez = ref.e[2];
    t.rx = ref.d[0]; t.ry = ref.d[1]; t.rz = ref.d[2];
    t.du_par = (float)(upar * 1.0001 + 2e-6);
    t.du_perp = (float)(uperp * 1.0001 + 2e-6);
    t.dv_par = (float)(vpar * 1.0001 + 2e-6);
    t.dv_perp = (float)(vperp * 1.0001 + 2e-6);
    t.d_orig = (float)(dorig * 1.0001 + 1e-7);
    return t;
}

static void order_lines(const std::vector<LineGeom>& lines, std::vector<int>& order, std::vector<SlotCone>& cones) {
    const int L = (int)lines.size();
    order.resize(L);
    std::iota(order.begin(), order.end(), 0);
    bisect_lines(lines, order.data(), L);
    const int slots = (L + 31) / 32;
    cones.assign(slots, SlotCone{0, 0, 0, 0, 0, 0, 0, 0, 0, 2, 2, 2, 2, 2});
    for (int s = 0; s < slots; s++) {
        const int lo = s * 32, hi = std::min(L, lo + 32);
        const Dir3 m = unit_mean(lines, order.data() + lo, hi - lo);
        int best = order[lo];
        double best_dot = -2.0;
        for (int i = lo; i < hi; i++) {
            const float* d = lines[order[i]].d;
            const double dot = d[0] * m.x + d[1] * m.y + d[2] * m.z;
            if (dot > best_dot) { best_dot = dot; best = order[i]; }
        }
        const LineGeom& ref = lines[best];
        double upar = 0, uperp = 0, vpar = 0, vperp = 0, dd = 0;
        for (int i = lo; i < hi; i++) {
            const LineGeom& g = lines[order[i]];
            double dl[3], de[3], pl = 0, pe = 0, c = 0;
            for (int k = 0; k < 3; k++) {
                dl[k] = (double)g.l[k] - ref.l[k];
                de[k] = (double)g.e[k] - ref.e[k];
                pl += dl[k] * ref.d[k];
                pe += de[k] * ref.d[k];
                c += ((double)g.d[k] - ref.d[k]) * ((double)g.d[k] - ref.d[k]);
            }
            double ql = 0, qe = 0;
            for (int k = 0; k < 3; k++) {
                const double xl = dl[k] - pl * ref.d[k], xe = de[k] - pe * ref.d[k];
                ql += xl * xl;
                qe += xe * xe;
            }
            upar = std::max(upar, std::fabs(pl));
            uperp = std::max(uperp, std::sqrt(ql));
            vpar = std::max(vpar, std::fabs(pe));
            vperp = std::max(vperp, std::sqrt(qe));
            dd = std::max(dd, std::sqrt(c));
        }
        SlotCone cone;
        cone.lx = ref.l[0]; cone.ly = ref.l[1]; cone.lz = ref.l[2];
        cone.ex = ref.e[0]; cone.ey = ref.e[1]; cone.ez = ref.e[2];
        cone.rx = ref.d[0]; cone.ry = ref.d[1]; cone.rz = ref.d[2];
        // margins for the float rounding of the test's products (the frames are
        // unit vectors to float precision, so their own rounding is covered too)
        cone.du_par = (float)(upar * 1.0001 + 2e-6);
        cone.du_perp = (float)(uperp * 1.0001 + 2e-6);
        cone.dv_par = (float)(vpar * 1.0001 + 2e-6);
        cone.dv_perp = (float)(vperp * 1.0001 + 2e-6);
        cone.dd = (float)(dd * 1.0001 + 2e-6);
        cones[s] = cone;
    }
}

void Simulator::prepare_lines() {
    if (lines_valid_) return;
    lines_dev_.reserve(std::max<size_t>(1, lines_.size()) * sizeof(LineGeom), stream_);
    if (!lines_.empty())
        BCSIM_CUDA(cudaMemcpyAsync(lines_dev_.get(), lines_.data(), lines_.size() * sizeof(LineGeom),
                                   cudaMemcpyHostToDevice, stream_));
    std::vector<int> order;
    std::vector<SlotCone> cones;
    order_lines(lines_, order, cones);
    line_rank_.assign(order.size(), 0);
    for (size_t i = 0; i < order.size(); i++) line_rank_[order[i]] = (int)i;
    line_order_dev_.reserve(std::max<size_t>(1, order.size()) * sizeof(int), stream_);
    cones_dev_.reserve(std::max<size_t>(1, cones.size()) * sizeof(SlotCone), stream_);
    if (!order.empty()) {
        BCSIM_CUDA(cudaMemcpyAsync(line_order_dev_.get(), order.data(), order.size() * sizeof(int),
                                   cudaMemcpyHostToDevice, stream_));
        BCSIM_CUDA(cudaMemcpyAsync(cones_dev_.get(), cones.data(), cones.size() * sizeof(SlotCone),
                                   cudaMemcpyHostToDevice, stream_));
    }
    BCSIM_CUDA(cudaStreamSynchronize(stream_));
    lines_valid_ = true;
}

double Simulator::fixed_point_bound() const {
    double s = fixed_sum_abs_;
    for (const auto& d : splines_) s += d.sum_abs_amp;
    const double wmax = beam_type_ == BEAM_LUT ? lut_absmax_ : 1.0;
    return s * wmax;
}

// Packed LUT: at (r, l, e) the corners (c[r][l][e], c[r][l][e+1], c[r+1][l][e],
// c[r+1][l][e+1]), zero past the last sample.
// Packed table: at (r, l, e) the corners needed by one trilinear lookup with
// radial index r, (c[r][l][e], c[r][l][e+1], c[r+1][l][e], c[r+1][l][e+1]).
// With radial_diff the last two hold the radial differences
// c[r+1][.][.] - c[r][.][.] instead (the float subtraction the fp64-mode
// kernels would otherwise do per lookup: same value, one instruction less per
// radial interpolation); the reference-arithmetic kernels take the corners.
static std::vector<float4> pack_lut(const std::vector<float>& c, int nr, int nl, int ne, bool radial_diff) {
    std::vector<float4> p((size_t)nr * nl * ne);
    auto at = [&](int r, int l, int e) -> float {
        if (r >= nr || l >= nl || e >= ne) return 0.0f;
        return c[((size_t)r * nl + l) * ne + e];
    };
    for (int r = 0; r < nr; r++)
        for (int l = 0; l < nl; l++)
            for (int e = 0; e < ne; e++) {
                const float c0 = at(r, l, e), c1 = at(r, l, e + 1), c2 = at(r + 1, l, e), c3 = at(r + 1, l, e + 1);
                p[((size_t)r * nl + l) * ne + e] = radial_diff ? make_float4(c0, c1, c2 - c0, c3 - c1) : make_float4(c0, c1, c2, c3);
            }
    return p;
}

// ---------------------------------------------------------------------------
// simulate
// ---------------------------------------------------------------------------
namespace {
// Stage timer of store_kernel_details: stop() records the interval's end and
// hands both events to the simulator's pending list without waiting, so that
// timing a simulation does not hold the host between its stages (a wait there
// would leave the GPU idle until the next stage is launched); the intervals are
// read once the simulation has finished (Simulator::resolve_timings).
struct EventTimer {
    bool on;
    cudaStream_t s;
    std::vector<PendingTiming>* out;
    cudaEvent_t a = nullptr;
    EventTimer(bool enabled, cudaStream_t st, std::vector<PendingTiming>* pending)
        : on(enabled), s(st), out(pending) {
        if (on) {
            cudaEventCreate(&a);
            cudaEventRecord(a, s);
        }
    }
    ~EventTimer() {
        if (a) cudaEventDestroy(a);
    }
    void restart() { if (on) cudaEventRecord(a, s); }
    void stop(const char* key) {
        if (!on) return;
        cudaEvent_t b = nullptr;
        cudaEventCreate(&b);
        cudaEventRecord(b, s);
        out->push_back({key, a, b});
        // a fresh start event: the handed-over one keeps its timestamp
        cudaEventCreate(&a);
        cudaEventRecord(a, s);
    }
};
}  // namespace

// The pending stage intervals, in the order they were stopped, into debug_.
void Simulator::resolve_timings() {
    for (PendingTiming& t : pending_timings_) {
        float ms = 0.0f;
        if (cudaEventSynchronize(t.b) == cudaSuccess && cudaEventElapsedTime(&ms, t.a, t.b) == cudaSuccess)
            debug_[t.key].push_back(ms);
        cudaEventDestroy(t.a);
        cudaEventDestroy(t.b);
    }
    pending_timings_.clear();
}

// ---------------------------------------------------------------------------
// prepare: everything the host computes or uploads for one configuration
// ---------------------------------------------------------------------------
// Fixed-point scale 2^S of the bins: S = floor(61 - log2(sum |a| * max weight)),
// so that no sum of contributions can overflow int64.
void Simulator::set_fixed_point_scale(SimParams& p) const {
    const double bound = fixed_point_bound();
    int S = 0;
    if (bound > 0.0 && std::isfinite(bound)) S = (int)std::floor(61.0 - std::log2(bound * 1.001));
    S = std::max(-100, std::min(100, S));
    p.log2scale = S;
    p.scale = std::ldexp(1.0f, S);
}

// What the sorted shared-origin records depend on: the scatterers (by version),
// the origin, the common time and the kernel constants.
uint64_t Simulator::records_key_of(const Plan& P) const {
    uint64_t key = data_version_ * 1000003ull;
    auto mix = [&](const void* ptr, size_t n) {
        const unsigned char* c = static_cast<const unsigned char*>(ptr);
        for (size_t i = 0; i < n; i++) key = (key ^ c[i]) * 1099511628211ull;
    };
    mix(lines_[0].o, sizeof(lines_[0].o));
    mix(&timestamps_[0], sizeof(float));
    mix(&P.p, sizeof(P.p));
    mix(&P.b, sizeof(P.b));
    return key;
}

// The shapes a plan depends on: dataset sizes and spline knots (not the values).
std::vector<double> Simulator::data_shape() const {
    std::vector<double> v{(double)fixed_n_};
    for (const auto& d : splines_) {
        v.push_back((double)d.n);
        v.push_back((double)d.num_cs);
        v.push_back((double)d.degree);
        for (float k : d.knots) v.push_back((double)k);
    }
    return v;
}

void Simulator::prepare() {
    throw_if_not_configured();
    if (amplitude_nonfinite_) throw SimError(BCSIM_E_INVALID, "Nan in scatterer projection.");
    ensure_device();
    if (plan_.version == cfg_version_) return;
    if (plan_.version != ~0ull && plan_.static_version == static_version_ && plan_.data_shape == data_shape()) {
        // only scatterer values changed (a new frame of the same phantom shape):
        // the plan stands but for the fixed-point scale and the records' identity
        set_fixed_point_scale(plan_.p);
        if (plan_.n_shared > 0) plan_.records_key = records_key_of(plan_);
        plan_.version = cfg_version_;
        return;
    }
    const cudaStream_t st = stream_;
    const int L = num_lines_;
    if (ns_ <= 0) throw SimError(BCSIM_E_INVALID, "line length gives no RF samples");
    if (ns_ >= (int64_t)1 << 30) throw SimError(BCSIM_E_INVALID, "too many RF samples per line");
    const int ns = (int)ns_;
    prepare_excitation_tables();
    prepare_lines();
    Plan& P = plan_;
    P = Plan();

    // beam
    BeamDev& b = P.b;
    std::memset(&b, 0, sizeof(b));
    b.type = beam_type_;
    if (beam_type_ == BEAM_GAUSSIAN) {
        const double log2e = 1.4426950408889634;
        b.gl = (float)(log2e / (2.0 * (double)sigma_l_ * (double)sigma_l_));
        b.ge = (float)(log2e / (2.0 * (double)sigma_e_ * (double)sigma_e_));
        b.two_sl2 = 2 * sigma_l_ * sigma_l_;
        b.two_se2 = 2 * sigma_e_ * sigma_e_;
    } else {
        if (!lut_uploaded_ || lut_packed_mode_ != mode_) {
            const auto packed = pack_lut(lut_, lut_nr_, lut_nl_, lut_ne_, mode_ == MODE_FP64);
            lut4_.reserve(packed.size() * sizeof(float4), stream_);
            BCSIM_CUDA(cudaMemcpyAsync(lut4_.get(), packed.data(), packed.size() * sizeof(float4), cudaMemcpyHostToDevice, st));
            BCSIM_CUDA(cudaStreamSynchronize(st));
            lut_uploaded_ = true;
            lut_packed_mode_ = mode_;
        }
        b.lut4 = lut4_.as<float4>();
        b.nr = lut_nr_; b.nl = lut_nl_; b.ne = lut_ne_;
        b.rf = lut_ext_[0]; b.lf = lut_ext_[2]; b.ef = lut_ext_[4];
        if (mode_ == MODE_FP64) {
            b.dr = ((double)lut_ext_[1] - (double)lut_ext_[0]) / (lut_nr_ - 1);
            b.dl = ((double)lut_ext_[3] - (double)lut_ext_[2]) / (lut_nl_ - 1);
            b.de = ((double)lut_ext_[5] - (double)lut_ext_[4]) / (lut_ne_ - 1);
        } else {
            // BeamProfile.cpp:72-74: float difference divided by an int
            b.dr = (double)((lut_ext_[1] - lut_ext_[0]) / (lut_nr_ - 1));
            b.dl = (double)((lut_ext_[3] - lut_ext_[2]) / (lut_nl_ - 1));
            b.de = (double)((lut_ext_[5] - lut_ext_[4]) / (lut_ne_ - 1));
        }
        b.inv_dr = (float)(1.0 / b.dr);
        b.inv_dr_lo = (float)(1.0 / b.dr - (double)b.inv_dr);
        b.inv_dl = (float)(1.0 / b.dl);
        b.inv_de = (float)(1.0 / b.de);
    }

    // simulation constants
    SimParams& p = P.p;
    std::memset(&p, 0, sizeof(p));
    p.ns = ns;
    p.num_lines = L;
    p.phase_delay = phase_delay_ ? 1 : 0;
    p.arc = arc_ ? 1 : 0;
    p.mode = mode_;
    p.fs = fs_; p.c = sound_speed_; p.fd = fd_;
    p.fs_d = fs_; p.c_d = sound_speed_; p.fd_d = fd_;
    const double k = 2.0 * (double)fs_ / (double)sound_speed_;
    p.k_hi = (float)k;
    p.k_lo = (float)(k - (double)p.k_hi);
    p.two_pi_fd_over_fs = (float)(6.283185307179586 * (double)fd_ / (double)fs_);
    set_fixed_point_scale(p);
    p.wide_cta = wide_cta_ ? 1 : 0;
    p.lut_smem = lut_smem_ ? 1 : 0;
    p.err_flag = err_flag_dev_.as<int>();
    // exact culling ranges (fp64 mode): outside them the weight is exactly 0
    if (mode_ == MODE_FP64 && cull_) {
        double llo, lhi, elo, ehi;
        if (beam_type_ == BEAM_GAUSSIAN) {
            // exp2f(-q) is exactly 0 for q >= 151, q = l^2 gl + e^2 ge
            const double rl = std::sqrt(151.0 / (double)b.gl), re = std::sqrt(151.0 / (double)b.ge);
            llo = -rl; lhi = rl; elo = -re; ehi = re;
        } else {
            // table coordinate -1 < t < n-1  <=>  first - spacing < x < last
            llo = (double)lut_ext_[2] - b.dl; lhi = lut_ext_[3];
            elo = (double)lut_ext_[4] - b.de; ehi = lut_ext_[5];
        }
        const double ml = 1e-3 * (std::fabs(llo) + std::fabs(lhi)) + 1e-7;
        const double me = 1e-3 * (std::fabs(elo) + std::fabs(ehi)) + 1e-7;
        p.cull = std::isfinite(llo + lhi + elo + ehi) ? 1 : 0;
        p.cull_l_lo = (float)(llo - ml); p.cull_l_hi = (float)(lhi + ml);
        p.cull_e_lo = (float)(elo - me); p.cull_e_hi = (float)(ehi + me);
        p.cull_rho_per_bin = (float)((double)sound_speed_ / (2.0 * (double)fs_) * 1.0001);
    }

    // per-line spline knot intervals and basis (CpuAlgorithm.cpp:101-133)
    std::vector<std::vector<int>> mus(splines_.size());
    std::vector<std::vector<LineBasis>> bases(splines_.size());
    for (size_t d = 0; d < splines_.size(); d++) {
        const SplineDataset& ds = splines_[d];
        if (ds.n == 0) continue;
        if (ds.num_cs <= ds.degree) throw SimError(BCSIM_E_INVALID, "too few spline control points for given degree");
        mus[d].resize(L);
        bases[d].resize(L);
        for (int i = 0; i < L; i++) {
            const float t = timestamps_[i];
            const int mu = knot_interval(ds.knots, t);
            if (mu < 0) throw SimError(BCSIM_E_INVALID, "compute_knot_interval : could not determine knot interval");
            const int lo = mu - ds.degree;
            if (lo < 0 || mu >= ds.num_cs) throw SimError(BCSIM_E_INVALID, "spline evaluation index out of range");
            LineBasis lb;
            std::memset(&lb, 0, sizeof(lb));
            for (int j = 0; j < ds.num_cs; j++) {
                double v;
                if (mode_ == MODE_FP64) v = bspline_basis_d(j, ds.degree, (double)t, ds.knots);
                else v = bspline_basis_f(j, ds.degree, t, ds.knots);
                if (j < lo || j > mu) {
                    // sanity_check_spline_lower_upper_bound (common_utils.hpp:51-60)
                    if (std::fabs(v) > 1e-6) throw SimError(BCSIM_E_INVALID, "b-spline basis bounds failed sanity check");
                } else {
                    const float hi = (float)v;
                    lb.hi[j - lo] = hi;
                    lb.lo[j - lo] = mode_ == MODE_FP64 ? (float)(v - (double)hi) : 0.0f;
                }
            }
            lb.mu = mu;
            mus[d][i] = mu;
            bases[d][i] = lb;
        }
    }

    P.shared = shared_origin_ && arc_;
    // splines go through the shared path when every line sees them at one time
    P.spline_shared.assign(splines_.size(), 0);
    P.n_shared = P.shared ? fixed_n_ : 0;
    if (P.shared && timestamps_equal_ && render_once_) {
        for (size_t d = 0; d < splines_.size(); d++) {
            if (splines_[d].n > 0) {
                P.spline_shared[d] = 1;
                P.n_shared += splines_[d].n;
            }
        }
    }

    // lines of a per-pair tile: sorted by knot interval (splines), then by
    // direction; a tile of splines spans at most 64 control points (so that the
    // kernel stages at least 32 scatterers per chunk)
    auto make_tiles = [&](const std::vector<int>* mu, int degree, std::vector<int>& ids, std::vector<LineTile>& tiles) {
        ids.resize(L);
        std::iota(ids.begin(), ids.end(), 0);
        std::sort(ids.begin(), ids.end(), [&](int a, int c) {
            const int ma = mu ? (*mu)[a] : 0, mc = mu ? (*mu)[c] : 0;
            return ma != mc ? ma < mc : line_rank_[a] < line_rank_[c];
        });
        const int per = tile_lines_ > 0 ? std::min(tile_lines_, PAIR_THREADS) : PAIR_THREADS;
        tiles.clear();
        int i = 0;
        while (i < L) {
            LineTile t;
            t.first = i;
            t.mu = mu ? (*mu)[ids[i]] : 0;
            int j = i;
            while (j < L && j - i < per && (!mu || (*mu)[ids[j]] - t.mu + degree + 1 <= 64)) j++;
            t.count = j - i;
            t.span = mu ? (*mu)[ids[j - 1]] - t.mu + degree + 1 : 1;
            tiles.push_back(t);
            i = j;
        }
    };
    std::vector<LineTile> all_tiles;
    std::vector<TileBox> all_boxes;
    std::vector<int> all_ids;
    std::vector<LineBasis> all_basis;
    P.tile_cull = mode_ == MODE_FP64 && cull_ && P.p.cull;
    auto add_gen = [&](int kind, int d) {
        std::vector<int> ids;
        std::vector<LineTile> tiles;
        make_tiles(kind == 1 ? &mus[d] : nullptr, kind == 1 ? splines_[d].degree : 0, ids, tiles);
        GenLaunch g;
        g.kind = kind;
        g.d = d;
        g.tile_off = all_tiles.size();
        g.num_tiles = tiles.size();
        // CTAs as wide as the widest tile: a job of fewer lines than a full tile
        // launches no warps without lines
        int most = 1;
        for (const auto& t : tiles) most = std::max(most, t.count);
        g.threads = std::min(PAIR_THREADS, (most + 31) / 32 * 32);
        g.basis_off = all_basis.size();
        const size_t id_off = all_ids.size();
        if (P.tile_cull)
            for (auto& t : tiles) all_boxes.push_back(make_tile_box(lines_, ids.data() + t.first, t.count));
        for (auto& t : tiles) t.first += (int)id_off;
        all_tiles.insert(all_tiles.end(), tiles.begin(), tiles.end());
        all_ids.insert(all_ids.end(), ids.begin(), ids.end());
        if (kind == 1) all_basis.insert(all_basis.end(), bases[d].begin(), bases[d].end());
        P.gl.push_back(g);
    };
    if (fixed_n_ > 0) add_gen(0, -1);
    for (size_t d = 0; d < splines_.size(); d++)
        if (splines_[d].n > 0) add_gen(1, (int)d);
    gen_tiles_.reserve(std::max<size_t>(1, all_tiles.size()) * sizeof(LineTile), stream_);
    gen_line_ids_.reserve(std::max<size_t>(1, all_ids.size()) * sizeof(int), stream_);
    gen_basis_.reserve(std::max<size_t>(1, all_basis.size()) * sizeof(LineBasis), stream_);
    if (!all_tiles.empty())
        BCSIM_CUDA(cudaMemcpyAsync(gen_tiles_.get(), all_tiles.data(), all_tiles.size() * sizeof(LineTile), cudaMemcpyHostToDevice, st));
    if (!all_ids.empty())
        BCSIM_CUDA(cudaMemcpyAsync(gen_line_ids_.get(), all_ids.data(), all_ids.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    if (!all_basis.empty())
        BCSIM_CUDA(cudaMemcpyAsync(gen_basis_.get(), all_basis.data(), all_basis.size() * sizeof(LineBasis), cudaMemcpyHostToDevice, st));
    gen_boxes_.reserve(std::max<size_t>(1, all_boxes.size()) * sizeof(TileBox), stream_);
    if (!all_boxes.empty())
        BCSIM_CUDA(cudaMemcpyAsync(gen_boxes_.get(), all_boxes.data(), all_boxes.size() * sizeof(TileBox), cudaMemcpyHostToDevice, st));

    // device buffers
    const int stride = phase_delay_ ? 2 : 1;
    P.bins_bytes = (size_t)L * ns * stride * sizeof(unsigned long long);
    bins_[cur_].reserve(P.bins_bytes, stream_);
    rec().counts.reserve(4 * sizeof(int), stream_);
    pair_counts_.reserve(4 * sizeof(unsigned long long), stream_);
    out_.reserve((size_t)L * nd_ * sizeof(float2), stream_);
    P.spline_off.assign(splines_.size(), -1);
    if (P.n_shared > 0) {
        const int64_t N = P.n_shared;
        int64_t off = fixed_n_;
        std::vector<double> bd(64 * std::max<size_t>(1, splines_.size()), 0.0);
        std::vector<float> bf(64 * std::max<size_t>(1, splines_.size()), 0.0f);
        for (size_t d = 0; d < splines_.size(); d++) {
            if (!P.spline_shared[d]) continue;
            const SplineDataset& ds = splines_[d];
            const int lo = mus[d][0] - ds.degree;
            for (int k2 = 0; k2 <= ds.degree; k2++) {
                // exact double basis for the render (bit parity with the FP64 oracle)
                bd[64 * d + k2] = bspline_basis_d(lo + k2, ds.degree, (double)timestamps_[0], ds.knots);
                bf[64 * d + k2] = bases[d][0].hi[k2];
            }
            P.spline_off[d] = off;
            P.spline_first_cs.resize(splines_.size(), 0);
            P.spline_first_cs[d] = lo;
            off += ds.n;
        }
        spl_basis_d_.reserve(bd.size() * sizeof(double), stream_);
        spl_basis_f_.reserve(bf.size() * sizeof(float), stream_);
        BCSIM_CUDA(cudaMemcpyAsync(spl_basis_d_.get(), bd.data(), bd.size() * sizeof(double), cudaMemcpyHostToDevice, st));
        BCSIM_CUDA(cudaMemcpyAsync(spl_basis_f_.get(), bf.data(), bf.size() * sizeof(float), cudaMemcpyHostToDevice, st));
        // sort key: the bin (ns + 2 values) above a 10-bit angular cell (32 x 32
        // octahedral cells), fewer cell bits where the bins need more than 22.
        // Cells only where a bin holds two words of records on average: with
        // fewer, a word spans several bins and the cells buy nothing for their
        // radix-sort pass and the kernel's word test.  (Not tied to culling, so
        // that culling on and off see the same record order.)
        int end_bit = 1;
        while ((1ll << end_bit) < (int64_t)ns + 2) end_bit++;
        P.p.cell_bits = N >= 64 * (int64_t)ns ? std::max(0, std::min(10, 32 - end_bit)) & ~1 : 0;
        P.end_bit = end_bit + P.p.cell_bits;
        reserve_records(rec(), P);
        // records per CTA: enough CTAs to fill the GPU several times over, a
        // multiple of the fold group (512 records when chunks of 512 fill the
        // GPU, else 128), so that results do not depend on the chunk
        P.p.fold = (N + 511) / 512 >= 4 * 152 ? 512 : 128;
        int chunk = 1024;
        while (chunk > P.p.fold && (N + chunk - 1) / chunk < 4 * 152) chunk /= 2;
        P.chunk = chunk;
        P.records_key = records_key_of(P);
    }
    // the host vectors above are pageable: finish their copies before they go
    BCSIM_CUDA(cudaStreamSynchronize(st));
    P.version = cfg_version_;
    P.static_version = static_version_;
    P.data_shape = data_shape();
    if (autotune_) autotune();
}

// Buffers of one record set for plan P (P.end_bit set; fills P.sort_tmp_bytes).
void Simulator::reserve_records(RecordSet& R, Plan& P) {
    R.counts.reserve(4 * sizeof(int), stream_);
    const int64_t N = P.n_shared;
    if (N <= 0) return;
    R.keys_in.reserve(N * sizeof(uint32_t), stream_);
    R.vals_in.reserve(N * sizeof(uint32_t), stream_);
    R.keys_out.reserve(N * sizeof(uint32_t), stream_);
    R.vals_out.reserve(N * sizeof(uint32_t), stream_);
    R.recA.reserve(N * sizeof(float4), stream_);
    R.recB.reserve(N * sizeof(float4), stream_);
    R.records.reserve((size_t)N * 2 * sizeof(float4), stream_);
    size_t tmp_bytes = 0;
    BCSIM_CUDA(radix_sort_pairs(nullptr, &tmp_bytes, R.keys_in.as<uint32_t>(), R.keys_out.as<uint32_t>(),
                                R.vals_in.as<uint32_t>(), R.vals_out.as<uint32_t>(), N, P.end_bit, stream_));
    R.sort_tmp.reserve(tmp_bytes, stream_);
    P.sort_tmp_bytes = tmp_bytes;
}

// The shared-origin records in bin order (unless the set already holds them):
// per-scatterer prep, radix sort by bin, bin-range counts, gather.
void Simulator::enqueue_records(cudaStream_t st, int* launches) {
    const Plan& P = plan_;
    RecordSet& R = rec();
    if (P.n_shared <= 0 || (record_cache_ && R.key == P.records_key)) return;
    const SimParams& p = P.p;
    const BeamDev& b = P.b;
    const int64_t N = P.n_shared;
    const int ns = (int)ns_;
    const float* origin = lines_[0].o;
    if (fixed_n_ > 0) {
        ++*launches;
        BCSIM_CUDA(launch_prep_shared(fixed_src(), fixed_n_, 0, origin, p, b, R.keys_in.as<uint32_t>(),
                                      R.vals_in.as<uint32_t>(), R.recA.as<float4>(), R.recB.as<float4>(), st));
    }
    for (size_t d = 0; d < splines_.size(); d++) {
        if (!P.spline_shared[d]) continue;
        const SplineDataset& ds = splines_[d];
        ++*launches;
        BCSIM_CUDA(launch_prep_shared_spline(ds.cps_dev(), ds.amps_dev(), ds.n, ds.num_cs,
                                             P.spline_first_cs[d], ds.degree, spl_basis_d_.as<double>() + 64 * d,
                                             spl_basis_f_.as<float>() + 64 * d, P.spline_off[d], origin, p, b,
                                             R.keys_in.as<uint32_t>(), R.vals_in.as<uint32_t>(), R.recA.as<float4>(),
                                             R.recB.as<float4>(), st));
    }
    size_t tmp_bytes = P.sort_tmp_bytes;
    BCSIM_CUDA(radix_sort_pairs(R.sort_tmp.get(), &tmp_bytes, R.keys_in.as<uint32_t>(), R.keys_out.as<uint32_t>(),
                                R.vals_in.as<uint32_t>(), R.vals_out.as<uint32_t>(), N, P.end_bit, st));
    *launches += 3;   // init, count, finish
    BCSIM_CUDA(launch_count_keys(R.keys_out.as<uint32_t>(), N, ns, P.p.cell_bits, R.counts.as<int>(), st));
    ++*launches;
    BCSIM_CUDA(launch_gather_records(R.vals_out.as<uint32_t>(), R.counts.as<int>(), N, R.recA.as<float4>(),
                                     R.recB.as<float4>(), R.records.as<float4>(), N, st));
    R.key = P.records_key;
}

// ---------------------------------------------------------------------------
// enqueue: device work only (capturable: no allocation, no host copy, no sync)
// ---------------------------------------------------------------------------
void Simulator::enqueue(cudaStream_t st, float2* dev_out, bool timing, float* host_out, bool wait_copies,
                        bool staged) {
    const Plan& P = plan_;
    const SimParams& p = P.p;
    const BeamDev& b = P.b;
    const int L = num_lines_;
    const int ns = (int)ns_;
    EventTimer total(timing, st, &pending_timings_);
    EventTimer timer(timing, st, &pending_timings_);
    unsigned long long* bins = bins_[cur_].as<unsigned long long>();
    RecordSet& R = rec();
    int launches = 0;   // kernels of this library launched (the radix sort's are counted apart)
    const LineGeom* lines_d = lines_dev_.as<LineGeom>();
    // the bins are cleared on the side stream, after st's earlier work (the
    // previous convolution read them), while the records are prepared; st
    // waits for it before the first kernel that writes bins
    if (!staged) {
        const cudaStream_t side = side_stream_.s;
        EventTimer mt(timing, side, &pending_timings_);
        BCSIM_CUDA(cudaEventRecord(ev_fork_.e, st));
        BCSIM_CUDA(cudaStreamWaitEvent(side, ev_fork_.e, 0));
        if (timing) mt.restart();
        BCSIM_CUDA(cudaMemsetAsync(bins, 0, P.bins_bytes, side));
        BCSIM_CUDA(cudaEventRecord(ev_join_.e, side));
        if (timing) mt.stop("kernel_memset_ms");
    }
    bool joined = staged;
    auto join_bins = [&]() {
        if (!joined) BCSIM_CUDA(cudaStreamWaitEvent(st, ev_join_.e, 0));
        joined = true;
    };
    unsigned long long* pair_counts = nullptr;   // instrumented run (count_pairs)
    if (count_pairs_ && p.mode == MODE_FP64) {
        pair_counts = pair_counts_.as<unsigned long long>();
        BCSIM_CUDA(cudaMemsetAsync(pair_counts, 0, 4 * sizeof(unsigned long long), st));
    }

    if (P.n_shared > 0) {
        const int64_t N = P.n_shared;
        timer.restart();
        if (!staged) enqueue_records(st, &launches);
        if (timing) timer.stop("prep_sort_ms");
        timer.restart();

        join_bins();
        ++launches;
        BCSIM_CUDA(launch_project_shared(R.records.as<float4>(), N, R.counts.as<int>(), N, P.chunk, lines_d,
                                         line_order_dev_.as<int>(), cones_dev_.as<SlotCone>(), L, p, b, bins,
                                         pair_counts, st));
        // near-origin residue, per pair
        for (const GenLaunch& g : P.gl) {
            if (g.kind == 0) {
                ++launches;
                BCSIM_CUDA(launch_project_generic(fixed_src(), nullptr, nullptr, fixed_n_, 0, 0,
                                                  R.vals_out.as<uint32_t>(), R.counts.as<int>(), 0, lines_d,
                                                  gen_line_ids_.as<int>(), gen_tiles_.as<LineTile>() + g.tile_off,
                                                  (int)g.num_tiles, nullptr, p, b, bins, st, P.tile_cull ? gen_boxes_.as<TileBox>() + g.tile_off : nullptr,
                                                  pair_counts, g.threads));
            } else if (P.spline_shared[g.d]) {
                const SplineDataset& ds = splines_[g.d];
                ++launches;
                BCSIM_CUDA(launch_project_generic(nullptr, ds.cps_dev(), ds.amps_dev(), ds.n, ds.num_cs,
                                                  ds.degree, R.vals_out.as<uint32_t>(), R.counts.as<int>(),
                                                  P.spline_off[g.d], lines_d, gen_line_ids_.as<int>(),
                                                  gen_tiles_.as<LineTile>() + g.tile_off, (int)g.num_tiles,
                                                  gen_basis_.as<LineBasis>() + g.basis_off, p, b, bins, st, P.tile_cull ? gen_boxes_.as<TileBox>() + g.tile_off : nullptr,
                                                  pair_counts, g.threads));
            }
        }
        if (timing) timer.stop("fixed_projection_kernel_ms");
    }

    // per-pair path
    join_bins();
    timer.restart();
    for (const GenLaunch& g : P.gl) {
        if (g.kind == 0) {
            if (P.shared) continue;
            ++launches;
                BCSIM_CUDA(launch_project_generic(fixed_src(), nullptr, nullptr, fixed_n_, 0, 0, nullptr,
                                              nullptr, 0, lines_d, gen_line_ids_.as<int>(),
                                              gen_tiles_.as<LineTile>() + g.tile_off, (int)g.num_tiles, nullptr, p,
                                              b, bins, st, P.tile_cull ? gen_boxes_.as<TileBox>() + g.tile_off : nullptr,
                                                  pair_counts, g.threads));
        } else {
            if (P.spline_shared[g.d]) continue;
            const SplineDataset& ds = splines_[g.d];
            ++launches;
                BCSIM_CUDA(launch_project_generic(nullptr, ds.cps_dev(), ds.amps_dev(), ds.n, ds.num_cs,
                                              ds.degree, nullptr, nullptr, 0, lines_d, gen_line_ids_.as<int>(),
                                              gen_tiles_.as<LineTile>() + g.tile_off, (int)g.num_tiles,
                                              gen_basis_.as<LineBasis>() + g.basis_off, p, b, bins, st, P.tile_cull ? gen_boxes_.as<TileBox>() + g.tile_off : nullptr,
                                                  pair_counts, g.threads));
        }
    }
    if (timing) timer.stop(P.shared ? "spline_projection_kernel_ms" : "fixed_projection_kernel_ms");

    // convolution + demodulation + decimation; with a host destination in
    // blocks of lines, each block's IQ copied out while the next is convolved
    // (in a stream of frames, wait_copies off, the copies overlap the next frame
    // instead: one block)
    timer.restart();
    const bool use_fft = convolution_ == 2 || (convolution_ == 0 && fft_ok_ && fft_faster(L, nd_, tap_count_, M_, sms_));
    last_route_fft_ = use_fft;
    route_known_ = true;
    const int nblocks = (host_out && L >= 1024 && wait_copies) ? 4 : 1;
    while ((int)ev_blocks_.size() < nblocks) {
        cudaEvent_t e = nullptr;
        BCSIM_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ev_blocks_.push_back(e);
    }
    const int stride_bins = p.phase_delay ? 2 : 1;
    // seeded noise on the time projection (noise_amplitude > 0), keyed by the
    // seed, this simulation's frame number, the line and the sample
    NoiseParams nz{};
    if (noise_amplitude_ > 0.0f) {
        nz.sigma = noise_amplitude_;
        nz.key0 = (uint32_t)noise_seed_;
        nz.key1 = (uint32_t)(noise_seed_ >> 32);
        nz.frame = noise_frame_++;
    }
    for (int k = 0; k < nblocks; k++) {
        const int l0 = (int)((int64_t)L * k / nblocks), l1 = (int)((int64_t)L * (k + 1) / nblocks);
        if (l1 <= l0) continue;
        nz.line0 = l0;
        ++launches;
        if (use_fft)
            BCSIM_CUDA(launch_fft_convolve_demodulate(bins + (int64_t)l0 * ns * stride_bins, l1 - l0, ns,
                                                      p.phase_delay, std::ldexp(1.0f, -p.log2scale),
                                                      fft_spec_dev_.as<float2>(), fft_tw_dev_.as<float2>(), M_,
                                                      decimation_, (int)nd_, demod_dev_.as<float2>(),
                                                      dev_out + (int64_t)l0 * nd_, st, &nz));
        else
            BCSIM_CUDA(launch_convolve_demodulate(bins + (int64_t)l0 * ns * stride_bins, l1 - l0, ns, p.phase_delay,
                                                  std::ldexp(1.0f, -p.log2scale), taps_pm_dev_.as<float2>(),
                                                  ph_off_dev_.as<int>(), ntaps_pm_, max_ph_taps_, (int)tap_count_,
                                                  (int)tap_start_, M_, center_, decimation_, (int)nd_,
                                                  demod_dev_.as<float2>(), dev_out + (int64_t)l0 * nd_, st, &nz));
        if (host_out) {
            const cudaStream_t cs = copy_stream_.s;
            BCSIM_CUDA(cudaEventRecord(ev_blocks_[k], st));
            BCSIM_CUDA(cudaStreamWaitEvent(cs, ev_blocks_[k], 0));
            BCSIM_CUDA(cudaMemcpyAsync(host_out + 2 * (int64_t)l0 * nd_, dev_out + (int64_t)l0 * nd_,
                                       (size_t)(l1 - l0) * nd_ * sizeof(float2), cudaMemcpyDeviceToHost, cs));
        }
    }
    if (host_out) {
        BCSIM_CUDA(cudaEventRecord(ev_copied_.e, copy_stream_.s));
        if (wait_copies) BCSIM_CUDA(cudaStreamWaitEvent(st, ev_copied_.e, 0));
    }
    if (timing) {
        timer.stop("kernel_convolve_demodulate_ms");
        total.stop("total_ms");
    }
    last_launches_ = launches;
}

void Simulator::simulate(float2* dev_out, float* host_out) {
    prepare();
    if (store_details_) debug_.clear();
    drop_timings();
    const cudaStream_t st = stream_;
    enqueue(st, dev_out, store_details_, host_out);
    if (count_pairs_ && mode_ == MODE_FP64) {
        unsigned long long c[4] = {0, 0, 0, 0};
        BCSIM_CUDA(cudaMemcpyAsync(c, pair_counts_.get(), sizeof c, cudaMemcpyDeviceToHost, st));
        BCSIM_CUDA(cudaStreamSynchronize(st));
        debug_["evaluated_pairs"] = {(double)c[0]};
        debug_["weighted_pairs"] = {(double)c[1]};
        debug_["idle_walk_steps"] = {(double)c[2]};
        debug_["per_pair_evaluated_pairs"] = {(double)c[3]};
    }
    if (host_out) {
        EventTimer timer(store_details_, st, &pending_timings_);
        // (the IQ was copied by enqueue, overlapped with the convolution)
        // the bounded-wait error flag travels with the result (one synchronisation)
        if (!flag_host_.p) BCSIM_CUDA(cudaMallocHost(&flag_host_.p, sizeof(int)));
        BCSIM_CUDA(enqueue_error_flag_read(err_flag_dev_.as<int>(), flag_host_.p, st));
        if (store_details_) timer.stop("kernel_memcpy_ms");
        BCSIM_CUDA(cudaStreamSynchronize(st));
        if (store_details_) resolve_timings();
        if (*flag_host_.p) check_device_flag();   // clears the flag and reports
    } else if (store_details_) {
        resolve_timings();   // waits for the simulation (timed calls only)
    }
}

void Simulator::check_device_flag() {
    ensure_device();
    int flag = 0;
    BCSIM_CUDA(read_and_clear_error_flag(err_flag_dev_.as<int>(), &flag, stream_));
    if (flag) throw SimError(BCSIM_E_INTERNAL, "a bounded device wait gave up; results are incomplete");
}

void Simulator::raise_device_flag() {
    ensure_device();
    const int one = 1;
    BCSIM_CUDA(cudaMemcpyAsync(err_flag_dev_.get(), &one, sizeof(int), cudaMemcpyHostToDevice, stream_));
    BCSIM_CUDA(cudaStreamSynchronize(stream_));
}

// Launch shapes from measurement, per shape class (path, beam, phase delay,
// scatterer and line count buckets, spline degree): the per-pair projection's
// lines per tile {128, 96, 64}, then the shared-origin kernel's scatterers
// (records) per CTA {128 ... 1024}; each candidate timed on this
// configuration (best of two) and the fastest kept.  No shape changes the results (fixed-point sums; FP32 partial sums
// aligned to absolute record indices), only the time.
void Simulator::autotune() {
    if (autotuning_) return;
    auto bucket = [](int64_t v) { int b = 0; while (v > 1) { v >>= 1; b++; } return b; };
    bool has_pair = false;
    for (const GenLaunch& g : plan_.gl)
        has_pair = has_pair || (g.kind == 0 ? !plan_.shared : !plan_.spline_shared[g.d]);
    const int64_t n_pairs = total_num_scatterers();
    const std::string key = std::to_string(plan_.shared) + "/" + std::to_string(beam_type_) + "/" +
                            std::to_string(phase_delay_) + "/" + std::to_string(bucket(n_pairs)) + "/" +
                            std::to_string(bucket(num_lines_)) + "/" +
                            std::to_string(splines_.empty() ? -1 : splines_[0].degree) + "/" +
                            std::to_string(has_pair);
    struct Tuned {
        int chunk, tile_lines;
    };
    static std::mutex mtx;
    static std::map<std::string, Tuned> cache;
    struct Guard {
        bool& f;
        explicit Guard(bool& x) : f(x) { f = true; }
        ~Guard() { f = false; }
    } guard(autotuning_);
    auto replan = [&](int tl) {
        tile_lines_ = tl;
        plan_.version = ~0ull;   // rebuild the tiles for the new line count
        prepare();
    };
    {
        std::lock_guard<std::mutex> lock(mtx);
        auto it = cache.find(key);
        if (it != cache.end()) {
            const Tuned t = it->second;
            if (t.tile_lines != tile_lines_) replan(t.tile_lines);
            if (plan_.n_shared > 0) plan_.chunk = t.chunk;
            return;
        }
    }
    const cudaStream_t st = stream_;
    out_.reserve((size_t)num_lines_ * nd_ * sizeof(float2), stream_);
    cudaEvent_t e0, e1;
    BCSIM_CUDA(cudaEventCreate(&e0));
    BCSIM_CUDA(cudaEventCreate(&e1));
    auto time_it = [&]() {
        float ms_min = 1e30f;
        for (int rep = 0; rep < 2; rep++) {
            BCSIM_CUDA(cudaEventRecord(e0, st));
            enqueue(st, out_.as<float2>(), false);
            BCSIM_CUDA(cudaEventRecord(e1, st));
            BCSIM_CUDA(cudaEventSynchronize(e1));
            float ms = 0.0f;
            BCSIM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            ms_min = std::min(ms_min, ms);
        }
        return ms_min;
    };
    Tuned best{plan_.chunk, tile_lines_};
    float best_ms = 1e30f;
    enqueue(st, out_.as<float2>(), false);   // records, warm-up
    if (has_pair) {
        for (int tl : {0, 96, 64}) {
            if (tl != tile_lines_) replan(tl);
            enqueue(st, out_.as<float2>(), false);
            const float ms = time_it();
            if (ms < best_ms) { best_ms = ms; best = Tuned{plan_.chunk, tl}; }
        }
        if (best.tile_lines != tile_lines_) replan(best.tile_lines);
    }
    if (plan_.n_shared > 0) {
        const std::vector<int> chunks = plan_.p.fold == 512 ? std::vector<int>{512, 1024}
                                                            : std::vector<int>{128, 256, 512, 1024};
        best_ms = 1e30f;
        for (int c : chunks) {
            plan_.chunk = c;
            const float ms = time_it();
            if (ms < best_ms) { best_ms = ms; best.chunk = c; }
        }
        plan_.chunk = best.chunk;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::lock_guard<std::mutex> lock(mtx);
    cache[key] = best;
    log(0, "autotune " + key + ": records per CTA " + std::to_string(best.chunk) + ", lines per tile " +
               std::to_string(best.tile_lines));
}

void Simulator::simulate_host(float* host_out, int64_t cap_complex, int64_t* lines, int64_t* samples) {
    throw_if_not_configured();
    int64_t L = 0, nd = 0;
    output_shape(&L, &nd);
    if (lines) *lines = L;
    if (samples) *samples = nd;
    if (!host_out || cap_complex < L * nd)
        throw SimError(BCSIM_E_CAPACITY, "output buffer too small: need " + std::to_string(L * nd) + " complex values");
    ensure_device();
    out_.reserve((size_t)L * nd * sizeof(float2), stream_);
    simulate(out_.as<float2>(), host_out);
}

void Simulator::simulate_fixed_frames(const float* const* frames, int64_t n, int num_frames, float* const* outs,
                                      int64_t cap_complex) {
    if (num_frames <= 0) return;
    if (n <= 0 || !frames || !outs) throw SimError(BCSIM_E_INVALID, "simulate_fixed_frames: invalid data");
    for (int k = 0; k < num_frames; k++)
        if (!frames[k] || !outs[k]) throw SimError(BCSIM_E_INVALID, "simulate_fixed_frames: null frame or output");
    ensure_device();
    int64_t L = 0, nd = 0;
    output_shape(&L, &nd);
    if (cap_complex < L * nd)
        throw SimError(BCSIM_E_CAPACITY, "output buffer too small: need " + std::to_string(L * nd) + " complex values");
    const size_t bytes = (size_t)n * sizeof(float4);
    for (int b = 0; b < 2; b++) {
        frame_xyza_[b].reserve(bytes, stream_);
        frame_scratch_[b].reserve(abs_sum_scratch_bytes(), stream_);
        frame_out_[b].reserve((size_t)L * nd * sizeof(float2), stream_);
    }
    if (!frame_bounds_.p) BCSIM_CUDA(cudaMallocHost(&frame_bounds_.p, sizeof(FrameBounds)));
    BCSIM_CUDA(cudaStreamSynchronize(stream_));   // the buffers exist before the upload stream uses them
    const cudaStream_t up = upload_stream_.s;
    // frame k: into buffer k & 1, once the frame that read it last (k - 2) is done
    auto upload = [&](int k) {
        const int b = k & 1;
        if (k >= 2) BCSIM_CUDA(cudaStreamWaitEvent(up, ev_consumed_[b].e, 0));
        BCSIM_CUDA(cudaMemcpyAsync(frame_xyza_[b].get(), frames[k], bytes, cudaMemcpyHostToDevice, up));
        BCSIM_CUDA(abs_sum_enqueue(frame_xyza_[b].as<float>() + 3, 4, n, frame_scratch_[b].get(),
                                   &frame_bounds_.p->sum[b], &frame_bounds_.p->nonfinite[b], up));
        BCSIM_CUDA(cudaEventRecord(ev_uploaded_[b].e, up));
    };
    // afterwards (or on an error) the frame last installed is the fixed dataset
    int installed = -1;
    auto settle = [&]() {
        cudaStreamSynchronize(up);
        cudaStreamSynchronize(prep_stream_.s);
        cudaStreamSynchronize(copy_stream_.s);
        cudaStreamSynchronize(stream_);
        if (installed >= 0) std::swap(fixed_xyza_, frame_xyza_[installed & 1]);
        fixed_src_ = nullptr;
    };
    const cudaStream_t ps = prep_stream_.s;
    bool sets_ready = false;
    try {
        upload(0);
        for (int k = 0; k < num_frames; k++) {
            const int b = k & 1;
            if (k + 1 < num_frames) upload(k + 1);
            BCSIM_CUDA(cudaEventSynchronize(ev_uploaded_[b].e));   // frame k's amplitude bound
            fixed_src_ = frame_xyza_[b].as<float4>();
            installed = k;
            fixed_n_ = n;
            num_fixed_sets_ = 1;
            fixed_sum_abs_ = frame_bounds_.p->sum[b];
            amplitude_nonfinite_ = frame_bounds_.p->nonfinite[b] != 0;
            cfg_version_++;
            data_version_++;
            cur_ = b;   // bins and record set b
            prepare();   // a new frame of the same shape: the scale and the records' identity
            if (!sets_ready) {
                for (int c = 0; c < 2; c++) {
                    bins_[c].reserve(plan_.bins_bytes, stream_);
                    reserve_records(rs_[c], plan_);
                }
                BCSIM_CUDA(cudaStreamSynchronize(stream_));   // before the prep stream uses them
                sets_ready = true;
            }
            // frame k's bins cleared and records prepared on the prep stream, once
            // frame k - 2 (the last user of set b) is done: while frame k - 1 runs
            BCSIM_CUDA(cudaStreamWaitEvent(ps, ev_uploaded_[b].e, 0));
            if (k >= 2) BCSIM_CUDA(cudaStreamWaitEvent(ps, ev_consumed_[b].e, 0));
            BCSIM_CUDA(cudaMemsetAsync(bins_[b].get(), 0, plan_.bins_bytes, ps));
            int launches = 0;
            enqueue_records(ps, &launches);
            BCSIM_CUDA(cudaEventRecord(ev_staged_[b].e, ps));
            BCSIM_CUDA(cudaStreamWaitEvent(stream_, ev_staged_[b].e, 0));
            // two device outputs too: frame k + 1 is convolved while frame k's
            // last block is still copied to the host
            if (k >= 2) BCSIM_CUDA(cudaStreamWaitEvent(stream_, ev_out_free_[b].e, 0));
            enqueue(stream_, frame_out_[b].as<float2>(), false, outs[k], false, true);
            BCSIM_CUDA(cudaEventRecord(ev_consumed_[b].e, stream_));
            BCSIM_CUDA(cudaEventRecord(ev_out_free_[b].e, copy_stream_.s));
        }
        BCSIM_CUDA(cudaStreamWaitEvent(stream_, ev_copied_.e, 0));   // the last frame's copies
        if (!flag_host_.p) BCSIM_CUDA(cudaMallocHost(&flag_host_.p, sizeof(int)));
        BCSIM_CUDA(enqueue_error_flag_read(err_flag_dev_.as<int>(), flag_host_.p, stream_));
    } catch (...) {
        settle();
        throw;
    }
    settle();
    if (*flag_host_.p) check_device_flag();
}

// The spline counterpart of simulate_fixed_frames: per frame the reference's
// clear_spline_scatterers + add_spline_scatterers + simulate_lines
// (LibBCSim.hpp:63-70,81), with frame k+1's control points uploaded, laid out
// [K][n] and their amplitude bound reduced on the upload stream while frame k
// is simulated.  The frames share one shape (degree, knots, n, num_cs), so the
// plan (line bases, tiles, culling boxes) is kept; each frame redoes the
// fixed-point scale.
void Simulator::simulate_spline_frames(int degree, const float* knots, int num_knots, const float* const* cps_frames,
                                       const float* const* amps_frames, int64_t n, int num_cs, int num_frames,
                                       float* const* outs, int64_t cap_complex) {
    if (num_frames <= 0) return;
    if (n <= 0 || num_cs <= 0 || !cps_frames || !amps_frames || !outs || num_knots < 0 || (num_knots > 0 && !knots))
        throw SimError(BCSIM_E_INVALID, "simulate_spline_frames: invalid data");
    // src/python/PythonInterface.cpp:150-153, as add_spline_scatterers
    if (num_knots != num_cs + degree + 1)
        throw SimError(BCSIM_E_INVALID, "add_spline_scatterers : mismatch in number of nodes, degree and control points");
    if (degree < 0 || degree > MAX_SPLINE_DEGREE)
        throw SimError(BCSIM_E_INVALID, "add_spline_scatterers : spline degree must be in [0, " +
                                            std::to_string(MAX_SPLINE_DEGREE) + "]");
    for (int k = 0; k < num_frames; k++)
        if (!cps_frames[k] || !amps_frames[k] || !outs[k])
            throw SimError(BCSIM_E_INVALID, "simulate_spline_frames: null frame or output");
    ensure_device();
    int64_t L = 0, nd = 0;
    output_shape(&L, &nd);
    if (cap_complex < L * nd)
        throw SimError(BCSIM_E_CAPACITY, "output buffer too small: need " + std::to_string(L * nd) + " complex values");
    const size_t raw_bytes = (size_t)n * num_cs * 3 * sizeof(float);
    const size_t cps_bytes = (size_t)num_cs * n * sizeof(float4);
    const size_t amp_bytes = (size_t)n * sizeof(float);
    for (int b = 0; b < 2; b++) {
        frame_raw_[b].reserve(raw_bytes, stream_);
        frame_cps_[b].reserve(cps_bytes, stream_);
        frame_amps_[b].reserve(amp_bytes, stream_);
        frame_scratch_[b].reserve(abs_sum_scratch_bytes(), stream_);
        frame_out_[b].reserve((size_t)L * nd * sizeof(float2), stream_);
    }
    if (!frame_bounds_.p) BCSIM_CUDA(cudaMallocHost(&frame_bounds_.p, sizeof(FrameBounds)));
    BCSIM_CUDA(cudaStreamSynchronize(stream_));   // the buffers exist before the upload stream uses them
    const cudaStream_t up = upload_stream_.s;
    // frame k: into buffer k & 1, once the frame that read it last (k - 2) is done
    auto upload = [&](int k) {
        const int b = k & 1;
        if (k >= 2) BCSIM_CUDA(cudaStreamWaitEvent(up, ev_consumed_[b].e, 0));
        BCSIM_CUDA(cudaMemcpyAsync(frame_raw_[b].get(), cps_frames[k], raw_bytes, cudaMemcpyHostToDevice, up));
        BCSIM_CUDA(launch_spline_transpose(frame_raw_[b].as<float>(), n, num_cs, frame_cps_[b].as<float4>(), up));
        BCSIM_CUDA(cudaMemcpyAsync(frame_amps_[b].get(), amps_frames[k], amp_bytes, cudaMemcpyHostToDevice, up));
        BCSIM_CUDA(abs_sum_enqueue(frame_amps_[b].as<float>(), 1, n, frame_scratch_[b].get(),
                                   &frame_bounds_.p->sum[b], &frame_bounds_.p->nonfinite[b], up));
        BCSIM_CUDA(cudaEventRecord(ev_uploaded_[b].e, up));
    };
    // one spline dataset of the frames' shape in place of the spline datasets
    splines_.clear();
    {
        SplineDataset ds;
        ds.degree = degree;
        ds.num_cs = num_cs;
        ds.knots.assign(knots, knots + num_knots);
        ds.n = n;
        splines_.push_back(std::move(ds));
    }
    // a non-finite amplitude stays reported as after the per-frame calls (only
    // clearing the fixed datasets resets it)
    const bool base_nonfinite = amplitude_nonfinite_;
    cfg_version_++;
    data_version_++;
    // afterwards (or on an error) the frame last installed is the spline dataset
    int installed = -1;
    auto settle = [&]() {
        cudaStreamSynchronize(up);
        cudaStreamSynchronize(copy_stream_.s);
        cudaStreamSynchronize(side_stream_.s);
        cudaStreamSynchronize(stream_);
        SplineDataset& ds = splines_[0];
        if (installed >= 0) {
            std::swap(ds.cps, frame_cps_[installed & 1]);
            std::swap(ds.amps, frame_amps_[installed & 1]);
        }
        ds.cps_src = nullptr;
        ds.amps_src = nullptr;
        if (installed < 0) splines_.clear();   // nothing was installed: no spline dataset
    };
    try {
        upload(0);
        for (int k = 0; k < num_frames; k++) {
            const int b = k & 1;
            if (k + 1 < num_frames) upload(k + 1);
            BCSIM_CUDA(cudaEventSynchronize(ev_uploaded_[b].e));   // frame k's amplitude bound
            SplineDataset& ds = splines_[0];
            ds.cps_src = frame_cps_[b].as<float4>();
            ds.amps_src = frame_amps_[b].as<float>();
            ds.sum_abs_amp = frame_bounds_.p->sum[b];
            amplitude_nonfinite_ = base_nonfinite || frame_bounds_.p->nonfinite[b] != 0;
            installed = k;
            cfg_version_++;
            data_version_++;
            prepare();   // a new frame of the same shape: the fixed-point scale
            BCSIM_CUDA(cudaStreamWaitEvent(stream_, ev_uploaded_[b].e, 0));
            // two device outputs: frame k + 1 runs while frame k's IQ is copied out
            if (k >= 2) BCSIM_CUDA(cudaStreamWaitEvent(stream_, ev_out_free_[b].e, 0));
            enqueue(stream_, frame_out_[b].as<float2>(), false, outs[k], false);
            BCSIM_CUDA(cudaEventRecord(ev_consumed_[b].e, stream_));
            BCSIM_CUDA(cudaEventRecord(ev_out_free_[b].e, copy_stream_.s));
        }
        BCSIM_CUDA(cudaStreamWaitEvent(stream_, ev_copied_.e, 0));   // the last frame's copies
        if (!flag_host_.p) BCSIM_CUDA(cudaMallocHost(&flag_host_.p, sizeof(int)));
        BCSIM_CUDA(enqueue_error_flag_read(err_flag_dev_.as<int>(), flag_host_.p, stream_));
    } catch (...) {
        settle();
        throw;
    }
    settle();
    if (*flag_host_.p) check_device_flag();
}

void Simulator::simulate_device(void* dev_out, int64_t cap_complex) {
    throw_if_not_configured();
    int64_t L = 0, nd = 0;
    output_shape(&L, &nd);
    if (!dev_out || cap_complex < L * nd)
        throw SimError(BCSIM_E_CAPACITY, "output buffer too small: need " + std::to_string(L * nd) + " complex values");
    simulate(static_cast<float2*>(dev_out), nullptr);
}

void Simulator::simulate_packet(int P, float prt, float2* dev_out, int64_t cap_complex) {
    throw_if_not_configured();
    if (P < 1) throw SimError(BCSIM_E_INVALID, "packet size must be at least 1");
    int64_t L = 0, nd = 0;
    output_shape(&L, &nd);
    const int64_t frame = L * nd;
    if (!dev_out || cap_complex < (int64_t)P * frame)
        throw SimError(BCSIM_E_CAPACITY, "output buffer too small: need " + std::to_string((int64_t)P * frame) +
                                              " complex values");
    ensure_device();
    if (splines_.empty()) {
        // fixed scatterers do not move: every frame of the packet is the same
        simulate(dev_out, nullptr);
        for (int k = 1; k < P; k++)
            BCSIM_CUDA(cudaMemcpyAsync(dev_out + k * frame, dev_out, (size_t)frame * sizeof(float2),
                                       cudaMemcpyDeviceToDevice, stream_));
    } else {
        std::vector<float> o((size_t)3 * L), d((size_t)3 * L), l((size_t)3 * L);
        for (int64_t i = 0; i < L; i++)
            for (int c = 0; c < 3; c++) {
                o[3 * i + c] = lines_[i].o[c];
                d[3 * i + c] = lines_[i].d[c];
                l[3 * i + c] = lines_[i].l[c];
            }
        const std::vector<float> t0 = timestamps_;
        const float len = line_length_;
        std::vector<float> t(t0.size());
        try {
            for (int k = 0; k < P; k++) {
                // scanline.get_timestamp() + packet_no * color_prt, in float
                for (size_t i = 0; i < t.size(); i++) t[i] = t0[i] + (float)k * prt;
                set_scan_sequence(o.data(), d.data(), l.data(), t.data(), (int)L, len);
                simulate(dev_out + k * frame, nullptr);
            }
        } catch (...) {
            set_scan_sequence(o.data(), d.data(), l.data(), t0.data(), (int)L, len);
            throw;
        }
        set_scan_sequence(o.data(), d.data(), l.data(), t0.data(), (int)L, len);
    }
    check_device_flag();
}

void Simulator::clone_from(Simulator& o) {
    o.ensure_device();
    ensure_device();
    verbose_ = o.verbose_;
    sound_speed_ = o.sound_speed_;
    noise_amplitude_ = o.noise_amplitude_;
    noise_seed_ = o.noise_seed_;
    noise_frame_ = 0;
    arc_ = o.arc_;
    decimation_ = o.decimation_;
    phase_delay_ = o.phase_delay_;
    cuda_streams_ = o.cuda_streams_;
    threads_per_block_ = o.threads_per_block_;
    mode_ = o.mode_;
    fir_tail_ = o.fir_tail_;
    convolution_ = o.convolution_;
    tile_lines_ = o.tile_lines_;
    cull_ = o.cull_;
    render_once_ = o.render_once_;
    record_cache_ = o.record_cache_;
    autotune_ = o.autotune_;
    wide_cta_ = o.wide_cta_;
    lut_smem_ = o.lut_smem_;
    excitation_set_ = o.excitation_set_;
    taps_ = o.taps_;
    center_ = o.center_;
    fs_ = o.fs_;
    fd_ = o.fd_;
    beam_type_ = o.beam_type_;
    sigma_l_ = o.sigma_l_;
    sigma_e_ = o.sigma_e_;
    lut_ = o.lut_;
    lut_nr_ = o.lut_nr_; lut_nl_ = o.lut_nl_; lut_ne_ = o.lut_ne_;
    for (int i = 0; i < 6; i++) lut_ext_[i] = o.lut_ext_[i];
    lut_absmax_ = o.lut_absmax_;
    lut_uploaded_ = false;
    fixed_n_ = o.fixed_n_;
    num_fixed_sets_ = o.num_fixed_sets_;
    fixed_sum_abs_ = o.fixed_sum_abs_;
    amplitude_nonfinite_ = o.amplitude_nonfinite_;
    if (fixed_n_ > 0) {
        fixed_xyza_.reserve((size_t)fixed_n_ * sizeof(float4), stream_);
        BCSIM_CUDA(cudaMemcpyAsync(fixed_xyza_.get(), o.fixed_xyza_.get(), (size_t)fixed_n_ * sizeof(float4),
                                   cudaMemcpyDeviceToDevice, stream_));
    }
    splines_.clear();
    for (const SplineDataset& src : o.splines_) {
        SplineDataset ds;
        ds.degree = src.degree;
        ds.num_cs = src.num_cs;
        ds.knots = src.knots;
        ds.n = src.n;
        ds.sum_abs_amp = src.sum_abs_amp;
        if (src.n > 0 && src.num_cs > 0) {
            ds.cps.reserve((size_t)src.num_cs * src.n * sizeof(float4), stream_);
            BCSIM_CUDA(cudaMemcpyAsync(ds.cps.get(), src.cps.get(), (size_t)src.num_cs * src.n * sizeof(float4),
                                       cudaMemcpyDeviceToDevice, stream_));
        }
        if (src.n > 0) {
            ds.amps.reserve((size_t)src.n * sizeof(float), stream_);
            BCSIM_CUDA(cudaMemcpyAsync(ds.amps.get(), src.amps.get(), (size_t)src.n * sizeof(float),
                                       cudaMemcpyDeviceToDevice, stream_));
        }
        splines_.push_back(std::move(ds));
    }
    BCSIM_CUDA(cudaStreamSynchronize(stream_));
    scan_set_ = false;
    tables_valid_ = false;
    lines_valid_ = false;
    cfg_version_++;
    static_version_++;
    data_version_++;
}

int64_t Simulator::samples_for(float line_length) const { return num_rf_samples(sound_speed_, line_length, fs_); }

size_t Simulator::footprint_bytes(int num_lines, int64_t ns_req) const {
    size_t n_all = (size_t)fixed_n_;
    size_t b = (size_t)fixed_n_ * sizeof(float4);
    for (const auto& d : splines_) {
        b += (size_t)d.num_cs * d.n * sizeof(float4) + (size_t)d.n * sizeof(float);
        n_all += d.n;
    }
    b += n_all * (4 * sizeof(uint32_t) + 4 * sizeof(float4));        // sort keys/values, records
    const size_t ns = (size_t)std::max<int64_t>(ns_req, 1);
    b += (size_t)num_lines * ns * 2 * sizeof(unsigned long long);    // bins
    b += (size_t)num_lines * ns * sizeof(float2);                    // output (upper bound)
    b += (size_t)lut_.size() * sizeof(float4);
    return b;
}

}  // namespace bcsim_gb300
