// engine.hpp -- the GB300 COLE simulator behind the C ABI.
//
// One Simulator mirrors one bcsim::IAlgorithm instance of the reference GPU
// algorithm (src/core/algorithm/GpuAlgorithm.hpp:48-162): string parameters,
// excitation, scan sequence, beam profile and scatterer datasets are configured
// in any order the reference CPU algorithm accepts, scatterers are copied to the
// device when added and stay resident, and simulate_lines() runs the whole
// projection -> convolution -> demodulation -> decimation pipeline on one CUDA
// stream.
#pragma once
#include <cuda_runtime.h>

#include <complex>
#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "kernels.hpp"

namespace bcsim_gb300 {

// Failure carrying one of the BCSIM_E_* codes and the reference's message.
struct SimError : public std::runtime_error {
    int code;
    SimError(int c, const std::string& msg) : std::runtime_error(msg), code(c) {}
};

// Owning device allocation that only grows.  With a stream it is allocated and
// freed in that stream's order from the device's memory pool (no device-wide
// synchronisation, as cudaFree would cause: a simulator that serves requests
// of changing size never stalls the other streams); growth is geometric.
class DeviceBuffer {
public:
    DeviceBuffer() = default;
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    DeviceBuffer(DeviceBuffer&& o) noexcept : ptr_(o.ptr_), bytes_(o.bytes_), stream_(o.stream_) {
        o.ptr_ = nullptr;
        o.bytes_ = 0;
    }
    DeviceBuffer& operator=(DeviceBuffer&& o) noexcept;
    ~DeviceBuffer();
    void reserve(size_t bytes, cudaStream_t stream = nullptr);   // grow (contents not kept)
    void release();
    void* get() const { return ptr_; }
    template <typename T> T* as() const { return static_cast<T*>(ptr_); }
    size_t bytes() const { return bytes_; }

private:
    void* ptr_ = nullptr;
    size_t bytes_ = 0;
    cudaStream_t stream_ = nullptr;   // stream-ordered allocation on this stream (null: cudaMalloc)
};

// Pinned host landing places of the two in-flight frames' amplitude bounds.
struct FrameBounds {
    double sum[2];
    int nonfinite[2];
};
struct PinnedFrameBounds {
    FrameBounds* p = nullptr;
    PinnedFrameBounds() = default;
    PinnedFrameBounds(const PinnedFrameBounds&) = delete;
    PinnedFrameBounds& operator=(const PinnedFrameBounds&) = delete;
    ~PinnedFrameBounds() {
        if (p) cudaFreeHost(p);
    }
};

// Pinned host int (the error flag's landing place), freed with its owner.
struct PinnedInt {
    int* p = nullptr;
    PinnedInt() = default;
    PinnedInt(const PinnedInt&) = delete;
    PinnedInt& operator=(const PinnedInt&) = delete;
    ~PinnedInt() {
        if (p) cudaFreeHost(p);
    }
};

// A simulator's stream, destroyed (after its work) when the simulator goes --
// declared before the simulator's buffers, so that those are freed first, in
// its order.
struct OwnedStream {
    cudaStream_t s = nullptr;
    OwnedStream() = default;
    OwnedStream(const OwnedStream&) = delete;
    OwnedStream& operator=(const OwnedStream&) = delete;
    ~OwnedStream() {
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    }
};

struct SplineDataset {
    int degree = 0;
    int num_cs = 0;
    std::vector<float> knots;
    DeviceBuffer cps;      // float4 [num_cs][n] (x, y, z, 0)
    DeviceBuffer amps;     // float [n]
    int64_t n = 0;
    double sum_abs_amp = 0.0;
    // simulate_spline_frames: the current frame's buffers, read in place of the
    // owned ones while a stream of frames runs (not owned)
    const float4* cps_src = nullptr;
    const float* amps_src = nullptr;
    const float4* cps_dev() const { return cps_src ? cps_src : cps.as<float4>(); }
    const float* amps_dev() const { return amps_src ? amps_src : amps.as<float>(); }
};

typedef void (*LogFn)(int level, const char* message, void* user);

// One per-pair launch of a simulation: the fixed scatterers (kind 0) or spline
// dataset d (kind 1), with its line tiles and per-line basis.
struct GenLaunch {
    int kind;
    int d;
    size_t tile_off, num_tiles, basis_off;
    int threads;   // CTA size: the largest tile's line count rounded up to warps
};

// Host-side plan of one configuration: launch constants and shapes, built by
// prepare() and reused until the configuration changes.
struct Plan {
    uint64_t version = ~0ull;
    uint64_t static_version = ~0ull;   // configuration apart from scatterer values
    std::vector<double> data_shape;    // dataset sizes and spline knots it was built for
    SimParams p;
    BeamDev b;
    bool shared = false;
    int64_t n_shared = 0;
    std::vector<char> spline_shared;
    std::vector<int64_t> spline_off;
    std::vector<int> spline_first_cs;
    std::vector<GenLaunch> gl;
    bool tile_cull = false;   // per-pair tiles carry culling boxes
    size_t bins_bytes = 0;
    size_t sort_tmp_bytes = 0;
    int end_bit = 1;
    int chunk = 1024;
    uint64_t records_key = 0;
};

// The shared-origin records of one simulation: sort keys and values, the
// unsorted and the sorted record planes, the sort's scratch and the bin-range
// counts, and the key of the records they hold.
struct RecordSet {
    DeviceBuffer keys_in, vals_in, keys_out, vals_out, recA, recB, records, sort_tmp, counts;
    uint64_t key = 0;
};

// An event without timing, destroyed with its owner.
// A stage interval of a timed simulation (store_kernel_details): its start
// and end events, read after the simulation has finished.
struct PendingTiming {
    const char* key;
    cudaEvent_t a, b;
};

struct OwnedEvent {
    cudaEvent_t e = nullptr;
    OwnedEvent() = default;
    OwnedEvent(const OwnedEvent&) = delete;
    OwnedEvent& operator=(const OwnedEvent&) = delete;
    ~OwnedEvent() {
        if (e) cudaEventDestroy(e);
    }
};

class Simulator {
public:
    Simulator();
    ~Simulator();

    void set_parameter(const std::string& key, const std::string& value);
    std::string get_parameter(const std::string& key) const;
    void set_excitation(const float* samples, int n, int center_index, float fs, float demod_freq);
    void set_scan_sequence(const float* origins, const float* dirs, const float* lats, const float* timestamps,
                           int num_lines, float line_length);
    void set_analytical_profile(float sigma_lateral, float sigma_elevational);
    void set_lookup_profile(const float* samples, int nr, int nl, int ne, float r0, float r1, float l0, float l1,
                            float e0, float e1);
    void clear_fixed_scatterers();
    void add_fixed_scatterers(const float* xyza, int64_t n);
    void clear_spline_scatterers();
    void add_spline_scatterers(int degree, const float* knots, int num_knots, const float* cps, const float* amps,
                               int64_t n, int num_cs);
    int64_t total_num_scatterers() const;
    void output_shape(int64_t* lines, int64_t* samples) const;

    // Runs the pipeline into device memory dev_out (complex64 [L][nd]); if
    // host_out is given, also copies to it and synchronises.
    void simulate(float2* dev_out, float* host_out);
    // Host work of simulate_lines for the current configuration (cached).
    void prepare();
    // Device work of simulate_lines on stream st into dev_out: launches only,
    // no allocation, no synchronisation (can be graph-captured after
    // prepare()).  With host_out (pinned or pageable host memory), the
    // convolution runs in blocks of lines and each block's IQ is copied to
    // host_out on a copy stream while the next block is convolved; st then
    // waits for the copies unless wait_copies is false (ev_copied_ marks them).
    // staged: the bins (bins_[cur_]) are already cleared and the records
    // (rs_[cur_]) prepared, with st waiting for both (simulate_fixed_frames).
    void enqueue(cudaStream_t st, float2* dev_out, bool timing, float* host_out = nullptr, bool wait_copies = true,
                 bool staged = false);
    // Copy the whole configuration of o (parameters, excitation, beam, scatterer
    // datasets -- device copies; not the scan sequence) into this simulator.
    void clone_from(Simulator& o);
    // Take o's scan sequence (after clone_from, whose configuration it needs).
    void copy_scan_from(const Simulator& o);
    // Device bytes this simulator holds or will hold for num_lines lines of ns samples.
    size_t footprint_bytes(int num_lines, int64_t ns) const;
    // Samples per line this configuration gives for a line length.
    int64_t samples_for(float line_length) const;
    int64_t num_lines() const { return num_lines_; }
    int64_t num_out_samples() const { return nd_; }
    float2* internal_output() { return out_.as<float2>(); }
    uint64_t config_version() const { return cfg_version_; }
    // Seeded noise on: every simulation draws the next frame's noise (a
    // captured graph would replay one frame's).
    bool noisy() const { return noise_amplitude_ > 0.0f; }
    // Throws if a bounded device wait of this simulator's kernels gave up since
    // the last check (and clears the flag).
    void check_device_flag();
    // Test hook: sets the device error flag as a bounded wait that gave up
    // would (host-side injection; no kernel is involved).
    void raise_device_flag();
    // Copy of the device error flag into host_flag (pinned), in st's order.
    cudaError_t enqueue_flag_read(int* host_flag, cudaStream_t st) {
        return enqueue_error_flag_read(err_flag_dev_.as<int>(), host_flag, st);
    }
    void simulate_host(float* host_out, int64_t cap_complex, int64_t* lines, int64_t* samples);
    void simulate_device(void* dev_out, int64_t cap_complex);
    // A colour-Doppler packet (MainWindow.cpp:664-694): P frames of the scan,
    // frame k with every line's timestamp advanced by k * prt, into device
    // memory [P][L][nd].  The scan sequence is restored afterwards.
    void simulate_packet(int P, float prt, float2* dev_out, int64_t cap_complex);
    // A stream of frames of fixed scatterers: frame k (n scatterers, host
    // float4 xyza, replacing the fixed datasets) simulated into host IQ outs[k]
    // (cap_complex values each), as clear + add_fixed_scatterers +
    // simulate_lines per frame would, bit for bit.  Frame k+1's upload and
    // amplitude bound run on their own stream, and its bins clear and record
    // preparation on another, while frame k is simulated (bins and records
    // double-buffered).  Afterwards the last frame is the fixed dataset.
    void simulate_fixed_frames(const float* const* frames, int64_t n, int num_frames, float* const* outs,
                               int64_t cap_complex);
    // A stream of spline frames: frame k replaces the spline datasets with one of
    // the given degree and knots, control points cps_frames[k] ([n][num_cs][3])
    // and amplitudes amps_frames[k] ([n]), and is simulated into outs[k]; frame
    // k+1 is uploaded while frame k runs.  Bit for bit clear_spline_scatterers +
    // add_spline_scatterers + simulate per frame.
    void simulate_spline_frames(int degree, const float* knots, int num_knots, const float* const* cps_frames,
                                const float* const* amps_frames, int64_t n, int num_cs, int num_frames,
                                float* const* outs, int64_t cap_complex);

    std::vector<double> get_debug_data(const std::string& key) const;
    void set_logger(LogFn fn, void* user) { log_fn_ = fn; log_user_ = user; }
    cudaStream_t stream();

private:
    void log(int level, const std::string& msg) const;
    void ensure_device();
    void throw_if_not_configured() const;
    void prepare_excitation_tables();
    void prepare_lines();
    void autotune();
    double fixed_point_bound() const;
    void set_fixed_point_scale(SimParams& p) const;
    uint64_t records_key_of(const Plan& P) const;
    std::vector<double> data_shape() const;
    const float4* fixed_src() const { return fixed_src_ ? fixed_src_ : fixed_xyza_.as<float4>(); }
    RecordSet& rec() { return rs_[cur_]; }
    void reserve_records(RecordSet& R, Plan& P);
    // record preparation (prep, sort, counts, gather) into rec(), on st
    void enqueue_records(cudaStream_t st, int* launches);

    // configuration
    int device_ = 0;
    bool device_ready_ = false;
    OwnedStream owned_stream_;
    OwnedStream side_stream_;   // bins cleared here while the records are prepared
    OwnedStream copy_stream_;   // IQ copied to the host here while later lines are convolved
    OwnedStream upload_stream_;   // simulate_fixed_frames: the next frame's upload
    OwnedEvent ev_fork_, ev_join_, ev_copied_;
    OwnedStream prep_stream_;     // simulate_fixed_frames: the next frame's bins clear and records
    OwnedEvent ev_uploaded_[2], ev_consumed_[2];   // per frame buffer: upload done / last reader done
    OwnedEvent ev_staged_[2];   // a frame's bins cleared and records prepared
    std::vector<cudaEvent_t> ev_blocks_;   // one per convolution block (owned, see ~Simulator)
    PinnedInt flag_host_;
    DeviceBuffer err_flag_dev_;   // this simulator's device error flag (SimParams::err_flag)
    cudaStream_t stream_ = nullptr;   // owned_stream_.s
    int verbose_ = 0;
    float sound_speed_ = 1540.0f;
    float noise_amplitude_ = 0.0f;
    uint64_t noise_seed_ = 0;
    uint32_t noise_frame_ = 0;   // frame number of the next simulation's noise
    bool arc_ = true;
    int decimation_ = 1;
    bool phase_delay_ = false;
    int cuda_streams_ = 2;
    int threads_per_block_ = 128;
    bool store_details_ = false;
    int mode_ = MODE_FP64;
    double fir_tail_ = 1e-10;
    int convolution_ = 0;   // 0 = automatic, 1 = direct FIR, 2 = FFT
    int tile_lines_ = 0;   // 0 = automatic
    bool cull_ = true;     // exact culling of zero-weight (scatterer, line-slot) pairs
    // splines seen by every line at one time from one origin are rendered once
    // into shared-origin records (the reference's render at a common timestamp,
    // GpuAlgorithm.cpp:181-187); off: the per-pair path evaluates them per line
    bool render_once_ = true;
    bool record_cache_ = true;   // reuse the sorted shared-origin records while their inputs are unchanged
    bool autotune_ = false;
    bool autotuning_ = false;    // inside autotune(): its own re-plans do not tune again
    bool wide_cta_ = true;       // shared-origin kernel launch shape (see launch_project_shared)
    bool lut_smem_ = true;       // wide shared-origin kernel: stage the chunk's lookup-table planes in shared memory
    bool count_pairs_ = false;   // instrumented shared-origin kernel: visited / non-zero (record, line) pairs
    int last_launches_ = 0;      // kernels of this library launched by the last enqueue
    DeviceBuffer pair_counts_;
    DeviceBuffer ingest_scratch_;
    DeviceBuffer gen_boxes_;        // TileBox per per-pair tile   // amplitude reductions of add_*_scatterers
    uint64_t cfg_version_ = 1;   // bumped by every configuration change
    uint64_t static_version_ = 1;   // bumped by every change but new scatterer values
    uint64_t data_version_ = 1;  // bumped by every scatterer change
    Plan plan_;

    bool excitation_set_ = false;
    std::vector<float> taps_;
    int center_ = 0;
    float fs_ = 0.0f, fd_ = 0.0f;

    bool scan_set_ = false;
    int num_lines_ = 0;
    float line_length_ = 0.0f;
    int64_t ns_ = 0;
    std::vector<LineGeom> lines_;
    std::vector<float> timestamps_;
    bool shared_origin_ = false;
    bool timestamps_equal_ = false;

    int beam_type_ = 0;   // 0 = not configured
    float sigma_l_ = 0.0f, sigma_e_ = 0.0f;
    std::vector<float> lut_;
    int lut_nr_ = 0, lut_nl_ = 0, lut_ne_ = 0;
    float lut_ext_[6] = {0, 0, 0, 0, 0, 0};
    double lut_absmax_ = 0.0;
    DeviceBuffer lut4_;
    bool lut_uploaded_ = false;
    int lut_packed_mode_ = -1;   // precision mode the uploaded packing is for (pack_lut)

    // all fixed datasets, appended into one float4 [n] array (x, y, z, a)
    DeviceBuffer fixed_xyza_;
    DeviceBuffer frame_xyza_[2], frame_scratch_[2], frame_out_[2];   // simulate_fixed_frames' double buffers
    DeviceBuffer frame_raw_[2], frame_cps_[2], frame_amps_[2];       // simulate_spline_frames' double buffers
    OwnedEvent ev_out_free_[2];   // a frame output buffer's copy to the host done
    PinnedFrameBounds frame_bounds_;
    const float4* fixed_src_ = nullptr;   // the fixed scatterers the kernels read: fixed_xyza_ unless a frame's
    int64_t fixed_n_ = 0;
    int num_fixed_sets_ = 0;
    double fixed_sum_abs_ = 0.0;
    bool amplitude_nonfinite_ = false;
    std::vector<SplineDataset> splines_;

    // derived device state
    bool tables_valid_ = false;
    int64_t M_ = 0, nd_ = 0;
    int64_t tap_start_ = 0, tap_count_ = 0;
    std::vector<float> fir_key_taps_;   // inputs of the current FIR window
    int64_t fir_key_M_ = -1;
    double fir_key_tail_ = -1.0;
    DeviceBuffer demod_dev_, taps_pm_dev_, ph_off_dev_;
    std::vector<float2> fir_taps_host_;   // the FIR window taps, in window order
    std::vector<std::complex<double>> analytic_spec_;   // FFT_M(h) * hilbert mask, for the FFT route
    bool fft_ok_ = false;          // the FFT route (fftconv.cu) fits this configuration
    bool last_route_fft_ = false;  // the route the last simulation took
    bool route_known_ = false;
    int sms_ = 0;
    DeviceBuffer fft_spec_dev_, fft_tw_dev_;   // its tables, for fft_key_*
    std::vector<float> fft_key_taps_;
    int64_t fft_key_M_ = -1;
    int fft_key_center_ = -1;
    int ntaps_pm_ = 0, max_ph_taps_ = 0;
    bool lines_valid_ = false;
    DeviceBuffer lines_dev_, line_order_dev_, cones_dev_;
    std::vector<int> line_rank_;   // position of each line in the direction-ordered sequence
    // bins and records: set cur_ (the second set only for simulate_fixed_frames,
    // whose next frame is cleared and prepared while the current one runs)
    DeviceBuffer bins_[2], out_;
    RecordSet rs_[2];
    int cur_ = 0;
    DeviceBuffer gen_tiles_, gen_line_ids_, gen_basis_, spl_basis_d_, spl_basis_f_;
    std::vector<float> pinned_dummy_;

    std::map<std::string, std::vector<double>> debug_;
    std::vector<PendingTiming> pending_timings_;   // stage intervals recorded, not yet read
    void resolve_timings();
    void drop_timings();
    LogFn log_fn_ = nullptr;
    void* log_user_ = nullptr;
};

}  // namespace bcsim_gb300
