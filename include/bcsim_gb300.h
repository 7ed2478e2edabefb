/*
 * bcsim_gb300.h -- C ABI of the GB300 COLE ultrasound line simulator.
 *
 * This is the drop-in boundary for the reference's algorithm interface
 * bcsim::IAlgorithm (src/core/LibBCSim.hpp:42-91) and its factory
 * bcsim::Create (src/core/LibBCSim.cpp:39-49), flattened to plain pointers and
 * sizes so that any FFI (ctypes, cgo, JNI, N-API) or the C++ IAlgorithm adapter
 * (openbcsim_gb300/adapter/GB300Algorithm.hpp) can bind it.  Each function cites the reference member it
 * replaces.
 *
 * Conventions
 *   - Every function returns an int status: BCSIM_OK (0) or a BCSIM_E_* code.
 *     No C++ exception crosses this boundary.  The message of the last failure
 *     on a handle (the text the reference would have put in its
 *     std::runtime_error) is returned by bcsim_last_error().
 *   - Inputs are copied by the callee before the call returns (the semantics of
 *     the reference GPU algorithm, src/core/algorithm/GpuScatterers.cpp:42-46);
 *     the caller keeps ownership of every pointer it passes.
 *   - Vectors are float32 [n][3] row-major (x, y, z); IQ output is complex64
 *     stored as interleaved float pairs, line-major: out[line][sample][re, im].
 *   - One handle is not thread-safe (as the reference); distinct handles are.
 */
#ifndef BCSIM_GB300_H
#define BCSIM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BCSIM_OK              0
#define BCSIM_E_INVALID       1   /* bad argument or configuration (std::runtime_error) */
#define BCSIM_E_NOT_CONFIGURED 2  /* simulate_lines before configuration            */
#define BCSIM_E_CUDA          3   /* CUDA runtime failure                            */
#define BCSIM_E_CAPACITY      4   /* caller buffer too small                         */
#define BCSIM_E_MEMORY        5   /* device/host allocation refused                  */
#define BCSIM_E_INTERNAL      6   /* internal invariant (std::logic_error)           */
#define BCSIM_E_PENDING       7   /* request not finished within the wait timeout    */

typedef struct bcsim_handle bcsim_handle;

/* bcsim::Create(sim_type)  (src/core/LibBCSim.cpp:39-49).  Accepted type: "gpu".
 * Any other string fails with "Illegal algorithm type: <type>". */
int bcsim_create(const char* sim_type, bcsim_handle** out);

/* IAlgorithm destructor. */
int bcsim_destroy(bcsim_handle* h);

/* Message of the last failed call on h ("" if none).  Valid until the next call on h.
 * With h == NULL: the message of the calling thread's last failed bcsim_create. */
const char* bcsim_last_error(const bcsim_handle* h);

/* IAlgorithm::set_parameter (src/core/LibBCSim.hpp:51; keys of
 * src/core/algorithm/BaseAlgorithm.cpp:48-87 and GpuAlgorithm.cpp:68-107):
 *   verbose, sound_speed, noise_amplitude, use_arc_projection, radial_decimation,
 *   phase_delay, gpu_device, cuda_streams, threads_per_block, store_kernel_details,
 * plus this engine's own keys:
 *   precision_mode ("fp64" | "reference"), fir_tail_energy, convolution ("auto" | "fir" | "fft"),
 *   tile_lines, autotune, cull, record_cache, render_once (splines at one shared
 *   timestamp and origin rendered once, the reference's GpuAlgorithm.cpp:181-187). */
int bcsim_set_parameter(bcsim_handle* h, const char* key, const char* value);

/* IAlgorithm::get_parameter (GpuAlgorithm.cpp:761-773): num_cuda_devices,
 * cur_device_name, and the value of any settable key.  Writes a NUL-terminated
 * string of at most cap bytes. */
int bcsim_get_parameter(const bcsim_handle* h, const char* key, char* buf, int cap);

/* IAlgorithm::set_excitation (LibBCSim.hpp:72; ExcitationSignal BCSimConfig.hpp:79-92). */
int bcsim_set_excitation(bcsim_handle* h, const float* samples, int num_samples, int center_index,
                         float sampling_frequency, float demod_freq);

/* IAlgorithm::set_scan_sequence (LibBCSim.hpp:69) with the Scanline checks of
 * src/core/ScanSequence.cpp:37-70 applied to every line (elevational direction =
 * lateral x direction, orthonormal to 1e-4).  origins/directions/lateral_dirs:
 * float [num_lines][3]; timestamps: float [num_lines]. */
int bcsim_set_scan_sequence(bcsim_handle* h, const float* origins, const float* directions,
                            const float* lateral_dirs, const float* timestamps, int num_lines,
                            float line_length);

/* IAlgorithm::set_analytical_profile with a GaussianBeamProfile
 * (LibBCSim.hpp:75; BeamProfile.hpp:52-84). */
int bcsim_set_analytical_profile(bcsim_handle* h, float sigma_lateral, float sigma_elevational);

/* IAlgorithm::set_lookup_profile with a LUTBeamProfile (LibBCSim.hpp:78;
 * BeamProfile.hpp:88-142).  samples: float [nr][nl][ne] row-major
 * (radial, lateral, elevational); extents are the first and last sample positions. */
int bcsim_set_lookup_profile(bcsim_handle* h, const float* samples, int nr, int nl, int ne,
                             float r_first, float r_last, float l_first, float l_last,
                             float e_first, float e_last);

/* IAlgorithm::clear_fixed_scatterers / add_fixed_scatterers (LibBCSim.hpp:57-60).
 * xyza: float [n][4] = (x, y, z, amplitude), the row layout of the reference's
 * Python binding (src/python/PythonInterface.cpp:84-101). */
int bcsim_clear_fixed_scatterers(bcsim_handle* h);
int bcsim_add_fixed_scatterers(bcsim_handle* h, const float* xyza, int64_t n);
/* clear_fixed_scatterers + add_fixed_scatterers in one call. */
int bcsim_set_fixed_scatterers(bcsim_handle* h, const float* xyza, int64_t n);

/* IAlgorithm::clear_spline_scatterers / add_spline_scatterers (LibBCSim.hpp:63-66;
 * SplineScatterers BCSimConfig.hpp:126-165).  knots: float [num_knots] with
 * num_knots = num_cs + degree + 1; control_points: float [n][num_cs][3];
 * amplitudes: float [n]. */
int bcsim_clear_spline_scatterers(bcsim_handle* h);
int bcsim_add_spline_scatterers(bcsim_handle* h, int degree, const float* knots, int num_knots,
                                const float* control_points, const float* amplitudes, int64_t n,
                                int num_cs);
/* clear_spline_scatterers + add_spline_scatterers in one call. */
int bcsim_set_spline_scatterers(bcsim_handle* h, int degree, const float* knots, int num_knots,
                                const float* control_points, const float* amplitudes, int64_t n,
                                int num_cs);

/* IAlgorithm::get_total_num_scatterers (LibBCSim.hpp:87). */
int bcsim_get_total_num_scatterers(const bcsim_handle* h, int64_t* out);

/* Shape of the IQ output of the current configuration: num_lines lines of
 * num_samples = ceil(ns / radial_decimation) complex samples, where
 * ns = floor(fs * 2 * line_length / sound_speed + 0.5) (common_utils.hpp:38-41). */
int bcsim_get_output_shape(const bcsim_handle* h, int64_t* num_lines, int64_t* num_samples);

/* IAlgorithm::simulate_lines (LibBCSim.hpp:81).  out: host buffer of
 * cap_complex complex64 values, filled as out[line][sample]; the shape is
 * returned in num_lines / num_samples.  Blocks until the IQ is on the host. */
int bcsim_simulate_lines(bcsim_handle* h, float* out, int64_t cap_complex,
                         int64_t* num_lines, int64_t* num_samples);

/* A stream of frames of fixed scatterers (beside IAlgorithm: the reference's
 * per-frame clear_fixed_scatterers + add_fixed_scatterers + simulate_lines,
 * LibBCSim.hpp:57-60,81, in one call).  Frame k, xyza_frames[k] (float [n][4]),
 * replaces the fixed datasets and is simulated into iq_out_frames[k] (host,
 * cap_complex complex64 values, [num_lines][num_samples]) -- bit for bit what
 * those three calls per frame give.  Frame k+1 is uploaded (and its amplitude
 * bound reduced) on a stream of its own while frame k is simulated; pinned host
 * frames let the copies overlap.  Blocks until every frame's IQ is on the host;
 * the last frame stays the fixed dataset.  An error stops at the failing frame
 * (which then is the fixed dataset). */
int bcsim_simulate_fixed_frames(bcsim_handle* h, const float* const* xyza_frames, int64_t n, int num_frames,
                                float* const* iq_out_frames, int64_t cap_complex);

/* A stream of spline frames (beside IAlgorithm: the reference's per-frame
 * clear_spline_scatterers + add_spline_scatterers + simulate_lines,
 * LibBCSim.hpp:63-70,81, in one call).  Every frame has the given degree and
 * knots (num_knots = num_cs + degree + 1); frame k's control points
 * cps_frames[k] (float [n][num_cs][3]) and amplitudes amps_frames[k] (float
 * [n]) replace the spline datasets and frame k is simulated into
 * iq_out_frames[k] (host, cap_complex complex64 values,
 * [num_lines][num_samples]) -- bit for bit what those three calls per frame
 * give.  Frame k+1 is uploaded, laid out and its amplitude bound reduced on a
 * stream of its own while frame k is simulated; pinned host frames let the
 * copies overlap.  Blocks until every frame's IQ is on the host; the last
 * frame stays the spline dataset.  An error stops at the failing frame (which
 * then is the spline dataset). */
int bcsim_simulate_spline_frames(bcsim_handle* h, int degree, const float* knots, int num_knots,
                                 const float* const* cps_frames, const float* const* amps_frames, int64_t n,
                                 int num_cs, int num_frames, float* const* iq_out_frames, int64_t cap_complex);

/* simulate_lines into a device buffer (complex64 [num_lines][num_samples], at
 * least 16-byte aligned) on the handle's stream, without a host copy and
 * without synchronising.  For callers that keep the IQ on the GPU. */
int bcsim_simulate_lines_device(bcsim_handle* h, void* device_out, int64_t cap_complex);

/* The CUDA stream (a cudaStream_t) all work of h is issued on. */
int bcsim_get_stream(const bcsim_handle* h, void** stream);

/* IAlgorithm::get_debug_data (LibBCSim.hpp:84; keys of GpuAlgorithm.cpp:196-358
 * when store_kernel_details is on: kernel_memset_ms, fixed_projection_kernel_ms,
 * spline_projection_kernel_ms, kernel_convolve_demodulate_ms, kernel_memcpy_ms,
 * plus prep_sort_ms, total_ms).  Writes up to cap doubles; *n receives the count. */
int bcsim_get_debug_data(const bcsim_handle* h, const char* key, double* out, int64_t cap, int64_t* n);

/* IAlgorithm::set_logger (LibBCSim.hpp:90): fn(level, message, user) receives the
 * messages the reference writes to its ILog (levels 0 DEBUG, 1 INFO, 2 WARNING,
 * 3 FATAL).  fn = NULL restores the silent default (DummyLog). */
typedef void (*bcsim_log_fn)(int level, const char* message, void* user);
int bcsim_set_logger(bcsim_handle* h, bcsim_log_fn fn, void* user);

/* Fault injection for tests (no counterpart in the reference).  The engine's
 * kernels wait for their asynchronous copies with bounded waits; one that gives
 * up sets the handle's device error flag and returns, and the next call that
 * synchronises with the result (bcsim_simulate_lines, the frames, packet and
 * imaging calls, a batch run) fails with BCSIM_E_INTERNAL ("a bounded device
 * wait gave up; results are incomplete") and clears the flag.  This sets the
 * flag from the host, as such a wait would, so that the error path can be
 * tested without any device fault. */
int bcsim_debug_raise_wait_flag(bcsim_handle* h);

/* ---------------------------------------------------------------------------
 * Batched simulation (the reference has none: its GPU algorithm runs one
 * simulation per simulate_lines call, one line at a time, GpuAlgorithm.cpp:189-265).
 * A batch groups configured handles; running it prepares every handle, then
 * submits all of their device work at once, each handle on its own stream, and
 * from the second unchanged run on replays that submission as one captured CUDA
 * graph.  Results are identical to each handle's own bcsim_simulate_lines.
 * ------------------------------------------------------------------------- */
typedef struct bcsim_batch bcsim_batch;
int bcsim_batch_create(bcsim_handle* const* handles, int count, int use_graph, bcsim_batch** out);
int bcsim_batch_destroy(bcsim_batch* b);
const char* bcsim_batch_last_error(const bcsim_batch* b);
/* Run all jobs; host_outs[i] (may be NULL) receives job i's IQ (caps[i] complex
 * values), as bcsim_simulate_lines would.  Blocks until done. */
int bcsim_batch_run(bcsim_batch* b, float* const* host_outs, const int64_t* caps);
/* Run all jobs into device buffers without waiting; *stream (if not NULL)
 * receives the stream that completes when every job is done. */
int bcsim_batch_run_device(bcsim_batch* b, void* const* device_outs, const int64_t* caps, void** stream);

/* ---------------------------------------------------------------------------
 * Request server (no counterpart in the reference, whose callers run one
 * simulate_lines at a time, e.g. src/qt5gui/MainWindow.cpp:656-735).
 * Phantoms -- configured handles: parameters, excitation, beam, scatterers --
 * are copied once and stay resident on the device.  Each request asks for
 * scan lines of one phantom.  A worker thread admits requests strictly in
 * arrival order while fewer than max_in_flight (default 3) are on the GPU and a
 * simulator slot of their phantom is free -- up to max_slots_per_phantom slots
 * while the device-memory budget allows, the first ones made and prepared when
 * the phantom is added -- and runs admitted requests concurrently on separate
 * streams (continuous batching: the host prepares the next request while the
 * GPU runs the current ones).  A request's IQ is identical to
 * bcsim_simulate_lines of its phantom with its lines, whatever else is in
 * flight.
 * ------------------------------------------------------------------------- */
typedef struct bcsim_server bcsim_server;
int bcsim_server_create(int64_t hbm_budget_bytes, int max_slots_per_phantom, bcsim_server** out);
int bcsim_server_destroy(bcsim_server* s);
const char* bcsim_server_last_error(const bcsim_server* s);
/* Requests on the GPU at once (>= 1; default 3). */
int bcsim_server_set_max_in_flight(bcsim_server* s, int max_in_flight);
/* Copies the configuration and scatterers of a configured handle; *phantom_id
 * identifies it in requests.  The handle stays the caller's. */
int bcsim_server_add_phantom(bcsim_server* s, bcsim_handle* configured, int* phantom_id);
/* Queues a request; returns at once with its id. */
int bcsim_server_submit(bcsim_server* s, int phantom_id, const float* origins, const float* directions,
                        const float* lateral_dirs, const float* timestamps, int num_lines, float line_length,
                        int radial_decimation, int64_t* request_id);
/* Waits up to timeout_ms (-1: no limit) for a request; BCSIM_E_PENDING if not
 * done.  On success copies the IQ (complex64 [num_lines][num_samples]) into out
 * and releases the request; latency_ms = submit to result on the host. */
int bcsim_server_wait(bcsim_server* s, int64_t request_id, float* out, int64_t cap_complex, int64_t* num_lines,
                      int64_t* num_samples, double* latency_ms, int timeout_ms);
/* Admission by device memory: a request is admitted when a slot of its
 * phantom is free (or can be made within the budget) and the device memory its
 * slot has to grow by is available (free device memory plus the stream-ordered
 * pool's reserved-but-unused bytes, less 256 MiB).  A request that does not fit
 * waits while others are in flight; one that cannot fit with nothing in flight,
 * or whose footprint exceeds hbm_budget_bytes, fails with BCSIM_E_MEMORY.  A
 * request whose scan or timestamps are invalid fails with the reference's
 * message; the others are unaffected. */
/* Counters: completed and failed requests, latency percentiles over completed
 * requests, projections done, device bytes held by slots, queued requests. */
int bcsim_server_stats(bcsim_server* s, int64_t* completed, int64_t* failed, double* p50_ms, double* p99_ms,
                       int64_t* projections, int64_t* hbm_in_use, int64_t* queue_depth);
/* Fault injection for tests, all on the host: WAIT_FLAG raises the device
 * error flag of the next admitted request's slot (as a bounded wait that gave
 * up would: that request fails with BCSIM_E_INTERNAL); WORKER_THROW makes the
 * worker's next dispatch throw (that request fails with BCSIM_E_INTERNAL,
 * "injected worker failure"); FREE_MEMORY_CAP caps the device memory that
 * admission sees at `value` bytes (value < 0 removes the cap). */
#define BCSIM_SERVER_INJECT_WAIT_FLAG 1
#define BCSIM_SERVER_INJECT_WORKER_THROW 2
#define BCSIM_SERVER_INJECT_FREE_MEMORY_CAP 3
int bcsim_server_debug_inject(bcsim_server* s, int what, int64_t value);

/* Allocation-free simulation (no counterpart in the reference).
 *
 * For callers that cannot allocate GPU memory -- pipelines that reserve all
 * device memory once at start-up, processes whose device memory belongs to
 * another framework's pool -- this one call simulates fixed scatterers with an
 * analytic Gaussian beam without allocating anything on the device: the caller
 * passes the scatterers d_xyza (device, float4 [n] = x, y, z, amplitude) and the
 * output d_out (device, complex64 [num_lines][ceil(ns / radial_decimation)]);
 * the scan lines and excitation are host arrays as in bcsim_set_scan_sequence /
 * bcsim_set_excitation.  All intermediates live in one static device array of
 * about 31.3 MiB that every GPU loading this library holds until exit.  Limits:
 * num_lines <= 4096, num_lines * ns * (phase_delay ? 2 : 1) <= 3932160,
 * ns + num_samples - 1 <= 65536.  amplitude_sum_bound must bound sum |a|
 * (it sets the fixed-point scale of the bins): a bound below the measured sum
 * fails the call, and so does a non-finite amplitude ("Nan in scatterer
 * projection."), both before anything is written.  d_xyza and d_out must be
 * device (or managed) memory of the current device.  The first call on each
 * device looks up the static array's address (make it before any stream
 * capture).  Calls share the array: calls that overlap on the GPU race, so
 * issue them on one stream.  The call is synchronous: it returns once the IQ
 * is in d_out.  On failure a message is written to err (err_cap bytes). */
int bcsim_simulate_fixed_noalloc(const void* d_xyza, int64_t n, const float* origins, const float* directions,
                                 const float* lateral_dirs, int num_lines, float line_length, float sound_speed,
                                 const float* samples, int num_samples, int center_index, float sampling_frequency,
                                 float demod_freq, float sigma_lateral, float sigma_elevational,
                                 int use_arc_projection, int phase_delay, int radial_decimation,
                                 float amplitude_sum_bound, void* d_out, int64_t cap_complex, void* stream,
                                 char* err, int err_cap);

/* ---- Post-processing on the device: B-mode and colour Doppler ------------
 *
 * The reference forms images on the host after simulate_lines, in its GUI's
 * refresh worker (src/qt5gui/RefreshWorker.hpp:179-395) with
 * bcsim::get_max_value / log_compress_frame (src/utils/BCSimConvenience.cpp:57-83)
 * and CpuCartesianator (src/utils/cartesianator/Cartesianator.cpp:107-205).
 * These entry points run the same steps as kernels on the handle's stream.
 * Layouts: IQ complex64 [num_lines][num_samples] (a packet: [frames][lines]
 * [samples]); beam space [beam][range]; images [ny][nx], x fastest; colour
 * pixels 4 bytes (blue, green, red, alpha). */
#define BCSIM_GEOMETRY_SECTOR 0
#define BCSIM_GEOMETRY_LINEAR 1

/* bcsim::SectorScanGeometry / LinearScanGeometry (src/utils/ScanGeometry.hpp:44-78)
 * plus the Cartesianator's output size. */
typedef struct {
    int kind;     /* BCSIM_GEOMETRY_SECTOR or BCSIM_GEOMETRY_LINEAR      */
    float width;  /* sector: opening angle [rad]; linear: width [m]     */
    float depth;  /* sector: depth [m]; linear: maximum range [m]       */
    float tilt;   /* sector: tilt [rad]; linear: unused                 */
    int nx, ny;   /* output image size [pixels], each >= 2              */
} bcsim_scan_geometry;

/* B-mode of one IQ frame (host iq): envelope |iq|; normalisation by
 * `normalize` (<= 0: the frame's largest envelope, as the worker's
 * auto-normalisation); 20 log10(gain * env / normalize) mapped by dyn_range
 * [dB] to [0, 255], clamped, truncated to bytes; scan conversion by
 * `geometry` into image [ny][nx] (geometry and image may be NULL: beam space
 * only).  beamspace ([num_lines][num_samples] bytes) and normalize_used may
 * be NULL. */
int bcsim_bmode_image(bcsim_handle* h, const float* iq, int64_t num_lines, int64_t num_samples, float dyn_range,
                      float gain, float normalize, const bcsim_scan_geometry* geometry, uint8_t* image,
                      uint8_t* beamspace, float* normalize_used);
/* The same from a configured simulator: simulate_lines, then the B-mode, the
 * IQ staying on the device. */
int bcsim_simulate_bmode(bcsim_handle* h, float dyn_range, float gain, float normalize,
                         const bcsim_scan_geometry* geometry, uint8_t* image, uint8_t* beamspace,
                         float* normalize_used);
/* Scan conversion of a float beam space [num_beams][num_range] into image [ny][nx]. */
int bcsim_scan_convert(bcsim_handle* h, const float* beamspace, int64_t num_beams, int64_t num_range,
                       const bcsim_scan_geometry* geometry, float* image);
/* A colour-Doppler packet (src/qt5gui/MainWindow.cpp:664-694): packet_size
 * frames of the configured scan, frame k with every timestamp advanced by
 * k * prt; out complex64 [packet_size][num_lines][num_samples].  The scan
 * sequence is left as configured. */
int bcsim_simulate_packet(bcsim_handle* h, int packet_size, float prt, float* out, int64_t cap_complex);
/* Autocorrelation estimates of a packet (host iq_packet, packet_size >= 2):
 * per sample R0 = sum |x_k - mean|^2 and velocity = arg sum conj(x_k) x_(k+1)
 * (RefreshWorker.hpp:262-300) into r0 / velocity ([num_lines][num_samples],
 * either may be NULL); with a geometry, the colour image (power threshold
 * 0.001 of the largest R0; red for velocity >= 0, blue below) into bgra
 * [ny][nx][4]. */
int bcsim_color_doppler(bcsim_handle* h, const float* iq_packet, int packet_size, int64_t num_lines,
                        int64_t num_samples, float* r0, float* velocity, const bcsim_scan_geometry* geometry,
                        uint8_t* bgra);
/* The same from a configured simulator: the packet is simulated and estimated
 * on the device. */
int bcsim_simulate_color_doppler(bcsim_handle* h, int packet_size, float prt, float* r0, float* velocity,
                                 const bcsim_scan_geometry* geometry, uint8_t* bgra);

#ifdef __cplusplus
}
#endif
#endif /* BCSIM_GB300_H */
