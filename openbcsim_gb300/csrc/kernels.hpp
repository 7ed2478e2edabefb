// kernels.hpp -- structures shared by the host engine and the CUDA kernels, and
// the host-side launchers of every kernel.
#pragma once
#include <complex>
#include <cstdint>
#include <cuda_runtime.h>

#include "noise.cuh"

namespace bcsim_gb300 {

// One scan line as the kernels see it: origin, radial, lateral and elevational
// unit vectors (elevational = lateral x radial, computed on the host in float as
// src/core/ScanSequence.cpp:40 does).
struct LineGeom {
    float o[3];
    float d[3];
    float l[3];
    float e[3];
};

enum BeamType : int { BEAM_GAUSSIAN = 1, BEAM_LUT = 2 };
enum PrecisionMode : int { MODE_FP64 = 0, MODE_REFERENCE = 1 };

// Beam profile constants.
struct BeamDev {
    int type;
    // Gaussian, fp64 mode: w = exp2(-(l^2 * gl + e^2 * ge)), gl = log2(e) / (2 sigma_l^2)
    float gl, ge;
    // Gaussian, reference mode: w = expf(-(l*l/two_sl2 + e*e/two_se2)) (BeamProfile.cpp:49-56)
    float two_sl2, two_se2;
    // Lookup table: packed corners (fp64 mode: with radial differences), see pack_lut() in engine.cpp
    const float4* lut4;
    int nr, nl, ne;
    float rf, lf, ef;          // first sample positions
    float inv_dr, inv_dl, inv_de;  // 1 / spacing (fp64 mode, per-pair coordinates)
    float inv_dr_lo;           // 1/dr - inv_dr: 1/dr as a float pair (fp64-mode record prep)
    double dr, dl, de;         // spacing as the mode defines it (double)
};

// Constants of one simulation.
struct SimParams {
    int ns;                    // time samples per line (before decimation)
    int num_lines;
    int phase_delay;
    int arc;
    int mode;                  // PrecisionMode
    float fs, c, fd;
    double fs_d, c_d, fd_d;
    float k_hi, k_lo;          // 2 fs / c as a float pair (fp64 generic path)
    float two_pi_fd_over_fs;   // phase per sample of sub-sample delay
    float scale;               // fixed-point scale 2^S for bin accumulation
    int log2scale;
    // exact culling in the shared-origin kernel: a line's weight is exactly 0
    // outside cull_l_lo < l < cull_l_hi, cull_e_lo < e < cull_e_hi
    int cull;
    float cull_l_lo, cull_l_hi, cull_e_lo, cull_e_hi;
    float cull_rho_per_bin;    // upper bound of 1 / (2 fs / c)
    int wide_cta;              // shared-origin kernel: 1024-thread CTAs for >= 512 lines
    int lut_smem;              // wide shared-origin kernel: lookup-table planes in shared memory
    int fold;                  // shared-origin kernel: FP32 run sums folded at record indices k*fold (power of 2)
    int cell_bits;             // shared-origin records: sort key = bin << cell_bits | angular cell of the direction
    int* err_flag;             // the simulator's device error flag: set to 1 when a bounded wait gives up (may be null)
};

// Frame spread of a slot of 32 lines (consecutive in the kernel's line order):
// a reference frame (lateral l, elevational e, radial r) and, for the
// differences dl = l_k - l and de = e_k - e of every line k of the slot, their
// largest component along r (du_par, dv_par) and largest part normal to r
// (du_perp, dv_perp), and the largest |r_k - r| (dd).  For a scatterer at
// offset A = t r + A_perp from the origin every line's lateral coordinate then
// lies within |t| du_par + |A_perp| du_perp of A.l (elevational alike), and
// every line's radial coordinate within |A| dd of A.r.
struct SlotCone {
    float lx, ly, lz, ex, ey, ez, rx, ry, rz;
    float du_par, du_perp, dv_par, dv_perp, dd;
};

// A tile of lines for the per-pair projection kernel: `count` lines taken from
// line_ids[first ...].  For splines the tile's lines need control points
// mu - degree .. mu - degree + span - 1 (the union of their windows; lines are
// sorted by knot interval, so a tile spans few intervals).
struct LineTile {
    int first;
    int count;
    int mu;     // smallest knot interval of the tile's lines
    int span;   // control points staged per scatterer
};

// Extent of a per-pair line tile for culling: a reference line (origin o,
// frame l, e, r), the frame spread of the tile's lines about it (as in
// SlotCone) and the largest distance of a tile line's origin from o.
struct TileBox {
    float ox, oy, oz;
    float lx, ly, lz, ex, ey, ez, rx, ry, rz;
    float du_par, du_perp, dv_par, dv_perp, d_orig;
};

// Lines per CTA of the per-pair kernel (the largest line tile).
constexpr int PAIR_THREADS = 128;

// Per-line spline basis: p+1 non-zero basis values as float pairs (hi, lo),
// starting at control point mu - degree.
constexpr int MAX_SPLINE_DEGREE = 7;
struct LineBasis {
    float hi[MAX_SPLINE_DEGREE + 1];
    float lo[MAX_SPLINE_DEGREE + 1];
    int mu;   // knot interval
};

// Shared-origin records, in bin order, as two planes of float4:
//   A = (dx, dy, dz, amplitude * cos(phase))   relative to the common origin
//   B = (amplitude * sin(phase), radial LUT fraction, radial LUT index bits, bin bits)

// ---------------------------------------------------------------------------
// launchers (all asynchronous on `stream`; return cudaGetLastError())
// ---------------------------------------------------------------------------

// Per scatterer, from a shared line origin: exact bin index (fp64 or reference
// arithmetic), phase-rotated amplitude and LUT radial coordinate.  Writes sort
// keys (bin index, or ns for near-origin scatterers that need the per-pair path,
// or ns+1 for scatterers that no line can see, shifted left by p.cell_bits above
// the angular cell of the scatterer's direction), identity values and the
// unsorted records.
cudaError_t launch_prep_shared(const float4* xyza, int64_t n, int64_t out_offset, const float origin[3],
                               const SimParams& p, const BeamDev& b, uint32_t* keys, uint32_t* vals,
                               float4* recA, float4* recB, cudaStream_t stream);

// Same, for spline scatterers evaluated at one common timestamp in double.
cudaError_t launch_prep_shared_spline(const float4* cps, const float* amps, int64_t n, int num_cs, int first_cs,
                                      int degree, const double* basis_d, const float* basis_f,
                                      int64_t out_offset, const float origin[3], const SimParams& p,
                                      const BeamDev& b, uint32_t* keys, uint32_t* vals, float4* recA,
                                      float4* recB, cudaStream_t stream);

// Sorted keys -> counts: counts[0] = #bins < ns, counts[1] = #bins == ns, with
// bin = key >> cell_bits (counts needs 4 ints).
cudaError_t launch_count_keys(const uint32_t* sorted_keys, int64_t n, int ns, int cell_bits, int* counts,
                              cudaStream_t stream);

// Sorted values -> record planes in bin order (plane B starts at out + plane).
cudaError_t launch_gather_records(const uint32_t* sorted_vals, const int* counts, int64_t n, const float4* recA,
                                  const float4* recB, float4* out, int64_t plane, cudaStream_t stream);

// Projection of the counts[0] sorted records onto all lines (lines share the
// origin); `chunk` records per CTA, lines taken in the order line_order[] with
// slot cones[] per 32 of them.  pair_counts (fp64 mode only; normally null):
// when set, a counting variant adds the (record, line) pairs it visits to
// pair_counts[0], those with a non-zero beam weight to pair_counts[1] and the
// warp walk steps in which no lane had a non-zero weight to pair_counts[2].
cudaError_t launch_project_shared(const float4* records, int64_t plane, const int* counts, int64_t n, int chunk,
                                  const LineGeom* lines, const int* line_order, const SlotCone* cones,
                                  int num_lines, const SimParams& p, const BeamDev& b, unsigned long long* bins,
                                  unsigned long long* pair_counts, cudaStream_t stream);

// Per-pair projection: fixed scatterers (cps == nullptr) or splines, arbitrary
// lines.  If index_list is given, the entries index_list[counts[0] ...
// counts[0]+counts[1]) that fall in [list_lo, list_lo + n) are projected, as
// scatterer (entry - list_lo) -- the near-origin residue of the shared path;
// otherwise scatterers [0, n).  With boxes (one per tile, fp64 mode with exact
// culling), a scatterer that no line of a tile can see with a contribution
// that survives the fixed-point rounding is left out of that tile.  pair_counts
// (normally null): pair_counts[3] += the (scatterer, line) pairs evaluated.
// threads: the CTA size, a multiple of 32 no smaller than any tile's line
// count and at most PAIR_THREADS.
cudaError_t launch_project_generic(const float4* xyza, const float4* cps, const float* amps, int64_t n,
                                   int num_cs, int degree, const uint32_t* index_list, const int* counts,
                                   int64_t list_lo,
                                   const LineGeom* lines, const int* line_ids, const LineTile* tiles,
                                   int num_tiles, const LineBasis* basis, const SimParams& p, const BeamDev& b,
                                   unsigned long long* bins, cudaStream_t stream, const TileBox* boxes = nullptr,
                                   unsigned long long* pair_counts = nullptr, int threads = PAIR_THREADS);

// Fused convolution with the analytic pulse (direct FIR over a tap window),
// IQ demodulation and radial decimation, from fixed-point bins to complex64.
// taps_pm/ph_off: the window's taps in phase-major order for this decimation
// and the phase table (see make_phase_major_taps), ntaps_pm = ph_off[D],
// max_ph_taps = the longest phase.
cudaError_t launch_convolve_demodulate(const unsigned long long* bins, int num_lines, int ns, int phase_delay,
                                       float inv_scale, const float2* taps_pm, const int* ph_off, int ntaps_pm,
                                       int max_ph_taps, int num_taps, int tap_start, int64_t M, int center,
                                       int decimation, int nd, const float2* demod, float2* out, cudaStream_t stream,
                                       const NoiseParams* noise = nullptr);

// The same by FFT (fftconv.cu): the full length-M circular convolution with
// the analytic pulse, one line per CTA in shared memory, for power-of-two
// 256 <= M <= FFT_MAX_M.  spec/tw: the tables of make_fft_tables (M entries
// each, 16-byte aligned).
constexpr int64_t FFT_MAX_M = 16384;
bool fft_convolution_supported(int64_t M);
// F: the largest power of two dividing D, at most 16 (the decimation folded
// into the spectrum); the shared memory of one CTA.
int fft_fold(int D);
size_t fft_convolution_smem(int64_t M);
// Host: H = FFT_M(h) * hilbert_mask in natural order (double) -> spec, the
// spectrum in the forward transform's output order, times
// exp(+j 2 pi center k / M) / M; tw[e] = exp(-j 2 pi e / M), e < M.
void make_fft_tables(const std::complex<double>* H, int64_t M, int center, float2* spec, float2* tw);
cudaError_t launch_fft_convolve_demodulate(const unsigned long long* bins, int num_lines, int ns, int phase_delay,
                                           float inv_scale, const float2* spec, const float2* tw, int64_t M,
                                           int decimation, int nd, const float2* demod, float2* out,
                                           cudaStream_t stream, const NoiseParams* noise = nullptr);

// Host: the FIR window taps[0..W) rearranged for the convolution kernel:
// phase ph (0..D-1) holds, for t = 0, 1, ..., the tap w = W - 1 - (ph + t*D),
// zero-padded to a multiple of 4; off[0..D] are the phases' offsets and
// off[D+1+2ph], off[D+2+2ph] the range of 4-tap iterations of phase ph that
// hold the excitation's support (non-zero real parts; real parts below 1e-9
// of the largest are set to 0).  out/off must hold W + 4*D and 3*D + 1
// entries.  Returns the total count; *max_ph receives the longest padded phase.
int make_phase_major_taps(const float2* taps, int W, int D, float2* out, int* off, int* max_ph);

// Radix sort of (key, value) pairs: key bits [0, end_bit).  temp == nullptr
// queries the scratch size into *temp_bytes.
cudaError_t radix_sort_pairs(void* temp, size_t* temp_bytes, const uint32_t* keys_in, uint32_t* keys_out,
                             const uint32_t* vals_in, uint32_t* vals_out, int64_t n, int end_bit,
                             cudaStream_t stream);

}  // namespace bcsim_gb300

namespace bcsim_gb300 {
// Scatterer ingestion (ingest.cu).  Spline control points [n][num_cs][3] ->
// [num_cs][n] float4 (x, y, z, 0).
cudaError_t launch_spline_transpose(const float* raw, int64_t n, int num_cs, float4* out, cudaStream_t stream);
// Sum of |vals[i * stride]| over i < n (double, fixed reduction order) and
// whether any value is not finite, into *sum / *nonfinite; synchronises the
// stream.  scratch: abs_sum_scratch_bytes() of device memory.
size_t abs_sum_scratch_bytes();
cudaError_t abs_sum(const float* vals, int64_t stride, int64_t n, void* scratch, double* sum, int* nonfinite,
                    cudaStream_t stream);
// The same without synchronising: *sum and *nonfinite (pinned host memory) are
// written in stream order.
cudaError_t abs_sum_enqueue(const float* vals, int64_t stride, int64_t n, void* scratch, double* sum, int* nonfinite,
                            cudaStream_t stream);

// A simulator's device error flag (SimParams::err_flag), which a kernel sets
// when a bounded wait gives up: read it into *flag and clear it, synchronising
// the stream.
cudaError_t read_and_clear_error_flag(int* dev_flag, int* flag, cudaStream_t stream);
// Copy of the error flag into host memory (pinned: asynchronous), in stream order.
cudaError_t enqueue_error_flag_read(const int* dev_flag, int* host_flag, cudaStream_t stream);
}
