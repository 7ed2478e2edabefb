/*
 * cole_case.h -- plain-C description of one COLE line simulation, shared by the
 * CPU oracle (cole_oracle.c) and the driver around the compiled reference CPU
 * algorithm (ref_driver.cpp).
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library includes this file.
 *
 * The fields mirror the inputs of bcsim::IAlgorithm (src/core/LibBCSim.hpp:42-91):
 * excitation (src/core/BCSimConfig.hpp:79-92), scan lines (src/core/ScanSequence.hpp:39-123),
 * the two beam profiles (src/core/BeamProfile.hpp:38-142), fixed and spline
 * scatterer datasets (src/core/BCSimConfig.hpp:94-165) and the string parameters
 * of BaseAlgorithm (src/core/algorithm/BaseAlgorithm.cpp:48-87).
 */
#ifndef COLE_CASE_H
#define COLE_CASE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define COLE_BEAM_GAUSSIAN 1
#define COLE_BEAM_LUT      2

/* Oracle arithmetic modes. */
#define COLE_MODE_FP64  0  /* everything in double; the tolerance reference        */
#define COLE_MODE_REF32 1  /* the reference CPU's float expressions for projection */
                           /* and demodulation, double FFT convolution             */

typedef struct {
    int            degree;
    int            num_knots;        /* = num_cs + degree + 1                      */
    const float*   knots;            /* [num_knots]                                */
    int64_t        num_scatterers;
    int            num_cs;           /* control points per scatterer (K)           */
    const float*   control_points;   /* [N][K][3]  (x, y, z)                       */
    const float*   amplitudes;       /* [N]                                        */
} cole_spline_set;

typedef struct {
    /* excitation signal */
    const float* taps;
    int          num_taps;
    int          center_index;
    float        fs;
    float        demod_freq;
    /* parameters */
    float        sound_speed;
    int          use_arc_projection;
    int          phase_delay;
    int          radial_decimation;
    /* beam profile */
    int          beam;
    float        sigma_lateral;
    float        sigma_elevational;
    const float* lut;                /* [nr][nl][ne] row-major                     */
    int          lut_nr, lut_nl, lut_ne;
    float        lut_r[2], lut_l[2], lut_e[2];
    /* scan sequence */
    int          num_lines;
    float        line_length;
    const float* origins;            /* [L][3] */
    const float* directions;         /* [L][3] */
    const float* lateral_dirs;       /* [L][3] */
    const float* timestamps;         /* [L]    */
    /* fixed scatterer datasets */
    int             num_fixed_sets;
    const int64_t*  fixed_counts;    /* [num_fixed_sets]                           */
    const float* const* fixed_xyza;  /* [num_fixed_sets] -> [N][4] (x, y, z, a)    */
    /* spline scatterer datasets */
    int                    num_spline_sets;
    const cole_spline_set* spline_sets;
    /* seeded complex noise N(0, noise_sigma) on every time-projection sample
     * j < ns (noise_amplitude, CpuAlgorithm.cpp:340-347), keyed by (noise_seed,
     * noise_frame, line, j); 0 = off.  Not read by the reference driver. */
    float        noise_sigma;
    uint64_t     noise_seed;
    uint32_t     noise_frame;
} cole_case;

#ifdef __cplusplus
}
#endif
#endif
