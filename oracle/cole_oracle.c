/*
 * cole_oracle.c -- CPU restatement of the reference COLE line simulator.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the parity checker for the GPU engine and
 * the "port" CPU baseline timed by bench.py.  The product library never links,
 * loads or calls it.
 *
 * It restates, in plain C, the algorithm of the reference's CPU path:
 *   per-line driver            src/core/algorithm/CpuAlgorithm.cpp:278-368
 *   fixed projection loop      src/core/algorithm/CpuAlgorithm.cpp:50-97
 *   spline projection loop     src/core/algorithm/CpuAlgorithm.cpp:99-183
 *   number of samples          src/core/algorithm/common_utils.hpp:38-41
 *   spline sanity check        src/core/algorithm/common_utils.hpp:51-60
 *   FFT convolver + Hilbert    src/core/BeamConvolver.cpp:45-91,
 *                              src/core/discrete_hilbert_mask.hpp:36-66
 *   next power of two          src/core/fft.cpp:80-82
 *   Gaussian / LUT beam        src/core/BeamProfile.cpp:49-51, 79-130
 *   B-spline basis             src/core/bspline.hpp:44-91
 *   Gaussian pulse             src/utils/GaussPulse.cpp:33-70
 *
 * Two arithmetic modes:
 *   COLE_MODE_FP64  -- every derived quantity in double (inputs are float32 and are
 *                      promoted on load).  This is the tolerance reference.
 *   COLE_MODE_REF32 -- the projection (distances, bin index, beam weight, phase,
 *                      bin accumulation) and the demodulation use the reference's
 *                      own float/double expressions, so that the bins match the
 *                      compiled reference bit for bit; only the FFT convolution runs
 *                      in double.  Build with -ffp-contract=off.
 *
 * The convolution is an exact length-M circular convolution computed with an
 * iterative radix-2 FFT in double (written here; the reference uses its own
 * recursive float FFT).
 */
#include "cole_case.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_OK 0
#define ORACLE_ERR 1

static const double TWO_PI_D = 6.283185307179586; /* literal used by CpuAlgorithm.cpp:89,175 */

/* ------------------------------------------------------------------------- */
/* Small helpers                                                              */
/* ------------------------------------------------------------------------- */

/* compute_num_rf_samples<float> (common_utils.hpp:38-41): the intermediate
 * max_time is rounded to float, the product fs*max_time is a float product. */
int64_t oracle_num_rf_samples(float sound_speed, float line_length, float fs) {
    const float max_time = (float)(2.0 * line_length / sound_speed);
    const float prod = fs * max_time;
    return (int64_t)floor(prod + 0.5);
}

/* next_power_of_two (fft.cpp:80-82): pow(2, ceil(log(n)/log(2))). */
int64_t oracle_next_pow2(int64_t n) {
    return (int64_t)pow(2.0, ceil(log((double)n) / log(2.0)));
}

/* discrete_hilbert_mask (discrete_hilbert_mask.hpp:36-66). */
void oracle_hilbert_mask(int64_t n, double* out) {
    for (int64_t i = 0; i < n; i++) {
        double k = 0.0;
        if ((n % 2) == 0) {
            if (i == 0 || i == n / 2) k = 1.0;
            else if (i >= 1 && i <= n / 2 - 1) k = 2.0;
        } else {
            if (i == 0) k = 1.0;
            else if (i >= 1 && i < (n + 1) / 2) k = 2.0;
        }
        out[i] = k;
    }
}

/* In-place iterative radix-2 FFT in double.  sign = -1 forward, +1 inverse
 * (unscaled).  n must be a power of two. */
static void fft_inplace(double* re, double* im, int64_t n, int sign) {
    int64_t j = 0;
    for (int64_t i = 1; i < n; i++) {
        int64_t bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            double t = re[i]; re[i] = re[j]; re[j] = t;
            t = im[i]; im[i] = im[j]; im[j] = t;
        }
    }
    for (int64_t len = 2; len <= n; len <<= 1) {
        const int64_t half = len >> 1;
        const double ang = sign * TWO_PI_D / (double)len;
        for (int64_t k = 0; k < half; k++) {
            /* twiddles computed directly, not by recurrence, to keep the error flat */
            const double wr = cos(ang * (double)k), wi = sin(ang * (double)k);
            for (int64_t s = 0; s < n; s += len) {
                const int64_t a = s + k, b = s + k + half;
                const double xr = re[b] * wr - im[b] * wi;
                const double xi = re[b] * wi + im[b] * wr;
                re[b] = re[a] - xr; im[b] = im[a] - xi;
                re[a] += xr;        im[a] += xi;
            }
        }
    }
}

/* fft_conv (fft.cpp:94-120): linear convolution of two real sequences through
 * a power-of-two FFT.  out has nx+nh-1 entries. */
int oracle_fft_conv(const double* x, int nx, const double* h, int nh, double* out) {
    const int64_t n = nx + nh - 1;
    const int64_t m = oracle_next_pow2(n);
    double* ar = calloc((size_t)m, sizeof(double));
    double* ai = calloc((size_t)m, sizeof(double));
    double* br = calloc((size_t)m, sizeof(double));
    double* bi = calloc((size_t)m, sizeof(double));
    if (!ar || !ai || !br || !bi) { free(ar); free(ai); free(br); free(bi); return -1; }
    for (int i = 0; i < nx; i++) ar[i] = x[i];
    for (int i = 0; i < nh; i++) br[i] = h[i];
    fft_inplace(ar, ai, m, -1);
    fft_inplace(br, bi, m, -1);
    for (int64_t k = 0; k < m; k++) {
        const double r = ar[k] * br[k] - ai[k] * bi[k];
        const double i = ar[k] * bi[k] + ai[k] * br[k];
        ar[k] = r; ai[k] = i;
    }
    fft_inplace(ar, ai, m, +1);
    for (int64_t k = 0; k < n; k++) out[k] = ar[k] / (double)m;
    free(ar); free(ai); free(br); free(bi);
    return (int)n;
}

/* direct_conv (src/utils/SignalProcessing.cpp; pinned by
 * src/utils/unittest/test_SignalProcessing.cpp:6-27). */
int oracle_direct_conv_i64(const int64_t* x, int nx, const int64_t* h, int nh, int64_t* out) {
    const int n = nx + nh - 1;
    for (int k = 0; k < n; k++) {
        int64_t s = 0;
        for (int j = 0; j < nh; j++) {
            const int i = k - j;
            if (i >= 0 && i < nx) s += x[i] * h[j];
        }
        out[k] = s;
    }
    return n;
}

/* Analytic excitation spectrum H = FFT_M(taps) * hilbert_mask(M)
 * (BeamConvolver.cpp:77-91), in double.  hr/hi have M entries. */
void oracle_analytic_spectrum(const float* taps, int ntaps, int64_t M, double* hr, double* hi) {
    double* mask = malloc(sizeof(double) * (size_t)M);
    for (int64_t i = 0; i < M; i++) { hr[i] = 0.0; hi[i] = 0.0; }
    for (int i = 0; i < ntaps && i < M; i++) hr[i] = (double)taps[i];
    fft_inplace(hr, hi, M, -1);
    oracle_hilbert_mask(M, mask);
    for (int64_t i = 0; i < M; i++) { hr[i] *= mask[i]; hi[i] *= mask[i]; }
    free(mask);
}

/* ------------------------------------------------------------------------- */
/* Gaussian pulse (GaussPulse.cpp:33-70), float/double exactly as written.     */
/* ------------------------------------------------------------------------- */
static double gauss_time_limit(double fc, double bw, double bwr, double tpr) {
    const double PI = 4 * atan(1.0);
    const double E = exp(1.0);
    const double f_cutoff = bw * fc;
    return sqrt(-tpr / (20.0 * (-PI * PI * f_cutoff * f_cutoff / (log(pow(10.0, bwr / 20.0)))) * log10(E)));
}

static float gauss_pulse_f(float t, float fc, float bw, float bwr) {
    const float PI = (float)(4 * atan(1.0));
    const float f_cutoff = bw * fc;
    const float ftp = (float)(f_cutoff * t);
    const float ppf = PI * PI * ftp * ftp;
    const double env = exp(ppf / (log(pow(10.0, bwr / 20.0))));
    const float arg = 2 * PI * fc * t;
    return (float)(env * (double)cosf(arg));
}

int oracle_gaussian_excitation(float fc, float bw, float fs, float* out, int cap, int* center_index) {
    const double lim = gauss_time_limit(fc, bw, -6.0, -60.0);
    const int n = (int)(2 * lim * fs);
    for (int i = 0; i < n && i < cap; i++) {
        const float t = (float)(i - n / 2) / fs;
        out[i] = gauss_pulse_f(t, fc, bw, -6.0f);
    }
    if (center_index) *center_index = n / 2;
    return n;
}

/* ------------------------------------------------------------------------- */
/* B-splines (bspline.hpp:44-112) in double and in float                      */
/* ------------------------------------------------------------------------- */
static double special_div_d(double num, double den) {
    if (fabs(num) < 1e-6 && fabs(den) < 1e-6) return 0.0;
    return num / den;
}
static float special_div_f(float num, float den) {
    if (fabs((double)num) < 1e-6 && fabs((double)den) < 1e-6) return 0.0f;
    return num / den;
}
double oracle_bspline_basis_d(int j, int p, double x, const float* k) {
    if (p == 0) return (x >= (double)k[j] && x < (double)k[j + 1]) ? 1.0 : 0.0;
    const double left = special_div_d((x - (double)k[j]) * oracle_bspline_basis_d(j, p - 1, x, k),
                                      (double)k[j + p] - (double)k[j]);
    const double right = special_div_d(((double)k[j + 1 + p] - x) * oracle_bspline_basis_d(j + 1, p - 1, x, k),
                                       (double)k[j + 1 + p] - (double)k[j + 1]);
    return left + right;
}
float oracle_bspline_basis_f(int j, int p, float x, const float* k) {
    if (p == 0) return (x >= k[j] && x < k[j + 1]) ? 1.0f : 0.0f;
    const float left = special_div_f((x - k[j]) * oracle_bspline_basis_f(j, p - 1, x, k), k[j + p] - k[j]);
    const float right = special_div_f((k[j + 1 + p] - x) * oracle_bspline_basis_f(j + 1, p - 1, x, k), k[j + 1 + p] - k[j + 1]);
    return left + right;
}
/* compute_knot_interval (bspline.hpp:74-82); -1 where the reference throws. */
int oracle_knot_interval(const float* knots, int nk, float t) {
    for (int i = 0; i < nk - 1; i++)
        if (t >= knots[i] && t < knots[i + 1]) return i;
    return -1;
}
/* uniform_regular_knot_vector (bspline.hpp:95-112), float. */
int oracle_uniform_regular_knots(int n, int p, float t0, float t1, float* out, int cap) {
    if (n < p + 1) return -1;
    int c = 0;
    for (int i = 0; i < p; i++) { if (c < cap) out[c] = t0; c++; }
    const int num_middle = n + 1 - p;
    for (int i = 0; i < num_middle; i++) {
        if (c < cap) out[c] = t0 + i * (t1 - t0) / (num_middle - 1);
        c++;
    }
    for (int i = 0; i < p; i++) { if (c < cap) out[c] = t1; c++; }
    return c;
}

/* ------------------------------------------------------------------------- */
/* Beam profiles                                                              */
/* ------------------------------------------------------------------------- */
typedef struct {
    int beam;
    double two_sl2_d, two_se2_d;   /* 2 sigma^2, double */
    float two_sl2_f, two_se2_f;    /* 2*sigma*sigma, float (BeamProfile.cpp:53-56) */
    const float* lut;
    int nr, nl, ne;
    float rf, lf, ef;              /* first sample positions */
    double dr_d, dl_d, de_d;       /* spacing computed in double */
    double dr_f, dl_f, de_f;       /* spacing computed as the reference does (float) */
} beam_t;

static double lut_value_d(const beam_t* b, double r, double l, double e) {
    const double tr = (r - (double)b->rf) / b->dr_d;
    const double tl = (l - (double)b->lf) / b->dl_d;
    const double te = (e - (double)b->ef) / b->de_d;
    /* the reference's index test (BeamProfile.cpp:94-103) for trunc-toward-zero
     * indices i0 = int(t), i1 = int(t+1) accepts exactly -1 < t < n-1 */
    if (!(tr > -1.0 && tr < (double)(b->nr - 1))) return 0.0;
    if (!(tl > -1.0 && tl < (double)(b->nl - 1))) return 0.0;
    if (!(te > -1.0 && te < (double)(b->ne - 1))) return 0.0;
    const int r0 = (int)tr, r1 = (int)(tr + 1), l0 = (int)tl, l1 = (int)(tl + 1), e0 = (int)te, e1 = (int)(te + 1);
    const double fr = tr - r0, fl = tl - l0, fe = te - e0;
#define LUTD(ir, il, ie) ((double)b->lut[((int64_t)(ir) * b->nl + (il)) * b->ne + (ie)])
    const double c00 = (1.0 - fr) * LUTD(r0, l0, e0) + fr * LUTD(r1, l0, e0);
    const double c10 = (1.0 - fr) * LUTD(r0, l1, e0) + fr * LUTD(r1, l1, e0);
    const double c01 = (1.0 - fr) * LUTD(r0, l0, e1) + fr * LUTD(r1, l0, e1);
    const double c11 = (1.0 - fr) * LUTD(r0, l1, e1) + fr * LUTD(r1, l1, e1);
#undef LUTD
    const double c0 = (1.0 - fl) * c00 + fl * c10;
    const double c1 = (1.0 - fl) * c01 + fl * c11;
    return (1.0 - fe) * c0 + fe * c1;
}

/* LUTBeamProfile::sampleProfile (BeamProfile.cpp:79-130) with its float/double mix. */
static float lut_value_f(const beam_t* b, float r, float l, float e) {
    const double tr = (double)(r - b->rf) / b->dr_f;
    const double tl = (double)(l - b->lf) / b->dl_f;
    const double te = (double)(e - b->ef) / b->de_f;
    if (!(tr > -1.0 && tr < (double)(b->nr - 1))) return 0.0f;
    if (!(tl > -1.0 && tl < (double)(b->nl - 1))) return 0.0f;
    if (!(te > -1.0 && te < (double)(b->ne - 1))) return 0.0f;
    const int r0 = (int)tr, r1 = (int)(tr + 1), l0 = (int)tl, l1 = (int)(tl + 1), e0 = (int)te, e1 = (int)(te + 1);
    const float fr = (float)(tr - r0), fl = (float)(tl - l0), fe = (float)(te - e0);
#define LUTF(ir, il, ie) (b->lut[((int64_t)(ir) * b->nl + (il)) * b->ne + (ie)])
    const float c00 = (1.0f - fr) * LUTF(r0, l0, e0) + fr * LUTF(r1, l0, e0);
    const float c10 = (1.0f - fr) * LUTF(r0, l1, e0) + fr * LUTF(r1, l1, e0);
    const float c01 = (1.0f - fr) * LUTF(r0, l0, e1) + fr * LUTF(r1, l0, e1);
    const float c11 = (1.0f - fr) * LUTF(r0, l1, e1) + fr * LUTF(r1, l1, e1);
#undef LUTF
    const float c0 = (1.0f - fl) * c00 + fl * c10;
    const float c1 = (1.0f - fl) * c01 + fl * c11;
    return (1.0f - fe) * c0 + fe * c1;
}

/* ------------------------------------------------------------------------- */
/* One line                                                                   */
/* ------------------------------------------------------------------------- */
typedef struct {
    double ox, oy, oz, rx, ry, rz, lx, ly, lz, ex, ey, ez;   /* double copies */
    float ofx, ofy, ofz, rfx, rfy, rfz, lfx, lfy, lfz, efx, efy, efz;
    float t;
} line_t;

/* Scanline: elevational = lateral x direction, in float (ScanSequence.cpp:37-41,
 * vector3.hpp:97-103). */
static void make_line(const cole_case* c, int i, line_t* ln) {
    const float* o = c->origins + 3 * i;
    const float* d = c->directions + 3 * i;
    const float* l = c->lateral_dirs + 3 * i;
    ln->ofx = o[0]; ln->ofy = o[1]; ln->ofz = o[2];
    ln->rfx = d[0]; ln->rfy = d[1]; ln->rfz = d[2];
    ln->lfx = l[0]; ln->lfy = l[1]; ln->lfz = l[2];
    ln->efx = l[1] * d[2] - d[1] * l[2];
    ln->efy = d[0] * l[2] - l[0] * d[2];
    ln->efz = l[0] * d[1] - d[0] * l[1];
    ln->ox = o[0]; ln->oy = o[1]; ln->oz = o[2];
    ln->rx = d[0]; ln->ry = d[1]; ln->rz = d[2];
    ln->lx = l[0]; ln->ly = l[1]; ln->lz = l[2];
    ln->ex = ln->efx; ln->ey = ln->efy; ln->ez = ln->efz;
    ln->t = c->timestamps[i];
}

typedef struct {
    const cole_case* c;
    int mode;
    int64_t ns, M, nd;
    double two_pi_fd;          /* for the FP64 phase */
    beam_t beam;
    const double* Hr;          /* analytic excitation spectrum [M] */
    const double* Hi;
} ctx_t;

/* Accumulate one scatterer at double-precision position (px,py,pz) into the bins
 * (FP64 mode).  spline selects the spline path's index expression
 * r*2/(c*dt) (CpuAlgorithm.cpp:161-162) over the fixed path's r*2*fs/c (:75). */
static void project_fp64(const ctx_t* x, const line_t* ln, double px, double py, double pz, double amp_in,
                         int spline, double* bre, double* bim) {
    const cole_case* c = x->c;
    const double dx = px - ln->ox, dy = py - ln->oy, dz = pz - ln->oz;
    double r = dx * ln->rx + dy * ln->ry + dz * ln->rz;
    const double l = dx * ln->lx + dy * ln->ly + dz * ln->lz;
    const double e = dx * ln->ex + dy * ln->ey + dz * ln->ez;
    if (c->use_arc_projection) r = copysign(sqrt(dx * dx + dy * dy + dz * dz), r);
    double t;
    if (spline) {
        const double dt = 1.0 / (double)c->fs;
        t = r * 2.0 / ((double)c->sound_speed * dt);
    } else {
        t = r * 2.0 * (double)c->fs / (double)c->sound_speed;
    }
    const double fidx = floor(t + 0.5);
    double w;
    if (x->beam.beam == COLE_BEAM_GAUSSIAN) {
        w = exp(-(l * l / x->beam.two_sl2_d + e * e / x->beam.two_se2_d));
    } else {
        w = lut_value_d(&x->beam, r, l, e);
    }
    const double amp = w * amp_in;
    if (!(fidx >= 0.0 && fidx < (double)x->ns)) return;
    const int64_t idx = (int64_t)fidx;
    if (c->phase_delay) {
        const double delay = ((double)idx - t) / (double)c->fs;
        const double ph = TWO_PI_D * (double)c->demod_freq * delay;
        bre[idx] += amp * cos(ph);
        bim[idx] += amp * sin(ph);
    } else {
        bre[idx] += amp;
    }
}

/* The reference's float projection (CpuAlgorithm.cpp:58-95 / 144-181). */
static void project_ref32(const ctx_t* x, const line_t* ln, float px, float py, float pz, float amp_in,
                          int spline, float* bre, float* bim) {
    const cole_case* c = x->c;
    const float tx = px - ln->ofx, ty = py - ln->ofy, tz = pz - ln->ofz;
    float r = tx * ln->rfx + ty * ln->rfy + tz * ln->rfz;
    const float l = tx * ln->lfx + ty * ln->lfy + tz * ln->lfz;
    const float e = tx * ln->efx + ty * ln->efy + tz * ln->efz;
    if (c->use_arc_projection) r = copysignf(sqrtf(tx * tx + ty * ty + tz * tz), r);
    double t;
    if (spline) {
        const float dt = (float)(1.0 / c->fs);
        t = r * 2.0 / (double)(c->sound_speed * dt);
    } else {
        t = r * 2.0 * c->fs / (double)c->sound_speed;
    }
    const double fl = floor(t + 0.5f);
    float w;
    if (x->beam.beam == COLE_BEAM_GAUSSIAN) {
        w = expf(-(l * l / x->beam.two_sl2_f + e * e / x->beam.two_se2_f));
    } else {
        w = lut_value_f(&x->beam, r, l, e);
    }
    const float amp = w * amp_in;
    if (!(fl >= 0.0 && fl < (double)x->ns)) return;
    const int idx = (int)fl;
    if (c->phase_delay) {
        const float ss_delay = (float)((idx - t) / c->fs);
        const float phase = (float)(TWO_PI_D * c->demod_freq * ss_delay);
        bre[idx] += amp * cosf(phase);
        bim[idx] += amp * sinf(phase);
    } else {
        bre[idx] += amp;
    }
}

/* Time-projection of every dataset onto one line (CpuAlgorithm.cpp:314-338).
 * FP64 mode accumulates into wr/wi, REF32 mode into the float bins fr/fi; both
 * have M entries, the first ns of which are written. */
static int project_line(const ctx_t* x, int line_no, double* wr, double* wi, float* fr, float* fi,
                        char* err, int errcap) {
    const cole_case* c = x->c;
    line_t ln;
    make_line(c, line_no, &ln);
    const int64_t M = x->M;
    for (int64_t i = 0; i < M; i++) { wr[i] = 0.0; wi[i] = 0.0; }
    if (x->mode == COLE_MODE_REF32) for (int64_t i = 0; i < M; i++) { fr[i] = 0.0f; fi[i] = 0.0f; }

    for (int s = 0; s < c->num_fixed_sets; s++) {
        const float* p = c->fixed_xyza[s];
        for (int64_t i = 0; i < c->fixed_counts[s]; i++) {
            if (x->mode == COLE_MODE_FP64)
                project_fp64(x, &ln, p[4 * i], p[4 * i + 1], p[4 * i + 2], p[4 * i + 3], 0, wr, wi);
            else
                project_ref32(x, &ln, p[4 * i], p[4 * i + 1], p[4 * i + 2], p[4 * i + 3], 0, fr, fi);
        }
    }
    for (int s = 0; s < c->num_spline_sets; s++) {
        const cole_spline_set* ss = &c->spline_sets[s];
        const int K = ss->num_cs, p = ss->degree;
        if (K <= p) {
            snprintf(err, (size_t)errcap, "too few spline control points for given degree");
            return ORACLE_ERR;
        }
        const int mu = oracle_knot_interval(ss->knots, ss->num_knots, ln.t);
        if (mu < 0) {
            snprintf(err, (size_t)errcap, "compute_knot_interval : could not determine knot interval");
            return ORACLE_ERR;
        }
        const int lo = mu - p, hi = mu;
        if (lo < 0 || hi >= K) {
            snprintf(err, (size_t)errcap, "spline evaluation index out of range");
            return ORACLE_ERR;
        }
        double bd[64];
        float bf[64];
        double* bdv = K <= 64 ? bd : malloc(sizeof(double) * (size_t)K);
        float* bfv = K <= 64 ? bf : malloc(sizeof(float) * (size_t)K);
        for (int i = 0; i < K; i++) {
            bdv[i] = oracle_bspline_basis_d(i, p, (double)ln.t, ss->knots);
            bfv[i] = oracle_bspline_basis_f(i, p, ln.t, ss->knots);
        }
        /* sanity_check_spline_lower_upper_bound (common_utils.hpp:51-60) on the
         * basis the mode uses */
        int bad = 0;
        for (int i = 0; i < K; i++) {
            if (i >= lo && i <= hi) continue;
            const double v = x->mode == COLE_MODE_FP64 ? bdv[i] : (double)bfv[i];
            if (fabs(v) > 1e-6) bad = 1;
        }
        if (bad) {
            if (bdv != bd) free(bdv);
            if (bfv != bf) free(bfv);
            snprintf(err, (size_t)errcap, "b-spline basis bounds failed sanity check");
            return ORACLE_ERR;
        }
        for (int64_t n = 0; n < ss->num_scatterers; n++) {
            const float* cp = ss->control_points + (size_t)n * K * 3;
            if (x->mode == COLE_MODE_FP64) {
                double px = 0.0, py = 0.0, pz = 0.0;
                for (int i = lo; i <= hi; i++) {
                    px += (double)cp[3 * i] * bdv[i];
                    py += (double)cp[3 * i + 1] * bdv[i];
                    pz += (double)cp[3 * i + 2] * bdv[i];
                }
                project_fp64(x, &ln, px, py, pz, ss->amplitudes[n], 1, wr, wi);
            } else {
                float px = 0.0f, py = 0.0f, pz = 0.0f;
                for (int i = lo; i <= hi; i++) {
                    px += cp[3 * i] * bfv[i];
                    py += cp[3 * i + 1] * bfv[i];
                    pz += cp[3 * i + 2] * bfv[i];
                }
                project_ref32(x, &ln, px, py, pz, ss->amplitudes[n], 1, fr, fi);
            }
        }
        if (bdv != bd) free(bdv);
        if (bfv != bf) free(bfv);
    }
    return ORACLE_OK;
}

/* Philox4x32-10 (Salmon, Moraes, Dror and Shaw, SC 2011): ten rounds of two
 * 32x32->64 multiplications, the key bumped by the Weyl constants between rounds. */
static void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; r++) {
        if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        c[0] = n0; c[1] = (uint32_t)p1; c[2] = n2; c[3] = (uint32_t)p0;
    }
}

/* The Philox block itself, for known-answer tests. */
void oracle_philox4x32_10(uint32_t* c, uint32_t k0, uint32_t k1) { philox4x32_10(c, k0, k1); }

/* Unit-variance noise (re, im) of sample j of line `line` in frame `frame`:
 * Philox block of counter (j, line, frame, 0x6e6f6973) under the 64-bit seed;
 * Box-Muller of u1 = (w0 >> 8 + 1/2) 2^-24 and u2 = (w1 >> 8) 2^-24, in double. */
void oracle_bin_noise(uint64_t seed, uint32_t frame, int line, int64_t j, double* re, double* im) {
    uint32_t c[4] = {(uint32_t)j, (uint32_t)line, frame, 0x6e6f6973u};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    const double u1 = ((double)(c[0] >> 8) + 0.5) * 0x1p-24;
    const double u2 = (double)(c[1] >> 8) * 0x1p-24;
    const double rad = sqrt(-2.0 * log(u1));
    *re = rad * cos(TWO_PI_D * u2);
    *im = rad * sin(TWO_PI_D * u2);
}

static int simulate_one_line(const ctx_t* x, int line_no, double* wr, double* wi, float* fr, float* fi,
                             float* out, char* err, int errcap) {
    const cole_case* c = x->c;
    const int64_t M = x->M, ns = x->ns;
    const int prc = project_line(x, line_no, wr, wi, fr, fi, err, errcap);
    if (prc != ORACLE_OK) return prc;

    if (x->mode == COLE_MODE_REF32) {
        for (int64_t i = 0; i < ns; i++) {
            /* BCSIM_ENABLE_NAN_CHECK (CpuAlgorithm.cpp:330-338) */
            if (fr[i] != fr[i] || fi[i] != fi[i]) {
                snprintf(err, (size_t)errcap, "Nan in scatterer projection.");
                return ORACLE_ERR;
            }
            wr[i] = fr[i]; wi[i] = fi[i];
        }
    } else {
        for (int64_t i = 0; i < ns; i++) {
            if (wr[i] != wr[i] || wi[i] != wi[i]) {
                snprintf(err, (size_t)errcap, "Nan in scatterer projection.");
                return ORACLE_ERR;
            }
        }
    }
    /* Gaussian noise on the time projection (CpuAlgorithm.cpp:340-347), seeded */
    if (c->noise_sigma > 0.0f) {
        for (int64_t i = 0; i < ns; i++) {
            double nr, ni;
            oracle_bin_noise(c->noise_seed, c->noise_frame, line_no, i, &nr, &ni);
            wr[i] += (double)c->noise_sigma * nr;
            wi[i] += (double)c->noise_sigma * ni;
        }
    }

    /* circular convolution with the analytic pulse (BeamConvolver.cpp:64-73) */
    fft_inplace(wr, wi, M, -1);
    for (int64_t k = 0; k < M; k++) {
        const double a = wr[k] * x->Hr[k] - wi[k] * x->Hi[k];
        const double b = wr[k] * x->Hi[k] + wi[k] * x->Hr[k];
        wr[k] = a; wi[k] = b;
    }
    fft_inplace(wr, wi, M, +1);
    const double invM = 1.0 / (double)M;
    const int D = c->radial_decimation;
    const int64_t center = c->center_index;

    /* demodulation (CpuAlgorithm.cpp:353-358) and decimation (:362-365) */
    if (x->mode == COLE_MODE_FP64) {
        const double nf = (double)c->demod_freq / (double)c->fs;
        for (int64_t m = 0; m < x->nd; m++) {
            const int64_t i = m * D;
            const double yr = wr[center + i] * invM, yi = wi[center + i] * invM;
            const double ph = -TWO_PI_D * nf * (double)i;
            const double cs = cos(ph), sn = sin(ph);
            out[2 * m] = (float)(yr * cs - yi * sn);
            out[2 * m + 1] = (float)(yr * sn + yi * cs);
        }
    } else {
        const float TWO_PI = (float)(2.0 * 4.0 * atan(1.0));
        const float nf = c->demod_freq / c->fs;
        const float a = -TWO_PI * nf;
        for (int64_t m = 0; m < x->nd; m++) {
            const int64_t i = m * D;
            const float yr = (float)(wr[center + i] * invM), yi = (float)(wi[center + i] * invM);
            const float arg = a * (float)i;
            const float cs = cosf(arg), sn = sinf(arg);
            out[2 * m] = yr * cs - yi * sn;
            out[2 * m + 1] = yr * sn + yi * cs;
        }
    }
    return ORACLE_OK;
}

/* ------------------------------------------------------------------------- */
/* Public entry                                                               */
/* ------------------------------------------------------------------------- */
int64_t oracle_num_out_samples(const cole_case* c) {
    const int64_t ns = oracle_num_rf_samples(c->sound_speed, c->line_length, c->fs);
    const int D = c->radial_decimation;
    return D > 0 ? (ns + D - 1) / D : 0;
}

/* Derived sizes and beam constants for one case. */
static int setup_ctx(const cole_case* c, int mode, ctx_t* xp, char* err, int errcap) {
    ctx_t x;
    memset(&x, 0, sizeof(x));
    x.c = c;
    x.mode = mode;
    x.ns = oracle_num_rf_samples(c->sound_speed, c->line_length, c->fs);
    x.M = oracle_next_pow2(x.ns + c->num_taps - 1);
    x.nd = (x.ns + c->radial_decimation - 1) / c->radial_decimation;
    if ((int64_t)c->center_index + (x.nd - 1) * c->radial_decimation >= x.M || c->center_index < 0) {
        snprintf(err, (size_t)errcap, "excitation center index outside the convolution buffer");
        return ORACLE_ERR;
    }
    x.beam.beam = c->beam;
    x.beam.two_sl2_d = 2.0 * (double)c->sigma_lateral * (double)c->sigma_lateral;
    x.beam.two_se2_d = 2.0 * (double)c->sigma_elevational * (double)c->sigma_elevational;
    x.beam.two_sl2_f = 2 * c->sigma_lateral * c->sigma_lateral;
    x.beam.two_se2_f = 2 * c->sigma_elevational * c->sigma_elevational;
    if (c->beam == COLE_BEAM_LUT) {
        x.beam.lut = c->lut;
        x.beam.nr = c->lut_nr; x.beam.nl = c->lut_nl; x.beam.ne = c->lut_ne;
        x.beam.rf = c->lut_r[0]; x.beam.lf = c->lut_l[0]; x.beam.ef = c->lut_e[0];
        x.beam.dr_d = ((double)c->lut_r[1] - (double)c->lut_r[0]) / (c->lut_nr - 1);
        x.beam.dl_d = ((double)c->lut_l[1] - (double)c->lut_l[0]) / (c->lut_nl - 1);
        x.beam.de_d = ((double)c->lut_e[1] - (double)c->lut_e[0]) / (c->lut_ne - 1);
        /* BeamProfile.cpp:72-74: float difference divided by an int, stored as double */
        x.beam.dr_f = (double)((c->lut_r[1] - c->lut_r[0]) / (c->lut_nr - 1));
        x.beam.dl_f = (double)((c->lut_l[1] - c->lut_l[0]) / (c->lut_nl - 1));
        x.beam.de_f = (double)((c->lut_e[1] - c->lut_e[0]) / (c->lut_ne - 1));
    }
    *xp = x;
    return ORACLE_OK;
}

/* The time-projection bins of one line (first ns entries, complex as re/im
 * pairs), before convolution. */
int oracle_project_bins(const cole_case* c, int mode, int line_no, double* out_bins, int64_t cap_pairs,
                        char* err, int errcap) {
    ctx_t x;
    if (setup_ctx(c, mode, &x, err, errcap) != ORACLE_OK) return ORACLE_ERR;
    if (cap_pairs < x.ns) { snprintf(err, (size_t)errcap, "output buffer too small"); return ORACLE_ERR; }
    double* wr = malloc(sizeof(double) * (size_t)x.M);
    double* wi = malloc(sizeof(double) * (size_t)x.M);
    float* fr = malloc(sizeof(float) * (size_t)x.M);
    float* fi = malloc(sizeof(float) * (size_t)x.M);
    const int rc = project_line(&x, line_no, wr, wi, fr, fi, err, errcap);
    if (rc == ORACLE_OK) {
        for (int64_t i = 0; i < x.ns; i++) {
            out_bins[2 * i] = x.mode == COLE_MODE_REF32 ? (double)fr[i] : wr[i];
            out_bins[2 * i + 1] = x.mode == COLE_MODE_REF32 ? (double)fi[i] : wi[i];
        }
    }
    free(wr); free(wi); free(fr); free(fi);
    return rc;
}

/* Simulate all lines.  out: float [L][nd][2].  line_begin/line_end select a
 * contiguous subset of the lines (the rows of out are that subset). */
int oracle_simulate(const cole_case* c, int mode, int num_threads, int line_begin, int line_end,
                    float* out, int64_t out_cap_floats, char* err, int errcap) {
    if (c->num_lines <= 0) { snprintf(err, (size_t)errcap, "Scan sequence not configured."); return ORACLE_ERR; }
    if (c->beam != COLE_BEAM_GAUSSIAN && c->beam != COLE_BEAM_LUT) {
        snprintf(err, (size_t)errcap, "Beam profile not configured.");
        return ORACLE_ERR;
    }
    if (c->radial_decimation <= 0) { snprintf(err, (size_t)errcap, "illegal radial decimation value"); return ORACLE_ERR; }
    int64_t total = 0;
    for (int s = 0; s < c->num_fixed_sets; s++) total += c->fixed_counts[s];
    for (int s = 0; s < c->num_spline_sets; s++) total += c->spline_sets[s].num_scatterers;
    if (total == 0) { snprintf(err, (size_t)errcap, "no scatterers are configured"); return ORACLE_ERR; }
    if (line_begin < 0) line_begin = 0;
    if (line_end > c->num_lines || line_end < 0) line_end = c->num_lines;

    ctx_t x;
    if (setup_ctx(c, mode, &x, err, errcap) != ORACLE_OK) return ORACLE_ERR;
    if ((int64_t)(line_end - line_begin) * x.nd * 2 > out_cap_floats) {
        snprintf(err, (size_t)errcap, "output buffer too small");
        return ORACLE_ERR;
    }
    double* Hr = malloc(sizeof(double) * (size_t)x.M);
    double* Hi = malloc(sizeof(double) * (size_t)x.M);
    oracle_analytic_spectrum(c->taps, c->num_taps, x.M, Hr, Hi);
    x.Hr = Hr; x.Hi = Hi;

    int status = ORACLE_OK;
#ifdef _OPENMP
    if (num_threads > 0) omp_set_num_threads(num_threads);
#endif
#pragma omp parallel
    {
        double* wr = malloc(sizeof(double) * (size_t)x.M);
        double* wi = malloc(sizeof(double) * (size_t)x.M);
        float* fr = malloc(sizeof(float) * (size_t)x.M);
        float* fi = malloc(sizeof(float) * (size_t)x.M);
        char lerr[256];
        lerr[0] = 0;
#pragma omp for schedule(dynamic, 1)
        for (int ln = line_begin; ln < line_end; ln++) {
            if (status != ORACLE_OK) continue;
            const int rc = simulate_one_line(&x, ln, wr, wi, fr, fi, out + (int64_t)(ln - line_begin) * x.nd * 2, lerr, 256);
            if (rc != ORACLE_OK) {
#pragma omp critical
                {
                    if (status == ORACLE_OK) {
                        status = rc;
                        snprintf(err, (size_t)errcap, "%s", lerr);
                    }
                }
            }
        }
        free(wr); free(wi); free(fr); free(fi);
    }
    free(Hr);
    free(Hi);
    return status;
}
