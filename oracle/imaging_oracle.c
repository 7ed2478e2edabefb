/* imaging_oracle.c -- CPU restatement of the reference's image formation after
 * simulate_lines.  TEST INFRASTRUCTURE ONLY: the checker of the device
 * post-processing (openbcsim_gb300/csrc/imaging.cu); part of liboracle.so.
 *
 *   oracle_max_value          bcsim::get_max_value            src/utils/BCSimConvenience.cpp:57-63
 *   oracle_envelope           std::abs of each IQ sample       src/qt5gui/RefreshWorker.hpp:185-196
 *   oracle_log_compress       bcsim::log_compress_frame        src/utils/BCSimConvenience.cpp:65-83
 *                             and the byte conversion          src/qt5gui/RefreshWorker.hpp:226-236
 *   oracle_scan_convert_*     CpuCartesianator<T>::Do{Sector,Linear}Transform
 *                                                              src/utils/cartesianator/Cartesianator.cpp:107-205
 *                             with the extents of              src/utils/ScanGeometry.hpp:44-78
 *   oracle_color_doppler      R0 / arg R1 estimation           src/qt5gui/RefreshWorker.hpp:262-306
 *   oracle_color_image        normalise, threshold, colour map src/qt5gui/RefreshWorker.hpp:309-395
 *
 * Float expressions follow the reference's operation order; compiled with
 * -ffp-contract=off (oracle/Makefile) so that nothing is fused.  The libm calls
 * (cabsf, log10f, atan2f, cosf) are the ones the reference makes through
 * std::abs / std::log10 / std::atan2 / std::cos of float arguments.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>

/* static_cast<unsigned char>(float) as x86 performs it: truncation to a 32-bit
 * integer (INT_MIN when out of range or NaN), then the low byte. */
static uint8_t to_byte(float v) {
    int32_t i;
    if (v != v || v >= 2147483648.0f || v < -2147483648.0f) i = INT32_MIN;
    else i = (int32_t)v;
    return (uint8_t)(uint32_t)i;
}

float oracle_max_value(const float* v, int64_t n) {
    float m = v[0];
    for (int64_t i = 1; i < n; i++)
        if (v[i] > m) m = v[i];
    return m;
}

void oracle_envelope(const float* iq, int64_t n, float* env) {
    for (int64_t i = 0; i < n; i++) env[i] = cabsf(iq[2 * i] + I * iq[2 * i + 1]);
}

void oracle_log_compress(const float* env, int64_t n, float dyn_range, float normalize, float gain, float* out_f,
                         uint8_t* out_b) {
    for (int64_t i = 0; i < n; i++) {
        float pixel = env[i];
        pixel = (float)(20.0 * log10f(gain * pixel / normalize));
        pixel = (float)((255.0 / dyn_range) * (pixel + dyn_range));
        if (pixel < 0.0f) pixel = 0.0f;
        if (pixel >= 255.0f) pixel = 255.0f;
        if (out_f) out_f[i] = pixel;
        if (out_b) out_b[i] = to_byte(pixel);
    }
}

/* Extents and grid of the Cartesianator for a geometry (kind 0: sector, 1: linear). */
typedef struct {
    float x_min, x_max, y_min, y_max;
    float theta_min, theta_max; /* sector */
} extent_t;

static extent_t geometry_extent(int kind, float width, float depth, float tilt) {
    extent_t e;
    if (kind == 0) {
        const float PI = (float)(4.0 * atanf(1.0f));
        e.theta_min = 0.5f * PI - 0.5f * width + tilt;
        e.theta_max = 0.5f * PI + 0.5f * width + tilt;
        e.x_min = (float)(depth * cosf(e.theta_max));
        e.x_max = (float)(depth * cosf(e.theta_min));
        e.y_min = 0.0f;
        e.y_max = depth;
    } else {
        e.x_min = -0.5f * width;
        e.x_max = 0.5f * width;
        e.y_min = 0.0f;
        e.y_max = depth;
        e.theta_min = e.theta_max = 0.0f;
    }
    return e;
}

/* One output pixel of either transform, samples read through get(beam, range). */
#define SCAN_BODY(GET)                                                                                        \
    const extent_t E = geometry_extent(kind, width, depth, tilt);                                             \
    const float dx = (E.x_max - E.x_min) / (float)(nx - 1);                                                   \
    const float dy = (E.y_max - E.y_min) / (float)(ny - 1);                                                   \
    for (int xi = 0; xi < nx; xi++) {                                                                         \
        for (int yi = 0; yi < ny; yi++) {                                                                     \
            const float x = E.x_min + (float)xi * dx;                                                         \
            const float y = E.y_min + (float)yi * dy;                                                         \
            float value;                                                                                      \
            if (kind == 0) {                                                                                  \
                const float range_min = 0.0f, range_max = depth;                                             \
                const float dr = (range_max - range_min) / (range - 1);                                       \
                const float dt = (E.theta_max - E.theta_min) / (beams - 1);                                   \
                const float r = sqrtf(x * x + y * y);                                                         \
                float theta;                                                                                  \
                if (fabsf(x) > 1e-6) theta = atan2f(y, x);                                                    \
                else theta = (float)(atan(1) * 2);                                                            \
                const int r_idx0 = (int)floorf((r - range_min) / dr);                                         \
                const int t_idx0 = (int)floorf((theta - E.theta_min) / dt);                                   \
                const int r_idx1 = r_idx0 + 1, t_idx1 = t_idx0 + 1;                                           \
                const float s00 = (r_idx0 >= 0 && r_idx0 < range && t_idx0 >= 0 && t_idx0 < beams) ? GET(t_idx0, r_idx0) : 0.0f; \
                const float s01 = (r_idx0 >= 0 && r_idx0 < range && t_idx1 >= 0 && t_idx1 < beams) ? GET(t_idx1, r_idx0) : 0.0f; \
                const float s10 = (r_idx1 >= 0 && r_idx1 < range && t_idx0 >= 0 && t_idx0 < beams) ? GET(t_idx0, r_idx1) : 0.0f; \
                const float s11 = (r_idx1 >= 0 && r_idx1 < range && t_idx1 >= 0 && t_idx1 < beams) ? GET(t_idx1, r_idx1) : 0.0f; \
                const float range0 = range_min + r_idx0 * dr;                                                 \
                const float range1 = range0 + dr;                                                             \
                const float theta0 = E.theta_min + t_idx0 * dt;                                               \
                const float theta1 = theta0 + dt;                                                             \
                value = 1.0f / ((range1 - range0) * (theta1 - theta0)) *                                      \
                        (s00 * (range1 - r) * (theta1 - theta) + s10 * (r - range0) * (theta1 - theta) +      \
                         s01 * (range1 - r) * (theta - theta0) + s11 * (r - range0) * (theta - theta0));      \
            } else {                                                                                          \
                const float bx_min = -0.5f * width, bx_max = 0.5f * width, by_min = 0.0f, by_max = depth;     \
                const float bs_dx = (bx_max - bx_min) / (beams - 1);                                          \
                const float bs_dy = (by_max - by_min) / (range - 1);                                          \
                const int x_idx0 = (int)floorf((x - bx_min) / bs_dx);                                         \
                const int y_idx0 = (int)floorf((y - by_min) / bs_dy);                                         \
                const int x_idx1 = x_idx0 + 1, y_idx1 = y_idx0 + 1;                                           \
                const float s00 = (y_idx0 >= 0 && y_idx0 < range && x_idx0 >= 0 && x_idx0 < beams) ? GET(x_idx0, y_idx0) : 0.0f; \
                const float s01 = (y_idx0 >= 0 && y_idx0 < range && x_idx1 >= 0 && x_idx1 < beams) ? GET(x_idx1, y_idx0) : 0.0f; \
                const float s10 = (y_idx1 >= 0 && y_idx1 < range && x_idx0 >= 0 && x_idx0 < beams) ? GET(x_idx0, y_idx1) : 0.0f; \
                const float s11 = (y_idx1 >= 0 && y_idx1 < range && x_idx1 >= 0 && x_idx1 < beams) ? GET(x_idx1, y_idx1) : 0.0f; \
                const float y0 = by_min + y_idx0 * bs_dy;                                                     \
                const float y1 = y0 + bs_dy;                                                                  \
                const float x0 = bx_min + x_idx0 * bs_dx;                                                     \
                const float x1 = x0 + bs_dx;                                                                  \
                value = 1.0f / ((y1 - y0) * (x1 - x0)) *                                                      \
                        (s00 * (y1 - y) * (x1 - x) + s10 * (y - y0) * (x1 - x) + s01 * (y1 - y) * (x - x0) +  \
                         s11 * (y - y0) * (x - x0));                                                          \
            }                                                                                                 \
            STORE((int64_t)nx * yi + xi, value);                                                              \
        }                                                                                                     \
    }

void oracle_scan_convert_f32(const float* in, int beams, int range, int kind, float width, float depth, float tilt,
                             int nx, int ny, float* out) {
#define GET(b, r) in[(int64_t)range * (b) + (r)]
#define STORE(i, v) out[i] = (v)
    SCAN_BODY(GET)
#undef GET
#undef STORE
}

void oracle_scan_convert_u8(const uint8_t* in, int beams, int range, int kind, float width, float depth, float tilt,
                            int nx, int ny, uint8_t* out) {
#define GET(b, r) (float)in[(int64_t)range * (b) + (r)]
#define STORE(i, v) out[i] = to_byte(v)
    SCAN_BODY(GET)
#undef GET
#undef STORE
}

/* packet: complex64 [P][n] interleaved; r0 / vel: [n] */
void oracle_color_doppler(const float* packet, int P, int64_t n, float* r0_out, float* vel_out) {
    for (int64_t i = 0; i < n; i++) {
        float r0 = 0.0f, r1r = 0.0f, r1i = 0.0f;
        float mr = 0.0f, mi = 0.0f;
        for (int k = 0; k < P; k++) {
            mr += packet[2 * ((int64_t)k * n + i)];
            mi += packet[2 * ((int64_t)k * n + i) + 1];
        }
        mr = mr / (float)P;
        mi = mi / (float)P;
        for (int k = 0; k < P; k++) {
            const float a = packet[2 * ((int64_t)k * n + i)] - mr;
            const float b = packet[2 * ((int64_t)k * n + i) + 1] - mi;
            /* (z * conj(z)).real() with conj(z) = (a, -b): a*a - b*(-b) */
            r0 += a * a - b * (-b);
        }
        for (int k = 0; k < P - 1; k++) {
            const float pr = packet[2 * ((int64_t)k * n + i)], pi = -packet[2 * ((int64_t)k * n + i) + 1];
            const float xr = packet[2 * ((int64_t)(k + 1) * n + i)], xi = packet[2 * ((int64_t)(k + 1) * n + i) + 1];
            r1r += pr * xr - pi * xi;
            r1i += pr * xi + pi * xr;
        }
        r0_out[i] = r0;
        vel_out[i] = atan2f(r1i, r1r);
    }
}

void oracle_color_image(const float* r0, const float* vel, int beams, int range, int kind, float width, float depth,
                        float tilt, int nx, int ny, float* work_power, float* work_vel, float* work_beam,
                        uint8_t* bgra) {
    const int64_t n = (int64_t)beams * range;
    const float mx = oracle_max_value(r0, n);
    for (int64_t i = 0; i < n; i++) work_beam[i] = r0[i] / mx;
    oracle_scan_convert_f32(work_beam, beams, range, kind, width, depth, tilt, nx, ny, work_power);
    oracle_scan_convert_f32(vel, beams, range, kind, width, depth, tilt, nx, ny, work_vel);
    for (int64_t i = 0; i < (int64_t)nx * ny; i++) {
        uint8_t alpha = 0, red = 0, green = 0, blue = 0;
        if (work_power[i] >= 0.001f) {
            const float phase_angle = work_vel[i];
            const uint8_t cv = to_byte(255.0f * fabsf(phase_angle) / 3.14159f);
            alpha = 255;
            if (phase_angle >= 0.0) red = cv;
            else blue = cv;
        }
        bgra[4 * i + 3] = alpha;
        bgra[4 * i + 2] = red;
        bgra[4 * i + 1] = green;
        bgra[4 * i + 0] = blue;
    }
}
