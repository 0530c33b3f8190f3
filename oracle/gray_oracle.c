/*
 * gray_oracle.c -- CPU restatement of GRay's differentiable Gaussian ray tracer.
 *
 * TEST INFRASTRUCTURE ONLY (the checker for gray_gb300's CUDA path; see gray_oracle.h).
 * Build: oracle/Makefile (gcc -O2 -ffp-contract=off -fPIC -shared -pthread).
 *
 * Reference routines restated here (paths inside graphdeco-inria/gray):
 *   cuda/utils/kernel.cu:3-42         scaling factor, Gaussian response, alpha
 *   cuda/utils/activations.cu:5-70    sigmoid / exp / normalize activations and their backward
 *   cuda/optix/bvh_wrapper.cu:8-59    instance transform and visibility (snapshot)
 *   cuda/core/camera.h:17-36          primary ray generation
 *   cuda/shaders.cu:10-67             intersection program (hit test, full transmittance, hit log)
 *   cuda/core/per_pixel_linked_list.h:21-32   fp16 rounding of distance and alpha
 *   cuda/forward_pass.cu:6-151        32-slot multi-pass selection and compositing
 *   cuda/backward_pass.cu:2-142       reverse replay and gradients
 *   cuda/utils/sh.cu:224-304          SH colour forward and backward
 *   cuda/opt/adam.cu:6-83             fused Adam
 * Deliberate, documented differences from the reference (shared with the CUDA path):
 *   - the all-hit "skipped" sums (forward_pass.cu:50-56, 92-93) are accumulated exactly in
 *     64-bit fixed point (alpha16 in 2^-24 units times the colour in 2^-24 units, clamped to
 *     [-64, 64]) instead of an order-dependent fp32 running sum;
 *   - the full transmittance (shaders.cu:55-56, an fp32 product in traversal order) is the
 *     exponential of a fixed-point sum of log(1 - alpha), so it does not depend on the order;
 *   - hits with equal fp16 distance are ordered by gaussian id (the reference uses OptiX
 *     traversal order, which is not reproducible);
 *   - IEEE division/sqrt and this file's own exp/log instead of --use_fast_math intrinsics;
 *   - the object-space ray is M (o - mu) with M = diag(1/s) R^T instead of OptiX's numeric
 *     inverse of the 3x4 instance transform.
 */
#include "gray_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

static inline uint32_t f2u(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}
static inline float u2f(uint32_t u) {
    float f;
    memcpy(&f, &u, 4);
    return f;
}

/* ------------------------------------------------------------------------------------------ */
/* exp: Cody & Waite argument reduction (x = k ln2 + r, |r| <= ln2/2, ln2 split in two floats)  */
/* followed by the degree-7 Taylor polynomial of e^r in Horner form.                          */
/* ------------------------------------------------------------------------------------------ */
float orc_expf(float x) {
    if (x != x) return x;
    if (x > 89.0f) return INFINITY;
    if (x < -104.0f) return 0.0f;
    float k = rintf(x * 0x1.715476p+0f);
    float r = fmaf(-k, 0x1.62ep-1f, x);
    r = fmaf(-k, 0x1.0bfbe8p-15f, r);
    float p = 0x1.a01a02p-13f;
    p = fmaf(p, r, 0x1.6c16c2p-10f);
    p = fmaf(p, r, 0x1.111112p-7f);
    p = fmaf(p, r, 0x1.555556p-5f);
    p = fmaf(p, r, 0x1.555556p-3f);
    p = fmaf(p, r, 0x1.0p-1f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    int ki = (int)k;
    if (ki > 127) {
        p = p * 2.0f;
        ki -= 1;
    }
    if (ki < -126) {
        p = p * u2f((uint32_t)(ki + 64 + 127) << 23);
        return p * 0x1.0p-64f;
    }
    return p * u2f((uint32_t)(ki + 127) << 23);
}

/* log: x = m 2^e with m in [sqrt(1/2), sqrt(2)], log m = 2 atanh(s), s = (m-1)/(m+1),     */
/* atanh series to s^11, then e ln2 added with the same two-float split of ln2.              */
float orc_logf(float x) {
    if (x != x) return x;
    if (x < 0.0f) return NAN;
    if (x == 0.0f) return -INFINITY;
    if (x == INFINITY) return x;
    uint32_t u = f2u(x);
    int e = 0;
    if (u < 0x00800000u) {
        x = x * 0x1.0p23f;
        u = f2u(x);
        e = -23;
    }
    e += (int)(u >> 23) - 127;
    float m = u2f((u & 0x007fffffu) | 0x3f800000u);
    if (m > 0x1.6a09e6p+0f) {
        m = m * 0.5f;
        e += 1;
    }
    float f = m - 1.0f;
    float s = f / (2.0f + f);
    float z = s * s;
    float q = 0x1.745d18p-4f;
    q = fmaf(q, z, 0x1.c71c72p-4f);
    q = fmaf(q, z, 0x1.24924ap-3f);
    q = fmaf(q, z, 0x1.99999ap-3f);
    q = fmaf(q, z, 0x1.555556p-2f);
    float two_s = 2.0f * s;
    float lm = fmaf(two_s * z, q, two_s);
    float ef = (float)e;
    return fmaf(ef, 0x1.62ep-1f, fmaf(ef, 0x1.0bfbe8p-15f, lm));
}

static inline float orc_powf(float a, float b) { return orc_expf(b * orc_logf(a)); }

/* float -> binary16, round to nearest even (matches the hardware cvt.rn.f16.f32) */
uint16_t orc_f2h(float f) {
    uint32_t x = f2u(f);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t ax = x & 0x7fffffffu;
    if (ax >= 0x7f800000u) return (uint16_t)(sign | (ax > 0x7f800000u ? 0x7e00u : 0x7c00u));
    if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);
    if (ax <= 0x33000000u) return (uint16_t)sign;
    if (ax < 0x38800000u) {
        uint32_t m = (ax & 0x7fffffu) | 0x800000u;
        int sh = 126 - (int)(ax >> 23);
        uint32_t mh = m >> sh;
        uint32_t rem = m & ((1u << sh) - 1u);
        uint32_t half = 1u << (sh - 1);
        if (rem > half || (rem == half && (mh & 1u))) mh++;
        return (uint16_t)(sign | mh);
    }
    uint32_t r = ax - 0x38000000u;
    uint32_t mh = r >> 13;
    uint32_t rem = r & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (mh & 1u))) mh++;
    return (uint16_t)(sign | mh);
}

float orc_h2f(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 0x1fu;
    uint32_t m = h & 0x3ffu;
    if (e == 0) {
        float v = (float)m * 0x1.0p-24f;
        return sign ? -v : v;
    }
    if (e == 31) return u2f(sign | 0x7f800000u | (m << 13));
    return u2f(sign | ((e + 112u) << 23) | (m << 13));
}

/* MAX_ALPHA (the double literal 0.9999) times a times b, rounded once to float.  The product */
/* a*b is split exactly with an FMA and 0.9999 is carried as a float pair.                    */
float orc_maxalpha_mul(float a, float b) {
    const float c_hi = 0x1.fff2e4p-1f, c_lo = 0x1.1d14e4p-26f;
    float p = a * b;
    float e = fmaf(a, b, -p);
    return fmaf(c_hi, p, fmaf(c_hi, e, c_lo * p));
}

/* beta^n rounded to float; computed by binary exponentiation in double */
float orc_adam_pow(float beta, int n) {
    double b = (double)beta, r = 1.0;
    unsigned int k = (unsigned int)(n < 0 ? 0 : n);
    while (k) {
        if (k & 1u) r *= b;
        b *= b;
        k >>= 1;
    }
    return (float)r;
}

static inline float sigmoid_act(float x) { return 1.0f / (1.0f + orc_expf(-x)); }

/* cuda/utils/kernel.cu:3-22 */
float orc_scaling_factor(float opacity, float alpha_threshold, float exp_power) {
    if (opacity <= alpha_threshold) return 0.0f;
    float log_ratio = orc_logf(opacity / alpha_threshold);
    if (exp_power == 1.0f) return sqrtf(2.0f * log_ratio);
    if (exp_power == 2.0f) return sqrtf(sqrtf(4.0f * log_ratio));
    if (exp_power == 3.0f) {
        float v = sqrtf(6.0f * log_ratio);
        return v == 0.0f ? 0.0f : orc_expf(orc_logf(v) * 0x1.555556p-2f);
    }
    float k = 2.0f * exp_power;
    return orc_powf(k * log_ratio, 1.0f / k);
}

/* cuda/utils/kernel.cu:24-38, with d = |x|^2 */
static inline float eval_gaussian(float d, float exp_power) {
    if (exp_power == 1.0f) return orc_expf(-0.5f * d);
    if (exp_power == 2.0f) return orc_expf(-0.25f * d * d);
    if (exp_power == 3.0f) return orc_expf(-(d * d * d) / 6.0f);
    float k = 2.0f * exp_power;
    return orc_expf(-orc_powf(d, exp_power) / k);
}

float orc_eval_gaussian(float d, float exp_power) { return eval_gaussian(d, exp_power); }

/* ------------------------------------------------------------------------------------------ */
/* snapshot: cuda/optix/bvh_wrapper.cu:8-59                                                   */
/* ------------------------------------------------------------------------------------------ */
static void quat_to_rows(const float *q, float R[9]) {
    float r = q[0], x = q[1], y = q[2], z = q[3];
    float norm = sqrtf(r * r + x * x + y * y + z * z);
    r = r / norm;
    x = x / norm;
    y = y / norm;
    z = z / norm;
    R[0] = 1.0f - 2.0f * (y * y + z * z);
    R[1] = 2.0f * (x * y - r * z);
    R[2] = 2.0f * (x * z + r * y);
    R[3] = 2.0f * (x * y + r * z);
    R[4] = 1.0f - 2.0f * (x * x + z * z);
    R[5] = 2.0f * (y * z - r * x);
    R[6] = 2.0f * (x * z - r * y);
    R[7] = 2.0f * (y * z + r * x);
    R[8] = 1.0f - 2.0f * (x * x + y * y);
}

void orc_snapshot(int n, const float *mean, const float *rotation, const float *scale, const float *opacity,
                  float alpha_threshold, float exp_power, float gsf, float *geom, float *l2w, float *aabb,
                  uint8_t *visible) {
    for (int i = 0; i < n; i++) {
        float o = sigmoid_act(opacity[i]);
        float sf = orc_scaling_factor(o, alpha_threshold, exp_power);
        float s[3];
        for (int k = 0; k < 3; k++) s[k] = orc_expf(scale[3 * i + k]) * sf * gsf;
        float R[9];
        quat_to_rows(rotation + 4 * i, R);
        const float *mu = mean + 3 * i;
        int vis = sf > 0.0f && s[0] > 0.0f && s[1] > 0.0f && s[2] > 0.0f && isfinite(s[0]) && isfinite(s[1]) &&
                  isfinite(s[2]) && isfinite(mu[0]) && isfinite(mu[1]) && isfinite(mu[2]);
        float *g = geom + 12 * i;
        float *L = l2w + 12 * i;
        for (int r = 0; r < 3; r++) {
            for (int c = 0; c < 3; c++) {
                g[4 * r + c] = vis ? R[3 * c + r] / s[r] : 0.0f;
                L[4 * r + c] = R[3 * r + c] * s[c];
            }
            g[4 * r + 3] = mu[r];
            L[4 * r + 3] = mu[r];
        }
        float *b = aabb + 8 * i;
        if (vis) {
            float pad_mu = 2.0e-6f * (fabsf(mu[0]) + fabsf(mu[1]) + fabsf(mu[2]));
            for (int r = 0; r < 3; r++) {
                float a0 = L[4 * r + 0], a1 = L[4 * r + 1], a2 = L[4 * r + 2];
                float h = sqrtf(a0 * a0 + a1 * a1 + a2 * a2);
                h = h + h * 1.0e-4f + pad_mu + 1.0e-30f;
                b[r] = mu[r] - h;
                b[4 + r] = mu[r] + h;
            }
        } else {
            for (int r = 0; r < 3; r++) {
                float c = isfinite(mu[0]) && isfinite(mu[1]) && isfinite(mu[2]) ? mu[r] : 0.0f;
                b[r] = c;
                b[4 + r] = c;
            }
        }
        b[3] = 0.0f;
        b[7] = 0.0f;
        visible[i] = (uint8_t)vis;
    }
}

void orc_forward_prep(int n, const float *opacity, float alpha_threshold, float exp_power, float *live) {
    for (int i = 0; i < n; i++) {
        float o = sigmoid_act(opacity[i]);
        live[2 * i] = o;
        live[2 * i + 1] = orc_scaling_factor(o, alpha_threshold, exp_power);
    }
}

/* ------------------------------------------------------------------------------------------ */
/* camera: cuda/core/camera.h:17-36 (no jitter); c2w row-major 3x3, w2c rows = c2w columns     */
/* ------------------------------------------------------------------------------------------ */
void orc_camera_rays(int width, int height, float fov_y, const float *origin, const float *c2w, float *ray_o,
                     float *ray_d) {
    float view_size = tanf(fov_y / 2.0f);
    float aspect = (float)width / (float)height;
    for (int j = 0; j < height; j++) {
        for (int i = 0; i < width; i++) {
            float y = view_size * (1.0f - 2.0f * ((float)j + 0.5f) / (float)height);
            float x = aspect * view_size * (2.0f * ((float)i + 0.5f) / (float)width - 1.0f);
            float v[3];
            for (int k = 0; k < 3; k++) v[k] = c2w[3 * k + 0] * x + c2w[3 * k + 1] * y - c2w[3 * k + 2];
            float inv = 1.0f / sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            size_t p = (size_t)j * width + i;
            for (int k = 0; k < 3; k++) {
                ray_d[3 * p + k] = v[k] * inv;
                ray_o[3 * p + k] = origin[k];
            }
        }
    }
}

/* ------------------------------------------------------------------------------------------ */
/* SH colour (cuda/utils/sh.cu:224-304), real basis in closed polynomial form                 */
/* ------------------------------------------------------------------------------------------ */
#define SH_C0 0.28209479177387814f
#define SH_C1 0.48860251190291992f
#define SH_C2_0 1.0925484305920792f
#define SH_C2_2 0.31539156525252005f
#define SH_C2_4 0.54627421529603959f
#define SH_C3_0 0.59004358992664352f
#define SH_C3_1 2.8906114426405538f
#define SH_C3_2 0.45704579946446572f
#define SH_C3_3 0.3731763325901154f
#define SH_C3_5 1.4453057213202769f

static void sh_basis(float x, float y, float z, float b[15]) {
    float xx = x * x, yy = y * y, zz = z * z;
    b[0] = -SH_C1 * y;
    b[1] = SH_C1 * z;
    b[2] = -SH_C1 * x;
    b[3] = SH_C2_0 * (x * y);
    b[4] = -SH_C2_0 * (y * z);
    b[5] = SH_C2_2 * (2.0f * zz - xx - yy);
    b[6] = -SH_C2_0 * (x * z);
    b[7] = SH_C2_4 * (xx - yy);
    b[8] = -SH_C3_0 * (y * (3.0f * xx - yy));
    b[9] = SH_C3_1 * (x * y * z);
    b[10] = -SH_C3_2 * (y * (4.0f * zz - xx - yy));
    b[11] = SH_C3_3 * (z * (2.0f * zz - 3.0f * xx - 3.0f * yy));
    b[12] = -SH_C3_2 * (x * (4.0f * zz - xx - yy));
    b[13] = SH_C3_5 * (z * (xx - yy));
    b[14] = -SH_C3_0 * (x * (xx - 3.0f * yy));
}

/* d b_i / d(x, y, z) treating the three direction components as independent */
static void sh_basis_grad(float x, float y, float z, float dx[15], float dy[15], float dz[15]) {
    float xx = x * x, yy = y * y, zz = z * z;
    dx[0] = 0.0f;           dy[0] = -SH_C1;         dz[0] = 0.0f;
    dx[1] = 0.0f;           dy[1] = 0.0f;           dz[1] = SH_C1;
    dx[2] = -SH_C1;         dy[2] = 0.0f;           dz[2] = 0.0f;
    dx[3] = SH_C2_0 * y;    dy[3] = SH_C2_0 * x;    dz[3] = 0.0f;
    dx[4] = 0.0f;           dy[4] = -SH_C2_0 * z;   dz[4] = -SH_C2_0 * y;
    dx[5] = SH_C2_2 * (-2.0f * x); dy[5] = SH_C2_2 * (-2.0f * y); dz[5] = SH_C2_2 * (4.0f * z);
    dx[6] = -SH_C2_0 * z;   dy[6] = 0.0f;           dz[6] = -SH_C2_0 * x;
    dx[7] = SH_C2_4 * (2.0f * x); dy[7] = SH_C2_4 * (-2.0f * y); dz[7] = 0.0f;
    dx[8] = -SH_C3_0 * (6.0f * x * y);
    dy[8] = -SH_C3_0 * (3.0f * xx - 3.0f * yy);
    dz[8] = 0.0f;
    dx[9] = SH_C3_1 * (y * z);
    dy[9] = SH_C3_1 * (x * z);
    dz[9] = SH_C3_1 * (x * y);
    dx[10] = -SH_C3_2 * (-2.0f * x * y);
    dy[10] = -SH_C3_2 * (4.0f * zz - xx - 3.0f * yy);
    dz[10] = -SH_C3_2 * (8.0f * y * z);
    dx[11] = SH_C3_3 * (-6.0f * x * z);
    dy[11] = SH_C3_3 * (-6.0f * y * z);
    dz[11] = SH_C3_3 * (6.0f * zz - 3.0f * xx - 3.0f * yy);
    dx[12] = -SH_C3_2 * (4.0f * zz - 3.0f * xx - yy);
    dy[12] = -SH_C3_2 * (-2.0f * x * y);
    dz[12] = -SH_C3_2 * (8.0f * x * z);
    dx[13] = SH_C3_5 * (2.0f * x * z);
    dy[13] = SH_C3_5 * (-2.0f * y * z);
    dz[13] = SH_C3_5 * (xx - yy);
    dx[14] = -SH_C3_0 * (3.0f * xx - 3.0f * yy);
    dy[14] = -SH_C3_0 * (-6.0f * x * y);
    dz[14] = 0.0f;
}

static inline int sh_count(int degree) { return degree <= 0 ? 0 : degree == 1 ? 3 : degree == 2 ? 8 : 15; }

void orc_sh_forward(int n, int degree, int num_rest, const float *mean, const float *cam, const float *sh_dc,
                    const float *sh_rest, float *channels) {
    if (degree > 3) degree = 3;
    int nb = sh_count(degree);
    for (int i = 0; i < n; i++) {
        float v[3];
        for (int k = 0; k < 3; k++) v[k] = mean[3 * i + k] - cam[k];
        float len2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
        float inv = 1.0f / sqrtf(fmaxf(len2, 1e-20f));
        float b[15];
        sh_basis(v[0] * inv, v[1] * inv, v[2] * inv, b);
        for (int c = 0; c < 3; c++) {
            float acc = SH_C0 * sh_dc[3 * i + c];
            for (int j = 0; j < nb; j++) acc = fmaf(b[j], sh_rest[((size_t)i * num_rest + j) * 3 + c], acc);
            acc = acc + 0.5f;
            channels[3 * i + c] = fmaxf(acc, 0.0f);
        }
    }
}

void orc_sh_backward(int n, int degree, int num_rest, const float *mean, const float *cam, const float *sh_rest,
                     const float *channels, const float *grad_channels, const uint8_t *was_visible,
                     float *grad_sh_dc, float *grad_sh_rest, float *grad_mean) {
    if (degree > 3) degree = 3;
    int nb = sh_count(degree);
    for (int i = 0; i < n; i++) {
        if (!was_visible[i]) continue;
        float v[3];
        for (int k = 0; k < 3; k++) v[k] = mean[3 * i + k] - cam[k];
        float len2 = fmaxf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2], 1e-20f);
        float inv = 1.0f / sqrtf(len2);
        float x = v[0] * inv, y = v[1] * inv, z = v[2] * inv;
        float g[3];
        for (int c = 0; c < 3; c++) g[c] = channels[3 * i + c] <= 0.0f ? 0.0f : grad_channels[3 * i + c];
        for (int c = 0; c < 3; c++) grad_sh_dc[3 * i + c] = SH_C0 * g[c];
        float b[15], dx[15], dy[15], dz[15];
        sh_basis(x, y, z, b);
        sh_basis_grad(x, y, z, dx, dy, dz);
        float gd[3] = {0.0f, 0.0f, 0.0f};
        for (int j = 0; j < nb; j++) {
            const float *cf = sh_rest + ((size_t)i * num_rest + j) * 3;
            float *gr = grad_sh_rest + ((size_t)i * num_rest + j) * 3;
            for (int c = 0; c < 3; c++) gr[c] = b[j] * g[c];
            float gc = cf[0] * g[0] + cf[1] * g[1] + cf[2] * g[2];
            gd[0] = fmaf(dx[j], gc, gd[0]);
            gd[1] = fmaf(dy[j], gc, gd[1]);
            gd[2] = fmaf(dz[j], gc, gd[2]);
        }
        float inv3 = inv * inv * inv;
        float dv = v[0] * gd[0] + v[1] * gd[1] + v[2] * gd[2];
        for (int k = 0; k < 3; k++) grad_mean[3 * i + k] = grad_mean[3 * i + k] + (gd[k] * inv - v[k] * (dv * inv3));
    }
}

/* ------------------------------------------------------------------------------------------ */
/* LBVH: Morton codes, stable key sort, Karras (2012) hierarchy, bottom-up boxes              */
/* ------------------------------------------------------------------------------------------ */
static uint32_t expand10(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

typedef struct {
    uint32_t key, id;
} keyid;
static int cmp_keyid(const void *a, const void *b) {
    const keyid *x = (const keyid *)a, *y = (const keyid *)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return x->id < y->id ? -1 : (x->id > y->id);
}

static inline int clz32(uint32_t v) { return v ? __builtin_clz(v) : 32; }
static inline int lbvh_delta(const uint32_t *codes, int n, int i, int j) {
    if (j < 0 || j > n - 1) return -1;
    uint32_t a = codes[i], b = codes[j];
    if (a == b) return 32 + clz32((uint32_t)i ^ (uint32_t)j);
    return clz32(a ^ b);
}

#define LEAF_BIT 0x80000000u

void orc_lbvh_build(int n, const float *aabb, const uint8_t *visible, orc_bvh *out) {
    (void)visible;
    memset(out, 0, sizeof(*out));
    out->n = n;
    if (n <= 0) return;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = 0; i < n; i++) {
        const float *b = aabb + 8 * i;
        float c[3];
        int fin = 1;
        for (int k = 0; k < 3; k++) {
            c[k] = (b[k] + b[4 + k]) * 0.5f;
            fin = fin && isfinite(c[k]);
        }
        if (!fin) continue;
        for (int k = 0; k < 3; k++) {
            lo[k] = fminf(lo[k], c[k]);
            hi[k] = fmaxf(hi[k], c[k]);
        }
    }
    keyid *kv = (keyid *)malloc(sizeof(keyid) * (size_t)n);
    for (int i = 0; i < n; i++) {
        const float *b = aabb + 8 * i;
        uint32_t q[3];
        int fin = 1;
        for (int k = 0; k < 3; k++) {
            float c = (b[k] + b[4 + k]) * 0.5f;
            fin = fin && isfinite(c);
            float ext = hi[k] - lo[k];
            float t = ext > 0.0f ? (c - lo[k]) / ext : 0.0f;
            float s = fminf(fmaxf(t * 1024.0f, 0.0f), 1023.0f);
            q[k] = fin ? (uint32_t)s : 0u;
        }
        kv[i].key = fin ? ((expand10(q[0]) << 2) | (expand10(q[1]) << 1) | expand10(q[2])) : 0x40000000u;
        kv[i].id = (uint32_t)i;
    }
    qsort(kv, (size_t)n, sizeof(keyid), cmp_keyid);
    out->codes = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n);
    out->order = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n);
    out->leaf_parent = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    for (int i = 0; i < n; i++) {
        out->codes[i] = kv[i].key;
        out->order[i] = kv[i].id;
        out->leaf_parent[i] = -1;
    }
    free(kv);
    int ni = n - 1;
    out->nodes = (float *)calloc((size_t)(ni > 0 ? ni : 1) * 16, sizeof(float));
    out->int_parent = (int32_t *)malloc(sizeof(int32_t) * (size_t)(ni > 0 ? ni : 1));
    for (int i = 0; i < ni; i++) out->int_parent[i] = -1;
    const uint32_t *codes = out->codes;
    for (int i = 0; i < ni; i++) {
        int d = lbvh_delta(codes, n, i, i + 1) - lbvh_delta(codes, n, i, i - 1) >= 0 ? 1 : -1;
        int dmin = lbvh_delta(codes, n, i, i - d);
        int lmax = 2;
        while (lbvh_delta(codes, n, i, i + lmax * d) > dmin) lmax *= 2;
        int l = 0;
        for (int t = lmax / 2; t >= 1; t /= 2)
            if (lbvh_delta(codes, n, i, i + (l + t) * d) > dmin) l += t;
        int j = i + l * d;
        int dnode = lbvh_delta(codes, n, i, j);
        int s = 0;
        int t = l;
        do {
            t = (t + 1) / 2;
            if (lbvh_delta(codes, n, i, i + (s + t) * d) > dnode) s += t;
        } while (t > 1);
        int gamma = i + s * d + (d < 0 ? d : 0);
        int lo_i = i < j ? i : j, hi_i = i < j ? j : i;
        uint32_t c0, c1;
        if (lo_i == gamma) {
            c0 = out->order[gamma] | LEAF_BIT;
            out->leaf_parent[gamma] = i;
        } else {
            c0 = (uint32_t)gamma;
            out->int_parent[gamma] = i;
        }
        if (hi_i == gamma + 1) {
            c1 = out->order[gamma + 1] | LEAF_BIT;
            out->leaf_parent[gamma + 1] = i;
        } else {
            c1 = (uint32_t)(gamma + 1);
            out->int_parent[gamma + 1] = i;
        }
        float *nd = out->nodes + 16 * (size_t)i;
        uint32_t leaves = (uint32_t)(hi_i - lo_i + 1); /* word 14: leaves below the node */
        uint32_t leaves0 = (uint32_t)(gamma - lo_i + 1); /* word 15: leaves below child 0 */
        memcpy(nd + 12, &c0, 4);
        memcpy(nd + 13, &c1, 4);
        memcpy(nd + 14, &leaves, 4);
        memcpy(nd + 15, &leaves0, 4);
    }
    orc_lbvh_refit(out, aabb);
}

static void refit_node(orc_bvh *b, const float *aabb, int i, float box[6]) {
    float *nd = b->nodes + 16 * (size_t)i;
    uint32_t c[2];
    memcpy(&c[0], nd + 12, 4);
    memcpy(&c[1], nd + 13, 4);
    for (int s = 0; s < 2; s++) {
        float cb[6];
        if (c[s] & LEAF_BIT) {
            const float *a = aabb + 8 * (size_t)(c[s] & ~LEAF_BIT);
            for (int k = 0; k < 3; k++) {
                cb[k] = a[k];
                cb[3 + k] = a[4 + k];
            }
        } else {
            refit_node(b, aabb, (int)c[s], cb);
        }
        memcpy(nd + 6 * s, cb, sizeof(cb));
    }
    for (int k = 0; k < 3; k++) {
        box[k] = fminf(nd[k], nd[6 + k]);
        box[3 + k] = fmaxf(nd[3 + k], nd[9 + k]);
    }
}
void orc_lbvh_refit(orc_bvh *b, const float *aabb) {
    if (b->n <= 0) return;
    float box[6];
    if (b->n == 1) {
        const float *a = aabb + 8 * (size_t)b->order[0];
        for (int k = 0; k < 3; k++) {
            box[k] = a[k];
            box[3 + k] = a[4 + k];
        }
    } else {
        refit_node(b, aabb, 0, box);
    }
    for (int k = 0; k < 3; k++) {
        b->root_box[k] = box[k];
        b->root_box[4 + k] = box[3 + k];
    }
    b->root_box[3] = b->root_box[7] = 0.0f;
}

static void store_root_box(orc_bvh *b, const float box[6]) {
    for (int k = 0; k < 3; k++) {
        b->root_box[k] = box[k];
        b->root_box[4 + k] = box[3 + k];
    }
    b->root_box[3] = b->root_box[7] = 0.0f;
}

int orc_lbvh_refit_climb(orc_bvh *b, const float *aabb) {
    const int n = b->n;
    if (n <= 0) return 0;
    int status = 0;
    uint32_t *flags = (uint32_t *)calloc((size_t)(n > 1 ? n - 1 : 1), sizeof(uint32_t));
    for (int k = 0; k < n; k++) {
        const uint32_t gid = b->order[k];
        const float *a = aabb + 8 * (size_t)gid;
        float box[6] = {a[0], a[1], a[2], a[4], a[5], a[6]};
        int p = n > 1 ? b->leaf_parent[k] : -1;
        if (p < 0) {
            store_root_box(b, box);
            continue;
        }
        uint32_t link = gid | LEAF_BIT;
        int guard = 0;
        for (; guard < 128; guard++) {
            float *nd = b->nodes + 16 * (size_t)p;
            uint32_t c0;
            memcpy(&c0, nd + 12, 4);
            memcpy(nd + 6 * (c0 == link ? 0 : 1), box, sizeof(box));
            if (flags[p]++ == 0u) break;
            for (int q = 0; q < 3; q++) {
                box[q] = fminf(nd[q], nd[6 + q]);
                box[3 + q] = fmaxf(nd[3 + q], nd[9 + q]);
            }
            const int pp = b->int_parent[p];
            if (pp < 0) {
                store_root_box(b, box);
                break;
            }
            link = (uint32_t)p;
            p = pp;
        }
        if (guard == 128) status |= 4;
    }
    free(flags);
    return status;
}

void orc_lbvh_free(orc_bvh *b) {
    free(b->nodes);
    free(b->codes);
    free(b->order);
    free(b->int_parent);
    free(b->leaf_parent);
    memset(b, 0, sizeof(*b));
}

/* ------------------------------------------------------------------------------------------ */
/* trace forward                                                                               */
/* ------------------------------------------------------------------------------------------ */
typedef struct {
    int hit;
    float dist, alpha;
} is_result;

/* a.b as an FMA chain: fma(a2, b2, fma(a1, b1, a0 * b0)) (the GPU kernels use the same chain) */
static inline float fdot3(const float *a, const float *b) { return fmaf(a[2], b[2], fmaf(a[1], b[1], a[0] * b[0])); }

/* cuda/shaders.cu:10-67.  g = 12-float snapshot row block, o/sf live. */
static inline is_result intersect(const float *g, float o, float sf, const float ro[3], const float rd[3],
                                  const orc_trace_cfg *cfg) {
    is_result res = {0, 0.0f, 0.0f};
    if (o <= cfg->alpha_threshold) return res;
    float rel[3] = {ro[0] - g[3], ro[1] - g[7], ro[2] - g[11]};
    float lo[3], ld[3];
    for (int r = 0; r < 3; r++) {
        const float *m = g + 4 * r;
        lo[r] = fdot3(m, rel);
        ld[r] = fdot3(m, rd);
    }
    /* world distance of the max-density point: t = -<lo,ld>/<ld,ld> (d is a unit vector) */
    float b = fdot3(lo, ld);
    if (b > 0.0f) return res;
    float t = -b / fdot3(ld, ld);
    float u[3] = {fmaf(t, ld[0], lo[0]), fmaf(t, ld[1], lo[1]), fmaf(t, ld[2], lo[2])};
    float sq = fdot3(u, u);
    if (sq > 1.0f) return res;
    float dist = t;
    if (!(dist >= cfg->znear && dist <= cfg->zfar)) {
        /* the ray segment [znear, zfar] must still touch the instance's unit box (OptiX AABB test) */
        float t0 = cfg->znear, t1 = cfg->zfar;
        for (int k = 0; k < 3; k++) {
            float inv = 1.0f / ld[k];
            float ta = (-1.0f - lo[k]) * inv, tb = (1.0f - lo[k]) * inv;
            float tn = fminf(ta, tb), tf = fmaxf(ta, tb);
            t0 = fmaxf(t0, tn);
            t1 = fminf(t1, tf);
        }
        if (!(t0 <= t1)) return res;
    }
    float x[3] = {u[0] * sf, u[1] * sf, u[2] * sf};
    float d = fdot3(x, x);
    float gv = eval_gaussian(d, cfg->exp_power);
    res.hit = 1;
    res.dist = dist;
    res.alpha = orc_maxalpha_mul(gv, o);
    return res;
}

/* Hit decision of intersect() for an object-space ray (lo, ld): b = <lo,ld> <= 0 and the
 * max-density point inside the unit sphere (the range test, which only removes hits, left out). */
static int hit_local(const float lo[3], const float ld[3]) {
    const float b = fdot3(lo, ld);
    if (b > 0.0f) return 0;
    const float t = -b / fdot3(ld, ld);
    const float u[3] = {fmaf(t, ld[0], lo[0]), fmaf(t, ld[1], lo[1]), fmaf(t, ld[2], lo[2])};
    return !(fdot3(u, u) > 1.0f);
}

/* Restatement of the CUDA path's division-free pretest (may_hit_local): 0 means "certainly no
 * hit".  Not part of the reference's algorithm: the kernels use it to skip pairs before the
 * intersection program, so it must never reject a pair that hit_local() accepts. */
static int may_hit_local(const float lo[3], const float ld[3]) {
    const float b = fdot3(lo, ld);
    if (b > 0.0f) return 0;
    const float L = fdot3(ld, ld);
    const float p0 = lo[2] * ld[1], p1 = lo[0] * ld[2], p2 = lo[1] * ld[0];
    const float c[3] = {fmaf(lo[1], ld[2], -p0), fmaf(lo[2], ld[0], -p1), fmaf(lo[0], ld[1], -p2)};
    const float C = fdot3(c, c);
    const float li = fmaxf(fabsf(lo[0]), fmaxf(fabsf(lo[1]), fabsf(lo[2])));
    const float q4 = li * 0x1.0p-22f;
    const float k = fmaf(q4, fmaf(q4, 0.25f, 1.0f), 1.0f + 0x1.0p-18f);
    return !(C > L * k && li <= 0x1.0p40f && L >= 0x1.0p-60f && L <= 0x1.0p40f);
}

/* Restatement of the CUDA path's ellipsoid-plane cull (frustum_ellipsoid, one plane): 1 means
 * "the ellipsoid {mu + L u : |u| <= 1} lies below the threshold w along n" (the packet's rays cannot
 * reach it).  Not part of the reference's algorithm: a checker of the cull's rounding margin. */
static int ellipsoid_plane_cull(const float n[3], const float *l2w, float w) {
    const float *r0 = l2w, *r1 = l2w + 4, *r2 = l2w + 8;
    const float sd = fmaf(n[2], r2[3], fmaf(n[1], r1[3], n[0] * r0[3]));
    const float e0 = fmaf(r2[0], n[2], fmaf(r1[0], n[1], r0[0] * n[0]));
    const float e1 = fmaf(r2[1], n[2], fmaf(r1[1], n[1], r0[1] * n[0]));
    const float e2 = fmaf(r2[2], n[2], fmaf(r1[2], n[1], r0[2] * n[0]));
    const float gap = w - sd;
    return gap > 0x1.0p-60f && fmaf(e2, e2, fmaf(e1, e1, e0 * e0)) * 1.00006f < gap * gap;
}

int orc_cull_check(int n, const float *normals, const float *l2w, const float *thresholds, const double *planes,
                   int64_t *counts) {
    int64_t culled = 0, wrong = 0;
    for (int i = 0; i < n; i++) {
        const float *nn = normals + 3 * (size_t)i, *g = l2w + 12 * (size_t)i;
        if (!ellipsoid_plane_cull(nn, g, thresholds[i])) continue;
        culled++;
        /* exact: the ellipsoid's highest point along n is n.mu + |L^T n| */
        double sd = 0.0, ext = 0.0;
        for (int r = 0; r < 3; r++) sd += (double)nn[r] * (double)g[4 * r + 3];
        for (int c = 0; c < 3; c++) {
            double e = 0.0;
            for (int r = 0; r < 3; r++) e += (double)g[4 * r + c] * (double)nn[r];
            ext += e * e;
        }
        if (!(sd + sqrt(ext) < planes[i])) wrong++;
    }
    counts[0] = culled;
    counts[1] = wrong;
    return wrong != 0;
}

int orc_pretest_check(int n, const float *lo, const float *ld, int64_t *counts) {
    int64_t hits = 0, maybes = 0, violations = 0;
    for (int i = 0; i < n; i++) {
        const int h = hit_local(lo + 3 * (size_t)i, ld + 3 * (size_t)i);
        const int m = may_hit_local(lo + 3 * (size_t)i, ld + 3 * (size_t)i);
        hits += h;
        maybes += m;
        violations += h && !m;
    }
    counts[0] = hits;
    counts[1] = maybes;
    counts[2] = violations;
    return violations != 0;
}

typedef struct {
    uint64_t *keys;
    size_t n, cap;
    int32_t *stack;
} ray_scratch;

static void push_key(ray_scratch *s, uint64_t k) {
    if (s->n == s->cap) {
        s->cap = s->cap ? 2 * s->cap : 256;
        s->keys = (uint64_t *)realloc(s->keys, s->cap * sizeof(uint64_t));
    }
    s->keys[s->n++] = k;
}

static int cmp_u64(const void *a, const void *b) {
    uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return x < y ? -1 : (x > y);
}

typedef struct {
    int64_t lfx; /* sum of log(1 - alpha) in 2^-40 fixed point (full transmittance) */
    float ft;
    int64_t afx, cfx[3];
    int32_t nhit;
} hit_acc;

/* v * 2^k truncated to a signed 64-bit integer (clamped, NaN -> 0): the fixed-point form of the
 * all-hit sums, so that their value does not depend on the order in which hits are found */
static inline int64_t to_fixed(float v, float scale) {
    float t = v * scale;
    if (!(t == t)) t = 0.0f;
    if (t > 0x1.0p62f) t = 0x1.0p62f;
    if (t < -0x1.0p62f) t = -0x1.0p62f;
    return (int64_t)t;
}

/* Full transmittance prod(1 - alpha) (cuda/shaders.cu:55-56 multiplies in traversal order) kept
 * order-independent: log(1 - alpha) summed in 2^-40 fixed point, exponentiated once per ray; below
 * -105 (exp underflows to 0) no further terms are added. */
#define LOG_FIX_FLOOR (-105LL * (1LL << 40))
static inline void add_log_transmittance(int64_t *s, float alpha) {
    if (*s > LOG_FIX_FLOOR) *s += to_fixed(orc_logf(1.0f - alpha), 0x1.0p40f);
}
static inline float full_transmittance(int64_t s) { return orc_expf((float)s * 0x1.0p-40f); }

/* colour in 2^-24 fixed point, clamped to [-64, 64]; a tail-sum term is alpha16 (2^-24 units) times
 * this, an exact 64-bit product in 2^-48 units */
static inline int32_t colour_fixed(float c) { return (int32_t)to_fixed(fminf(fmaxf(c, -64.0f), 64.0f), 0x1.0p24f); }
static inline int64_t mul_fixed(int64_t a16fix, int32_t cfix) { return (int64_t)(int32_t)a16fix * (int64_t)cfix; }

static inline void record_hit(hit_acc *acc, ray_scratch *scr, uint32_t gid, is_result h, const float *channels,
                              float znear) {
    add_log_transmittance(&acc->lfx, h.alpha);
    uint16_t a16 = orc_f2h(h.alpha), d16 = orc_f2h(h.dist);
    float af = orc_h2f(a16);
    const float *c = channels + 3 * (size_t)gid;
    const int64_t a = to_fixed(af, 0x1.0p24f);
    acc->afx += a;
    for (int k = 0; k < 3; k++) acc->cfx[k] += mul_fixed(a, colour_fixed(c[k]));
    acc->nhit++;
    if (orc_h2f(d16) > znear) push_key(scr, ((uint64_t)d16 << 48) | ((uint64_t)gid << 16) | a16);
}

static inline int slab(const float *bx, const float ro[3], const float inv[3], float eps) {
    float tn = 0.0f, tf = INFINITY;
    for (int k = 0; k < 3; k++) {
        float ta = (bx[k] - eps - ro[k]) * inv[k];
        float tb = (bx[3 + k] + eps - ro[k]) * inv[k];
        tn = fmaxf(tn, fminf(ta, tb));
        tf = fminf(tf, fmaxf(ta, tb));
    }
    return tn <= tf;
}

typedef struct {
    int nrays;
    const float *ray_o, *ray_d;
    int n;
    const float *geom, *live, *channels;
    const uint8_t *visible;
    const orc_bvh *bvh;
    const orc_trace_cfg *cfg;
    float *out_rgb, *out_depth, *out_T, *out_fullT, *out_rem;
    int32_t *out_nhit, *out_nacc;
    const int64_t *comp_offsets;
    uint32_t *comp_ids;
    int next;
    pthread_mutex_t mu;
} fwd_job;

static void trace_one(fwd_job *J, int r, ray_scratch *scr) {
    const orc_trace_cfg *cfg = J->cfg;
    const float *ro = J->ray_o + 3 * (size_t)r, *rd = J->ray_d + 3 * (size_t)r;
    hit_acc acc = {0, 1.0f, 0, {0, 0, 0}, 0};
    scr->n = 0;
    if (rd[0] == 0.0f && rd[1] == 0.0f && rd[2] == 0.0f) {
        /* inactive pixel (cuda/shaders.cu:86-88): nothing is written */
        J->out_nhit[r] = -1;
        J->out_nacc[r] = 0;
        return;
    }
    if (J->bvh == NULL) {
        for (int g = 0; g < J->n; g++) {
            if (!J->visible[g]) continue;
            is_result h = intersect(J->geom + 12 * (size_t)g, J->live[2 * g], J->live[2 * g + 1], ro, rd, cfg);
            if (h.hit) record_hit(&acc, scr, (uint32_t)g, h, J->channels, cfg->znear);
        }
    } else {
        const orc_bvh *b = J->bvh;
        float inv[3];
        for (int k = 0; k < 3; k++) {
            float dk = rd[k];
            if (fabsf(dk) < 1e-20f) dk = dk < 0.0f ? -1e-20f : 1e-20f;
            inv[k] = 1.0f / dk;
        }
        float eps = 2.0e-6f * (fabsf(ro[0]) + fabsf(ro[1]) + fabsf(ro[2]));
        float rb[6] = {b->root_box[0], b->root_box[1], b->root_box[2], b->root_box[4], b->root_box[5],
                       b->root_box[6]};
        if (b->n > 0 && slab(rb, ro, inv, eps)) {
            if (b->n == 1) {
                uint32_t g = b->order[0];
                if (J->visible[g]) {
                    is_result h = intersect(J->geom + 12 * (size_t)g, J->live[2 * g], J->live[2 * g + 1], ro, rd, cfg);
                    if (h.hit) record_hit(&acc, scr, g, h, J->channels, cfg->znear);
                }
            } else {
                int sp = 0;
                scr->stack[sp++] = 0;
                while (sp > 0) {
                    int ni = scr->stack[--sp];
                    const float *nd = b->nodes + 16 * (size_t)ni;
                    for (int s = 0; s < 2; s++) {
                        uint32_t c;
                        memcpy(&c, nd + 12 + s, 4);
                        if (!slab(nd + 6 * s, ro, inv, eps)) continue;
                        if (c & LEAF_BIT) {
                            uint32_t g = c & ~LEAF_BIT;
                            if (!J->visible[g]) continue;
                            is_result h =
                                intersect(J->geom + 12 * (size_t)g, J->live[2 * g], J->live[2 * g + 1], ro, rd, cfg);
                            if (h.hit) record_hit(&acc, scr, g, h, J->channels, cfg->znear);
                        } else if (sp < 256) {
                            scr->stack[sp++] = (int32_t)c;
                        }
                    }
                }
            }
        }
    }
    qsort(scr->keys, scr->n, sizeof(uint64_t), cmp_u64);

    /* consumer: cuda/forward_pass.cu:46-125 on the (d16, id)-sorted stream */
    float T = 1.0f, C[3] = {0.0f, 0.0f, 0.0f}, depth = 0.0f;
    int pass = 0, slots = 0, nacc = 0;
    float tmin_sel = cfg->znear, last_d = cfg->znear;
    int64_t off = J->comp_offsets ? J->comp_offsets[r] : 0;
    for (size_t i = 0; i < scr->n; i++) {
        uint64_t key = scr->keys[i];
        float d = orc_h2f((uint16_t)(key >> 48));
        if (!(d > tmin_sel)) continue;
        if (slots == cfg->pass_slots) {
            pass++;
            if (pass >= cfg->max_passes) break;
            tmin_sel = last_d;
            if (!(tmin_sel < cfg->zfar)) break;
            slots = 0;
            if (!(d > tmin_sel)) continue;
        }
        slots++;
        last_d = d;
        if (!(d < cfg->zfar)) break;
        uint32_t gid = (uint32_t)(key >> 16);
        float a = orc_h2f((uint16_t)(key & 0xffffu));
        const float *c = J->channels + 3 * (size_t)gid;
        const int64_t afix = to_fixed(a, 0x1.0p24f);
        acc.afx -= afix;
        for (int k = 0; k < 3; k++) acc.cfx[k] -= mul_fixed(afix, colour_fixed(c[k]));
        float w = T * a;
        for (int k = 0; k < 3; k++) C[k] = C[k] + c[k] * w;
        if (cfg->render_depth) depth = depth + d * w;
        T = T * (1.0f - a);
        if (J->comp_ids && J->comp_offsets) J->comp_ids[off + nacc] = gid;
        nacc++;
        if (T < cfg->t_threshold) break;
    }
    acc.ft = full_transmittance(acc.lfx);
    float rT = T - acc.ft;
    float rem[3] = {0.0f, 0.0f, 0.0f};
    if (acc.afx > 0) {
        float sa = (float)acc.afx * 0x1.0p-24f;
        for (int k = 0; k < 3; k++) rem[k] = ((float)acc.cfx[k] * 0x1.0p-48f) / sa;
    }
    for (int k = 0; k < 3; k++) C[k] = C[k] + rT * rem[k];
    if (cfg->render_depth) depth = depth / fmaxf(1.0f - T, cfg->eps_forward_normalization);
    for (int k = 0; k < 3; k++) C[k] = C[k] + cfg->bg[k] * acc.ft;
    for (int k = 0; k < 3; k++) {
        J->out_rgb[3 * (size_t)r + k] = C[k];
        J->out_rem[3 * (size_t)r + k] = rem[k];
    }
    J->out_depth[r] = depth;
    J->out_T[r] = T;
    J->out_fullT[r] = acc.ft;
    J->out_nhit[r] = acc.nhit;
    J->out_nacc[r] = nacc;
}

static void *fwd_worker(void *arg) {
    fwd_job *J = (fwd_job *)arg;
    ray_scratch scr = {NULL, 0, 0, (int32_t *)malloc(sizeof(int32_t) * 256)};
    for (;;) {
        pthread_mutex_lock(&J->mu);
        int r0 = J->next;
        J->next += 64;
        pthread_mutex_unlock(&J->mu);
        if (r0 >= J->nrays) break;
        int r1 = r0 + 64 < J->nrays ? r0 + 64 : J->nrays;
        for (int r = r0; r < r1; r++) trace_one(J, r, &scr);
    }
    free(scr.keys);
    free(scr.stack);
    return NULL;
}

int orc_hardware_threads(void) {
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    return n > 0 ? (int)n : 1;
}

void orc_trace_forward(int nrays, const float *ray_o, const float *ray_d, int n, const float *geom,
                       const float *live, const float *channels, const uint8_t *visible, const orc_bvh *bvh,
                       const orc_trace_cfg *cfg, float *out_rgb, float *out_depth, float *out_T, float *out_fullT,
                       float *out_rem, int32_t *out_nhit, int32_t *out_nacc, const int64_t *comp_offsets,
                       uint32_t *comp_ids, int nthreads) {
    fwd_job J = {nrays, ray_o, ray_d, n, geom, live, channels, visible, bvh, cfg, out_rgb, out_depth, out_T,
                 out_fullT, out_rem, out_nhit, out_nacc, comp_offsets, comp_ids, 0, PTHREAD_MUTEX_INITIALIZER};
    if (nthreads <= 0) nthreads = orc_hardware_threads();
    if (nthreads == 1) {
        fwd_worker(&J);
        return;
    }
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, fwd_worker, &J);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(th);
}

/* ------------------------------------------------------------------------------------------ */
/* trace backward: cuda/backward_pass.cu:2-142                                                 */
/* ------------------------------------------------------------------------------------------ */
static inline void atomic_add_double(double *addr, double v) {
    uint64_t old_bits, new_bits;
    double old_v, new_v;
    __atomic_load(addr, &old_v, __ATOMIC_RELAXED);
    do {
        new_v = old_v + v;
        memcpy(&old_bits, &old_v, 8);
        memcpy(&new_bits, &new_v, 8);
    } while (!__atomic_compare_exchange((uint64_t *)addr, &old_bits, &new_bits, 0, __ATOMIC_RELAXED,
                                        __ATOMIC_RELAXED) &&
             (memcpy(&old_v, &old_bits, 8), 1));
}

typedef struct {
    int r0, r1, launch_w, launch_h;
    const float *ray_o, *ray_d, *pix_T, *pix_fullT, *pix_rem, *grad_out;
    const int64_t *comp_offsets;
    const uint32_t *comp_ids;
    const float *geom, *l2w, *opacity, *scale, *rotation, *channels;
    const orc_trace_cfg *cfg;
    float eps_scale_grad;
    double *grad;
    int atomic;
} bwd_job;

static void backward_range(const bwd_job *J) {
    const int launch_w = J->launch_w, launch_h = J->launch_h;
    const float *ray_o = J->ray_o, *ray_d = J->ray_d, *pix_T = J->pix_T, *pix_fullT = J->pix_fullT;
    const float *pix_rem = J->pix_rem, *grad_out = J->grad_out, *geom = J->geom, *l2w = J->l2w;
    const float *opacity = J->opacity, *scale = J->scale, *rotation = J->rotation, *channels = J->channels;
    const int64_t *comp_offsets = J->comp_offsets;
    const uint32_t *comp_ids = J->comp_ids;
    const orc_trace_cfg *cfg = J->cfg;
    const float eps_scale_grad = J->eps_scale_grad;
    double *grad = J->grad;
    const float npix = (float)(launch_w * launch_h);
    for (int r = J->r0; r < J->r1; r++) {
        const float *ro = ray_o + 3 * (size_t)r, *rd = ray_d + 3 * (size_t)r;
        const float *gout = grad_out + 3 * (size_t)r;
        const float *rem = pix_rem + 3 * (size_t)r;
        float Tfin = pix_T[r], fT = pix_fullT[r];
        float gT = 0.0f, T = Tfin;
        float dbg = cfg->bg[0] * gout[0] + cfg->bg[1] * gout[1] + cfg->bg[2] * gout[2];
        float drem = rem[0] * gout[0] + rem[1] * gout[1] + rem[2] * gout[2];
        for (int64_t e = comp_offsets[r + 1] - 1; e >= comp_offsets[r]; e--) {
            uint32_t gid = comp_ids[e];
            const float *g = geom + 12 * (size_t)gid, *L = l2w + 12 * (size_t)gid;
            float o = sigmoid_act(opacity[gid]);
            float s[3];
            for (int k = 0; k < 3; k++) s[k] = orc_expf(scale[3 * (size_t)gid + k]);
            const float *qr = rotation + 4 * (size_t)gid;
            float qlen = sqrtf(qr[0] * qr[0] + qr[1] * qr[1] + qr[2] * qr[2] + qr[3] * qr[3]);
            float q[4] = {qr[0] / qlen, qr[1] / qlen, qr[2] / qlen, qr[3] / qlen};
            const float *c = channels + 3 * (size_t)gid;
            float sf = orc_scaling_factor(o, cfg->alpha_threshold, cfg->exp_power);

            float rel[3] = {ro[0] - g[3], ro[1] - g[7], ro[2] - g[11]};
            float lo[3], ld[3];
            for (int k = 0; k < 3; k++) {
                const float *m = g + 4 * k;
                lo[k] = fdot3(m, rel);
                ld[k] = fdot3(m, rd);
            }
            float b = fdot3(lo, ld);
            float td = -b / fdot3(ld, ld);
            float x[3];
            for (int k = 0; k < 3; k++) x[k] = fmaf(td, ld[k], lo[k]) * sf;
            float sq = fdot3(x, x);
            float gv = eval_gaussian(sq, cfg->exp_power);
            float alpha = orc_maxalpha_mul(gv, o);

            float om = 1.0f - alpha;
            float w = T / om * alpha;
            float dgc = gout[0] * c[0] + gout[1] * c[1] + gout[2] * c[2];
            float ga = (dgc - gT) * T / om;
            ga = ga + -fT / om * dbg;
            ga = ga + -((Tfin - fT) / om) * drem;
            gT = gT + (dgc - gT) * alpha;
            float go = orc_maxalpha_mul(ga, gv);
            go = go * o * (1.0f - o);
            float ggv = orc_maxalpha_mul(ga, o);
            float gsq;
            if (cfg->exp_power == 1.0f) gsq = gv;
            else if (cfg->exp_power == 2.0f) gsq = gv * sq;
            else if (cfg->exp_power == 3.0f) gsq = gv * sq * sq;
            else gsq = gv * orc_powf(sq, cfg->exp_power - 1.0f);
            float gxl[3];
            for (int k = 0; k < 3; k++) gxl[k] = -x[k] * gsq * ggv;
            float gxw[3];
            for (int k = 0; k < 3; k++) gxw[k] = (g[k] * gxl[0] + g[4 + k] * gxl[1] + g[8 + k] * gxl[2]) * sf;
            float gl[3][3];
            for (int i = 0; i < 3; i++)
                for (int k = 0; k < 3; k++) gl[i][k] = -gxw[i] * x[k];
            float den[3];
            for (int k = 0; k < 3; k++) den[k] = s[k] * sf + eps_scale_grad;
            float gs[3];
            for (int k = 0; k < 3; k++) {
                float a0 = gl[0][k] * (L[0 + k] / den[k]);
                float a1 = gl[1][k] * (L[4 + k] / den[k]);
                float a2 = gl[2][k] * (L[8 + k] / den[k]);
                gs[k] = (a0 + a1 + a2) * s[k];
            }
            float gr[3][3];
            for (int i = 0; i < 3; i++)
                for (int k = 0; k < 3; k++) gr[i][k] = gl[i][k] * s[k];
            /* d R(q) / d q contracted with gr (q = (r, x, y, z) normalised) */
            float qw = q[0], qx = q[1], qy = q[2], qz = q[3];
            float g_r = 2.0f * qx * (gr[2][1] - gr[1][2]) + 2.0f * qy * (gr[0][2] - gr[2][0]) +
                        2.0f * qz * (gr[1][0] - gr[0][1]);
            float g_x = -4.0f * qx * (gr[1][1] + gr[2][2]) + 2.0f * qy * (gr[0][1] + gr[1][0]) +
                        2.0f * qz * (gr[0][2] + gr[2][0]) + 2.0f * qw * (gr[2][1] - gr[1][2]);
            float g_y = 2.0f * qx * (gr[0][1] + gr[1][0]) - 4.0f * qy * (gr[0][0] + gr[2][2]) +
                        2.0f * qz * (gr[1][2] + gr[2][1]) + 2.0f * qw * (gr[0][2] - gr[2][0]);
            float g_z = 2.0f * qx * (gr[0][2] + gr[2][0]) + 2.0f * qy * (gr[1][2] + gr[2][1]) -
                        4.0f * qz * (gr[0][0] + gr[1][1]) + 2.0f * qw * (gr[1][0] - gr[0][1]);
            float gq[4] = {g_r, g_x, g_y, g_z};
            float dq = gq[0] * qr[0] + gq[1] * qr[1] + gq[2] * qr[2] + gq[3] * qr[3];
            float l3 = qlen * qlen * qlen;
            double *G = grad + 16 * (size_t)gid;
            double v[16];
            for (int k = 0; k < 4; k++) v[k] = (double)(dq * -qr[k] / l3 + gq[k] / qlen);
            for (int k = 0; k < 3; k++) v[4 + k] = (double)(-gxw[k]);
            v[7] = (double)go;
            for (int k = 0; k < 3; k++) v[8 + k] = (double)gs[k];
            v[11] = (double)(w / npix);
            for (int k = 0; k < 3; k++) v[12 + k] = (double)(gout[k] * w);
            v[15] = 1.0;
            if (J->atomic)
                for (int k = 0; k < 16; k++) atomic_add_double(G + k, v[k]);
            else
                for (int k = 0; k < 16; k++) G[k] += v[k];
            T = T / om;
        }
    }
}

static void *bwd_worker(void *arg) {
    backward_range((const bwd_job *)arg);
    return NULL;
}

void orc_trace_backward(int nrays, int launch_w, int launch_h, const float *ray_o, const float *ray_d,
                        const float *pix_T, const float *pix_fullT, const float *pix_rem, const float *grad_out,
                        const int64_t *comp_offsets, const uint32_t *comp_ids, int n, const float *geom,
                        const float *l2w, const float *opacity, const float *scale, const float *rotation,
                        const float *channels, const orc_trace_cfg *cfg, float eps_scale_grad, double *grad,
                        int nthreads) {
    (void)n;
    if (nthreads <= 0) nthreads = orc_hardware_threads();
    if (nthreads > nrays) nthreads = nrays > 0 ? nrays : 1;
    bwd_job base = {0, nrays, launch_w, launch_h, ray_o, ray_d, pix_T, pix_fullT, pix_rem, grad_out, comp_offsets,
                    comp_ids, geom, l2w, opacity, scale, rotation, channels, cfg, eps_scale_grad, grad, nthreads > 1};
    if (nthreads == 1) {
        backward_range(&base);
        return;
    }
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
    bwd_job *jobs = (bwd_job *)malloc(sizeof(bwd_job) * (size_t)nthreads);
    for (int t = 0; t < nthreads; t++) {
        jobs[t] = base;
        jobs[t].r0 = (int)((long long)nrays * t / nthreads);
        jobs[t].r1 = (int)((long long)nrays * (t + 1) / nthreads);
        pthread_create(&th[t], NULL, bwd_worker, &jobs[t]);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(th);
    free(jobs);
}

/* ------------------------------------------------------------------------------------------ */
/* fused Adam: cuda/opt/adam.cu:6-83                                                           */
/* ------------------------------------------------------------------------------------------ */
typedef struct {
    float b1, b2, eps, ibc1, ibc2; /* ibc = 1 / (1 - beta^(step+1)) */
    int zero;
} adam_k;

static inline void adam_el(const adam_k *a, float *p, float *m, float *v, float *g, float lr) {
    float gg = *g;
    float mm = a->b1 * *m + (1.0f - a->b1) * gg;
    float vv = a->b2 * *v + (1.0f - a->b2) * gg * gg;
    float mh = mm * a->ibc1;
    float vh = vv * a->ibc2;
    *p = *p - lr * mh / (sqrtf(vh) + a->eps);
    *m = mm;
    *v = vv;
    if (a->zero) *g = gg * 0.0f;
}

void orc_adam_step(orc_adam_state *s, int step, int zero_grads, int update_channels, float beta1, float beta2,
                   float eps, int enable_sh, int laziness) {
    adam_k a = {beta1, beta2, eps, 1.0f / (1.0f - orc_adam_pow(beta1, step + 1)),
                1.0f / (1.0f - orc_adam_pow(beta2, step + 1)), zero_grads};
    for (int i = 0; i < s->n; i++) {
        for (int k = 0; k < 3; k++) {
            size_t j = 3 * (size_t)i + k;
            if (update_channels) adam_el(&a, s->channels + j, s->m_channels + j, s->v_channels + j, s->g_channels + j, s->lr_channels);
            else if (zero_grads) s->g_channels[j] = 0.0f;
        }
        adam_el(&a, s->opacity + i, s->m_opacity + i, s->v_opacity + i, s->g_opacity + i, s->lr_opacity);
        for (int k = 0; k < 3; k++) {
            size_t j = 3 * (size_t)i + k;
            adam_el(&a, s->mean + j, s->m_mean + j, s->v_mean + j, s->g_mean + j, s->lr_mean);
        }
        for (int k = 0; k < 4; k++) {
            size_t j = 4 * (size_t)i + k;
            adam_el(&a, s->rotation + j, s->m_rotation + j, s->v_rotation + j, s->g_rotation + j, s->lr_rotation);
        }
        for (int k = 0; k < 3; k++) {
            size_t j = 3 * (size_t)i + k;
            adam_el(&a, s->scale + j, s->m_scale + j, s->v_scale + j, s->g_scale + j, s->lr_scale);
        }
    }
    if (enable_sh && laziness > 0 && step % laziness == 0) {
        for (int i = 0; i < s->n; i++) {
            for (int k = 0; k < 3; k++) {
                size_t j = 3 * (size_t)i + k;
                adam_el(&a, s->sh_dc + j, s->m_sh_dc + j, s->v_sh_dc + j, s->g_sh_dc + j, s->lr_sh_dc);
            }
            for (int c = 0; c < s->num_rest; c++)
                for (int k = 0; k < 3; k++) {
                    size_t j = ((size_t)i * s->num_rest + c) * 3 + k;
                    adam_el(&a, s->sh_rest + j, s->m_sh_rest + j, s->v_sh_rest + j, s->g_sh_rest + j, s->lr_sh_rest);
                }
        }
    }
}

/* ------------------------------------------------------------------------------------------ */
/* ellipsoid view: cuda/ellipsoid_viewer.cu:1-94 (closest hit on each Gaussian's support        */
/* ellipsoid, flat shading).  Brute force over all Gaussians: the winner (smallest distance in  */
/* [znear, zfar], equal distances -> smaller id) does not depend on visiting order.            */
/* ------------------------------------------------------------------------------------------ */
static void local_ray3(const float *g, const float ro[3], const float rd[3], float lo[3], float ld[3]) {
    float rel[3] = {ro[0] - g[3], ro[1] - g[7], ro[2] - g[11]};
    for (int r = 0; r < 3; r++) {
        lo[r] = fdot3(g + 4 * r, rel);
        ld[r] = fdot3(g + 4 * r, rd);
    }
}

/* cuda/ellipsoid_viewer.cu:23-62: near root if at or beyond tmin, else far root */
static int ellipsoid_hit(const float *g, const float ro[3], const float rd[3], float tmin, float *t) {
    float lo[3], ld[3];
    local_ray3(g, ro, rd, lo, ld);
    if (fdot3(lo, ld) > 0.0f) return 0;
    float norm = sqrtf(fdot3(ld, ld));
    float dn[3] = {ld[0] / norm, ld[1] / norm, ld[2] / norm};
    float smid = -fdot3(lo, dn);
    float u[3] = {fmaf(smid, dn[0], lo[0]), fmaf(smid, dn[1], lo[1]), fmaf(smid, dn[2], lo[2])};
    float sq = fdot3(u, u);
    if (sq > 1.0f) return 0;
    float hc = sqrtf(1.0f - sq);
    float t0 = (smid - hc) / norm, t1 = (smid + hc) / norm;
    *t = t0 >= tmin ? t0 : t1;
    return *t >= tmin;
}

/* cuda/ellipsoid_viewer.cu:55-59, 66-93: world normal = M^T (object normal), flat shading */
static void ellipsoid_shade(const float *g, const float ro[3], const float rd[3], float t, const float *c,
                            float *rgb) {
    float lo[3], ld[3];
    local_ray3(g, ro, rd, lo, ld);
    float norm = sqrtf(fdot3(ld, ld));
    float dn[3] = {ld[0] / norm, ld[1] / norm, ld[2] / norm};
    float tn = t * norm;
    float ln[3] = {fmaf(tn, dn[0], lo[0]), fmaf(tn, dn[1], lo[1]), fmaf(tn, dn[2], lo[2])};
    float ll = sqrtf(fdot3(ln, ln));
    for (int k = 0; k < 3; k++) ln[k] = ln[k] / ll;
    float wn[3];
    for (int k = 0; k < 3; k++) wn[k] = fmaf(ln[2], g[8 + k], fmaf(ln[1], g[4 + k], ln[0] * g[k]));
    float wl = sqrtf(fdot3(wn, wn));
    for (int k = 0; k < 3; k++) wn[k] = wn[k] / wl;
    float dl = sqrtf(fdot3(rd, rd));
    float vd[3] = {rd[0] / dl, rd[1] / dl, rd[2] / dl};
    float align = fmaxf(0.5f, -fdot3(vd, wn));
    for (int k = 0; k < 3; k++) rgb[k] = align * (c[k] + 0.15f);
}

typedef struct {
    int nrays;
    const float *ray_o, *ray_d;
    int n;
    const float *geom, *live, *channels;
    float znear, zfar, min_opacity;
    const float *bg;
    float *out_rgb, *out_depth;
    int32_t *out_id;
    int next;
    pthread_mutex_t mu;
} ell_job;

static void *ell_worker(void *arg) {
    ell_job *J = (ell_job *)arg;
    for (;;) {
        pthread_mutex_lock(&J->mu);
        int r0 = J->next;
        J->next += 64;
        pthread_mutex_unlock(&J->mu);
        if (r0 >= J->nrays) break;
        int r1 = r0 + 64 < J->nrays ? r0 + 64 : J->nrays;
        for (int r = r0; r < r1; r++) {
            const float *ro = J->ray_o + 3 * (size_t)r, *rd = J->ray_d + 3 * (size_t)r;
            float *rgb = J->out_rgb + 3 * (size_t)r;
            if (sqrtf(rd[0] * rd[0] + rd[1] * rd[1] + rd[2] * rd[2]) == 0.0f) {
                J->out_id[r] = -2; /* inactive pixel: outputs untouched */
                continue;
            }
            float best = J->zfar;
            int64_t bid = -1;
            for (int i = 0; i < J->n; i++) {
                if (J->live[2 * (size_t)i] < J->min_opacity) continue;
                float t;
                if (!ellipsoid_hit(J->geom + 12 * (size_t)i, ro, rd, J->znear, &t)) continue;
                if (t < best || (t == best && bid < 0)) {
                    best = t;
                    bid = i;
                }
            }
            J->out_id[r] = (int32_t)bid;
            if (bid < 0) {
                for (int k = 0; k < 3; k++) rgb[k] = J->bg[k];
                J->out_depth[r] = 0.0f;
            } else {
                ellipsoid_shade(J->geom + 12 * (size_t)bid, ro, rd, best, J->channels + 3 * (size_t)bid, rgb);
                J->out_depth[r] = best;
            }
        }
    }
    return NULL;
}

void orc_ellipsoids(int nrays, const float *ray_o, const float *ray_d, int n, const float *geom, const float *live,
                    const float *channels, float znear, float zfar, float min_opacity, const float *bg,
                    float *out_rgb, float *out_depth, int32_t *out_id, int nthreads) {
    ell_job J = {nrays, ray_o, ray_d, n, geom, live, channels, znear, zfar, min_opacity, bg, out_rgb, out_depth,
                 out_id, 0, PTHREAD_MUTEX_INITIALIZER};
    if (nthreads <= 0) nthreads = orc_hardware_threads();
    if (nthreads == 1) {
        ell_worker(&J);
        return;
    }
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, ell_worker, &J);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(th);
}
