/*
 * gray_oracle.h -- CPU restatement of GRay's differentiable Gaussian ray tracer.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path in
 * gray_gb300/; it is never linked into, loaded by, or called from the product.
 * Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
 * arm use it.
 *
 * Every function restates the arithmetic of one reference routine (citations
 * are paths inside the graphdeco-inria/gray source tree).  The floating-point
 * expression trees match the CUDA kernels operation for operation (no FMA
 * contraction: built with -ffp-contract=off; fmaf only where written), and the
 * transcendental functions are this project's own (Cody-Waite reduction +
 * Taylor/atanh series), so hit lists, fp16 keys and composited transmittance
 * agree bit-for-bit with the GPU for identical inputs.
 *
 * Parity of this oracle with the reference is pinned by tests/golden/ (fixtures
 * generated from the reference's own test scenes, tests/test_single_gaussian.py
 * and tests/test_multiple_gaussians.py, whose compositing loops are restated in
 * FP64).  SH, Adam and BVH parity are not covered by any reference test and are
 * "parity unpinned" against the reference (pinned only against the restated
 * formulas).
 */
#ifndef GRAY_ORACLE_H
#define GRAY_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- scalar math (own implementations, identical on GPU) ---- */
float orc_expf(float x);
float orc_logf(float x);
uint16_t orc_f2h(float f);
float orc_h2f(uint16_t h);
float orc_scaling_factor(float opacity, float alpha_threshold, float exp_power);
float orc_maxalpha_mul(float a, float b);
/* Gaussian response at squared local radius d (cuda/utils/kernel.cu:24-38), as the GPU evaluates it */
float orc_eval_gaussian(float d, float exp_power);
float orc_adam_pow(float beta, int n);

/* ---- per-Gaussian snapshot (populate_bvh_kernel, cuda/optix/bvh_wrapper.cu:8-59) ----
 * geom:  N x 12 floats  = rows (M00 M01 M02 mux | M10 M11 M12 muy | M20 M21 M22 muz),
 *        M = diag(1/(s*sf*gsf)) R^T  (world -> unit-sphere frame)
 * l2w:   N x 12 floats  = rows of R diag(s*sf*gsf) (w unused)
 * aabb:  N x 8 floats   = (minx miny minz pad maxx maxy maxz pad), empty if invisible
 * visible: N bytes
 */
void orc_snapshot(int n, const float *mean, const float *rotation, const float *scale, const float *opacity,
                  float alpha_threshold, float exp_power, float global_scale_factor, float *geom, float *l2w,
                  float *aabb, uint8_t *visible);

/* live per-forward values: live[2i] = sigmoid(opacity), live[2i+1] = scaling factor */
void orc_forward_prep(int n, const float *opacity, float alpha_threshold, float exp_power, float *live);

/* ---- camera (cuda/core/camera.h:17-36) ---- */
void orc_camera_rays(int width, int height, float fov_y, const float *origin, const float *c2w, float *ray_o,
                     float *ray_d);

/* ---- SH colour (cuda/utils/sh.cu:224-304) ---- */
void orc_sh_forward(int n, int degree, int num_rest, const float *mean, const float *cam_origin, const float *sh_dc,
                    const float *sh_rest, float *channels);
void orc_sh_backward(int n, int degree, int num_rest, const float *mean, const float *cam_origin,
                     const float *sh_rest, const float *channels, const float *grad_channels,
                     const uint8_t *was_visible, float *grad_sh_dc, float *grad_sh_rest, float *grad_mean);

/* ---- LBVH (Karras 2012), own construction restated for the GPU build ---- */
typedef struct {
    int n;                 /* leaves */
    float *nodes;          /* (n-1) x 16 floats: c0 box (6), c1 box (6), child0, child1 (as uint32 bits), pad */
    uint32_t *codes;       /* n: Morton code (sorted, key order) */
    uint32_t *order;       /* n: sorted leaf position -> gaussian id */
    int32_t *int_parent;   /* n-1: parent of internal node (-1 root) */
    int32_t *leaf_parent;  /* n: parent of sorted leaf position (-1 if n == 1) */
    float root_box[8];
} orc_bvh;

void orc_lbvh_build(int n, const float *aabb, const uint8_t *visible, orc_bvh *out);
void orc_lbvh_refit(orc_bvh *bvh, const float *aabb);
/* The GPU refit's bottom-up protocol (gray_gb300/csrc/lbvh.cu refit_kernel), one climber per sorted
 * leaf run to completion in leaf order: a climber stores its box in its parent's slot and counts its
 * visit; the first arriver stops, the second unions the two child boxes and climbs on.  A climb of
 * more than 128 levels stops and sets bit 4 (GRAY_STATUS_REFIT_TIMEOUT) of the returned status.
 * The parent links are bvh->int_parent / leaf_parent, so a caller can plant a corrupt chain. */
int orc_lbvh_refit_climb(orc_bvh *bvh, const float *aabb);
void orc_lbvh_free(orc_bvh *bvh);

/* ---- trace forward (cuda/shaders.cu:10-67 + cuda/forward_pass.cu:6-151) ---- */
typedef struct {
    float exp_power, alpha_threshold, t_threshold;
    float znear, zfar, eps_forward_normalization;
    float bg[3];
    int render_depth;
    int pass_slots;     /* BUFFER_SIZE (32 in the reference) */
    int max_passes;     /* MAX_ITERATIONS (99 in the reference) */
} orc_trace_cfg;

/* out_*: per ray.  comp_offsets (optional, r+1 entries, caller-filled prefix sums of a previous
 * out_nacc) selects where composited gaussian ids are written.  bvh == NULL -> brute force. */
void orc_trace_forward(int nrays, const float *ray_o, const float *ray_d, int n, const float *geom,
                       const float *live, const float *channels, const uint8_t *visible, const orc_bvh *bvh,
                       const orc_trace_cfg *cfg, float *out_rgb, float *out_depth, float *out_T, float *out_fullT,
                       float *out_rem, int32_t *out_nhit, int32_t *out_nacc, const int64_t *comp_offsets,
                       uint32_t *comp_ids, int nthreads);

/* ---- trace backward (cuda/backward_pass.cu:2-142) ----
 * grads are accumulated in double: grad[N*16] laid out as
 * (rot4 | mean3, opacity | scale3, pruning | channels3, count) */
void orc_trace_backward(int nrays, int launch_w, int launch_h, const float *ray_o, const float *ray_d,
                        const float *pix_T, const float *pix_fullT, const float *pix_rem, const float *grad_out,
                        const int64_t *comp_offsets, const uint32_t *comp_ids, int n, const float *geom,
                        const float *l2w, const float *opacity, const float *scale, const float *rotation,
                        const float *channels, const orc_trace_cfg *cfg, float eps_scale_grad, double *grad,
                        int nthreads);

/* ---- fused Adam (cuda/opt/adam.cu:6-83) ----
 * arrays follow the reference holders; step = total_num_steps after the increment. */
typedef struct {
    int n, num_rest;
    float *channels, *opacity, *mean, *rotation, *scale, *sh_dc, *sh_rest;
    float *g_channels, *g_opacity, *g_mean, *g_rotation, *g_scale, *g_sh_dc, *g_sh_rest;
    float *m_channels, *m_opacity, *m_mean, *m_rotation, *m_scale, *m_sh_dc, *m_sh_rest;
    float *v_channels, *v_opacity, *v_mean, *v_rotation, *v_scale, *v_sh_dc, *v_sh_rest;
    float lr_channels, lr_opacity, lr_mean, lr_rotation, lr_scale, lr_sh_dc, lr_sh_rest;
} orc_adam_state;
void orc_adam_step(orc_adam_state *s, int step, int zero_grads, int update_channels, float beta1, float beta2,
                   float eps, int enable_sh, int sh_update_laziness);

/* ---- ellipsoid view (cuda/ellipsoid_viewer.cu:1-94) ----
 * live = [n,2] (opacity or -inf if invisible, sf); out_id = winning gaussian, -1 miss, -2 inactive
 * ray (outputs untouched). */
void orc_ellipsoids(int nrays, const float *ray_o, const float *ray_d, int n, const float *geom, const float *live,
                    const float *channels, float znear, float zfar, float min_opacity, const float *bg,
                    float *out_rgb, float *out_depth, int32_t *out_id, int nthreads);

int orc_hardware_threads(void);

/* Checker of the CUDA path's division-free hit pretest (not a reference routine): for n object-space
 * rays (lo, ld; 3 floats each) counts the pairs the exact hit decision accepts (counts[0]), the pairs
 * the pretest keeps (counts[1]) and the accepted pairs it would drop (counts[2]; returns counts[2] != 0). */
int orc_pretest_check(int n, const float *lo, const float *ld, int64_t *counts);

/* Checker of the CUDA path's ellipsoid-plane cull (not a reference routine): for n planes (normals,
 * 3 floats each; the cull's thresholds w, which hold the plane's rounding margin; the planes' exact
 * offsets) and ellipsoids (l2w rows, 12 floats each) counts the culls (counts[0]) and the culls that
 * FP64 says are wrong, the ellipsoid reaching the plane (counts[1]; returns counts[1] != 0). */
int orc_cull_check(int n, const float *normals, const float *l2w, const float *thresholds, const double *planes,
                   int64_t *counts);

#ifdef __cplusplus
}
#endif
#endif
