// scene.cu -- per-Gaussian kernels: instance snapshot, per-forward preparation (live opacity,
// scaling factor, SH colour) and the post-backward gradient fold with the SH backward.
#include "gray_device.cuh"
#include "gray_internal.h"

namespace gray {

// Real SH basis without the DC term, degrees 1..3 (15 functions) in the reference's order
// (cuda/utils/sh.cu:54-67: per degree l, m = l..1 -> sqrt2 Im, m = 0, m = 1..l -> sqrt2 Re).
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

__device__ __forceinline__ void sh_basis(float x, float y, float z, float b[15]) {
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

__device__ __forceinline__ void sh_basis_grad(float x, float y, float z, float dx[15], float dy[15], float dz[15]) {
    float xx = x * x, yy = y * y, zz = z * z;
    dx[0] = 0.0f;          dy[0] = -SH_C1;          dz[0] = 0.0f;
    dx[1] = 0.0f;          dy[1] = 0.0f;            dz[1] = SH_C1;
    dx[2] = -SH_C1;        dy[2] = 0.0f;            dz[2] = 0.0f;
    dx[3] = SH_C2_0 * y;   dy[3] = SH_C2_0 * x;     dz[3] = 0.0f;
    dx[4] = 0.0f;          dy[4] = -SH_C2_0 * z;    dz[4] = -SH_C2_0 * y;
    dx[5] = SH_C2_2 * (-2.0f * x); dy[5] = SH_C2_2 * (-2.0f * y); dz[5] = SH_C2_2 * (4.0f * z);
    dx[6] = -SH_C2_0 * z;  dy[6] = 0.0f;            dz[6] = -SH_C2_0 * x;
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

__device__ __forceinline__ int sh_count(int degree) {
    return degree <= 0 ? 0 : degree == 1 ? 3 : degree == 2 ? 8 : 15;
}

// ---------------------------------------------------------------------------------------------
// Instance snapshot (reference: populate_bvh_kernel + create_transform_matrix,
// cuda/optix/bvh_wrapper.cu:8-59).  Writes the world->unit-sphere rows (M | mu), the
// unit-sphere->world rows R diag(s), the leaf box and the visibility of each Gaussian.
// ---------------------------------------------------------------------------------------------
__global__ void snapshot_kernel(int n, const float *__restrict__ mean, const float4 *__restrict__ rotation,
                                const float *__restrict__ scale, const float *__restrict__ opacity,
                                const float *__restrict__ cfg_alpha_threshold, const float *__restrict__ cfg_exp_power,
                                const float *__restrict__ cfg_gsf, float4 *__restrict__ geom, float4 *__restrict__ l2w,
                                float4 *__restrict__ aabb, uint8_t *__restrict__ visible) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float athr = *cfg_alpha_threshold, p = *cfg_exp_power, gsf = *cfg_gsf;
    float o = sigmoid_act(opacity[i]);
    float sf = scaling_factor(o, athr, p);
    float s[3];
#pragma unroll
    for (int k = 0; k < 3; k++) s[k] = gexp(scale[3 * i + k]) * sf * gsf;
    float4 q = rotation[i];
    float r = q.x, x = q.y, y = q.z, z = q.w;
    float norm = sqrtf(r * r + x * x + y * y + z * z);
    r = r / norm;
    x = x / norm;
    y = y / norm;
    z = z / norm;
    float R[9];
    R[0] = 1.0f - 2.0f * (y * y + z * z);
    R[1] = 2.0f * (x * y - r * z);
    R[2] = 2.0f * (x * z + r * y);
    R[3] = 2.0f * (x * y + r * z);
    R[4] = 1.0f - 2.0f * (x * x + z * z);
    R[5] = 2.0f * (y * z - r * x);
    R[6] = 2.0f * (x * z - r * y);
    R[7] = 2.0f * (y * z + r * x);
    R[8] = 1.0f - 2.0f * (x * x + y * y);
    float mu[3] = {mean[3 * i], mean[3 * i + 1], mean[3 * i + 2]};
    bool vis = sf > 0.0f && s[0] > 0.0f && s[1] > 0.0f && s[2] > 0.0f && isfinite(s[0]) && isfinite(s[1]) &&
               isfinite(s[2]) && isfinite(mu[0]) && isfinite(mu[1]) && isfinite(mu[2]);
    float L[9];
#pragma unroll
    for (int rr = 0; rr < 3; rr++) {
#pragma unroll
        for (int c = 0; c < 3; c++) L[3 * rr + c] = R[3 * rr + c] * s[c];
    }
#pragma unroll
    for (int rr = 0; rr < 3; rr++) {
        float4 gr;
        gr.x = vis ? R[rr] / s[rr] : 0.0f;
        gr.y = vis ? R[3 + rr] / s[rr] : 0.0f;
        gr.z = vis ? R[6 + rr] / s[rr] : 0.0f;
        gr.w = mu[rr];
        geom[3 * i + rr] = gr;
        l2w[3 * i + rr] = make_float4(L[3 * rr], L[3 * rr + 1], L[3 * rr + 2], mu[rr]);
    }
    float4 bmin, bmax;
    if (vis) {
        float pad_mu = 2.0e-6f * (fabsf(mu[0]) + fabsf(mu[1]) + fabsf(mu[2]));
        float h[3];
#pragma unroll
        for (int rr = 0; rr < 3; rr++) {
            float a0 = L[3 * rr], a1 = L[3 * rr + 1], a2 = L[3 * rr + 2];
            float hh = sqrtf(a0 * a0 + a1 * a1 + a2 * a2);
            h[rr] = hh + hh * 1.0e-4f + pad_mu + 1.0e-30f;
        }
        bmin = make_float4(mu[0] - h[0], mu[1] - h[1], mu[2] - h[2], 0.0f);
        bmax = make_float4(mu[0] + h[0], mu[1] + h[1], mu[2] + h[2], 0.0f);
    } else {
        bool fin = isfinite(mu[0]) && isfinite(mu[1]) && isfinite(mu[2]);
        bmin = fin ? make_float4(mu[0], mu[1], mu[2], 0.0f) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        bmax = bmin;
    }
    aabb[2 * i] = bmin;
    aabb[2 * i + 1] = bmax;
    visible[i] = vis ? 1 : 0;
}

cudaError_t launch_snapshot(const gray_params &p, cudaStream_t s) {
    const gray_gaussians &g = p.gaussians;
    if (g.count <= 0) return cudaSuccess;
    snapshot_kernel<<<blocks_for(g.count), kThreads, 0, s>>>(
        g.count, g.mean, reinterpret_cast<const float4 *>(g.rotation), g.scale, g.opacity, p.config.alpha_threshold,
        p.config.exp_power, p.config.global_scale_factor, reinterpret_cast<float4 *>(p.scene.geom),
        reinterpret_cast<float4 *>(p.scene.l2w), reinterpret_cast<float4 *>(p.scene.aabb), p.scene.visible);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Per-forward preparation: live opacity and scaling factor for the intersection test
// (cuda/shaders.cu:21-24, 51-53 read them per hit), and the SH colour
// (reference: sh_forward_kernel, cuda/utils/sh.cu:224-247).  SH coefficient rows are staged
// through shared memory with coalesced loads.
// ---------------------------------------------------------------------------------------------
constexpr int kPrepThreads = 128;

template <typename SHT>
__device__ __forceinline__ float sh_load(const SHT *p);
template <>
__device__ __forceinline__ float sh_load<float>(const float *p) {
    return *p;
}
template <>
__device__ __forceinline__ float sh_load<__half>(const __half *p) {
    return __half2float(*p);
}

template <typename SHT>
__global__ void __launch_bounds__(kPrepThreads) forward_prep_kernel(
    int n, int num_rest, const float *__restrict__ opacity, const uint8_t *__restrict__ visible,
    const float *__restrict__ cfg_alpha_threshold, const float *__restrict__ cfg_exp_power,
    const uint8_t *__restrict__ cfg_enable_sh, const int32_t *__restrict__ current_sh_degree, int max_sh_degree,
    const float *__restrict__ mean, const float *__restrict__ cam_origin, const SHT *__restrict__ sh_dc,
    const SHT *__restrict__ sh_rest, float *__restrict__ channels, float2 *__restrict__ live,
    uint8_t *__restrict__ was_visible, uint32_t *__restrict__ total_num_calls, uint32_t *__restrict__ hit_counter,
    int reset_frame) {
    extern __shared__ float stage[];  // kPrepThreads * num_rest * 3 floats
    const int i0 = blockIdx.x * kPrepThreads;
    const int i = i0 + threadIdx.x;
    if (reset_frame && blockIdx.x == 0 && threadIdx.x == 0) {
        *total_num_calls += 1u;
        *hit_counter = 0u;
    }
    const bool enable_sh = *cfg_enable_sh != 0;
    int degree = *current_sh_degree;
    degree = min(min(degree, 3), max_sh_degree);
    const int nb = enable_sh ? sh_count(degree) : 0;
    if (nb > 0) {
        // coalesced staging of this block's rows of sh_rest ([n, num_rest, 3])
        const int rows = min(kPrepThreads, n - i0);
        const int per = num_rest * 3;
        const long long base = (long long)i0 * per;
        for (int t = threadIdx.x; t < rows * per; t += kPrepThreads) stage[t] = sh_load<SHT>(sh_rest + base + t);
    }
    __syncthreads();
    if (i >= n) return;
    if (reset_frame) was_visible[i] = 0;
    const float athr = *cfg_alpha_threshold, pw = *cfg_exp_power;
    float o = sigmoid_act(opacity[i]);
    float sf = scaling_factor(o, athr, pw);
    live[i] = make_float2(visible[i] ? o : __int_as_float(0xff800000), sf);
    if (!enable_sh) return;
    float v[3];
#pragma unroll
    for (int k = 0; k < 3; k++) v[k] = mean[3 * i + k] - cam_origin[k];
    float len2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    float inv = 1.0f / sqrtf(fmaxf(len2, 1e-20f));
    float b[15];
    sh_basis(v[0] * inv, v[1] * inv, v[2] * inv, b);
    const float *row = stage + threadIdx.x * num_rest * 3;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        float acc = SH_C0 * sh_load<SHT>(sh_dc + 3 * i + c);
#pragma unroll
        for (int j = 0; j < 15; j++)
            if (j < nb) acc = fmaf(b[j], row[3 * j + c], acc);
        acc = acc + 0.5f;
        channels[3 * i + c] = fmaxf(acc, 0.0f);
    }
}

cudaError_t launch_forward_prep(const gray_params &p, bool reset_frame, cudaStream_t s) {
    const gray_gaussians &g = p.gaussians;
    if (reset_frame && g.count <= 0) {
        // still count the call and empty the hit list
        cudaError_t e = cudaMemsetAsync(p.hitlist.total_words, 0, sizeof(uint32_t), s);
        return e;
    }
    if (g.count <= 0) return cudaSuccess;
    const int num_rest = g.num_sh_coeffs;
    const size_t smem = (size_t)kPrepThreads * (size_t)(num_rest > 0 ? num_rest : 1) * 3 * sizeof(float);
    const unsigned int blocks = blocks_for(g.count, kPrepThreads);
    if (g.sh_is_fp16) {
        forward_prep_kernel<__half><<<blocks, kPrepThreads, smem, s>>>(
            g.count, num_rest, g.opacity, p.scene.visible, p.config.alpha_threshold, p.config.exp_power,
            p.config.enable_sh, g.current_sh_degree, g.max_sh_degree, g.mean, p.camera.origin,
            reinterpret_cast<const __half *>(g.sh_coeffs_dc), reinterpret_cast<const __half *>(g.sh_coeffs_rest),
            g.channels, reinterpret_cast<float2 *>(p.scene.live), g.was_visible, p.metadata.total_num_calls,
            p.hitlist.total_words, reset_frame ? 1 : 0);
    } else {
        forward_prep_kernel<float><<<blocks, kPrepThreads, smem, s>>>(
            g.count, num_rest, g.opacity, p.scene.visible, p.config.alpha_threshold, p.config.exp_power,
            p.config.enable_sh, g.current_sh_degree, g.max_sh_degree, g.mean, p.camera.origin,
            reinterpret_cast<const float *>(g.sh_coeffs_dc), reinterpret_cast<const float *>(g.sh_coeffs_rest),
            g.channels, reinterpret_cast<float2 *>(p.scene.live), g.was_visible, p.metadata.total_num_calls,
            p.hitlist.total_words, reset_frame ? 1 : 0);
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Batched preparation: live values once and the SH colour of every Gaussian for each of
// `nviews` camera origins (one pass over the SH coefficients serves all views).  Same
// arithmetic as forward_prep_kernel, so a view's colours are bit-identical to a plain forward.
// ---------------------------------------------------------------------------------------------
template <typename SHT>
__global__ void __launch_bounds__(kPrepThreads) batch_prep_kernel(
    int n, int num_rest, const float *__restrict__ opacity, const uint8_t *__restrict__ visible,
    const float *__restrict__ cfg_alpha_threshold, const float *__restrict__ cfg_exp_power,
    const uint8_t *__restrict__ cfg_enable_sh, const int32_t *__restrict__ current_sh_degree, int max_sh_degree,
    const float *__restrict__ mean, const float *__restrict__ origins, int nviews, const SHT *__restrict__ sh_dc,
    const SHT *__restrict__ sh_rest, const float *__restrict__ channels_in, float *__restrict__ channels_out,
    float2 *__restrict__ live) {
    extern __shared__ float stage[];
    const int i0 = blockIdx.x * kPrepThreads;
    const int i = i0 + threadIdx.x;
    const bool enable_sh = *cfg_enable_sh != 0;
    int degree = min(min(*current_sh_degree, 3), max_sh_degree);
    const int nb = enable_sh ? sh_count(degree) : 0;
    if (nb > 0) {
        const int rows = min(kPrepThreads, n - i0);
        const int per = num_rest * 3;
        const long long base = (long long)i0 * per;
        for (int t = threadIdx.x; t < rows * per; t += kPrepThreads) stage[t] = sh_load<SHT>(sh_rest + base + t);
    }
    __syncthreads();
    if (i >= n) return;
    const float athr = *cfg_alpha_threshold, pw = *cfg_exp_power;
    float o = sigmoid_act(opacity[i]);
    float sf = scaling_factor(o, athr, pw);
    live[i] = make_float2(visible[i] ? o : __int_as_float(0xff800000), sf);
    const float m0 = mean[3 * i], m1 = mean[3 * i + 1], m2 = mean[3 * i + 2];
    const float *row = stage + threadIdx.x * num_rest * 3;
    float dc[3];
#pragma unroll
    for (int c = 0; c < 3; c++) dc[c] = enable_sh ? sh_load<SHT>(sh_dc + 3 * i + c) : 0.0f;
    for (int v = 0; v < nviews; v++) {
        float *out = channels_out + ((size_t)v * n + i) * 3;
        if (!enable_sh) {
            out[0] = channels_in[3 * i];
            out[1] = channels_in[3 * i + 1];
            out[2] = channels_in[3 * i + 2];
            continue;
        }
        const float v0 = m0 - origins[3 * v], v1 = m1 - origins[3 * v + 1], v2 = m2 - origins[3 * v + 2];
        float len2 = v0 * v0 + v1 * v1 + v2 * v2;
        float inv = 1.0f / sqrtf(fmaxf(len2, 1e-20f));
        float b[15];
        sh_basis(v0 * inv, v1 * inv, v2 * inv, b);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            float acc = SH_C0 * dc[c];
#pragma unroll
            for (int j = 0; j < 15; j++)
                if (j < nb) acc = fmaf(b[j], row[3 * j + c], acc);
            acc = acc + 0.5f;
            out[c] = fmaxf(acc, 0.0f);
        }
    }
}

cudaError_t launch_batch_prep(const gray_params &p, const float *origins, int nviews, float *channels_out,
                              cudaStream_t s) {
    const gray_gaussians &g = p.gaussians;
    if (g.count <= 0 || nviews <= 0) return cudaSuccess;
    const int num_rest = g.num_sh_coeffs;
    const size_t smem = (size_t)kPrepThreads * (size_t)(num_rest > 0 ? num_rest : 1) * 3 * sizeof(float);
    const unsigned int blocks = blocks_for(g.count, kPrepThreads);
    if (g.sh_is_fp16) {
        batch_prep_kernel<__half><<<blocks, kPrepThreads, smem, s>>>(
            g.count, num_rest, g.opacity, p.scene.visible, p.config.alpha_threshold, p.config.exp_power,
            p.config.enable_sh, g.current_sh_degree, g.max_sh_degree, g.mean, origins, nviews,
            reinterpret_cast<const __half *>(g.sh_coeffs_dc), reinterpret_cast<const __half *>(g.sh_coeffs_rest),
            g.channels, channels_out, reinterpret_cast<float2 *>(p.scene.live));
    } else {
        batch_prep_kernel<float><<<blocks, kPrepThreads, smem, s>>>(
            g.count, num_rest, g.opacity, p.scene.visible, p.config.alpha_threshold, p.config.exp_power,
            p.config.enable_sh, g.current_sh_degree, g.max_sh_degree, g.mean, origins, nviews,
            reinterpret_cast<const float *>(g.sh_coeffs_dc), reinterpret_cast<const float *>(g.sh_coeffs_rest),
            g.channels, channels_out, reinterpret_cast<float2 *>(p.scene.live));
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Gradient fold + SH backward.  The trace backward accumulates per-Gaussian gradients with
// 16-byte vector reductions into grad_acc ([n,16]: rot4 | mean3 opacity | scale3 pruning |
// channels3 count); this kernel adds them to the reference-layout gradient arrays, sets
// was_visible, clears grad_acc and runs the SH backward for visible Gaussians (reference:
// sh_backward_kernel, cuda/utils/sh.cu:249-287).
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kPrepThreads) fold_sh_backward_kernel(
    int n, int num_rest, float4 *__restrict__ grad_acc, float *__restrict__ grad_rotation,
    float *__restrict__ grad_mean, float *__restrict__ grad_opacity, float *__restrict__ grad_scale,
    float *__restrict__ pruning_weight, float *__restrict__ grad_channels, uint8_t *__restrict__ was_visible,
    const uint8_t *__restrict__ cfg_enable_sh, const int32_t *__restrict__ current_sh_degree, int max_sh_degree,
    const float *__restrict__ mean, const float *__restrict__ cam_origin, const float *__restrict__ sh_rest,
    const float *__restrict__ channels, float *__restrict__ grad_sh_dc, float *__restrict__ grad_sh_rest) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 a0 = grad_acc[4 * i], a1 = grad_acc[4 * i + 1], a2 = grad_acc[4 * i + 2], a3 = grad_acc[4 * i + 3];
    const bool vis = a3.w > 0.0f;
    if (!vis) return;  // untouched accumulator rows are already zero
    const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    grad_acc[4 * i] = z;
    grad_acc[4 * i + 1] = z;
    grad_acc[4 * i + 2] = z;
    grad_acc[4 * i + 3] = z;
    was_visible[i] = 1;
    float4 *gr = reinterpret_cast<float4 *>(grad_rotation) + i;
    float4 r = *gr;
    *gr = make_float4(r.x + a0.x, r.y + a0.y, r.z + a0.z, r.w + a0.w);
    grad_mean[3 * i] = grad_mean[3 * i] + a1.x;
    grad_mean[3 * i + 1] = grad_mean[3 * i + 1] + a1.y;
    grad_mean[3 * i + 2] = grad_mean[3 * i + 2] + a1.z;
    grad_opacity[i] = grad_opacity[i] + a1.w;
    grad_scale[3 * i] = grad_scale[3 * i] + a2.x;
    grad_scale[3 * i + 1] = grad_scale[3 * i + 1] + a2.y;
    grad_scale[3 * i + 2] = grad_scale[3 * i + 2] + a2.z;
    pruning_weight[i] = pruning_weight[i] + a2.w;
    float gch[3];
    gch[0] = grad_channels[3 * i] + a3.x;
    gch[1] = grad_channels[3 * i + 1] + a3.y;
    gch[2] = grad_channels[3 * i + 2] + a3.z;
    grad_channels[3 * i] = gch[0];
    grad_channels[3 * i + 1] = gch[1];
    grad_channels[3 * i + 2] = gch[2];
    if (!*cfg_enable_sh) return;
    int degree = min(min(*current_sh_degree, 3), max_sh_degree);
    const int nb = sh_count(degree);
    float v[3];
#pragma unroll
    for (int k = 0; k < 3; k++) v[k] = mean[3 * i + k] - cam_origin[k];
    float len2 = fmaxf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2], 1e-20f);
    float inv = 1.0f / sqrtf(len2);
    float x = v[0] * inv, y = v[1] * inv, zc = v[2] * inv;
    float g[3];
#pragma unroll
    for (int c = 0; c < 3; c++) g[c] = channels[3 * i + c] <= 0.0f ? 0.0f : gch[c];
#pragma unroll
    for (int c = 0; c < 3; c++) grad_sh_dc[3 * i + c] = SH_C0 * g[c];
    if (nb == 0) {
        return;
    }
    float b[15], dx[15], dy[15], dz[15];
    sh_basis(x, y, zc, b);
    sh_basis_grad(x, y, zc, dx, dy, dz);
    float gd0 = 0.0f, gd1 = 0.0f, gd2 = 0.0f;
    const float *cf = sh_rest + (size_t)i * num_rest * 3;
    float *gro = grad_sh_rest + (size_t)i * num_rest * 3;
#pragma unroll
    for (int j = 0; j < 15; j++) {
        if (j < nb) {
            gro[3 * j] = b[j] * g[0];
            gro[3 * j + 1] = b[j] * g[1];
            gro[3 * j + 2] = b[j] * g[2];
            float gc = cf[3 * j] * g[0] + cf[3 * j + 1] * g[1] + cf[3 * j + 2] * g[2];
            gd0 = fmaf(dx[j], gc, gd0);
            gd1 = fmaf(dy[j], gc, gd1);
            gd2 = fmaf(dz[j], gc, gd2);
        }
    }
    float inv3 = inv * inv * inv;
    float dv = v[0] * gd0 + v[1] * gd1 + v[2] * gd2;
    grad_mean[3 * i] = grad_mean[3 * i] + (gd0 * inv - v[0] * (dv * inv3));
    grad_mean[3 * i + 1] = grad_mean[3 * i + 1] + (gd1 * inv - v[1] * (dv * inv3));
    grad_mean[3 * i + 2] = grad_mean[3 * i + 2] + (gd2 * inv - v[2] * (dv * inv3));
}

cudaError_t launch_fold_and_sh_backward(const gray_params &p, cudaStream_t s) {
    const gray_gaussians &g = p.gaussians;
    if (g.count <= 0) return cudaSuccess;
    fold_sh_backward_kernel<<<blocks_for(g.count, kPrepThreads), kPrepThreads, 0, s>>>(
        g.count, g.num_sh_coeffs, reinterpret_cast<float4 *>(p.scene.grad_acc), g.grad_rotation, g.grad_mean,
        g.grad_opacity, g.grad_scale, g.pruning_weight, g.grad_channels, g.was_visible, p.config.enable_sh,
        g.current_sh_degree, g.max_sh_degree, g.mean, p.camera.origin,
        reinterpret_cast<const float *>(g.sh_coeffs_rest), g.channels, g.grad_sh_coeffs_dc, g.grad_sh_coeffs_rest);
    return cudaGetLastError();
}

}  // namespace gray
