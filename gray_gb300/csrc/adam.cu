// adam.cu -- one fused Adam launch over every parameter group (reference: adam_step_base_kernel and
// adam_step_sh_kernel, cuda/opt/adam.cu:13-83).
//
// The groups are flat float streams ([N,3] means are 3N floats, SH rest is 45N floats, ...), so
// the kernel is elementwise: a block takes units of 2048 consecutive floats of one group with
// float4 loads, which keeps every access coalesced.  The step count, betas, epsilon, learning rates and
// flags are read from device memory (no host synchronisation).  Arithmetic follows
// cuda/opt/adam.cu:13-22 including the bias-correction exponent step + 1 with `step` already
// incremented.
#include "gray_device.cuh"
#include "gray_internal.h"

namespace gray {

constexpr int kAdamThreads = 256;
constexpr int kAdamPerBlock = 8 * kAdamThreads;  // floats per work unit: two float4 per thread
constexpr int kMaxGroups = 7;

enum GroupKind : int { kPlain = 0, kChannels = 1, kSh = 2 };

struct AdamGroup {
    float *p, *m, *v, *g;
    long long count;
    const float *lr;
    int kind;
};

struct AdamArgs {
    AdamGroup grp[kMaxGroups];
    long long block_start[kMaxGroups + 1];
    int ngroups;
    const uint32_t *total_num_steps;
    const float *beta_1, *beta_2, *epsilon;
    const uint8_t *zero_grads, *update_channels, *enable_sh;
    const int32_t *laziness;
};

__global__ void step_count_kernel(uint32_t *total_num_steps) { *total_num_steps += 1u; }

// ibc1 / ibc2 = 1 / (1 - beta^(step+1)): the bias corrections as multiplications, leaving one
// division and one square root per element (the kernel is otherwise issue-bound on GB300).
__device__ __forceinline__ void adam_one(float &p, float &m, float &v, float &g, float lr, float b1, float b2,
                                         float ibc1, float ibc2, float eps, bool zero) {
    const float gg = g;
    m = b1 * m + (1.0f - b1) * gg;
    v = b2 * v + (1.0f - b2) * gg * gg;
    const float mh = m * ibc1;
    const float vh = v * ibc2;
    p = p - lr * mh / (sqrtf(vh) + eps);
    if (zero) g = gg * 0.0f;
}

// One float4 of one group (or the scalar tail of a group whose length is not a multiple of 4).
__device__ __forceinline__ void adam_vec(const AdamGroup &G, long long e0, bool do_adam, float lr, float b1, float b2,
                                         float bc1, float bc2, float eps, bool zero, bool vec, float4 p, float4 m,
                                         float4 v, float4 g) {
    if (vec) {
        if (do_adam) {
            adam_one(p.x, m.x, v.x, g.x, lr, b1, b2, bc1, bc2, eps, zero);
            adam_one(p.y, m.y, v.y, g.y, lr, b1, b2, bc1, bc2, eps, zero);
            adam_one(p.z, m.z, v.z, g.z, lr, b1, b2, bc1, bc2, eps, zero);
            adam_one(p.w, m.w, v.w, g.w, lr, b1, b2, bc1, bc2, eps, zero);
            *reinterpret_cast<float4 *>(G.p + e0) = p;
            *reinterpret_cast<float4 *>(G.m + e0) = m;
            *reinterpret_cast<float4 *>(G.v + e0) = v;
        } else {
            g = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        if (zero) *reinterpret_cast<float4 *>(G.g + e0) = g;
    } else {
        for (long long e = e0; e < G.count && e < e0 + 4; e++) {
            if (do_adam) {
                float pp = G.p[e], mm = G.m[e], vv = G.v[e], gg = G.g[e];
                adam_one(pp, mm, vv, gg, lr, b1, b2, bc1, bc2, eps, zero);
                G.p[e] = pp;
                G.m[e] = mm;
                G.v[e] = vv;
                if (zero) G.g[e] = gg;
            } else {
                G.g[e] = 0.0f;
            }
        }
    }
}

// Persistent grid: each block computes the bias corrections once, then takes units of
// kAdamPerBlock floats of one group (grid-stride); a thread loads both of its float4s of every
// stream before updating either, so 128 bytes per thread are in flight.
__global__ void __launch_bounds__(kAdamThreads) adam_kernel(const AdamArgs a) {
    __shared__ float s_bc[2];
    const int step = (int)*a.total_num_steps;
    const float b1 = *a.beta_1, b2 = *a.beta_2, eps = *a.epsilon;
    const bool zero = *a.zero_grads != 0;
    const bool sh_on = *a.enable_sh && *a.laziness > 0 && step % *a.laziness == 0;
    const bool chan_on = *a.update_channels != 0;
    if (threadIdx.x == 0) {
        s_bc[0] = 1.0f / (1.0f - adam_pow(b1, step + 1));
        s_bc[1] = 1.0f / (1.0f - adam_pow(b2, step + 1));
    }
    __syncthreads();
    const float bc1 = s_bc[0], bc2 = s_bc[1];
    const long long units = a.block_start[a.ngroups];
    int gi = 0;
    for (long long u = blockIdx.x; u < units; u += gridDim.x) {
        while (gi + 1 < a.ngroups && u >= a.block_start[gi + 1]) gi++;
        const AdamGroup &G = a.grp[gi];
        if (G.kind == kSh && !sh_on) continue;
        const bool do_adam = !(G.kind == kChannels && !chan_on);
        if (!do_adam && !zero) continue;
        const float lr = *G.lr;
        const long long e0 = (u - a.block_start[gi]) * kAdamPerBlock + 4LL * threadIdx.x;
        const long long e1 = e0 + kAdamPerBlock / 2;
        const bool aligned = ((reinterpret_cast<uintptr_t>(G.p) | reinterpret_cast<uintptr_t>(G.m) |
                               reinterpret_cast<uintptr_t>(G.v) | reinterpret_cast<uintptr_t>(G.g)) & 15u) == 0;
        const bool v0 = aligned && e0 + 3 < G.count, v1 = aligned && e1 + 3 < G.count;
        const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        float4 p0 = z, m0 = z, q0 = z, g0 = z, p1 = z, m1 = z, q1 = z, g1 = z;
        if (v0) {
            p0 = *reinterpret_cast<const float4 *>(G.p + e0);
            m0 = *reinterpret_cast<const float4 *>(G.m + e0);
            q0 = *reinterpret_cast<const float4 *>(G.v + e0);
            g0 = *reinterpret_cast<const float4 *>(G.g + e0);
        }
        if (v1) {
            p1 = *reinterpret_cast<const float4 *>(G.p + e1);
            m1 = *reinterpret_cast<const float4 *>(G.m + e1);
            q1 = *reinterpret_cast<const float4 *>(G.v + e1);
            g1 = *reinterpret_cast<const float4 *>(G.g + e1);
        }
        if (e0 < G.count) adam_vec(G, e0, do_adam, lr, b1, b2, bc1, bc2, eps, zero, v0, p0, m0, q0, g0);
        if (e1 < G.count) adam_vec(G, e1, do_adam, lr, b1, b2, bc1, bc2, eps, zero, v1, p1, m1, q1, g1);
    }
}

cudaError_t launch_adam(const gray_params &p, cudaStream_t s) {
    const gray_gaussians &g = p.gaussians;
    step_count_kernel<<<1, 1, 0, s>>>(p.metadata.total_num_steps);
    if (g.count <= 0) return cudaGetLastError();
    const long long n = g.count;
    AdamArgs a;
    int k = 0;
    auto add = [&](float *pp, float *mm, float *vv, float *gg, long long cnt, const float *lr, int kind) {
        a.grp[k] = AdamGroup{pp, mm, vv, gg, cnt, lr, kind};
        k++;
    };
    add(g.channels, g.first_moment_channels, g.second_moment_channels, g.grad_channels, 3 * n, g.lr_channels, kChannels);
    add(g.opacity, g.first_moment_opacity, g.second_moment_opacity, g.grad_opacity, n, g.lr_opacity, kPlain);
    add(g.mean, g.first_moment_mean, g.second_moment_mean, g.grad_mean, 3 * n, g.lr_mean, kPlain);
    add(g.rotation, g.first_moment_rotation, g.second_moment_rotation, g.grad_rotation, 4 * n, g.lr_rotation, kPlain);
    add(g.scale, g.first_moment_scale, g.second_moment_scale, g.grad_scale, 3 * n, g.lr_scale, kPlain);
    add(reinterpret_cast<float *>(g.sh_coeffs_dc), g.first_moment_sh_coeffs_dc, g.second_moment_sh_coeffs_dc,
        g.grad_sh_coeffs_dc, 3 * n, g.lr_sh_dc, kSh);
    if (g.num_sh_coeffs > 0)
        add(reinterpret_cast<float *>(g.sh_coeffs_rest), g.first_moment_sh_coeffs_rest,
            g.second_moment_sh_coeffs_rest, g.grad_sh_coeffs_rest, 3 * n * g.num_sh_coeffs, g.lr_sh_rest, kSh);
    a.ngroups = k;
    long long blocks = 0;
    for (int i = 0; i < k; i++) {
        a.block_start[i] = blocks;
        blocks += (a.grp[i].count + kAdamPerBlock - 1) / kAdamPerBlock;
    }
    a.block_start[k] = blocks;
    a.total_num_steps = p.metadata.total_num_steps;
    a.beta_1 = g.beta_1;
    a.beta_2 = g.beta_2;
    a.epsilon = g.epsilon;
    a.zero_grads = p.config.zero_grads;
    a.update_channels = p.config.update_channels;
    a.enable_sh = p.config.enable_sh;
    a.laziness = g.sh_update_laziness;
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, adam_kernel, kAdamThreads, 0)) != cudaSuccess)
        return e;
    const long long want = (long long)sms * (per_sm > 0 ? per_sm : 1);
    adam_kernel<<<(unsigned int)(blocks < want ? blocks : want), kAdamThreads, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace gray
