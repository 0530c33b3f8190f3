// scene.cu -- per-Gaussian kernels: instance snapshot, per-forward preparation (live opacity,
// scaling factor, SH colour) and the post-backward gradient fold with the SH backward.
#include "gray_bulk.cuh"
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
// The snapshot of one Gaussian from its parameters (mean, rotation quaternion (r, x, y, z), log
// scales, logit opacity): rows g of (M | mu), rows w of (L | mu), its leaf box and visibility.
struct SnapRecord {
    float4 g[3], w[3], bmin, bmax;
    bool vis;
};

__device__ __forceinline__ void snapshot_one(const float mu_in[3], float4 q, const float log_s[3], float logit_o,
                                             float athr, float p, float gsf, SnapRecord &out) {
    float o = sigmoid_act(logit_o);
    float sf = scaling_factor(o, athr, p);
    float s[3];
#pragma unroll
    for (int k = 0; k < 3; k++) s[k] = gexp(log_s[k]) * sf * gsf;
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
    const float mu[3] = {mu_in[0], mu_in[1], mu_in[2]};
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
        out.g[rr] = gr;
        out.w[rr] = make_float4(L[3 * rr], L[3 * rr + 1], L[3 * rr + 2], mu[rr]);
    }
    if (vis) {
        float pad_mu = 2.0e-6f * (fabsf(mu[0]) + fabsf(mu[1]) + fabsf(mu[2]));
        float h[3];
#pragma unroll
        for (int rr = 0; rr < 3; rr++) {
            float a0 = L[3 * rr], a1 = L[3 * rr + 1], a2 = L[3 * rr + 2];
            float hh = sqrtf(a0 * a0 + a1 * a1 + a2 * a2);
            h[rr] = hh + hh * 1.0e-4f + pad_mu + 1.0e-30f;
        }
        out.bmin = make_float4(mu[0] - h[0], mu[1] - h[1], mu[2] - h[2], 0.0f);
        out.bmax = make_float4(mu[0] + h[0], mu[1] + h[1], mu[2] + h[2], 0.0f);
    } else {
        bool fin = isfinite(mu[0]) && isfinite(mu[1]) && isfinite(mu[2]);
        out.bmin = fin ? make_float4(mu[0], mu[1], mu[2], 0.0f) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        out.bmax = out.bmin;
    }
    out.vis = vis;
}

// One thread per Gaussian of [first, n): the short tail of the bulk-pipelined kernel, and the
// whole snapshot when a pointer is not 16-byte aligned.
__global__ void snapshot_kernel(int first, int n, const float *__restrict__ mean, const float4 *__restrict__ rotation,
                                const float *__restrict__ scale, const float *__restrict__ opacity,
                                const float *__restrict__ cfg_alpha_threshold, const float *__restrict__ cfg_exp_power,
                                const float *__restrict__ cfg_gsf, float4 *__restrict__ geom, float4 *__restrict__ l2w,
                                float4 *__restrict__ aabb, uint8_t *__restrict__ visible) {
    const int i = first + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float mu[3] = {mean[3 * i], mean[3 * i + 1], mean[3 * i + 2]};
    const float ls[3] = {scale[3 * i], scale[3 * i + 1], scale[3 * i + 2]};
    SnapRecord r;
    snapshot_one(mu, rotation[i], ls, opacity[i], *cfg_alpha_threshold, *cfg_exp_power, *cfg_gsf, r);
#pragma unroll
    for (int k = 0; k < 3; k++) {
        geom[3 * i + k] = r.g[k];
        l2w[3 * i + k] = r.w[k];
    }
    aabb[2 * i] = r.bmin;
    aabb[2 * i + 1] = r.bmax;
    visible[i] = r.vis ? 1 : 0;
}

// Bulk-pipelined snapshot: a persistent block takes tiles of kSnapTile consecutive Gaussians.  One
// thread loads a tile's parameter rows (mean, rotation, scale, opacity: 44 B per Gaussian, four
// contiguous ranges) into shared memory with bulk copies completing on an mbarrier, double-buffered
// so that the next tile's loads are in flight while this one is computed; each thread computes one
// Gaussian and writes its records into a shared-memory copy of the tile's output ranges, which one
// thread then stores with four bulk copies (geom, l2w, aabb, visible: 129 B per Gaussian) while the
// block goes on.  Every copy starts on a 16-byte boundary and spans a multiple of 16 bytes (the
// launcher checks the pointers; the tile is a multiple of 16 Gaussians).  Gaussians past the last
// full tile go to snapshot_kernel.
constexpr int kSnapTile = 128;
static_assert(kSnapTile % 16 == 0, "every per-tile range must span a multiple of 16 bytes");

struct SnapIn {
    float mean[3 * kSnapTile];
    float4 rotation[kSnapTile];
    float scale[3 * kSnapTile];
    float opacity[kSnapTile];
};
struct SnapOut {
    float4 geom[3 * kSnapTile];
    float4 l2w[3 * kSnapTile];
    float4 aabb[2 * kSnapTile];
    uint8_t visible[kSnapTile];
};
constexpr uint32_t kSnapInBytes = 44u * kSnapTile;

__device__ __forceinline__ void snap_issue_loads(SnapIn &in, uint64_t *bar, int tile, const float *mean,
                                                 const float4 *rotation, const float *scale, const float *opacity) {
    const size_t g0 = (size_t)tile * kSnapTile;
    mbar_expect_tx(bar, kSnapInBytes);
    bulk_load(in.mean, mean + 3 * g0, 12u * kSnapTile, bar);
    bulk_load(in.rotation, rotation + g0, 16u * kSnapTile, bar);
    bulk_load(in.scale, scale + 3 * g0, 12u * kSnapTile, bar);
    bulk_load(in.opacity, opacity + g0, 4u * kSnapTile, bar);
}

__global__ void __launch_bounds__(kSnapTile) snapshot_bulk_kernel(
    int tiles, const float *__restrict__ mean, const float4 *__restrict__ rotation, const float *__restrict__ scale,
    const float *__restrict__ opacity, const float *__restrict__ cfg_alpha_threshold,
    const float *__restrict__ cfg_exp_power, const float *__restrict__ cfg_gsf, float4 *__restrict__ geom,
    float4 *__restrict__ l2w, float4 *__restrict__ aabb, uint8_t *__restrict__ visible, int32_t *__restrict__ status) {
    __shared__ __align__(16) SnapIn in[2];
    __shared__ __align__(16) SnapOut out;
    __shared__ __align__(8) uint64_t bar[2];
    const int t = threadIdx.x;
    if (t == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
    }
    __syncthreads();
    const float athr = *cfg_alpha_threshold, pw = *cfg_exp_power, gsf = *cfg_gsf;
    int tile = blockIdx.x;
    if (t == 0 && tile < tiles) snap_issue_loads(in[0], &bar[0], tile, mean, rotation, scale, opacity);
    int it = 0;
    bool timed_out = false;
    for (; tile < tiles; it++, tile += gridDim.x) {
        const int st = it & 1;
        const int next = tile + gridDim.x;
        if (t == 0 && next < tiles) {
            // in[st ^ 1] was last read in the previous tile, before its barriers
            fence_proxy_async();
            snap_issue_loads(in[st ^ 1], &bar[st ^ 1], next, mean, rotation, scale, opacity);
        }
        const bool ok = __syncthreads_and(mbar_wait(&bar[st], (uint32_t)(it >> 1) & 1u, kBulkWaitNs));
        if (!ok) {
            if (t == 0) atomicOr(status, GRAY_STATUS_COPY_TIMEOUT);
            timed_out = true;
            break;
        }
        SnapRecord r;
        {
            const float mu[3] = {in[st].mean[3 * t], in[st].mean[3 * t + 1], in[st].mean[3 * t + 2]};
            const float ls[3] = {in[st].scale[3 * t], in[st].scale[3 * t + 1], in[st].scale[3 * t + 2]};
            snapshot_one(mu, in[st].rotation[t], ls, in[st].opacity[t], athr, pw, gsf, r);
        }
        if (t == 0) bulk_wait_read();  // the previous tile's stores have read the staging
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 3; k++) {
            out.geom[3 * t + k] = r.g[k];
            out.l2w[3 * t + k] = r.w[k];
        }
        out.aabb[2 * t] = r.bmin;
        out.aabb[2 * t + 1] = r.bmax;
        out.visible[t] = r.vis ? 1 : 0;
        fence_proxy_async();
        __syncthreads();
        if (t == 0) {
            const size_t g0 = (size_t)tile * kSnapTile;
            bulk_store(geom + 3 * g0, out.geom, 48u * kSnapTile);
            bulk_store(l2w + 3 * g0, out.l2w, 48u * kSnapTile);
            bulk_store(aabb + 2 * g0, out.aabb, 32u * kSnapTile);
            bulk_store(visible + g0, out.visible, kSnapTile);
            bulk_commit();
        }
    }
    if (t == 0) {
        bulk_wait_all();
        if (timed_out) {
            // the loads still in flight (this tile's and the next one's) get their own bounded
            // waits, so that no copy targets this block's shared memory after it exits
            mbar_wait(&bar[it & 1], (uint32_t)(it >> 1) & 1u, kBulkWaitNs);
            if (tile + (int)gridDim.x < tiles)
                mbar_wait(&bar[(it + 1) & 1], (uint32_t)((it + 1) >> 1) & 1u, kBulkWaitNs);
        }
    }
}

cudaError_t launch_snapshot(const gray_params &p, cudaStream_t s) {
    const gray_gaussians &g = p.gaussians;
    const int n = g.count;
    if (n <= 0) return cudaSuccess;
    const float4 *rot = reinterpret_cast<const float4 *>(g.rotation);
    float4 *geom = reinterpret_cast<float4 *>(p.scene.geom), *l2w = reinterpret_cast<float4 *>(p.scene.l2w),
           *aabb = reinterpret_cast<float4 *>(p.scene.aabb);
    const bool bulk = p.status && aligned16(g.mean) && aligned16(g.rotation) && aligned16(g.scale) &&
                      aligned16(g.opacity) && aligned16(geom) && aligned16(l2w) && aligned16(aabb) &&
                      aligned16(p.scene.visible);
    const int tiles = bulk ? n / kSnapTile : 0;
    if (tiles > 0) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaError_t e;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
        if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, snapshot_bulk_kernel, kSnapTile, 0)) !=
            cudaSuccess)
            return e;
        const int want = sms * (per_sm > 0 ? per_sm : 1);
        snapshot_bulk_kernel<<<tiles < want ? tiles : want, kSnapTile, 0, s>>>(
            tiles, g.mean, rot, g.scale, g.opacity, p.config.alpha_threshold, p.config.exp_power,
            p.config.global_scale_factor, geom, l2w, aabb, p.scene.visible, p.status);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    const int first = tiles * kSnapTile;
    if (first < n)
        snapshot_kernel<<<blocks_for(n - first), kThreads, 0, s>>>(
            first, n, g.mean, rot, g.scale, g.opacity, p.config.alpha_threshold, p.config.exp_power,
            p.config.global_scale_factor, geom, l2w, aabb, p.scene.visible);
    return cudaGetLastError();
}

// The bounded wait of the pipelines above, made to run out: 16 bytes are announced on the phase and
// none are copied, so it never completes.
__global__ void copy_wait_selftest_kernel(int32_t *status, uint64_t limit_ns) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
        mbar_expect_tx(&bar, 16u);
    }
    __syncthreads();
    if (!__syncthreads_and(mbar_wait(&bar, 0u, limit_ns)) && threadIdx.x == 0)
        atomicOr(status, GRAY_STATUS_COPY_TIMEOUT);
}

cudaError_t launch_copy_wait_selftest(int32_t *status, uint64_t limit_ns, cudaStream_t s) {
    copy_wait_selftest_kernel<<<1, 32, 0, s>>>(status, limit_ns);
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

// SH colour of one Gaussian seen from cam (reference: sh_forward_kernel, cuda/utils/sh.cu:224-247);
// dc and row (its 3 * nb rest coefficients, coefficient-major) in the storage type.
template <typename SHT>
__device__ __forceinline__ void sh_colour(const float mu[3], const float *cam, const SHT *dc, const SHT *row, int nb,
                                          float out[3]) {
    float v[3];
#pragma unroll
    for (int k = 0; k < 3; k++) v[k] = mu[k] - cam[k];
    float len2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    float inv = 1.0f / sqrtf(fmaxf(len2, 1e-20f));
    float b[15];
    sh_basis(v[0] * inv, v[1] * inv, v[2] * inv, b);
#pragma unroll
    for (int c = 0; c < 3; c++) {
        float acc = SH_C0 * sh_load<SHT>(dc + c);
#pragma unroll
        for (int j = 0; j < 15; j++)
            if (j < nb) acc = fmaf(b[j], sh_load<SHT>(row + 3 * j + c), acc);
        acc = acc + 0.5f;
        out[c] = fmaxf(acc, 0.0f);
    }
}

// One thread per Gaussian of [first, n), SH rows staged through shared memory with coalesced loads:
// the tail of the bulk-pipelined kernel, and the whole pass when a pointer is not 16-byte aligned.
// count_call: this launch counts the forward call and empties the backward hit list.
template <typename SHT>
__global__ void __launch_bounds__(kPrepThreads) forward_prep_kernel(
    int first, int n, int num_rest, const float *__restrict__ opacity, const uint8_t *__restrict__ visible,
    const float *__restrict__ cfg_alpha_threshold, const float *__restrict__ cfg_exp_power,
    const uint8_t *__restrict__ cfg_enable_sh, const int32_t *__restrict__ current_sh_degree, int max_sh_degree,
    const float *__restrict__ mean, const float *__restrict__ cam_origin, const SHT *__restrict__ sh_dc,
    const SHT *__restrict__ sh_rest, float *__restrict__ channels, float2 *__restrict__ live,
    uint8_t *__restrict__ was_visible, uint32_t *__restrict__ total_num_calls, uint32_t *__restrict__ hit_counter,
    int reset_frame, int count_call) {
    extern __shared__ __align__(16) unsigned char prep_smem[];
    SHT *stage = reinterpret_cast<SHT *>(prep_smem);  // kPrepThreads * num_rest * 3 coefficients
    const int i0 = first + blockIdx.x * kPrepThreads;
    const int i = i0 + threadIdx.x;
    if (count_call && blockIdx.x == 0 && threadIdx.x == 0) {
        *total_num_calls += 1u;
        *hit_counter = 0u;
    }
    const bool enable_sh = *cfg_enable_sh != 0;
    int degree = *current_sh_degree;
    degree = min(min(degree, 3), max_sh_degree);
    const int nb = enable_sh ? sh_count(degree) : 0;
    const int per = num_rest * 3;
    if (nb > 0) {
        const int rows = min(kPrepThreads, n - i0);
        const long long base = (long long)i0 * per;
        for (int t = threadIdx.x; t < rows * per; t += kPrepThreads) stage[t] = sh_rest[base + t];
    }
    __syncthreads();
    if (i >= n) return;
    if (reset_frame) was_visible[i] = 0;
    const float athr = *cfg_alpha_threshold, pw = *cfg_exp_power;
    float o = sigmoid_act(opacity[i]);
    float sf = scaling_factor(o, athr, pw);
    live[i] = make_float2(visible[i] ? o : __int_as_float(0xff800000), sf);
    if (!enable_sh) return;
    const float mu[3] = {mean[3 * i], mean[3 * i + 1], mean[3 * i + 2]};
    float col[3];
    sh_colour<SHT>(mu, cam_origin, sh_dc + 3 * i, stage + threadIdx.x * per, nb, col);
#pragma unroll
    for (int c = 0; c < 3; c++) channels[3 * i + c] = col[c];
}

// Bulk-pipelined forward preparation: a persistent block takes tiles of kPrepTile consecutive
// Gaussians; one thread loads a tile's inputs (opacity, mean, snapshot visibility, and with SH on
// the DC and rest coefficients: contiguous ranges) into one of two shared-memory stages with bulk
// copies completing on an mbarrier, so the next tile's loads are in flight while this one is
// computed; each thread computes one Gaussian into a shared-memory copy of the tile's outputs
// (live values, colours, the reset visited flags), stored by one thread with bulk copies.  Stage
// layout (byte offsets, T = kPrepTile, b = sizeof(SHT)): opacity 0, mean 4T, visible 16T, sh_dc 17T,
// sh_rest 17T + 3Tb; every range spans a multiple of 16 bytes.  Shared memory: 16 B of barriers,
// two stages, then the output copy (colours 12T, live 8T, flags T).
constexpr int kPrepTile = 64;
static_assert(kPrepTile % 16 == 0, "every per-tile range must span a multiple of 16 bytes");
constexpr int kPrepBlocksPerSm = 4;

__host__ __device__ __forceinline__ uint32_t prep_stage_bytes(int num_rest, uint32_t sb) {
    return 17u * kPrepTile + 3u * kPrepTile * sb + (uint32_t)kPrepTile * 3u * (uint32_t)num_rest * sb;
}
__host__ __device__ __forceinline__ uint32_t prep_smem_bytes(int num_rest, uint32_t sb) {
    return 16u + 2u * prep_stage_bytes(num_rest, sb) + 21u * kPrepTile;
}

template <typename SHT>
__device__ __forceinline__ void prep_issue_loads(unsigned char *stg, uint64_t *bar, int tile, int per, bool dc,
                                                 bool rest, const float *opacity, const float *mean,
                                                 const uint8_t *visible, const SHT *sh_dc, const SHT *sh_rest) {
    constexpr uint32_t T = kPrepTile, sb = sizeof(SHT);
    const size_t g0 = (size_t)tile * T;
    const uint32_t rest_bytes = T * (uint32_t)per * sb;
    mbar_expect_tx(bar, 17u * T + (dc ? 3u * T * sb : 0u) + (rest ? rest_bytes : 0u));
    bulk_load(stg, opacity + g0, 4u * T, bar);
    bulk_load(stg + 4 * T, mean + 3 * g0, 12u * T, bar);
    bulk_load(stg + 16 * T, visible + g0, T, bar);
    if (dc) bulk_load(stg + 17 * T, sh_dc + 3 * g0, 3u * T * sb, bar);
    if (rest) bulk_load(stg + 17 * T + 3 * T * sb, sh_rest + g0 * per, rest_bytes, bar);
}

template <typename SHT>
__global__ void __launch_bounds__(kPrepTile) forward_prep_bulk_kernel(
    int tiles, int num_rest, const float *__restrict__ opacity, const uint8_t *__restrict__ visible,
    const float *__restrict__ cfg_alpha_threshold, const float *__restrict__ cfg_exp_power,
    const uint8_t *__restrict__ cfg_enable_sh, const int32_t *__restrict__ current_sh_degree, int max_sh_degree,
    const float *__restrict__ mean, const float *__restrict__ cam_origin, const SHT *__restrict__ sh_dc,
    const SHT *__restrict__ sh_rest, float *__restrict__ channels, float2 *__restrict__ live,
    uint8_t *__restrict__ was_visible, uint32_t *__restrict__ total_num_calls, uint32_t *__restrict__ hit_counter,
    int reset_frame, int32_t *__restrict__ status) {
    constexpr uint32_t T = kPrepTile, sb = sizeof(SHT);
    extern __shared__ __align__(16) unsigned char prep_smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(prep_smem);
    const int per = 3 * num_rest;
    const uint32_t stage_bytes = prep_stage_bytes(num_rest, sb);
    unsigned char *stages = prep_smem + 16;
    unsigned char *outb = stages + 2 * stage_bytes;
    float *ch_out = reinterpret_cast<float *>(outb);
    float2 *live_out = reinterpret_cast<float2 *>(outb + 12 * T);
    uint8_t *wv_out = outb + 20 * T;
    const int t = threadIdx.x;
    if (reset_frame && blockIdx.x == 0 && t == 0) {
        *total_num_calls += 1u;
        *hit_counter = 0u;
    }
    const bool enable_sh = *cfg_enable_sh != 0;
    int degree = *current_sh_degree;
    degree = min(min(degree, 3), max_sh_degree);
    const int nb = enable_sh ? sh_count(degree) : 0;
    const float athr = *cfg_alpha_threshold, pw = *cfg_exp_power;
    const float cam[3] = {cam_origin[0], cam_origin[1], cam_origin[2]};
    if (t == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
    }
    __syncthreads();
    int tile = blockIdx.x;
    if (t == 0 && tile < tiles)
        prep_issue_loads<SHT>(stages, &bar[0], tile, per, enable_sh, nb > 0, opacity, mean, visible, sh_dc, sh_rest);
    int it = 0;
    bool timed_out = false;
    for (; tile < tiles; it++, tile += gridDim.x) {
        const int st = it & 1;
        const int next = tile + gridDim.x;
        if (t == 0 && next < tiles) {
            fence_proxy_async();  // stage st ^ 1 was last read in the previous tile, before its barriers
            prep_issue_loads<SHT>(stages + (st ^ 1) * stage_bytes, &bar[st ^ 1], next, per, enable_sh, nb > 0,
                                  opacity, mean, visible, sh_dc, sh_rest);
        }
        const bool ok = __syncthreads_and(mbar_wait(&bar[st], (uint32_t)(it >> 1) & 1u, kBulkWaitNs));
        if (!ok) {
            if (t == 0) atomicOr(status, GRAY_STATUS_COPY_TIMEOUT);
            timed_out = true;
            break;
        }
        const unsigned char *stg = stages + st * stage_bytes;
        const float o = sigmoid_act(reinterpret_cast<const float *>(stg)[t]);
        const float sf = scaling_factor(o, athr, pw);
        const float2 lv = make_float2(stg[16 * T + t] ? o : __int_as_float(0xff800000), sf);
        float col[3] = {0.0f, 0.0f, 0.0f};
        if (enable_sh) {
            const float *m = reinterpret_cast<const float *>(stg + 4 * T) + 3 * t;
            const float mu[3] = {m[0], m[1], m[2]};
            const SHT *dc = reinterpret_cast<const SHT *>(stg + 17 * T) + 3 * t;
            const SHT *row = reinterpret_cast<const SHT *>(stg + 17 * T + 3 * T * sb) + per * t;
            sh_colour<SHT>(mu, cam, dc, row, nb, col);
        }
        if (t == 0) bulk_wait_read();  // the previous tile's stores have read the output copy
        __syncthreads();
        live_out[t] = lv;
#pragma unroll
        for (int c = 0; c < 3; c++) ch_out[3 * t + c] = col[c];
        wv_out[t] = 0;
        fence_proxy_async();
        __syncthreads();
        if (t == 0) {
            const size_t g0 = (size_t)tile * T;
            bulk_store(live + g0, live_out, 8u * T);
            if (enable_sh) bulk_store(channels + 3 * g0, ch_out, 12u * T);
            if (reset_frame) bulk_store(was_visible + g0, wv_out, T);
            bulk_commit();
        }
    }
    if (t == 0) {
        bulk_wait_all();
        if (timed_out) {
            // bounded waits for the loads still in flight before the block's shared memory goes
            mbar_wait(&bar[it & 1], (uint32_t)(it >> 1) & 1u, kBulkWaitNs);
            if (tile + (int)gridDim.x < tiles)
                mbar_wait(&bar[(it + 1) & 1], (uint32_t)((it + 1) >> 1) & 1u, kBulkWaitNs);
        }
    }
}

template <typename SHT>
static cudaError_t forward_prep_typed(const gray_params &p, bool reset_frame, cudaStream_t s) {
    const gray_gaussians &g = p.gaussians;
    const int n = g.count, num_rest = g.num_sh_coeffs;
    const SHT *dc = reinterpret_cast<const SHT *>(g.sh_coeffs_dc);
    const SHT *rest = reinterpret_cast<const SHT *>(g.sh_coeffs_rest);
    float2 *live = reinterpret_cast<float2 *>(p.scene.live);
    const uint32_t smem = prep_smem_bytes(num_rest, sizeof(SHT));
    const bool bulk = p.status && smem <= 48u * 1024u && aligned16(g.opacity) && aligned16(g.mean) &&
                      aligned16(p.scene.visible) && aligned16(dc) && (num_rest == 0 || aligned16(rest)) &&
                      aligned16(g.channels) && aligned16(live) && aligned16(g.was_visible);
    const int tiles = bulk ? n / kPrepTile : 0;
    cudaError_t e;
    if (tiles > 0) {
        int dev = 0, sms = 0, per_sm = 0;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
        if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, forward_prep_bulk_kernel<SHT>, kPrepTile,
                                                               smem)) != cudaSuccess)
            return e;
        // at most kPrepBlocksPerSm blocks per SM: the forward's tile schedule runs beside this kernel
        // on another stream, and its blocks need shared memory too
        const int want = sms * min(per_sm > 0 ? per_sm : 1, kPrepBlocksPerSm);
        forward_prep_bulk_kernel<SHT><<<tiles < want ? tiles : want, kPrepTile, smem, s>>>(
            tiles, num_rest, g.opacity, p.scene.visible, p.config.alpha_threshold, p.config.exp_power,
            p.config.enable_sh, g.current_sh_degree, g.max_sh_degree, g.mean, p.camera.origin, dc, rest, g.channels,
            live, g.was_visible, p.metadata.total_num_calls, p.hitlist.total_words, reset_frame ? 1 : 0, p.status);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    const int first = tiles * kPrepTile;
    if (first < n) {
        const size_t tail_smem = (size_t)kPrepThreads * (size_t)(num_rest > 0 ? num_rest : 1) * 3 * sizeof(SHT);
        forward_prep_kernel<SHT><<<blocks_for(n - first, kPrepThreads), kPrepThreads, tail_smem, s>>>(
            first, n, num_rest, g.opacity, p.scene.visible, p.config.alpha_threshold, p.config.exp_power,
            p.config.enable_sh, g.current_sh_degree, g.max_sh_degree, g.mean, p.camera.origin, dc, rest, g.channels,
            live, g.was_visible, p.metadata.total_num_calls, p.hitlist.total_words, reset_frame ? 1 : 0,
            reset_frame && tiles == 0 ? 1 : 0);
    }
    return cudaGetLastError();
}

cudaError_t launch_forward_prep(const gray_params &p, bool reset_frame, cudaStream_t s) {
    const gray_gaussians &g = p.gaussians;
    if (reset_frame && g.count <= 0) {
        // still count the call and empty the hit list
        cudaError_t e = cudaMemsetAsync(p.hitlist.total_words, 0, sizeof(uint32_t), s);
        return e;
    }
    if (g.count <= 0) return cudaSuccess;
    return g.sh_is_fp16 ? forward_prep_typed<__half>(p, reset_frame, s) : forward_prep_typed<float>(p, reset_frame, s);
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
