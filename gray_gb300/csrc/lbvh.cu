// lbvh.cu -- linear BVH over the Gaussians' leaf boxes (replaces the OptiX instance
// acceleration structure built in cuda/optix/bvh_wrapper.h:89-115 and refit in :25-39).
//
// Build: scene bounds of the leaf-box centroids -> 30-bit Morton codes -> stable LSD radix
// sort of (code, gaussian id) with 8-bit digits (4 passes, no CUB) -> Karras (2012)
// hierarchy, one thread per internal node -> bottom-up boxes.
// Refit: bottom-up boxes only; each internal node is finished by the second of its two
// children to arrive (one visit counter per node, no spinning): first inside blocks of 256 sorted
// leaves with shared-memory counters, then the upper tree from a queue of block-boundary nodes.
//
// Node layout (16 floats): child0 box (minx miny minz maxx maxy maxz), child1 box, child0 link,
// child1 link, leaves below the node, leaves below child0 (both as uint32 bits).  A link with
// GRAY_LEAF_BIT set names a Gaussian; otherwise an internal node.  Parents (int_parent per internal
// node, leaf_parent per sorted leaf) carry kSecondChild when the node or leaf is its parent's second
// child, so a refit knows which child box it fills without reading the parent; the root's parent
// is -1.  Everything here is deterministic; the CPU oracle restates it bit-exactly.
#include "gray_device.cuh"
#include "gray_internal.h"

namespace gray {

__device__ __forceinline__ uint32_t f2ord(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__global__ void bounds_init_kernel(uint32_t *bounds) {
    int t = threadIdx.x;
    if (t < 3) bounds[t] = 0xFFFFFFFFu;
    else if (t < 6) bounds[t] = 0u;
}

// Scene bounds of the leaf-box centroids (finite ones only).  A grid-stride loop keeps each thread's
// min/max in registers; warps and then the block reduce them, and one thread per block folds the
// block's six values into the six global words (order-preserving encodings, so integer atomics do
// float min/max).  min/max are exact, so the result does not depend on the order of the work.
constexpr int kBoundsThreads = 256;
constexpr int kBoundsMaxBlocks = 1216;

__global__ void __launch_bounds__(kBoundsThreads) bounds_kernel(int n, const float4 *__restrict__ aabb,
                                                                uint32_t *__restrict__ bounds) {
    __shared__ float part[kBoundsThreads / 32][6];
    float lo[3] = {__int_as_float(0x7f800000), __int_as_float(0x7f800000), __int_as_float(0x7f800000)};
    float hi[3] = {__int_as_float(0xff800000), __int_as_float(0xff800000), __int_as_float(0xff800000)};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 a = aabb[2 * i], b = aabb[2 * i + 1];
        const float c[3] = {(a.x + b.x) * 0.5f, (a.y + b.y) * 0.5f, (a.z + b.z) * 0.5f};
        if (isfinite(c[0]) && isfinite(c[1]) && isfinite(c[2])) {
#pragma unroll
            for (int k = 0; k < 3; k++) {
                lo[k] = fminf(lo[k], c[k]);
                hi[k] = fmaxf(hi[k], c[k]);
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], off));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], off));
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            part[warp][k] = lo[k];
            part[warp][3 + k] = hi[k];
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int w = 1; w < kBoundsThreads / 32; w++) {
#pragma unroll
            for (int k = 0; k < 3; k++) {
                lo[k] = fminf(lo[k], part[w][k]);
                hi[k] = fmaxf(hi[k], part[w][3 + k]);
            }
        }
#pragma unroll
        for (int k = 0; k < 3; k++) {
            if (lo[k] <= hi[k]) {
                atomicMin(&bounds[k], f2ord(lo[k]));
                atomicMax(&bounds[3 + k], f2ord(hi[k]));
            }
        }
    }
}

__device__ __forceinline__ uint32_t expand10(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__global__ void morton_kernel(int n, const float4 *__restrict__ aabb, const uint32_t *__restrict__ bounds,
                              uint32_t *__restrict__ codes, uint32_t *__restrict__ ids) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 a = aabb[2 * i], b = aabb[2 * i + 1];
    float c[3] = {(a.x + b.x) * 0.5f, (a.y + b.y) * 0.5f, (a.z + b.z) * 0.5f};
    bool fin = true;
    uint32_t q[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        fin = fin && isfinite(c[k]);
        float lo = ord2f(bounds[k]), hi = ord2f(bounds[3 + k]);
        float ext = hi - lo;
        float t = ext > 0.0f ? (c[k] - lo) / ext : 0.0f;
        float s = fminf(fmaxf(t * 1024.0f, 0.0f), 1023.0f);
        q[k] = fin ? (uint32_t)s : 0u;
    }
    codes[i] = fin ? ((expand10(q[0]) << 2) | (expand10(q[1]) << 1) | expand10(q[2])) : 0x40000000u;
    ids[i] = (uint32_t)i;
}

// ---------------------------------------------------------------------------------------------
// Stable LSD radix sort, 8-bit digits.  A tile is kSortThreads x kSortItems keys processed in
// kSortItems rounds of kSortThreads consecutive keys, so tile order == round-major order.
// ---------------------------------------------------------------------------------------------
// (kSortThreads, kSortItems, kSortTile and sort_tmp_words are in gray_internal.h)
constexpr int kSortWarps = kSortThreads / 32;

__global__ void __launch_bounds__(kSortThreads) radix_hist_kernel(int n, int shift, const uint32_t *__restrict__ keys,
                                                                 uint32_t *__restrict__ counts, int tiles) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * kSortTile;
#pragma unroll
    for (int r = 0; r < kSortItems; r++) {
        int idx = base + r * kSortThreads + threadIdx.x;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 0xFFu], 1u);
    }
    __syncthreads();
    counts[threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of each digit's row of tile counts (counts is digit-major: counts[d * tiles + tile]),
// one block per digit, coalesced; the row's total goes to totals[d].  The scatter kernel adds each
// digit's base (the exclusive scan of the 256 totals) itself.
constexpr int kScanThreads = 512;

__global__ void __launch_bounds__(kScanThreads) radix_row_scan_kernel(uint32_t *__restrict__ counts, int tiles,
                                                                      uint32_t *__restrict__ totals) {
    __shared__ uint32_t wsum[kScanThreads / 32];
    __shared__ uint32_t carry;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    uint32_t *row = counts + (size_t)blockIdx.x * tiles;
    if (t == 0) carry = 0u;
    __syncthreads();
    for (int c0 = 0; c0 < tiles; c0 += kScanThreads) {
        const int i = c0 + t;
        const uint32_t v = i < tiles ? row[i] : 0u;
        uint32_t x = v;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += y;
        }
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = lane < kScanThreads / 32 ? wsum[lane] : 0u;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, w, off);
                if (lane >= off) w += y;
            }
            if (lane < kScanThreads / 32) wsum[lane] = w;  // inclusive over warps
        }
        __syncthreads();
        const uint32_t before = carry + (warp > 0 ? wsum[warp - 1] : 0u);
        if (i < tiles) row[i] = before + x - v;
        __syncthreads();
        if (t == 0) carry += wsum[kScanThreads / 32 - 1];
        __syncthreads();
    }
    if (t == 0) totals[blockIdx.x] = carry;
}

__global__ void __launch_bounds__(kSortThreads) radix_scatter_kernel(int n, int shift,
                                                                    const uint32_t *__restrict__ keys_in,
                                                                    const uint32_t *__restrict__ vals_in,
                                                                    uint32_t *__restrict__ keys_out,
                                                                    uint32_t *__restrict__ vals_out,
                                                                    const uint32_t *__restrict__ offsets, int tiles,
                                                                    const uint32_t *__restrict__ totals) {
    __shared__ uint32_t warp_cnt[kSortWarps][256];
    __shared__ uint32_t digit_run[256];
    __shared__ uint32_t digit_off[256];
    __shared__ uint32_t wsum[kSortWarps];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    digit_run[t] = 0;
    {   // digit t's base: exclusive scan of the 256 digit totals (one per thread)
        const uint32_t v = totals[t];
        uint32_t x = v;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += y;
        }
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        uint32_t before = 0u;
        for (int w = 0; w < warp; w++) before += wsum[w];
        digit_off[t] = before + x - v + offsets[t * tiles + blockIdx.x];
    }
    const uint32_t lanemask_lt = (1u << lane) - 1u;
    const int base = blockIdx.x * kSortTile;
    for (int r = 0; r < kSortItems; r++) {
#pragma unroll
        for (int w = 0; w < kSortWarps; w++) warp_cnt[w][t] = 0;
        __syncthreads();
        const int idx = base + r * kSortThreads + t;
        const bool valid = idx < n;
        uint32_t key = valid ? keys_in[idx] : 0u, val = valid ? vals_in[idx] : 0u;
        uint32_t digit = valid ? (key >> shift) & 0xFFu : 256u + (uint32_t)lane;  // invalid lanes never match
        uint32_t peers = __match_any_sync(0xffffffffu, digit);
        uint32_t rank = __popc(peers & lanemask_lt);
        if (valid && rank == 0) warp_cnt[warp][digit] = __popc(peers);
        __syncthreads();
        {   // per digit: exclusive prefix over warps, continuing the tile's running count
            uint32_t run = digit_run[t];
#pragma unroll
            for (int w = 0; w < kSortWarps; w++) {
                uint32_t c = warp_cnt[w][t];
                warp_cnt[w][t] = run;
                run += c;
            }
            digit_run[t] = run;
        }
        __syncthreads();
        if (valid) {
            uint32_t pos = digit_off[digit] + warp_cnt[warp][digit] + rank;
            keys_out[pos] = key;
            vals_out[pos] = val;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------------------------
// Karras (2012) hierarchy over sorted codes; ties broken by sorted position.
// ---------------------------------------------------------------------------------------------
constexpr int32_t kSecondChild = 1 << 30;  // parent-word flag: the second child (counts are below 2^30)
constexpr int32_t kParentMask = kSecondChild - 1;

__device__ __forceinline__ int lbvh_delta(const uint32_t *codes, int n, int i, int j) {
    if (j < 0 || j > n - 1) return -1;
    uint32_t a = codes[i], b = codes[j];
    if (a == b) return 32 + __clz((uint32_t)i ^ (uint32_t)j);
    return __clz(a ^ b);
}

__global__ void karras_kernel(int n, const uint32_t *__restrict__ codes, const uint32_t *__restrict__ order,
                              float *__restrict__ nodes, int32_t *__restrict__ int_parent,
                              int32_t *__restrict__ leaf_parent) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int d = lbvh_delta(codes, n, i, i + 1) - lbvh_delta(codes, n, i, i - 1) >= 0 ? 1 : -1;
    int dmin = lbvh_delta(codes, n, i, i - d);
    int lmax = 2;
    while (lbvh_delta(codes, n, i, i + lmax * d) > dmin) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (lbvh_delta(codes, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = lbvh_delta(codes, n, i, j);
    int s = 0, t = l;
    do {
        t = (t + 1) / 2;
        if (lbvh_delta(codes, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    int gamma = i + s * d + (d < 0 ? d : 0);
    int lo_i = min(i, j), hi_i = max(i, j);
    uint32_t c0, c1;
    if (lo_i == gamma) {
        c0 = order[gamma] | GRAY_LEAF_BIT;
        leaf_parent[gamma] = i;
    } else {
        c0 = (uint32_t)gamma;
        int_parent[gamma] = i;
    }
    if (hi_i == gamma + 1) {
        c1 = order[gamma + 1] | GRAY_LEAF_BIT;
        leaf_parent[gamma + 1] = i | kSecondChild;
    } else {
        c1 = (uint32_t)(gamma + 1);
        int_parent[gamma + 1] = i | kSecondChild;
    }
    // words 14 and 15: leaves below the node and below its first child (the forward's frontier
    // walk reads them)
    float4 *nd = reinterpret_cast<float4 *>(nodes) + 4 * (size_t)i;
    nd[3] = make_float4(__uint_as_float(c0), __uint_as_float(c1), __uint_as_float((uint32_t)(hi_i - lo_i + 1)),
                        __uint_as_float((uint32_t)(gamma - lo_i + 1)));
    if (i == 0) int_parent[0] = -1;
}

// ---------------------------------------------------------------------------------------------
// Bottom-up boxes.  One thread per sorted leaf; the second child to reach a node unions the
// two child boxes and carries on to the parent.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ void store_child_box(float *nodes, int node, int slot, const float b[6]) {
    float *nd = nodes + 16 * (size_t)node + 6 * slot;
#pragma unroll
    for (int k = 0; k < 6; k++) __stcg(nd + k, b[k]);
}

// atomicAdd with acquire-release semantics at GPU scope: the child box stored before it is visible
// to whichever thread observes the count after it, and that thread sees the sibling's box (the
// release/acquire pair replaces two full fences).
__device__ __forceinline__ uint32_t add_acq_rel(uint32_t *p, uint32_t v) {
    uint32_t old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

// A climb longer than any tree of 2^31 leaves can be (its parent links form a cycle or the
// tree is corrupt) stops and reports instead of looping on.
__device__ __forceinline__ void refit_gave_up(int32_t *status) {
    if (status) atomicOr(status, GRAY_STATUS_REFIT_TIMEOUT);
}

__global__ void refit_kernel(int n, const float4 *__restrict__ aabb, const uint32_t *__restrict__ order,
                             const int32_t *__restrict__ leaf_parent, const int32_t *__restrict__ int_parent,
                             float *__restrict__ nodes, uint32_t *__restrict__ flags, float *__restrict__ root_box,
                             int32_t *__restrict__ status) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t gid = order[k];
    float4 a = aabb[2 * gid], b = aabb[2 * gid + 1];
    float box[6] = {a.x, a.y, a.z, b.x, b.y, b.z};
    int pw = n > 1 ? leaf_parent[k] : -1;  // parent word: index | kSecondChild, or -1
    if (pw < 0) {
        root_box[0] = box[0];
        root_box[1] = box[1];
        root_box[2] = box[2];
        root_box[3] = 0.0f;
        root_box[4] = box[3];
        root_box[5] = box[4];
        root_box[6] = box[5];
        root_box[7] = 0.0f;
        return;
    }
    for (int guard = 0; guard < 128; guard++) {
        const int p = pw & kParentMask;
        store_child_box(nodes, p, (pw & kSecondChild) ? 1 : 0, box);
        if (add_acq_rel(&flags[p], 1u) == 0u) return;
        const float *nd = nodes + 16 * (size_t)p;
        float u[6];
#pragma unroll
        for (int q = 0; q < 3; q++) {
            u[q] = fminf(__ldcg(nd + q), __ldcg(nd + 6 + q));
            u[3 + q] = fmaxf(__ldcg(nd + 3 + q), __ldcg(nd + 9 + q));
        }
#pragma unroll
        for (int q = 0; q < 6; q++) box[q] = u[q];
        pw = int_parent[p];
        if (pw < 0) {
            root_box[0] = box[0];
            root_box[1] = box[1];
            root_box[2] = box[2];
            root_box[3] = 0.0f;
            root_box[4] = box[3];
            root_box[5] = box[4];
            root_box[6] = box[5];
            root_box[7] = 0.0f;
            return;
        }
    }
    refit_gave_up(status);
}

__device__ __forceinline__ void write_root_box(float *root_box, const float box[6]) {
    root_box[0] = box[0];
    root_box[1] = box[1];
    root_box[2] = box[2];
    root_box[3] = 0.0f;
    root_box[4] = box[3];
    root_box[5] = box[4];
    root_box[6] = box[5];
    root_box[7] = 0.0f;
}

// Two-phase refit.  Phase 1: a block takes kThreads consecutive sorted leaves and climbs, as
// refit_kernel does, through the internal nodes whose leaf range lies inside the block's (a Karras
// node's index is one end of its range, so a local node's index is inside the block too).  The block
// first loads the link / leaf-count words (node words 12-15) and the parents of the nodes indexed
// base .. base + kThreads - 1 into shared memory, so the local climb makes no dependent global loads;
// visit counters and the children's boxes are in shared memory too, and the second arriver writes
// the whole 64-byte node (both child boxes and the unchanged link words): full 32-byte sectors, no
// partial-sector writes for the memory system to merge.  A climber tracks its subtree's leaf range
// [lo, hi]; a parent reached through child 0 covers [lo, lo + leaves - 1], through child 1
// [hi - leaves + 1, hi].  At the first node whose range crosses the block's edge the climber stores
// its box in the node and counts its visit in global memory; the second arriver there appends the
// node to a queue (at most one node per block boundary: the one that splits it) instead of climbing
// on, so no block stays resident for a long climb.  Phase 2: one thread per queued node climbs the
// rest of the tree with the global protocol.  Boxes are min/max unions, so the result does not
// depend on the order of the work.
__global__ void __launch_bounds__(kThreads) refit_local_kernel(int n, const float4 *__restrict__ aabb,
                                                               const uint32_t *__restrict__ order,
                                                               const int32_t *__restrict__ leaf_parent,
                                                               const int32_t *__restrict__ int_parent,
                                                               float *__restrict__ nodes, uint32_t *__restrict__ flags,
                                                               uint32_t *__restrict__ queue, float *__restrict__ root_box,
                                                               int32_t *__restrict__ status) {
    __shared__ uint32_t sflag[kThreads];
    __shared__ float sbox[kThreads][12];  // the children's boxes at each local node, one slot per child
                                          // (both may store before either counts its visit)
    __shared__ uint4 stopo[kThreads];    // node words 12-15 of the nodes base .. base + kThreads - 1
    __shared__ int32_t spar[kThreads];   // their parents
    const int base = blockIdx.x * kThreads;
    const int t = threadIdx.x;
    sflag[t] = 0u;
    if (base + t < n - 1) {
        stopo[t] = __ldcg(reinterpret_cast<const uint4 *>(nodes) + 4 * (size_t)(base + t) + 3);
        spar[t] = int_parent[base + t];
    }
    __syncthreads();
    const int k = base + t;
    if (k >= n) return;
    const uint32_t gid = order[k];
    const float4 a = aabb[2 * gid], b = aabb[2 * gid + 1];
    float box[6] = {a.x, a.y, a.z, b.x, b.y, b.z};
    int pw = n > 1 ? leaf_parent[k] : -1;  // parent word: index | kSecondChild, or -1
    if (pw < 0) {
        write_root_box(root_box, box);
        return;
    }
    int lo = k, hi = k;
    for (int guard = 0; guard < 128; guard++) {
        const int p = pw & kParentMask;
        const int slot = (pw & kSecondChild) ? 1 : 0;
        const bool in_block = p >= base && p < base + kThreads;
        uint4 q3;
        int pnext;
        if (in_block) {
            q3 = stopo[p - base];
            pnext = spar[p - base];
        } else {
            q3 = __ldcg(reinterpret_cast<const uint4 *>(nodes) + 4 * (size_t)p + 3);
            pnext = int_parent[p];
        }
        const int leaves = (int)q3.z;
        const int plo = slot == 0 ? lo : hi - leaves + 1, phi = slot == 0 ? lo + leaves - 1 : hi;
        if (plo < base || phi >= base + kThreads) {
            // the parent's range leaves the block: box into the node, global counter, then phase 2
            store_child_box(nodes, p, slot, box);
            if (add_acq_rel(&flags[p], 1u) == 0u) return;
            const uint32_t at = atomicAdd(queue, 1u);
            queue[1 + at] = (uint32_t)p;
            return;
        }
        // p is local (its range lies inside the block, and p is one end of it)
        float *sb = sbox[p - base];
#pragma unroll
        for (int q = 0; q < 6; q++) sb[6 * slot + q] = box[q];
        __threadfence_block();
        if (atomicAdd(&sflag[p - base], 1u) == 0u) return;
        __threadfence_block();
        float sib[6];
#pragma unroll
        for (int q = 0; q < 6; q++) sib[q] = sb[6 * (1 - slot) + q];
        const float *c0 = slot == 0 ? box : sib, *c1 = slot == 0 ? sib : box;
        float4 *nd = reinterpret_cast<float4 *>(nodes) + 4 * (size_t)p;
        __stcg(nd, make_float4(c0[0], c0[1], c0[2], c0[3]));
        __stcg(nd + 1, make_float4(c0[4], c0[5], c1[0], c1[1]));
        __stcg(nd + 2, make_float4(c1[2], c1[3], c1[4], c1[5]));
        __stcg(nd + 3, make_float4(__uint_as_float(q3.x), __uint_as_float(q3.y), __uint_as_float(q3.z),
                                   __uint_as_float(q3.w)));
#pragma unroll
        for (int q = 0; q < 3; q++) {
            box[q] = fminf(box[q], sib[q]);
            box[3 + q] = fmaxf(box[3 + q], sib[3 + q]);
        }
        lo = plo;
        hi = phi;
        pw = pnext;
        if (pw < 0) {
            write_root_box(root_box, box);
            return;
        }
    }
    refit_gave_up(status);
}

__global__ void __launch_bounds__(kThreads) refit_top_kernel(const int32_t *__restrict__ int_parent,
                                                             float *__restrict__ nodes, uint32_t *__restrict__ flags,
                                                             const uint32_t *__restrict__ queue,
                                                             float *__restrict__ root_box, int32_t *__restrict__ status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= queue[0]) return;
    int p = (int)queue[1 + i];
    for (int guard = 0; guard < 128; guard++) {
        // both child boxes of p are complete; its parent word (index and which child p is) is read
        // with them, so a level costs one load round trip and one atomic
        const float *nd = nodes + 16 * (size_t)p;
        const int pw = int_parent[p];
        float box[6];
#pragma unroll
        for (int q = 0; q < 3; q++) {
            box[q] = fminf(__ldcg(nd + q), __ldcg(nd + 6 + q));
            box[3 + q] = fmaxf(__ldcg(nd + 3 + q), __ldcg(nd + 9 + q));
        }
        if (pw < 0) {
            write_root_box(root_box, box);
            return;
        }
        const int pp = pw & kParentMask;
        store_child_box(nodes, pp, (pw & kSecondChild) ? 1 : 0, box);
        if (add_acq_rel(&flags[pp], 1u) == 0u) return;
        p = pp;
    }
    refit_gave_up(status);
}

cudaError_t launch_lbvh_refit(const gray_params &p, cudaStream_t s) {
    const int n = p.gaussians.count;
    if (n <= 0) return cudaSuccess;
    const gray_scene &sc = p.scene;
    cudaError_t e;
    if (n > 1) {
        e = cudaMemsetAsync(sc.refit_flags, 0, sizeof(uint32_t) * (size_t)(n - 1), s);
        if (e != cudaSuccess) return e;
    }
    const unsigned int blocks = blocks_for(n);
    if (sc.sort_tmp && n > 1) {
        // queue in the sort scratch (free outside a build's sort): count, then <= blocks - 1 nodes
        uint32_t *queue = sc.sort_tmp;
        if ((e = cudaMemsetAsync(queue, 0, sizeof(uint32_t), s)) != cudaSuccess) return e;
        refit_local_kernel<<<blocks, kThreads, 0, s>>>(n, reinterpret_cast<const float4 *>(sc.aabb), sc.order,
                                                       sc.leaf_parent, sc.int_parent, sc.nodes, sc.refit_flags, queue,
                                                       sc.root_box, p.status);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        refit_top_kernel<<<blocks_for(blocks), kThreads, 0, s>>>(sc.int_parent, sc.nodes, sc.refit_flags, queue,
                                                                 sc.root_box, p.status);
        return cudaGetLastError();
    }
    refit_kernel<<<blocks, kThreads, 0, s>>>(n, reinterpret_cast<const float4 *>(sc.aabb), sc.order, sc.leaf_parent,
                                             sc.int_parent, sc.nodes, sc.refit_flags, sc.root_box, p.status);
    return cudaGetLastError();
}

cudaError_t launch_lbvh_build(const gray_params &p, cudaStream_t s) {
    const int n = p.gaussians.count;
    if (n <= 0) return cudaSuccess;
    const gray_scene &sc = p.scene;
    cudaError_t e;
    bounds_init_kernel<<<1, 32, 0, s>>>(sc.bounds);
    bounds_kernel<<<min(blocks_for(n, kBoundsThreads), (unsigned)kBoundsMaxBlocks), kBoundsThreads, 0, s>>>(
        n, reinterpret_cast<const float4 *>(sc.aabb), sc.bounds);
    morton_kernel<<<blocks_for(n), kThreads, 0, s>>>(n, reinterpret_cast<const float4 *>(sc.aabb), sc.bounds, sc.codes,
                                                    sc.order);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const int tiles = (n + kSortTile - 1) / kSortTile;
    uint32_t *keys_alt = sc.sort_tmp, *vals_alt = sc.sort_tmp + n, *counts = sc.sort_tmp + 2 * (size_t)n;
    uint32_t *totals = counts + 256 * (size_t)tiles;
    uint32_t *kin = sc.codes, *vin = sc.order, *kout = keys_alt, *vout = vals_alt;
    for (int shift = 0; shift < 32; shift += 8) {
        radix_hist_kernel<<<tiles, kSortThreads, 0, s>>>(n, shift, kin, counts, tiles);
        radix_row_scan_kernel<<<256, kScanThreads, 0, s>>>(counts, tiles, totals);
        radix_scatter_kernel<<<tiles, kSortThreads, 0, s>>>(n, shift, kin, vin, kout, vout, counts, tiles, totals);
        uint32_t *tk = kin, *tv = vin;
        kin = kout;
        vin = vout;
        kout = tk;
        vout = tv;
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // four passes: the sorted keys/ids are back in codes/order
    if (n > 1) {
        karras_kernel<<<blocks_for(n - 1), kThreads, 0, s>>>(n, sc.codes, sc.order, sc.nodes, sc.int_parent,
                                                            sc.leaf_parent);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return launch_lbvh_refit(p, s);
}

}  // namespace gray
