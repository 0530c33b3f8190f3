// trace.cu -- forward and backward ray tracing of the Gaussians on the LBVH.
//
// Forward (replaces the OptiX launch of cuda/shaders.cu:69-106 with cuda/forward_pass.cu):
//   A block renders an 8x16-pixel tile, each warp a 4x8 (or 8x4) pixel packet of camera rays that
//   share one origin.  A per-tile kernel first walks the top of the BVH with the tile's frustum and
//   records the tile's frontier (the nodes of at most 64 leaves it reaches, sorted front to back);
//   every packet traversal starts there.  The packet traverses as a frustum: each step pops up to
//   32 nodes (one per lane) from a per-warp shared-memory stack, tests both child boxes against the
//   frustum, pushes the nearer child last and queues leaves; queued leaves are culled by an exact
//   ellipsoid-frustum test, cached in shared memory, tested by every lane against its own ray with a
//   division-free conservative pretest, and the lanes then walk their masks of possible hits through
//   the intersection program of cuda/shaders.cu:10-67, which decides each hit.  The first traversal accumulates, over ALL hits, the full transmittance
//   (an order-independent fixed-point sum of log(1 - alpha)) and the alpha-weighted colour sums of
//   the reference's truncated-tail estimate, and every traversal keeps the KB nearest hits above a
//   resume key in a per-lane shared-memory buffer of 64-bit keys (fp16 distance | gaussian id |
//   fp16 alpha).  The buffer is consumed by a state machine that reproduces the reference's
//   32-slot multi-pass selection exactly (pass boundaries, the strict `distance > tmin` drop of
//   equal distances, the 99-pass cap, zfar, t_threshold).  Composited ids are appended to the
//   backward hit list in warp-aggregated segments.  Rays from Python, jittered rays and packets
//   whose traversal overflows the shared stack take a per-ray slab traversal instead.
// Backward (cuda/backward_pass.cu:2-142): one thread per pixel walks its segments back to front,
//   recomputes alpha in fp32 and reduces the 16 per-hit gradient values into the per-Gaussian
//   accumulator: lanes holding the same Gaussian combine in a tree, and the lowest issues four
//   16-byte vector reductions.
#include "gray_bulk.cuh"
#include "gray_device.cuh"
#include "gray_internal.h"

namespace gray {

constexpr int kBlockWarpsX = 2, kBlockWarpsY = 2;  // 2x2 warp tiles per block
constexpr int kWarps = kBlockWarpsX * kBlockWarpsY;
constexpr int kFwdThreads = kWarps * 32;
constexpr int kStackWords = 2;               // warp-uniform stack of 64 entries in 2 registers per lane
constexpr int kStackMax = 32 * kStackWords;
constexpr int kPassSlots = 32;               // BUFFER_SIZE, cuda/forward_pass.cu:4
constexpr int kMaxPasses = 99;               // MAX_ITERATIONS, cuda/forward_pass.cu:3
constexpr int kMaxTraversals = 4 * kMaxPasses * 2;  // bound on re-traversals of one ray
constexpr unsigned kFull = 0xffffffffu;
constexpr int kWideStack = 256;  // per-warp shared stack of the frustum traversal
constexpr int kCand = 32;        // leaves processed per flush (one per lane)
constexpr int kQueue = 3 * kCand; // per-warp queue of leaves: < kCand before a step, + up to 64 per step
constexpr int kSchedHeader = 64;  // schedule words before the per-tile estimates
// Header words [kSchedZeroWords, kSchedHeader) outlive a forward: the automatic kernel choice (see
// plan_forward) keeps there the packet counts of the last scheduled forward and the choice the scan
// kernel made from them; only the words before them are cleared at the start of a schedule.
constexpr int kSchedZeroWords = 48;
constexpr int kStatPackets = 48;   // packets traced by the last scheduled forward
constexpr int kStatRetraced = 49;  // of them, packets that need more than one traversal with 16 slots
constexpr int kStatChoice = 50;    // kernel of the automatic choice: kChoiceNarrow or kChoiceWide
constexpr uint32_t kChoiceNarrow = 1u, kChoiceWide = 2u;
// the wide kernel (32 hit slots, four blocks per SM) is chosen when more than kWideSixteenths / 16
// of the last forward's packets need more than one traversal with 16 slots (counted the same way by
// both kernels, so the choice does not depend on which one ran), the narrow one (16 slots, six blocks
// per SM) otherwise
constexpr uint32_t kWideSixteenths = 2u;
// Per pixel tile, the BVH frontier its frustum reaches (kFrontierWords words: count, then up to
// kFrontierMax node or leaf entries); a count of kFrontierNone means "start at the root".  A frontier
// goes onto the traversal stack, so it leaves room there for the traversal's own pushes (up to 64
// per step; the stack above a frontier peaks near 70 entries on the benchmark scene).
constexpr int kFrontierWords = GRAY_FRONTIER_WORDS;
constexpr int kFrontierMax = kFrontierWords - 1;
constexpr int kFrontierSort = 256;  // sort buffer of the frontier walk (a power of two > kFrontierMax)
constexpr uint32_t kFrontierNone = 0xFFFFFFFFu;
constexpr int kFrontierCutDefault = 64;  // frontier nodes hold at most this many leaves

struct FwdArgs {
    uint32_t alloc_w, render_w, render_h;
    int n;
    int tile_w, tile_h;  // pixels of one warp packet (tile_w * tile_h == 32)
    const float *cam_origin, *fov, *w2c, *znear, *zfar;
    const float *exp_power, *alpha_threshold, *t_threshold, *eps_fwd, *bg;
    const uint8_t *render_depth, *needs_ray_output, *rays_from_python, *jitter, *grads_enabled;
    const uint8_t *render_ellipsoids;
    const float *ellipsoid_min_opacity;
    int display;  // forward_pass_display: colour only, whatever grads_enabled holds
    int auto_role;  // 0, or kChoiceNarrow / kChoiceWide: the launch of the automatic choice this is
    uint32_t *schedule;  // work order of the pixel tiles (null: tiles in launch order)
    int tiles_x, ntiles;
    uint32_t *frontier;  // per-tile BVH frontiers (null: packets start at the root)
    uint32_t frontier_cut;
    uint32_t *super_frontier;  // per super-tile coarse frontiers seeding the tile walks (null: root)
    int super_x;               // super-tiles per row
    const uint32_t *total_num_calls;
    const float4 *geom, *l2w;
    const float2 *live;
    const float *channels;
    const float4 *nodes;
    const float *root_box;
    float *out_rgb, *out_depth, *out_T, *out_fullT, *out_rem, *ray_o, *ray_d;
    int32_t *stat_hit, *stat_acc;
    uint32_t *head, *counter, *pool;
    uint32_t pool_size;
    int32_t *status;
};

// PCG32 output hash (O'Neill 2014) for the optional sub-pixel jitter.
__device__ __forceinline__ uint32_t pcg_hash(uint32_t v) {
    uint32_t state = v * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}

// Ray against an axis-aligned box widened by the ray's rounding margin eps:
// t = (b -/+ eps - o) * inv computed as fma(b, inv, c) with c_lo = -(o + eps) inv, c_hi = (eps - o) inv.
struct SlabRay {
    f3 inv, clo, chi;
};

__device__ __forceinline__ SlabRay make_slab_ray(f3 ro, f3 rd, float eps) {
    SlabRay r;
    float dx = fabsf(rd.x) < 1e-20f ? (rd.x < 0.0f ? -1e-20f : 1e-20f) : rd.x;
    float dy = fabsf(rd.y) < 1e-20f ? (rd.y < 0.0f ? -1e-20f : 1e-20f) : rd.y;
    float dz = fabsf(rd.z) < 1e-20f ? (rd.z < 0.0f ? -1e-20f : 1e-20f) : rd.z;
    r.inv = mk3(1.0f / dx, 1.0f / dy, 1.0f / dz);
    r.clo = mk3(-(ro.x + eps) * r.inv.x, -(ro.y + eps) * r.inv.y, -(ro.z + eps) * r.inv.z);
    r.chi = mk3((eps - ro.x) * r.inv.x, (eps - ro.y) * r.inv.y, (eps - ro.z) * r.inv.z);
    return r;
}

__device__ __forceinline__ bool slab_hit(const float bmin[3], const float bmax[3], const SlabRay &r) {
    float ta = fmaf(bmin[0], r.inv.x, r.clo.x), tb = fmaf(bmax[0], r.inv.x, r.chi.x);
    float tn = fminf(ta, tb), tf = fmaxf(ta, tb);
    ta = fmaf(bmin[1], r.inv.y, r.clo.y);
    tb = fmaf(bmax[1], r.inv.y, r.chi.y);
    tn = fmaxf(tn, fminf(ta, tb));
    tf = fminf(tf, fmaxf(ta, tb));
    ta = fmaf(bmin[2], r.inv.z, r.clo.z);
    tb = fmaf(bmax[2], r.inv.z, r.chi.z);
    tn = fmaxf(tn, fminf(ta, tb));
    tf = fminf(tf, fmaxf(ta, tb));
    return tn <= tf && tf >= 0.0f;
}

struct LaneState {
    // all-hit accumulators (first traversal only); ft is set from lfx when the ray finishes
    long long lfx;
    float ft;
    long long afx, cfx0, cfx1, cfx2;
    int nhit;
    // selection buffer of the current traversal
    int kcount, ncand;
    unsigned long long kmax;
    // resume key for the next traversal
    unsigned long long resume;
    bool has_resume;
};

// What one ray traces against.
struct TraceScene {
    const float4 *geom;
    const float4 *l2w;  // rows (L | mu) for the leaf cull of the frustum traversal (may be null)
    const float2 *live;
    const float *channels;
    const float4 *nodes;
    const float *root_box;
    int n;
};

struct TraceKnobs {
    float znear, zfar, athr, pw, tthr;
    bool render_depth;
};

// Backward hit list sink (counter == nullptr: do not record).
struct HitSink {
    uint32_t *counter, *pool;
    uint32_t pool_size;
};

struct RayResult {
    float T, C0, C1, C2, depth;
    LaneState st;
    int nacc;
    uint32_t head;
    bool retraced;  // the packet traversed, or with 16 hit slots would have traversed, more than once
};

// Intersection program + all-hit sums + selection for one (ray, Gaussian) pair whose snapshot rows,
// live values and colour the caller has fetched.
// LO: the rows' w column holds the object-space origin (local_origin) instead of the mean.
template <int KB, bool LO = false>
__device__ __forceinline__ void on_leaf_data(uint32_t gid, const float4 g0, const float4 g1, const float4 g2,
                                             const float2 lv, int cf0, int cf1, int cf2, bool first, f3 ro, f3 rd,
                                             const TraceKnobs &k, LaneState &st,
                                             unsigned long long (*kbuf)[kFwdThreads]) {
    float dist, alpha;
    if constexpr (LO) {
        if (!intersect_lo(g0, g1, g2, lv.x, lv.y, rd, k.athr, k.pw, k.znear, k.zfar, dist, alpha)) return;
    } else {
        if (!intersect(g0, g1, g2, lv.x, lv.y, ro, rd, k.athr, k.pw, k.znear, k.zfar, dist, alpha)) return;
    }
    const uint16_t a16 = f2h_bits(alpha), d16 = f2h_bits(dist);
    if (first) {
        add_log_transmittance(st.lfx, alpha);
        const long long a = alpha16_fixed(a16);
        st.afx += a;
        st.cfx0 += mul_fixed(a, cf0);
        st.cfx1 += mul_fixed(a, cf1);
        st.cfx2 += mul_fixed(a, cf2);
        st.nhit++;
    }
    if (!(h2f_bits(d16) > k.znear)) return;
    const unsigned long long key =
        ((unsigned long long)d16 << 48) | ((unsigned long long)gid << 16) | (unsigned long long)a16;
    if (st.has_resume && !(key > st.resume)) return;
    st.ncand++;
    const int t = threadIdx.x;
    int pos;
    if (st.kcount < KB) {
        pos = st.kcount++;
    } else if (key < st.kmax) {
        pos = KB - 1;
    } else {
        return;
    }
    while (pos > 0) {
        unsigned long long prev = kbuf[pos - 1][t];
        if (prev < key) break;
        kbuf[pos][t] = prev;
        pos--;
    }
    kbuf[pos][t] = key;
    if (st.kcount == KB) st.kmax = kbuf[KB - 1][t];
}

template <int KB>
__device__ __forceinline__ void on_leaf(const TraceScene &sc, uint32_t gid, bool want, bool first, f3 ro, f3 rd,
                                        const TraceKnobs &k, LaneState &st, unsigned long long (*kbuf)[kFwdThreads]) {
    if (!want) return;
    // every load up front (the colour too): one memory round trip per hit
    const float4 g0 = sc.geom[3 * gid], g1 = sc.geom[3 * gid + 1], g2 = sc.geom[3 * gid + 2];
    const float2 lv = sc.live[gid];
    const float *cp = sc.channels + 3 * (size_t)gid;
    on_leaf_data<KB>(gid, g0, g1, g2, lv, colour_fixed(cp[0]), colour_fixed(cp[1]), colour_fixed(cp[2]), first, ro,
                     rd, k, st, kbuf);
}

// Per-warp shared-memory copy of the queued leaves' records, filled once per flush by the lanes
// (one candidate each, all loads in flight together) and read by every lane afterwards.
struct CandCache {
    float4 g[kCand][3];  // snapshot rows with the packet's object-space origin: (M | M (o - mu))
    int4 c[kCand];       // colour in 2^-24 fixed point (x, y, z), live opacity bits (w)
    float sf[kCand];     // live scaling factor
};

__device__ __forceinline__ void stack_push(uint32_t &stk0, uint32_t &stk1, int &sp, uint32_t v, int lane,
                                           int32_t *status) {
    if (sp < kStackMax) {
        if (lane == (sp & 31)) {
            if ((sp >> 5) == 0) stk0 = v;
            else stk1 = v;
        }
        sp++;
    } else {
        raise_status(status, GRAY_STATUS_STACK_OVERFLOW);
    }
}

// Frustum of a packet of primary rays sharing one origin o: four side planes through the origin and
// the plane through the origin orthogonal to the packet's mean direction (nothing behind it can be
// hit).  Normals n point inside.  Stored per warp in shared memory as per-plane constants of the
// two tests below: pn[p] = (n, box threshold), pa[p] = (|n|, ellipsoid threshold).
struct Frustum {
    float4 pn[5];
    float4 pa[5];
};

// Frustum of the rays through the pixels [x0, x1] x [y0, y1] of a pinhole camera: the rays of the
// corner pixels span a convex cone that contains every ray of the rectangle.  root_box bounds every
// box and mean the tests will see, which bounds their rounding error: with M the largest finite
// coordinate magnitude of the root box, the tests' sums have magnitude at most |n|_1 (4M + 2|o|_1)
// and a few roundings of 2^-24 each; the thresholds leave 1e-5 of that (about 170 roundings).
// Boxes with an infinite or NaN coordinate (beyond M) give an infinite or NaN sum and always pass.
__device__ __forceinline__ float3 camera_ray3(const float *w, float fov, int px, int py, uint32_t width,
                                              uint32_t height);

// Plane e of the frustum (e < 4: the side through corner rays e and e+1; e = 4: the near plane
// orthogonal to the corners' sum).
__device__ __forceinline__ void frustum_plane(int e, f3 o, const f3 d[4], const float *root_box, float4 &pn,
                                              float4 &pa) {
    const f3 c = mk3(d[0].x + d[1].x + d[2].x + d[3].x, d[0].y + d[1].y + d[2].y + d[3].y,
                     d[0].z + d[1].z + d[2].z + d[3].z);
    float m = 0.0f;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const float v = fabsf(root_box[i]);
        if (i != 3 && i != 7 && v <= 0x1.fffffep127f) m = fmaxf(m, v);
    }
    const float o1 = fabsf(o.x) + fabsf(o.y) + fabsf(o.z);
    f3 nn = c;
    if (e < 4) {
        const f3 a = d[e], b = d[(e + 1) & 3];
        nn = mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
        if (dot3(nn, c) < 0.0f) nn = mk3(-nn.x, -nn.y, -nn.z);
    }
    const float n1 = fabsf(nn.x) + fabsf(nn.y) + fabsf(nn.z);
    const float no = fdot3(nn, o);
    const float mbox = 1e-5f * n1 * (4.0f * m + 2.0f * o1) + 1e-30f;
    const float mell = 1e-5f * n1 * (3.0f * m + o1) + 1e-30f;
    pn = make_float4(nn.x, nn.y, nn.z, 2.0f * no - mbox);
    pa = make_float4(fabsf(nn.x), fabsf(nn.y), fabsf(nn.z), no - mell);
}

// The frustum built by a whole warp (every lane calls this): lanes 0-3 trace one corner ray each,
// lanes 0-4 write one plane each.
__device__ __forceinline__ void make_frustum_warp(Frustum &fr, f3 o, const float *w2c, float fov, int x0, int y0,
                                                  int x1, int y1, uint32_t width, uint32_t height,
                                                  const float *root_box) {
    const int lane = threadIdx.x & 31;
    float3 dl = make_float3(0.0f, 0.0f, 0.0f);
    if (lane < 4) dl = camera_ray3(w2c, fov, (lane == 1 || lane == 2) ? x1 : x0, lane >= 2 ? y1 : y0, width, height);
    f3 d[4];
#pragma unroll
    for (int e = 0; e < 4; e++)
        d[e] = mk3(__shfl_sync(0xffffffffu, dl.x, e), __shfl_sync(0xffffffffu, dl.y, e), __shfl_sync(0xffffffffu, dl.z, e));
    if (lane < 5) frustum_plane(lane, o, d, root_box, fr.pn[lane], fr.pa[lane]);
    __syncwarp();
}

// Conservative box-frustum test: false only when the box lies entirely outside one plane by more
// than a rounding margin.  The box's largest signed distance along n, times two, is
// n.(bmin + bmax) + |n|.(bmax - bmin) - 2 n.o.  A NaN never culls.
__device__ __forceinline__ bool frustum_box(const Frustum &fr, const float bmin[3], const float bmax[3]) {
    const float sx = bmin[0] + bmax[0], sy = bmin[1] + bmax[1], sz = bmin[2] + bmax[2];
    const float dx = bmax[0] - bmin[0], dy = bmax[1] - bmin[1], dz = bmax[2] - bmin[2];
#pragma unroll
    for (int p = 0; p < 5; p++) {
        const float4 n = fr.pn[p], a = fr.pa[p];
        const float v = fmaf(a.z, dz, fmaf(a.y, dy, fmaf(a.x, dx, fmaf(n.z, sz, fmaf(n.y, sy, n.x * sx)))));
        if (v < n.w) return false;
    }
    return true;
}

// Conservative frustum test of a Gaussian's support ellipsoid {mu + L u : |u| <= 1} (L, mu = the
// snapshot's l2w rows): false only when the ellipsoid lies outside one plane by more than a rounding
// margin.  The ellipsoid's extent along a normal n is |L^T n| (taken 3e-5 larger for its own
// rounding), compared squared with the gap between the plane's threshold and the centre's signed
// distance (no square root; a gap below 2^-60, so that its square stays a normal float, an
// infinite extent or a NaN never culls).
// A ray can only hit a Gaussian whose ellipsoid it crosses, so a leaf whose ellipsoid misses the
// packet's frustum holds no hit of the packet even when its box passed.
__device__ __forceinline__ bool frustum_ellipsoid(const Frustum &fr, const float4 *l2w) {
    const float4 r0 = l2w[0], r1 = l2w[1], r2 = l2w[2];
#pragma unroll
    for (int p = 0; p < 5; p++) {
        const float4 n = fr.pn[p];
        const float sd = fmaf(n.z, r2.w, fmaf(n.y, r1.w, n.x * r0.w));
        const float e0 = fmaf(r2.x, n.z, fmaf(r1.x, n.y, r0.x * n.x));
        const float e1 = fmaf(r2.y, n.z, fmaf(r1.y, n.y, r0.y * n.x));
        const float e2 = fmaf(r2.z, n.z, fmaf(r1.z, n.y, r0.z * n.x));
        const float gap = fr.pa[p].w - sd;
        if (gap > 0x1.0p-60f && fmaf(e2, e2, fmaf(e1, e1, e0 * e0)) * 1.00006f < gap * gap) return false;
    }
    return true;
}

// Processes the packet's queued leaves (cand[0, nc), at most kCand = 32; every lane of the warp calls
// this together).  (1) Lane j takes candidate j: it tests the candidate's ellipsoid against the
// packet frustum and fetches its snapshot rows, live values and colour; the survivors are
// compacted into the warp's shared-memory cache, each with its object-space ray origin (the
// packet's rays share the origin, so it is computed once per candidate, not once per lane).  (2) Every lane runs the hit test of its own ray
// against every cached candidate and keeps a 32-bit mask of its possible hits (may_hit: division-free
// and conservative, a superset of the hits).  (3) The lanes walk their masks together, one candidate
// per lane per step, through the intersection program, which decides the hit, and the selection.
// The order in which a lane sees its hits does not matter: the all-hit sums are order-independent
// and the selection is by key.  The cache keeps each candidate's object-space ray origin in place of
// its mean (computed once by the fetching lane with local_origin, the arithmetic of local_ray).
template <int KB>
__device__ __forceinline__ void flush_candidates(const TraceScene &sc, const TraceKnobs &k, f3 ro, f3 rd, bool want,
                                                 bool first, LaneState &st, unsigned long long (*kbuf)[kFwdThreads],
                                                 const Frustum &fr, uint32_t *cand, CandCache &cc, int nc) {
    const int lane = threadIdx.x & 31;
    const uint32_t lanemask_lt = (1u << lane) - 1u;
    uint32_t gid = 0;
    bool keep = false;
    float4 g0, g1, g2;
    int4 cv;
    float sfv = 0.0f;
    if (lane < nc) {
        gid = cand[lane];
        g0 = sc.geom[3 * (size_t)gid];
        g1 = sc.geom[3 * (size_t)gid + 1];
        g2 = sc.geom[3 * (size_t)gid + 2];
        const float2 lv = sc.live[gid];
        const float *cp = sc.channels + 3 * (size_t)gid;
        cv = make_int4(colour_fixed(cp[0]), colour_fixed(cp[1]), colour_fixed(cp[2]), __float_as_int(lv.x));
        sfv = lv.y;
        keep = sc.l2w ? frustum_ellipsoid(fr, sc.l2w + 3 * (size_t)gid) : true;
        const f3 lo = local_origin(g0, g1, g2, ro);
        g0.w = lo.x;
        g1.w = lo.y;
        g2.w = lo.z;
    }
    const uint32_t bal = __ballot_sync(kFull, keep);
    __syncwarp();  // every read of cand[] precedes the compacting writes
    if (keep) {
        const int slot = __popc(bal & lanemask_lt);
        cand[slot] = gid;
        cc.g[slot][0] = g0;
        cc.g[slot][1] = g1;
        cc.g[slot][2] = g2;
        cc.c[slot] = cv;
        cc.sf[slot] = sfv;
    }
    nc = __popc(bal);
    __syncwarp();
    uint32_t mask = 0u;
    if (want) {
        for (int j = 0; j < nc; j++) {
            if (may_hit_lo(cc.g[j][0], cc.g[j][1], cc.g[j][2], __int_as_float(cc.c[j].w), rd, k.athr))
                mask |= 1u << j;
        }
    }
    while (__any_sync(kFull, mask != 0u)) {
        if (mask != 0u) {
            const int j = __ffs(mask) - 1;
            mask &= mask - 1u;
            const int4 c = cc.c[j];
            on_leaf_data<KB, true>(cand[j], cc.g[j][0], cc.g[j][1], cc.g[j][2],
                                   make_float2(__int_as_float(c.w), cc.sf[j]), c.x, c.y, c.z, first, ro, rd, k, st,
                                   kbuf);
        }
    }
    __syncwarp();
}

// One full traversal of the packet (camera rays with a common origin) with the node work spread
// over the lanes: each step pops up to 32 nodes, one per lane, tests their child boxes against the
// packet frustum, pushes surviving internal children and queues surviving leaves; queued leaves
// are then intersected by every lane with its own ray (on_leaf).  With a tile frontier (at
// front_base + front_off: count, entries; a count of kFrontierNone or a null base: none; base and
// offset are kept apart so that a kernel-parameter base needs no register) the traversal starts there instead
// of at the root: the frontier goes onto the stack with its first entry on top, and a frontier leaf
// is queued when it is popped.  Returns false if the shared stack overflowed (the caller then
// repeats the traversal per ray).
template <int KB>
__device__ __forceinline__ bool traverse_frustum(const TraceScene &sc, const TraceKnobs &k, f3 ro, f3 rd, bool want,
                                                 bool first, LaneState &st, unsigned long long (*kbuf)[kFwdThreads],
                                                 const Frustum &fr, uint32_t *stk, uint32_t *cand,
                                                 CandCache &cc, const uint32_t *front_base, uint32_t front_off,
                                                 int32_t *status) {
    const int lane = threadIdx.x & 31;
    const uint32_t lanemask_lt = (1u << lane) - 1u;
    const int n = sc.n;
    const float *rb = sc.root_box;
    const float rmin[3] = {rb[0], rb[1], rb[2]}, rmax[3] = {rb[4], rb[5], rb[6]};
    if (n <= 0 || !frustum_box(fr, rmin, rmax)) return true;
    if (n == 1) {
        on_leaf<KB>(sc, 0u, want, first, ro, rd, k, st, kbuf);
        return true;
    }
    const uint32_t *front = front_base ? front_base + front_off : nullptr;
    int sp = front ? (int)front[0] : -1, nc = 0;
    if (sp >= 0 && sp <= kFrontierMax) {
        for (int i = lane; i < sp; i += 32) stk[sp - 1 - i] = front[1 + i];
    } else {
        if (lane == 0) stk[0] = 0u;
        sp = 1;
    }
    __syncwarp();
    bool ok = true, draining = false;
    long long budget = (long long)n;  // a valid tree pushes each internal node at most once per traversal
    for (;;) {
        if (!draining) {
            if (sp == 0) {
                draining = true;
            } else if (--budget < 0) {
                raise_status(status, GRAY_STATUS_STACK_OVERFLOW);
                draining = true;
            } else {
                const int take = sp < 32 ? sp : 32;
                uint32_t node = GRAY_NULL;
                if (lane < take) node = stk[sp - 1 - lane];
                __syncwarp();
                sp -= take;
                // children as (a, b) = (nearer, farther) along the packet's mean direction
                bool pa = false, pb = false;
                uint32_t ca = 0, cb = 0;
                if (node != GRAY_NULL) {
                    if (node & GRAY_LEAF_BIT) {
                        ca = node;  // a leaf of the tile's frontier: queued below
                        pa = true;
                    } else if (node >= (uint32_t)(n - 1)) {
                        raise_status(status, GRAY_STATUS_STACK_OVERFLOW);
                    } else {
                        const float4 q0 = sc.nodes[4 * node], q1 = sc.nodes[4 * node + 1],
                                     q2 = sc.nodes[4 * node + 2], q3 = sc.nodes[4 * node + 3];
                        const float b0min[3] = {q0.x, q0.y, q0.z}, b0max[3] = {q0.w, q1.x, q1.y};
                        const float b1min[3] = {q1.z, q1.w, q2.x}, b1max[3] = {q2.y, q2.z, q2.w};
                        const uint32_t c0 = __float_as_uint(q3.x), c1 = __float_as_uint(q3.y);
                        const bool p0 = frustum_box(fr, b0min, b0max), p1 = frustum_box(fr, b1min, b1max);
                        // box centres (times 2) projected on the mean direction; the origin is common
                        const float4 c = fr.pn[4];
                        const float s0 = fmaf(q0.z + q1.y, c.z, fmaf(q0.y + q1.x, c.y, (q0.x + q0.w) * c.x));
                        const float s1 = fmaf(q2.x + q2.w, c.z, fmaf(q1.w + q2.z, c.y, (q1.z + q2.y) * c.x));
                        const bool sw = s1 < s0;
                        ca = sw ? c1 : c0;
                        cb = sw ? c0 : c1;
                        pa = sw ? p1 : p0;
                        pb = sw ? p0 : p1;
                    }
                }
                const bool ia = pa && !(ca & GRAY_LEAF_BIT), ib = pb && !(cb & GRAY_LEAF_BIT);
                const bool la = pa && (ca & GRAY_LEAF_BIT) && (ca & ~GRAY_LEAF_BIT) < (uint32_t)n;
                const bool lb = pb && (cb & GRAY_LEAF_BIT) && (cb & ~GRAY_LEAF_BIT) < (uint32_t)n;
                // The popped nodes are in visit order (lane 0 took the top).  Their internal children
                // go back so that the next pops see lane 0's nearer child first, then its farther
                // one, then lane 1's, ...; the leaves are queued in the same order.
                const uint32_t ma = __ballot_sync(kFull, ia), mb = __ballot_sync(kFull, ib);
                const int ni = __popc(ma) + __popc(mb);
                if (sp + ni > kWideStack) {
                    ok = false;  // frontier too wide for the shared stack
                    break;
                }
                const int above = __popc(ma & lanemask_lt) + __popc(mb & lanemask_lt);
                if (ia) stk[sp + ni - 1 - above] = ca;
                if (ib) stk[sp + ni - 1 - above - (ia ? 1 : 0)] = cb;
                sp += ni;
                // queue the leaves found (nc < kCand before the step, at most 64 added)
                const uint32_t qa = __ballot_sync(kFull, la), qb = __ballot_sync(kFull, lb);
                const int before = nc + __popc(qa & lanemask_lt) + __popc(qb & lanemask_lt);
                if (la) cand[before] = ca & ~GRAY_LEAF_BIT;
                if (lb) cand[before + (la ? 1 : 0)] = cb & ~GRAY_LEAF_BIT;
                nc += __popc(qa) + __popc(qb);
                __syncwarp();
            }
        }
        // keep the queue below kCand before the next step (a step adds at most 64 < kQueue - kCand)
        while (nc >= kCand || (draining && nc > 0)) {
            // process the first kCand queued leaves, then move the rest to the front
            const int take = nc < kCand ? nc : kCand;
            flush_candidates<KB>(sc, k, ro, rd, want, first, st, kbuf, fr, cand, cc, take);
            const int rest = nc - take;
            const uint32_t r0 = lane < rest ? cand[kCand + lane] : 0u;
            const uint32_t r1 = lane + 32 < rest ? cand[kCand + 32 + lane] : 0u;
            __syncwarp();
            if (lane < rest) cand[lane] = r0;
            if (lane + 32 < rest) cand[32 + lane] = r1;
            __syncwarp();
            nc = rest;
        }
        if (draining) break;
    }
    __syncwarp();
    return ok;
}

// Trace the warp's 32 rays (one per lane; `alive` lanes only) through the scene: traversal,
// selection, compositing (cuda/forward_pass.cu:6-151 minus the write-out).  Every lane of the
// warp must call this together.
template <int KB>
__device__ __forceinline__ void trace_ray(const TraceScene &sc, const TraceKnobs &k, f3 ro, f3 rd, bool alive,
                                          bool grads, const HitSink &hs, int32_t *status,
                                          unsigned long long (*kbuf)[kFwdThreads], RayResult &res,
                                          const Frustum *fr = nullptr, uint32_t *wstk = nullptr,
                                          uint32_t *wcand = nullptr, CandCache *wcc = nullptr,
                                          const uint32_t *front_base = nullptr, uint32_t front_off = 0) {
    const int lane = threadIdx.x & 31;
    LaneState &st = res.st;
    st.lfx = 0;
    st.afx = st.cfx0 = st.cfx1 = st.cfx2 = 0;
    st.nhit = 0;
    st.kcount = 0;
    st.ncand = 0;
    st.kmax = 0;
    st.resume = 0;
    st.has_resume = false;
    float T = 1.0f, C0 = 0.0f, C1 = 0.0f, C2 = 0.0f, depth = 0.0f;
    int pass = 0, slots = 0, nacc = 0;
    float tmin_sel = k.znear, last_d = k.znear;
    bool done = !alive;
    uint32_t head = GRAY_NULL;

    bool first = true;
    int traversals = 0;
    // the packet needs a second traversal with a 16-slot buffer: some lane of a 32-slot kernel goes
    // on past the 16 nearest keys of its first traversal (the same 16 the narrow kernel holds)
    bool deep = false;
    const int n = sc.n;
    while (__any_sync(kFull, !done)) {
        const bool want = !done;
        st.kcount = 0;
        st.ncand = 0;
        // ---------------- traversal ----------------
        bool per_ray = fr == nullptr;
        if (!per_ray &&
            !traverse_frustum<KB>(sc, k, ro, rd, want, first, st, kbuf, *fr, wstk, wcand, *wcc, front_base, front_off,
                                      status)) {
            // the frustum traversal gave up (stack overflow): discard what it gathered, trace per ray
            st.kcount = 0;
            st.ncand = 0;
            if (first) {
                st.lfx = 0;
                st.afx = st.cfx0 = st.cfx1 = st.cfx2 = 0;
                st.nhit = 0;
            }
            per_ray = true;
        }
        if (!per_ray) {
        } else if (n == 1) {
            // (the per-ray path's ray data is built here, so it holds no registers in the frustum path)
            const SlabRay sr = make_slab_ray(ro, rd, 2.0e-6f * (fabsf(ro.x) + fabsf(ro.y) + fabsf(ro.z)));
            const float *rb = sc.root_box;
            const float bmin[3] = {rb[0], rb[1], rb[2]}, bmax[3] = {rb[4], rb[5], rb[6]};
            bool h = want && slab_hit(bmin, bmax, sr);
            if (__any_sync(kFull, h)) on_leaf<KB>(sc, 0u, h, first, ro, rd, k, st, kbuf);
        } else if (n > 1) {
            const SlabRay sr = make_slab_ray(ro, rd, 2.0e-6f * (fabsf(ro.x) + fabsf(ro.y) + fabsf(ro.z)));
            // packet lead direction for the near/far child order (any deterministic choice is valid)
            float lx = alive ? rd.x : 0.0f, ly = alive ? rd.y : 0.0f, lz = alive ? rd.z : 0.0f;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                lx += __shfl_xor_sync(kFull, lx, off);
                ly += __shfl_xor_sync(kFull, ly, off);
                lz += __shfl_xor_sync(kFull, lz, off);
            }
            uint32_t stk0 = 0, stk1 = 0;  // entry e lives in lane e%32, word e/32
            int sp = 0;
            {
                const float *rb = sc.root_box;
                const float bmin[3] = {rb[0], rb[1], rb[2]}, bmax[3] = {rb[4], rb[5], rb[6]};
                bool h = want && slab_hit(bmin, bmax, sr);
                if (__any_sync(kFull, h)) {
                    if (lane == 0) stk0 = 0u;
                    sp = 1;
                }
            }
            long long budget = 2LL * n;  // pops of a valid tree per traversal are < n
            while (sp > 0) {
                if (--budget < 0) {
                    raise_status(status, GRAY_STATUS_STACK_OVERFLOW);
                    break;
                }
                sp--;
                const uint32_t word = (sp >> 5) == 0 ? stk0 : stk1;
                const uint32_t node = __shfl_sync(kFull, word, sp & 31);
                if (node >= (uint32_t)(n - 1)) {
                    raise_status(status, GRAY_STATUS_STACK_OVERFLOW);
                    continue;
                }
                const float4 q0 = sc.nodes[4 * node], q1 = sc.nodes[4 * node + 1], q2 = sc.nodes[4 * node + 2],
                             q3 = sc.nodes[4 * node + 3];
                const float b0min[3] = {q0.x, q0.y, q0.z}, b0max[3] = {q0.w, q1.x, q1.y};
                const float b1min[3] = {q1.z, q1.w, q2.x}, b1max[3] = {q2.y, q2.z, q2.w};
                const uint32_t c0 = __float_as_uint(q3.x), c1 = __float_as_uint(q3.y);
                const bool h0 = want && slab_hit(b0min, b0max, sr);
                const bool h1 = want && slab_hit(b1min, b1max, sr);
                const bool any0 = __any_sync(kFull, h0), any1 = __any_sync(kFull, h1);
                if (!any0 && !any1) continue;
                // near child first along the packet's lead direction
                const float p0 = (b0min[0] + b0max[0]) * lx + (b0min[1] + b0max[1]) * ly + (b0min[2] + b0max[2]) * lz;
                const float p1 = (b1min[0] + b1max[0]) * lx + (b1min[1] + b1max[1]) * ly + (b1min[2] + b1max[2]) * lz;
                const bool swap = p1 < p0;
                const uint32_t cn = swap ? c1 : c0, cf = swap ? c0 : c1;
                const bool an = swap ? any1 : any0, af = swap ? any0 : any1;
                const bool hn = swap ? h1 : h0, hf = swap ? h0 : h1;
                // far internal child goes deeper in the stack, near internal child on top;
                // leaves are processed right away, near first
                if (af && !(cf & GRAY_LEAF_BIT)) stack_push(stk0, stk1, sp, cf, lane, status);
                if (an && (cn & GRAY_LEAF_BIT)) {
                    const uint32_t gid = cn & ~GRAY_LEAF_BIT;
                    if (gid < (uint32_t)n) on_leaf<KB>(sc, gid, hn, first, ro, rd, k, st, kbuf);
                }
                if (af && (cf & GRAY_LEAF_BIT)) {
                    const uint32_t gid = cf & ~GRAY_LEAF_BIT;
                    if (gid < (uint32_t)n) on_leaf<KB>(sc, gid, hf, first, ro, rd, k, st, kbuf);
                }
                if (an && !(cn & GRAY_LEAF_BIT)) stack_push(stk0, stk1, sp, cn, lane, status);
            }
        }
        // ---------------- consume (cuda/forward_pass.cu:46-125) ----------------
        int nc = 0;
        if (want) {
            const int t = threadIdx.x;
            const unsigned long long last_key = st.kcount > 0 ? kbuf[st.kcount - 1][t] : 0ull;
            for (int i = 0; i < st.kcount; i++) {
                if constexpr (KB > 16) {
                    if (i == 16 && first) deep = true;
                }
                const unsigned long long key = kbuf[i][t];
                const float d = h2f_bits((uint16_t)(key >> 48));
                if (!(d > tmin_sel)) continue;
                if (slots == kPassSlots) {
                    pass++;
                    if (pass >= kMaxPasses) {
                        done = true;
                        break;
                    }
                    tmin_sel = last_d;
                    if (!(tmin_sel < k.zfar)) {
                        done = true;
                        break;
                    }
                    slots = 0;
                    if (!(d > tmin_sel)) continue;
                }
                slots++;
                last_d = d;
                if (!(d < k.zfar)) {
                    done = true;
                    break;
                }
                const uint32_t gid = (uint32_t)(key >> 16);
                const float al = h2f_bits((uint16_t)(key & 0xFFFFu));
                const float *c = sc.channels + 3 * (size_t)gid;
                const float cx = c[0], cy = c[1], cz = c[2];
                const long long a = alpha16_fixed((uint16_t)(key & 0xFFFFu));
                st.afx -= a;
                st.cfx0 -= mul_fixed(a, colour_fixed(cx));
                st.cfx1 -= mul_fixed(a, colour_fixed(cy));
                st.cfx2 -= mul_fixed(a, colour_fixed(cz));
                const float w = T * al;
                C0 = C0 + cx * w;
                C1 = C1 + cy * w;
                C2 = C2 + cz * w;
                if (k.render_depth) depth = depth + d * w;
                T = T * (1.0f - al);
                kbuf[nc][t] = gid;
                nc++;
                nacc++;
                if (T < k.tthr) {
                    done = true;
                    break;
                }
            }
            if (!done) {
                if (st.ncand > st.kcount) {
                    // resume after the last key looked at; entries at or below the active pass
                    // threshold would be dropped anyway, so skip them at the traversal
                    unsigned long long r = last_key;
                    const bool exact = pass > 0 || slots == kPassSlots;
                    if (exact) {
                        const float thr = slots == kPassSlots ? fmaxf(last_d, tmin_sel) : tmin_sel;
                        const unsigned long long skip = ((unsigned long long)f2h_bits(thr) << 48) | 0xFFFFFFFFFFFFull;
                        r = skip > r ? skip : r;
                    }
                    st.resume = r;
                    st.has_resume = true;
                    if (++traversals > kMaxTraversals) {
                        raise_status(status, GRAY_STATUS_STACK_OVERFLOW);
                        done = true;
                    }
                } else {
                    done = true;
                }
            }
        }
        // ---------------- backward hit list segment (warp aggregated) ----------------
        if (grads) {
            const uint32_t need = nc > 0 ? (uint32_t)nc + 2u : 0u;
            uint32_t incl = need;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                uint32_t v = __shfl_up_sync(kFull, incl, off);
                if (lane >= off) incl += v;
            }
            const uint32_t total = __shfl_sync(kFull, incl, 31);
            uint32_t base = 0;
            if (total > 0) {
                if (lane == 31) base = atomicAdd(hs.counter, total);
                base = __shfl_sync(kFull, base, 31);
            }
            if (need > 0) {
                const uint32_t off = base + incl - need;
                const bool fits = base <= hs.pool_size && total <= hs.pool_size - base;
                if (fits) {
                    hs.pool[off] = head;
                    hs.pool[off + 1] = (uint32_t)nc;
                    for (int j = 0; j < nc; j++) hs.pool[off + 2 + j] = (uint32_t)kbuf[j][threadIdx.x];
                    head = off;
                } else {
                    raise_status(status, GRAY_STATUS_HITLIST_OVERFLOW);
                }
            }
        }
        first = false;
    }
    res.T = T;
    res.C0 = C0;
    res.C1 = C1;
    res.C2 = C2;
    st.ft = full_transmittance(st.lfx);
    res.depth = depth;
    res.nacc = nacc;
    res.head = head;
    res.retraced = __any_sync(kFull, traversals > 0 || deep);
}

// Truncated-tail estimate and background (cuda/forward_pass.cu:131-142).
__device__ __forceinline__ void finish_ray(RayResult &r, const float *bg, float eps_fwd, bool render_depth,
                                           float &r0, float &r1, float &r2) {
    const LaneState &st = r.st;
    const float rT = r.T - st.ft;
    r0 = r1 = r2 = 0.0f;
    if (st.afx > 0) {
        const float sa = __ll2float_rn(st.afx) * 0x1.0p-24f;
        r0 = (__ll2float_rn(st.cfx0) * 0x1.0p-48f) / sa;
        r1 = (__ll2float_rn(st.cfx1) * 0x1.0p-48f) / sa;
        r2 = (__ll2float_rn(st.cfx2) * 0x1.0p-48f) / sa;
    }
    r.C0 = r.C0 + rT * r0;
    r.C1 = r.C1 + rT * r1;
    r.C2 = r.C2 + rT * r2;
    if (render_depth) r.depth = r.depth / fmaxf(1.0f - r.T, eps_fwd);
    r.C0 = r.C0 + bg[0] * st.ft;
    r.C1 = r.C1 + bg[1] * st.ft;
    r.C2 = r.C2 + bg[2] * st.ft;
}

// Primary ray of pixel (px, py) of a width x height pinhole camera (cuda/core/camera.h:17-36).
__device__ __forceinline__ f3 camera_ray(const float *w, float fov, int px, int py, uint32_t width, uint32_t height,
                                         float jx, float jy) {
    const float view_size = tanf(fov / 2.0f);
    const float aspect = (float)width / (float)height;
    const float fx = (float)px + jx, fy = (float)py + jy;
    const float y = view_size * (1.0f - 2.0f * (fy + 0.5f) / (float)height);
    const float x = aspect * view_size * (2.0f * (fx + 0.5f) / (float)width - 1.0f);
    f3 v = mk3(w[0] * x + w[3] * y - w[6], w[1] * x + w[4] * y - w[7], w[2] * x + w[5] * y - w[8]);
    const float inv = 1.0f / sqrtf(dot3(v, v));
    return mk3(v.x * inv, v.y * inv, v.z * inv);
}

__device__ __forceinline__ float3 camera_ray3(const float *w, float fov, int px, int py, uint32_t width,
                                              uint32_t height) {
    const f3 r = camera_ray(w, fov, px, py, width, height, 0.0f, 0.0f);
    return make_float3(r.x, r.y, r.z);
}

// Shared memory of a forward block.
template <int KB>
struct FwdShared {
    unsigned long long kbuf[KB][kFwdThreads];
    Frustum sfr[kWarps];
    uint32_t sstk[kWarps][kWideStack];
    uint32_t scand[kWarps][kQueue];
    CandCache scc[kWarps];
    uint32_t front[kFrontierWords];  // the tile's BVH frontier (count, entries)
};

// Packet (wx, wy) of pixel tile (bx, by) (a tile is 2x2 packets of tile_w x tile_h pixels), traced
// by the calling warp; front_base + front_off: the tile's BVH frontier (count, entries), or a null base.
template <int KB>
__device__ __forceinline__ bool forward_packet(const FwdArgs &a, int bx, int by, int wx, int wy,
                                               const uint32_t *front_base, uint32_t front_off, FwdShared<KB> &sh) {
    unsigned long long(*kbuf)[kFwdThreads] = sh.kbuf;
    Frustum *sfr = sh.sfr;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int px = bx * (a.tile_w * kBlockWarpsX) + wx * a.tile_w + (lane % a.tile_w);
    const int py = by * (a.tile_h * kBlockWarpsY) + wy * a.tile_h + (lane / a.tile_w);
    const bool inside = px < (int)a.render_w && py < (int)a.render_h;
    const uint32_t pixel = (uint32_t)py * a.alloc_w + (uint32_t)px;

    TraceKnobs k;
    k.znear = *a.znear;
    k.zfar = *a.zfar;
    k.athr = *a.alpha_threshold;
    k.pw = *a.exp_power;
    k.tthr = *a.t_threshold;
    k.render_depth = *a.render_depth != 0;
    const bool grads = !a.display && *a.grads_enabled != 0;
    const TraceScene sc{a.geom, a.l2w, a.live, a.channels, a.nodes, a.root_box, a.n};
    const HitSink hs{a.counter, a.pool, a.pool_size};

    // ---- ray generation (cuda/shaders.cu:76-88) ----
    f3 ro = mk3(0.0f, 0.0f, 0.0f), rd = mk3(0.0f, 0.0f, 0.0f);
    bool alive = false;
    // every lane holds the camera origin, inactive ones too (a packet's candidates get their
    // object-space origin from whichever lane fetches them)
    if (!*a.rays_from_python) ro = mk3(a.cam_origin[0], a.cam_origin[1], a.cam_origin[2]);
    if (inside) {
        if (*a.rays_from_python) {
            ro = mk3(a.ray_o[3 * pixel], a.ray_o[3 * pixel + 1], a.ray_o[3 * pixel + 2]);
            rd = mk3(a.ray_d[3 * pixel], a.ray_d[3 * pixel + 1], a.ray_d[3 * pixel + 2]);
        } else {
            ro = mk3(a.cam_origin[0], a.cam_origin[1], a.cam_origin[2]);
            float jx = 0.0f, jy = 0.0f;
            if (*a.jitter) {
                uint32_t h = pcg_hash(pixel ^ pcg_hash(*a.total_num_calls));
                jx = (float)(h & 0xFFFFu) * 0x1.0p-16f - 0.5f;
                jy = (float)(h >> 16) * 0x1.0p-16f - 0.5f;
            }
            rd = camera_ray(a.w2c, *a.fov, px, py, a.render_w, a.render_h, jx, jy);
        }
        alive = !(sqrtf(dot3(rd, rd)) == 0.0f);
    }

    // camera rays of the packet share the origin: trace with the frustum traversal
    const bool frustum = !*a.rays_from_python && !*a.jitter;
    if (frustum) {
        const int x0 = px - lane % a.tile_w, y0 = py - lane / a.tile_w;
        const int x1 = x0 + a.tile_w - 1, y1 = y0 + a.tile_h - 1;
        make_frustum_warp(sfr[warp], mk3(a.cam_origin[0], a.cam_origin[1], a.cam_origin[2]), a.w2c, *a.fov, x0, y0, x1,
                          y1, a.render_w, a.render_h, a.root_box);
    }
    RayResult r;
    trace_ray<KB>(sc, k, ro, rd, alive, grads, hs, a.status, kbuf, r, frustum ? &sfr[warp] : nullptr, sh.sstk[warp],
                  sh.scand[warp], &sh.scc[warp], frustum ? front_base : nullptr, front_off);

    if (!inside) return r.retraced;
    if (!alive) {
        a.head[pixel] = GRAY_NULL;  // inactive pixel: empty list, nothing else written
        return r.retraced;
    }
    float r0, r1, r2;
    finish_ray(r, a.bg, *a.eps_fwd, k.render_depth, r0, r1, r2);
    a.out_rgb[3 * pixel] = r.C0;
    a.out_rgb[3 * pixel + 1] = r.C1;
    a.out_rgb[3 * pixel + 2] = r.C2;
    if (grads) {
        a.out_depth[pixel] = r.depth;
        a.out_T[pixel] = r.T;
        a.out_fullT[pixel] = r.st.ft;
        a.out_rem[3 * pixel] = r0;
        a.out_rem[3 * pixel + 1] = r1;
        a.out_rem[3 * pixel + 2] = r2;
        a.ray_o[3 * pixel] = ro.x;
        a.ray_o[3 * pixel + 1] = ro.y;
        a.ray_o[3 * pixel + 2] = ro.z;
        a.ray_d[3 * pixel] = rd.x;
        a.ray_d[3 * pixel + 1] = rd.y;
        a.ray_d[3 * pixel + 2] = rd.z;
        a.stat_hit[pixel] += r.st.nhit;
        a.stat_acc[pixel] += r.nacc;
        a.head[pixel] = r.head;
    } else {
        const bool nro = *a.needs_ray_output != 0;
        if (k.render_depth || nro) a.out_depth[pixel] = r.depth;
        if (nro) {
            a.ray_d[3 * pixel] = rd.x;
            a.ray_d[3 * pixel + 1] = rd.y;
            a.ray_d[3 * pixel + 2] = rd.z;
        }
        a.head[pixel] = GRAY_NULL;
    }
    return r.retraced;
}

// One block's pixel tile (bx, by): its four packets, one per warp; the tile's frontier is copied
// into shared memory once by the block.  Returns whether the calling warp's packet needs more than
// one traversal with 16 hit slots (RayResult::retraced).
template <int KB>
__device__ __forceinline__ bool forward_tile(const FwdArgs &a, int bx, int by, FwdShared<KB> &sh) {
    const int warp = threadIdx.x >> 5;
    {   // every thread of the block gets here together
        const uint32_t *src = a.frontier ? a.frontier + (size_t)(by * a.tiles_x + bx) * kFrontierWords : nullptr;
        const uint32_t cnt = src ? src[0] : kFrontierNone;
        const bool use = cnt <= (uint32_t)kFrontierMax;
        if (use)
            for (uint32_t i = threadIdx.x; i < cnt; i += kFwdThreads) sh.front[1 + i] = src[1 + i];
        if (threadIdx.x == 0) sh.front[0] = use ? cnt : kFrontierNone;
        __syncthreads();
    }
    return forward_packet<KB>(a, bx, by, warp % kBlockWarpsX, warp / kBlockWarpsX, sh.front, 0u, sh);
}

// Grid launch: block (x, y) renders tile (x, y).
template <int KB, int MINB>
__global__ void __launch_bounds__(kFwdThreads, MINB) trace_forward_kernel(const FwdArgs a) {
    __shared__ FwdShared<KB> sh;
    if (*a.render_ellipsoids) return;  // the ellipsoid view (ellipsoid_kernel) renders this frame
    forward_tile<KB>(a, blockIdx.x, blockIdx.y, sh);
}

// Persistent launch: the blocks take tiles from the schedule's order, densest first, until none is
// left (a separate kernel, so the grid launch keeps its register allocation).
// The packets it traced, and those that traverse more than once with a 16-slot buffer (whatever KB
// is), are added to the schedule's statistics words (the automatic kernel choice of the next forward
// reads them).
template <int KB, int MINB>
__global__ void __launch_bounds__(kFwdThreads, MINB) trace_forward_sched_kernel(const FwdArgs a) {
    __shared__ FwdShared<KB> sh;
    __shared__ uint32_t s_next, s_packets, s_retraced;
    if (*a.render_ellipsoids) return;
    // automatic choice: both kernels are launched, the one the scan kernel did not choose leaves
    if (a.auto_role != 0 && a.schedule[kStatChoice] != (uint32_t)a.auto_role) return;
    if (threadIdx.x == 0) {
        s_packets = 0u;
        s_retraced = 0u;
    }
    for (;;) {
        __syncthreads();  // every thread is done with the previous tile (s_next, the frontier, counts)
        if (threadIdx.x == 0) s_next = atomicAdd(a.schedule, 1u);
        __syncthreads();
        const uint32_t t = s_next;
        if (t >= (uint32_t)a.ntiles) break;
        const uint32_t tile = a.schedule[kSchedHeader + a.ntiles + t];
        const bool again =
            forward_tile<KB>(a, (int)(tile % (uint32_t)a.tiles_x), (int)(tile / (uint32_t)a.tiles_x), sh);
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&s_packets, 1u);
            if (again) atomicAdd(&s_retraced, 1u);
        }
    }
    if (threadIdx.x == 0 && s_packets > 0u) {
        atomicAdd(&a.schedule[kStatPackets], s_packets);
        atomicAdd(&a.schedule[kStatRetraced], s_retraced);
    }
}

// Persistent launch with packets taken per warp: every warp claims the next packet (a quarter of a
// pixel tile, tiles in the schedule's densest-first order) from the global counter on its own, so no
// warp waits at a block barrier for a tile's slowest packet; a tile's four packets usually land on
// different SMs, though, so they no longer share an L1.  Packets read their tile's frontier from
// the schedule buffer (L2).
template <int KB, int MINB>
__global__ void __launch_bounds__(kFwdThreads, MINB) trace_forward_claim_kernel(const FwdArgs a) {
    __shared__ FwdShared<KB> sh;
    if (*a.render_ellipsoids) return;
    for (;;) {
        uint32_t q = 0u;
        if ((threadIdx.x & 31) == 0) q = atomicAdd(a.schedule, 1u);
        q = __shfl_sync(kFull, q, 0);
        if (q >= (uint32_t)kWarps * (uint32_t)a.ntiles) break;
        const uint32_t tile = a.schedule[kSchedHeader + a.ntiles + q / kWarps], sub = q % kWarps;
        forward_packet<KB>(a, (int)(tile % (uint32_t)a.tiles_x), (int)(tile / (uint32_t)a.tiles_x),
                                       (int)(sub % kBlockWarpsX), (int)(sub / kBlockWarpsX), a.frontier,
                                       tile * (uint32_t)kFrontierWords, sh);
    }
}

// ---------------------------------------------------------------------------------------------
// Work order of the forward's tiles and their BVH frontiers.  A tile's work follows the number of
// Gaussians its rays meet (per-packet time correlates 0.92 with hits), so the estimate is the number
// of leaves under the BVH nodes its frustum reaches, cut where a node holds at most `cut` leaves.
// Tiles are then counting-sorted by log2 of the estimate, largest first, so the launch does not end
// with a dense tile started late.  The nodes at the cut (and leaves reached above it) are the tile's
// frontier: every ray of the tile that hits a Gaussian reaches it through one of them, so the tile's
// packets start their traversals there instead of at the root (the top levels are walked once per
// tile, not once per packet traversal).  The frontier is sorted by its boxes' centres along the
// tile's mean direction, so packets visit it roughly front to back.  The tiles' walks share their
// top: a first pass walks each super-tile (kSuperTiles x kSuperTiles tiles) down to nodes of at
// most kSuperCut leaves and stores them with their boxes; a tile's walk then starts from its
// super-tile's entries, testing each entry's own box against the tile's frustum, instead of from the
// root.  Every leaf a ray of the tile can hit lies under an entry of the super-tile (its ancestors
// meet the tile's frustum, hence the super-tile's), so the tile still reaches it.  Schedule words:
// [0] work counter, [1..33] bucket counts/cursors, [kSchedHeader, +ntiles) estimates, [kSchedHeader +
// ntiles, +ntiles) order, then (when frontiers are on) kFrontierWords words per tile, then
// kSuperWords words per super-tile.
// ---------------------------------------------------------------------------------------------
constexpr int kCostCut = 512;
constexpr int kCostStack = 256;
constexpr int kSuperTiles = 4;
constexpr uint32_t kSuperCut = 1024;
constexpr int kSuperMax = 255;          // entries of a super-tile frontier (fits the walk's buffer)
constexpr int kSuperEntryWords = 8;     // link, leaves below, box min xyz, box max xyz
constexpr int kSuperWords = 1 + kSuperMax * kSuperEntryWords;

struct FrontierScratch {
    Frustum fr;
    uint32_t stk[kCostStack];
    float key[kFrontierSort];
    uint32_t val[kFrontierSort];
};

// What the super-tile walk also keeps of each frontier entry.
struct SuperScratch {
    float box[kFrontierSort][6];
    uint32_t leaves[kFrontierSort];
};

// Bitonic sort of the warp's nf (key, link) frontier entries (fs.key / fs.val, nf <= 32 * E) by key,
// written to out[1 .. nf].  The network runs in registers: element i sits in lane i % 32, slot i / 32;
// the partner at distance j < 32 is the same slot of lane ^ j (a shuffle), at j >= 32 the slot
// e ^ (j / 32) of the same lane.  Padding keys are +inf (sorted last); each pair (lower, upper)
// swaps iff (ascending ? k_upper < k_lower : k_lower < k_upper), so NaN keys never move and ties
// keep their places.
template <int E>
__device__ __forceinline__ void frontier_sort_out(const FrontierScratch &fs, int nf, uint32_t *out) {
    const int lane = threadIdx.x & 31;
    float k[E];
    uint32_t v[E];
#pragma unroll
    for (int e = 0; e < E; e++) {
        const int i = e * 32 + lane;
        k[e] = i < nf ? fs.key[i] : __int_as_float(0x7f800000);
        v[e] = i < nf ? fs.val[i] : GRAY_NULL;
    }
#pragma unroll
    for (int kk = 2; kk <= 32 * E; kk <<= 1) {
#pragma unroll
        for (int j = kk >> 1; j > 0; j >>= 1) {
            if (j >= 32) {
#pragma unroll
                for (int e = 0; e < E; e++) {
                    const int f = e ^ (j >> 5);
                    if (f > e) {
                        const bool up = ((e * 32 + lane) & kk) == 0;
                        const float kl = k[e], ku = k[f];
                        if (up ? (ku < kl) : (kl < ku)) {
                            k[e] = ku;
                            k[f] = kl;
                            const uint32_t t = v[e];
                            v[e] = v[f];
                            v[f] = t;
                        }
                    }
                }
            } else {
#pragma unroll
                for (int e = 0; e < E; e++) {
                    const float ko = __shfl_xor_sync(kFull, k[e], j);
                    const uint32_t vo = __shfl_xor_sync(kFull, v[e], j);
                    const bool up = ((e * 32 + lane) & kk) == 0;
                    const bool lower = (lane & j) == 0;
                    const float kl = lower ? k[e] : ko, ku = lower ? ko : k[e];
                    if (up ? (ku < kl) : (kl < ku)) {
                        k[e] = ko;
                        v[e] = vo;
                    }
                }
            }
        }
    }
#pragma unroll
    for (int e = 0; e < E; e++) {
        const int i = e * 32 + lane;
        if (i < nf) out[1 + i] = v[e];
    }
}

// One warp walks the top of the BVH for a pixel rectangle whose frustum is in fs.fr: returns (on
// every lane) the number of leaves under the frontier, the nodes of at most `cut` leaves (and the
// leaves) it reaches; with `out`, writes the frontier there sorted front to back (count + entries),
// or a count of kFrontierNone when the walk was cut short, the frontier does not fit or the tree is
// malformed.  n > 1.  seed (may be null; a count above kSuperMax means none): a super-tile frontier
// to start from instead of the root -- each entry whose box meets this frustum is walked further
// (more than `cut` leaves) or is a frontier entry.  SUPER: the walk of a super-tile; with `out` it
// writes its entries unsorted with their leaf counts and boxes (kSuperWords words), or
// kFrontierNone when they do not fit.
template <bool SUPER>
__device__ __forceinline__ uint32_t frontier_walk(const float4 *nodes, int n, uint32_t cut, FrontierScratch &fs,
                                               SuperScratch *ss, uint32_t *out, const uint32_t *seed) {
    const int lane = threadIdx.x & 31;
    const uint32_t lanemask_lt = (1u << lane) - 1u;
    const Frustum &fr = fs.fr;
    const float4 cdir = fr.pn[4];  // the near plane's normal: the rectangle's mean direction
    uint32_t est = 0;
    int nf = 0, sp = 0;
    bool complete = true, stop = false;
    const uint32_t nseed = seed ? seed[0] : kFrontierNone;
    if (nseed <= (uint32_t)kSuperMax) {
        for (int b0 = 0; b0 < (int)nseed; b0 += 32) {
            const int i = b0 + lane;
            bool push = false, rec = false, bad = false;
            uint32_t link = 0;
            float key = 0.0f;
            if (i < (int)nseed) {
                const uint32_t *e = seed + 1 + (size_t)i * kSuperEntryWords;
                link = e[0];
                const uint32_t lv = e[1];
                const float bmin[3] = {__uint_as_float(e[2]), __uint_as_float(e[3]), __uint_as_float(e[4])};
                const float bmax[3] = {__uint_as_float(e[5]), __uint_as_float(e[6]), __uint_as_float(e[7])};
                if (frustum_box(fr, bmin, bmax)) {
                    if (link & GRAY_LEAF_BIT) {
                        rec = (link & ~GRAY_LEAF_BIT) < (uint32_t)n;
                        bad = !rec;
                        est += rec ? 1u : 0u;
                    } else if (link < (uint32_t)(n - 1)) {
                        push = lv > cut;
                        rec = !push;
                        if (rec) est += lv;
                    } else {
                        bad = true;
                    }
                    key = fmaf(bmin[2] + bmax[2], cdir.z, fmaf(bmin[1] + bmax[1], cdir.y, (bmin[0] + bmax[0]) * cdir.x));
                }
            }
            if (__any_sync(kFull, bad)) complete = false;
            const uint32_t mp = __ballot_sync(kFull, push);
            if (sp + __popc(mp) > kCostStack) {
                complete = false;  // an estimate from what was reached is enough
                stop = true;
                break;
            }
            if (push) fs.stk[sp + __popc(mp & lanemask_lt)] = link;
            sp += __popc(mp);
            const uint32_t mr = __ballot_sync(kFull, rec);
            const int at = nf + __popc(mr & lanemask_lt);
            if (rec && at < kFrontierSort) {
                fs.key[at] = key;
                fs.val[at] = link;
            }
            nf += __popc(mr);
        }
    } else {
        if (lane == 0) fs.stk[0] = 0u;
        sp = 1;
    }
    __syncwarp();
    for (int guard = 0; sp > 0 && !stop; guard++) {
        if (guard >= 4096) {
            complete = false;
            break;
        }
        const int take = sp < 32 ? sp : 32;
        uint32_t node = GRAY_NULL;
        if (lane < take) node = fs.stk[sp - 1 - lane];
        __syncwarp();
        sp -= take;
        // children as (a, b) = (nearer, farther) along the rectangle's mean direction, as the forward
        uint32_t ca = 0, cb = 0, la = 0, lb = 0;  // children and the leaves below them
        bool pa = false, pb = false, bad = false;
        float sa = 0.0f, sb = 0.0f;
        float boxa[6], boxb[6];
        if (node != GRAY_NULL) {
            if (node >= (uint32_t)(n - 1)) {
                bad = true;
            } else {
                const float4 q0 = nodes[4 * node], q1 = nodes[4 * node + 1], q2 = nodes[4 * node + 2],
                             q3 = nodes[4 * node + 3];
                const float b0min[3] = {q0.x, q0.y, q0.z}, b0max[3] = {q0.w, q1.x, q1.y};
                const float b1min[3] = {q1.z, q1.w, q2.x}, b1max[3] = {q2.y, q2.z, q2.w};
                const uint32_t c0 = __float_as_uint(q3.x), c1 = __float_as_uint(q3.y);
                const uint32_t l0 = __float_as_uint(q3.w), l1 = __float_as_uint(q3.z) - l0;
                const bool p0 = frustum_box(fr, b0min, b0max), p1 = frustum_box(fr, b1min, b1max);
                const float s0 = fmaf(q0.z + q1.y, cdir.z, fmaf(q0.y + q1.x, cdir.y, (q0.x + q0.w) * cdir.x));
                const float s1 = fmaf(q2.x + q2.w, cdir.z, fmaf(q1.w + q2.z, cdir.y, (q1.z + q2.y) * cdir.x));
                const bool sw = s1 < s0;
                ca = sw ? c1 : c0;
                cb = sw ? c0 : c1;
                pa = sw ? p1 : p0;
                pb = sw ? p0 : p1;
                sa = sw ? s1 : s0;
                sb = sw ? s0 : s1;
                la = sw ? l1 : l0;
                lb = sw ? l0 : l1;
                if constexpr (SUPER) {
                    const float c0b[6] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y};
                    const float c1b[6] = {q1.z, q1.w, q2.x, q2.y, q2.z, q2.w};
#pragma unroll
                    for (int k = 0; k < 6; k++) {
                        boxa[k] = sw ? c1b[k] : c0b[k];
                        boxb[k] = sw ? c0b[k] : c1b[k];
                    }
                }
            }
        }
        // internal children above the cut are walked further; leaves and nodes at the cut are
        // frontier entries
        bool ia = false, ib = false, fa = false, fb = false;
        if (pa) {
            if (ca & GRAY_LEAF_BIT) {
                fa = (ca & ~GRAY_LEAF_BIT) < (uint32_t)n;
                bad = bad || !fa;
                est += fa ? 1u : 0u;
            } else if (ca < (uint32_t)(n - 1)) {
                ia = la > cut;
                fa = !ia;
                if (fa) est += la;
            } else {
                bad = true;
            }
        }
        if (pb) {
            if (cb & GRAY_LEAF_BIT) {
                fb = (cb & ~GRAY_LEAF_BIT) < (uint32_t)n;
                bad = bad || !fb;
                est += fb ? 1u : 0u;
            } else if (cb < (uint32_t)(n - 1)) {
                ib = lb > cut;
                fb = !ib;
                if (fb) est += lb;
            } else {
                bad = true;
            }
        }
        // a malformed tree: leave it to the forward's own checks (root start)
        if (__any_sync(kFull, bad)) complete = false;
        const uint32_t ma = __ballot_sync(kFull, ia), mb = __ballot_sync(kFull, ib);
        const int ni = __popc(ma) + __popc(mb);
        if (sp + ni > kCostStack) {
            complete = false;  // an estimate from what was reached is enough
            break;
        }
        const int above = __popc(ma & lanemask_lt) + __popc(mb & lanemask_lt);
        if (ia) fs.stk[sp + ni - 1 - above] = ca;
        if (ib) fs.stk[sp + ni - 1 - above - (ia ? 1 : 0)] = cb;
        sp += ni;
        const uint32_t qa = __ballot_sync(kFull, fa), qb = __ballot_sync(kFull, fb);
        const int before = nf + __popc(qa & lanemask_lt) + __popc(qb & lanemask_lt);
        if (fa && before < kFrontierSort) {
            fs.key[before] = sa;
            fs.val[before] = ca;
            if constexpr (SUPER) {
                ss->leaves[before] = (ca & GRAY_LEAF_BIT) ? 1u : la;
#pragma unroll
                for (int k = 0; k < 6; k++) ss->box[before][k] = boxa[k];
            }
        }
        const int bb = before + (fa ? 1 : 0);
        if (fb && bb < kFrontierSort) {
            fs.key[bb] = sb;
            fs.val[bb] = cb;
            if constexpr (SUPER) {
                ss->leaves[bb] = (cb & GRAY_LEAF_BIT) ? 1u : lb;
#pragma unroll
                for (int k = 0; k < 6; k++) ss->box[bb][k] = boxb[k];
            }
        }
        nf += __popc(qa) + __popc(qb);
        __syncwarp();
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) est += __shfl_xor_sync(kFull, est, off);
    if (!out) return est;
    if constexpr (SUPER) {
        if (complete && nf <= kSuperMax) {
            for (int i = lane; i < nf; i += 32) {
                uint32_t *e = out + 1 + (size_t)i * kSuperEntryWords;
                e[0] = fs.val[i];
                e[1] = ss->leaves[i];
#pragma unroll
                for (int k = 0; k < 6; k++) e[2 + k] = __float_as_uint(ss->box[i][k]);
            }
            if (lane == 0) out[0] = (uint32_t)nf;
        } else if (lane == 0) {
            out[0] = kFrontierNone;
        }
        return est;
    }
    if (complete && nf <= kFrontierMax) {
        if (nf <= 32) frontier_sort_out<1>(fs, nf, out);
        else if (nf <= 64) frontier_sort_out<2>(fs, nf, out);
        else if (nf <= 128) frontier_sort_out<4>(fs, nf, out);
        else frontier_sort_out<8>(fs, nf, out);
        if (lane == 0) out[0] = (uint32_t)nf;
    } else if (lane == 0) {
        out[0] = kFrontierNone;
    }
    return est;
}

// Coarse frontiers of the super-tiles (kSuperTiles x kSuperTiles block tiles each), one warp each.
__global__ void __launch_bounds__(32) super_cost_kernel(const FwdArgs a, int bw, int bh, int nsuper) {
    __shared__ FrontierScratch fs;
    __shared__ SuperScratch ss;
    const int st = blockIdx.x, lane = threadIdx.x;
    if (st >= nsuper) return;
    uint32_t *out = a.super_frontier + (size_t)st * kSuperWords;
    const int n = a.n;
    if (!*a.rays_from_python && !*a.jitter && !*a.render_ellipsoids && n > 1) {
        const int x0 = (st % a.super_x) * kSuperTiles * bw, y0 = (st / a.super_x) * kSuperTiles * bh;
        const int x1 = min(x0 + kSuperTiles * bw, (int)a.render_w) - 1;
        const int y1 = min(y0 + kSuperTiles * bh, (int)a.render_h) - 1;
        make_frustum_warp(fs.fr, mk3(a.cam_origin[0], a.cam_origin[1], a.cam_origin[2]), a.w2c, *a.fov, x0, y0, x1, y1,
                          a.render_w, a.render_h, a.root_box);
        frontier_walk<true>(a.nodes, n, kSuperCut, fs, &ss, out, nullptr);
    } else if (lane == 0) {
        out[0] = kFrontierNone;
    }
}

__global__ void __launch_bounds__(32) tile_cost_kernel(const FwdArgs a, int bw, int bh) {
    __shared__ FrontierScratch fs;
    const int tile = blockIdx.x, lane = threadIdx.x;
    uint32_t *out = a.frontier ? a.frontier + (size_t)tile * kFrontierWords : nullptr;
    uint32_t est = 0;
    const int n = a.n;
    if (!*a.rays_from_python && !*a.jitter && !*a.render_ellipsoids && n > 1) {
        const int x0 = (tile % a.tiles_x) * bw, y0 = (tile / a.tiles_x) * bh;
        const int x1 = min(x0 + bw, (int)a.render_w) - 1, y1 = min(y0 + bh, (int)a.render_h) - 1;
        make_frustum_warp(fs.fr, mk3(a.cam_origin[0], a.cam_origin[1], a.cam_origin[2]), a.w2c, *a.fov, x0, y0, x1, y1,
                          a.render_w, a.render_h, a.root_box);
        const uint32_t *seed = nullptr;
        if (a.super_frontier) {
            const int sx = (tile % a.tiles_x) / kSuperTiles, sy = (tile / a.tiles_x) / kSuperTiles;
            seed = a.super_frontier + (size_t)(sy * a.super_x + sx) * kSuperWords;
        }
        est = frontier_walk<false>(a.nodes, n, a.frontier_cut > 0 ? a.frontier_cut : (uint32_t)kCostCut, fs, nullptr,
                                   out, seed);
    } else if (out && lane == 0) {
        out[0] = kFrontierNone;
    }
    if (lane == 0) {
        a.schedule[kSchedHeader + tile] = est;
        const uint32_t key = est ? (uint32_t)__clz(est) : 32u;  // larger estimate -> smaller key
        atomicAdd(&a.schedule[1 + key], 1u);
    }
}

// Bucket offsets of the densest-first order; and the automatic kernel choice for this forward from
// the last scheduled forward's packet counts (the narrow kernel when there are none yet).
__global__ void sched_scan_kernel(uint32_t *sched) {
    if (threadIdx.x != 0) return;
    uint32_t acc = 0;
    for (int k = 0; k <= 32; k++) {
        const uint32_t c = sched[1 + k];
        sched[1 + k] = acc;
        acc += c;
    }
    const uint32_t packets = sched[kStatPackets], retraced = sched[kStatRetraced];
    uint32_t choice = sched[kStatChoice];
    if (choice != kChoiceNarrow && choice != kChoiceWide) choice = kChoiceNarrow;
    if (packets > 0u && retraced <= packets)
        choice = (unsigned long long)retraced * 16ull > (unsigned long long)packets * kWideSixteenths ? kChoiceWide
                                                                                                     : kChoiceNarrow;
    sched[kStatChoice] = choice;
    sched[kStatPackets] = 0u;
    sched[kStatRetraced] = 0u;
}

__global__ void sched_scatter_kernel(uint32_t *sched, int ntiles) {
    const int tile = blockIdx.x * blockDim.x + threadIdx.x;
    if (tile >= ntiles) return;
    const uint32_t est = sched[kSchedHeader + tile];
    const uint32_t key = est ? (uint32_t)__clz(est) : 32u;
    const uint32_t pos = atomicAdd(&sched[1 + key], 1u);
    if (pos < (uint32_t)ntiles) sched[kSchedHeader + ntiles + pos] = (uint32_t)tile;
}

// ---------------------------------------------------------------------------------------------
// Ellipsoid view (reference: cuda/ellipsoid_viewer.cu:1-94): closest-hit ray tracing of each
// Gaussian's support ellipsoid (the unit sphere of its snapshot frame), flat-shaded.  A Gaussian
// takes part if its snapshot marked it visible and its live opacity is >= ellipsoid_min_opacity.
// Per Gaussian the hit distance is the near root t0 = (s - h) / |ld| of the object-space ray when
// t0 >= znear, else the far root t1 = (s + h) / |ld|; the ray keeps the smallest distance in
// [znear, zfar] (equal distances: the smaller gaussian id, where OptiX keeps whichever its
// traversal reported first).  Output: RGB = max(0.5, <-view, normal>) (colour + 0.15) and depth =
// t, or the background and depth 0 on a miss; an inactive pixel (zero direction) is left as is.
// ---------------------------------------------------------------------------------------------
constexpr int kEllStack = 64;

// Distance of the ray's hit on Gaussian gid's ellipsoid, if it has one at or beyond tmin.
__device__ __forceinline__ bool ellipsoid_hit(const float4 g0, const float4 g1, const float4 g2, f3 ro, f3 rd,
                                              float tmin, float &t) {
    LocalHit h;
    local_ray(g0, g1, g2, ro, rd, h);
    if (h.b > 0.0f) return false;  // centre behind the ray
    const float norm = sqrtf(fdot3(h.ld, h.ld));
    const f3 dn = mk3(h.ld.x / norm, h.ld.y / norm, h.ld.z / norm);
    const float smid = -fdot3(h.lo, dn);
    const f3 u = mk3(fmaf(smid, dn.x, h.lo.x), fmaf(smid, dn.y, h.lo.y), fmaf(smid, dn.z, h.lo.z));
    const float sq = fdot3(u, u);
    if (sq > 1.0f) return false;
    const float hc = sqrtf(1.0f - sq);
    const float t0 = (smid - hc) / norm, t1 = (smid + hc) / norm;
    t = t0 >= tmin ? t0 : t1;
    return t >= tmin;
}

// Flat shading of the winning hit: object-space normal at the hit, carried to world space by the
// transpose of the snapshot matrix M (the inverse-transpose of the instance transform).
__device__ __forceinline__ void ellipsoid_shade(const float4 g0, const float4 g1, const float4 g2, f3 ro, f3 rd,
                                                float t, const float *c, float &r0, float &r1, float &r2) {
    LocalHit h;
    local_ray(g0, g1, g2, ro, rd, h);
    const float norm = sqrtf(fdot3(h.ld, h.ld));
    const f3 dn = mk3(h.ld.x / norm, h.ld.y / norm, h.ld.z / norm);
    const float tn = t * norm;
    f3 ln = mk3(fmaf(tn, dn.x, h.lo.x), fmaf(tn, dn.y, h.lo.y), fmaf(tn, dn.z, h.lo.z));
    const float ll = sqrtf(fdot3(ln, ln));
    ln = mk3(ln.x / ll, ln.y / ll, ln.z / ll);
    f3 wn = mk3(fmaf(ln.z, g2.x, fmaf(ln.y, g1.x, ln.x * g0.x)), fmaf(ln.z, g2.y, fmaf(ln.y, g1.y, ln.x * g0.y)),
                fmaf(ln.z, g2.z, fmaf(ln.y, g1.z, ln.x * g0.z)));
    const float wl = sqrtf(fdot3(wn, wn));
    wn = mk3(wn.x / wl, wn.y / wl, wn.z / wl);
    const float dl = sqrtf(fdot3(rd, rd));
    const f3 vd = mk3(rd.x / dl, rd.y / dl, rd.z / dl);
    const float align = fmaxf(0.5f, -fdot3(vd, wn));
    r0 = align * (c[0] + 0.15f);
    r1 = align * (c[1] + 0.15f);
    r2 = align * (c[2] + 0.15f);
}

// Entry distance of the ray into a box (slab test of SlabRay), or false if it misses.
__device__ __forceinline__ bool slab_enter(const float bmin[3], const float bmax[3], const SlabRay &r, float &tn) {
    float ta = fmaf(bmin[0], r.inv.x, r.clo.x), tb = fmaf(bmax[0], r.inv.x, r.chi.x);
    float n0 = fminf(ta, tb), f0 = fmaxf(ta, tb);
    ta = fmaf(bmin[1], r.inv.y, r.clo.y);
    tb = fmaf(bmax[1], r.inv.y, r.chi.y);
    n0 = fmaxf(n0, fminf(ta, tb));
    f0 = fminf(f0, fmaxf(ta, tb));
    ta = fmaf(bmin[2], r.inv.z, r.clo.z);
    tb = fmaf(bmax[2], r.inv.z, r.chi.z);
    n0 = fmaxf(n0, fminf(ta, tb));
    f0 = fminf(f0, fmaxf(ta, tb));
    tn = n0;
    return n0 <= f0 && f0 >= 0.0f;
}

__device__ __forceinline__ void ellipsoid_leaf(const FwdArgs &a, uint32_t gid, f3 ro, f3 rd, float znear, float minop,
                                               float &best, uint32_t &bid) {
    if (a.live[gid].x < minop) return;
    float t;
    if (!ellipsoid_hit(a.geom[3 * gid], a.geom[3 * gid + 1], a.geom[3 * gid + 2], ro, rd, znear, t)) return;
    if (t < best || (t == best && gid < bid)) {
        best = t;
        bid = gid;
    }
}

constexpr int kEllTileX = 16, kEllTileY = 8;

__device__ __forceinline__ void ellipsoid_pixel(const FwdArgs &a, int px, int py) {
    if (px >= (int)a.render_w || py >= (int)a.render_h) return;
    const uint32_t pixel = (uint32_t)py * a.alloc_w + (uint32_t)px;
    if (!a.display && *a.grads_enabled) raise_status(a.status, GRAY_STATUS_BAD_MODE);
    f3 ro, rd;
    if (*a.rays_from_python) {
        ro = mk3(a.ray_o[3 * pixel], a.ray_o[3 * pixel + 1], a.ray_o[3 * pixel + 2]);
        rd = mk3(a.ray_d[3 * pixel], a.ray_d[3 * pixel + 1], a.ray_d[3 * pixel + 2]);
    } else {
        ro = mk3(a.cam_origin[0], a.cam_origin[1], a.cam_origin[2]);
        float jx = 0.0f, jy = 0.0f;
        if (*a.jitter) {
            uint32_t h = pcg_hash(pixel ^ pcg_hash(*a.total_num_calls));
            jx = (float)(h & 0xFFFFu) * 0x1.0p-16f - 0.5f;
            jy = (float)(h >> 16) * 0x1.0p-16f - 0.5f;
        }
        rd = camera_ray(a.w2c, *a.fov, px, py, a.render_w, a.render_h, jx, jy);
    }
    a.head[pixel] = GRAY_NULL;  // no backward hit list for this frame
    if (sqrtf(dot3(rd, rd)) == 0.0f) return;
    const float znear = *a.znear, minop = *a.ellipsoid_min_opacity;
    float best = *a.zfar;
    uint32_t bid = GRAY_NULL;
    const int n = a.n;
    const SlabRay sr = make_slab_ray(ro, rd, 2.0e-6f * (fabsf(ro.x) + fabsf(ro.y) + fabsf(ro.z)));
    if (n == 1) {
        ellipsoid_leaf(a, 0u, ro, rd, znear, minop, best, bid);
    } else if (n > 1) {
        uint32_t stk[kEllStack];
        int sp = 0;
        float tr;
        const float *rb = a.root_box;
        const float rmin[3] = {rb[0], rb[1], rb[2]}, rmax[3] = {rb[4], rb[5], rb[6]};
        if (slab_enter(rmin, rmax, sr, tr) && tr <= best) stk[sp++] = 0u;
        long long budget = 2LL * n;
        while (sp > 0) {
            if (--budget < 0) {
                raise_status(a.status, GRAY_STATUS_STACK_OVERFLOW);
                break;
            }
            const uint32_t node = stk[--sp];
            if (node >= (uint32_t)(n - 1)) {
                raise_status(a.status, GRAY_STATUS_STACK_OVERFLOW);
                continue;
            }
            const float4 q0 = a.nodes[4 * node], q1 = a.nodes[4 * node + 1], q2 = a.nodes[4 * node + 2],
                         q3 = a.nodes[4 * node + 3];
            const float b0min[3] = {q0.x, q0.y, q0.z}, b0max[3] = {q0.w, q1.x, q1.y};
            const float b1min[3] = {q1.z, q1.w, q2.x}, b1max[3] = {q2.y, q2.z, q2.w};
            const uint32_t c0 = __float_as_uint(q3.x), c1 = __float_as_uint(q3.y);
            float t0, t1;
            bool h0 = slab_enter(b0min, b0max, sr, t0) && t0 <= best;
            bool h1 = slab_enter(b1min, b1max, sr, t1) && t1 <= best;
            // leaves right away (they may shrink `best` before the boxes are pushed)
            if (h0 && (c0 & GRAY_LEAF_BIT)) {
                if ((c0 & ~GRAY_LEAF_BIT) < (uint32_t)n) ellipsoid_leaf(a, c0 & ~GRAY_LEAF_BIT, ro, rd, znear, minop, best, bid);
                h0 = false;
            }
            if (h1 && (c1 & GRAY_LEAF_BIT)) {
                if ((c1 & ~GRAY_LEAF_BIT) < (uint32_t)n) ellipsoid_leaf(a, c1 & ~GRAY_LEAF_BIT, ro, rd, znear, minop, best, bid);
                h1 = false;
            }
            h0 = h0 && t0 <= best;
            h1 = h1 && t1 <= best;
            // far child deeper in the stack, near child on top
            const bool near1 = h0 && h1 && t1 < t0;
            const uint32_t first = near1 ? c0 : c1, second = near1 ? c1 : c0;
            const bool hf = near1 ? h0 : h1, hs = near1 ? h1 : h0;
            if (sp + (int)hf + (int)hs > kEllStack) {
                raise_status(a.status, GRAY_STATUS_STACK_OVERFLOW);
                break;
            }
            if (hf) stk[sp++] = first;
            if (hs) stk[sp++] = second;
        }
    }
    float r0 = a.bg[0], r1 = a.bg[1], r2 = a.bg[2], depth = 0.0f;
    if (bid != GRAY_NULL) {
        ellipsoid_shade(a.geom[3 * bid], a.geom[3 * bid + 1], a.geom[3 * bid + 2], ro, rd, best,
                        a.channels + 3 * (size_t)bid, r0, r1, r2);
        depth = best;
    }
    a.out_rgb[3 * pixel] = r0;
    a.out_rgb[3 * pixel + 1] = r1;
    a.out_rgb[3 * pixel + 2] = r2;
    a.out_depth[pixel] = depth;
}

// Grid-stride over 16x8-pixel tiles (a few blocks per SM): the launch made on every forward costs
// little when the view is off.
__global__ void __launch_bounds__(kEllTileX * kEllTileY) ellipsoid_kernel(const FwdArgs a, int tiles_x, int ntiles) {
    if (!*a.render_ellipsoids) return;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x)
        ellipsoid_pixel(a, (t % tiles_x) * kEllTileX + threadIdx.x, (t / tiles_x) * kEllTileY + threadIdx.y);
}

// ---------------------------------------------------------------------------------------------
// Batched render: many views (of one or several resident scenes) in one persistent launch.
// Warps pull 32-ray packets from a global counter; packet -> (view, tile) through the views'
// packet offsets.  Forward only (no gradients, no hit lists); per view the output is RGB.
// A view's packets form groups of 2x2 (group_offset numbers them across views); with a frontier
// buffer, batch_frontier_kernel first writes each group's BVH frontier and the packets of the group
// start their traversals there, as the plain forward's blocks do.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ int batch_view_of(const gray_batch_view *views, int nviews, uint32_t packet) {
    int v = 0;
    while (v + 1 < nviews && views[v + 1].packet_offset <= packet) v++;
    return v;
}

__global__ void __launch_bounds__(32) batch_frontier_kernel(const gray_batch_scene *__restrict__ scenes,
                                                            const gray_batch_view *__restrict__ views, int nviews,
                                                            uint32_t *__restrict__ frontier, int tile_w,
                                                            uint32_t cut) {
    __shared__ FrontierScratch fs;
    const uint32_t group = blockIdx.x;
    const int lane = threadIdx.x;
    int v = 0;
    while (v + 1 < nviews && views[v + 1].group_offset <= group) v++;
    const gray_batch_view &vw = views[v];
    const gray_batch_scene &bs = scenes[vw.scene];
    uint32_t *out = frontier + (size_t)group * kFrontierWords;
    const int tile_h = 32 / tile_w;
    const uint32_t tiles_x = (vw.width + tile_w - 1) / tile_w;
    const uint32_t gxn = (tiles_x + 1) / 2, local = group - vw.group_offset;
    const int x0 = (int)((local % gxn) * 2 * tile_w), y0 = (int)((local / gxn) * 2 * tile_h);
    if (bs.n <= 1 || x0 >= (int)vw.width || y0 >= (int)vw.height) {
        if (lane == 0) out[0] = kFrontierNone;
        return;
    }
    const int x1 = min(x0 + 2 * tile_w, (int)vw.width) - 1, y1 = min(y0 + 2 * tile_h, (int)vw.height) - 1;
    make_frustum_warp(fs.fr, mk3(vw.origin[0], vw.origin[1], vw.origin[2]), vw.w2c, vw.fov_y, x0, y0, x1, y1, vw.width,
                      vw.height, bs.root_box);
    frontier_walk<false>(reinterpret_cast<const float4 *>(bs.nodes), bs.n, cut, fs, nullptr, out, nullptr);
}

template <int KB, int MINB>
__global__ void __launch_bounds__(kFwdThreads, MINB)
    trace_batch_kernel(const gray_batch_scene *__restrict__ scenes, const gray_batch_view *__restrict__ views,
                       int nviews, uint32_t total_packets, float *__restrict__ out, uint32_t *__restrict__ counter,
                       int tile_w, const uint32_t *__restrict__ frontier, uint32_t total_groups,
                       int32_t *status) {
    __shared__ unsigned long long kbuf[KB][kFwdThreads];
    __shared__ Frustum sfr[kWarps];
    __shared__ uint32_t sstk[kWarps][kWideStack];
    __shared__ uint32_t scand[kWarps][kQueue];
    __shared__ CandCache scc[kWarps];
    // the packet's scene and view parameters live in shared memory (read where used), which keeps
    // them out of the registers the traversal needs
    __shared__ TraceScene s_sc[kWarps];
    __shared__ TraceKnobs s_k[kWarps];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tile_h = 32 / tile_w;
    for (;;) {
        __syncwarp();
        uint32_t packet = 0;
        if (lane == 0) packet = atomicAdd(counter, 1u);
        packet = __shfl_sync(kFull, packet, 0);
        if (packet >= total_packets) break;
        const gray_batch_view &vw = views[batch_view_of(views, nviews, packet)];
        const gray_batch_scene &bs = scenes[vw.scene];
        const uint32_t local = packet - vw.packet_offset;
        const uint32_t tiles_x = (vw.width + tile_w - 1) / tile_w;
        const int px = (int)((local % tiles_x) * tile_w) + lane % tile_w;
        const int py = (int)((local / tiles_x) * tile_h) + lane / tile_w;
        const bool inside = px < (int)vw.width && py < (int)vw.height;
        if (lane == 0) {
            TraceKnobs &k = s_k[warp];
            k.znear = vw.znear;
            k.zfar = vw.zfar;
            k.athr = bs.alpha_threshold;
            k.pw = bs.exp_power;
            k.tthr = bs.t_threshold;
            k.render_depth = false;
            s_sc[warp] = TraceScene{reinterpret_cast<const float4 *>(bs.geom), reinterpret_cast<const float4 *>(bs.l2w),
                                    reinterpret_cast<const float2 *>(bs.live), vw.channels,
                                    reinterpret_cast<const float4 *>(bs.nodes), bs.root_box, bs.n};
        }
        __syncwarp();
        const TraceScene &sc = s_sc[warp];
        const TraceKnobs &k = s_k[warp];
        const HitSink hs{nullptr, nullptr, 0};
        f3 ro = mk3(vw.origin[0], vw.origin[1], vw.origin[2]);
        f3 rd = mk3(0.0f, 0.0f, 0.0f);
        if (inside) rd = camera_ray(vw.w2c, vw.fov_y, px, py, vw.width, vw.height, 0.0f, 0.0f);
        {
            const int x0 = (int)((local % tiles_x) * tile_w), y0 = (int)((local / tiles_x) * tile_h);
            make_frustum_warp(sfr[warp], ro, vw.w2c, vw.fov_y, x0, y0, x0 + tile_w - 1, y0 + tile_h - 1, vw.width,
                              vw.height, s_sc[warp].root_box);
        }
        const uint32_t *front = nullptr;
        uint32_t front_off = 0u;
        if (frontier) {
            const uint32_t tx = local % tiles_x, ty = local / tiles_x;
            const uint32_t grp = vw.group_offset + (ty / 2) * ((tiles_x + 1) / 2) + tx / 2;
            if (grp < total_groups) {  // else: from the root
                front = frontier;
                front_off = grp * (uint32_t)kFrontierWords;
            }
        }
        RayResult r;
        trace_ray<KB>(sc, k, ro, rd, inside, false, hs, status, kbuf, r, &sfr[warp], sstk[warp], scand[warp],
                      &scc[warp], front, front_off);
        if (!inside) continue;
        float r0, r1, r2;
        finish_ray(r, bs.bg, 1e-12f, false, r0, r1, r2);
        float *o = out + vw.out_offset + 3 * ((size_t)py * vw.width + px);
        o[0] = r.C0;
        o[1] = r.C1;
        o[2] = r.C2;
    }
}

static FwdArgs forward_args(const gray_params &p, bool display) {
    FwdArgs a;
    a.display = display ? 1 : 0;
    a.auto_role = 0;
    a.alloc_w = p.image_width;
    a.render_w = p.render_width;
    a.render_h = p.render_height;
    a.n = p.gaussians.count;
    a.cam_origin = p.camera.origin;
    a.fov = p.camera.vertical_fov_radians;
    a.w2c = p.camera.rotation_w2c;
    a.znear = p.camera.znear;
    a.zfar = p.camera.zfar;
    a.exp_power = p.config.exp_power;
    a.alpha_threshold = p.config.alpha_threshold;
    a.t_threshold = p.config.t_threshold;
    a.eps_fwd = p.config.eps_forward_normalization;
    a.bg = p.config.background_channels;
    a.render_depth = p.config.render_depth;
    a.needs_ray_output = p.config.needs_ray_output;
    a.rays_from_python = p.config.rays_from_python;
    a.jitter = p.config.jitter_primary_rays;
    a.grads_enabled = p.metadata.grads_enabled;
    a.total_num_calls = p.metadata.total_num_calls;
    a.geom = reinterpret_cast<const float4 *>(p.scene.geom);
    a.l2w = reinterpret_cast<const float4 *>(p.scene.l2w);
    a.live = reinterpret_cast<const float2 *>(p.scene.live);
    a.channels = p.gaussians.channels;
    a.nodes = reinterpret_cast<const float4 *>(p.scene.nodes);
    a.root_box = p.scene.root_box;
    a.out_rgb = p.framebuffer.output_channels;
    a.out_depth = p.framebuffer.output_depth;
    a.out_T = p.framebuffer.transmittance;
    a.out_fullT = p.framebuffer.full_transmittance;
    a.out_rem = p.framebuffer.remaining_channels_estimate;
    a.ray_o = p.framebuffer.ray_origin;
    a.ray_d = p.framebuffer.ray_direction;
    a.stat_hit = p.stats.num_gaussians_hit;
    a.stat_acc = p.stats.num_gaussians_accumulated;
    a.head = p.hitlist.head_per_pixel;
    a.counter = p.hitlist.total_words;
    a.pool = p.hitlist.pool;
    a.pool_size = p.hitlist.size;
    a.status = p.status;
    a.render_ellipsoids = p.config.render_ellipsoids;
    a.ellipsoid_min_opacity = p.config.ellipsoid_min_opacity;
    a.tile_w = 8;
    a.tile_h = 4;
    a.schedule = nullptr;
    a.frontier = nullptr;
    a.frontier_cut = 0;
    a.super_frontier = nullptr;
    a.super_x = 0;
    return a;
}

cudaError_t launch_ellipsoids(const gray_params &p, bool display, cudaStream_t s) {
    const FwdArgs a = forward_args(p, display);
    const int tiles_x = (int)((p.render_width + kEllTileX - 1) / kEllTileX);
    const int ntiles = tiles_x * (int)((p.render_height + kEllTileY - 1) / kEllTileY);
    if (ntiles <= 0) return cudaSuccess;
    int dev = 0, sms = 0;
    cudaError_t e;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    const int grid = ntiles < 8 * sms ? ntiles : 8 * sms;
    ellipsoid_kernel<<<grid, dim3(kEllTileX, kEllTileY), 0, s>>>(a, tiles_x, ntiles);
    return cudaGetLastError();
}

// Launch shape of one forward: the kernel arguments, the trace kernel and its grid, and whether the
// tile schedule (work estimate, densest-first order, per-tile BVH frontier) is used.
struct FwdPlan {
    FwdArgs a;
    const void *kern;
    const void *kern_wide;  // automatic choice: the wide kernel, launched after `kern` (else null)
    dim3 grid;
    int bw, bh;
    bool sched;
    int nsuper;  // super-tiles whose coarse frontiers seed the tile walks (0: tiles walk from the root)
};

static FwdPlan plan_forward(const gray_params &p, bool display) {
    FwdPlan q;
    q.nsuper = 0;
    FwdArgs &a = q.a;
    a = forward_args(p, display);
    // variant: bits 0-1 select (buffer size, register cap), bit 2 the packet shape, bits 3-4 the
    // tile frontier's cut (64 leaves, 32, 128, no frontier), bit 5 packets claimed per warp
    // (trace_forward_claim_kernel) instead of tiles per block
    // variant 0 (the default) chooses between the narrow and the wide kernel of kDefaultTraceVariant's
    // packet shape and cut from the last scheduled forward's re-traversals: the 16-slot hit buffer with
    // six blocks per SM is faster where few rays composite more than 16 hits, the 32-slot one with
    // four blocks where many do (a re-traversal repeats the packet's whole traversal)
    const bool automatic = p.trace_variant <= 0;
    const int v = p.trace_variant > 0 ? p.trace_variant : kDefaultTraceVariant;
    const int fcut = (v >> 3) & 3;
    const bool claim = (v & 32) != 0;
    q.kern_wide = nullptr;
    a.tile_w = (v & 4) ? 4 : 8;
    a.tile_h = 32 / a.tile_w;
    q.bw = a.tile_w * kBlockWarpsX;
    q.bh = a.tile_h * kBlockWarpsY;
    q.grid = dim3((p.render_width + q.bw - 1) / q.bw, (p.render_height + q.bh - 1) / q.bh);
    a.tiles_x = (int)q.grid.x;
    a.ntiles = (int)(q.grid.x * q.grid.y);
    a.schedule = nullptr;
    const size_t words = gray_schedule_words_for(p.image_width, p.image_height);
    q.sched = p.hitlist.schedule && a.ntiles > 0 && (size_t)a.ntiles <= (words - kSchedHeader) / 2;
#define GRAY_FWD_KERNEL(KB, MINB)                                                                   \
    (!q.sched ? reinterpret_cast<const void *>(&trace_forward_kernel<KB, MINB>)                     \
     : claim  ? reinterpret_cast<const void *>(&trace_forward_claim_kernel<KB, MINB>)               \
              : reinterpret_cast<const void *>(&trace_forward_sched_kernel<KB, MINB>))
    switch (v & 3) {
        case 0: q.kern = GRAY_FWD_KERNEL(32, 1); break;
        case 1: q.kern = GRAY_FWD_KERNEL(32, 4); break;
        case 2: q.kern = GRAY_FWD_KERNEL(16, 1); break;
        default: q.kern = GRAY_FWD_KERNEL(16, 6); break;
    }
#undef GRAY_FWD_KERNEL
    if (q.sched) {
        a.schedule = p.hitlist.schedule;
        if (automatic) {
            q.kern = reinterpret_cast<const void *>(&trace_forward_sched_kernel<16, 6>);
            q.kern_wide = reinterpret_cast<const void *>(&trace_forward_sched_kernel<32, 4>);
        }
        a.frontier_cut = fcut == 0 ? kFrontierCutDefault : fcut == 1 ? 32u : fcut == 2 ? 128u : 0u;
        if (a.frontier_cut > 0 && (size_t)a.ntiles <= (words - kSchedHeader) / (2 + kFrontierWords))
            a.frontier = a.schedule + kSchedHeader + 2 * (size_t)a.ntiles;
        if (a.frontier) {
            // super-tiles after the tiles' frontiers, when the buffer holds them
            const int sx = (a.tiles_x + kSuperTiles - 1) / kSuperTiles;
            const int sy = ((int)q.grid.y + kSuperTiles - 1) / kSuperTiles;
            const size_t used = (size_t)kSchedHeader + (2 + (size_t)kFrontierWords) * (size_t)a.ntiles;
            if (used + (size_t)sx * (size_t)sy * kSuperWords <= words) {
                a.super_frontier = a.frontier + (size_t)a.ntiles * kFrontierWords;
                a.super_x = sx;
                q.nsuper = sx * sy;
            }
        }
    }
    return q;
}

bool trace_forward_has_schedule(const gray_params &p) { return plan_forward(p, false).sched; }

cudaError_t launch_trace_schedule(const gray_params &p, bool display, cudaStream_t s) {
    const FwdPlan q = plan_forward(p, display);
    if (!q.sched) return cudaSuccess;
    // densest tiles first: per-tile estimate and frontier, bucket by log2 of the estimate, order
    cudaError_t e;
    if ((e = cudaMemsetAsync(q.a.schedule, 0, sizeof(uint32_t) * kSchedZeroWords, s)) != cudaSuccess) return e;
    if (q.nsuper > 0) super_cost_kernel<<<q.nsuper, 32, 0, s>>>(q.a, q.bw, q.bh, q.nsuper);
    tile_cost_kernel<<<q.a.ntiles, 32, 0, s>>>(q.a, q.bw, q.bh);
    sched_scan_kernel<<<1, 32, 0, s>>>(q.a.schedule);
    sched_scatter_kernel<<<(q.a.ntiles + 255) / 256, 256, 0, s>>>(q.a.schedule, q.a.ntiles);
    return cudaGetLastError();
}

cudaError_t launch_trace_forward(const gray_params &p, bool display, bool schedule_ready, cudaStream_t s) {
    FwdPlan q = plan_forward(p, display);
    cudaError_t e;
    if (!q.sched) {
        void *args[] = {&q.a};
        if ((e = cudaLaunchKernel(q.kern, q.grid, dim3(kFwdThreads), args, 0, s)) != cudaSuccess) return e;
        return cudaGetLastError();
    }
    if (!schedule_ready && (e = launch_trace_schedule(p, display, s)) != cudaSuccess) return e;
    int dev = 0, sms = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    // persistent grids that take the tiles in the schedule's order; with the automatic choice both
    // kernels are launched and the one not chosen returns at once
    const void *kerns[2] = {q.kern, q.kern_wide};
    const int roles[2] = {q.kern_wide ? (int)kChoiceNarrow : 0, (int)kChoiceWide};
    for (int i = 0; i < 2 && kerns[i]; i++) {
        int per_sm = 0;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kerns[i], kFwdThreads, 0)) != cudaSuccess)
            return e;
        const unsigned int want = (unsigned int)(sms * (per_sm > 0 ? per_sm : 1));
        const dim3 grid(want < (unsigned int)q.a.ntiles ? want : (unsigned int)q.a.ntiles, 1, 1);
        FwdArgs a = q.a;
        a.auto_role = roles[i];
        void *args[] = {&a};
        if ((e = cudaLaunchKernel(kerns[i], grid, dim3(kFwdThreads), args, 0, s)) != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

size_t gray_schedule_words_for(uint32_t width, uint32_t height) {
    // estimates and order for any tile shape (tiles of at least 8x8 pixels), frontiers for tiles
    // of 8x16 or 16x8 pixels (the forward's block tiles)
    const size_t t8 = (size_t)((width + 7) / 8) * (size_t)((height + 7) / 8);
    const size_t ta = (size_t)((width + 7) / 8) * (size_t)((height + 15) / 16);
    const size_t tb = (size_t)((width + 15) / 16) * (size_t)((height + 7) / 8);
    // and the coarse frontiers of their super-tiles (kSuperTiles x kSuperTiles tiles)
    const size_t k = kSuperTiles;
    const size_t sa = (((width + 7) / 8 + k - 1) / k) * (((height + 15) / 16 + k - 1) / k);
    const size_t sb = (((width + 15) / 16 + k - 1) / k) * (((height + 7) / 8 + k - 1) / k);
    return (size_t)kSchedHeader + 2 * t8 + (ta > tb ? ta : tb) * kFrontierWords + (sa > sb ? sa : sb) * kSuperWords;
}

cudaError_t launch_trace_batch(const gray_batch_scene *scenes, const gray_batch_view *views, int nviews,
                               uint32_t total_packets, float *out, uint32_t *counter, uint32_t *frontier,
                               uint32_t total_groups, int variant, int blocks_per_sm, int32_t *status,
                               cudaStream_t s) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    const int v = variant > 0 ? variant : kDefaultTraceVariant;
    const int tile_w = (v & 4) ? 4 : 8;
    const int fcut = (v >> 3) & 3;
    const uint32_t cut = fcut == 0 ? kFrontierCutDefault : fcut == 1 ? 32u : fcut == 2 ? 128u : 0u;
    const unsigned int grid = (unsigned int)(sms * (blocks_per_sm > 0 ? blocks_per_sm : 4));
    if ((e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), s)) != cudaSuccess) return e;
    if (!frontier || cut == 0 || total_groups == 0) {
        frontier = nullptr;
    } else {
        batch_frontier_kernel<<<total_groups, 32, 0, s>>>(scenes, views, nviews, frontier, tile_w, cut);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    const uint32_t *fr = frontier;
    switch (v & 3) {
        case 0: trace_batch_kernel<32, 1><<<grid, kFwdThreads, 0, s>>>(scenes, views, nviews, total_packets, out, counter, tile_w, fr, total_groups, status); break;
        case 1: trace_batch_kernel<32, 4><<<grid, kFwdThreads, 0, s>>>(scenes, views, nviews, total_packets, out, counter, tile_w, fr, total_groups, status); break;
        case 2: trace_batch_kernel<16, 1><<<grid, kFwdThreads, 0, s>>>(scenes, views, nviews, total_packets, out, counter, tile_w, fr, total_groups, status); break;
        default: trace_batch_kernel<16, 6><<<grid, kFwdThreads, 0, s>>>(scenes, views, nviews, total_packets, out, counter, tile_w, fr, total_groups, status); break;
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Backward
// ---------------------------------------------------------------------------------------------
struct BwdArgs {
    uint32_t alloc_w, render_w, render_h;
    int n;
    const float *exp_power, *alpha_threshold, *eps_scale_grad, *bg;
    const float4 *geom, *rec;
    const float *pix_T, *pix_fullT, *pix_rem, *ray_o, *ray_d, *grad_out;
    const uint32_t *head, *pool;
    uint32_t pool_size;
    float *grad_acc;
    int32_t *status;
};

__device__ __forceinline__ void red_add4(float *addr, float x, float y, float z, float w) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(x), "f"(y), "f"(z), "f"(w));
}

// Adds one hit's 16 gradient values to the Gaussian's accumulator row.  Neighbouring pixels
// composite the same Gaussians at the same replay step (on the benchmark scene a warp's lanes form
// groups of 16 on average, often the whole warp), and vector reductions on one row serialise in L2,
// so the lanes that hold the same Gaussian first combine their values and the lowest of them issues
// the four reductions.  The combination is a tree over the group's ranks: every lane knows the next
// member of its group (`nxt`, the member `s` ranks further after the round of stride s, found by
// pointer jumping), and in the round of stride s the members whose rank is a multiple of 2s add
// the partial sum of the member s ranks further; after ceil(log2(largest group)) rounds the lowest
// member holds the group's sum (16 shuffles per round instead of 16 per member).
__device__ __forceinline__ void reduce_hit(float *row, uint32_t gid, float (&v)[16]) {
    const unsigned active = __activemask();
    const unsigned grp = __match_any_sync(active, gid);
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const int rank = __popc(grp & below);
    const int gmax = (int)__reduce_max_sync(active, (unsigned)__popc(grp));
    const unsigned above = grp & ~below & ~(1u << lane);
    int nxt = above ? __ffs(above) - 1 : -1;  // the member one rank further, -1: none
    for (int s = 1; s < gmax; s <<= 1) {
        const int src = nxt >= 0 ? nxt : lane;
        const bool take = nxt >= 0 && (rank & (2 * s - 1)) == 0;
#pragma unroll
        for (int k = 0; k < 16; k++) {
            const float t = __shfl_sync(active, v[k], src);
            if (take) v[k] += t;
        }
        const int jump = __shfl_sync(active, nxt, src);
        nxt = nxt >= 0 ? jump : -1;
    }
    if (rank == 0) {
        red_add4(row, v[0], v[1], v[2], v[3]);
        red_add4(row + 4, v[4], v[5], v[6], v[7]);
        red_add4(row + 8, v[8], v[9], v[10], v[11]);
        red_add4(row + 12, v[12], v[13], v[14], v[15]);
    }
}

// Per-Gaussian backward record: what the reverse replay needs of one Gaussian besides its snapshot
// rows (M | mu), precomputed once per backward pass instead of once per composited hit.  Written
// from the state the forward used: live opacity o and scaling factor sf, colour c, current log-scale
// and rotation q, snapshot L2W rows L.  24 floats (6 x float4):
//   [o, sf, 1/|q|, s0] [s1, s2, c0, c1] [c2, K00, K01, K02] [K10, K11, K12, K20] [K21, K22, 0, 0]
//   [qn0, qn1, qn2, qn3]
// with s = exp(scale), K_rk = L_rk / (s_k sf + eps_scale_grad) * s_k (the scale gradient's factor,
// cuda/backward_pass.cu:101-111) and qn = q / |q|.
constexpr int kRecVec = 6;

__device__ __forceinline__ void bwd_record_one(float2 lv, const float log_s[3], float4 q, const float ch[3], float4 L0,
                                               float4 L1, float4 L2, float eps, float4 r[kRecVec]) {
    const float sf = lv.y;
    float s[3];
#pragma unroll
    for (int k = 0; k < 3; k++) s[k] = gexp(log_s[k]);
    const float qlen = sqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
    const float d0 = s[0] * sf + eps, d1 = s[1] * sf + eps, d2 = s[2] * sf + eps;
    r[0] = make_float4(lv.x, sf, 1.0f / qlen, s[0]);
    r[1] = make_float4(s[1], s[2], ch[0], ch[1]);
    r[2] = make_float4(ch[2], L0.x / d0 * s[0], L0.y / d1 * s[1], L0.z / d2 * s[2]);
    r[3] = make_float4(L1.x / d0 * s[0], L1.y / d1 * s[1], L1.z / d2 * s[2], L2.x / d0 * s[0]);
    r[4] = make_float4(L2.y / d1 * s[1], L2.z / d2 * s[2], 0.0f, 0.0f);
    r[5] = make_float4(q.x / qlen, q.y / qlen, q.z / qlen, q.w / qlen);
}

// One thread per Gaussian of [first, n): the tail of the bulk-pipelined kernel, and the whole pass
// when a pointer is not 16-byte aligned.
__global__ void __launch_bounds__(256) bwd_record_kernel(int first, int n, const float2 *__restrict__ live,
                                                         const float *__restrict__ scale,
                                                         const float4 *__restrict__ rotation,
                                                         const float *__restrict__ channels,
                                                         const float4 *__restrict__ l2w,
                                                         const float *__restrict__ eps_scale_grad,
                                                         float4 *__restrict__ rec) {
    const int i = first + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float ls[3] = {scale[3 * i], scale[3 * i + 1], scale[3 * i + 2]};
    const float ch[3] = {channels[3 * i], channels[3 * i + 1], channels[3 * i + 2]};
    float4 r[kRecVec];
    bwd_record_one(live[i], ls, rotation[i], ch, l2w[3 * i], l2w[3 * i + 1], l2w[3 * i + 2], *eps_scale_grad, r);
    float4 *o = rec + kRecVec * (size_t)i;
#pragma unroll
    for (int k = 0; k < kRecVec; k++) o[k] = r[k];
}

// Bulk-pipelined record pass: persistent blocks take tiles of kRecTile Gaussians; one thread loads
// a tile's inputs (live, scale, rotation, channels, l2w rows: 96 B per Gaussian, five contiguous
// ranges) into one of two shared-memory stages with bulk copies completing on an mbarrier, so the
// next tile's loads are in flight while this one is computed, and stores the tile's records (96 B
// per Gaussian) from a shared-memory copy with one bulk copy.  Every copy starts on a 16-byte
// boundary and spans a multiple of 16 bytes (the launcher checks the pointers).
constexpr int kRecTile = 128;
static_assert(kRecTile % 16 == 0, "every per-tile range must span a multiple of 16 bytes");

struct RecIn {
    float4 l2w[3 * kRecTile];
    float4 rotation[kRecTile];
    float2 live[kRecTile];
    float scale[3 * kRecTile];
    float channels[3 * kRecTile];
};
constexpr uint32_t kRecInBytes = 96u * kRecTile;

__device__ __forceinline__ void rec_issue_loads(RecIn &in, uint64_t *bar, int tile, const float2 *live,
                                                const float *scale, const float4 *rotation, const float *channels,
                                                const float4 *l2w) {
    const size_t g0 = (size_t)tile * kRecTile;
    mbar_expect_tx(bar, kRecInBytes);
    bulk_load(in.l2w, l2w + 3 * g0, 48u * kRecTile, bar);
    bulk_load(in.rotation, rotation + g0, 16u * kRecTile, bar);
    bulk_load(in.live, live + g0, 8u * kRecTile, bar);
    bulk_load(in.scale, scale + 3 * g0, 12u * kRecTile, bar);
    bulk_load(in.channels, channels + 3 * g0, 12u * kRecTile, bar);
}

__global__ void __launch_bounds__(kRecTile) bwd_record_bulk_kernel(
    int tiles, const float2 *__restrict__ live, const float *__restrict__ scale, const float4 *__restrict__ rotation,
    const float *__restrict__ channels, const float4 *__restrict__ l2w, const float *__restrict__ eps_scale_grad,
    float4 *__restrict__ rec, int32_t *__restrict__ status) {
    __shared__ __align__(16) RecIn in[2];
    __shared__ __align__(16) float4 out[kRecVec * kRecTile];
    __shared__ __align__(8) uint64_t bar[2];
    const int t = threadIdx.x;
    if (t == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
    }
    __syncthreads();
    const float eps = *eps_scale_grad;
    int tile = blockIdx.x;
    if (t == 0 && tile < tiles) rec_issue_loads(in[0], &bar[0], tile, live, scale, rotation, channels, l2w);
    int it = 0;
    bool timed_out = false;
    for (; tile < tiles; it++, tile += gridDim.x) {
        const int st = it & 1;
        const int next = tile + gridDim.x;
        if (t == 0 && next < tiles) {
            fence_proxy_async();  // in[st ^ 1] was last read in the previous tile, before its barriers
            rec_issue_loads(in[st ^ 1], &bar[st ^ 1], next, live, scale, rotation, channels, l2w);
        }
        const bool ok = __syncthreads_and(mbar_wait(&bar[st], (uint32_t)(it >> 1) & 1u, kBulkWaitNs));
        if (!ok) {
            if (t == 0) atomicOr(status, GRAY_STATUS_COPY_TIMEOUT);
            timed_out = true;
            break;
        }
        float4 r[kRecVec];
        {
            const RecIn &x = in[st];
            const float ls[3] = {x.scale[3 * t], x.scale[3 * t + 1], x.scale[3 * t + 2]};
            const float ch[3] = {x.channels[3 * t], x.channels[3 * t + 1], x.channels[3 * t + 2]};
            bwd_record_one(x.live[t], ls, x.rotation[t], ch, x.l2w[3 * t], x.l2w[3 * t + 1], x.l2w[3 * t + 2], eps,
                           r);
        }
        if (t == 0) bulk_wait_read();  // the previous tile's store has read the output copy
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kRecVec; k++) out[kRecVec * t + k] = r[k];
        fence_proxy_async();
        __syncthreads();
        if (t == 0) {
            bulk_store(rec + kRecVec * (size_t)tile * kRecTile, out, 16u * kRecVec * kRecTile);
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

// What one composited hit reads: the snapshot rows and the backward record (9 x 16 B).
struct BwdHit {
    float4 g0, g1, g2, r0, r1, r2, r3, r4, r5;
};

__device__ __forceinline__ void load_hit(const BwdArgs &a, uint32_t gid, BwdHit &h) {
    const float4 *gp = a.geom + 3 * (size_t)gid, *rp = a.rec + kRecVec * (size_t)gid;
    h.g0 = __ldg(gp);
    h.g1 = __ldg(gp + 1);
    h.g2 = __ldg(gp + 2);
    h.r0 = __ldg(rp);
    h.r1 = __ldg(rp + 1);
    h.r2 = __ldg(rp + 2);
    h.r3 = __ldg(rp + 3);
    h.r4 = __ldg(rp + 4);
    h.r5 = __ldg(rp + 5);
}

// Reverse-order walk of a pixel's segment chain (newest segment first, each segment back to front).
struct HitCursor {
    uint32_t seg, prev;
    int e, guard;
};

// Next composited gaussian id; false at the end of the list or on a corrupt list (status raised).
__device__ __forceinline__ bool next_gid(const BwdArgs &a, HitCursor &c, uint32_t &gid) {
    for (;;) {
        while (c.e >= 0) {
            gid = a.pool[c.seg + 2u + (uint32_t)c.e];
            c.e--;
            if (gid < (uint32_t)a.n) return true;
        }
        if (c.prev == GRAY_NULL) return false;
        c.seg = c.prev;
        if (c.seg + 2u > a.pool_size || ++c.guard > kPassSlots * kMaxPasses + 1) {
            raise_status(a.status, GRAY_STATUS_HITLIST_OVERFLOW);
            return false;
        }
        c.prev = a.pool[c.seg];
        const uint32_t cnt = a.pool[c.seg + 1];
        if (cnt > a.pool_size - c.seg - 2u) {
            raise_status(a.status, GRAY_STATUS_HITLIST_OVERFLOW);
            return false;
        }
        c.e = (int)cnt - 1;
    }
}

// Pixel-constant inputs of the replay.
struct BwdPixel {
    f3 ro, rd, gout;
    float Tfin, fT, dbg, drem, inv_npix, pw;
};

// One step of the reverse replay (cuda/backward_pass.cu:17-137) for hit h; T and gT are the
// running transmittance and colour-gradient tail.
__device__ __forceinline__ void replay_hit(const BwdArgs &a, const BwdPixel &px, uint32_t gid, const BwdHit &h,
                                           float &T, float &gT) {
    const float o = h.r0.x, sf = h.r0.y, iq = h.r0.z;
    const f3 s = mk3(h.r0.w, h.r1.x, h.r1.y);
    const f3 c = mk3(h.r1.z, h.r1.w, h.r2.x);
    LocalHit lh;
    local_ray(h.g0, h.g1, h.g2, px.ro, px.rd, lh);
    closest_point(lh);
    const f3 x = mk3(lh.u.x * sf, lh.u.y * sf, lh.u.z * sf);
    const float sq = fdot3(x, x);
    const float gv = eval_gaussian(sq, px.pw);
    const float alpha = maxalpha_mul(gv, o);

    // one reciprocal of (1 - alpha) instead of four divisions (the reference divides each time,
    // cuda/backward_pass.cu:51-59,141); the gradients differ from it by rounding only
    const float om = 1.0f - alpha;
    const float rom = 1.0f / om;
    const float Tr = T * rom;
    const float w = Tr * alpha;
    const float dgc = dot3(px.gout, c);
    float ga = (dgc - gT) * Tr;
    ga = ga + -(px.fT * rom) * px.dbg;
    ga = ga + -((px.Tfin - px.fT) * rom) * px.drem;
    gT = gT + (dgc - gT) * alpha;
    float go = maxalpha_mul(ga, gv);
    go = go * o * (1.0f - o);
    const float ggv = maxalpha_mul(ga, o);
    float gsq;
    if (px.pw == 1.0f) gsq = gv;
    else if (px.pw == 2.0f) gsq = gv * sq;
    else if (px.pw == 3.0f) gsq = gv * sq * sq;
    else gsq = gv * gpow(sq, px.pw - 1.0f);
    const f3 gxl = mk3(-x.x * gsq * ggv, -x.y * gsq * ggv, -x.z * gsq * ggv);
    const f3 gxw = mk3((h.g0.x * gxl.x + h.g1.x * gxl.y + h.g2.x * gxl.z) * sf,
                       (h.g0.y * gxl.x + h.g1.y * gxl.y + h.g2.y * gxl.z) * sf,
                       (h.g0.z * gxl.x + h.g1.z * gxl.y + h.g2.z * gxl.z) * sf);
    // d loss / d L2W rows: -gxw_r * x
    const f3 gl0 = mk3(-gxw.x * x.x, -gxw.x * x.y, -gxw.x * x.z);
    const f3 gl1 = mk3(-gxw.y * x.x, -gxw.y * x.y, -gxw.y * x.z);
    const f3 gl2 = mk3(-gxw.z * x.x, -gxw.z * x.y, -gxw.z * x.z);
    const f3 gs = mk3(gl0.x * h.r2.y + gl1.x * h.r3.x + gl2.x * h.r3.w,
                      gl0.y * h.r2.z + gl1.y * h.r3.y + gl2.y * h.r4.x,
                      gl0.z * h.r2.w + gl1.z * h.r3.z + gl2.z * h.r4.y);
    // rotation-matrix gradient and its pull-back to the quaternion through the normalisation
    const float r00 = gl0.x * s.x, r01 = gl0.y * s.y, r02 = gl0.z * s.z;
    const float r10 = gl1.x * s.x, r11 = gl1.y * s.y, r12 = gl1.z * s.z;
    const float r20 = gl2.x * s.x, r21 = gl2.y * s.y, r22 = gl2.z * s.z;
    const float qw = h.r5.x, qx = h.r5.y, qy = h.r5.z, qz = h.r5.w;
    const float g_r = 2.0f * qx * (r21 - r12) + 2.0f * qy * (r02 - r20) + 2.0f * qz * (r10 - r01);
    const float g_x = -4.0f * qx * (r11 + r22) + 2.0f * qy * (r01 + r10) + 2.0f * qz * (r02 + r20) +
                      2.0f * qw * (r21 - r12);
    const float g_y = 2.0f * qx * (r01 + r10) - 4.0f * qy * (r00 + r22) + 2.0f * qz * (r12 + r21) +
                      2.0f * qw * (r02 - r20);
    const float g_z = 2.0f * qx * (r02 + r20) + 2.0f * qy * (r12 + r21) - 4.0f * qz * (r00 + r11) +
                      2.0f * qw * (r10 - r01);
    // (g - (g . qn) qn) / |q| == g / |q| - (g . q) q / |q|^3 (cuda/utils/activations.cu:68-70)
    const float dq = g_r * qw + g_x * qx + g_y * qy + g_z * qz;
    float v[16] = {(g_r - dq * qw) * iq, (g_x - dq * qx) * iq, (g_y - dq * qy) * iq, (g_z - dq * qz) * iq,
                   -gxw.x, -gxw.y, -gxw.z, go, gs.x, gs.y, gs.z, w * px.inv_npix,
                   px.gout.x * w, px.gout.y * w, px.gout.z * w, 1.0f};
    reduce_hit(a.grad_acc + 16 * (size_t)gid, gid, v);
    T = Tr;
}

// One thread per pixel walks its composited hits back to front (16x8-pixel blocks of four 8x4-pixel
// warps: neighbouring pixels composite the same Gaussians, which the lanes combine cheaply).
__global__ void __launch_bounds__(128) trace_backward_kernel(const BwdArgs a) {
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    const int px = blockIdx.x * 16 + (w & 1) * 8 + (l & 7);
    const int py = blockIdx.y * 8 + (w >> 1) * 4 + (l >> 3);
    if (px >= (int)a.render_w || py >= (int)a.render_h) return;
    const uint32_t pixel = (uint32_t)py * a.alloc_w + (uint32_t)px;
    HitCursor cur;
    cur.seg = a.head[pixel];
    if (cur.seg == GRAY_NULL) return;
    if (cur.seg + 2u > a.pool_size) {
        raise_status(a.status, GRAY_STATUS_HITLIST_OVERFLOW);
        return;
    }
    cur.prev = a.pool[cur.seg];
    {
        const uint32_t cnt = a.pool[cur.seg + 1];
        if (cnt > a.pool_size - cur.seg - 2u) {
            raise_status(a.status, GRAY_STATUS_HITLIST_OVERFLOW);
            return;
        }
        cur.e = (int)cnt - 1;
    }
    cur.guard = 1;
    BwdPixel P;
    P.pw = *a.exp_power;
    P.Tfin = a.pix_T[pixel];
    P.fT = a.pix_fullT[pixel];
    const f3 rem = mk3(a.pix_rem[3 * pixel], a.pix_rem[3 * pixel + 1], a.pix_rem[3 * pixel + 2]);
    P.ro = mk3(a.ray_o[3 * pixel], a.ray_o[3 * pixel + 1], a.ray_o[3 * pixel + 2]);
    P.rd = mk3(a.ray_d[3 * pixel], a.ray_d[3 * pixel + 1], a.ray_d[3 * pixel + 2]);
    P.gout = mk3(a.grad_out[3 * pixel], a.grad_out[3 * pixel + 1], a.grad_out[3 * pixel + 2]);
    const f3 bg = mk3(a.bg[0], a.bg[1], a.bg[2]);
    P.dbg = dot3(bg, P.gout);
    P.drem = dot3(rem, P.gout);
    P.inv_npix = 1.0f / (float)(a.render_w * a.render_h);
    float gT = 0.0f, T = P.Tfin;
    uint32_t gid;
    if (!next_gid(a, cur, gid)) return;
    do {
        BwdHit h;
        load_hit(a, gid, h);
        replay_hit(a, P, gid, h, T, gT);
    } while (next_gid(a, cur, gid));
}

cudaError_t launch_trace_backward(const gray_params &p, cudaStream_t s) {
    const int n = p.gaussians.count;
    if (n > 0) {
        const float2 *live = reinterpret_cast<const float2 *>(p.scene.live);
        const float4 *rot = reinterpret_cast<const float4 *>(p.gaussians.rotation);
        const float4 *l2w = reinterpret_cast<const float4 *>(p.scene.l2w);
        float4 *rec = reinterpret_cast<float4 *>(p.scene.bwd_rec);
        const bool bulk = p.status && aligned16(live) && aligned16(p.gaussians.scale) && aligned16(rot) &&
                          aligned16(p.gaussians.channels) && aligned16(l2w) && aligned16(rec);
        const int tiles = bulk ? n / kRecTile : 0;
        cudaError_t e;
        if (tiles > 0) {
            int dev = 0, sms = 0, per_sm = 0;
            if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
            if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
            if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bwd_record_bulk_kernel, kRecTile, 0)) !=
                cudaSuccess)
                return e;
            const int want = sms * (per_sm > 0 ? per_sm : 1);
            bwd_record_bulk_kernel<<<tiles < want ? tiles : want, kRecTile, 0, s>>>(
                tiles, live, p.gaussians.scale, rot, p.gaussians.channels, l2w, p.config.eps_scale_grad, rec,
                p.status);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
        }
        const int first = tiles * kRecTile;
        if (first < n)
            bwd_record_kernel<<<(unsigned int)((n - first + 255) / 256), 256, 0, s>>>(
                first, n, live, p.gaussians.scale, rot, p.gaussians.channels, l2w, p.config.eps_scale_grad, rec);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    BwdArgs a;
    a.alloc_w = p.image_width;
    a.render_w = p.render_width;
    a.render_h = p.render_height;
    a.n = n;
    a.exp_power = p.config.exp_power;
    a.alpha_threshold = p.config.alpha_threshold;
    a.eps_scale_grad = p.config.eps_scale_grad;
    a.bg = p.config.background_channels;
    a.geom = reinterpret_cast<const float4 *>(p.scene.geom);
    a.rec = reinterpret_cast<const float4 *>(p.scene.bwd_rec);
    a.pix_T = p.framebuffer.transmittance;
    a.pix_fullT = p.framebuffer.full_transmittance;
    a.pix_rem = p.framebuffer.remaining_channels_estimate;
    a.ray_o = p.framebuffer.ray_origin;
    a.ray_d = p.framebuffer.ray_direction;
    a.grad_out = p.framebuffer.grad_output_channels;
    a.head = p.hitlist.head_per_pixel;
    a.pool = p.hitlist.pool;
    a.pool_size = p.hitlist.size;
    a.grad_acc = p.scene.grad_acc;
    a.status = p.status;
    dim3 grid((p.render_width + 15) / 16, (p.render_height + 7) / 8);
    trace_backward_kernel<<<grid, 128, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace gray
