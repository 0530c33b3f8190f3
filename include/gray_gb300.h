/*
 * gray_gb300.h -- C ABI of the GB300-native Gaussian ray tracer (libgray_gb300.so).
 *
 * The library replaces the OptiX path behind GRay's torch binding
 * (graphdeco-inria/gray: cuda/raytracer.cpp:3-13 registers torch.classes.gray.Raytracer,
 * whose methods are defined in cuda/raytracer.h:88-149).  Every entry point here is one of
 * those methods, taking the same state the reference keeps in its `Params` block
 * (cuda/params.h:12-31): plain device pointers owned by the caller, image and scene sizes,
 * and the CUDA stream to run on.  No torch types cross this boundary.
 *
 * Conventions
 *  - All pointers in the structs are device pointers unless stated otherwise.  Runtime knobs
 *    are one-element device arrays read by the kernels, exactly like the reference's
 *    ConfigDataHolder tensors (cuda/core/config.h:5-22), so they can change without a host
 *    round trip.
 *  - `stream` is a cudaStream_t passed as void*; 0 selects the legacy default stream.
 *  - Return value: GRAY_OK or a GRAY_ERR_* code; gray_last_error() gives the message.
 *    Conditions that only the device can detect (hit-list overflow, traversal-stack overflow,
 *    an exhausted spin budget, a bulk-copy wait that ran out) are OR-ed into `*status` (a device
 *    int32) instead of trapping;
 *    the host reads it after synchronising.
 *  - Layouts follow the reference holders (cuda/core/gaussians.h:70-160): mean [N,3],
 *    rotation [N,4] (r,x,y,z, unnormalised), scale [N,3] (log), opacity [N,1] (logit),
 *    channels [N,3], sh_coeffs_dc [N,1,3], sh_coeffs_rest [N,K,3] (fp32, or fp16 when
 *    sh_is_fp16), framebuffer arrays [H_alloc, W_alloc, C].
 */
#ifndef GRAY_GB300_H
#define GRAY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GRAY_OK 0
#define GRAY_ERR_INVALID_ARGUMENT 1
#define GRAY_ERR_CUDA 2
#define GRAY_ERR_OUT_OF_RANGE 3

/* bits of the device status word */
#define GRAY_STATUS_HITLIST_OVERFLOW 1    /* backward hit list full (reference: PPLL overflow __trap) */
#define GRAY_STATUS_STACK_OVERFLOW 2      /* BVH traversal stack exhausted */
#define GRAY_STATUS_REFIT_TIMEOUT 4       /* bottom-up refit spin budget exhausted */
#define GRAY_STATUS_BAD_MODE 8            /* render_ellipsoids set on a forward with gradients enabled
                                             (reference: assertion, gray/raytracer.py:142-144) */
#define GRAY_STATUS_COPY_TIMEOUT 16       /* a bulk (TMA) copy of a streaming kernel did not complete
                                             within its wait limit; the kernel stopped early */

/* Gaussian parameters and optimiser state (cuda/core/gaussians.h:7-65). */
typedef struct gray_gaussians {
    int32_t count;
    int32_t max_sh_degree;
    int32_t num_sh_coeffs;        /* (max_sh_degree + 1)^2 - 1 */
    int32_t sh_is_fp16;           /* inference_only: SH stored as binary16 */
    int32_t *current_sh_degree;   /* [1] */

    float *mean, *rotation, *scale, *opacity, *channels;
    void *sh_coeffs_dc, *sh_coeffs_rest;

    float *lr_mean, *lr_rotation, *lr_scale, *lr_opacity, *lr_channels, *lr_sh_dc, *lr_sh_rest; /* [0] read */
    float *beta_1, *beta_2, *epsilon;
    int32_t *sh_update_laziness;

    float *grad_mean, *grad_rotation, *grad_scale, *grad_opacity, *grad_channels, *grad_sh_coeffs_dc,
        *grad_sh_coeffs_rest;
    float *first_moment_mean, *first_moment_rotation, *first_moment_scale, *first_moment_opacity,
        *first_moment_channels, *first_moment_sh_coeffs_dc, *first_moment_sh_coeffs_rest;
    float *second_moment_mean, *second_moment_rotation, *second_moment_scale, *second_moment_opacity,
        *second_moment_channels, *second_moment_sh_coeffs_dc, *second_moment_sh_coeffs_rest;

    float *pruning_weight;
    int32_t *pruning_counter;
    uint8_t *was_visible;
    float *marked;
} gray_gaussians;

/* Pinhole camera (cuda/core/camera.h:8-15); rotation_w2c rows are the c2w columns. */
typedef struct gray_camera {
    float *origin;               /* [3] */
    float *vertical_fov_radians; /* [1] */
    float *rotation_c2w;         /* [3,3] */
    float *rotation_w2c;         /* [3,3] */
    float *znear, *zfar;         /* [1] each */
} gray_camera;

/* Runtime knobs (cuda/core/config.h:5-22); every field is a one-element device array. */
typedef struct gray_config {
    float *exp_power, *alpha_threshold, *t_threshold;
    uint8_t *jitter_primary_rays;
    float *global_scale_factor, *eps_forward_normalization, *eps_scale_grad;
    float *background_channels; /* [3] */
    uint8_t *render_depth, *render_ellipsoids;
    float *ellipsoid_min_opacity;
    uint8_t *rays_from_python, *zero_grads, *enable_sh, *needs_ray_output, *update_channels;
} gray_config;

/* Per-pixel outputs and saved state (cuda/core/framebuffer.h:22-31). */
typedef struct gray_framebuffer {
    float *output_channels;            /* [H,W,3] */
    float *output_depth;               /* [H,W,1] */
    float *transmittance;              /* [H,W,1] */
    float *full_transmittance;         /* [H,W,1] */
    float *remaining_channels_estimate;/* [H,W,3] */
    float *ray_origin, *ray_direction; /* [H,W,3] */
    float *grad_output_channels;       /* [H,W,3] */
} gray_framebuffer;

/* cuda/core/metadata.h:3-10 */
typedef struct gray_metadata {
    uint8_t *run_forward_pass, *run_backward_pass, *grads_enabled;
    uint32_t *total_num_calls, *total_num_steps;
} gray_metadata;

/* cuda/core/stats.h:3-6 (per-pixel counters, accumulated while grads are enabled) */
typedef struct gray_stats {
    int32_t *num_gaussians_hit, *num_gaussians_accumulated;
} gray_stats;

/* Backward hit list (replaces the reference's backward per-pixel linked list,
 * cuda/core/per_pixel_linked_list.h:5-62).  Composited gaussian ids are stored per pixel as
 * a chain of segments [prev_segment, count, id_0 .. id_{count-1}] in `pool` (u32 words);
 * head_per_pixel holds the newest segment of each pixel (0xFFFFFFFF = none). */
typedef struct gray_hitlist {
    uint32_t *head_per_pixel; /* [H_alloc * W_alloc] */
    uint32_t *total_words;    /* [1] bump counter */
    uint32_t *pool;           /* [size] */
    uint32_t size;
    uint32_t *schedule;       /* [gray_schedule_words(W_alloc, H_alloc)] work order of the forward's
                                 pixel tiles (dense tiles first), each tile's BVH frontier and the
                                 coarse frontiers of 4x4-tile super-tiles that seed the tiles' walks;
                                 NULL: tiles in launch order, traversals from the root */
} gray_hitlist;

/* Scene-side workspace owned by the caller (sizes in the comments; sort_tmp from gray_sort_tmp_words). */
typedef struct gray_scene {
    float *geom;        /* [N,12] snapshot rows (M | mu), M = diag(1/s) R^T          */
    float *l2w;         /* [N,12] snapshot rows (L | mu), L = R diag(s)               */
    float *aabb;        /* [N,8]  leaf boxes (min xyz, pad, max xyz, pad)             */
    uint8_t *visible;   /* [N]    snapshot visibility (populate_bvh_kernel mask)      */
    float *live;        /* [N,2]  per-forward (sigmoid(opacity), scaling factor)      */
    float *grad_acc;    /* [N,16] backward accumulators, zero between passes          */
    float *nodes;       /* [max(N-1,1),16] BVH2 nodes: child boxes + child links      */
    int32_t *int_parent;  /* [max(N-1,1)] parent of each internal node, with bit 30 set when the
                             node is its parent's second child; -1 for the root */
    int32_t *leaf_parent; /* [N] indexed by sorted leaf position, same encoding */
    uint32_t *order;      /* [N] sorted leaf position -> gaussian id */
    uint32_t *codes;      /* [N] Morton codes in sorted order */
    uint32_t *refit_flags;/* [max(N-1,1)] */
    uint32_t *sort_tmp;   /* [sort_tmp_words] radix-sort scratch of a rebuild; a refit queues the
                             upper tree's first nodes in it (may be NULL for gray_update_bvh: the
                             refit then climbs the whole tree with global counters, slower) */
    float *root_box;      /* [8] */
    uint32_t *bounds;     /* [8] order-preserving encoded scene bounds (scratch) */
    float *bwd_rec;       /* [N,24] per-Gaussian backward record, written at the start of each
                             backward pass (training tracers; may be NULL for inference) */
    int32_t bvh_valid;    /* host flag: a rebuild has been done for this count */
} gray_scene;

typedef struct gray_params {
    uint32_t image_width, image_height;   /* allocated framebuffer */
    uint32_t render_width, render_height; /* active top-left rectangle (set_render_resolution) */
    gray_camera camera;
    gray_config config;
    gray_framebuffer framebuffer;
    gray_gaussians gaussians;
    gray_metadata metadata;
    gray_stats stats;
    gray_hitlist hitlist;
    gray_scene scene;
    int32_t *status; /* device int32, GRAY_STATUS_* bits */
    /* forward-trace kernel variant: bits 0-1 = physical hit buffer of 32 or 16 keys and register
     * cap, bit 2 = 8x4 or 4x8 pixel packets, bits 3-4 = where a pixel tile's traversals start (BVH
     * nodes of at most 64, 32 or 128 leaves that the tile's frustum reaches, or the root), bit 5 =
     * how the scheduled launch hands out work (one pixel tile per block, or one packet per warp).
     * 0 (default): 4x8 packets from 64-leaf frontiers, with the 16-key buffer (six blocks per SM)
     * or the 32-key one (four blocks per SM) chosen on the device from the previous scheduled
     * forward of the same schedule buffer (the 32-key one when more than 1/8 of its packets
     * traversed more than once); both kernels are launched and the one not chosen returns at once.
     * Results are identical for every variant; only speed differs. */
    int32_t trace_variant;
} gray_params;

/* ---- batched rendering (many views, one persistent launch) ----
 * No reference counterpart: the reference renders one view per OptiX launch
 * (cuda/raytracer.h:104-114 forward_pass_display).  A batch renders any number of views of one or
 * several resident scenes, each at its own resolution, forward only (inference), in one launch
 * whose warps pull 32-ray packets from a global counter.  Per pixel the result is bit-identical to
 * gray_forward_pass_display of the same view. */
typedef struct gray_batch_scene {
    const float *geom, *live, *nodes, *root_box; /* a scene's gray_scene buffers after rebuild/update */
    const float *l2w;                            /* its gray_scene.l2w (may be NULL: no leaf culling) */
    int32_t n;                                   /* Gaussian count */
    float exp_power, alpha_threshold, t_threshold;
    float bg[3];
    int32_t pad;
} gray_batch_scene;

typedef struct gray_batch_view {
    float origin[3];
    float w2c[9];          /* rows = camera axes (rotation_w2c of CameraDataHolder) */
    float fov_y, znear, zfar;
    uint32_t width, height;
    uint32_t scene;        /* index into the scene table */
    uint32_t packet_offset;/* first packet of this view; views in increasing order */
    uint32_t group_offset; /* first frontier group of this view (gray_batch_groups); increasing */
    uint64_t out_offset;   /* float index of pixel (0,0): RGB, row-major, width x height */
    const float *channels; /* [n,3] colours of the view's scene for this view (gray_batch_prep) */
} gray_batch_view;

/* Packets (32-ray tiles) of a width x height view for a kernel variant. */
uint32_t gray_batch_packets(uint32_t width, uint32_t height, int32_t variant);

/* Frontier groups (2x2 packets) of a width x height view for a kernel variant; a batch's frontier
 * buffer holds GRAY_FRONTIER_WORDS words per group of all its views. */
uint32_t gray_batch_groups(uint32_t width, uint32_t height, int32_t variant);
#define GRAY_FRONTIER_WORDS 161
uint32_t gray_frontier_words(void);

/* Per-view colours of one scene: live values (as forward_pass_display) and, when enable_sh, the SH
 * colour of every Gaussian for each of the nviews camera origins (device [nviews,3]) into
 * channels_out (device [nviews,n,3]); without SH the scene's channels are copied per view. */
int gray_batch_prep(const gray_params *p, const float *origins, int32_t nviews, float *channels_out, void *stream);

/* Render the views (device arrays scenes[], views[]) into out; work_counter is one device word
 * the launch resets and consumes; frontier is a device workspace of total_groups *
 * GRAY_FRONTIER_WORDS words (NULL: every traversal starts at the root) into which the launch first
 * writes each packet group's BVH frontier (a group index at or beyond total_groups, from an
 * inconsistent group_offset, starts at the root); variant as gray_params.trace_variant;
 * blocks_per_sm sizes the persistent grid (0 = 4). */
int gray_render_batch(const gray_batch_scene *scenes, const gray_batch_view *views, int32_t nviews,
                      uint32_t total_packets, float *out, uint32_t *work_counter, uint32_t *frontier,
                      uint32_t total_groups, int32_t variant, int32_t blocks_per_sm, int32_t *status,
                      void *stream);

/* Workspace sizes in 32-bit words for n Gaussians: sort_tmp_words. */
size_t gray_sort_tmp_words(int32_t n);

/* Words of gray_hitlist.schedule for a width x height framebuffer (no counterpart in the reference:
 * the forward estimates each pixel tile's work from the BVH, runs the densest tiles first and starts
 * each tile's traversals at the BVH nodes the tile's frustum reaches). */
size_t gray_schedule_words(uint32_t width, uint32_t height);

/* Raytracer::forward_pass (cuda/raytracer.h:88-102): counts the call, resets the backward
 * hit list and was_visible, evaluates SH colours (if enable_sh) and traces the render
 * rectangle.  grads_enabled must have been set by the caller (MetaDataHolder::update). */
int gray_forward_pass(const gray_params *p, void *stream);

/* Raytracer::forward_pass_display (cuda/raytracer.h:104-114): SH + trace, no resets. */
int gray_forward_pass_display(const gray_params *p, void *stream);

/* Raytracer::backward_pass (cuda/raytracer.h:116-124): reverse replay of the hit lists into the
 * gradient arrays (and pruning_weight, was_visible), then the SH backward. */
int gray_backward_pass(const gray_params *p, void *stream);

/* Raytracer::step (cuda/raytracer.h:126-133 -> cuda/opt/adam.cu:70-83): total_num_steps += 1
 * and one fused Adam step over all parameter groups (SH every sh_update_laziness steps). */
int gray_step(const gray_params *p, void *stream);

/* Raytracer::update_bvh (cuda/raytracer.h:135 -> cuda/optix/bvh_wrapper.h:25-39): snapshot the
 * current parameters into the instance records and refit the hierarchy's boxes. */
int gray_update_bvh(const gray_params *p, void *stream);

/* Raytracer::rebuild_bvh (cuda/raytracer.h:137-142 -> cuda/optix/bvh_wrapper.h:89-115): snapshot
 * and full LBVH build (Morton codes, radix sort, Karras hierarchy, bottom-up boxes). */
int gray_rebuild_bvh(const gray_params *p, void *stream);

/* Optional timing of every launch made by the entry points above, with CUDA events recorded
 * on the caller's stream around each kernel group (forward_prep, trace_forward, trace_backward,
 * fold_sh_backward, adam, snapshot, refit, lbvh_build).  No reference counterpart: profiling
 * support for the benchmark harness.  enable(1, capacity) pre-creates 2*capacity events and
 * clears the records; enable(0, 0) stops recording.  collect() waits for the recorded events,
 * writes "name total_ms launches\n" lines into buf and clears the records; it returns the
 * length of the full text, or minus a GRAY_ERR_* code.  Not thread-safe; not for use inside stream capture. */
int gray_profiler_enable(int on, int capacity);
int gray_profiler_collect(char *buf, size_t buflen);

/* Raytracer::rebuild_bvh without caller-provided scratch.  No counterpart in the reference: an
 * addition for callers that cannot allocate device memory (a host that owns the whole device
 * budget, such as an engine or viewer plugin, or a point in its code where its allocator must
 * not be entered).  Same outputs as gray_rebuild_bvh (snapshot records, nodes, parents, order,
 * codes, root box, all in p->scene); p->scene.sort_tmp, .bounds and .refit_flags are ignored
 * and may be NULL.  The scratch is a fixed device array inside the library, sized for at most
 * GRAY_STATIC_MAX_GAUSSIANS Gaussians (about 3.3 MB, held by every device that loads the
 * library until the process exits); larger counts return GRAY_ERR_OUT_OF_RANGE.  The first call
 * in each CUDA context (the device's primary context, or a driver-API context the caller made
 * current) looks up that array's device address in that context (cudaGetSymbolAddress) and
 * caches it under the context's id, so make the first call before any stream capture; a
 * context re-created after cudaDeviceReset gets its own look-up.  Every call shares the one
 * array: calls whose work overlaps on the GPU (other streams, other threads) race and must be
 * serialised by the caller.  No allocation of any kind is made.  A later gray_update_bvh still
 * needs the caller's scene.refit_flags (one visit counter per internal node): the array is the
 * rebuild's only. */
#define GRAY_STATIC_MAX_GAUSSIANS 262144
int gray_rebuild_bvh_static(const gray_params *p, void *stream);

/* Self-test of the bounded copy wait that the streaming kernels use (no reference counterpart:
 * failure detection without a GPU fault).  One block announces 16 bytes on an mbarrier phase and
 * copies nothing, so the phase never completes; the wait gives up after limit_ns nanoseconds
 * (at most 2 s), sets GRAY_STATUS_COPY_TIMEOUT in *status and the kernel returns.  Nothing else is
 * read or written. */
int gray_selftest_copy_wait(int32_t *status, uint64_t limit_ns, void *stream);

/* Message of the last error returned on the calling thread. */
const char *gray_last_error(void);

/* Library version string. */
const char *gray_version(void);

#ifdef __cplusplus
}
#endif
#endif
