// capi.cu -- extern "C" entry points of libgray_gb300.so (declared in include/gray_gb300.h).
//
// Each entry point is one method of the reference's torch-bound Raytracer
// (cuda/raytracer.h:88-149); it validates the caller's state, launches the kernels on the
// given stream and returns immediately (no host synchronisation, no allocation).
#include <cstdio>
#include <cstring>
#include <string>

#include "gray_internal.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const char *what) {
    g_last_error = what;
    return code;
}

int cuda_fail(cudaError_t e, const char *where) {
    g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
    return GRAY_ERR_CUDA;
}

#define GRAY_TRY(expr, where)                                \
    do {                                                     \
        cudaError_t _e = (expr);                             \
        if (_e != cudaSuccess) return cuda_fail(_e, where);  \
    } while (0)

bool frame_ok(const gray_params *p) {
    return p->render_width >= 1 && p->render_height >= 1 && p->render_width <= p->image_width &&
           p->render_height <= p->image_height;
}

int check_common(const gray_params *p) {
    if (!p) return fail(GRAY_ERR_INVALID_ARGUMENT, "null params");
    if (p->gaussians.count < 0) return fail(GRAY_ERR_INVALID_ARGUMENT, "negative Gaussian count");
    if (!frame_ok(p))
        return fail(GRAY_ERR_OUT_OF_RANGE, "render resolution must be positive and within the allocated framebuffer");
    if ((size_t)p->image_width * (size_t)p->image_height >= (size_t)0xFFFFFFFFu)
        return fail(GRAY_ERR_OUT_OF_RANGE, "framebuffer too large for 32-bit pixel ids");
    if (p->gaussians.count > 0x7FFFFFFF - 1 || (uint32_t)p->gaussians.count >= 0x80000000u)
        return fail(GRAY_ERR_OUT_OF_RANGE, "too many Gaussians");
    return GRAY_OK;
}

int check_trace(const gray_params *p) {
    int e = check_common(p);
    if (e) return e;
    if (p->gaussians.count > 0 && !p->scene.bvh_valid)
        return fail(GRAY_ERR_INVALID_ARGUMENT, "the BVH is stale: call rebuild_bvh after creating or resizing");
    if (!p->hitlist.head_per_pixel || !p->hitlist.pool || !p->hitlist.total_words)
        return fail(GRAY_ERR_INVALID_ARGUMENT, "missing backward hit list buffers");
    if (!p->framebuffer.output_channels || !p->scene.geom || !p->scene.live || !p->scene.nodes)
        return fail(GRAY_ERR_INVALID_ARGUMENT, "missing framebuffer or scene buffers");
    return GRAY_OK;
}

}  // namespace

extern "C" {

size_t gray_sort_tmp_words(int32_t n) { return gray::sort_tmp_words(n); }

int gray_forward_pass(const gray_params *p, void *stream) {
    int e = check_trace(p);
    if (e) return e;
    cudaStream_t s = (cudaStream_t)stream;
    GRAY_TRY(gray::launch_forward_prep(*p, true, s), "forward_prep");
    GRAY_TRY(gray::launch_trace_forward(*p, s), "trace_forward");
    return GRAY_OK;
}

int gray_forward_pass_display(const gray_params *p, void *stream) {
    int e = check_trace(p);
    if (e) return e;
    cudaStream_t s = (cudaStream_t)stream;
    GRAY_TRY(gray::launch_forward_prep(*p, false, s), "forward_prep");
    GRAY_TRY(gray::launch_trace_forward(*p, s), "trace_forward");
    return GRAY_OK;
}

int gray_backward_pass(const gray_params *p, void *stream) {
    int e = check_trace(p);
    if (e) return e;
    if (p->gaussians.sh_is_fp16) return fail(GRAY_ERR_INVALID_ARGUMENT, "backward_pass needs an inference_only=False raytracer");
    if (!p->scene.grad_acc || !p->gaussians.grad_mean)
        return fail(GRAY_ERR_INVALID_ARGUMENT, "missing gradient buffers");
    cudaStream_t s = (cudaStream_t)stream;
    GRAY_TRY(gray::launch_trace_backward(*p, s), "trace_backward");
    GRAY_TRY(gray::launch_fold_and_sh_backward(*p, s), "fold_sh_backward");
    return GRAY_OK;
}

int gray_step(const gray_params *p, void *stream) {
    int e = check_common(p);
    if (e) return e;
    if (p->gaussians.sh_is_fp16) return fail(GRAY_ERR_INVALID_ARGUMENT, "step needs an inference_only=False raytracer");
    if (!p->gaussians.first_moment_mean || !p->metadata.total_num_steps)
        return fail(GRAY_ERR_INVALID_ARGUMENT, "missing optimiser state");
    GRAY_TRY(gray::launch_adam(*p, (cudaStream_t)stream), "adam");
    return GRAY_OK;
}

int gray_update_bvh(const gray_params *p, void *stream) {
    int e = check_common(p);
    if (e) return e;
    if (p->gaussians.count > 0 && !p->scene.bvh_valid)
        return fail(GRAY_ERR_INVALID_ARGUMENT, "update_bvh before rebuild_bvh");
    cudaStream_t s = (cudaStream_t)stream;
    GRAY_TRY(gray::launch_snapshot(*p, s), "snapshot");
    GRAY_TRY(gray::launch_lbvh_refit(*p, s), "refit");
    return GRAY_OK;
}

int gray_rebuild_bvh(const gray_params *p, void *stream) {
    int e = check_common(p);
    if (e) return e;
    if (!p->scene.geom || !p->scene.nodes || !p->scene.sort_tmp)
        return fail(GRAY_ERR_INVALID_ARGUMENT, "missing scene workspace");
    cudaStream_t s = (cudaStream_t)stream;
    GRAY_TRY(gray::launch_snapshot(*p, s), "snapshot");
    GRAY_TRY(gray::launch_lbvh_build(*p, s), "lbvh_build");
    return GRAY_OK;
}

const char *gray_last_error(void) { return g_last_error.c_str(); }

const char *gray_version(void) { return "gray_gb300 0.1 (sm_103a)"; }

}  // extern "C"
