// gray_internal.h -- launchers shared between the translation units of libgray_gb300.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gray_gb300.h"

namespace gray {

// forward-kernel variant used when gray_params.trace_variant (or a batch launch's variant) is 0:
// 4x8 packets, 16-entry k-buffer, 6 blocks per SM
constexpr int kDefaultTraceVariant = 7;

// scene.cu
cudaError_t launch_snapshot(const gray_params &p, cudaStream_t s);
// reset_frame: zero was_visible, count the call and empty the backward hit list (forward_pass)
cudaError_t launch_forward_prep(const gray_params &p, bool reset_frame, cudaStream_t s);
cudaError_t launch_fold_and_sh_backward(const gray_params &p, cudaStream_t s);
// a wait on an mbarrier phase that never completes, which must give up and report
cudaError_t launch_copy_wait_selftest(int32_t *status, uint64_t limit_ns, cudaStream_t s);
cudaError_t launch_batch_prep(const gray_params &p, const float *origins, int nviews, float *channels_out,
                              cudaStream_t s);

// lbvh.cu
cudaError_t launch_lbvh_build(const gray_params &p, cudaStream_t s);
cudaError_t launch_lbvh_refit(const gray_params &p, cudaStream_t s);
// radix sort: a block sorts a tile of kSortThreads x kSortItems keys
constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;
// sort scratch of a rebuild of n Gaussians: second key and value buffers, then 256 digit counts
// per tile, then the 256 digit totals
constexpr size_t sort_tmp_words(int n) {
    return 2 * (size_t)n + 256 * (size_t)(n > 0 ? (n + kSortTile - 1) / kSortTile : 1) + 256;
}

// trace.cu
// display: forward_pass_display (colour only; no hit lists or saved state, whatever grads_enabled holds)
// the forward's tile schedule (per-tile work estimate and BVH frontier, densest-first order); it
// reads only the BVH and the camera, so it may run on another stream than forward_prep
bool trace_forward_has_schedule(const gray_params &p);
cudaError_t launch_trace_schedule(const gray_params &p, bool display, cudaStream_t s);
// schedule_ready: launch_trace_schedule has been issued for this forward (and ordered before s)
cudaError_t launch_trace_forward(const gray_params &p, bool display, bool schedule_ready, cudaStream_t s);
size_t gray_schedule_words_for(uint32_t width, uint32_t height);
// ellipsoid view; a no-op launch unless config.render_ellipsoids is set
cudaError_t launch_ellipsoids(const gray_params &p, bool display, cudaStream_t s);
cudaError_t launch_trace_backward(const gray_params &p, cudaStream_t s);
cudaError_t launch_trace_batch(const gray_batch_scene *scenes, const gray_batch_view *views, int nviews,
                               uint32_t total_packets, float *out, uint32_t *counter, uint32_t *frontier,
                               uint32_t total_groups, int variant, int blocks_per_sm, int32_t *status,
                               cudaStream_t s);

// adam.cu
cudaError_t launch_adam(const gray_params &p, cudaStream_t s);

// capi.cu: message returned by gray_last_error() on this thread
void set_last_error(const char *what);
// capi.cu: sets the message and returns GRAY_ERR_CUDA
int cuda_fail(cudaError_t e, const char *where);
// capi.cu: argument checks every entry point makes (params present, sizes within range)
int check_common(const gray_params *p);

// capi.cu: records CUDA events around a launcher on its stream while gray_profiler_enable is on
class ProfScope {
  public:
    ProfScope(const char *name, cudaStream_t s);
    ~ProfScope();

  private:
    int ev_;
    cudaStream_t s_;
};

// Run one launcher inside a profiler scope on stream `strm`; return its error from the enclosing
// entry point.  GRAY_LAUNCH uses the cudaStream_t named `s` in scope.
#define GRAY_LAUNCH_ON(name, strm, expr)                                   \
    do {                                                                   \
        cudaError_t _e;                                                    \
        {                                                                  \
            ::gray::ProfScope _ps(name, strm);                             \
            _e = (expr);                                                   \
        }                                                                  \
        if (_e != cudaSuccess) return ::gray::cuda_fail(_e, name);         \
    } while (0)
#define GRAY_LAUNCH(name, expr) GRAY_LAUNCH_ON(name, s, expr)

// noalloc.cu: unique id of the calling thread's current CUDA context (false when the driver
// cannot tell, or no context is current)
bool current_context_id(unsigned long long *id);

constexpr int kThreads = 256;
inline unsigned int blocks_for(long long n, int threads = kThreads) {
    return (unsigned int)((n + threads - 1) / threads);
}

}  // namespace gray
