// capi.cu -- extern "C" entry points of libgray_gb300.so (declared in include/gray_gb300.h).
//
// Each entry point is one method of the reference's torch-bound Raytracer
// (cuda/raytracer.h:88-149); it validates the caller's state, launches the kernels on the
// given stream and returns immediately (no host synchronisation, no device allocation; the forward
// entry points make one side stream and two events per host thread and context on first use).
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gray_internal.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const char *what) {
    g_last_error = what;
    return code;
}

bool frame_ok(const gray_params *p) {
    return p->render_width >= 1 && p->render_height >= 1 && p->render_width <= p->image_width &&
           p->render_height <= p->image_height;
}

int check_common_impl(const gray_params *p) {
    if (!p) return fail(GRAY_ERR_INVALID_ARGUMENT, "null params");
    if (p->gaussians.count < 0) return fail(GRAY_ERR_INVALID_ARGUMENT, "negative Gaussian count");
    if (!frame_ok(p))
        return fail(GRAY_ERR_OUT_OF_RANGE, "render resolution must be positive and within the allocated framebuffer");
    if ((size_t)p->image_width * (size_t)p->image_height >= (size_t)0xFFFFFFFFu)
        return fail(GRAY_ERR_OUT_OF_RANGE, "framebuffer too large for 32-bit pixel ids");
    if (p->gaussians.count > (1 << 30))  // the BVH's parent words keep bit 30 for a flag
        return fail(GRAY_ERR_OUT_OF_RANGE, "too many Gaussians (at most 2^30)");
    return GRAY_OK;
}

int check_trace(const gray_params *p) {
    int e = check_common_impl(p);
    if (e) return e;
    if (p->gaussians.count > 0 && !p->scene.bvh_valid)
        return fail(GRAY_ERR_INVALID_ARGUMENT, "the BVH is stale: call rebuild_bvh after creating or resizing");
    if (!p->hitlist.head_per_pixel || !p->hitlist.pool || !p->hitlist.total_words)
        return fail(GRAY_ERR_INVALID_ARGUMENT, "missing backward hit list buffers");
    if (!p->framebuffer.output_channels || !p->scene.geom || !p->scene.live || !p->scene.nodes)
        return fail(GRAY_ERR_INVALID_ARGUMENT, "missing framebuffer or scene buffers");
    return GRAY_OK;
}

// ---- optional per-launch timing (CUDA events on the launching stream) ----
struct ProfRecord {
    const char *name;
    int ev;  // index of the start event; stop is ev + 1
};
bool g_prof_on = false;
std::vector<cudaEvent_t> g_prof_events;
std::vector<ProfRecord> g_prof_records;

}  // namespace

namespace gray {

void set_last_error(const char *what) { g_last_error = what; }

int cuda_fail(cudaError_t e, const char *where) {
    g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
    return GRAY_ERR_CUDA;
}

int check_common(const gray_params *p) { return check_common_impl(p); }

ProfScope::ProfScope(const char *name, cudaStream_t s) : ev_(-1), s_(s) {
    if (!g_prof_on) return;
    const int ev = (int)g_prof_records.size() * 2;
    if (ev + 1 >= (int)g_prof_events.size()) return;  // pool exhausted: stop recording rather than allocate
    g_prof_records.push_back(ProfRecord{name, ev});
    ev_ = ev;
    cudaEventRecord(g_prof_events[ev], s_);
}

ProfScope::~ProfScope() {
    if (ev_ >= 0) cudaEventRecord(g_prof_events[ev_ + 1], s_);
}

}  // namespace gray

using gray::check_common;
using gray::cuda_fail;

namespace {

// The calling thread's second stream in one CUDA context, with a fork and a join event; made on first
// use in that context (highest priority: the forward's tile schedule, which it carries, is on the
// critical path) and released when the thread exits.
struct SideStream {
    unsigned long long ctx;
    cudaStream_t s;
    cudaEvent_t fork, join;
};
struct SideStreams {
    std::vector<SideStream> v;
    ~SideStreams() {
        // work still queued on a stream completes before its resources go; a context already
        // torn down (process exit, cudaDeviceReset) only makes these calls return an error
        for (const SideStream &x : v) {
            cudaEventDestroy(x.fork);
            cudaEventDestroy(x.join);
            cudaStreamDestroy(x.s);
        }
    }
};
thread_local SideStreams t_side;

// false when no side stream can be had (no context id, or a creation failed): run serially
bool side_stream(SideStream *out) {
    unsigned long long id = 0;
    if (!gray::current_context_id(&id)) return false;
    for (const SideStream &x : t_side.v)
        if (x.ctx == id) {
            *out = x;
            return true;
        }
    SideStream x{id, nullptr, nullptr, nullptr};
    int lo = 0, hi = 0;
    bool ok = cudaDeviceGetStreamPriorityRange(&lo, &hi) == cudaSuccess &&
              cudaStreamCreateWithPriority(&x.s, cudaStreamNonBlocking, hi) == cudaSuccess &&
              cudaEventCreateWithFlags(&x.fork, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&x.join, cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        if (x.fork) cudaEventDestroy(x.fork);
        if (x.s) cudaStreamDestroy(x.s);
        cudaGetLastError();  // leave no stale error for the launches that follow
        return false;
    }
    t_side.v.push_back(x);
    *out = x;
    return true;
}

// forward_prep (live values, colours) and the tile schedule (per-tile BVH frontier and work order,
// from the BVH and the camera only) read and write disjoint state: the schedule runs on the side
// stream between a fork and a join event while forward_prep runs on s, and the trace follows both.
int forward(const gray_params *p, bool display, cudaStream_t s) {
    SideStream side;
    const bool overlap = gray::trace_forward_has_schedule(*p) && side_stream(&side);
    if (overlap) {
        cudaError_t e;
        if ((e = cudaEventRecord(side.fork, s)) != cudaSuccess) return cuda_fail(e, "fork");
        if ((e = cudaStreamWaitEvent(side.s, side.fork, 0)) != cudaSuccess) return cuda_fail(e, "fork");
        GRAY_LAUNCH_ON("tile_schedule", side.s, gray::launch_trace_schedule(*p, display, side.s));
        if ((e = cudaEventRecord(side.join, side.s)) != cudaSuccess) return cuda_fail(e, "join");
    }
    GRAY_LAUNCH("forward_prep", gray::launch_forward_prep(*p, !display, s));
    if (overlap) {
        cudaError_t e = cudaStreamWaitEvent(s, side.join, 0);
        if (e != cudaSuccess) return cuda_fail(e, "join");
    }
    GRAY_LAUNCH("trace_forward", gray::launch_trace_forward(*p, display, overlap, s));
    GRAY_LAUNCH("ellipsoids", gray::launch_ellipsoids(*p, display, s));
    return GRAY_OK;
}

}  // namespace

extern "C" {

int gray_profiler_enable(int on, int capacity) {
    if (on) {
        if ((int)g_prof_events.size() < 2 * capacity) {
            for (int i = (int)g_prof_events.size(); i < 2 * capacity; i++) {
                cudaEvent_t e;
                cudaError_t err = cudaEventCreate(&e);
                if (err != cudaSuccess) return cuda_fail(err, "profiler event");
                g_prof_events.push_back(e);
            }
        }
        g_prof_records.clear();
    }
    g_prof_on = on != 0;
    return GRAY_OK;
}

int gray_profiler_collect(char *buf, size_t buflen) {
    // per launcher name: total milliseconds and launch count
    std::vector<std::pair<std::string, std::pair<double, int>>> agg;
    for (const ProfRecord &r : g_prof_records) {
        cudaError_t err = cudaEventSynchronize(g_prof_events[r.ev + 1]);
        if (err != cudaSuccess) return -cuda_fail(err, "profiler sync");
        float ms = 0.0f;
        err = cudaEventElapsedTime(&ms, g_prof_events[r.ev], g_prof_events[r.ev + 1]);
        if (err != cudaSuccess) return -cuda_fail(err, "profiler elapsed");
        bool found = false;
        for (auto &a : agg)
            if (a.first == r.name) {
                a.second.first += ms;
                a.second.second += 1;
                found = true;
            }
        if (!found) agg.push_back({r.name, {ms, 1}});
    }
    std::string out;
    for (auto &a : agg) {
        char line[160];
        snprintf(line, sizeof(line), "%s %.6f %d\n", a.first.c_str(), a.second.first, a.second.second);
        out += line;
    }
    if (buf && buflen) {
        strncpy(buf, out.c_str(), buflen - 1);
        buf[buflen - 1] = 0;
    }
    g_prof_records.clear();
    return (int)out.size();
}

size_t gray_sort_tmp_words(int32_t n) { return gray::sort_tmp_words(n); }

size_t gray_schedule_words(uint32_t width, uint32_t height) { return gray::gray_schedule_words_for(width, height); }

int gray_forward_pass(const gray_params *p, void *stream) {
    int e = check_trace(p);
    if (e) return e;
    return forward(p, false, (cudaStream_t)stream);
}

int gray_forward_pass_display(const gray_params *p, void *stream) {
    int e = check_trace(p);
    if (e) return e;
    return forward(p, true, (cudaStream_t)stream);
}

int gray_backward_pass(const gray_params *p, void *stream) {
    int e = check_trace(p);
    if (e) return e;
    if (p->gaussians.sh_is_fp16) return fail(GRAY_ERR_INVALID_ARGUMENT, "backward_pass needs an inference_only=False raytracer");
    if (!p->scene.grad_acc || !p->scene.bwd_rec || !p->gaussians.grad_mean)
        return fail(GRAY_ERR_INVALID_ARGUMENT, "missing gradient buffers");
    cudaStream_t s = (cudaStream_t)stream;
    GRAY_LAUNCH("trace_backward", gray::launch_trace_backward(*p, s));
    GRAY_LAUNCH("fold_sh_backward", gray::launch_fold_and_sh_backward(*p, s));
    return GRAY_OK;
}

int gray_step(const gray_params *p, void *stream) {
    int e = check_common(p);
    if (e) return e;
    if (p->gaussians.sh_is_fp16) return fail(GRAY_ERR_INVALID_ARGUMENT, "step needs an inference_only=False raytracer");
    if (!p->gaussians.first_moment_mean || !p->metadata.total_num_steps)
        return fail(GRAY_ERR_INVALID_ARGUMENT, "missing optimiser state");
    cudaStream_t s = (cudaStream_t)stream;
    GRAY_LAUNCH("adam", gray::launch_adam(*p, s));
    return GRAY_OK;
}

int gray_update_bvh(const gray_params *p, void *stream) {
    int e = check_common(p);
    if (e) return e;
    if (p->gaussians.count > 0 && !p->scene.bvh_valid)
        return fail(GRAY_ERR_INVALID_ARGUMENT, "update_bvh before rebuild_bvh");
    if (p->gaussians.count > 1 && !p->scene.refit_flags)
        return fail(GRAY_ERR_INVALID_ARGUMENT,
                    "update_bvh needs scene.refit_flags (one visit counter per internal node), also after "
                    "gray_rebuild_bvh_static");
    cudaStream_t s = (cudaStream_t)stream;
    GRAY_LAUNCH("snapshot", gray::launch_snapshot(*p, s));
    GRAY_LAUNCH("refit", gray::launch_lbvh_refit(*p, s));
    return GRAY_OK;
}

int gray_rebuild_bvh(const gray_params *p, void *stream) {
    int e = check_common(p);
    if (e) return e;
    if (!p->scene.geom || !p->scene.nodes || !p->scene.sort_tmp)
        return fail(GRAY_ERR_INVALID_ARGUMENT, "missing scene workspace");
    cudaStream_t s = (cudaStream_t)stream;
    GRAY_LAUNCH("snapshot", gray::launch_snapshot(*p, s));
    GRAY_LAUNCH("lbvh_build", gray::launch_lbvh_build(*p, s));
    return GRAY_OK;
}

uint32_t gray_batch_packets(uint32_t width, uint32_t height, int32_t variant) {
    const int v = variant > 0 ? variant : gray::kDefaultTraceVariant;
    const uint32_t tw = (v & 4) ? 4u : 8u, th = 32u / tw;
    return ((width + tw - 1) / tw) * ((height + th - 1) / th);
}

uint32_t gray_batch_groups(uint32_t width, uint32_t height, int32_t variant) {
    const int v = variant > 0 ? variant : gray::kDefaultTraceVariant;
    const uint32_t tw = (v & 4) ? 4u : 8u, th = 32u / tw;
    const uint32_t tx = (width + tw - 1) / tw, ty = (height + th - 1) / th;
    return ((tx + 1) / 2) * ((ty + 1) / 2);
}

uint32_t gray_frontier_words(void) { return GRAY_FRONTIER_WORDS; }

int gray_batch_prep(const gray_params *p, const float *origins, int32_t nviews, float *channels_out, void *stream) {
    int e = check_common(p);
    if (e) return e;
    if (nviews < 0 || (nviews > 0 && (!origins || !channels_out)))
        return fail(GRAY_ERR_INVALID_ARGUMENT, "batch_prep: bad views");
    cudaStream_t s = (cudaStream_t)stream;
    GRAY_LAUNCH("batch_prep", gray::launch_batch_prep(*p, origins, nviews, channels_out, s));
    return GRAY_OK;
}

int gray_render_batch(const gray_batch_scene *scenes, const gray_batch_view *views, int32_t nviews,
                      uint32_t total_packets, float *out, uint32_t *work_counter, uint32_t *frontier,
                      uint32_t total_groups, int32_t variant, int32_t blocks_per_sm, int32_t *status,
                      void *stream) {
    if (nviews <= 0 || !scenes || !views || !out || !work_counter)
        return fail(GRAY_ERR_INVALID_ARGUMENT, "render_batch: missing buffers");
    if (blocks_per_sm < 0 || blocks_per_sm > 32) return fail(GRAY_ERR_OUT_OF_RANGE, "render_batch: blocks_per_sm");
    cudaStream_t s = (cudaStream_t)stream;
    GRAY_LAUNCH("trace_batch", gray::launch_trace_batch(scenes, views, nviews, total_packets, out, work_counter,
                                                        frontier, total_groups, variant, blocks_per_sm, status, s));
    return GRAY_OK;
}

int gray_selftest_copy_wait(int32_t *status, uint64_t limit_ns, void *stream) {
    if (!status) return fail(GRAY_ERR_INVALID_ARGUMENT, "selftest_copy_wait: status is NULL");
    if (limit_ns > 2000000000ull) return fail(GRAY_ERR_OUT_OF_RANGE, "selftest_copy_wait: limit above 2 s");
    cudaStream_t s = (cudaStream_t)stream;
    GRAY_LAUNCH("selftest_copy_wait", gray::launch_copy_wait_selftest(status, limit_ns, s));
    return GRAY_OK;
}

const char *gray_last_error(void) { return g_last_error.c_str(); }

const char *gray_version(void) { return "gray_gb300 0.1 (sm_103a)"; }

}  // extern "C"
