// noalloc.cu -- BVH rebuild for callers that cannot allocate device memory.
//
// A rebuild needs transient scratch besides its outputs: the radix sort's second key/value
// buffers and digit histograms, the scene-bounds words and one visit counter per internal node.
// gray_rebuild_bvh takes that scratch from the caller (gray_scene.sort_tmp, .bounds,
// .refit_flags).  Some hosts own every byte of device memory themselves -- a viewer or engine
// plugin running inside a fixed, pre-reserved budget, or a caller whose allocator must not be
// entered at this point -- and cannot hand out extra buffers.  gray_rebuild_bvh_static serves
// them: the scratch lives in the file-scope device array below, sized for at most
// GRAY_STATIC_MAX_GAUSSIANS Gaussians, so the entry point itself allocates nothing.
#include <mutex>
#include <string>

#include "gray_internal.h"

namespace {

constexpr int kMaxStatic = GRAY_STATIC_MAX_GAUSSIANS;
constexpr size_t kSortWordsMax = 2 * (size_t)kMaxStatic + 256 * (size_t)((kMaxStatic + 2047) / 2048);
constexpr size_t kFlagWordsMax = (size_t)kMaxStatic;  // >= internal nodes (n - 1)
constexpr size_t kBoundsWords = 8;
constexpr size_t kStaticWords = kSortWordsMax + kFlagWordsMax + kBoundsWords;

// One copy per device that loads this library, kept until the process exits.  In host code
// `g_static_scratch` is only a stand-in symbol; its device address comes from
// cudaGetSymbolAddress below.
static __device__ __align__(256) uint32_t g_static_scratch[kStaticWords];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
uint32_t *g_static_ptr[kMaxDevices] = {nullptr};

int fail(int code, const std::string &what) {
    gray::set_last_error(what.c_str());
    return code;
}

}  // namespace

extern "C" {

int gray_rebuild_bvh_static(const gray_params *p, void *stream) {
    if (!p) return fail(GRAY_ERR_INVALID_ARGUMENT, "null params");
    const int n = p->gaussians.count;
    if (n < 0) return fail(GRAY_ERR_INVALID_ARGUMENT, "negative Gaussian count");
    if (n > kMaxStatic)
        return fail(GRAY_ERR_OUT_OF_RANGE, "gray_rebuild_bvh_static supports at most " +
                                               std::to_string(kMaxStatic) + " Gaussians, got " + std::to_string(n) +
                                               "; use gray_rebuild_bvh with caller-provided scratch");
    if (!p->scene.geom || !p->scene.l2w || !p->scene.aabb || !p->scene.visible || !p->scene.nodes ||
        !p->scene.int_parent || !p->scene.leaf_parent || !p->scene.order || !p->scene.codes || !p->scene.root_box)
        return fail(GRAY_ERR_INVALID_ARGUMENT, "missing scene output buffers");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(GRAY_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(GRAY_ERR_OUT_OF_RANGE, "device ordinal out of range");
    uint32_t *scratch = nullptr;
    {
        // set-up, once per device, with that device current (the first call on each device)
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_static_ptr[dev]) {
            void *ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_static_scratch);
            if (e != cudaSuccess)
                return fail(GRAY_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_static_ptr[dev] = static_cast<uint32_t *>(ptr);
        }
        scratch = g_static_ptr[dev];
    }
    gray_params q = *p;
    q.scene.sort_tmp = scratch;
    q.scene.refit_flags = scratch + kSortWordsMax;
    q.scene.bounds = scratch + kSortWordsMax + kFlagWordsMax;
    q.scene.bvh_valid = 1;
    cudaStream_t s = (cudaStream_t)stream;
    // the build clears what must start at zero (visit counters, bounds) before using it
    if ((e = gray::launch_snapshot(q, s)) != cudaSuccess)
        return fail(GRAY_ERR_CUDA, std::string("snapshot: ") + cudaGetErrorString(e));
    if ((e = gray::launch_lbvh_build(q, s)) != cudaSuccess)
        return fail(GRAY_ERR_CUDA, std::string("lbvh_build: ") + cudaGetErrorString(e));
    return GRAY_OK;
}

}  // extern "C"
