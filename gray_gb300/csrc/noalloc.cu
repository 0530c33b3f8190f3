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
#include <cuda.h>

#include <mutex>
#include <string>
#include <vector>

#include "gray_internal.h"

namespace {

constexpr int kMaxStatic = GRAY_STATIC_MAX_GAUSSIANS;
constexpr size_t kSortWordsMax = gray::sort_tmp_words(kMaxStatic);
constexpr size_t kFlagWordsMax = (size_t)kMaxStatic;  // >= internal nodes (n - 1)
constexpr size_t kBoundsWords = 8;
constexpr size_t kStaticWords = kSortWordsMax + kFlagWordsMax + kBoundsWords;
static_assert(kSortWordsMax >= gray::sort_tmp_words(kMaxStatic - 1), "sort scratch must cover every allowed count");

// One copy per device context that loads this library, kept until the process exits.  In host
// code `g_static_scratch` is only a stand-in symbol; its device address comes from
// cudaGetSymbolAddress below.
static __device__ __align__(256) uint32_t g_static_scratch[kStaticWords];

// The array's address is looked up once per CUDA context (with that context current) and cached
// under the context's unique id.  The module holding the array is loaded separately in every
// context -- a driver-API context of the caller's, or a primary context re-created after
// cudaDeviceReset -- so an address is only good in the context it was looked up in.
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

struct CachedScratch {
    unsigned long long ctx_id;
    uint32_t *ptr;
};

std::mutex g_mu;
std::vector<CachedScratch> g_cache;
std::once_flag g_driver_resolved;
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

int fail(int code, const std::string &what) {
    gray::set_last_error(what.c_str());
    return code;
}

void resolve_driver_entry_points_once() {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
        g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(fn);
    fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
        g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(fn);
}

void resolve_driver_entry_points() { std::call_once(g_driver_resolved, resolve_driver_entry_points_once); }

// Device address of g_static_scratch in the calling thread's current context.
int scratch_address(uint32_t **out) {
    std::lock_guard<std::mutex> lock(g_mu);
    unsigned long long id = 0;
    bool have_id = gray::current_context_id(&id);
    if (have_id)
        for (const CachedScratch &c : g_cache)
            if (c.ctx_id == id) {
                *out = c.ptr;
                return GRAY_OK;
            }
    // set-up in this context: look the address up (this also makes the runtime's primary context
    // current when no context was)
    void *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_static_scratch);
    if (e != cudaSuccess) return fail(GRAY_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    *out = static_cast<uint32_t *>(ptr);
    if (!have_id) have_id = gray::current_context_id(&id);
    if (have_id) g_cache.push_back(CachedScratch{id, *out});  // without context ids: look up on every call
    return GRAY_OK;
}

}  // namespace

namespace gray {

bool current_context_id(unsigned long long *id) {
    resolve_driver_entry_points();
    if (!g_ctx_get_current || !g_ctx_get_id) return false;
    CUcontext ctx = nullptr;
    return g_ctx_get_current(&ctx) == CUDA_SUCCESS && ctx && g_ctx_get_id(ctx, id) == CUDA_SUCCESS;
}

}  // namespace gray

extern "C" {

int gray_rebuild_bvh_static(const gray_params *p, void *stream) {
    if (p && p->gaussians.count > kMaxStatic)
        return fail(GRAY_ERR_OUT_OF_RANGE, "gray_rebuild_bvh_static supports at most " +
                                               std::to_string(kMaxStatic) + " Gaussians, got " +
                                               std::to_string(p->gaussians.count) +
                                               "; use gray_rebuild_bvh with caller-provided scratch");
    int err = gray::check_common(p);
    if (err) return err;
    if (!p->scene.geom || !p->scene.l2w || !p->scene.aabb || !p->scene.visible || !p->scene.nodes ||
        !p->scene.int_parent || !p->scene.leaf_parent || !p->scene.order || !p->scene.codes || !p->scene.root_box)
        return fail(GRAY_ERR_INVALID_ARGUMENT, "missing scene output buffers");
    uint32_t *scratch = nullptr;
    if ((err = scratch_address(&scratch)) != GRAY_OK) return err;
    gray_params q = *p;
    q.scene.sort_tmp = scratch;
    q.scene.refit_flags = scratch + kSortWordsMax;
    q.scene.bounds = scratch + kSortWordsMax + kFlagWordsMax;
    q.scene.bvh_valid = 1;
    cudaStream_t s = (cudaStream_t)stream;
    // the build clears what must start at zero (visit counters, bounds) before using it
    GRAY_LAUNCH("snapshot", gray::launch_snapshot(q, s));
    GRAY_LAUNCH("lbvh_build", gray::launch_lbvh_build(q, s));
    return GRAY_OK;
}

}  // extern "C"
