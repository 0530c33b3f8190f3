// gray_torch.cpp -- torch.classes.gray.* over the C ABI of libgray_gb300.so, built as libgray.so.
//
// graphdeco-inria/gray registers its OptiX ray tracer as TorchScript custom classes
// (cuda/raytracer.cpp:3-13): CameraDataHolder, ConfigDataHolder, Framebuffer, GaussianDataHolder,
// MetaDataHolder, StatsDataHolder, PPLLDataHolder and Raytracer, with the constructor and methods of
// cuda/raytracer.h:160-183 and the tensor attributes of each holder's bind() (cuda/core/*.h).  This
// file registers the same classes, constructors, methods and attribute names, so the reference's
// gray/raytracer.py, which finds "libgray.so" in its build folder (gray/raytracer.py:9-27) and calls
// torch.classes.load_library on it, runs unchanged on GB300.  Every method fills a gray_params block
// from the holders' tensors and calls the matching extern "C" entry point on the current torch
// stream; no kernel lives here.
//
// Differences a caller can observe, all deliberate:
//  - the forward per-pixel linked list is not materialised (hits are selected during traversal):
//    get_ppll_forward_data() holds one-element buffers; the backward holder's gaussian_ids is the
//    segment pool of the backward hit list (include/gray_gb300.h, gray_hitlist);
//  - no host synchronisation inside a method (the reference reads enable_sh and other flags with
//    .item() and ends Adam with cudaDeviceSynchronize); device-side conditions (hit-list overflow,
//    traversal limit) are OR-ed into a status word instead of __trap(): the next method call that
//    finds a non-zero status (copied to pinned host memory after every call) raises RuntimeError,
//    and check_status() synchronises and raises at once;
//  - rows added when a holder grows are zeroed (torch's resize_ leaves them uninitialised).
#include <ATen/ATen.h>
#include <c10/core/GradMode.h>
#include <c10/cuda/CUDAStream.h>
#include <cuda_runtime.h>
#include <torch/custom_class.h>
#include <torch/library.h>

#include <cstring>
#include <string>

#include "../../include/gray_gb300.h"

namespace {

constexpr int64_t kChannels = 3;
constexpr double kMaxAlpha = 0.9999;
constexpr uint32_t kNullPtr = 0xFFFFFFFFu;

using at::Tensor;

at::TensorOptions f32() { return at::TensorOptions().dtype(at::kFloat).device(at::kCUDA); }
at::TensorOptions f16() { return at::TensorOptions().dtype(at::kHalf).device(at::kCUDA); }
at::TensorOptions i32() { return at::TensorOptions().dtype(at::kInt).device(at::kCUDA); }
at::TensorOptions u8b() { return at::TensorOptions().dtype(at::kBool).device(at::kCUDA); }

template <typename T>
T *ptr(const Tensor &t) {
    return t.defined() && t.numel() > 0 ? reinterpret_cast<T *>(t.data_ptr()) : nullptr;
}

void check(int rc, const char *what) {
    if (rc != GRAY_OK) TORCH_CHECK(false, what, ": ", gray_last_error());
}

// resize_ keeping the leading rows; rows added by growing are zeroed
void resize_rows(Tensor &t, at::IntArrayRef shape) {
    const int64_t old = t.size(0);
    t.resize_(shape);
    if (shape[0] > old) t.narrow(0, old, shape[0] - old).zero_();
}

// ---- holders (cuda/core/*.h) ----

struct CameraDataHolder : torch::CustomClassHolder {
    Tensor origin = at::zeros({3}, f32());
    Tensor vertical_fov_radians = at::zeros({1}, f32());
    Tensor rotation_c2w = at::zeros({3, 3}, f32());
    Tensor rotation_w2c = at::zeros({3, 3}, f32());
    Tensor znear = at::zeros({1}, f32());
    Tensor zfar = at::zeros({1}, f32());

    void set_pose(const Tensor &c2w_origin, const Tensor &c2w_rotation) {
        TORCH_CHECK(c2w_rotation.sizes() == at::IntArrayRef({3, 3}), "c2w_rotation must be 3x3");
        TORCH_CHECK(c2w_origin.sizes() == at::IntArrayRef({3}), "c2w_origin must be 3");
        rotation_c2w.copy_(c2w_rotation);
        origin.copy_(c2w_origin);
        rotation_w2c.copy_(c2w_rotation.transpose(0, 1));
    }
};

struct ConfigDataHolder : torch::CustomClassHolder {  // defaults of cuda/core/config.h:27-47
    Tensor exp_power = at::full({1}, 2.0, f32());
    Tensor alpha_threshold = at::full({1}, 0.01, f32());
    Tensor t_threshold = at::full({1}, 0.01, f32());
    Tensor jitter_primary_rays = at::zeros({1}, u8b());
    Tensor global_scale_factor = at::ones({1}, f32());
    Tensor eps_forward_normalization = at::full({1}, 1e-12, f32());
    Tensor eps_scale_grad = at::full({1}, 1e-12, f32());
    Tensor background_channels = at::zeros({kChannels}, f32());
    Tensor render_depth = at::zeros({1}, u8b());
    Tensor render_ellipsoids = at::zeros({1}, u8b());
    Tensor ellipsoid_min_opacity = at::zeros({1}, f32());
    Tensor rays_from_python = at::zeros({1}, u8b());
    Tensor zero_grads = at::ones({1}, u8b());
    Tensor enable_sh = at::ones({1}, u8b());
    Tensor has_pre_mlp = at::zeros({1}, u8b());
    Tensor needs_ray_output = at::zeros({1}, u8b());
    Tensor update_channels = at::ones({1}, u8b());
};

struct FramebufferDataHolder : torch::CustomClassHolder {
    Tensor output_channels, output_depth, transmittance, full_transmittance, remaining_channels_estimate, ray_origin,
        ray_direction, grad_output_channels;

    FramebufferDataHolder(int64_t w, int64_t h)
        : output_channels(at::zeros({h, w, kChannels}, f32())), output_depth(at::zeros({h, w, 1}, f32())),
          transmittance(at::zeros({h, w, 1}, f32())), full_transmittance(at::zeros({h, w, 1}, f32())),
          remaining_channels_estimate(at::zeros({h, w, kChannels}, f32())), ray_origin(at::zeros({h, w, 3}, f32())),
          ray_direction(at::zeros({h, w, 3}, f32())), grad_output_channels(at::zeros({h, w, kChannels}, f32())) {}
};

#define GRAY_PARAM_GROUPS(X) X(mean) X(rotation) X(scale) X(opacity) X(channels) X(sh_coeffs_dc) X(sh_coeffs_rest)

struct GaussianDataHolder : torch::CustomClassHolder {
    int64_t count = 1, max_sh_degree, num_sh_coeffs;
    bool inference_only;
    Tensor current_sh_degree = at::zeros({1}, i32());
#define DECL(n) Tensor n, grad_##n, first_moment_##n, second_moment_##n;
    GRAY_PARAM_GROUPS(DECL)
#undef DECL
    Tensor lr_mean, lr_rotation, lr_scale, lr_opacity, lr_channels, lr_sh_dc, lr_sh_rest;
    Tensor beta_1 = at::full({1}, 0.9, f32()), beta_2 = at::full({1}, 0.999, f32());
    Tensor epsilon = at::full({1}, 1e-15, f32());
    Tensor sh_update_laziness = at::ones({1}, i32());
    Tensor pruning_weight = at::zeros({1, 1}, f32()), pruning_counter = at::zeros({1, 1}, i32());
    Tensor was_visible = at::zeros({1, 1}, u8b()), marked = at::zeros({1, 1}, f32());

    GaussianDataHolder(int64_t max_sh_degree_, bool inference_only_)
        : max_sh_degree(max_sh_degree_), num_sh_coeffs((max_sh_degree_ + 1) * (max_sh_degree_ + 1) - 1),
          inference_only(inference_only_) {
        TORCH_CHECK(max_sh_degree >= 0 && max_sh_degree <= 3, "sh_max_degree must be in 0..3");
        const auto sh = inference_only ? f16() : f32();
        mean = at::zeros({1, 3}, f32());
        rotation = at::zeros({1, 4}, f32());
        scale = at::zeros({1, 3}, f32());
        opacity = at::zeros({1, 1}, f32());
        channels = at::zeros({1, kChannels}, f32());
        sh_coeffs_dc = at::zeros({1, 1, kChannels}, sh);
        sh_coeffs_rest = at::zeros({1, num_sh_coeffs, kChannels}, sh);
        for (Tensor *t : {&lr_mean, &lr_rotation, &lr_scale, &lr_opacity, &lr_channels, &lr_sh_dc, &lr_sh_rest})
            *t = at::ones({1, 1}, f32());
#define ZERO_LIKE(n)                                        \
    grad_##n = at::zeros(n.sizes(), f32());                 \
    first_moment_##n = at::zeros(n.sizes(), f32());         \
    second_moment_##n = at::zeros(n.sizes(), f32());
        GRAY_PARAM_GROUPS(ZERO_LIKE)
#undef ZERO_LIKE
        link_grads();
    }

    std::vector<int64_t> shape(const char *group, int64_t n) const {
        if (!strcmp(group, "sh_coeffs_dc")) return {n, 1, kChannels};
        if (!strcmp(group, "sh_coeffs_rest")) return {n, num_sh_coeffs, kChannels};
        const int64_t w = !strcmp(group, "rotation") ? 4 : !strcmp(group, "opacity") ? 1 : 3;
        return {n, w};
    }

    void link_grads() {
        if (inference_only) return;
#define LINK(n) n.mutable_grad() = grad_##n;
        GRAY_PARAM_GROUPS(LINK)
#undef LINK
    }

    // cuda/core/gaussians.h:198-263: only shrinking is allowed once populated
    void resize(int64_t n) {
        TORCH_CHECK(n >= 0, "negative Gaussian count");
        if (count > 1) TORCH_CHECK(n <= count, "The new number of Gaussians must not be larger than the current count.");
        at::NoGradGuard no_grad;
        count = n;
#define RESIZE_PARAM(g) \
    g.mutable_grad() = Tensor(); \
    resize_rows(g, shape(#g, n));
        GRAY_PARAM_GROUPS(RESIZE_PARAM)
#undef RESIZE_PARAM
        for (Tensor *t : {&lr_mean, &lr_rotation, &lr_scale, &lr_opacity, &lr_channels, &lr_sh_dc, &lr_sh_rest}) {
            const Tensor first = t->reshape({-1}).narrow(0, 0, 1).clone();
            const int64_t old = t->size(0);
            t->resize_({n, 1});
            if (n > old) t->narrow(0, old, n - old).copy_(first.expand({n - old}).reshape({n - old, 1}));
        }
        if (!inference_only) {
#define RESIZE_STATE(g)                              \
    resize_rows(grad_##g, shape(#g, n));             \
    resize_rows(first_moment_##g, shape(#g, n));     \
    resize_rows(second_moment_##g, shape(#g, n));
            GRAY_PARAM_GROUPS(RESIZE_STATE)
#undef RESIZE_STATE
            resize_rows(pruning_weight, {n, 1});
            resize_rows(pruning_counter, {n, 1});
            resize_rows(marked, {n, 1});
        }
        resize_rows(was_visible, {n, 1});
        link_grads();
    }

    void increment_sh_degree() {
        at::NoGradGuard no_grad;
        if (current_sh_degree.item<int32_t>() < max_sh_degree) current_sh_degree.add_(1);
    }

    gray_gaussians reify() const {
        gray_gaussians g;
        std::memset(&g, 0, sizeof(g));
        g.count = (int32_t)count;
        g.max_sh_degree = (int32_t)max_sh_degree;
        g.num_sh_coeffs = (int32_t)num_sh_coeffs;
        g.sh_is_fp16 = inference_only ? 1 : 0;
        g.current_sh_degree = ptr<int32_t>(current_sh_degree);
        g.mean = ptr<float>(mean);
        g.rotation = ptr<float>(rotation);
        g.scale = ptr<float>(scale);
        g.opacity = ptr<float>(opacity);
        g.channels = ptr<float>(channels);
        g.sh_coeffs_dc = ptr<void>(sh_coeffs_dc);
        g.sh_coeffs_rest = ptr<void>(sh_coeffs_rest);
        g.lr_mean = ptr<float>(lr_mean);
        g.lr_rotation = ptr<float>(lr_rotation);
        g.lr_scale = ptr<float>(lr_scale);
        g.lr_opacity = ptr<float>(lr_opacity);
        g.lr_channels = ptr<float>(lr_channels);
        g.lr_sh_dc = ptr<float>(lr_sh_dc);
        g.lr_sh_rest = ptr<float>(lr_sh_rest);
        g.beta_1 = ptr<float>(beta_1);
        g.beta_2 = ptr<float>(beta_2);
        g.epsilon = ptr<float>(epsilon);
        g.sh_update_laziness = ptr<int32_t>(sh_update_laziness);
        if (!inference_only) {
#define STATE(n)                                                  \
    g.grad_##n = ptr<float>(grad_##n);                            \
    g.first_moment_##n = ptr<float>(first_moment_##n);            \
    g.second_moment_##n = ptr<float>(second_moment_##n);
            GRAY_PARAM_GROUPS(STATE)
#undef STATE
        }
        g.pruning_weight = ptr<float>(pruning_weight);
        g.pruning_counter = ptr<int32_t>(pruning_counter);
        g.was_visible = ptr<uint8_t>(was_visible);
        g.marked = ptr<float>(marked);
        return g;
    }
};

struct MetaDataHolder : torch::CustomClassHolder {
    Tensor run_forward_pass = at::ones({1}, u8b());
    Tensor run_backward_pass = at::ones({1}, u8b());
    Tensor grads_enabled = at::ones({1}, u8b());
    Tensor total_num_calls = at::zeros({1}, i32());
    Tensor total_num_steps = at::zeros({1}, i32());

    void update() {
        grads_enabled.fill_(c10::GradMode::is_enabled());
        total_num_calls.add_(1);
    }
};

struct StatsDataHolder : torch::CustomClassHolder {
    Tensor num_gaussians_hit, num_gaussians_accumulated;
    StatsDataHolder(int64_t w, int64_t h)
        : num_gaussians_hit(at::zeros({h, w}, i32())), num_gaussians_accumulated(at::zeros({h, w}, i32())) {}
    void reset() {
        num_gaussians_hit.zero_();
        num_gaussians_accumulated.zero_();
    }
};

// The backward holder's gaussian_ids is the segment pool of the backward hit list.
struct PPLLDataHolder : torch::CustomClassHolder {
    Tensor head_per_pixel, total_hits = at::zeros({1}, i32()), gaussian_ids, distances, alphas, previous_entries;
    int64_t size;
    PPLLDataHolder(int64_t w, int64_t h, int64_t size_) : size(std::max<int64_t>(size_, 1)) {
        head_per_pixel = at::full({h, w}, (int64_t)(int32_t)kNullPtr, i32());
        gaussian_ids = at::zeros({size}, i32());
        distances = at::zeros({0}, f16());
        alphas = at::zeros({0}, f16());
        previous_entries = at::zeros({0}, i32());
    }
};

// ---- Raytracer (cuda/raytracer.h:29-184) ----

struct Raytracer : torch::CustomClassHolder {
    int64_t width, height, alloc_width, alloc_height;
    bool inference_only;
    c10::intrusive_ptr<CameraDataHolder> camera_data = c10::make_intrusive<CameraDataHolder>();
    c10::intrusive_ptr<ConfigDataHolder> config_data = c10::make_intrusive<ConfigDataHolder>();
    c10::intrusive_ptr<FramebufferDataHolder> framebuffer_data;
    c10::intrusive_ptr<GaussianDataHolder> gaussian_data;
    c10::intrusive_ptr<MetaDataHolder> meta_data = c10::make_intrusive<MetaDataHolder>();
    c10::intrusive_ptr<StatsDataHolder> stats_data;
    c10::intrusive_ptr<PPLLDataHolder> ppll_forward_data, ppll_backward_data;

    // library workspace (include/gray_gb300.h, gray_scene / gray_hitlist.schedule)
    Tensor geom, l2w, aabb, visible, live, grad_acc, nodes, int_parent, leaf_parent, order, codes, refit_flags,
        sort_tmp, root_box, bounds, bwd_rec, schedule;
    Tensor status = at::zeros({1}, i32());
    int32_t *status_host = nullptr;  // pinned mirror of `status`, refreshed after every call
    bool bvh_valid = false;

    Raytracer(int64_t w, int64_t h, int64_t num_gaussians, int64_t sh_max_degree, int64_t ppll_forward_size,
              int64_t ppll_backward_size, bool inference_only_)
        : width(w), height(h), alloc_width(w), alloc_height(h), inference_only(inference_only_) {
        TORCH_CHECK(w >= 1 && h >= 1, "image size must be positive");
        (void)ppll_forward_size;  // the forward list is not materialised
        framebuffer_data = c10::make_intrusive<FramebufferDataHolder>(w, h);
        gaussian_data = c10::make_intrusive<GaussianDataHolder>(sh_max_degree, inference_only);
        stats_data = c10::make_intrusive<StatsDataHolder>(w, h);
        ppll_forward_data = c10::make_intrusive<PPLLDataHolder>(w, h, 1);
        ppll_backward_data = c10::make_intrusive<PPLLDataHolder>(w, h, inference_only ? 1 : ppll_backward_size);
        schedule = at::zeros({(int64_t)gray_schedule_words((uint32_t)w, (uint32_t)h)}, i32());
        TORCH_CHECK(cudaMallocHost(reinterpret_cast<void **>(&status_host), sizeof(int32_t)) == cudaSuccess,
                    "pinned status word");
        *status_host = 0;
        alloc_workspace(1);
        if (num_gaussians > 0) resize(num_gaussians);
    }

    ~Raytracer() override {
        if (status_host) cudaFreeHost(status_host);
    }

    void alloc_workspace(int64_t n) {
        const int64_t nn = std::max<int64_t>(n, 1), m = std::max<int64_t>(n - 1, 1);
        geom = at::zeros({nn, 12}, f32());
        l2w = at::zeros({nn, 12}, f32());
        aabb = at::zeros({nn, 8}, f32());
        visible = at::zeros({nn}, at::TensorOptions().dtype(at::kByte).device(at::kCUDA));
        live = at::zeros({nn, 2}, f32());
        grad_acc = at::zeros({nn, 16}, f32());
        nodes = at::zeros({m, 16}, f32());
        int_parent = at::zeros({m}, i32());
        leaf_parent = at::zeros({nn}, i32());
        order = at::zeros({nn}, i32());
        codes = at::zeros({nn}, i32());
        refit_flags = at::zeros({m}, i32());
        sort_tmp = at::zeros({std::max<int64_t>((int64_t)gray_sort_tmp_words((int32_t)n), 1)}, i32());
        root_box = at::zeros({8}, f32());
        bounds = at::zeros({8}, i32());
        bwd_rec = at::zeros({inference_only ? 1 : nn, 24}, f32());
        bvh_valid = false;
    }

    gray_params params() const {
        gray_params p;
        std::memset(&p, 0, sizeof(p));
        p.image_width = (uint32_t)alloc_width;
        p.image_height = (uint32_t)alloc_height;
        p.render_width = (uint32_t)width;
        p.render_height = (uint32_t)height;
        const CameraDataHolder &c = *camera_data;
        p.camera = gray_camera{ptr<float>(c.origin), ptr<float>(c.vertical_fov_radians), ptr<float>(c.rotation_c2w),
                               ptr<float>(c.rotation_w2c), ptr<float>(c.znear), ptr<float>(c.zfar)};
        const ConfigDataHolder &k = *config_data;
        p.config = gray_config{ptr<float>(k.exp_power), ptr<float>(k.alpha_threshold), ptr<float>(k.t_threshold),
                               ptr<uint8_t>(k.jitter_primary_rays), ptr<float>(k.global_scale_factor),
                               ptr<float>(k.eps_forward_normalization), ptr<float>(k.eps_scale_grad),
                               ptr<float>(k.background_channels), ptr<uint8_t>(k.render_depth),
                               ptr<uint8_t>(k.render_ellipsoids), ptr<float>(k.ellipsoid_min_opacity),
                               ptr<uint8_t>(k.rays_from_python), ptr<uint8_t>(k.zero_grads), ptr<uint8_t>(k.enable_sh),
                               ptr<uint8_t>(k.needs_ray_output), ptr<uint8_t>(k.update_channels)};
        const FramebufferDataHolder &f = *framebuffer_data;
        p.framebuffer = gray_framebuffer{ptr<float>(f.output_channels), ptr<float>(f.output_depth),
                                         ptr<float>(f.transmittance), ptr<float>(f.full_transmittance),
                                         ptr<float>(f.remaining_channels_estimate), ptr<float>(f.ray_origin),
                                         ptr<float>(f.ray_direction), ptr<float>(f.grad_output_channels)};
        p.gaussians = gaussian_data->reify();
        const MetaDataHolder &m = *meta_data;
        p.metadata = gray_metadata{ptr<uint8_t>(m.run_forward_pass), ptr<uint8_t>(m.run_backward_pass),
                                   ptr<uint8_t>(m.grads_enabled), ptr<uint32_t>(m.total_num_calls),
                                   ptr<uint32_t>(m.total_num_steps)};
        p.stats = gray_stats{ptr<int32_t>(stats_data->num_gaussians_hit), ptr<int32_t>(stats_data->num_gaussians_accumulated)};
        const PPLLDataHolder &b = *ppll_backward_data;
        p.hitlist = gray_hitlist{ptr<uint32_t>(b.head_per_pixel), ptr<uint32_t>(b.total_hits), ptr<uint32_t>(b.gaussian_ids),
                                 (uint32_t)b.size, ptr<uint32_t>(schedule)};
        p.scene = gray_scene{ptr<float>(geom), ptr<float>(l2w), ptr<float>(aabb), ptr<uint8_t>(visible), ptr<float>(live),
                             ptr<float>(grad_acc), ptr<float>(nodes), ptr<int32_t>(int_parent), ptr<int32_t>(leaf_parent),
                             ptr<uint32_t>(order), ptr<uint32_t>(codes), ptr<uint32_t>(refit_flags),
                             ptr<uint32_t>(sort_tmp), ptr<float>(root_box), ptr<uint32_t>(bounds),
                             inference_only ? nullptr : ptr<float>(bwd_rec), bvh_valid ? 1 : 0};
        p.status = ptr<int32_t>(status);
        p.trace_variant = 0;
        return p;
    }

    static const char *status_text(int32_t v) {
        if (v & GRAY_STATUS_HITLIST_OVERFLOW) return "backward hit list overflow (increase ppll_backward_size)";
        if (v & GRAY_STATUS_STACK_OVERFLOW) return "BVH traversal limit exceeded";
        if (v & GRAY_STATUS_REFIT_TIMEOUT) return "BVH refit gave up (corrupt tree)";
        if (v & GRAY_STATUS_BAD_MODE) return "render_ellipsoids=True is only supported for no-grad display renders";
        if (v & GRAY_STATUS_COPY_TIMEOUT) return "a bulk copy did not complete (streaming kernel stopped early)";
        return "unknown device status";
    }

    // Raises for a device-side condition that an earlier call reported (seen without a sync).
    void raise_reported() {
        const int32_t v = *(volatile int32_t *)status_host;
        if (v) {
            *status_host = 0;
            status.zero_();
            TORCH_CHECK(false, "gray: device status ", v, ": ", status_text(v));
        }
    }

    template <typename F>
    void call(F fn, const char *what) {
        raise_reported();
        const gray_params p = params();
        cudaStream_t s = c10::cuda::getCurrentCUDAStream().stream();
        check(fn(&p, (void *)s), what);
        cudaMemcpyAsync(status_host, p.status, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    }

    void forward_pass() {
        meta_data->grads_enabled.fill_(c10::GradMode::is_enabled());
        call(gray_forward_pass, "forward_pass");
    }
    void forward_pass_display() { call(gray_forward_pass_display, "forward_pass_display"); }
    void backward_pass() { call(gray_backward_pass, "backward_pass"); }
    void step() { call(gray_step, "step"); }
    void update_bvh() { call(gray_update_bvh, "update_bvh"); }
    void rebuild_bvh() {
        bvh_valid = true;
        try {
            call(gray_rebuild_bvh, "rebuild_bvh");
        } catch (...) {
            bvh_valid = false;
            throw;
        }
    }
    void resize(int64_t n) {
        gaussian_data->resize(n);
        alloc_workspace(gaussian_data->count);
    }
    void set_render_resolution(int64_t w, int64_t h) {
        TORCH_CHECK(w >= 1 && h >= 1, "render resolution must be positive");
        TORCH_CHECK(w <= alloc_width && h <= alloc_height, "render resolution cannot exceed the allocated framebuffer size");
        width = w;
        height = h;
    }
    void check_status() {
        cudaStream_t s = c10::cuda::getCurrentCUDAStream().stream();
        cudaStreamSynchronize(s);
        raise_reported();
        const int32_t v = status.item<int32_t>();
        if (v) {
            status.zero_();
            TORCH_CHECK(false, "gray: device status ", v, ": ", status_text(v));
        }
    }
};

}  // namespace

TORCH_LIBRARY(gray, m) {
    m.class_<CameraDataHolder>("CameraDataHolder")
        .def("set_pose", &CameraDataHolder::set_pose)
        .def_readonly("origin", &CameraDataHolder::origin)
        .def_readonly("vertical_fov_radians", &CameraDataHolder::vertical_fov_radians)
        .def_readonly("rotation_c2w", &CameraDataHolder::rotation_c2w)
        .def_readonly("rotation_w2c", &CameraDataHolder::rotation_w2c)
        .def_readonly("znear", &CameraDataHolder::znear)
        .def_readonly("zfar", &CameraDataHolder::zfar);

    m.class_<ConfigDataHolder>("ConfigDataHolder")
        .def_readonly("exp_power", &ConfigDataHolder::exp_power)
        .def_readonly("alpha_threshold", &ConfigDataHolder::alpha_threshold)
        .def_readonly("t_threshold", &ConfigDataHolder::t_threshold)
        .def_readonly("jitter_primary_rays", &ConfigDataHolder::jitter_primary_rays)
        .def_readonly("global_scale_factor", &ConfigDataHolder::global_scale_factor)
        .def_readonly("eps_forward_normalization", &ConfigDataHolder::eps_forward_normalization)
        .def_readonly("eps_scale_grad", &ConfigDataHolder::eps_scale_grad)
        .def_readonly("background_channels", &ConfigDataHolder::background_channels)
        .def_readonly("render_depth", &ConfigDataHolder::render_depth)
        .def_readonly("render_ellipsoids", &ConfigDataHolder::render_ellipsoids)
        .def_readonly("ellipsoid_min_opacity", &ConfigDataHolder::ellipsoid_min_opacity)
        .def_readonly("rays_from_python", &ConfigDataHolder::rays_from_python)
        .def_readonly("zero_grads", &ConfigDataHolder::zero_grads)
        .def_readonly("enable_sh", &ConfigDataHolder::enable_sh)
        .def_readonly("needs_ray_output", &ConfigDataHolder::needs_ray_output)
        .def_readonly("update_channels", &ConfigDataHolder::update_channels);

    m.class_<FramebufferDataHolder>("Framebuffer")
        .def_readonly("output_channels", &FramebufferDataHolder::output_channels)
        .def_readonly("output_depth", &FramebufferDataHolder::output_depth)
        .def_readonly("transmittance", &FramebufferDataHolder::transmittance)
        .def_readonly("full_transmittance", &FramebufferDataHolder::full_transmittance)
        .def_readonly("remaining_channels_estimate", &FramebufferDataHolder::remaining_channels_estimate)
        .def_readonly("ray_origin", &FramebufferDataHolder::ray_origin)
        .def_readonly("ray_direction", &FramebufferDataHolder::ray_direction)
        .def_readonly("grad_output_channels", &FramebufferDataHolder::grad_output_channels);

    auto g = m.class_<GaussianDataHolder>("GaussianDataHolder")
                 .def("increment_sh_degree", &GaussianDataHolder::increment_sh_degree)
                 .def_readonly("current_sh_degree", &GaussianDataHolder::current_sh_degree);
#define READ(n)                                                                  \
    g.def_readonly(#n, &GaussianDataHolder::n)                                   \
        .def_readonly("grad_" #n, &GaussianDataHolder::grad_##n)                 \
        .def_readonly("first_moment_" #n, &GaussianDataHolder::first_moment_##n) \
        .def_readonly("second_moment_" #n, &GaussianDataHolder::second_moment_##n);
    GRAY_PARAM_GROUPS(READ)
#undef READ
    g.def_readonly("lr_mean", &GaussianDataHolder::lr_mean)
        .def_readonly("lr_rotation", &GaussianDataHolder::lr_rotation)
        .def_readonly("lr_scale", &GaussianDataHolder::lr_scale)
        .def_readonly("lr_opacity", &GaussianDataHolder::lr_opacity)
        .def_readonly("lr_channels", &GaussianDataHolder::lr_channels)
        .def_readonly("lr_sh_dc", &GaussianDataHolder::lr_sh_dc)
        .def_readonly("lr_sh_rest", &GaussianDataHolder::lr_sh_rest)
        .def_readonly("beta_1", &GaussianDataHolder::beta_1)
        .def_readonly("beta_2", &GaussianDataHolder::beta_2)
        .def_readonly("epsilon", &GaussianDataHolder::epsilon)
        .def_readonly("sh_update_laziness", &GaussianDataHolder::sh_update_laziness)
        .def_readonly("pruning_weight", &GaussianDataHolder::pruning_weight)
        .def_readonly("pruning_counter", &GaussianDataHolder::pruning_counter)
        .def_readonly("was_visible", &GaussianDataHolder::was_visible)
        .def_readonly("marked", &GaussianDataHolder::marked);

    m.class_<MetaDataHolder>("MetaDataHolder")
        .def_readonly("grads_enabled", &MetaDataHolder::grads_enabled)
        .def_readonly("total_num_calls", &MetaDataHolder::total_num_calls)
        .def_readonly("total_num_steps", &MetaDataHolder::total_num_steps)
        .def("update", &MetaDataHolder::update);

    m.class_<StatsDataHolder>("StatsDataHolder")
        .def_readonly("num_gaussians_hit", &StatsDataHolder::num_gaussians_hit)
        .def_readonly("num_gaussians_accumulated", &StatsDataHolder::num_gaussians_accumulated)
        .def("reset", &StatsDataHolder::reset);

    m.class_<PPLLDataHolder>("PPLLDataHolder")
        .def_readonly("head_per_pixel", &PPLLDataHolder::head_per_pixel)
        .def_readonly("total_hits", &PPLLDataHolder::total_hits)
        .def_readonly("gaussian_ids", &PPLLDataHolder::gaussian_ids)
        .def_readonly("distances", &PPLLDataHolder::distances)
        .def_readonly("alphas", &PPLLDataHolder::alphas)
        .def_readonly("previous_entries", &PPLLDataHolder::previous_entries)
        .def_static("NULL_PTR", []() { return (int64_t)kNullPtr; });

    m.class_<Raytracer>("Raytracer")
        .def(torch::init<int64_t, int64_t, int64_t, int64_t, int64_t, int64_t, bool>())
        .def("forward_pass", &Raytracer::forward_pass)
        .def("forward_pass_display", &Raytracer::forward_pass_display)
        .def("backward_pass", &Raytracer::backward_pass)
        .def("step", &Raytracer::step)
        .def("update_bvh", &Raytracer::update_bvh)
        .def("rebuild_bvh", &Raytracer::rebuild_bvh)
        .def("resize", &Raytracer::resize)
        .def("set_render_resolution", &Raytracer::set_render_resolution)
        .def("check_status", &Raytracer::check_status)
        .def("get_camera", [](const c10::intrusive_ptr<Raytracer> &self) { return self->camera_data; })
        .def("get_config", [](const c10::intrusive_ptr<Raytracer> &self) { return self->config_data; })
        .def("get_framebuffer", [](const c10::intrusive_ptr<Raytracer> &self) { return self->framebuffer_data; })
        .def("get_gaussians", [](const c10::intrusive_ptr<Raytracer> &self) { return self->gaussian_data; })
        .def("get_metadata", [](const c10::intrusive_ptr<Raytracer> &self) { return self->meta_data; })
        .def("get_stats", [](const c10::intrusive_ptr<Raytracer> &self) { return self->stats_data; })
        .def("get_ppll_forward_data", [](const c10::intrusive_ptr<Raytracer> &self) { return self->ppll_forward_data; })
        .def("get_ppll_backward_data",
             [](const c10::intrusive_ptr<Raytracer> &self) { return self->ppll_backward_data; })
        .def("get_num_channels", [](const c10::intrusive_ptr<Raytracer> &self) { return kChannels; })
        .def("get_max_alpha", [](const c10::intrusive_ptr<Raytracer> &self) { return kMaxAlpha; });
}
