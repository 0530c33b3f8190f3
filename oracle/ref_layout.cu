// ref_layout.cu -- TEST INFRASTRUCTURE: prints, as JSON, the byte layout of the reference's kernel
// parameter structs (Gaussians, cuda/core/gaussians.h:7-65; Camera, cuda/core/camera.h:8-15; Adam,
// cuda/opt/adam.cu:5-11) as nvcc lays them out with the reference's defines.  `make -C oracle ref`
// writes it to oracle/ref_layout.json; a CPU test checks oracle/ref_kernels.py's ctypes mirrors
// against that file, so the launches of the reference's kernels pass correctly laid-out arguments.
#include <cstddef>
#include <cstdio>

#include "utils/sh.cu"
#include "opt/adam.cu"

#define FIELD(S, f) printf("%s    \"%s\": %zu", first ? "" : ",\n", #f, offsetof(S, f)), first = false

int main() {
    bool first = true;
    printf("{\n  \"Gaussians\": {\n");
    FIELD(Gaussians, count); FIELD(Gaussians, max_sh_degree); FIELD(Gaussians, num_sh_coeffs);
    FIELD(Gaussians, current_sh_degree); FIELD(Gaussians, mean); FIELD(Gaussians, rotation); FIELD(Gaussians, scale);
    FIELD(Gaussians, opacity); FIELD(Gaussians, channels); FIELD(Gaussians, sh_coeffs_dc);
    FIELD(Gaussians, sh_coeffs_rest); FIELD(Gaussians, lr_mean); FIELD(Gaussians, lr_rotation);
    FIELD(Gaussians, lr_scale); FIELD(Gaussians, lr_opacity); FIELD(Gaussians, lr_channels); FIELD(Gaussians, lr_sh_dc);
    FIELD(Gaussians, lr_sh_rest); FIELD(Gaussians, beta_1); FIELD(Gaussians, beta_2); FIELD(Gaussians, epsilon);
    FIELD(Gaussians, sh_update_laziness); FIELD(Gaussians, grad_mean); FIELD(Gaussians, grad_rotation);
    FIELD(Gaussians, grad_scale); FIELD(Gaussians, grad_opacity); FIELD(Gaussians, grad_channels);
    FIELD(Gaussians, grad_sh_coeffs_dc); FIELD(Gaussians, grad_sh_coeffs_rest); FIELD(Gaussians, first_moment_mean);
    FIELD(Gaussians, first_moment_rotation); FIELD(Gaussians, first_moment_scale); FIELD(Gaussians, first_moment_opacity);
    FIELD(Gaussians, first_moment_channels); FIELD(Gaussians, first_moment_sh_coeffs_dc);
    FIELD(Gaussians, first_moment_sh_coeffs_rest); FIELD(Gaussians, second_moment_mean);
    FIELD(Gaussians, second_moment_rotation); FIELD(Gaussians, second_moment_scale);
    FIELD(Gaussians, second_moment_opacity); FIELD(Gaussians, second_moment_channels);
    FIELD(Gaussians, second_moment_sh_coeffs_dc); FIELD(Gaussians, second_moment_sh_coeffs_rest);
    FIELD(Gaussians, pruning_weight); FIELD(Gaussians, pruning_counter); FIELD(Gaussians, was_visible);
    FIELD(Gaussians, marked); FIELD(Gaussians, sh_is_fp16);
    printf(",\n    \"__size__\": %zu\n  },\n  \"Camera\": {\n", sizeof(Gaussians));
    first = true;
    FIELD(Camera, origin); FIELD(Camera, vertical_fov_radians); FIELD(Camera, rotation_c2w); FIELD(Camera, rotation_w2c);
    FIELD(Camera, znear); FIELD(Camera, zfar);
    printf(",\n    \"__size__\": %zu\n  },\n  \"Adam\": {\n", sizeof(Camera));
    first = true;
    FIELD(Adam, step); FIELD(Adam, zero_grads); FIELD(Adam, beta1); FIELD(Adam, beta2); FIELD(Adam, epsilon);
    printf(",\n    \"__size__\": %zu\n  },\n  \"half3\": {\"__size__\": %zu}\n}\n", sizeof(Adam), sizeof(half3));
    return 0;
}
