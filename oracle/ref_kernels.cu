// ref_kernels.cu -- TEST INFRASTRUCTURE: the reference's own device code for SH, Adam and the
// Gaussian response, compiled unchanged into oracle/_ref/gray_ref.cubin (sm_103a) by
// `make -C oracle ref REF=<graphdeco-inria/gray checkout>`, with the reference's CUDA flags
// (CMakeLists.txt:82-91: fast math, ftz, approximate division and square root) and defines
// (CMakeLists.txt:64-67: CHANNELS=3, MAX_ALPHA=0.9999).
//
// The included files define, unchanged:
//   cuda/utils/sh.cu:224-304  sh_forward_kernel<float3>, sh_forward_kernel<half3>, sh_backward_kernel
//   cuda/opt/adam.cu:25-68    adam_step_base_kernel, adam_step_sh_kernel (and the Adam functor :5-23)
//   cuda/utils/kernel.cu:3-42 compute_scaling_factor, eval_gaussian, compute_alpha
// oracle/ref_kernels.py loads the cubin with the CUDA driver API and launches those kernels on the
// same inputs as gray_gb300's kernels.  Nothing in the package loads it.
#include "utils/sh.cu"
#include "opt/adam.cu"
#include "utils/kernel.cu"

// The kernel-function helpers are __device__ functions with no kernel of their own in the
// reference (they run inside its OptiX programs); this kernel evaluates them per element.
extern "C" __global__ void gray_ref_kernel_functions(int n, const float *opacity, const float *local_hit,
                                                     float alpha_threshold, float exp_power, float *scaling,
                                                     float *response, float *alpha) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    scaling[i] = compute_scaling_factor(opacity[i], alpha_threshold, exp_power);
    const float g = eval_gaussian(make_float3(local_hit[3 * i], local_hit[3 * i + 1], local_hit[3 * i + 2]), exp_power);
    response[i] = g;
    alpha[i] = compute_alpha(g, opacity[i], alpha_threshold);
}
