// nbg_lif_grad.cuh -- device pieces shared by the adjoint kernels.
#pragma once

// Fast-sigmoid surrogate derivative of the Heaviside spike, 1 / (1 + k|x|)^2.
__device__ __forceinline__ float surrogate(float x, float k) {
    const float d = 1.0f + k * fabsf(x);
    return 1.0f / (d * d);
}
