// Activation of the learned surrogate, shared by its training and inference kernels.
//
// GELU in its tanh form (Hendrycks & Gimpel, "Gaussian Error Linear Units"):
//   g(z) = z/2 (1 + tanh(u)),  u = sqrt(2/pi) (z + 0.044715 z^3),
// evaluated with the hardware tanh approximation (tanh.approx.f32, relative error about
// 2^-11, far below the bf16 rounding of the activations).  A handful of instructions per
// value instead of an erf evaluation: the epilogue of every surrogate GEMM runs it on each
// output, and with the erf form the epilogue, not the tensor cores, bounded the GEMMs.
#pragma once

__device__ __forceinline__ float tanh_hw(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float gelu(float z) {
    const float u = 0.7978845608028654f * fmaf(0.044715f * z * z, z, z);
    return 0.5f * z * (1.0f + tanh_hw(u));
}

// g'(z) = (1 + t)/2 + z/2 (1 - t^2) du/dz,  t = tanh(u),  du/dz = sqrt(2/pi) (1 + 3*0.044715 z^2)
__device__ __forceinline__ float gelu_grad(float z) {
    const float z2 = z * z;
    const float t = tanh_hw(0.7978845608028654f * fmaf(0.044715f * z2, z, z));
    const float du = 0.7978845608028654f * fmaf(0.134145f, z2, 1.0f);
    return 0.5f * (1.0f + t) + 0.5f * z * fmaf(-t, t, 1.0f) * du;
}
