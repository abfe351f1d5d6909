// mps_gelu.cuh — the activation of the learned warm-start network, shared by the training
// kernels (mma.sync) and the inference kernel (tcgen05).
#pragma once

// GELU in its tanh form (Hendrycks & Gimpel, "Gaussian Error Linear Units", 2016):
// gelu(x) = x/2 (1 + tanh(k0 (x + k1 x^3))), k0 = sqrt(2/pi), k1 = 0.044715, with the
// hardware tanh (tanh.approx.f32, one MUFU op); the network is trained with the same
// function, so the approximation is part of its definition.
#define GELU_K0 0.7978845608028654f
#define GELU_K1 0.044715f
#define GELU_K01 0.035677408136300125f   // k0 k1
__device__ __forceinline__ float tanhHw(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
// u = x (k0 + k0 k1 x^2), h = x/2, gelu = h + h t: five FP32 operations around the tanh
__device__ __forceinline__ float gelu(float x) {
    const float t = tanhHw(x * fmaf(GELU_K01, x * x, GELU_K0));
    const float h = 0.5f * x;
    return fmaf(h, t, h);
}
