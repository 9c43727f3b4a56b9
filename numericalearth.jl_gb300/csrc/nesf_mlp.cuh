// nesf_mlp.cuh -- layout of the warm-start network in device memory and its
// input features.
//
// The network maps 6 features of a cell -- bulk Richardson number, wind speed
// difference dU, dtheta_0 = theta_a - T_s0, dq_0 = q_a - q_s(T_s0) (g/kg), ln h and
// ln of a neutral momentum roughness -- to the transfer coefficients
// c_u = u* / dU, c_theta = theta* / dtheta_0, c_q = q* / dq_0 of the converged
// fixed point, through 6 -> 64 -> 64 -> 3 with GELU (tanh form) on the hidden
// layers. The features are normalised by stored means and deviations, the
// outputs de-normalised the same way. Weights are FP32 masters (padded to the
// tensor-core shapes: 16 inputs, 16 outputs) with BF16 copies that the tcgen05
// kernels read; the blob also holds the gradient and the Adam moments.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>

#include "nesf_device.cuh"

namespace nesf {
namespace mlp {

constexpr int kIn = 6, kInPad = 16, kHid = 64, kOut = 3, kOutPad = 16;

// FP32 parameter vector: w1 [64 x 16], b1 [64], w2 [64 x 64], b2 [64], w3 [16 x 64], b3 [16]
constexpr int kW1 = 0, kB1 = kW1 + kHid * kInPad, kW2 = kB1 + kHid, kB2 = kW2 + kHid * kHid, kW3 = kB2 + kHid,
              kB3 = kW3 + kOutPad * kHid, kParams = kB3 + kOutPad;

struct Blob {
    float p[kParams];              // parameters
    float g[kParams];              // gradient of the mean loss (accumulated by the training pass)
    float m[kParams], v[kParams];  // Adam moments
    float in_mu[8], in_sig[8];     // feature normalisation (6 used)
    float out_mu[4], out_sig[4];   // target normalisation (3 used)
    float loss[4];                 // [0] sum of squared errors of the last pass, [1] weight of it
    int32_t steps;                 // Adam steps taken
    int32_t error;                 // set when a bounded tensor-core wait gave up
    int32_t pad_[2];
    double stats[32];              // scratch of the normalisation fit (sums, sums of squares)
    __nv_bfloat16 w1h[kHid * kInPad], w2h[kHid * kHid], w3h[kOutPad * kHid];   // BF16 operands
};

// Features of a cell (FP32) from its interface state before the iteration.
struct Features {
    float f[kIn];
    float U, dth, dq;   // the scales that turn transfer coefficients into u*, theta*, q*
};

__device__ __forceinline__ Features warm_features(const DevIface<float>& P, float dU2, float tha, float Ts0, float qa,
                                                  float pa) {
    Features F;
    float qs = surface_specific_humidity(P, pa, Ts0);
    F.dth = tha - Ts0;
    F.dq = qa - qs;
    F.U = sqrtf(dU2 + 0.25f);                      // 0.5 m/s floor, the scale of gustiness
    float Tv = virtual_temperature(P, Ts0, qs);
    float delta = P.eps - 1.0f;
    float rib = P.g * P.h * (F.dth * (1.0f + delta * qs) + delta * Tv * F.dq) / (Tv * F.U * F.U);
    rib = fminf(fmaxf(rib, -5.0f), 5.0f);
    const DevRough<float>& r = P.rough[0];
    float z0;
    if (r.kind == NESF_ROUGHNESS_CONSTANT) {
        z0 = r.value;
    } else {
        float un = 0.035f * F.U;                   // neutral u* at 10 m over the sea
        z0 = r.charnock * un * un / r.g + (r.smooth > 0.0f ? r.smooth * r.nu / un : 0.0f);
    }
    F.f[0] = rib;
    F.f[1] = F.U;
    F.f[2] = F.dth;
    F.f[3] = 1e3f * F.dq;
    F.f[4] = logf(P.h);
    F.f[5] = logf(fmaxf(z0, 1e-7f));
    return F;
}

// Features at a work-list slot: 8 floats (the 6 inputs, dU, 0).
__device__ __forceinline__ void store_features(float* f, int64_t slot, const Features& F) {
    float4* q = (float4*)(f + slot * 8);
    q[0] = make_float4(F.f[0], F.f[1], F.f[2], F.f[3]);
    q[1] = make_float4(F.f[4], F.f[5], F.U, 0.0f);
}

// The network's guess of (u*, theta*, q*) at a slot (written by the inference pass
// as state, not coefficients), or null when there is none.
__device__ __forceinline__ const float* guess_at(const float* guess, int64_t slot, float (&xw)[3]) {
    if (!guess) return nullptr;
    float4 g = *(const float4*)(guess + slot * 4);
    xw[0] = g.x;
    xw[1] = g.y;
    xw[2] = g.z;
    return g.w > 0.0f ? xw : nullptr;
}

__device__ __forceinline__ float gelu(float x) {
    const float k = 0.7978845608028654f;          // sqrt(2 / pi)
    float u = k * (x + 0.044715f * x * x * x);
    return 0.5f * x * (1.0f + tanhf(u));
}

// Bias and GELU of two hidden units at once for inference: the packed FP32 instructions of
// this GPU (add/mul/fma.rn.f32x2: two lanes of FP32 per instruction) for the polynomial and
// the hardware's tanh approximation (tanh.approx.f32, relative error about 2^-11) per unit,
// GELU(z) = z/2 (1 + tanh(z (k + k c z^2))), k = sqrt(2/pi), c = 0.044715 -- gelu's function
// in about half the instructions of a scalar evaluation (the inference is issue-bound
// between its tensor-core stages). Inference only: its activations are rounded to BF16
// (2^-8) before the next layer anyway; training keeps tanhf, so that its gradients follow
// the restatement.
__device__ __forceinline__ uint64_t f2_pack(float a, float b) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void f2_unpack(uint64_t r, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ uint64_t f2_add(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t f2_mul(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t f2_fma(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ void gelu_bias_approx2(float& v0, float& v1, float2 b) {
    const float k = 0.7978845608028654f;          // sqrt(2 / pi)
    const float kc = k * 0.044715f;
    const uint64_t z = f2_add(f2_pack(v0, v1), f2_pack(b.x, b.y));
    const uint64_t u = f2_mul(z, f2_fma(f2_mul(z, z), f2_pack(kc, kc), f2_pack(k, k)));
    float u0, u1, t0, t1;
    f2_unpack(u, u0, u1);
    asm("tanh.approx.f32 %0, %1;" : "=f"(t0) : "f"(u0));
    asm("tanh.approx.f32 %0, %1;" : "=f"(t1) : "f"(u1));
    const uint64_t h = f2_mul(z, f2_pack(0.5f, 0.5f));
    f2_unpack(f2_fma(h, f2_pack(t0, t1), h), v0, v1);
}

__device__ __forceinline__ float gelu_grad(float x) {
    const float k = 0.7978845608028654f;
    float u = k * (x + 0.044715f * x * x * x);
    float t = tanhf(u);
    return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * k * (1.0f + 3.0f * 0.044715f * x * x);
}

}  // namespace mlp
}  // namespace nesf
