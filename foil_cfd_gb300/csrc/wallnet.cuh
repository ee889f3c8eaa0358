// Device building blocks of the learned u_tau seed: the 3-32-32-1 tanh
// network (BF16 weights, FP32 accumulation), Reichardt's law in FP32 (fast
// intrinsics as the reference's wall kernel, or the accurate library
// functions for the learned path's correction and residual) and in FP64, and
// the Newton solvers built from them.
//
// Reichardt's all-y+ law and its Newton solve follow the reference's wall
// model (src/sim/lbm_wallmodel.cu:31-95): u+ = ln(1 + kappa y+)/kappa
// + C (1 - e^{-y+/11} - (y+/11) e^{-y+/3}), g(u_tau) = u_tau u+(y u_tau/nu)
// - u_par, kappa = 0.41, C = 7.8.
#pragma once

#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "wallnet_types.h"

namespace fcfd {
namespace wallnet {

constexpr float kKappa = 0.41f;
constexpr float kC = 7.8f;
constexpr double kKappaD = 0.41;
constexpr double kCD = 7.8;
constexpr float kResidualTol = 1e-6f;  // learned path: relative |g| / u_par
constexpr double kNewtonTol = 1e-8;    // FP64 Newton: relative step
constexpr int kNewtonMaxIter = 100;

__device__ __forceinline__ float bf16_bits_to_f32(std::uint16_t b) {
    return __uint_as_float(static_cast<unsigned>(b) << 16);
}

/// Cooperative copy of the BF16 parameters into a block's shared FP32 copy.
__device__ __forceinline__ void load_params(const std::uint16_t* __restrict__ w, float* P) {
    for (int i = threadIdx.x; i < kParams; i += blockDim.x) P[i] = bf16_bits_to_f32(w[i]);
}

/// Network output (normalised target) for normalised inputs, FP32.
__device__ __forceinline__ float net_eval(const float* P, float x0, float x1, float x2) {
    float h1[kH];
#pragma unroll
    for (int j = 0; j < kH; ++j) {
        const float z = P[kOffB1 + j] + P[kOffW1 + 3 * j] * x0 + P[kOffW1 + 3 * j + 1] * x1
                      + P[kOffW1 + 3 * j + 2] * x2;
        h1[j] = tanhf(z);
    }
    float y = P[kOffB3];
#pragma unroll 4
    for (int j = 0; j < kH; ++j) {
        float z = P[kOffB2 + j];
#pragma unroll
        for (int k = 0; k < kH; ++k) z += P[kOffW2 + kH * j + k] * h1[k];
        y += P[kOffW3 + j] * tanhf(z);
    }
    return y;
}

/// Normalised inputs of one sample.
__device__ __forceinline__ void net_inputs(const Norm& nm, float ut, float ys, float nu, float& x0, float& x1,
                                           float& x2) {
    x0 = (logf(ut) - nm.inMean[0]) * nm.inInvStd[0];
    x1 = (logf(ys) - nm.inMean[1]) * nm.inInvStd[1];
    x2 = (logf(nu) - nm.inMean[2]) * nm.inInvStd[2];
}

/// u_tau seed from the network.
__device__ __forceinline__ float net_seed(const float* P, const Norm& nm, float ut, float ys, float nu) {
    float x0, x1, x2;
    net_inputs(nm, ut, ys, nu, x0, x1, x2);
    const float y = net_eval(P, x0, x1, x2);
    return ut * expf(nm.outMean + nm.outStd * y);
}

// ---- Reichardt's law --------------------------------------------------------

/// u+ and du+/dy+ with the fast intrinsics (the reference's evaluation).
__device__ __forceinline__ void reichardt_fast(float yp, float& up, float& dup) {
    const float e11 = __expf(-yp / 11.0f), e3 = __expf(-yp / 3.0f);
    up = __logf(1.0f + kKappa * yp) / kKappa + kC * (1.0f - e11 - (yp / 11.0f) * e3);
    dup = 1.0f / (1.0f + kKappa * yp)
        + kC * ((1.0f / 11.0f) * e11 - (1.0f / 11.0f) * e3 + (yp / 33.0f) * e3);
}

/// u+ and du+/dy+ with the accurate FP32 library functions.
__device__ __forceinline__ void reichardt_acc(float yp, float& up, float& dup) {
    const float e11 = expf(-yp / 11.0f), e3 = expf(-yp / 3.0f);
    up = log1pf(kKappa * yp) / kKappa + kC * (1.0f - e11 - (yp / 11.0f) * e3);
    dup = 1.0f / (1.0f + kKappa * yp)
        + kC * ((1.0f / 11.0f) * e11 - (1.0f / 11.0f) * e3 + (yp / 33.0f) * e3);
}

/// The reference's seed rule: the stored u_tau when positive, else
/// max(0.04 u_par, sqrt(nu u_par / y)).
__device__ __forceinline__ float reference_seed(float ut, float ys, float nu, float warm) {
    return warm > 0.0f ? warm : fmaxf(0.04f * ut, sqrtf(nu * ut / ys));
}

/// The reference's solve: 6 FP32 Newton iterations (fast intrinsics).
__device__ __forceinline__ float newton_reference(float ut, float ys, float nu, float seed) {
    float utau = seed;
#pragma unroll
    for (int it = 0; it < 6; ++it) {
        const float yp = fmaxf(ys * utau / nu, 1e-8f);
        float up, dup;
        reichardt_fast(yp, up, dup);
        const float g = utau * up - ut;
        const float dg = up + yp * dup;
        utau -= g / fmaxf(dg, 1e-6f);
        utau = fmaxf(utau, 0.0f);
    }
    return utau;
}

/// Full Newton in FP64 to a relative step <= 1e-8 (at most 100 iterations);
/// *iters += iterations taken.
__device__ __forceinline__ double newton64(double ut, double ys, double nu, double u, int* iters) {
    int it = 0;
    for (; it < kNewtonMaxIter; ++it) {
        const double yp = fmax(ys * u / nu, 1e-12);
        const double e11 = exp(-yp / 11.0), e3 = exp(-yp / 3.0);
        const double up = log(1.0 + kKappaD * yp) / kKappaD + kCD * (1.0 - e11 - (yp / 11.0) * e3);
        const double dup = 1.0 / (1.0 + kKappaD * yp) + kCD * (e11 / 11.0 - e3 / 11.0 + (yp / 33.0) * e3);
        const double g = u * up - ut;
        const double dg = up + yp * dup;
        const double step = g / dg;
        u -= step;
        if (u < 0.0) u = 0.0;
        if (fabs(step) <= kNewtonTol * fmax(u, 1e-300)) {
            ++it;
            break;
        }
    }
    *iters += it;
    return u;
}

/// The learned solve from a seed: one FP32 Newton correction with the
/// accurate functions; if the relative residual there exceeds 1e-6, FP64
/// Newton from the corrected value. Returns u_tau; *fallback = 1 when FP64
/// was taken.
__device__ __forceinline__ float learned_correct(float ut, float ys, float nu, float seed, int* fallback,
                                                 int* iters) {
    float u = fmaxf(seed, 1e-12f);
    float yp = ys * u / nu;
    float up, dup;
    reichardt_acc(yp, up, dup);
    float g = u * up - ut;
    const float dg = up + yp * dup;
    u = fmaxf(u - g / fmaxf(dg, 1e-6f), 1e-12f);
    yp = ys * u / nu;
    reichardt_acc(yp, up, dup);
    g = u * up - ut;
    if (fabsf(g) <= kResidualTol * ut) {
        *fallback = 0;
        return u;
    }
    *fallback = 1;
    return static_cast<float>(newton64(ut, ys, nu, u, iters));
}

} // namespace wallnet
} // namespace fcfd
