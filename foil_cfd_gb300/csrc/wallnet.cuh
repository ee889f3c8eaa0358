// Device building blocks of the learned u_tau seed: the 3-32-32-1 tanh
// network (BF16 weights, FP32 accumulation; the hidden layer as a warp-wide
// tensor-core contraction), Reichardt's law in FP32 (fast
// intrinsics as the reference's wall kernel, or the accurate library
// functions for the learned path's correction and residual) and in FP64, and
// the Newton solvers built from them.
//
// Reichardt's all-y+ law and its Newton solve follow the reference's wall
// model (src/sim/lbm_wallmodel.cu:30-73): u+ = ln(1 + kappa y+)/kappa
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

/// tanh z = 1 - 2 / (1 + e^{2z}) with the fast exponential and divide:
/// absolute error ~3e-7, exact limits +-1 (e^{2z} overflowing to inf gives 1).
__device__ __forceinline__ float tanh_fast(float z) {
    return 1.0f - __fdividef(2.0f, 1.0f + __expf(2.0f * z));
}

/// Two floats as one bf16x2 register (`lo` in the low half: the lower
/// k or n index of an mma fragment pair).
__device__ __forceinline__ unsigned bf16x2_bits(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const unsigned*>(&v);
}

/// d += A B for one 16x8x16 tile: A row-major bf16 (4 regs), B column-major
/// bf16 (2 regs), FP32 accumulators.
__device__ __forceinline__ void mma_16x8x16_bf16(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
    asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

/// Network output (normalised target) for the 32 samples of a warp, each
/// lane passing its own normalised inputs and receiving its own output. All
/// 32 lanes must call it together (lanes without a sample pass zeros).
///
/// The 32x32 hidden layer is one warp-wide contraction Z = H1 W2^T (rows =
/// the warp's samples, k = layer-1 units, n = layer-2 units) on the tensor
/// cores: 2 x 4 tiles of m16n8k16 over 2 k-steps. The weights are BF16
/// already; each FP32 activation is split into three BF16 terms
/// (h = hi + mid + lo to 2^-24 relative), so the products are those of the
/// FP32 activations, accumulated in FP32. Each lane computes the layer-1
/// activations its A fragments hold (samples g, g+8, g+16, g+24 with
/// g = lane / 4; units 2t, 2t+1, 2t+8, 2t+9 (+16) with t = lane % 4), and
/// the layer-2 activations and W3 products of its accumulator fragments;
/// the four lanes of a sample row sum their parts by shuffles.
__device__ __forceinline__ float net_eval_warp(const float* P, float x0, float x1, float x2) {
    __syncwarp();   // the fragments below assume the whole warp, converged
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    // Inputs of the lane's four A-fragment rows: sample g + 8 r.
    float in[4][3];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        in[r][0] = __shfl_sync(0xffffffffu, x0, g + 8 * r);
        in[r][1] = __shfl_sync(0xffffffffu, x1, g + 8 * r);
        in[r][2] = __shfl_sync(0xffffffffu, x2, g + 8 * r);
    }
    // Accumulators: [m tile][n tile][fragment], seeded with b2 of their column.
    float acc[2][4][4];
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
        const float b0 = P[kOffB2 + 8 * nt + 2 * t], b1 = P[kOffB2 + 8 * nt + 2 * t + 1];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            acc[mt][nt][0] = b0; acc[mt][nt][1] = b1;
            acc[mt][nt][2] = b0; acc[mt][nt][3] = b1;
        }
    }
#pragma unroll
    for (int kt = 0; kt < 2; ++kt) {
        // A fragments, three BF16 terms: reg q of tile mt holds row
        // 16 mt + g + 8 (q & 1), units 16 kt + 2t + 8 (q >> 1) + {0, 1}.
        unsigned a[3][2][4];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int r = 2 * mt + (q & 1);
                float h[2];
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const int k = 16 * kt + 2 * t + 8 * (q >> 1) + e;
                    float z = __fmaf_rn(P[kOffW1 + 3 * k], in[r][0], P[kOffB1 + k]);
                    z = __fmaf_rn(P[kOffW1 + 3 * k + 1], in[r][1], z);
                    z = __fmaf_rn(P[kOffW1 + 3 * k + 2], in[r][2], z);
                    h[e] = tanh_fast(z);
                }
#pragma unroll
                for (int term = 0; term < 3; ++term) {
                    const __nv_bfloat162 v = __floats2bfloat162_rn(h[0], h[1]);
                    a[term][mt][q] = *reinterpret_cast<const unsigned*>(&v);
                    h[0] = __fsub_rn(h[0], __low2float(v));
                    h[1] = __fsub_rn(h[1], __high2float(v));
                }
            }
        }
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            // B fragment: column n = 8 nt + g of W2^T, i.e. row n of W2;
            // units 16 kt + 2t (+1) and 16 kt + 2t + 8 (+1).
            const float* w = P + kOffW2 + kH * (8 * nt + g) + 16 * kt + 2 * t;
            const unsigned b0 = bf16x2_bits(w[0], w[1]);
            const unsigned b1 = bf16x2_bits(w[8], w[9]);
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                // Smallest term first.
                mma_16x8x16_bf16(acc[mt][nt], a[2][mt], b0, b1);
                mma_16x8x16_bf16(acc[mt][nt], a[1][mt], b0, b1);
                mma_16x8x16_bf16(acc[mt][nt], a[0][mt], b0, b1);
            }
        }
    }
    // Layer 2 and the output layer: accumulator (mt, nt, c) is row
    // 16 mt + g + 8 (c >> 1), unit 8 nt + 2t + (c & 1).
    float part[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int r = 2 * mt + (c >> 1);
                part[r] = __fmaf_rn(P[kOffW3 + 8 * nt + 2 * t + (c & 1)], tanh_fast(acc[mt][nt][c]), part[r]);
            }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        part[r] += __shfl_xor_sync(0xffffffffu, part[r], 1);
        part[r] += __shfl_xor_sync(0xffffffffu, part[r], 2);
    }
    // This lane's sample is row `lane`: held by lane 4 (lane % 8) as part[lane / 8].
    const int src = 4 * (lane & 7);
    const float v0 = __shfl_sync(0xffffffffu, part[0], src);
    const float v1 = __shfl_sync(0xffffffffu, part[1], src);
    const float v2 = __shfl_sync(0xffffffffu, part[2], src);
    const float v3 = __shfl_sync(0xffffffffu, part[3], src);
    const int r = lane >> 3;
    return P[kOffB3] + (r == 0 ? v0 : r == 1 ? v1 : r == 2 ? v2 : v3);
}

/// Normalised inputs of one sample.
__device__ __forceinline__ void net_inputs(const Norm& nm, float ut, float ys, float nu, float& x0, float& x1,
                                           float& x2) {
    x0 = (logf(ut) - nm.inMean[0]) * nm.inInvStd[0];
    x1 = (logf(ys) - nm.inMean[1]) * nm.inInvStd[1];
    x2 = (logf(nu) - nm.inMean[2]) * nm.inInvStd[2];
}

/// u_tau seeds of a warp's samples from the network (net_eval_warp: all 32
/// lanes call it together); `on` false: no sample in this lane, returns 0.
__device__ __forceinline__ float net_seed_warp(const float* P, const Norm& nm, float ut, float ys, float nu, bool on) {
    float x0 = 0.0f, x1 = 0.0f, x2 = 0.0f;
    if (on) net_inputs(nm, ut, ys, nu, x0, x1, x2);
    const float y = net_eval_warp(P, x0, x1, x2);
    return on ? ut * expf(nm.outMean + nm.outStd * y) : 0.0f;
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
