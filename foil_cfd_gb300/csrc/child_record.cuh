// Restriction pass 1 per coarse cell: the averaged children's moments with
// the density floor and the |u| <= 0.3 limiter, their non-equilibrium part,
// and the 96-byte scratch record the restriction filter reads (fneq[19],
// valid flag, rho, ux, uy, uz as six float4). Shared by the stand-alone
// child-average kernel and the fine collide that fuses it. Every multiply
// and add is an explicit round-to-nearest intrinsic in the reference's
// operation order, so the record rounds the same in a translation unit built
// with or without FMA contraction, and is bit-identical to the reference's
// childAvgFneq (src/sim/lbm_refine.cu:70-97) evaluated without contraction.
#pragma once

#include "d3q19.cuh"

namespace fcfd {

constexpr int kScratchVals = 24;   // per coarse cell: fneq[19], valid, rho, ux, uy, uz
constexpr int kScratchValid = 19;  // record layout: 6 float4, valid flag closes the fneq part
constexpr int kScratchRho = 20;

__device__ __forceinline__ float rn_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float rn_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rn_sub(float a, float b) { return __fsub_rn(a, b); }

/// Moments of fi with the density floor and the |u| <= 0.3 limiter.
__device__ __forceinline__ void limited_moments(const float (&fi)[kQ], float& rho, float& ux, float& uy,
                                                float& uz) {
    float r = 0.f, jx = 0.f, jy = 0.f, jz = 0.f;
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
        r = rn_add(r, fi[q]);
        jx = rn_add(jx, rn_mul(static_cast<float>(cx(q)), fi[q]));
        jy = rn_add(jy, rn_mul(static_cast<float>(cy(q)), fi[q]));
        jz = rn_add(jz, rn_mul(static_cast<float>(cz(q)), fi[q]));
    }
    r = fmaxf(r, kRhoFloor);
    const float inv = 1.0f / r;
    ux = rn_mul(jx, inv); uy = rn_mul(jy, inv); uz = rn_mul(jz, inv);
    const float u2 = rn_add(rn_add(rn_mul(ux, ux), rn_mul(uy, uy)), rn_mul(uz, uz));
    if (u2 > kMaxSimSpeed * kMaxSimSpeed) {
        const float sc = rn_mul(kMaxSimSpeed, 1.0f / sqrtf(u2));
        ux = rn_mul(ux, sc); uy = rn_mul(uy, sc); uz = rn_mul(uz, sc);
    }
    rho = r;
}

/// Second-order equilibrium (lbm_core.cu:65-73), operations in source order.
__device__ __forceinline__ float feq_q_rn(int q, float rho, float ux, float uy, float uz, float usq) {
    const float cdot = rn_add(rn_add(rn_mul(static_cast<float>(cx(q)), ux), rn_mul(static_cast<float>(cy(q)), uy)),
                              rn_mul(static_cast<float>(cz(q)), uz));
    const float cu = rn_mul(3.0f, cdot);
    const float poly = rn_sub(rn_add(rn_add(1.0f, cu), rn_mul(rn_mul(0.5f, cu), cu)), usq);
    return rn_mul(rn_mul(wgt(q), rho), poly);
}

/// Record of a coarse cell from the sum fi of its nFluid fluid children.
__device__ __forceinline__ void write_child_record(float (&fi)[kQ], int nFluid, float4* rec) {
    if (nFluid == 0) {
        rec[kScratchValid / 4] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    const float invN = 1.0f / static_cast<float>(nFluid);
#pragma unroll
    for (int q = 0; q < kQ; ++q) fi[q] = rn_mul(fi[q], invN);
    float rho, ux, uy, uz;
    limited_moments(fi, rho, ux, uy, uz);
    const float usq = rn_mul(1.5f, rn_add(rn_add(rn_mul(ux, ux), rn_mul(uy, uy)), rn_mul(uz, uz)));
    float r[kScratchVals];
#pragma unroll
    for (int q = 0; q < kQ; ++q) r[q] = rn_sub(fi[q], feq_q_rn(q, rho, ux, uy, uz, usq));
    r[kScratchValid] = 1.0f;
    r[kScratchRho] = rho; r[kScratchRho + 1] = ux; r[kScratchRho + 2] = uy; r[kScratchRho + 3] = uz;
#pragma unroll
    for (int k = 0; k < kScratchVals / 4; ++k) rec[k] = make_float4(r[4 * k], r[4 * k + 1], r[4 * k + 2], r[4 * k + 3]);
}

} // namespace fcfd
