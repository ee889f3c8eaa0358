// Restriction pass 1 per coarse cell: the averaged children's moments with
// the density floor and the |u| <= 0.3 limiter, their non-equilibrium part,
// and the scratch record the restriction filter reads (fneq[19], valid
// flag, rho, ux, uy, uz; 96 B with FP32 storage, 64 B with FP16). Shared by the stand-alone
// child-average kernel and the fine collide that fuses it.
//
// The scratch is planar: float4 k of record t sits at base[k * stride + t]
// (stride = records in the scratch), so the 32 lanes of a warp reading the
// same part of the records of 32 consecutive coarse cells read 512
// contiguous bytes, not 32 pieces 96 bytes apart. Every multiply
// and add is an explicit round-to-nearest intrinsic in the reference's
// operation order, so the record rounds the same in a translation unit built
// with or without FMA contraction, and is bit-identical to the reference's
// childAvgFneq (src/sim/lbm_refine.cu:70-97) evaluated without contraction.
#pragma once

#include "d3q19.cuh"

#include <cuda_fp16.h>

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
        // The hardware rsqrtf of the reference's GPU build (lbm_refine.cu:238,
        // 309); only cells beyond |u| = 0.3 take this branch.
        const float sc = rn_mul(kMaxSimSpeed, rsqrtf(u2));
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

/// Layout of a coarse cell's record by storage. FP32 storage: fneq[19] in
/// FP32, the valid flag, rho, ux, uy, uz -- six float4 (96 B), so the
/// restriction is bit-identical to the reference's. FP16 storage: fneq[19]
/// as halves (the precision of the stored deviations), the valid flag and
/// rho, ux, uy, uz in FP32 -- four float4 (64 B); the restriction's 19
/// neighbour reads per coarse cell then move 48 B each instead of 80 B.
template <class S> struct ChildRecord;

template <> struct ChildRecord<StoreF32> {
    static constexpr int kVec = kScratchVals / 4;
    __device__ __forceinline__ static void write(float4* rec, long long st, const float (&fneq)[kQ], float rho,
                                                 float ux, float uy, float uz) {
        float r[kScratchVals];
#pragma unroll
        for (int q = 0; q < kQ; ++q) r[q] = fneq[q];
        r[kScratchValid] = 1.0f;
        r[kScratchRho] = rho; r[kScratchRho + 1] = ux; r[kScratchRho + 2] = uy; r[kScratchRho + 3] = uz;
#pragma unroll
        for (int k = 0; k < kVec; ++k) rec[k * st] = make_float4(r[4 * k], r[4 * k + 1], r[4 * k + 2], r[4 * k + 3]);
    }
    __device__ __forceinline__ static void write_invalid(float4* rec, long long st) {
        rec[(kScratchValid / 4) * st] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    /// fneq of the record into out; false (out untouched) when not valid.
    __device__ __forceinline__ static bool load(const float4* rec, long long st, float (&out)[kQ]) {
        const float4 v4 = __ldg(rec + (kScratchValid / 4) * st);   // fneq[16..18], valid
        if (v4.w == 0.0f) return false;
        out[16] = v4.x; out[17] = v4.y; out[18] = v4.z;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float4 a = __ldg(rec + k * st);
            out[4 * k] = a.x; out[4 * k + 1] = a.y; out[4 * k + 2] = a.z; out[4 * k + 3] = a.w;
        }
        return true;
    }
    /// acc[q] += fneq[q] for every q when the record is valid.
    __device__ __forceinline__ static bool add(const float4* rec, long long st, float (&acc)[kQ]) {
        const float4 last = __ldg(rec + (kScratchValid / 4) * st);
        if (last.w == 0.0f) return false;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float4 a = __ldg(rec + k * st);
            acc[4 * k] += a.x; acc[4 * k + 1] += a.y; acc[4 * k + 2] += a.z; acc[4 * k + 3] += a.w;
        }
        acc[16] += last.x; acc[17] += last.y; acc[18] += last.z;
        return true;
    }
    __device__ __forceinline__ static float4 moments(const float4* rec, long long st) {
        return __ldg(rec + (kScratchRho / 4) * st);
    }
    /// As add, but every part of the record is read before the valid flag
    /// decides (a select keeps acc when the record is invalid), so the loads
    /// of successive neighbours do not wait on each other's flags.
    __device__ __forceinline__ static bool add_sel(const float4* rec, long long st, float (&acc)[kQ],
                                                   bool use = true) {
        float4 a[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) a[k] = __ldg(rec + k * st);
        const bool ok = use && a[4].w != 0.0f;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            acc[4 * k] = ok ? acc[4 * k] + a[k].x : acc[4 * k];
            acc[4 * k + 1] = ok ? acc[4 * k + 1] + a[k].y : acc[4 * k + 1];
            acc[4 * k + 2] = ok ? acc[4 * k + 2] + a[k].z : acc[4 * k + 2];
            acc[4 * k + 3] = ok ? acc[4 * k + 3] + a[k].w : acc[4 * k + 3];
        }
        acc[16] = ok ? acc[16] + a[4].x : acc[16];
        acc[17] = ok ? acc[17] + a[4].y : acc[17];
        acc[18] = ok ? acc[18] + a[4].z : acc[18];
        return ok;
    }
};

template <> struct ChildRecord<StoreF16> {
    static constexpr int kVec = 4;   // halves 0-7 | halves 8-15 | halves 16-18, valid | rho, u, v, w
    __device__ __forceinline__ static unsigned pack(float a, float b) {
        const __half2 h = __floats2half2_rn(a, b);
        return *reinterpret_cast<const unsigned*>(&h);
    }
    __device__ __forceinline__ static float2 unpack(unsigned u) {
        const __half2 h = *reinterpret_cast<const __half2*>(&u);
        return __half22float2(h);
    }
    __device__ __forceinline__ static void write(float4* rec, long long st, const float (&fneq)[kQ], float rho,
                                                 float ux, float uy, float uz) {
        uint4* r = reinterpret_cast<uint4*>(rec);
        r[0] = make_uint4(pack(fneq[0], fneq[1]), pack(fneq[2], fneq[3]), pack(fneq[4], fneq[5]),
                          pack(fneq[6], fneq[7]));
        r[st] = make_uint4(pack(fneq[8], fneq[9]), pack(fneq[10], fneq[11]), pack(fneq[12], fneq[13]),
                           pack(fneq[14], fneq[15]));
        r[2 * st] = make_uint4(pack(fneq[16], fneq[17]), pack(fneq[18], 0.0f), __float_as_uint(1.0f), 0u);
        rec[3 * st] = make_float4(rho, ux, uy, uz);
    }
    __device__ __forceinline__ static void write_invalid(float4* rec, long long st) {
        reinterpret_cast<uint4*>(rec)[2 * st] = make_uint4(0u, 0u, 0u, 0u);
    }
    __device__ __forceinline__ static bool load(const float4* rec, long long st, float (&out)[kQ]) {
        const uint4 c2 = __ldg(reinterpret_cast<const uint4*>(rec) + 2 * st);
        if (__uint_as_float(c2.z) == 0.0f) return false;
        const float2 p16 = unpack(c2.x), p18 = unpack(c2.y);
        out[16] = p16.x; out[17] = p16.y; out[18] = p18.x;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const uint4 c = __ldg(reinterpret_cast<const uint4*>(rec) + k * st);
            const unsigned w[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float2 p = unpack(w[j]);
                out[8 * k + 2 * j] = p.x; out[8 * k + 2 * j + 1] = p.y;
            }
        }
        return true;
    }
    __device__ __forceinline__ static bool add(const float4* rec, long long st, float (&acc)[kQ]) {
        const uint4 c2 = __ldg(reinterpret_cast<const uint4*>(rec) + 2 * st);
        if (__uint_as_float(c2.z) == 0.0f) return false;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const uint4 c = __ldg(reinterpret_cast<const uint4*>(rec) + k * st);
            const unsigned w[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float2 p = unpack(w[j]);
                acc[8 * k + 2 * j] += p.x; acc[8 * k + 2 * j + 1] += p.y;
            }
        }
        const float2 p16 = unpack(c2.x), p18 = unpack(c2.y);
        acc[16] += p16.x; acc[17] += p16.y; acc[18] += p18.x;
        return true;
    }
    __device__ __forceinline__ static float4 moments(const float4* rec, long long st) { return __ldg(rec + 3 * st); }
    __device__ __forceinline__ static bool add_sel(const float4* rec, long long st, float (&acc)[kQ],
                                                   bool use = true) {
        uint4 c[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) c[k] = __ldg(reinterpret_cast<const uint4*>(rec) + k * st);
        const bool ok = use && __uint_as_float(c[2].z) != 0.0f;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const unsigned w[4] = {c[k].x, c[k].y, c[k].z, c[k].w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float2 p = unpack(w[j]);
                acc[8 * k + 2 * j] = ok ? acc[8 * k + 2 * j] + p.x : acc[8 * k + 2 * j];
                acc[8 * k + 2 * j + 1] = ok ? acc[8 * k + 2 * j + 1] + p.y : acc[8 * k + 2 * j + 1];
            }
        }
        const float2 p16 = unpack(c[2].x), p18 = unpack(c[2].y);
        acc[16] = ok ? acc[16] + p16.x : acc[16];
        acc[17] = ok ? acc[17] + p16.y : acc[17];
        acc[18] = ok ? acc[18] + p18.x : acc[18];
        return ok;
    }
};

/// Record of a coarse cell from the sum fi of its nFluid fluid children
/// (sums of the deviations f - w_q when DEV), at rec = base + t of a planar
/// scratch of stride st.
template <class S, bool DEV = false>
__device__ __forceinline__ void write_child_record(float (&fi)[kQ], int nFluid, float4* rec, long long st) {
    if (nFluid == 0) {
        ChildRecord<S>::write_invalid(rec, st);
        return;
    }
    const float invN = 1.0f / static_cast<float>(nFluid);
#pragma unroll
    for (int q = 0; q < kQ; ++q) fi[q] = DEV ? rn_mul(fi[q], invN) + wgt(q) : rn_mul(fi[q], invN);
    float rho, ux, uy, uz;
    limited_moments(fi, rho, ux, uy, uz);
    const float usq = rn_mul(1.5f, rn_add(rn_add(rn_mul(ux, ux), rn_mul(uy, uy)), rn_mul(uz, uz)));
    float fneq[kQ];
#pragma unroll
    for (int q = 0; q < kQ; ++q) fneq[q] = rn_sub(fi[q], feq_q_rn(q, rho, ux, uy, uz, usq));
    ChildRecord<S>::write(rec, st, fneq, rho, ux, uy, uz);
}

} // namespace fcfd
