// iMEM slip-velocity wall function (Asmuth et al., Phys. Fluids 33:105111),
// the device half of the reference's wall model (src/sim/lbm_wallmodel.cu:
// 31-196): per listed wall cell, sample the velocity a few cells off the wall,
// Newton-solve Reichardt's law for u_tau (6 FP32 iterations, warm-started from
// the stored value), EMA-blend it, then solve the balance -- linear in u_w --
// that makes the cell's bounce-back links carry the modelled shear stress;
// fade the slip for sampled y+ in 3..6, clamp it, store it as half bits.
//
// The list is SoA with 32-bit cell indices (one thread per entry, coalesced);
// the Reichardt evaluation uses the fast __logf/__expf intrinsics like the
// reference, so the update agrees with it to FP32 rounding of those.
#include "d3q19.cuh"
#include "kernels.h"

#include <cuda_runtime.h>

namespace fcfd {
namespace {

constexpr float kKappa = 0.41f;      // von Karman constant
constexpr float kReichardtC = 7.8f;  // Reichardt outer coefficient
constexpr float kFadeY0 = 3.0f;      // low-y+ fade band
constexpr float kFadeY1 = 6.0f;
constexpr int kWallBlock = 128;

/// Reichardt's all-y+ law u+(y+).
__device__ __forceinline__ float reichardt(float yp) {
    return __logf(1.0f + kKappa * yp) / kKappa
         + kReichardtC * (1.0f - __expf(-yp / 11.0f) - (yp / 11.0f) * __expf(-yp / 3.0f));
}
/// d u+ / d y+ of Reichardt's law.
__device__ __forceinline__ float reichardt_d(float yp) {
    return 1.0f / (1.0f + kKappa * yp)
         + kReichardtC * ((1.0f / 11.0f) * __expf(-yp / 11.0f)
                          - (1.0f / 11.0f) * __expf(-yp / 3.0f)
                          + (yp / 33.0f) * __expf(-yp / 3.0f));
}

/// Newton on g(u_tau) = u_tau u+(y_s u_tau / nu) - u_t, 6 iterations.
__device__ __forceinline__ float solve_utau(float ut, float ys, float nu, float seed) {
    float utau = seed > 0.0f ? seed : fmaxf(0.04f * ut, sqrtf(nu * ut / ys));
#pragma unroll
    for (int it = 0; it < 6; ++it) {
        const float yp = fmaxf(ys * utau / nu, 1e-8f);
        const float up = reichardt(yp);
        const float g = utau * up - ut;
        const float dg = up + yp * reichardt_d(yp);
        utau -= g / fmaxf(dg, 1e-6f);
        utau = fmaxf(utau, 0.0f);
    }
    return utau;
}

template <class S>
__global__ void __launch_bounds__(kWallBlock)
wall_update_kernel(const typename S::T* __restrict__ f, long long n, WallListDev L,
                   std::uint16_t* __restrict__ uwx, std::uint16_t* __restrict__ uwy,
                   std::uint16_t* __restrict__ uwz, float nu, float utCut, float ema,
                   WallStatsDev* __restrict__ stats) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= L.count) return;
    const std::uint32_t cell = L.cellIdx[i];
    const float nX = L.nX[i], nY = L.nY[i], nZ = L.nZ[i];

    // Moments at the sample cell.
    const std::uint32_t sc = L.sampleIdx[i];
    float rho = 0.0f, jx = 0.0f, jy = 0.0f, jz = 0.0f;
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
        const float v = S::ld(f + q * n, sc, wgt(q));
        rho += v; jx += cx(q) * v; jy += cy(q) * v; jz += cz(q) * v;
    }
    rho = fmaxf(rho, kRhoFloor);
    const float inv = 1.0f / rho;
    const float ux = jx * inv, uy = jy * inv, uz = jz * inv;

    // Tangential component.
    const float un = ux * nX + uy * nY + uz * nZ;
    const float tx = ux - un * nX, ty = uy - un * nY, tz = uz - un * nZ;
    const float ut = sqrtf(tx * tx + ty * ty + tz * tz);
    if (ut < utCut) {
        // No meaningful tangential flow: plain bounce-back at this cell.
        L.uTau[i] = 0.0f;
        uwx[cell] = 0; uwy[cell] = 0; uwz[cell] = 0;
        return;
    }
    const float itx = tx / ut, ity = ty / ut, itz = tz / ut;

    const float ys = L.ys[i];
    const float prev = L.uTau[i];
    const float solved = solve_utau(ut, ys, nu, prev);
    const float utau = prev > 0.0f ? prev + ema * (solved - prev) : solved;
    L.uTau[i] = utau;

    // Wall force along t: F_t = M0 - u_w D over the solid links (outgoing
    // direction o = opp(q), c_o = -c_q).
    float m0 = 0.0f, dcoef = 0.0f;
    const std::uint32_t mask = L.linkMask[i];
#pragma unroll
    for (int q = 1; q < kQ; ++q) {
        if (!(mask & (1u << q))) continue;
        const int o = opp(q);
        const float ct = -(cx(q) * itx + cy(q) * ity + cz(q) * itz);
        const float fo = S::ld(f + o * n, cell, wgt(o));
        m0 += 2.0f * fo * ct;
        dcoef += 6.0f * wgt(q) * ct * ct;
    }
    // Stair-step facet area from the normal (45 degrees -> sqrt 2).
    const float maxN = fmaxf(fabsf(nX), fmaxf(fabsf(nY), fabsf(nZ)));
    const float aw = 1.0f / fmaxf(maxN, 0.1f);
    float uw = 0.0f;
    if (dcoef > 1e-6f) {
        const float target = rho * utau * utau * aw;
        const float sgn = m0 >= 0.0f ? 1.0f : -1.0f;
        uw = (m0 - sgn * target) / dcoef;
    }
    const float ypS = ys * utau / nu;
    const float fade = fminf(fmaxf((ypS - kFadeY0) / (kFadeY1 - kFadeY0), 0.0f), 1.0f);
    uw *= fade;
    const float cap = fminf(0.5f * ut, 0.5f * kMaxSimSpeed);
    const float uwc = fminf(fmaxf(uw, -cap), cap);
    uwx[cell] = __half_as_ushort(__float2half_rn(uwc * itx));
    uwy[cell] = __half_as_ushort(__float2half_rn(uwc * ity));
    uwz[cell] = __half_as_ushort(__float2half_rn(uwc * itz));

    const float yplus = ys * utau / nu;
    atomicAdd(&stats->sumYplus, yplus);
    atomicMax(&stats->maxYplusBits, __float_as_int(fmaxf(yplus, 0.0f)));
    atomicAdd(&stats->activeCells, 1);
    if (uwc != uw) atomicAdd(&stats->clampedCells, 1);
}

} // namespace

cudaError_t launch_wall_update(Storage s, const void* f, long long cells, WallListDev list,
                               std::uint16_t* uwx, std::uint16_t* uwy, std::uint16_t* uwz,
                               float nuLat, float utCutoff, float emaAlpha, WallStatsDev* stats,
                               cudaStream_t st) {
    if (list.count <= 0 || !list.cellIdx || !list.uTau || !f || !uwx || !uwy || !uwz || !stats)
        return cudaErrorInvalidValue;
    if (auto e = cudaMemsetAsync(stats, 0, sizeof(WallStatsDev), st); e != cudaSuccess) return e;
    const unsigned nb = static_cast<unsigned>((list.count + kWallBlock - 1) / kWallBlock);
    if (s == Storage::F32)
        wall_update_kernel<StoreF32><<<nb, kWallBlock, 0, st>>>(static_cast<const float*>(f), cells, list, uwx, uwy, uwz, nuLat, utCutoff, emaAlpha, stats);
    else
        wall_update_kernel<StoreF16><<<nb, kWallBlock, 0, st>>>(static_cast<const __half*>(f), cells, list, uwx, uwy, uwz, nuLat, utCutoff, emaAlpha, stats);
    return cudaGetLastError();
}

} // namespace fcfd
