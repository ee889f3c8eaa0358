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
// reference, so the update agrees with it to FP32 rounding of those. The
// statistics (sum and max of y+, active and clamped cells) are aggregated per
// warp before their atomics (the reference issues four atomics per cell).
//
// Two further u_tau solves can replace the reference's (template METHOD):
// full FP64 Newton to a relative step of 1e-8 from the same seed, and the
// learned seed (a 3-32-32-1 network, BF16 weights in shared memory, its
// hidden layer a warp-wide tensor-core contraction over the warp's 32 wall
// cells) with one FP32 correction and an FP64 fallback (wallnet.cuh).
//
// Kernels in an anonymous namespace, included by two translation units:
// wall_kernels.cu (FP16 storage and the harvest; nvcc's default multiply-add
// contraction) and wall_kernels_x.cu (FP32 storage, --fmad=false: the
// reference's expressions rounded as written, bit-identical to the
// reference's wall update compiled without contraction).
#pragma once

#include "d3q19.cuh"
#include "kernels.h"
#include "wallnet.cuh"

#include <cuda_runtime.h>

namespace fcfd {
namespace {

constexpr float kFadeY0 = 3.0f;      // low-y+ fade band
constexpr float kFadeY1 = 6.0f;
constexpr int kWallBlock = 128;

/// Moments at a wall entry's sample cell -> density and velocity.
template <class S>
__device__ __forceinline__ void sample_velocity(const typename S::T* __restrict__ f, long long n, std::uint32_t sc,
                                                float& rho, float& ux, float& uy, float& uz) {
    float r = 0.0f, jx = 0.0f, jy = 0.0f, jz = 0.0f;
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
        const float v = S::ld(f + q * n, sc, wgt(q));
        r += v; jx += cx(q) * v; jy += cy(q) * v; jz += cz(q) * v;
    }
    rho = fmaxf(r, kRhoFloor);
    const float inv = 1.0f / rho;
    ux = jx * inv; uy = jy * inv; uz = jz * inv;
}

template <class S, int METHOD>
__global__ void __launch_bounds__(kWallBlock)
wall_update_kernel(const typename S::T* __restrict__ f, long long n, WallListDev L,
                   std::uint16_t* __restrict__ uwx, std::uint16_t* __restrict__ uwy,
                   std::uint16_t* __restrict__ uwz, float nu, float utCut, float ema,
                   WallStatsDev* __restrict__ stats, wallnet::NetDev net) {
    constexpr bool kNet = METHOD == 2;
    __shared__ float P[kNet ? wallnet::kParams : 1];
    if (kNet) {
        wallnet::load_params(net.w, P);
        __syncthreads();
    }
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool active = false, clamped = false;
    int fallback = 0, iters = 0;
    float yplus = 0.0f;
    const bool valid = i < L.count;
    std::uint32_t cell = 0;
    float nX = 0.0f, nY = 0.0f, nZ = 0.0f, rho = 1.0f, tx = 0.0f, ty = 0.0f, tz = 0.0f, ut = 0.0f, ys = 1.0f;
    if (valid) {
        cell = L.cellIdx[i];
        nX = L.nX[i]; nY = L.nY[i]; nZ = L.nZ[i];
        float ux, uy, uz;
        sample_velocity<S>(f, n, L.sampleIdx[i], rho, ux, uy, uz);
        // Tangential component.
        const float un = ux * nX + uy * nY + uz * nZ;
        tx = ux - un * nX; ty = uy - un * nY; tz = uz - un * nZ;
        ut = sqrtf(tx * tx + ty * ty + tz * tz);
        ys = L.ys[i];
    }
    const bool on = valid && !(ut < utCut);
    // The learned seed is evaluated by the whole warp together.
    float netSeed = 0.0f;
    if constexpr (kNet) netSeed = wallnet::net_seed_warp(P, net.norm, ut, ys, nu, on);
    if (valid) {
        if (!on) {
            // No meaningful tangential flow: plain bounce-back at this cell.
            L.uTau[i] = 0.0f;
            uwx[cell] = 0; uwy[cell] = 0; uwz[cell] = 0;
        } else {
            active = true;
            const float itx = tx / ut, ity = ty / ut, itz = tz / ut;
            const float prev = L.uTau[i];
            float solved;
            if (METHOD == 0) {
                solved = wallnet::newton_reference(ut, ys, nu, wallnet::reference_seed(ut, ys, nu, prev));
            } else if (METHOD == 1) {
                solved = static_cast<float>(wallnet::newton64(ut, ys, nu, wallnet::reference_seed(ut, ys, nu, prev), &iters));
            } else {
                solved = wallnet::learned_correct(ut, ys, nu, netSeed, &fallback, &iters);
            }
            const float utau = prev > 0.0f ? prev + ema * (solved - prev) : solved;
            L.uTau[i] = utau;

            // Wall force along t: F_t = M0 - u_w D over the solid links
            // (outgoing direction o = opp(q), c_o = -c_q).
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
            yplus = fmaxf(ys * utau / nu, 0.0f);
            clamped = uwc != uw;
        }
    }

    // Warp-aggregated statistics.
    const unsigned act = __ballot_sync(0xffffffffu, active);
    const unsigned clp = __ballot_sync(0xffffffffu, clamped);
    const unsigned fbk = __ballot_sync(0xffffffffu, fallback != 0);
    float sum = yplus;
    int mx = __float_as_int(yplus);
    unsigned long long its = static_cast<unsigned long long>(iters);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_down_sync(0xffffffffu, sum, o);
        mx = max(mx, __shfl_down_sync(0xffffffffu, mx, o));
        its += __shfl_down_sync(0xffffffffu, its, o);
    }
    if ((threadIdx.x & 31) == 0 && act) {
        atomicAdd(&stats->sumYplus, sum);
        atomicMax(&stats->maxYplusBits, mx);
        atomicAdd(&stats->activeCells, __popc(act));
        if (clp) atomicAdd(&stats->clampedCells, __popc(clp));
        if (fbk) atomicAdd(&stats->fallbackCells, __popc(fbk));
        if (its) atomicAdd(&stats->newtonIters, its);
    }
}

template <class S>
__global__ void __launch_bounds__(kWallBlock)
wall_harvest_kernel(const typename S::T* __restrict__ f, long long n, WallListDev L, float utCut,
                    float* __restrict__ utOut, float* __restrict__ ysOut) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= L.count) return;
    const float nX = L.nX[i], nY = L.nY[i], nZ = L.nZ[i];
    float rho, ux, uy, uz;
    sample_velocity<S>(f, n, L.sampleIdx[i], rho, ux, uy, uz);
    const float un = ux * nX + uy * nY + uz * nZ;
    const float tx = ux - un * nX, ty = uy - un * nY, tz = uz - un * nZ;
    const float ut = sqrtf(tx * tx + ty * ty + tz * tz);
    utOut[i] = ut < utCut ? 0.0f : ut;
    ysOut[i] = L.ys[i];
}

template <class S, int M>
void launch_wall(const void* f, long long cells, WallListDev list, std::uint16_t* uwx, std::uint16_t* uwy,
                 std::uint16_t* uwz, float nu, float cut, float ema, WallStatsDev* stats, wallnet::NetDev net,
                 cudaStream_t st) {
    const unsigned nb = static_cast<unsigned>((list.count + kWallBlock - 1) / kWallBlock);
    wall_update_kernel<S, M><<<nb, kWallBlock, 0, st>>>(static_cast<const typename S::T*>(f), cells, list, uwx, uwy,
                                                        uwz, nu, cut, ema, stats, net);
}

template <class S>
void launch_wall_method(int method, const void* f, long long cells, WallListDev list, std::uint16_t* uwx,
                        std::uint16_t* uwy, std::uint16_t* uwz, float nu, float cut, float ema, WallStatsDev* stats,
                        wallnet::NetDev net, cudaStream_t st) {
    if (method == 1) launch_wall<S, 1>(f, cells, list, uwx, uwy, uwz, nu, cut, ema, stats, net, st);
    else if (method == 2) launch_wall<S, 2>(f, cells, list, uwx, uwy, uwz, nu, cut, ema, stats, net, st);
    else launch_wall<S, 0>(f, cells, list, uwx, uwy, uwz, nu, cut, ema, stats, net, st);
}


template <class S>
cudaError_t wall_update_launch(Storage s, const void* f, long long cells, WallListDev list, std::uint16_t* uwx,
                               std::uint16_t* uwy, std::uint16_t* uwz, float nuLat, float utCutoff, float emaAlpha,
                               WallStatsDev* stats, cudaStream_t st, int method, const wallnet::NetDev* net) {
    (void)s;
    if (list.count <= 0 || !list.cellIdx || !list.uTau || !f || !uwx || !uwy || !uwz || !stats)
        return cudaErrorInvalidValue;
    if (method < 0 || method > 2 || (method == 2 && (!net || !net->w))) return cudaErrorInvalidValue;
    if (auto e = cudaMemsetAsync(stats, 0, sizeof(WallStatsDev), st); e != cudaSuccess) return e;
    const wallnet::NetDev nd = net ? *net : wallnet::NetDev{};
    launch_wall_method<S>(method, f, cells, list, uwx, uwy, uwz, nuLat, utCutoff, emaAlpha, stats, nd, st);
    return cudaGetLastError();
}

} // namespace
} // namespace fcfd
