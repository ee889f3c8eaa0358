// 2:1 (generally m:1, m = 2..4) refinement-patch coupling, the reference's
// src/sim/lbm_refine.cu:70-429 physics on a GB300 work decomposition.
//
// Coarse -> fine fill: each target fine cell samples the 19 populations at
// its centre by trilinear interpolation over the 8 surrounding coarse cells
// (solid corners dropped and the weights renormalised), blended linearly
// between the two coarse time levels, splits them into feq + fneq, projects
// fneq onto the stress (Latt & Chopard 2006) and rescales it by
// tau_f / (m tau_c) (Dupuis & Chopard 2003). The reference launches this over
// every fine cell and exits early off the interface shell; here the launch
// covers a compact list of target cells (the shell per sub-step, or every
// non-solid fine cell when seeding).
//
// Fine -> coarse restriction: per coarse fluid cell of the patch minus a
// 2-cell band, average the m^3 fine children (solid children skipped), take
// fneq against the average's own equilibrium, filter fneq over the cell and
// its 18 lattice neighbours (Lagrava et al. 2012), regularise, rescale by
// m tau_c / tau_f and blend into the coarse post-collision state over a
// 3-cell edge ramp. The reference recomputes each neighbour's child average
// inside the filter (19 averages per cell); here pass 1 stores every child
// average once in scratch (one 96-byte record per coarse cell, stored
// planar: see child_record.cuh) and pass 2 filters from scratch.
//
// Built with --fmad=false: every expression keeps the reference's rounding,
// so fill and restriction are bit-identical to the reference kernels
// compiled without contraction (the limiter's rsqrtf is the same hardware
// instruction the reference's GPU build uses).
#include "child_record.cuh"
#include "d3q19.cuh"
#include "kernels.h"

#include <cuda_runtime.h>

#include <type_traits>

namespace fcfd {
namespace {

constexpr int kRefineBlock = 128;
constexpr int kRestrictBand = 2;   // coarse band skipped by the restriction
constexpr int kRestrictBlend = 3;  // edge-blend ramp width (coarse cells)

/// v folded into [0, n) for v in [-n, 2n): the fill's corners lie at most one
/// cell outside the coarse domain, so a compare replaces the division.
__device__ __forceinline__ int wrap1(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

/// Latt-Chopard projection of fneq onto the second-order Hermite space.
__device__ __forceinline__ void regularize(float (&fneq)[kQ]) {
    float pxx = 0.f, pyy = 0.f, pzz = 0.f, pxy = 0.f, pxz = 0.f, pyz = 0.f;
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
        const float v = fneq[q];
        pxx += cx(q) * cx(q) * v; pyy += cy(q) * cy(q) * v; pzz += cz(q) * cz(q) * v;
        pxy += cx(q) * cy(q) * v; pxz += cx(q) * cz(q) * v; pyz += cy(q) * cz(q) * v;
    }
    const float trace = (1.0f / 3.0f) * (pxx + pyy + pzz);
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
        const float qpi = cx(q) * cx(q) * pxx + cy(q) * cy(q) * pyy + cz(q) * cz(q) * pzz
                        + 2.0f * (cx(q) * cy(q) * pxy + cx(q) * cz(q) * pxz + cy(q) * cz(q) * pyz)
                        - trace;
        fneq[q] = 4.5f * wgt(q) * qpi;
    }
}


/// BLEND false: a time weight of 0, where s0 + 0 (s1 - s0) is s0 itself
/// (the sign of a zero sum aside, for which s1 is read), so the second time
/// level is not read. Identical to the blended form whenever the second
/// level is finite.
template <class S, bool BLEND>
__global__ void __launch_bounds__(kRefineBlock)
fill_kernel(const typename S::T* __restrict__ cT0, const typename S::T* __restrict__ cT1,
            const std::uint8_t* __restrict__ ckind, typename S::T* __restrict__ ff,
            const std::uint32_t* __restrict__ targets, int count, RefineGeom g, float invFactor,
            float tw, float neqScale, FastDiv divX, FastDiv divXY) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const std::uint32_t t = targets[i];
    const int zf = static_cast<int>(fdiv(t, divXY));
    const unsigned rem = t - static_cast<unsigned>(zf) * divXY.d;
    const int yf = static_cast<int>(fdiv(rem, divX));
    const int xf = static_cast<int>(rem - static_cast<unsigned>(yf) * divX.d);

    const float gx = static_cast<float>(g.boxX0) + (static_cast<float>(xf) + 0.5f) * invFactor - 0.5f;
    const float gy = static_cast<float>(g.boxY0) + (static_cast<float>(yf) + 0.5f) * invFactor - 0.5f;
    const float gz = (static_cast<float>(zf) + 0.5f) * invFactor - 0.5f;
    const int ix = static_cast<int>(floorf(gx)), iy = static_cast<int>(floorf(gy));
    const int iz = static_cast<int>(floorf(gz));
    const float tx = gx - ix, ty = gy - iy, tz = gz - iz;

    float w8[8];
    w8[0] = (1 - tx) * (1 - ty) * (1 - tz);
    w8[1] = tx * (1 - ty) * (1 - tz);
    w8[2] = (1 - tx) * ty * (1 - tz);
    w8[3] = tx * ty * (1 - tz);
    w8[4] = (1 - tx) * (1 - ty) * tz;
    w8[5] = tx * (1 - ty) * tz;
    w8[6] = (1 - tx) * ty * tz;
    w8[7] = tx * ty * tz;
    const int cnx = g.coarse.nx, cny = g.coarse.ny, cnz = g.coarse.nz;
    std::uint32_t corner[8];
    float wsum = 0.0f;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int X = wrap1(ix + (c & 1), cnx), Y = wrap1(iy + ((c >> 1) & 1), cny);
        const int Z = wrap1(iz + ((c >> 2) & 1), cnz);
        corner[c] = static_cast<std::uint32_t>(X) + static_cast<std::uint32_t>(cnx)
                  * (static_cast<std::uint32_t>(Y) + static_cast<std::uint32_t>(cny) * Z);
        if ((ckind[corner[c]] & kFlagMask) == kSolid) w8[c] = 0.0f;
        wsum += w8[c];
    }
    if (wsum < 1e-6f) return; // fully inside a parent solid: leave it
    const float iws = 1.0f / wsum;
#pragma unroll
    for (int c = 0; c < 8; ++c) w8[c] *= iws;

    const long long cn = g.coarse.cells(), fn = g.fine.cells();
    float fi[kQ];
    // FP16 storage sums the stored deviations and adds w_q once: with the
    // corner weights summing to one, sum w8 (w_q + g) = w_q + sum w8 g up to
    // rounding, without a weight add per corner load. FP32 keeps the
    // reference's expression.
    constexpr bool kDev = std::is_same_v<S, StoreF16>;
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
        float s0 = 0.0f, s1 = 0.0f;
        if constexpr (kDev) {
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                s0 += w8[c] * S::ld_dev(cT0 + q * cn, corner[c], wgt(q));
                if constexpr (BLEND) s1 += w8[c] * S::ld_dev(cT1 + q * cn, corner[c], wgt(q));
            }
            fi[q] = wgt(q) + (BLEND ? s0 + tw * (s1 - s0) : s0);
        } else if constexpr (BLEND) {
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                s0 += w8[c] * S::ld(cT0 + q * cn, corner[c], wgt(q));
                s1 += w8[c] * S::ld(cT1 + q * cn, corner[c], wgt(q));
            }
            fi[q] = s0 + tw * (s1 - s0);
        } else {
#pragma unroll
            for (int c = 0; c < 8; ++c) s0 += w8[c] * S::ld(cT0 + q * cn, corner[c], wgt(q));
            if (s0 == 0.0f) {
#pragma unroll
                for (int c = 0; c < 8; ++c) s1 += w8[c] * S::ld(cT1 + q * cn, corner[c], wgt(q));
                s0 = s0 + tw * (s1 - s0);
            }
            fi[q] = s0;
        }
    }
    float rho, ux, uy, uz;
    limited_moments(fi, rho, ux, uy, uz);
    const float usq = 1.5f * (ux * ux + uy * uy + uz * uz);
    float feq[kQ], fneq[kQ];
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
        feq[q] = feq_q(q, rho, ux, uy, uz, usq);
        fneq[q] = fi[q] - feq[q];
    }
    regularize(fneq);
#pragma unroll
    for (int q = 0; q < kQ; ++q) S::st(ff + q * fn, t, feq[q] + neqScale * fneq[q], wgt(q));
}

/// Pass 1: child average of every coarse cell of the restricted sub-box, as
/// one 96-byte record per coarse cell (six float4).
template <class S>
__global__ void __launch_bounds__(kRefineBlock)
child_avg_kernel(const typename S::T* __restrict__ ff, const std::uint8_t* __restrict__ fkind,
                 RefineGeom g, int rx0, int ry0, int rw, int rh, float* __restrict__ scratch) {
    const int lx = blockIdx.x * blockDim.x + threadIdx.x;
    if (lx >= rw) return;
    const int ly = blockIdx.y, zc = blockIdx.z;
    const long long t = lx + static_cast<long long>(rw) * (ly + static_cast<long long>(rh) * zc);
    const int m = g.factor;
    const int fx = m * (rx0 + lx - g.boxX0), fy = m * (ry0 + ly - g.boxY0), fz = m * zc;
    const long long fn = g.fine.cells();
    const unsigned fnx = g.fine.nx, fnxy = static_cast<unsigned>(g.fine.nx) * g.fine.ny;
    float fi[kQ];
#pragma unroll
    for (int q = 0; q < kQ; ++q) fi[q] = 0.0f;
    int nFluid = 0;
    for (int k = 0; k < m; ++k)
        for (int j = 0; j < m; ++j)
            for (int i = 0; i < m; ++i) {
                const unsigned c = static_cast<unsigned>(fx + i) + fnx * static_cast<unsigned>(fy + j)
                                 + fnxy * static_cast<unsigned>(fz + k);
                if ((fkind[c] & kFlagMask) == kSolid) continue;
                ++nFluid;
#pragma unroll
                for (int q = 0; q < kQ; ++q) fi[q] += S::ld(ff + q * fn, c, wgt(q));
            }
    const long long nrec = static_cast<long long>(rw) * rh * g.coarse.nz;
    write_child_record<S>(fi, nFluid, reinterpret_cast<float4*>(scratch) + t, nrec);
}

constexpr int kRestrictTX = 32, kRestrictTY = 2, kRestrictTZ = 2;

template <class S>
__global__ void __launch_bounds__(kRestrictTX * kRestrictTY * kRestrictTZ)
restrict_kernel(typename S::T* __restrict__ fc, const std::uint8_t* __restrict__ ckind,
                RefineGeom g, int rx0, int ry0, int rw, int rh, float neqScaleInv,
                const float* __restrict__ scratch, float* __restrict__ mRho,
                float* __restrict__ mU, float* __restrict__ mV, float* __restrict__ mW) {
    const int lx = blockIdx.x * kRestrictTX + threadIdx.x;
    const int ly = blockIdx.y * kRestrictTY + threadIdx.y;
    const int zc = blockIdx.z * kRestrictTZ + threadIdx.z;
    const int nz = g.coarse.nz;
    if (lx >= rw || ly >= rh || zc >= nz) return;
    const long long t = lx + static_cast<long long>(rw) * (ly + static_cast<long long>(rh) * zc);
    const int xc = rx0 + lx, yc = ry0 + ly;
    const long long cn = g.coarse.cells();
    const unsigned cell = static_cast<unsigned>(xc) + static_cast<unsigned>(g.coarse.nx)
                        * (static_cast<unsigned>(yc) + static_cast<unsigned>(g.coarse.ny) * zc);
    if ((ckind[cell] & kFlagMask) != kFluid) return;
    const float4* rec = reinterpret_cast<const float4*>(scratch);
    const long long nrec = static_cast<long long>(rw) * rh * nz;
    float fneq[kQ];
    if (!ChildRecord<S>::load(rec + t, nrec, fneq)) return;

    const int dEdge = min(min(lx, rw - 1 - lx), min(ly, rh - 1 - ly));
    const float blend = fminf(1.0f, static_cast<float>(dEdge + 1) / static_cast<float>(kRestrictBlend + 1));

    int nStencil = 1;
#pragma unroll
    for (int nb = 1; nb < kQ; ++nb) {
        const int nlx = lx + cx(nb), nly = ly + cy(nb);
        // A neighbour outside the box reads the cell's own record and is
        // dropped by the select, so no neighbour's loads wait on a branch.
        const bool inBox = nlx >= 0 && nlx < rw && nly >= 0 && nly < rh;
        const int nzw = zc + cz(nb) < 0 ? nz - 1 : (zc + cz(nb) >= nz ? 0 : zc + cz(nb));
        const long long tn = inBox ? nlx + static_cast<long long>(rw) * (nly + static_cast<long long>(rh) * nzw) : t;
        // Same per-q accumulation order as summing slot by slot.
        nStencil += ChildRecord<S>::add_sel(rec + tn, nrec, fneq, inBox) ? 1 : 0;
    }
    const float invS = 1.0f / static_cast<float>(nStencil);
#pragma unroll
    for (int q = 0; q < kQ; ++q) fneq[q] *= invS;
    regularize(fneq);
    const float4 m4 = ChildRecord<S>::moments(rec + t, nrec);
    const float rho = m4.x, ux = m4.y, uy = m4.z, uz = m4.w;
    const float usq = 1.5f * (ux * ux + uy * uy + uz * uz);
    float br = 0.f, bjx = 0.f, bjy = 0.f, bjz = 0.f;
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
        const float restricted = feq_q(q, rho, ux, uy, uz, usq) + neqScaleInv * fneq[q];
        const float existing = S::ld(fc + q * cn, cell, wgt(q));
        const float b = existing + blend * (restricted - existing);
        S::st(fc + q * cn, cell, b, wgt(q));
        br += b; bjx += cx(q) * b; bjy += cy(q) * b; bjz += cz(q) * b;
    }
    if (mRho) {
        br = fmaxf(br, kRhoFloor);
        const float bi = 1.0f / br;
        mRho[cell] = br; mU[cell] = bjx * bi; mV[cell] = bjy * bi; mW[cell] = bjz * bi;
    }
}

inline void sub_box(const RefineGeom& g, int& rx0, int& ry0, int& rw, int& rh) {
    rx0 = g.boxX0 + kRestrictBand;
    ry0 = g.boxY0 + kRestrictBand;
    rw = (g.boxX1 - kRestrictBand) - rx0;
    rh = (g.boxY1 - kRestrictBand) - ry0;
}

} // namespace

cudaError_t launch_fill_c2f(Storage s, const void* cT0, const void* cT1,
                            const std::uint8_t* coarseKind, void* fineF,
                            const std::uint32_t* targets, int count, const RefineGeom& g,
                            float timeWeight, float neqScale, cudaStream_t st) {
    if (!cT0 || !cT1 || !coarseKind || !fineF || g.factor < 2 || g.factor > 4)
        return cudaErrorInvalidValue;
    if (count <= 0) return cudaSuccess;
    const unsigned nb = static_cast<unsigned>((count + kRefineBlock - 1) / kRefineBlock);
    const float invF = 1.0f / static_cast<float>(g.factor);
    const bool blend = timeWeight != 0.0f;
    const FastDiv dx = fast_div(static_cast<unsigned>(g.fine.nx));
    const FastDiv dxy = fast_div(static_cast<unsigned>(g.fine.nx) * static_cast<unsigned>(g.fine.ny));
    if (s == Storage::F32)
        (blend ? fill_kernel<StoreF32, true> : fill_kernel<StoreF32, false>)<<<nb, kRefineBlock, 0, st>>>(
            static_cast<const float*>(cT0), static_cast<const float*>(cT1), coarseKind,
            static_cast<float*>(fineF), targets, count, g, invF, timeWeight, neqScale, dx, dxy);
    else
        (blend ? fill_kernel<StoreF16, true> : fill_kernel<StoreF16, false>)<<<nb, kRefineBlock, 0, st>>>(
            static_cast<const __half*>(cT0), static_cast<const __half*>(cT1), coarseKind,
            static_cast<__half*>(fineF), targets, count, g, invF, timeWeight, neqScale, dx, dxy);
    return cudaGetLastError();
}

long long restrict_scratch_floats(const RefineGeom& g) {
    int rx0, ry0, rw, rh;
    sub_box(g, rx0, ry0, rw, rh);
    if (rw <= 0 || rh <= 0) return 0;
    return static_cast<long long>(kScratchVals) * rw * rh * g.coarse.nz;
}

void restrict_sub_box(const RefineGeom& g, int& rx0, int& ry0, int& rw, int& rh) { sub_box(g, rx0, ry0, rw, rh); }

cudaError_t launch_restrict_f2c(Storage s, const void* fineF, const std::uint8_t* fineKind,
                                void* coarseF, const std::uint8_t* coarseKind,
                                const RefineGeom& g, float neqScaleInv, float* scratch,
                                float* rho, float* u, float* v, float* w, cudaStream_t st, bool childDone) {
    int rx0, ry0, rw, rh;
    sub_box(g, rx0, ry0, rw, rh);
    if (!fineF || !fineKind || !coarseF || !coarseKind || !scratch || rw <= 0 || rh <= 0
        || g.factor < 2 || g.factor > 4)
        return cudaErrorInvalidValue;
    const dim3 grid(static_cast<unsigned>((rw + kRefineBlock - 1) / kRefineBlock),
                    static_cast<unsigned>(rh), static_cast<unsigned>(g.coarse.nz));
    const bool macro = rho && u && v && w;
    const dim3 rblock(kRestrictTX, kRestrictTY, kRestrictTZ);
    const dim3 rgrid(static_cast<unsigned>((rw + kRestrictTX - 1) / kRestrictTX),
                     static_cast<unsigned>((rh + kRestrictTY - 1) / kRestrictTY),
                     static_cast<unsigned>((g.coarse.nz + kRestrictTZ - 1) / kRestrictTZ));
    if (s == Storage::F32) {
        if (!childDone)
            child_avg_kernel<StoreF32><<<grid, kRefineBlock, 0, st>>>(
                static_cast<const float*>(fineF), fineKind, g, rx0, ry0, rw, rh, scratch);
        restrict_kernel<StoreF32><<<rgrid, rblock, 0, st>>>(
            static_cast<float*>(coarseF), coarseKind, g, rx0, ry0, rw, rh, neqScaleInv, scratch,
            macro ? rho : nullptr, u, v, w);
    } else {
        if (!childDone)
            child_avg_kernel<StoreF16><<<grid, kRefineBlock, 0, st>>>(
                static_cast<const __half*>(fineF), fineKind, g, rx0, ry0, rw, rh, scratch);
        restrict_kernel<StoreF16><<<rgrid, rblock, 0, st>>>(
            static_cast<__half*>(coarseF), coarseKind, g, rx0, ry0, rw, rh, neqScaleInv, scratch,
            macro ? rho : nullptr, u, v, w);
    }
    return cudaGetLastError();
}

} // namespace fcfd
