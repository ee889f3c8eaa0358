// Per-cell building blocks of the stream-collide kernels and the kernel
// templates built from them: the one-cell-per-thread kernels (per row and
// over the flattened lattice), the fine collide with the restriction's child
// sums fused in, the staged kernel that streams x-rows through shared memory
// with bulk async copies, and the AA-pattern in-place kernels.
//
// Physics follows the reference step (src/sim/lbm_core.cu:213-475): per link
// the upstream neighbour's flag selects plain streaming, half-way bounce-back
// (opposite slot of this cell) or specular free slip (mirrored slot of the
// tangentially displaced cell); inlet cells are written with feq(1, u_in),
// outlets copy the upstream column; moments with a density floor of 0.05; a
// |u| <= 0.3 limiter; Smagorinsky tau_eff from the non-equilibrium stress
// (Hou et al. 1996); TRT with magic parameter Lambda.
//
// Two collision bodies, selected by the EXACT template flag:
//  * collide_exact: the reference kernel's expression tree (lbm_core.cu:
//    386-467) with zero-coefficient terms skipped (an exact identity). It is
//    bit-identical to the reference only in a translation unit compiled with
//    --fmad=false (collide_f32.cu), where no multiply-add is contracted.
//  * collide_dev: the same TRT + Smagorinsky update on the deviations
//    g_q = f_q - w_q (the FP16 storage format), with moments, stress and
//    TRT formed from opposite-pair sums/differences and the equilibrium's
//    second moment in closed form (rho/3 I + rho u u); reciprocals and square
//    roots by the hardware approximations. Fewer instructions, no weight add
//    per load or subtract per store, FP32-rounding-level different.
// Population access follows the body: Pop<S, DEV> loads and stores f (exact
// body) or g (deviation body); a bounce-back or mirrored slot has the weight
// of the link it replaces and the Ladd and interpolated bounce-back terms are
// affine with unit coefficient sum, so every gather path is the same in both
// forms.
//
// This header is included by exactly one translation unit per instantiation
// set; the kernels live in an anonymous namespace.
#pragma once

#include "child_record.cuh"
#include "d3q19.cuh"
#include "kernels.h"

#include <cuda_runtime.h>

#include <type_traits>

namespace fcfd {
namespace {

struct CollideArgs {
    int nx, ny, nz;
    long long n; // cells per direction slice
    float tau0, lambda, smagPre, uIn;
    int writeMacro;
    float *rho, *u, *v, *w;
    const std::uint16_t *uwx, *uwy, *uwz;
    int* status; // staged kernel: nonzero when a pipeline wait timed out
    const std::uint8_t* qFrac;   // q-LIBB cut bytes [cell * 19 + q], or null
    const std::uint32_t* ffMask; // q-LIBB two-node bits [cell]
    const uint2* links;          // pull-link classes per cell (launch_classify), or null
};

/// Byte offsets of the pulls of an interior cell (no periodic wrap on any
/// axis), from the cell's own slot in direction slice 0: pull[q] reaches the
/// source x - c_q in slice q, slice[q] the cell itself in slice q. Passed as
/// a __grid_constant__ kernel parameter, so each load and store of such a cell
/// is one 64-bit add of a constant-bank operand to the cell's base pointer
/// instead of a wrapped 3-D index and a slice product per direction.
struct PullOffsets {
    long long pull[kQ];
    long long slice[kQ];
};

template <class T>
__host__ PullOffsets pull_offsets(int nx, int ny, long long n) {
    PullOffsets o;
    const long long sx = nx, sxy = static_cast<long long>(nx) * ny;
    for (int q = 0; q < kQ; ++q) {
        o.slice[q] = q * n * static_cast<long long>(sizeof(T));
        o.pull[q] = (q * n - (cx(q) + sx * cy(q) + sxy * cz(q))) * static_cast<long long>(sizeof(T));
    }
    return o;
}

template <class T>
__device__ __forceinline__ const T* byte_add(const T* p, long long b) {
    return reinterpret_cast<const T*>(reinterpret_cast<const char*>(p) + b);
}
template <class T>
__device__ __forceinline__ T* byte_add(T* p, long long b) {
    return reinterpret_cast<T*>(reinterpret_cast<char*>(p) + b);
}

/// True when no pull of (x, y, z) wraps around a periodic axis.
__device__ __forceinline__ bool interior(int x, int y, int z, const CollideArgs& a) {
    return x > 0 && x < a.nx - 1 && y > 0 && y < a.ny - 1 && z > 0 && z < a.nz - 1;
}

/// Population access in f (DEV false) or deviation g = f - w_q (DEV true).
template <class S, bool DEV>
struct Pop {
    using T = typename S::T;
    __device__ __forceinline__ static float ld(const T* __restrict__ p, long long i, float w) {
        if constexpr (DEV) return S::ld_dev(p, i, w);
        else return S::ld(p, i, w);
    }
    __device__ __forceinline__ static void st(T* __restrict__ p, long long i, float v, float w) {
        if constexpr (DEV) S::st_dev(p, i, v, w);
        else S::st(p, i, v, w);
    }
    __device__ __forceinline__ static float lds(unsigned row, int i, float w) {
        if constexpr (DEV) return S::lds_dev(row, i, w);
        else return S::lds(row, i, w);
    }
    /// Coherent load, for a slot this kernel may have written.
    __device__ __forceinline__ static float ld_coherent(const T* p, float w) {
        const float v = static_cast<float>(*p);
        if constexpr (DEV) return std::is_same_v<T, float> ? v - w : v;
        else return std::is_same_v<T, float> ? v : w + v;
    }
};

__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// ---- equilibrium in the reference expression order ------------------------
__device__ __forceinline__ float dot_c(int q, float ux, float uy, float uz) {
    // (cx ux + cy uy) + cz uz with zero terms dropped and +-1 folded.
    float d = 0.0f;
    bool any = false;
    if (cx(q) != 0) { d = cx(q) > 0 ? ux : -ux; any = true; }
    if (cy(q) != 0) { const float t = cy(q) > 0 ? uy : -uy; d = any ? d + t : t; any = true; }
    if (cz(q) != 0) { const float t = cz(q) > 0 ? uz : -uz; d = any ? d + t : t; }
    return d;
}

/// Reference equilibrium19 (lbm_core.cu:65-73): (w rho)((1 + cu + cu cu/2) - usq).
__device__ __forceinline__ void eq19(float rho, float ux, float uy, float uz, float (&feq)[kQ]) {
    const float usq = 1.5f * (ux * ux + uy * uy + uz * uz);
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
        const float cu = 3.0f * dot_c(q, ux, uy, uz);
        feq[q] = (wgt(q) * rho) * (1.0f + cu + 0.5f * cu * cu - usq);
    }
}

// ---- collision bodies ------------------------------------------------------
__device__ __forceinline__ void collide_exact(float (&f)[kQ], float tau0, float lambda, float smagPre,
                                              float& rhoO, float& uxO, float& uyO, float& uzO) {
    float rho = 0.0f, jx = 0.0f, jy = 0.0f, jz = 0.0f;
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
        rho += f[q];
        if (cx(q) != 0) jx = cx(q) > 0 ? jx + f[q] : jx - f[q];
        if (cy(q) != 0) jy = cy(q) > 0 ? jy + f[q] : jy - f[q];
        if (cz(q) != 0) jz = cz(q) > 0 ? jz + f[q] : jz - f[q];
    }
    rho = fmaxf(rho, kRhoFloor);
    const float invRho = 1.0f / rho;
    float ux = jx * invRho, uy = jy * invRho, uz = jz * invRho;
    const float u2 = ux * ux + uy * uy + uz * uz;
    if (u2 > kMaxSimSpeed * kMaxSimSpeed) {
        // The hardware reciprocal square root, as the reference's GPU build
        // evaluates rsqrtf (lbm_core.cu:413); its CPU build and the oracle
        // use IEEE 1/sqrtf. Only cells beyond |u| = 0.3 take this branch.
        const float s = kMaxSimSpeed * rsqrtf(u2);
        ux *= s; uy *= s; uz *= s;
    }
    float feq[kQ];
    eq19(rho, ux, uy, uz, feq);
    float tauEff = tau0;
    if (smagPre > 0.0f) {
        float pxx = 0.0f, pyy = 0.0f, pzz = 0.0f, pxy = 0.0f, pxz = 0.0f, pyz = 0.0f;
#pragma unroll
        for (int q = 0; q < kQ; ++q) {
            const float fneq = f[q] - feq[q];
            if (cx(q) != 0) pxx += fneq;
            if (cy(q) != 0) pyy += fneq;
            if (cz(q) != 0) pzz += fneq;
            if (cx(q) * cy(q) != 0) pxy = cx(q) * cy(q) > 0 ? pxy + fneq : pxy - fneq;
            if (cx(q) * cz(q) != 0) pxz = cx(q) * cz(q) > 0 ? pxz + fneq : pxz - fneq;
            if (cy(q) * cz(q) != 0) pyz = cy(q) * cz(q) > 0 ? pyz + fneq : pyz - fneq;
        }
        const float qbar = sqrtf(pxx * pxx + pyy * pyy + pzz * pzz + 2.0f * (pxy * pxy + pxz * pxz + pyz * pyz));
        tauEff = 0.5f * (tau0 + sqrtf(tau0 * tau0 + smagPre * qbar * invRho));
    }
    const float omP = 1.0f / tauEff;
    const float tauM = 0.5f + lambda / (tauEff - 0.5f);
    const float omM = 1.0f / tauM;
    f[0] = f[0] - omP * (f[0] - feq[0]);
#pragma unroll
    for (int p = 1; p <= 9; ++p) {
        const int qa = 2 * p - 1, qb = 2 * p;
        const float sym = omP * (0.5f * (f[qa] + f[qb]) - 0.5f * (feq[qa] + feq[qb]));
        const float asym = omM * (0.5f * (f[qa] - f[qb]) - 0.5f * (feq[qa] - feq[qb]));
        const float fa = f[qa];
        f[qa] = fa - sym - asym;
        f[qb] = f[qb] - sym + asym;
    }
    rhoO = rho; uxO = ux; uyO = uy; uzO = uz;
}

// ---- arithmetic of the deviation body -----------------------------------------
// Every operation is an explicit round-to-nearest intrinsic (the fused
// multiply-adds written out where the body wants them), so the compiler
// contracts nothing on its own and the body rounds the same in every
// translation unit and kernel that includes it.
template <class V> struct Lane;
template <> struct Lane<float> {
    __device__ __forceinline__ static float s(float v) { return v; }
    __device__ __forceinline__ static float add(float a, float b) { return __fadd_rn(a, b); }
    __device__ __forceinline__ static float sub(float a, float b) { return __fsub_rn(a, b); }
    __device__ __forceinline__ static float mul(float a, float b) { return __fmul_rn(a, b); }
    __device__ __forceinline__ static float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
    __device__ __forceinline__ static float neg(float a) { return -a; }
    __device__ __forceinline__ static float rcp(float a) { return rcp_approx(a); }
    __device__ __forceinline__ static float sqrt(float a) { return sqrt_approx(a); }
};

/// Density floor of one lane: rho = max-floored 1 + dr, rm1 = rho - 1.
__device__ __forceinline__ void rho_floor(float dr, float& rho, float& rm1) {
    const float r = __fadd_rn(1.0f, dr);
    const bool floored = r < kRhoFloor;
    rho = floored ? kRhoFloor : r;
    rm1 = floored ? kRhoFloor - 1.0f : dr;
}

/// The |u| <= 0.3 limiter of one lane (u2 recomputed when it acts).
__device__ __forceinline__ void limit_u(float& ux, float& uy, float& uz, float& u2) {
    if (u2 > kMaxSimSpeed * kMaxSimSpeed) {
        const float sc = __fmul_rn(kMaxSimSpeed, rsqrtf(u2));
        ux = __fmul_rn(ux, sc); uy = __fmul_rn(uy, sc); uz = __fmul_rn(uz, sc);
        u2 = __fmaf_rn(uz, uz, __fmaf_rn(uy, uy, __fmul_rn(ux, ux)));
    }
}

/// c_a . u of pair direction a, components in the order x, y, z.
template <class V>
__device__ __forceinline__ V dot_lane(int a, V ux, V uy, V uz) {
    using L = Lane<V>;
    V d = L::s(0.0f);
    bool any = false;
    if (cx(a) != 0) { d = cx(a) > 0 ? ux : L::neg(ux); any = true; }
    if (cy(a) != 0) { d = any ? (cy(a) > 0 ? L::add(d, uy) : L::sub(d, uy)) : (cy(a) > 0 ? uy : L::neg(uy)); any = true; }
    if (cz(a) != 0) d = any ? (cz(a) > 0 ? L::add(d, uz) : L::sub(d, uz)) : (cz(a) > 0 ? uz : L::neg(uz));
    return d;
}

/// TRT + Smagorinsky collision on the deviations g_q = f_q - w_q of one cell.
template <class V>
__device__ __forceinline__ void collide_dev_lanes(V (&g)[kQ], float tau0, float lambda, float smagPre, V& rhoO,
                                                  V& uxO, V& uyO, V& uzO) {
    using L = Lane<V>;
    // Pair sums of f are s[p] + 2 w_p, differences d[p] as for f. The
    // update needs only these (symmetric and antisymmetric parts), so the
    // pair's own values are not kept.
    V s[10], d[10];
#pragma unroll
    for (int p = 1; p <= 9; ++p) {
        s[p] = L::add(g[2 * p - 1], g[2 * p]);
        d[p] = L::sub(g[2 * p - 1], g[2 * p]);
    }
    // Pair p has velocity c_{2p-1}: p1 (1,0,0) p2 (0,1,0) p3 (0,0,1)
    // p4 (1,1,0) p5 (1,0,1) p6 (0,1,1) p7 (1,-1,0) p8 (1,0,-1) p9 (0,1,-1).
    const V dr = L::add(L::add(L::add(g[0], L::add(L::add(s[1], s[2]), L::add(s[3], s[4]))),
                               L::add(L::add(s[5], s[6]), L::add(s[7], s[8]))),
                        s[9]);
    const V jx = L::add(L::add(L::add(d[1], d[4]), L::add(d[5], d[7])), d[8]);
    const V jy = L::add(L::add(L::add(d[2], d[4]), L::sub(d[6], d[7])), d[9]);
    const V jz = L::sub(L::add(L::add(d[3], d[5]), L::sub(d[6], d[8])), d[9]);
    V rho, rm1;   // rm1 = rho - 1
    rho_floor(dr, rho, rm1);
    const V inv = L::rcp(rho);
    V ux = L::mul(jx, inv), uy = L::mul(jy, inv), uz = L::mul(jz, inv);
    V u2 = L::fma(uz, uz, L::fma(uy, uy, L::mul(ux, ux)));
    limit_u(ux, uy, uz, u2);
    const V rux = L::mul(rho, ux), ruy = L::mul(rho, uy);
    V tauEff = L::s(tau0);
    if (smagPre > 0.0f) {
        // Non-equilibrium stress: the weights' share of the diagonal
        // (sum of w_q over c_a != 0 = 1/3) cancels against rho/3 up to rho - 1.
        const V r3 = L::mul(rm1, L::s(1.0f / 3.0f));
        const V nxx = L::fma(L::neg(rux), ux, L::sub(L::add(L::add(L::add(s[1], s[4]), L::add(s[5], s[7])), s[8]), r3));
        const V nyy = L::fma(L::neg(ruy), uy, L::sub(L::add(L::add(L::add(s[2], s[4]), L::add(s[6], s[7])), s[9]), r3));
        const V nzz = L::fma(L::neg(L::mul(rho, uz)), uz,
                             L::sub(L::add(L::add(L::add(s[3], s[5]), L::add(s[6], s[8])), s[9]), r3));
        const V nxy = L::fma(L::neg(rux), uy, L::sub(s[4], s[7]));
        const V nxz = L::fma(L::neg(rux), uz, L::sub(s[5], s[8]));
        const V nyz = L::fma(L::neg(ruy), uz, L::sub(s[6], s[9]));
        const V dia = L::fma(nzz, nzz, L::fma(nyy, nyy, L::mul(nxx, nxx)));
        const V off = L::fma(nyz, nyz, L::fma(nxz, nxz, L::mul(nxy, nxy)));
        const V qbar = L::sqrt(L::fma(L::s(2.0f), off, dia));
        const V inner = L::fma(L::mul(L::s(smagPre), qbar), inv, L::s(__fmul_rn(tau0, tau0)));
        tauEff = L::mul(L::s(0.5f), L::add(L::s(tau0), L::sqrt(inner)));
    }
    const V omP = L::rcp(tauEff);
    const V omM = L::rcp(L::fma(L::s(lambda), L::rcp(L::sub(tauEff, L::s(0.5f))), L::s(0.5f)));
    // feq_q - w_q = w_q (A + 4.5 rho (c_q.u)^2) + 3 w_q rho (c_q.u), A = rho - 1 - 1.5 rho u^2.
    const V A = L::fma(L::mul(L::s(-1.5f), rho), u2, rm1);
    const V r45 = L::mul(L::s(4.5f), rho);
    g[0] = L::fma(L::neg(omP), L::fma(L::s(-1.0f / 3.0f), A, g[0]), g[0]);
#pragma unroll
    for (int p = 1; p <= 9; ++p) {
        const int a = 2 * p - 1;
        const float w = wgt(a);
        const V cu = dot_lane<V>(a, ux, uy, uz);
        const V es = L::mul(L::s(w), L::fma(L::mul(r45, cu), cu, A));
        const V ea = L::mul(L::mul(L::s(3.0f * w), rho), cu);
        const V hs = L::mul(L::s(0.5f), s[p]), hd = L::mul(L::s(0.5f), d[p]);
        const V sym = L::fma(L::neg(omP), L::sub(hs, es), hs);
        const V asym = L::fma(L::neg(omM), L::sub(hd, ea), hd);
        g[a] = L::add(sym, asym);
        g[a + 1] = L::sub(sym, asym);
    }
    rhoO = rho; uxO = ux; uyO = uy; uzO = uz;
}

__device__ __forceinline__ void collide_dev(float (&g)[kQ], float tau0, float lambda, float smagPre,
                                            float& rhoO, float& uxO, float& uyO, float& uzO) {
    collide_dev_lanes<float>(g, tau0, lambda, smagPre, rhoO, uxO, uyO, uzO);
}

/// The collision of a cell's 19 populations: f with the exact body, the
/// deviations g with the fast one.
template <bool EXACT>
__device__ __forceinline__ void collide_body(float (&f)[kQ], const CollideArgs& a, float& r, float& ux, float& uy,
                                             float& uz) {
    if constexpr (EXACT) collide_exact(f, a.tau0, a.lambda, a.smagPre, r, ux, uy, uz);
    else collide_dev(f, a.tau0, a.lambda, a.smagPre, r, ux, uy, uz);
}

// ---- per-cell pieces ---------------------------------------------------------
struct Nbr {
    unsigned sx[3], sy[3], sz[3];
};

/// Source coordinates of a pull along each velocity component (x - c, wrapped).
__device__ __forceinline__ Nbr neighbours(int x, int y, int z, int nx, int ny, int nz) {
    Nbr b;
    b.sx[0] = wrap_inc(x, nx); b.sx[1] = x; b.sx[2] = wrap_dec(x, nx);
    b.sy[0] = wrap_inc(y, ny); b.sy[1] = y; b.sy[2] = wrap_dec(y, ny);
    b.sz[0] = wrap_inc(z, nz); b.sz[1] = z; b.sz[2] = wrap_dec(z, nz);
    return b;
}

/// Boundary (non-fluid) cell: inlet feq(1, u_in), outlets from the upstream
/// column, everything else untouched (lbm_core.cu:241-283).
template <class S>
__device__ __forceinline__ void boundary_cell(const typename S::T* __restrict__ src, typename S::T* __restrict__ dst,
                                              const CollideArgs& a, int flag, unsigned cell, int x, int y, int z) {
    const long long n = a.n;
    if (flag == kInlet) {
        float feq[kQ];
        eq19(1.0f, a.uIn, 0.0f, 0.0f, feq);
#pragma unroll
        for (int q = 0; q < kQ; ++q) S::st(dst + q * n, cell, feq[q], wgt(q));
        if (a.writeMacro) { a.rho[cell] = 1.0f; a.u[cell] = a.uIn; a.v[cell] = 0.0f; a.w[cell] = 0.0f; }
    } else if (flag == kOutlet || flag == kOutletEq) {
        const unsigned up = static_cast<unsigned>(wrap_dec(x, a.nx))
                          + static_cast<unsigned>(a.nx) * (static_cast<unsigned>(y) + static_cast<unsigned>(a.ny) * z);
        float g[kQ];
        float r = 0.0f, jx = 0.0f, jy = 0.0f, jz = 0.0f;
#pragma unroll
        for (int q = 0; q < kQ; ++q) {
            g[q] = S::ld(src + q * n, up, wgt(q));
            r += g[q];
            if (cx(q) != 0) jx = cx(q) > 0 ? jx + g[q] : jx - g[q];
            if (cy(q) != 0) jy = cy(q) > 0 ? jy + g[q] : jy - g[q];
            if (cz(q) != 0) jz = cz(q) > 0 ? jz + g[q] : jz - g[q];
        }
        const float inv = 1.0f / r;
        const float ux = jx * inv, uy = jy * inv, uz = jz * inv;
        if (flag == kOutletEq) {
            eq19(1.0f, ux, uy, uz, g);   // equilibrium outflow feq(1, u_upstream)
            r = 1.0f;
        }
#pragma unroll
        for (int q = 0; q < kQ; ++q) S::st(dst + q * n, cell, g[q], wgt(q));
        if (a.writeMacro) { a.rho[cell] = r; a.u[cell] = ux; a.v[cell] = uy; a.w[cell] = uz; }
    } else if (a.writeMacro) {
        a.rho[cell] = 1.0f; a.u[cell] = 0.0f; a.v[cell] = 0.0f; a.w[cell] = 0.0f;
    }
}

/// Bulk fluid cell: 19 plain pulls from global memory.
template <class S, bool DEV>
__device__ __forceinline__ void gather_bulk(const typename S::T* __restrict__ src, const CollideArgs& a,
                                            const Nbr& b, float (&f)[kQ]) {
    const unsigned unx = a.nx, uny = a.ny;
#pragma unroll
    for (int q = 0; q < kQ; ++q)
        f[q] = Pop<S, DEV>::ld(src + q * a.n, b.sx[1 + cx(q)] + unx * (b.sy[1 + cy(q)] + uny * b.sz[1 + cz(q)]),
                               wgt(q));
}

/// Bulk fluid cell away from the periodic faces: the same 19 pulls through
/// the constant offsets.
template <class S, bool DEV>
__device__ __forceinline__ void gather_interior(const typename S::T* __restrict__ src, const PullOffsets& o,
                                                unsigned cell, float (&f)[kQ]) {
    const typename S::T* base = src + cell;
#pragma unroll
    for (int q = 0; q < kQ; ++q) f[q] = Pop<S, DEV>::ld(byte_add(base, o.pull[q]), 0, wgt(q));
}

/// Store the 19 populations of `cell` (slice offsets when given).
template <class S, bool DEV>
__device__ __forceinline__ void store_cell(typename S::T* __restrict__ dst, const CollideArgs& a, unsigned cell,
                                           const float (&f)[kQ], const PullOffsets* o) {
    if (o) {
        typename S::T* base = dst + cell;
#pragma unroll
        for (int q = 0; q < kQ; ++q) Pop<S, DEV>::st(byte_add(base, o->slice[q]), 0, f[q], wgt(q));
    } else {
#pragma unroll
        for (int q = 0; q < kQ; ++q) Pop<S, DEV>::st(dst + q * a.n, cell, f[q], wgt(q));
    }
}

/// Near-wall fluid cell: the upstream flag picks the (slot, cell) pair per
/// link; the wall-model Ladd term 6 w_q (c_q . u_w) on solid links. LW: the
/// links' classes come from the cell's link word (a.links) instead of the
/// 18 neighbours' flags.
template <class S, bool WM, bool QL, bool DEV, bool LW = false>
__device__ __forceinline__ void gather_wall(const typename S::T* __restrict__ src,
                                            const std::uint8_t* __restrict__ kind, const CollideArgs& a,
                                            const Nbr& b, unsigned cell, int y, int z, float (&f)[kQ]) {
    const unsigned unx = a.nx, uny = a.ny;
    const long long n = a.n;
    float uwx = 0.0f, uwy = 0.0f, uwz = 0.0f;
    bool uwLoaded = false;
    using P = Pop<S, DEV>;
    unsigned long long lm = 0;
    if constexpr (LW) {
        const uint2 w = __ldg(a.links + cell);
        lm = static_cast<unsigned long long>(w.x) | (static_cast<unsigned long long>(w.y) << 32);
    }
    f[0] = P::ld(src, cell, wgt(0));
#pragma unroll
    for (int q = 1; q < kQ; ++q) {
        const unsigned X = b.sx[1 + cx(q)], Y = b.sy[1 + cy(q)], Z = b.sz[1 + cz(q)];
        const unsigned pn = X + unx * (Y + uny * Z);
        bool solid, slipY, slipZ;
        if constexpr (LW) {
            solid = (lm >> (q - 1)) & 1ull;
            slipY = (lm >> (17 + q)) & 1ull;
            slipZ = (lm >> (35 + q)) & 1ull;
        } else {
            const int nf = kind[pn] & kFlagMask;
            solid = nf == kSolid;
            slipY = is_slip_y(nf);
            slipZ = is_slip_z(nf);
        }
        const unsigned pY = X + unx * (static_cast<unsigned>(y) + uny * Z);
        const unsigned pZ = X + unx * (Y + uny * static_cast<unsigned>(z));
        const int qs = solid ? opp(q) : (slipY ? mir_y(q) : (slipZ ? mir_z(q) : q));
        const unsigned cs = solid ? cell : (slipY ? pY : (slipZ ? pZ : pn));
        float fq = P::ld(src + static_cast<long long>(qs) * n, cs, wgt(q));
        // Interpolated bounce-back (Bouzidi 2001) on a solid link with an
        // analytic cut fraction, in the reference's expression order
        // (lbm_core.cu:332-364): the wall sits at q = byte/255 of the link.
        if (QL && solid) {
            const std::uint8_t qb = a.qFrac[static_cast<long long>(cell) * kQ + q];
            if (qb != 0) {
                const float qf = static_cast<float>(qb) * (1.0f / 255.0f);
                const float fOut = P::ld(src + static_cast<long long>(q) * n, cell, wgt(q));
                if (qf >= 0.5f) {
                    const float inv2q = 0.5f / qf;
                    fq = inv2q * fOut + (1.0f - inv2q) * fq;
                } else if (a.ffMask[cell] & (1u << q)) {
                    // Second fluid node x + c_q (opposite the wall).
                    const unsigned pff = b.sx[1 - cx(q)] + unx * (b.sy[1 - cy(q)] + uny * b.sz[1 - cz(q)]);
                    const float fOutFF = P::ld(src + static_cast<long long>(q) * n, pff, wgt(q));
                    fq = 2.0f * qf * fOut + (1.0f - 2.0f * qf) * fOutFF;
                }
                // else: x + c_q solid (thin vane): keep the half-way value.
            }
        }
        if constexpr (WM) {
            if (solid) {
                if (!uwLoaded) {
                    uwx = __half2float(__ushort_as_half(a.uwx[cell]));
                    uwy = __half2float(__ushort_as_half(a.uwy[cell]));
                    uwz = __half2float(__ushort_as_half(a.uwz[cell]));
                    uwLoaded = true;
                }
                fq += (6.0f * wgt(q)) * dot_c(q, uwx, uwy, uwz);
            }
        }
        f[q] = fq;
    }
}

/// Near-wall interior cell whose wall links are all solid (bit q - 1 of
/// `solidMask`): the pulls of gather_wall through the constant offsets --
/// the own cell's opposite slot on a solid link, the upstream cell
/// otherwise -- with the same interpolated bounce-back and Ladd terms.
template <class S, bool WM, bool QL, bool DEV>
__device__ __forceinline__ void gather_solid_links(const typename S::T* __restrict__ src, const CollideArgs& a,
                                                   const PullOffsets& o, unsigned cell, int x, int y, int z,
                                                   unsigned solidMask, float (&f)[kQ]) {
    using P = Pop<S, DEV>;
    const typename S::T* base = src + cell;
    float uwx = 0.0f, uwy = 0.0f, uwz = 0.0f;
    if constexpr (WM) {
        uwx = __half2float(__ushort_as_half(a.uwx[cell]));
        uwy = __half2float(__ushort_as_half(a.uwy[cell]));
        uwz = __half2float(__ushort_as_half(a.uwz[cell]));
    }
    f[0] = P::ld(base, 0, wgt(0));
#pragma unroll
    for (int q = 1; q < kQ; ++q) {
        const bool solid = (solidMask >> (q - 1)) & 1u;
        float fq = P::ld(byte_add(base, solid ? o.slice[opp(q)] : o.pull[q]), 0, wgt(q));
        if (QL && solid) {
            const std::uint8_t qb = a.qFrac[static_cast<long long>(cell) * kQ + q];
            if (qb != 0) {
                const float qf = static_cast<float>(qb) * (1.0f / 255.0f);
                const float fOut = P::ld(byte_add(base, o.slice[q]), 0, wgt(q));
                if (qf >= 0.5f) {
                    const float inv2q = 0.5f / qf;
                    fq = inv2q * fOut + (1.0f - inv2q) * fq;
                } else if (a.ffMask[cell] & (1u << q)) {
                    const unsigned unx = a.nx, uny = a.ny;
                    const Nbr b = neighbours(x, y, z, a.nx, a.ny, a.nz);
                    const unsigned pff = b.sx[1 - cx(q)] + unx * (b.sy[1 - cy(q)] + uny * b.sz[1 - cz(q)]);
                    const float fOutFF = P::ld(src + static_cast<long long>(q) * a.n, pff, wgt(q));
                    fq = 2.0f * qf * fOut + (1.0f - 2.0f * qf) * fOutFF;
                }
            }
        }
        if constexpr (WM) {
            if (solid) fq += (6.0f * wgt(q)) * dot_c(q, uwx, uwy, uwz);
        }
        f[q] = fq;
    }
}

template <class S, bool EXACT>
__device__ __forceinline__ void finish_cell(typename S::T* __restrict__ dst, const CollideArgs& a, unsigned cell,
                                            float (&f)[kQ], const PullOffsets* o = nullptr) {
    float r, ux, uy, uz;
    collide_body<EXACT>(f, a, r, ux, uy, uz);
    store_cell<S, !EXACT>(dst, a, cell, f, o);
    if (a.writeMacro) { a.rho[cell] = r; a.u[cell] = ux; a.v[cell] = uy; a.w[cell] = uz; }
}

/// The 19 post-streaming populations of fluid cell (x, y, z): bulk cells by
/// plain pulls (constant offsets away from the periodic faces when `o` is
/// given), near-wall cells through their neighbours' flags.
template <class S, bool WM, bool QL, bool DEV, bool LW = false>
__device__ __forceinline__ void gather_fluid(const typename S::T* __restrict__ src,
                                             const std::uint8_t* __restrict__ kind, const CollideArgs& a,
                                             std::uint8_t k, unsigned cell, int x, int y, int z, float (&f)[kQ],
                                             const PullOffsets* o) {
    if (!(k & kNearWall)) {
        if (o && interior(x, y, z, a)) gather_interior<S, DEV>(src, *o, cell, f);
        else gather_bulk<S, DEV>(src, a, neighbours(x, y, z, a.nx, a.ny, a.nz), f);
        return;
    }
    // Near-wall cell. With the link classes at hand, an interior cell whose
    // wall links are all solid (the cells along a foil) pulls through the
    // constant offsets, a select per link choosing its own opposite slot over
    // the upstream cell; slip-wall cells and the periodic faces take the
    // general path (measured the same as a slip-aware select path, which
    // needs more registers).
    if (a.links && o && interior(x, y, z, a)) {
        const uint2 w = __ldg(a.links + cell);
        if (w.y == 0 && (w.x >> 18) == 0) {   // solid links only (no slip-wall bit)
            gather_solid_links<S, WM, QL, DEV>(src, a, *o, cell, x, y, z, w.x, f);
            return;
        }
    }
    gather_wall<S, WM, QL, DEV, LW>(src, kind, a, neighbours(x, y, z, a.nx, a.ny, a.nz), cell, y, z, f);
}

/// One full cell update at (x, y, z): boundary cells by flag, fluid cells
/// by their 19 pulls (bulk or near-wall path) and the collision.
template <class S, bool WM, bool EXACT, bool QL = false, bool LW = false>
__device__ __forceinline__ void collide_one(const typename S::T* __restrict__ src, typename S::T* __restrict__ dst,
                                            const std::uint8_t* __restrict__ kind, const CollideArgs& a, int x, int y,
                                            int z, const PullOffsets* o = nullptr) {
    const unsigned cell = static_cast<unsigned>(x)
                        + static_cast<unsigned>(a.nx) * (static_cast<unsigned>(y) + static_cast<unsigned>(a.ny) * z);
    const std::uint8_t k = kind[cell];
    const int flag = k & kFlagMask;
    if (flag != kFluid) {
        boundary_cell<S>(src, dst, a, flag, cell, x, y, z);
        return;
    }
    float f[kQ];
    gather_fluid<S, WM, QL, !EXACT, LW>(src, kind, a, k, cell, x, y, z, f, o);
    finish_cell<S, EXACT>(dst, a, cell, f, o);
}

// ---- one cell per thread -----------------------------------------------------
constexpr int kCellBlockX = 128;

template <class S, bool WM, bool EXACT, bool QL>
__global__ void __launch_bounds__(kCellBlockX, S::kCellMinBlocks)
collide_cell_kernel(const typename S::T* __restrict__ src, typename S::T* __restrict__ dst,
                    const std::uint8_t* __restrict__ kind, CollideArgs a, const __grid_constant__ PullOffsets off) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= a.nx) return;
    collide_one<S, WM, EXACT, QL>(src, dst, kind, a, x, blockIdx.y, blockIdx.z, &off);
}

// ---- one cell per thread over the flattened lattice -----------------------------
// For levels whose rows are not a multiple of 32 cells (the 616-cell fine
// rows of the airfoil patch), a row-per-block launch ends every row with a
// partly idle warp; here consecutive threads take consecutive cells across
// row boundaries. (x, y, z) come from two divisions by invariant integers
// (FastDiv, d3q19.cuh).

template <class S, bool WM, bool EXACT, bool QL>
__global__ void __launch_bounds__(kCellBlockX, S::kCellMinBlocks)
collide_flat_kernel(const typename S::T* __restrict__ src, typename S::T* __restrict__ dst,
                    const std::uint8_t* __restrict__ kind, CollideArgs a, const __grid_constant__ PullOffsets off,
                    FastDiv divX, FastDiv divY) {
    const unsigned cell = blockIdx.x * kCellBlockX + threadIdx.x;
    if (cell >= static_cast<unsigned long long>(a.n)) return;
    const unsigned row = fdiv(cell, divX);
    const unsigned z = fdiv(row, divY);
    collide_one<S, WM, EXACT, QL>(src, dst, kind, a, static_cast<int>(cell - row * divX.d),
                                  static_cast<int>(row - z * divY.d), static_cast<int>(z), &off);
}

// ---- AA-pattern in-place streaming (all-fluid periodic lattices) --------------
// One population array A instead of the A/B pair (Bailey, Myre, Walsh, Lilja,
// Wilson 2009, "Accelerating lattice Boltzmann fluid flow simulations using
// graphics processors"). Between steps the array holds one of two layouts:
//  * swapped:  A[opp(q)][x] = f*_q(x), each cell's post-collision populations
//    with the slots of every opposite pair exchanged;
//  * streamed: A[q][x] = f*_q(x - c_q), the post-streaming populations.
// An odd step reads the swapped layout from the upstream cells, f_q(x) =
// A[opp(q)][x - c_q], collides and writes f*_q(x) to A[q][x + c_q] -- the
// slot it read for direction opp(q) -- leaving the streamed layout. An even
// step reads A[q][x] of its own cell and writes f*_q(x) to A[opp(q)][x],
// leaving the swapped layout. Every cell writes exactly the slots it read and
// no other cell touches them, so the update is in place without races, and
// the non-coherent loads never see a slot another thread has written. The
// populations entering each collision are the A/B kernel's, so the results
// are identical bit for bit. Opposite directions share a weight, so the FP16
// deviation bytes move between slots unchanged.

/// Byte offsets from &A[0][x] of the odd-step read A[opp(q)][x - c_q] of an
/// interior cell; its write A[q][x + c_q] is the read offset of opp(q).
struct AAOffsets {
    long long rd[kQ];
};

template <class T>
__host__ AAOffsets aa_offsets(int nx, int ny, long long n) {
    AAOffsets o;
    const long long sx = nx, sxy = static_cast<long long>(nx) * ny;
    for (int q = 0; q < kQ; ++q)
        o.rd[q] = (opp(q) * n - (cx(q) + sx * cy(q) + sxy * cz(q))) * static_cast<long long>(sizeof(T));
    return o;
}

template <class S, bool EXACT, bool ODD>
__global__ void __launch_bounds__(kCellBlockX, S::kCellMinBlocks)
collide_aa_kernel(typename S::T* __restrict__ A, CollideArgs a, const __grid_constant__ AAOffsets off) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= a.nx) return;
    const int y = blockIdx.y, z = blockIdx.z;
    const unsigned unx = a.nx, uny = a.ny;
    const unsigned cell = static_cast<unsigned>(x) + unx * (static_cast<unsigned>(y) + uny * static_cast<unsigned>(z));
    const long long n = a.n;
    using P = Pop<S, !EXACT>;
    float f[kQ], r, ux, uy, uz;
    // One collision body for every path; the wrapped neighbour indices of a
    // face cell are formed again for the stores rather than held across it.
    const bool inner = ODD && interior(x, y, z, a);
    typename S::T* base = A + cell;
    if constexpr (!ODD) {
#pragma unroll
        for (int q = 0; q < kQ; ++q) f[q] = P::ld(A + q * n, cell, wgt(q));
    } else if (inner) {
#pragma unroll
        for (int q = 0; q < kQ; ++q) f[q] = P::ld(byte_add(base, off.rd[q]), 0, wgt(q));
    } else {
        const Nbr b = neighbours(x, y, z, a.nx, a.ny, a.nz);
#pragma unroll
        for (int q = 0; q < kQ; ++q)
            f[q] = P::ld(A + opp(q) * n, b.sx[1 + cx(q)] + unx * (b.sy[1 + cy(q)] + uny * b.sz[1 + cz(q)]), wgt(q));
    }
    collide_body<EXACT>(f, a, r, ux, uy, uz);
    if constexpr (!ODD) {
#pragma unroll
        for (int q = 0; q < kQ; ++q) P::st(A + opp(q) * n, cell, f[q], wgt(q));
    } else if (inner) {
#pragma unroll
        for (int q = 0; q < kQ; ++q) P::st(byte_add(base, off.rd[opp(q)]), 0, f[q], wgt(q));
    } else {
        const Nbr b = neighbours(x, y, z, a.nx, a.ny, a.nz);
#pragma unroll
        for (int q = 0; q < kQ; ++q)
            P::st(A + q * n, b.sx[1 - cx(q)] + unx * (b.sy[1 - cy(q)] + uny * b.sz[1 - cz(q)]), f[q], wgt(q));
    }
    if (a.writeMacro) { a.rho[cell] = r; a.u[cell] = ux; a.v[cell] = uy; a.w[cell] = uz; }
}

template <class S, bool EXACT>
cudaError_t launch_collide_aa_impl(void* fv, LevelDims d, const CollideParams& p, int odd, float* rho, float* u,
                                   float* v, float* w, cudaStream_t st) {
    using T = typename S::T;
    CollideArgs a{};
    a.nx = d.nx; a.ny = d.ny; a.nz = d.nz; a.n = d.cells();
    a.tau0 = p.tau; a.lambda = p.magicLambda; a.smagPre = p.smagPrefactor; a.uIn = p.uInlet;
    a.writeMacro = (p.writeMacro && rho && u && v && w) ? 1 : 0;
    a.rho = rho; a.u = u; a.v = v; a.w = w;
    T* f = static_cast<T*>(fv);
    const int bx = d.nx >= kCellBlockX ? kCellBlockX : ((d.nx + 31) / 32) * 32;
    const dim3 grid(static_cast<unsigned>((d.nx + bx - 1) / bx), static_cast<unsigned>(d.ny),
                    static_cast<unsigned>(d.nz));
    const AAOffsets off = aa_offsets<T>(d.nx, d.ny, a.n);
    if (odd) collide_aa_kernel<S, EXACT, true><<<grid, bx, 0, st>>>(f, a, off);
    else collide_aa_kernel<S, EXACT, false><<<grid, bx, 0, st>>>(f, a, off);
    return cudaGetLastError();
}

// ---- warm-restart flag edits (applyFlagEditsKernel, lbm_core.cu:644-717) -----
// mask 1: newly solid -> every population of both buffers zeroed; mask 2:
// newly fluid -> equilibrium of the mean rho, u of the neighbours (x + c_q,
// no wrap in x/y, periodic z) that are fluid and unedited, read from fA
// (rest state when there are none), written to both buffers. Edited cells
// never read each other, so the kernel has no races.
template <class S>
__global__ void apply_flag_edits_kernel(typename S::T* __restrict__ fA, typename S::T* __restrict__ fB,
                                        const std::uint8_t* __restrict__ flags,
                                        const std::uint8_t* __restrict__ mask, int nx, int ny, int nz) {
    const long long n = static_cast<long long>(nx) * ny * nz;
    const long long cell = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (cell >= n) return;
    const std::uint8_t edit = mask[cell];
    if (edit == 0) return;
    if (edit == 1) {
#pragma unroll
        for (int q = 0; q < kQ; ++q) {
            S::st(fA + q * n, cell, 0.0f, wgt(q));
            S::st(fB + q * n, cell, 0.0f, wgt(q));
        }
        return;
    }
    const long long nxny = static_cast<long long>(nx) * ny;
    const int z = static_cast<int>(cell / nxny);
    const long long rem = cell - static_cast<long long>(z) * nxny;
    const int y = static_cast<int>(rem / nx), x = static_cast<int>(rem - static_cast<long long>(y) * nx);
    float rho = 0.0f, ux = 0.0f, uy = 0.0f, uz = 0.0f;
    int found = 0;
    for (int q = 1; q < kQ; ++q) {
        const int xn = x + cx(q), yn = y + cy(q), zn = z + cz(q);
        if (xn < 0 || xn >= nx || yn < 0 || yn >= ny) continue;
        const int znw = zn < 0 ? nz - 1 : (zn >= nz ? 0 : zn);
        const long long nc = xn + static_cast<long long>(nx) * yn + nxny * znw;
        if (flags[nc] != kFluid || mask[nc] != 0) continue;
        float r = 0.0f, jx = 0.0f, jy = 0.0f, jz = 0.0f;
#pragma unroll
        for (int p = 0; p < kQ; ++p) {
            const float fq = S::ld(fA + p * n, nc, wgt(p));
            r += fq;
            jx += cx(p) * fq; jy += cy(p) * fq; jz += cz(p) * fq;
        }
        rho += r;
        ux += jx / r; uy += jy / r; uz += jz / r;
        ++found;
    }
    if (found > 0) {
        const float inv = 1.0f / static_cast<float>(found);
        rho *= inv; ux *= inv; uy *= inv; uz *= inv;
    } else {
        rho = 1.0f; ux = uy = uz = 0.0f;
    }
    float feq[kQ];
    eq19(rho, ux, uy, uz, feq);
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
        S::st(fA + q * n, cell, feq[q], wgt(q));
        S::st(fB + q * n, cell, feq[q], wgt(q));
    }
}

template <class S>
cudaError_t launch_apply_flag_edits_impl(void* fA, void* fB, const std::uint8_t* flags, const std::uint8_t* mask,
                                         LevelDims d, cudaStream_t st) {
    using T = typename S::T;
    const long long n = d.cells();
    apply_flag_edits_kernel<S><<<static_cast<unsigned>((n + 255) / 256), 256, 0, st>>>(
        static_cast<T*>(fA), static_cast<T*>(fB), flags, mask, d.nx, d.ny, d.nz);
    return cudaGetLastError();
}

// ---- last fine sub-step with the restriction's child averages fused in --------
// Factor-2 patches only. A thread owns one fine x column of a 2 x 2 (y, z)
// cell group and updates its four cells in the children's summation order
// (z, then y); the x partner of each child pair is the neighbouring lane.
// The child sums stay in registers split across the lane pair (even lane:
// directions 0..9, odd lane: 10..18): per cell one shuffle per direction
// pair hands each lane the partner's value it needs, and each lane adds the
// two children in the stand-alone pass's order (z, y, x; solid children
// skipped). With FP32 storage the values summed are the stored ones, exactly
// as a later load returns them (bit-identical to the separate pass); with
// FP16 storage they are the collided FP32 values before the half rounding.
// The even lane then collects the odd lane's sums and
// writes the scratch record. This saves the stand-alone pass's full re-read
// of the fine populations (measured 3 % faster than accumulating in shared
// memory).
constexpr int kFuseX = 128;

constexpr int kSplit = 10;   // directions summed by the even lane

template <class S, bool WM, bool EXACT, bool QL>
__global__ void __launch_bounds__(kFuseX, S::kChildMinBlocks)
collide_child_kernel(const typename S::T* __restrict__ src, typename S::T* __restrict__ dst,
                     const std::uint8_t* __restrict__ kind, CollideArgs a, ChildFuse cf,
                     const __grid_constant__ PullOffsets off) {
    const int x = blockIdx.x * kFuseX + threadIdx.x;
    const bool inX = x < a.nx;
    const bool even = (threadIdx.x & 1) == 0;
    const int lx = cf.boxX0 + (x >> 1) - cf.rx0, ly = cf.boxY0 + static_cast<int>(blockIdx.y) - cf.ry0;
    // Both lanes of a pair take the record decision of the even lane.
    const int xe = x & ~1;
    const bool record = xe + 1 < a.nx && lx >= 0 && lx < cf.rw && ly >= 0 && ly < cf.rh;
    float acc[kSplit];
#pragma unroll
    for (int k = 0; k < kSplit; ++k) acc[k] = 0.0f;
    int nFluid = 0;
    // The four cells' kind bytes, read up front (one byte each in a packed
    // word), so no cell's update waits on a kind load after the previous one.
    unsigned kinds = 0;
    if (inX) {
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int y = 2 * blockIdx.y + (c & 1), z = 2 * blockIdx.z + (c >> 1);
            kinds |= static_cast<unsigned>(kind[static_cast<unsigned>(x) + static_cast<unsigned>(a.nx)
                                                * (static_cast<unsigned>(y) + static_cast<unsigned>(a.ny) * z)])
                   << (8 * c);
        }
    }
    for (int kz = 0; kz < 2; ++kz)
        for (int jy = 0; jy < 2; ++jy) {
            const int y = 2 * blockIdx.y + jy, z = 2 * blockIdx.z + kz;
            float v[kQ];
            bool solid = true;
            if (inX) {
                const unsigned cell = static_cast<unsigned>(x)
                                    + static_cast<unsigned>(a.nx) * (static_cast<unsigned>(y) + static_cast<unsigned>(a.ny) * z);
                const std::uint8_t k = static_cast<std::uint8_t>(kinds >> (8 * (2 * kz + jy)));
                const int flag = k & kFlagMask;
                if (flag == kFluid) {
                    gather_fluid<S, WM, QL, !EXACT>(src, kind, a, k, cell, x, y, z, v, &off);
                    float rr, ux, uy, uz;
                    collide_body<EXACT>(v, a, rr, ux, uy, uz);
                    // FP32: the sums see the stored values exactly. FP16:
                    // the collided FP32 values (not their half round trip),
                    // the more accurate child average.
                    store_cell<S, !EXACT>(dst, a, cell, v, &off);
                    solid = false;
                } else {
                    boundary_cell<S>(src, dst, a, flag, cell, x, y, z);
                    if (flag != kSolid) {
                        // Written or untouched, the child average sees what dst holds.
                        const typename S::T* base = dst + cell;
#pragma unroll
                        for (int q = 0; q < kQ; ++q)
                            v[q] = Pop<S, !EXACT>::ld_coherent(byte_add(base, off.slice[q]), wgt(q));
                        solid = false;
                    }
                }
            }
            if (!solid) ++nFluid;
            const bool partnerSolid = __shfl_xor_sync(0xffffffffu, static_cast<int>(solid), 1) != 0;
            // Children in order: the even lane's first, then the odd lane's.
            const bool skipFirst = even ? solid : partnerSolid;
            const bool skipSecond = even ? partnerSolid : solid;
#pragma unroll
            for (int k = 0; k < kSplit; ++k) {
                const int qo = k + kSplit < kQ ? k + kSplit : kQ - 1;   // odd lane's direction
                const float send = even ? v[qo] : v[k];
                const float recv = __shfl_xor_sync(0xffffffffu, send, 1);
                const float own = even ? v[k] : v[qo];
                const float first = even ? own : recv, second = even ? recv : own;
                if (k + kSplit < kQ || even) {
                    float t = acc[k];
                    if (!skipFirst) t += first;
                    if (!skipSecond) t += second;
                    acc[k] = t;
                }
            }
        }
    // The even lane gathers the odd lane's sums (directions 10..18) and the
    // child count, then writes the record.
    const int nOdd = __shfl_xor_sync(0xffffffffu, nFluid, 1);
    float fi[kQ];
#pragma unroll
    for (int k = 0; k < kSplit; ++k) fi[k] = acc[k];
#pragma unroll
    for (int k = 0; k + kSplit < kQ; ++k) fi[k + kSplit] = __shfl_xor_sync(0xffffffffu, acc[k], 1);
    if (!record || !even) return;
    const long long t = lx + static_cast<long long>(cf.rw) * (ly + static_cast<long long>(cf.rh) * blockIdx.z);
    write_child_record<S, !EXACT>(fi, nFluid + nOdd, reinterpret_cast<float4*>(cf.scratch) + t,
                                  static_cast<long long>(cf.rw) * cf.rh * (a.nz / 2));
}

template <class S, bool EXACT>
cudaError_t launch_collide_child_impl(const void* srcv, void* dstv, const std::uint8_t* kind, LevelDims d,
                                      const CollideParams& p, SlipField slip, const ChildFuse& cf,
                                      cudaStream_t st) {
    using T = typename S::T;
    if (d.ny % 2 || d.nz % 2 || !cf.scratch) return cudaErrorInvalidValue;
    CollideArgs a;
    a.nx = d.nx; a.ny = d.ny; a.nz = d.nz; a.n = d.cells();
    a.tau0 = p.tau; a.lambda = p.magicLambda; a.smagPre = p.smagPrefactor; a.uIn = p.uInlet;
    a.writeMacro = 0;
    a.rho = a.u = a.v = a.w = nullptr;
    a.uwx = slip.uwx; a.uwy = slip.uwy; a.uwz = slip.uwz;
    a.status = nullptr;
    a.qFrac = p.qFrac; a.ffMask = p.ffMask;
    a.links = p.links;
    const dim3 block(kFuseX);
    const dim3 grid(static_cast<unsigned>((d.nx + kFuseX - 1) / kFuseX), static_cast<unsigned>(d.ny / 2),
                    static_cast<unsigned>(d.nz / 2));
    const T* src = static_cast<const T*>(srcv);
    T* dst = static_cast<T*>(dstv);
    const bool ql = a.qFrac != nullptr;
    const PullOffsets off = pull_offsets<T>(d.nx, d.ny, a.n);
    if (slip.active())
        (ql ? collide_child_kernel<S, true, EXACT, true> : collide_child_kernel<S, true, EXACT, false>)
            <<<grid, block, 0, st>>>(src, dst, kind, a, cf, off);
    else
        (ql ? collide_child_kernel<S, false, EXACT, true> : collide_child_kernel<S, false, EXACT, false>)
            <<<grid, block, 0, st>>>(src, dst, kind, a, cf, off);
    return cudaGetLastError();
}

// ---- staged: x-rows through shared memory with bulk async copies -------------
// A persistent CTA walks rows r = blockIdx.x + k * gridDim.x (r = y + ny z).
// For every row it needs, per direction q, the full source row (y - c_y,
// z - c_z) of slice q, plus the row's kind bytes. A producer warp brings them
// into a ring of shared-memory stages with one cp.async.bulk per row piece,
// each completing on the stage's "full" mbarrier (complete_tx); consumer
// warps wait on "full", compute their cells of the row, and release the stage
// on its "empty" mbarrier (one arrive per warp). There is no block-wide
// barrier per row: warps drift by up to the ring depth, and the bytes in
// flight are set by the ring, not by resident warps. Bulk fluid cells read
// their 19 pulls from the stage (x - c_x wraps inside the row); wall-adjacent
// and boundary cells use the global-memory paths. Requires rows of a
// multiple of 16 bytes. Every wait is bounded: on a timeout the kernel sets
// *status, lets its copies in flight land (bounded) and returns.
constexpr int kConsumerWarps = 15;
constexpr int kStagedThreads = (kConsumerWarps + 1) * 32;
constexpr int kMaxStages = 8;
constexpr long long kWaitLimit = 1LL << 18; // try_wait polls (each may sleep ~20 us) before a timeout

__device__ __forceinline__ unsigned smem_addr(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(std::uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(std::uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(std::uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(std::uint64_t* bar, unsigned parity) {
    // The suspend-time hint (ns) lets a waiting warp sleep until the phase
    // completes instead of re-polling and taking issue slots.
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity), "r"(20000u)
        : "memory");
    return ok != 0;
}
/// Bounded wait on a barrier phase; false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(std::uint64_t* bar, unsigned parity) {
    for (long long i = 0; i < kWaitLimit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void bulk_g2s(void* dstSmem, const void* srcGlobal, unsigned bytes, std::uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dstSmem)),
        "l"(srcGlobal), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

/// Shared-memory layout of the ring.
struct StageLayout {
    unsigned kindBytes;  // per stage, 16-byte multiple (row bytes + alignment prefix)
    unsigned popBytes;   // per stage: 19 rows
    __host__ __device__ static unsigned header() { return 256; }
};

template <class S>
__host__ __device__ inline StageLayout stage_layout(int nx) {
    StageLayout l;
    l.kindBytes = static_cast<unsigned>(((nx + 15 + 15) / 16) * 16);
    l.popBytes = static_cast<unsigned>(kQ) * static_cast<unsigned>(nx) * sizeof(typename S::T);
    return l;
}

template <class S>
__device__ __forceinline__ void issue_row(const typename S::T* __restrict__ src,
                                          const std::uint8_t* __restrict__ kind, unsigned char* kstage,
                                          typename S::T* pstage, std::uint64_t* bar, long long row,
                                          const CollideArgs& a, unsigned kindBytes) {
    using T = typename S::T;
    const int y = static_cast<int>(row % a.ny), z = static_cast<int>(row / a.ny);
    const unsigned rowBytes = static_cast<unsigned>(a.nx) * sizeof(T);
    // Kind row: copy from the 16-byte boundary at or below its start.
    const long long kstart = row * static_cast<long long>(a.nx);
    const long long kal = kstart & ~15LL;
    const unsigned kb = static_cast<unsigned>(((kstart - kal + a.nx + 15) / 16) * 16);
    mbar_expect_tx(bar, rowBytes * kQ + kb);
    bulk_g2s(kstage, kind + kal, kb, bar);
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
        int ys = y - cy(q), zs = z - cz(q);
        ys = ys < 0 ? ys + a.ny : (ys >= a.ny ? ys - a.ny : ys);
        zs = zs < 0 ? zs + a.nz : (zs >= a.nz ? zs - a.nz : zs);
        const T* g = src + q * a.n + static_cast<long long>(a.nx) * (ys + static_cast<long long>(a.ny) * zs);
        bulk_g2s(pstage + q * a.nx, g, rowBytes, bar);
    }
    (void)kindBytes;
}

template <class S, bool WM, bool EXACT, bool QL>
__global__ void __launch_bounds__(kStagedThreads, 2)
collide_staged_kernel(const typename S::T* __restrict__ src, typename S::T* __restrict__ dst,
                      const std::uint8_t* __restrict__ kind, CollideArgs a, int stages) {
    using T = typename S::T;
    extern __shared__ __align__(128) unsigned char smem[];
    std::uint64_t* full = reinterpret_cast<std::uint64_t*>(smem);
    std::uint64_t* empty = full + kMaxStages;
    const StageLayout L = stage_layout<S>(a.nx);
    unsigned char* kring = smem + StageLayout::header();
    T* pring = reinterpret_cast<T*>(kring + static_cast<size_t>(L.kindBytes) * stages);
    const long long rows = static_cast<long long>(a.ny) * a.nz;
    const long long G = gridDim.x;
    const int nx = a.nx;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t stageElems = static_cast<size_t>(kQ) * nx;

    if (threadIdx.x == 0) {
        for (int s = 0; s < stages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kConsumerWarps);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp == kConsumerWarps) {
        // ---- producer warp: one lane issues every copy ----
        if (lane == 0) {
            long long k = 0;
            for (;; ++k) {
                const long long r = blockIdx.x + k * G;
                if (r >= rows) break;
                const int s = static_cast<int>(k % stages);
                if (k >= stages && !mbar_wait(&empty[s], static_cast<unsigned>(((k / stages) - 1) & 1))) {
                    atomicExch(a.status, 1);
                    break;
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue_row<S>(src, kind, kring + static_cast<size_t>(L.kindBytes) * s, pring + stageElems * s,
                             &full[s], r, a, L.kindBytes);
            }
            // Let every copy this CTA issued land before the CTA can exit.
            for (long long j = k - stages; j < k; ++j)
                if (j >= 0) (void)mbar_wait(&full[j % stages], static_cast<unsigned>((j / stages) & 1));
        }
        return;
    }

    // ---- consumer warps ----
    // Row k is cut into 32-cell chunks; chunk j goes to warp
    // (j + k * nchunks) mod W, so the assignment rotates from row to row and
    // every warp does the same work over a few rows.
    const int nchunks = (nx + 31) / 32;
    for (long long k = 0;; ++k) {
        const long long r = blockIdx.x + k * G;
        if (r >= rows) break;
        const int s = static_cast<int>(k % stages);
        if (!mbar_wait(&full[s], static_cast<unsigned>((k / stages) & 1))) {
            atomicExch(a.status, 1);
            break;
        }
        const unsigned sbase = smem_addr(pring + stageElems * s);
        const long long kstart = r * static_cast<long long>(nx);
        const unsigned kbase = smem_addr(kring + static_cast<size_t>(L.kindBytes) * s) + static_cast<unsigned>(kstart & 15);
        const int y = static_cast<int>(r % a.ny), z = static_cast<int>(r / a.ny);
        const int j0 = static_cast<int>(((warp - (k * nchunks) % kConsumerWarps) % kConsumerWarps + kConsumerWarps)
                                        % kConsumerWarps);
        for (int j = j0; j < nchunks; j += kConsumerWarps) {
            const int x = j * 32 + lane;
            if (x >= nx) continue;
            const unsigned cell = static_cast<unsigned>(x) + static_cast<unsigned>(nx) * static_cast<unsigned>(r);
            unsigned short kb16;
            asm volatile("ld.shared.u8 %0, [%1];" : "=h"(kb16) : "r"(kbase + static_cast<unsigned>(x)));
            const std::uint8_t kb = static_cast<std::uint8_t>(kb16);
            const int flag = kb & kFlagMask;
            if (flag != kFluid) {
                boundary_cell<S>(src, dst, a, flag, cell, x, y, z);
                continue;
            }
            float f[kQ];
            if (!(kb & kNearWall)) {
                const int xs[3] = {wrap_inc(x, nx), x, wrap_dec(x, nx)};
                const unsigned rowBytes = static_cast<unsigned>(nx) * sizeof(T);
#pragma unroll
                for (int q = 0; q < kQ; ++q) f[q] = Pop<S, !EXACT>::lds(sbase + q * rowBytes, xs[1 + cx(q)], wgt(q));
            } else {
                const Nbr b = neighbours(x, y, z, nx, a.ny, a.nz);
                gather_wall<S, WM, QL, !EXACT>(src, kind, a, b, cell, y, z, f);
            }
            finish_cell<S, EXACT>(dst, a, cell, f);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
    }
}

// ---- launch ------------------------------------------------------------------
struct StagedPlan {
    int stages = 0;
    size_t smem = 0;
};

template <class S>
StagedPlan staged_plan(LevelDims d) {
    StagedPlan p;
    const size_t rowBytes = static_cast<size_t>(d.nx) * sizeof(typename S::T);
    if (rowBytes % 16 != 0 || d.nx < 8) return p;
    const StageLayout L = stage_layout<S>(d.nx);
    const size_t stageBytes = static_cast<size_t>(L.kindBytes) + L.popBytes;
    // Two CTAs per SM (113 KB each), each with as deep a ring as fits
    // (2..8 stages).
    const size_t budget = 113 * 1024 - StageLayout::header();
    const long long st = static_cast<long long>(budget / stageBytes);
    if (st < 2) return p;
    p.stages = static_cast<int>(st > kMaxStages ? kMaxStages : st);
    p.smem = StageLayout::header() + stageBytes * static_cast<size_t>(p.stages);
    return p;
}

inline int sm_count() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

template <class S, bool EXACT>
cudaError_t launch_collide_impl(const void* srcv, void* dstv, const std::uint8_t* kind, LevelDims d,
                                const CollideParams& p, float* rho, float* u, float* v, float* w, SlipField slip,
                                cudaStream_t st) {
    using T = typename S::T;
    CollideArgs a;
    a.nx = d.nx; a.ny = d.ny; a.nz = d.nz; a.n = d.cells();
    a.tau0 = p.tau; a.lambda = p.magicLambda; a.smagPre = p.smagPrefactor; a.uIn = p.uInlet;
    a.writeMacro = (p.writeMacro && rho && u && v && w) ? 1 : 0;
    a.rho = rho; a.u = u; a.v = v; a.w = w;
    a.uwx = slip.uwx; a.uwy = slip.uwy; a.uwz = slip.uwz;
    a.status = p.status;
    a.qFrac = p.qFrac; a.ffMask = p.ffMask;
    a.links = p.links;
    const T* src = static_cast<const T*>(srcv);
    T* dst = static_cast<T*>(dstv);
    const bool wm = slip.active();
    const StagedPlan plan = staged_plan<S>(d);
    // Automatic selection takes the one-cell kernel: on a GB300 the staged
    // ring measured slower (1.43-1.57 ms vs 0.89 ms per FP32 collide launch
    // on the 640x192x192 airfoil tunnel), its consumer warps being issue-bound
    // on shared-memory reads and ring bookkeeping.
    const bool staged = p.status && plan.stages >= 2 && p.kernel == 2;
    if (staged) {
        const bool ql = a.qFrac != nullptr;
        auto kern = wm ? (ql ? collide_staged_kernel<S, true, EXACT, true> : collide_staged_kernel<S, true, EXACT, false>)
                       : (ql ? collide_staged_kernel<S, false, EXACT, true> : collide_staged_kernel<S, false, EXACT, false>);
        // The dynamic shared-memory limit is a per-kernel attribute: raise it
        // once to the device's opt-in maximum (levels of one solver use
        // different stage sizes); occupancy is cached per (kernel, size).
        static const void* raised[8] = {};
        bool isRaised = false;
        for (const void* k : raised) isRaised |= (k == reinterpret_cast<const void*>(kern));
        if (!isRaised) {
            int dev = 0, optin = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
            if (static_cast<size_t>(optin) < plan.smem) return cudaErrorInvalidValue;
            if (auto e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
                e != cudaSuccess)
                return e;
            for (const void*& k : raised)
                if (!k) { k = reinterpret_cast<const void*>(kern); break; }
        }
        struct Entry { const void* k; size_t smem; int perSm; };
        static Entry cache[16] = {};
        int perSm = 0;
        for (const Entry& c : cache)
            if (c.k == reinterpret_cast<const void*>(kern) && c.smem == plan.smem) perSm = c.perSm;
        if (perSm == 0) {
            if (auto e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kern, kStagedThreads, plan.smem);
                e != cudaSuccess)
                return e;
            if (perSm < 1) perSm = 1;
            for (Entry& c : cache)
                if (c.k == nullptr) { c = Entry{reinterpret_cast<const void*>(kern), plan.smem, perSm}; break; }
        }
        const long long rows = static_cast<long long>(d.ny) * d.nz;
        long long grid = static_cast<long long>(sm_count()) * perSm;
        if (grid > rows) grid = rows;
        kern<<<static_cast<unsigned>(grid), kStagedThreads, plan.smem, st>>>(src, dst, kind, a, plan.stages);
        return cudaGetLastError();
    }
    const int bx = d.nx >= kCellBlockX ? kCellBlockX : ((d.nx + 31) / 32) * 32;
    const dim3 grid(static_cast<unsigned>((d.nx + bx - 1) / bx), static_cast<unsigned>(d.ny),
                    static_cast<unsigned>(d.nz));
    const PullOffsets off = pull_offsets<T>(d.nx, d.ny, a.n);
    if (d.nx % 32 != 0 && d.nx >= 2 && d.ny >= 2) {
        const FastDiv fx = fast_div(static_cast<unsigned>(d.nx)), fy = fast_div(static_cast<unsigned>(d.ny));
        const unsigned blocks = static_cast<unsigned>((a.n + kCellBlockX - 1) / kCellBlockX);
        const bool ql = a.qFrac != nullptr;
        auto kern = wm ? (ql ? collide_flat_kernel<S, true, EXACT, true> : collide_flat_kernel<S, true, EXACT, false>)
                       : (ql ? collide_flat_kernel<S, false, EXACT, true> : collide_flat_kernel<S, false, EXACT, false>);
        kern<<<blocks, kCellBlockX, 0, st>>>(src, dst, kind, a, off, fx, fy);
        return cudaGetLastError();
    }
    if (a.qFrac) {
        if (wm) collide_cell_kernel<S, true, EXACT, true><<<grid, bx, 0, st>>>(src, dst, kind, a, off);
        else collide_cell_kernel<S, false, EXACT, true><<<grid, bx, 0, st>>>(src, dst, kind, a, off);
    } else {
        if (wm) collide_cell_kernel<S, true, EXACT, false><<<grid, bx, 0, st>>>(src, dst, kind, a, off);
        else collide_cell_kernel<S, false, EXACT, false><<<grid, bx, 0, st>>>(src, dst, kind, a, off);
    }
    return cudaGetLastError();
}

} // namespace
} // namespace fcfd
