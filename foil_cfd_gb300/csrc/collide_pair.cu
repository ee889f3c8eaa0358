// Two-cells-per-thread stream-collide on Blackwell packed FP32 arithmetic.
//
// Each thread updates an x-pair of cells (x0, x0+1), x0 even. For the 9
// directions with c_x = 0 both pulled populations sit side by side, so they
// are fetched with one 8-byte (FP32) or 4-byte (FP16) load, and every store is
// one vector store; index arithmetic is shared by the pair. The collision of
// the two cells runs on float2 operands with the sm_100-family packed
// instructions (FADD2 / FMUL2 / FFMA2 via __fadd2_rn, __fmul2_rn,
// __ffma2_rn), which round each lane exactly like the scalar IEEE operation,
// so the pair costs about as many instructions as one cell did.
//
// Two collision bodies:
//  * reference order (FP32 storage): the reference kernel's expression tree,
//    lane by lane (src/sim/lbm_core.cu:386-467), no contraction (this unit is
//    built with --fmad=false) -- bit-identical to the reference step;
//  * pair-sum order (FP16 storage): moments, stress and TRT from opposite-pair
//    sums/differences with fused multiply-adds.
// Pairs in which a cell is not bulk fluid (boundary flags, wall neighbours)
// take a per-lane path with the same boundary handling as the one-cell
// kernels. Requires an even nx; odd nx grids use the one-cell kernels.
#include "d3q19.cuh"
#include "kernels.h"

#include <cuda_runtime.h>

namespace fcfd {
namespace {

constexpr int kPairBlock = 64; // threads per block = 128 cells of one x-row

struct PairArgs {
    int nx, ny, nz;
    long long n;
    float tau0, lambda, smagPre, uIn;
    int writeMacro;
    float *rho, *u, *v, *w;
    const std::uint16_t *uwx, *uwy, *uwz;
};

__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 sp(float s) { return make_float2(s, s); }

// ---- storage of pairs ------------------------------------------------------
struct PairF32 {
    using T = float;
    using S1 = StoreF32;
    __device__ __forceinline__ static float2 ld2(const T* p, long long i, float) {
        return __ldg(reinterpret_cast<const float2*>(p + i));
    }
    __device__ __forceinline__ static void st2(T* p, long long i, float2 v, float) {
        *reinterpret_cast<float2*>(p + i) = v;
    }
};
struct PairF16 {
    using T = __half;
    using S1 = StoreF16;
    __device__ __forceinline__ static float2 ld2(const T* p, long long i, float w) {
        const __half2 h = __ldg(reinterpret_cast<const __half2*>(p + i));
        return add2(__half22float2(h), sp(w));
    }
    __device__ __forceinline__ static void st2(T* p, long long i, float2 v, float w) {
        *reinterpret_cast<__half2*>(p + i) = __float22half2_rn(sub2(v, sp(w)));
    }
};

// ---- collision bodies -------------------------------------------------------
__device__ __forceinline__ float2 rcp2(float2 a) { return make_float2(1.0f / a.x, 1.0f / a.y); }

/// Reference expression order, both lanes (lbm_core.cu:386-467).
__device__ __forceinline__ void collide_ref2(float2 (&f)[kQ], float tau0, float lambda, float smagPre,
                                             float2& rhoO, float2& uxO, float2& uyO, float2& uzO) {
    float2 rho = sp(0.0f), jx = sp(0.0f), jy = sp(0.0f), jz = sp(0.0f);
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
        rho = add2(rho, f[q]);
        if (cx(q) != 0) jx = cx(q) > 0 ? add2(jx, f[q]) : sub2(jx, f[q]);
        if (cy(q) != 0) jy = cy(q) > 0 ? add2(jy, f[q]) : sub2(jy, f[q]);
        if (cz(q) != 0) jz = cz(q) > 0 ? add2(jz, f[q]) : sub2(jz, f[q]);
    }
    rho = make_float2(fmaxf(rho.x, kRhoFloor), fmaxf(rho.y, kRhoFloor));
    const float2 invRho = rcp2(rho);
    float2 ux = mul2(jx, invRho), uy = mul2(jy, invRho), uz = mul2(jz, invRho);
    float2 u2 = add2(add2(mul2(ux, ux), mul2(uy, uy)), mul2(uz, uz));
    constexpr float cap2 = kMaxSimSpeed * kMaxSimSpeed;
    if (u2.x > cap2 || u2.y > cap2) {
        if (u2.x > cap2) {
            const float s = kMaxSimSpeed * (1.0f / sqrtf(u2.x));
            ux.x *= s; uy.x *= s; uz.x *= s;
        }
        if (u2.y > cap2) {
            const float s = kMaxSimSpeed * (1.0f / sqrtf(u2.y));
            ux.y *= s; uy.y *= s; uz.y *= s;
        }
        u2 = add2(add2(mul2(ux, ux), mul2(uy, uy)), mul2(uz, uz));
    }
    // Equilibrium: (w rho) * (((1 + cu) + (0.5 cu) cu) - usq), cu = 3 (c . u).
    const float2 usq = mul2(sp(1.5f), u2);
    const float2 wr0 = mul2(sp(wgt(0)), rho), wr1 = mul2(sp(wgt(1)), rho), wr2 = mul2(sp(wgt(7)), rho);
    float2 feq[kQ];
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
        float2 dot = sp(0.0f);
        bool any = false;
        if (cx(q) != 0) { dot = cx(q) > 0 ? ux : make_float2(-ux.x, -ux.y); any = true; }
        if (cy(q) != 0) {
            if (any) dot = cy(q) > 0 ? add2(dot, uy) : sub2(dot, uy);
            else dot = cy(q) > 0 ? uy : make_float2(-uy.x, -uy.y);
            any = true;
        }
        if (cz(q) != 0) {
            if (any) dot = cz(q) > 0 ? add2(dot, uz) : sub2(dot, uz);
            else dot = cz(q) > 0 ? uz : make_float2(-uz.x, -uz.y);
        }
        const float2 cu = mul2(sp(3.0f), dot);
        const float2 t = sub2(add2(add2(sp(1.0f), cu), mul2(mul2(sp(0.5f), cu), cu)), usq);
        feq[q] = mul2(q == 0 ? wr0 : (q <= 6 ? wr1 : wr2), t);
    }
    float2 tauEff = sp(tau0);
    if (smagPre > 0.0f) {
        float2 pxx = sp(0.0f), pyy = sp(0.0f), pzz = sp(0.0f), pxy = sp(0.0f), pxz = sp(0.0f), pyz = sp(0.0f);
#pragma unroll
        for (int q = 0; q < kQ; ++q) {
            const float2 fneq = sub2(f[q], feq[q]);
            if (cx(q) != 0) pxx = add2(pxx, fneq);
            if (cy(q) != 0) pyy = add2(pyy, fneq);
            if (cz(q) != 0) pzz = add2(pzz, fneq);
            if (cx(q) * cy(q) != 0) pxy = cx(q) * cy(q) > 0 ? add2(pxy, fneq) : sub2(pxy, fneq);
            if (cx(q) * cz(q) != 0) pxz = cx(q) * cz(q) > 0 ? add2(pxz, fneq) : sub2(pxz, fneq);
            if (cy(q) * cz(q) != 0) pyz = cy(q) * cz(q) > 0 ? add2(pyz, fneq) : sub2(pyz, fneq);
        }
        const float2 s1 = add2(add2(mul2(pxx, pxx), mul2(pyy, pyy)), mul2(pzz, pzz));
        const float2 s2 = add2(add2(mul2(pxy, pxy), mul2(pxz, pxz)), mul2(pyz, pyz));
        const float2 ss = add2(s1, mul2(sp(2.0f), s2));
        const float2 qbar = make_float2(sqrtf(ss.x), sqrtf(ss.y));
        const float2 inner = add2(mul2(sp(tau0), sp(tau0)), mul2(mul2(sp(smagPre), qbar), invRho));
        tauEff = mul2(sp(0.5f), add2(sp(tau0), make_float2(sqrtf(inner.x), sqrtf(inner.y))));
    }
    const float2 omP = rcp2(tauEff);
    const float2 dm = sub2(tauEff, sp(0.5f));
    const float2 tauM = add2(sp(0.5f), make_float2(lambda / dm.x, lambda / dm.y));
    const float2 omM = rcp2(tauM);
    f[0] = sub2(f[0], mul2(omP, sub2(f[0], feq[0])));
#pragma unroll
    for (int p = 1; p <= 9; ++p) {
        const int a = 2 * p - 1, b = 2 * p;
        const float2 sym = mul2(omP, sub2(mul2(sp(0.5f), add2(f[a], f[b])), mul2(sp(0.5f), add2(feq[a], feq[b]))));
        const float2 asym = mul2(omM, sub2(mul2(sp(0.5f), sub2(f[a], f[b])), mul2(sp(0.5f), sub2(feq[a], feq[b]))));
        const float2 fa = f[a];
        f[a] = sub2(sub2(fa, sym), asym);
        f[b] = add2(sub2(f[b], sym), asym);
    }
    rhoO = rho; uxO = ux; uyO = uy; uzO = uz;
}

/// Pair-sum order with fused multiply-adds (FP16 storage).
__device__ __forceinline__ void collide_fast2(float2 (&f)[kQ], float tau0, float lambda, float smagPre,
                                              float2& rhoO, float2& uxO, float2& uyO, float2& uzO) {
    float2 s[10], d[10];
#pragma unroll
    for (int p = 1; p <= 9; ++p) {
        s[p] = add2(f[2 * p - 1], f[2 * p]);
        d[p] = sub2(f[2 * p - 1], f[2 * p]);
    }
    float2 rho = add2(add2(add2(f[0], add2(add2(s[1], s[2]), add2(s[3], s[4]))),
                           add2(add2(s[5], s[6]), add2(s[7], s[8]))), s[9]);
    const float2 jx = add2(add2(add2(d[1], d[4]), add2(d[5], d[7])), d[8]);
    const float2 jy = add2(add2(add2(d[2], d[4]), sub2(d[6], d[7])), d[9]);
    const float2 jz = sub2(add2(add2(d[3], d[5]), sub2(d[6], d[8])), d[9]);
    rho = make_float2(fmaxf(rho.x, kRhoFloor), fmaxf(rho.y, kRhoFloor));
    const float2 inv = make_float2(__frcp_rn(rho.x), __frcp_rn(rho.y));
    float2 ux = mul2(jx, inv), uy = mul2(jy, inv), uz = mul2(jz, inv);
    float2 u2 = fma2(uz, uz, fma2(uy, uy, mul2(ux, ux)));
    constexpr float cap2 = kMaxSimSpeed * kMaxSimSpeed;
    if (u2.x > cap2 || u2.y > cap2) {
        if (u2.x > cap2) { const float sc = kMaxSimSpeed * rsqrtf(u2.x); ux.x *= sc; uy.x *= sc; uz.x *= sc; }
        if (u2.y > cap2) { const float sc = kMaxSimSpeed * rsqrtf(u2.y); ux.y *= sc; uy.y *= sc; uz.y *= sc; }
        u2 = fma2(uz, uz, fma2(uy, uy, mul2(ux, ux)));
    }
    float2 tauEff = sp(tau0);
    if (smagPre > 0.0f) {
        const float2 pxx = add2(add2(add2(s[1], s[4]), add2(s[5], s[7])), s[8]);
        const float2 pyy = add2(add2(add2(s[2], s[4]), add2(s[6], s[7])), s[9]);
        const float2 pzz = add2(add2(add2(s[3], s[5]), add2(s[6], s[8])), s[9]);
        const float2 r3 = mul2(rho, sp(1.0f / 3.0f));
        const float2 rux = mul2(rho, ux), ruy = mul2(rho, uy), ruz = mul2(rho, uz);
        // Pi(f) - (rho/3 I + rho u u)
        const float2 nxx = sub2(sub2(pxx, r3), mul2(rux, ux));
        const float2 nyy = sub2(sub2(pyy, r3), mul2(ruy, uy));
        const float2 nzz = sub2(sub2(pzz, r3), mul2(ruz, uz));
        const float2 nxy = sub2(sub2(s[4], s[7]), mul2(rux, uy));
        const float2 nxz = sub2(sub2(s[5], s[8]), mul2(rux, uz));
        const float2 nyz = sub2(sub2(s[6], s[9]), mul2(ruy, uz));
        const float2 off = fma2(nyz, nyz, fma2(nxz, nxz, mul2(nxy, nxy)));
        const float2 ss = fma2(sp(2.0f), off, fma2(nzz, nzz, fma2(nyy, nyy, mul2(nxx, nxx))));
        const float2 qbar = make_float2(sqrtf(ss.x), sqrtf(ss.y));
        const float2 inner = fma2(mul2(sp(smagPre), qbar), inv, sp(tau0 * tau0));
        tauEff = mul2(sp(0.5f), add2(sp(tau0), make_float2(sqrtf(inner.x), sqrtf(inner.y))));
    }
    const float2 omP = make_float2(__frcp_rn(tauEff.x), __frcp_rn(tauEff.y));
    const float2 dm = sub2(tauEff, sp(0.5f));
    const float2 omM = make_float2(__frcp_rn(0.5f + __fdiv_rn(lambda, dm.x)),
                                   __frcp_rn(0.5f + __fdiv_rn(lambda, dm.y)));
    const float2 base = fma2(sp(-1.5f), u2, sp(1.0f));
    const float2 r0 = mul2(rho, sp(1.0f / 3.0f)), r1 = mul2(rho, sp(1.0f / 18.0f)), r2 = mul2(rho, sp(1.0f / 36.0f));
    f[0] = fma2(make_float2(-omP.x, -omP.y), sub2(f[0], mul2(r0, base)), f[0]);
    const float2 nomP = make_float2(-omP.x, -omP.y);
#pragma unroll
    for (int p = 1; p <= 9; ++p) {
        const int a = 2 * p - 1;
        const float2 wr = p <= 3 ? r1 : r2;
        float2 cu;
        {
            float2 t = sp(0.0f);
            bool any = false;
            if (cx(a) != 0) { t = cx(a) > 0 ? ux : make_float2(-ux.x, -ux.y); any = true; }
            if (cy(a) != 0) { t = any ? (cy(a) > 0 ? add2(t, uy) : sub2(t, uy)) : (cy(a) > 0 ? uy : make_float2(-uy.x, -uy.y)); any = true; }
            if (cz(a) != 0) { t = any ? (cz(a) > 0 ? add2(t, uz) : sub2(t, uz)) : (cz(a) > 0 ? uz : make_float2(-uz.x, -uz.y)); }
            cu = t;
        }
        const float2 es = mul2(wr, fma2(sp(4.5f), mul2(cu, cu), base));
        const float2 ea = mul2(mul2(sp(3.0f), wr), cu);
        const float2 t1 = mul2(omP, fma2(sp(0.5f), s[p], make_float2(-es.x, -es.y)));
        const float2 t2 = mul2(omM, fma2(sp(0.5f), d[p], make_float2(-ea.x, -ea.y)));
        const float2 fa = f[a];
        f[a] = sub2(sub2(fa, t1), t2);
        f[a + 1] = add2(sub2(f[a + 1], t1), t2);
    }
    (void)nomP;
    rhoO = rho; uxO = ux; uyO = uy; uzO = uz;
}

// ---- per-lane handling of pairs that touch a boundary or a wall -----------
/// Returns true when the lane's cell is fluid and its 19 pulled populations
/// are in out[]; otherwise the boundary cell has been written (as in the
/// one-cell kernels) and the lane is excluded from the collision.
template <class S1, bool WM, bool EXACT>
__device__ __forceinline__ bool lane_gather(const typename S1::T* __restrict__ src, typename S1::T* __restrict__ dst,
                                            const std::uint8_t* __restrict__ kind, const PairArgs& a, int x, int y,
                                            int z, unsigned cell, std::uint8_t k, float (&out)[kQ]) {
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const long long n = a.n;
    const unsigned unx = nx, uny = ny;
    const int flag = k & kFlagMask;
    const int xm = wrap_dec(x, nx), xp = wrap_inc(x, nx);
    const unsigned sx[3] = {static_cast<unsigned>(xp), static_cast<unsigned>(x), static_cast<unsigned>(xm)};
    const unsigned sy[3] = {static_cast<unsigned>(wrap_inc(y, ny)), static_cast<unsigned>(y),
                            static_cast<unsigned>(wrap_dec(y, ny))};
    const unsigned sz[3] = {static_cast<unsigned>(wrap_inc(z, nz)), static_cast<unsigned>(z),
                            static_cast<unsigned>(wrap_dec(z, nz))};
    if (flag != kFluid) {
        if (flag == kInlet) {
            // Reference equilibrium19(1, uIn, 0, 0).
            const float usq = 1.5f * (a.uIn * a.uIn + 0.0f * 0.0f + 0.0f * 0.0f);
#pragma unroll
            for (int q = 0; q < kQ; ++q) {
                const float cu = 3.0f * (cx(q) != 0 ? (cx(q) > 0 ? a.uIn : -a.uIn) : 0.0f);
                const float fe = (wgt(q) * 1.0f) * (1.0f + cu + 0.5f * cu * cu - usq);
                S1::st(dst + q * n, cell, fe, wgt(q));
            }
            if (a.writeMacro) { a.rho[cell] = 1.0f; a.u[cell] = a.uIn; a.v[cell] = 0.0f; a.w[cell] = 0.0f; }
        } else if (flag == kOutlet || flag == kOutletEq) {
            const unsigned up = static_cast<unsigned>(xm) + unx * (static_cast<unsigned>(y) + uny * z);
            float g[kQ];
            float r = 0.0f, jx = 0.0f, jy = 0.0f, jz = 0.0f;
#pragma unroll
            for (int q = 0; q < kQ; ++q) {
                g[q] = S1::ld(src + q * n, up, wgt(q));
                r += g[q];
                if (cx(q) != 0) jx = cx(q) > 0 ? jx + g[q] : jx - g[q];
                if (cy(q) != 0) jy = cy(q) > 0 ? jy + g[q] : jy - g[q];
                if (cz(q) != 0) jz = cz(q) > 0 ? jz + g[q] : jz - g[q];
            }
            const float inv = 1.0f / r;
            const float ux = jx * inv, uy = jy * inv, uz = jz * inv;
            if (flag == kOutletEq) {
                const float usq = 1.5f * (ux * ux + uy * uy + uz * uz);
#pragma unroll
                for (int q = 0; q < kQ; ++q) {
                    float dot = 0.0f;
                    bool any = false;
                    if (cx(q) != 0) { dot = cx(q) > 0 ? ux : -ux; any = true; }
                    if (cy(q) != 0) { const float t = cy(q) > 0 ? uy : -uy; dot = any ? dot + t : t; any = true; }
                    if (cz(q) != 0) { const float t = cz(q) > 0 ? uz : -uz; dot = any ? dot + t : t; }
                    const float cu = 3.0f * dot;
                    g[q] = wgt(q) * (1.0f + cu + 0.5f * cu * cu - usq);
                }
                r = 1.0f;
            }
#pragma unroll
            for (int q = 0; q < kQ; ++q) S1::st(dst + q * n, cell, g[q], wgt(q));
            if (a.writeMacro) { a.rho[cell] = r; a.u[cell] = ux; a.v[cell] = uy; a.w[cell] = uz; }
        } else if (a.writeMacro) {
            a.rho[cell] = 1.0f; a.u[cell] = 0.0f; a.v[cell] = 0.0f; a.w[cell] = 0.0f;
        }
        return false;
    }
    if (!(k & kNearWall)) {
#pragma unroll
        for (int q = 0; q < kQ; ++q)
            out[q] = S1::ld(src + q * n, sx[1 + cx(q)] + unx * (sy[1 + cy(q)] + uny * sz[1 + cz(q)]), wgt(q));
        return true;
    }
    float uwx = 0.0f, uwy = 0.0f, uwz = 0.0f;
    bool uwLoaded = false;
    out[0] = S1::ld(src, cell, wgt(0));
#pragma unroll
    for (int q = 1; q < kQ; ++q) {
        const unsigned X = sx[1 + cx(q)], Y = sy[1 + cy(q)], Z = sz[1 + cz(q)];
        const unsigned pn = X + unx * (Y + uny * Z);
        const int nf = kind[pn] & kFlagMask;
        const bool solid = nf == kSolid;
        const bool slipY = is_slip_y(nf);
        const bool slipZ = is_slip_z(nf);
        const unsigned pY = X + unx * (static_cast<unsigned>(y) + uny * Z);
        const unsigned pZ = X + unx * (Y + uny * static_cast<unsigned>(z));
        const int qs = solid ? opp(q) : (slipY ? mir_y(q) : (slipZ ? mir_z(q) : q));
        const unsigned cs = solid ? cell : (slipY ? pY : (slipZ ? pZ : pn));
        float fq = S1::ld(src + static_cast<long long>(qs) * n, cs, wgt(q));
        if constexpr (WM) {
            if (solid) {
                if (!uwLoaded) {
                    uwx = __half2float(__ushort_as_half(a.uwx[cell]));
                    uwy = __half2float(__ushort_as_half(a.uwy[cell]));
                    uwz = __half2float(__ushort_as_half(a.uwz[cell]));
                    uwLoaded = true;
                }
                float dot = 0.0f;
                bool any = false;
                if (cx(q) != 0) { dot = cx(q) > 0 ? uwx : -uwx; any = true; }
                if (cy(q) != 0) { const float t = cy(q) > 0 ? uwy : -uwy; dot = any ? dot + t : t; any = true; }
                if (cz(q) != 0) { const float t = cz(q) > 0 ? uwz : -uwz; dot = any ? dot + t : t; }
                fq += (6.0f * wgt(q)) * dot;
            }
        }
        out[q] = fq;
    }
    return true;
}

template <class PS, bool WM, bool EXACT>
__global__ void __launch_bounds__(kPairBlock)
collide_pair_kernel(const typename PS::T* __restrict__ src, typename PS::T* __restrict__ dst,
                    const std::uint8_t* __restrict__ kind, PairArgs a) {
    using S1 = typename PS::S1;
    const int x0 = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    if (x0 >= a.nx) return;
    const int y = blockIdx.y, z = blockIdx.z;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const long long n = a.n;
    const unsigned unx = nx, uny = ny;
    const unsigned cell = static_cast<unsigned>(x0) + unx * (static_cast<unsigned>(y) + uny * z);
    const std::uint16_t kk = __ldg(reinterpret_cast<const std::uint16_t*>(kind + cell));
    const std::uint8_t k0 = kk & 0xFF, k1 = kk >> 8;

    float2 f[kQ];
    bool act0 = true, act1 = true;
    if (kk == 0) {
        // Both cells bulk fluid.
        const unsigned yr[3] = {static_cast<unsigned>(wrap_inc(y, ny)), static_cast<unsigned>(y),
                                static_cast<unsigned>(wrap_dec(y, ny))};
        const unsigned zr[3] = {static_cast<unsigned>(wrap_inc(z, nz)), static_cast<unsigned>(z),
                                static_cast<unsigned>(wrap_dec(z, nz))};
        const unsigned xl = static_cast<unsigned>(wrap_dec(x0, nx));      // x0 - 1
        const unsigned xr = static_cast<unsigned>(wrap_inc(x0 + 1, nx));  // x0 + 2
#pragma unroll
        for (int q = 0; q < kQ; ++q) {
            const unsigned row = unx * (yr[1 + cy(q)] + uny * zr[1 + cz(q)]);
            const typename PS::T* p = src + q * n;
            if (cx(q) == 0) {
                f[q] = PS::ld2(p, row + x0, wgt(q));
            } else if (cx(q) > 0) { // pulls x0-1, x0
                f[q] = make_float2(S1::ld(p, row + xl, wgt(q)), S1::ld(p, row + x0, wgt(q)));
            } else {                // pulls x0+1, x0+2
                f[q] = make_float2(S1::ld(p, row + x0 + 1, wgt(q)), S1::ld(p, row + xr, wgt(q)));
            }
        }
    } else {
        float g0[kQ], g1[kQ];
        act0 = lane_gather<S1, WM, EXACT>(src, dst, kind, a, x0, y, z, cell, k0, g0);
        act1 = lane_gather<S1, WM, EXACT>(src, dst, kind, a, x0 + 1, y, z, cell + 1, k1, g1);
        if (!act0 && !act1) return;
#pragma unroll
        for (int q = 0; q < kQ; ++q) f[q] = make_float2(act0 ? g0[q] : g1[q], act1 ? g1[q] : g0[q]);
    }

    float2 rho, ux, uy, uz;
    if constexpr (EXACT) collide_ref2(f, a.tau0, a.lambda, a.smagPre, rho, ux, uy, uz);
    else collide_fast2(f, a.tau0, a.lambda, a.smagPre, rho, ux, uy, uz);

    if (act0 && act1) {
#pragma unroll
        for (int q = 0; q < kQ; ++q) PS::st2(dst + q * n, cell, f[q], wgt(q));
        if (a.writeMacro) {
            *reinterpret_cast<float2*>(a.rho + cell) = rho;
            *reinterpret_cast<float2*>(a.u + cell) = ux;
            *reinterpret_cast<float2*>(a.v + cell) = uy;
            *reinterpret_cast<float2*>(a.w + cell) = uz;
        }
    } else {
        const unsigned c = act0 ? cell : cell + 1;
#pragma unroll
        for (int q = 0; q < kQ; ++q) S1::st(dst + q * n, c, act0 ? f[q].x : f[q].y, wgt(q));
        if (a.writeMacro) {
            a.rho[c] = act0 ? rho.x : rho.y;
            a.u[c] = act0 ? ux.x : ux.y;
            a.v[c] = act0 ? uy.x : uy.y;
            a.w[c] = act0 ? uz.x : uz.y;
        }
    }
}

template <class PS, bool EXACT>
void dispatch(const void* src, void* dst, const std::uint8_t* kind, LevelDims d, const PairArgs& a, bool wm,
              cudaStream_t st) {
    const int pairs = d.nx / 2;
    const int bx = pairs >= kPairBlock ? kPairBlock : ((pairs + 31) / 32) * 32;
    const dim3 grid(static_cast<unsigned>((pairs + bx - 1) / bx), static_cast<unsigned>(d.ny),
                    static_cast<unsigned>(d.nz));
    auto* s = static_cast<const typename PS::T*>(src);
    auto* t = static_cast<typename PS::T*>(dst);
    if (wm) collide_pair_kernel<PS, true, EXACT><<<grid, bx, 0, st>>>(s, t, kind, a);
    else collide_pair_kernel<PS, false, EXACT><<<grid, bx, 0, st>>>(s, t, kind, a);
}

} // namespace

bool pair_kernel_applies(LevelDims d) { return d.nx >= 2 && (d.nx % 2) == 0; }

cudaError_t launch_collide_pair(Storage s, const void* src, void* dst, const std::uint8_t* kind, LevelDims d,
                                const CollideParams& p, float* rho, float* u, float* v, float* w, SlipField slip,
                                cudaStream_t st) {
    if (!pair_kernel_applies(d)) return cudaErrorInvalidValue;
    PairArgs a;
    a.nx = d.nx; a.ny = d.ny; a.nz = d.nz; a.n = d.cells();
    a.tau0 = p.tau; a.lambda = p.magicLambda; a.smagPre = p.smagPrefactor; a.uIn = p.uInlet;
    a.writeMacro = (p.writeMacro && rho && u && v && w) ? 1 : 0;
    a.rho = rho; a.u = u; a.v = v; a.w = w;
    a.uwx = slip.uwx; a.uwy = slip.uwy; a.uwz = slip.uwz;
    if (s == Storage::F32) dispatch<PairF32, true>(src, dst, kind, d, a, slip.active(), st);
    else dispatch<PairF16, false>(src, dst, kind, d, a, slip.active(), st);
    return cudaGetLastError();
}

} // namespace fcfd
