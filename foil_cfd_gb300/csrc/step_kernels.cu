// Fused D3Q19 stream-collide (pull scheme, TRT + Smagorinsky, optional iMEM
// moving-wall term) and the small per-level kernels around it: cell-kind
// classification, equilibrium / speck / macroscopic initialisation, the NaN
// watchdog and FP32 <-> storage conversion.
//
// Physics follows the reference step (src/sim/lbm_core.cu:213-475): per link
// the upstream neighbour's flag selects plain streaming, half-way bounce-back
// (opposite slot of this cell), or specular free slip (mirrored slot of the
// tangentially displaced cell); moments with a density floor of 0.05; a
// velocity limiter at |u| = 0.3; Smagorinsky tau_eff from the non-equilibrium
// stress (Hou et al. 1996); TRT with magic parameter Lambda.
//
// GB300 layout choices (not in the reference): the buffers are unpadded SoA
// and all three axes wrap periodically in the index math, so there is no
// ghost-plane refresh pass; a per-cell kind byte marks the fluid cells that
// touch a wall, so bulk cells stream without reading 18 neighbour flags; the
// collision works on opposite-pair sums/differences, with the equilibrium's
// second moment in closed form (rho/3 I + rho u u) instead of 19 fneq terms.
#include "d3q19.cuh"
#include "kernels.h"

#include <cuda_runtime.h>

namespace fcfd {
namespace {

constexpr int kCollideBlockX = 128;
constexpr int kBlock1D = 256;

struct CollideArgs {
    int nx, ny, nz;
    long long n; // cells per direction slice
    float tau0, lambda, smagPre, uIn;
    int writeMacro;
    float* rho;
    float* u;
    float* v;
    float* w;
    const std::uint16_t* uwx;
    const std::uint16_t* uwy;
    const std::uint16_t* uwz;
};

/// TRT + Smagorinsky collision of one cell, in place on f[19].
/// Pairs (a, a+1) for odd a carry opposite velocities, so with
/// s = f_a + f_b and d = f_a - f_b the moments, the momentum-flux tensor and
/// the TRT update are all formed from 9 sums and 9 differences.
__device__ __forceinline__ void collide_trt(float (&f)[kQ], float tau0,
                                            float lambda, float smagPre,
                                            float& rhoOut, float& uxOut,
                                            float& uyOut, float& uzOut) {
    float s[10], d[10];
#pragma unroll
    for (int p = 1; p <= 9; ++p) {
        s[p] = f[2 * p - 1] + f[2 * p];
        d[p] = f[2 * p - 1] - f[2 * p];
    }
    // Pair p has velocity c_{2p-1}: p1 (1,0,0) p2 (0,1,0) p3 (0,0,1)
    // p4 (1,1,0) p5 (1,0,1) p6 (0,1,1) p7 (1,-1,0) p8 (1,0,-1) p9 (0,1,-1).
    float rho = f[0] + ((s[1] + s[2]) + (s[3] + s[4])) + ((s[5] + s[6]) + (s[7] + s[8])) + s[9];
    const float jx = (d[1] + d[4]) + (d[5] + d[7]) + d[8];
    const float jy = (d[2] + d[4]) + (d[6] - d[7]) + d[9];
    const float jz = (d[3] + d[5]) + (d[6] - d[8]) - d[9];
    const float pxx = (s[1] + s[4]) + (s[5] + s[7]) + s[8];
    const float pyy = (s[2] + s[4]) + (s[6] + s[7]) + s[9];
    const float pzz = (s[3] + s[5]) + (s[6] + s[8]) + s[9];
    const float pxy = s[4] - s[7];
    const float pxz = s[5] - s[8];
    const float pyz = s[6] - s[9];

    rho = fmaxf(rho, kRhoFloor); // also scrubs a NaN density (IEEE fmax)
    const float inv = __frcp_rn(rho);
    float ux = jx * inv, uy = jy * inv, uz = jz * inv;
    float u2 = ux * ux + uy * uy + uz * uz;
    if (u2 > kMaxSimSpeed * kMaxSimSpeed) {
        const float sc = kMaxSimSpeed * rsqrtf(u2);
        ux *= sc; uy *= sc; uz *= sc;
        u2 = ux * ux + uy * uy + uz * uz;
    }

    float tauEff = tau0;
    if (smagPre > 0.0f) {
        // Non-equilibrium stress: Pi(f) - (rho/3 I + rho u u).
        const float r3 = rho * (1.0f / 3.0f);
        const float rux = rho * ux, ruy = rho * uy;
        const float nxx = pxx - r3 - rux * ux;
        const float nyy = pyy - r3 - ruy * uy;
        const float nzz = pzz - r3 - rho * uz * uz;
        const float nxy = pxy - rux * uy;
        const float nxz = pxz - rux * uz;
        const float nyz = pyz - ruy * uz;
        const float qbar = sqrtf(nxx * nxx + nyy * nyy + nzz * nzz
                                 + 2.0f * (nxy * nxy + nxz * nxz + nyz * nyz));
        tauEff = 0.5f * (tau0 + sqrtf(tau0 * tau0 + smagPre * qbar * inv));
    }
    const float omP = __frcp_rn(tauEff);
    const float tauM = 0.5f + __fdiv_rn(lambda, tauEff - 0.5f);
    const float omM = __frcp_rn(tauM);

    const float base = 1.0f - 1.5f * u2;
    const float r0 = rho * (1.0f / 3.0f);
    const float r1 = rho * (1.0f / 18.0f);
    const float r2 = rho * (1.0f / 36.0f);
    f[0] = f[0] - omP * (f[0] - r0 * base);
#pragma unroll
    for (int p = 1; p <= 9; ++p) {
        const int a = 2 * p - 1;
        const float wr = (p <= 3) ? r1 : r2;
        const float cu = cx(a) * ux + cy(a) * uy + cz(a) * uz;
        const float es = wr * (base + 4.5f * cu * cu);
        const float ea = (3.0f * wr) * cu;
        const float t1 = omP * (0.5f * s[p] - es);
        const float t2 = omM * (0.5f * d[p] - ea);
        f[a] = f[a] - t1 - t2;
        f[a + 1] = f[a + 1] - t1 + t2;
    }
    rhoOut = rho; uxOut = ux; uyOut = uy; uzOut = uz;
}

template <class S, bool WM>
__global__ void __launch_bounds__(kCollideBlockX)
collide_kernel(const typename S::T* __restrict__ src, typename S::T* __restrict__ dst,
               const std::uint8_t* __restrict__ kind, CollideArgs a) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= a.nx) return;
    const int y = blockIdx.y, z = blockIdx.z;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const long long n = a.n;
    const unsigned cell = static_cast<unsigned>(x)
        + static_cast<unsigned>(nx) * (static_cast<unsigned>(y) + static_cast<unsigned>(ny) * z);
    const std::uint8_t k = kind[cell];
    const int flag = k & kFlagMask;

    const int xm = wrap_dec(x, nx), xp = wrap_inc(x, nx);
    // Source coordinate of a pull along velocity component c: x - c.
    const unsigned sx[3] = {static_cast<unsigned>(xp), static_cast<unsigned>(x),
                            static_cast<unsigned>(xm)};
    const unsigned sy[3] = {static_cast<unsigned>(wrap_inc(y, ny)), static_cast<unsigned>(y),
                            static_cast<unsigned>(wrap_dec(y, ny))};
    const unsigned sz[3] = {static_cast<unsigned>(wrap_inc(z, nz)), static_cast<unsigned>(z),
                            static_cast<unsigned>(wrap_dec(z, nz))};
    const unsigned unx = static_cast<unsigned>(nx), uny = static_cast<unsigned>(ny);

    if (flag != kFluid) {
        // ---- boundary cells (reference lbm_core.cu:241-283) ----
        if (flag == kInlet) {
            const float usq = 1.5f * (a.uIn * a.uIn);
#pragma unroll
            for (int q = 0; q < kQ; ++q)
                S::st(dst + q * n, cell, feq_q(q, 1.0f, a.uIn, 0.0f, 0.0f, usq), wgt(q));
            if (a.writeMacro) {
                a.rho[cell] = 1.0f; a.u[cell] = a.uIn; a.v[cell] = 0.0f; a.w[cell] = 0.0f;
            }
        } else if (flag == kOutlet || flag == kOutletEq) {
            const unsigned up = static_cast<unsigned>(xm) + unx * (static_cast<unsigned>(y) + uny * z);
            float g[kQ];
            float r = 0.0f, jx = 0.0f, jy = 0.0f, jz = 0.0f;
#pragma unroll
            for (int q = 0; q < kQ; ++q) {
                g[q] = S::ld(src + q * n, up, wgt(q));
                r += g[q];
                jx += cx(q) * g[q]; jy += cy(q) * g[q]; jz += cz(q) * g[q];
            }
            const float inv = 1.0f / r;
            float ux = jx * inv, uy = jy * inv, uz = jz * inv;
            if (flag == kOutletEq) {
                // Equilibrium outflow: feq(1, u_upstream).
                const float usq = 1.5f * (ux * ux + uy * uy + uz * uz);
#pragma unroll
                for (int q = 0; q < kQ; ++q) g[q] = feq_q(q, 1.0f, ux, uy, uz, usq);
                r = 1.0f;
            }
#pragma unroll
            for (int q = 0; q < kQ; ++q) S::st(dst + q * n, cell, g[q], wgt(q));
            if (a.writeMacro) {
                a.rho[cell] = r; a.u[cell] = ux; a.v[cell] = uy; a.w[cell] = uz;
            }
        } else if (a.writeMacro) {
            a.rho[cell] = 1.0f; a.u[cell] = 0.0f; a.v[cell] = 0.0f; a.w[cell] = 0.0f;
        }
        return;
    }

    float f[kQ];
    if (!(k & kNearWall)) {
        // Bulk cell: every pull streams from the upstream neighbour.
#pragma unroll
        for (int q = 0; q < kQ; ++q) {
            const unsigned src_idx = sx[1 + cx(q)] + unx * (sy[1 + cy(q)] + uny * sz[1 + cz(q)]);
            f[q] = S::ld(src + q * n, src_idx, wgt(q));
        }
    } else {
        // Near-wall cell: the upstream flag picks the (slot, cell) pair.
        float uwx = 0.0f, uwy = 0.0f, uwz = 0.0f;
        bool uwLoaded = false;
        f[0] = S::ld(src, cell, wgt(0));
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
            float fq = S::ld(src + static_cast<long long>(qs) * n, cs, wgt(q));
            if constexpr (WM) {
                // Ladd moving-wall term 6 w_q (c_q . u_w) on solid links.
                if (solid) {
                    if (!uwLoaded) {
                        uwx = __half2float(__ushort_as_half(a.uwx[cell]));
                        uwy = __half2float(__ushort_as_half(a.uwy[cell]));
                        uwz = __half2float(__ushort_as_half(a.uwz[cell]));
                        uwLoaded = true;
                    }
                    fq += 6.0f * wgt(q) * (cx(q) * uwx + cy(q) * uwy + cz(q) * uwz);
                }
            }
            f[q] = fq;
        }
    }

    float rho, ux, uy, uz;
    collide_trt(f, a.tau0, a.lambda, a.smagPre, rho, ux, uy, uz);
#pragma unroll
    for (int q = 0; q < kQ; ++q) S::st(dst + q * n, cell, f[q], wgt(q));
    if (a.writeMacro) {
        a.rho[cell] = rho; a.u[cell] = ux; a.v[cell] = uy; a.w[cell] = uz;
    }
}

/// kind = flag | kNearWall for fluid cells with a solid/slip pull neighbour.
__global__ void classify_kernel(const std::uint8_t* __restrict__ flags,
                                std::uint8_t* __restrict__ kind, int nx, int ny, int nz) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= nx) return;
    const int y = blockIdx.y, z = blockIdx.z;
    const long long cell = x + static_cast<long long>(nx) * (y + static_cast<long long>(ny) * z);
    const std::uint8_t fl = flags[cell] & kFlagMask;
    std::uint8_t out = fl;
    if (fl == kFluid) {
        bool near = false;
#pragma unroll
        for (int q = 1; q < kQ; ++q) {
            int xs = x - cx(q), ys = y - cy(q), zs = z - cz(q);
            xs = xs < 0 ? xs + nx : (xs >= nx ? xs - nx : xs);
            ys = ys < 0 ? ys + ny : (ys >= ny ? ys - ny : ys);
            zs = zs < 0 ? zs + nz : (zs >= nz ? zs - nz : zs);
            const int nf = flags[xs + static_cast<long long>(nx) * (ys + static_cast<long long>(ny) * zs)] & kFlagMask;
            near |= (nf == kSolid) || is_slip_y(nf) || is_slip_z(nf);
        }
        if (near) out |= kNearWall;
    }
    kind[cell] = out;
}

template <class S>
__global__ void init_eq_kernel(typename S::T* __restrict__ f, const std::uint8_t* __restrict__ kind,
                               long long n, float uIn) {
    const long long c = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const float ux = ((kind[c] & kFlagMask) == kSolid) ? 0.0f : uIn;
    const float usq = 1.5f * (ux * ux);
#pragma unroll
    for (int q = 0; q < kQ; ++q) S::st(f + q * n, c, feq_q(q, 1.0f, ux, 0.0f, 0.0f, usq), wgt(q));
}

/// Spanwise speck perturbation (reference lbm_core.cu:130-160): adds
/// 3 w_q c_z w'(x, z) to the fluid cells' populations.
template <class S>
__global__ void speck_kernel(typename S::T* __restrict__ f, const std::uint8_t* __restrict__ kind,
                             int nx, int ny, int nz, float amp, float ph1, float ph2, float phX) {
    const long long c = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    const long long n = static_cast<long long>(nx) * ny * nz;
    if (c >= n) return;
    if ((kind[c] & kFlagMask) != kFluid) return;
    const long long nxny = static_cast<long long>(nx) * ny;
    const int z = static_cast<int>(c / nxny);
    const int x = static_cast<int>((c - z * nxny) % nx);
    const float tz = 6.2831853f * (static_cast<float>(z) + 0.5f) / nz;
    const float tx = 6.2831853f * (static_cast<float>(x) + 0.5f) / nx;
    const float wz = amp * (0.6f * __sinf(3.0f * tz + ph1) + 0.4f * __sinf(7.0f * tz + ph2))
                   * (1.0f + 0.3f * __sinf(2.0f * tx + phX));
#pragma unroll
    for (int q = 1; q < kQ; ++q) {
        if (cz(q) == 0) continue;
        typename S::T* p = f + q * n;
        S::st(p, c, S::ld(p, c, wgt(q)) + 3.0f * wgt(q) * cz(q) * wz, wgt(q));
    }
}

template <class S>
__global__ void init_macro_kernel(typename S::T* __restrict__ f, const std::uint8_t* __restrict__ kind,
                                  long long n, const float* __restrict__ rho,
                                  const float* __restrict__ u, const float* __restrict__ v,
                                  const float* __restrict__ w) {
    const long long c = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const bool solid = (kind[c] & kFlagMask) == kSolid;
    const float r = solid ? 1.0f : rho[c];
    const float ux = solid ? 0.0f : u[c], uy = solid ? 0.0f : v[c], uz = solid ? 0.0f : w[c];
    const float usq = 1.5f * (ux * ux + uy * uy + uz * uz);
#pragma unroll
    for (int q = 0; q < kQ; ++q) S::st(f + q * n, c, feq_q(q, r, ux, uy, uz, usq), wgt(q));
}

/// NaN / runaway watchdog on a prime-strided sample (lbm_core.cu:526-559):
/// verdict base+1 = non-finite populations, base+2 = |u| pinned at the cap.
template <class S>
__global__ void watchdog_kernel(const typename S::T* __restrict__ f, long long n,
                                long long offset, int* flag, int flagBase) {
    const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    const long long c = t * 4093 + offset;
    if (c >= n) return;
    float s = 0.0f, jx = 0.0f, jy = 0.0f, jz = 0.0f;
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
        const float v = S::ld(f + q * n, c, wgt(q));
        s += v; jx += cx(q) * v; jy += cy(q) * v; jz += cz(q) * v;
    }
    if (!isfinite(s)) {
        *flag = flagBase + 1;
    } else {
        const float sp2 = (jx * jx + jy * jy + jz * jz) / fmaxf(s * s, 1e-12f);
        const float cap = 0.95f * kMaxSimSpeed;
        if (sp2 > cap * cap) *flag = flagBase + 2;
    }
}

template <class S>
__global__ void f32_to_store_kernel(const float* __restrict__ in, typename S::T* __restrict__ out,
                                    long long n) {
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n * kQ) return;
    const int q = static_cast<int>(i / n);
    S::st(out, i, in[i], wgt(q));
}

template <class S>
__global__ void store_to_f32_kernel(const typename S::T* __restrict__ in, float* __restrict__ out,
                                    long long n) {
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n * kQ) return;
    const int q = static_cast<int>(i / n);
    out[i] = S::ld(in, i, wgt(q));
}

__global__ void fill_kernel(float* __restrict__ d, long long n, float v) {
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) d[i] = v;
}

inline unsigned blocks_for(long long n) {
    return static_cast<unsigned>((n + kBlock1D - 1) / kBlock1D);
}

inline dim3 plane_grid(const LevelDims& d, int bx) {
    return dim3(static_cast<unsigned>((d.nx + bx - 1) / bx), static_cast<unsigned>(d.ny),
                static_cast<unsigned>(d.nz));
}

template <class S, bool WM>
void collide_dispatch(const void* src, void* dst, const std::uint8_t* kind, LevelDims d,
                      const CollideArgs& args, cudaStream_t st) {
    const int bx = d.nx >= kCollideBlockX ? kCollideBlockX : ((d.nx + 31) / 32) * 32;
    collide_kernel<S, WM><<<plane_grid(d, bx), bx, 0, st>>>(
        static_cast<const typename S::T*>(src), static_cast<typename S::T*>(dst), kind, args);
}

} // namespace

cudaError_t launch_classify(const std::uint8_t* flags, std::uint8_t* kind, LevelDims d,
                            cudaStream_t st) {
    if (!flags || !kind || d.cells() <= 0) return cudaErrorInvalidValue;
    classify_kernel<<<plane_grid(d, 128), 128, 0, st>>>(flags, kind, d.nx, d.ny, d.nz);
    return cudaGetLastError();
}

cudaError_t launch_collide(Storage s, const void* src, void* dst, const std::uint8_t* kind,
                           LevelDims d, const CollideParams& p, float* rho, float* u, float* v,
                           float* w, SlipField slip, cudaStream_t st) {
    if (!src || !dst || !kind || d.cells() <= 0) return cudaErrorInvalidValue;
    CollideArgs a;
    a.nx = d.nx; a.ny = d.ny; a.nz = d.nz; a.n = d.cells();
    a.tau0 = p.tau; a.lambda = p.magicLambda; a.smagPre = p.smagPrefactor; a.uIn = p.uInlet;
    a.writeMacro = (p.writeMacro && rho && u && v && w) ? 1 : 0;
    a.rho = rho; a.u = u; a.v = v; a.w = w;
    a.uwx = slip.uwx; a.uwy = slip.uwy; a.uwz = slip.uwz;
    // FP32 storage runs the reference-order kernel (bit-identical to the
    // reference step without FMA contraction); FP16 storage runs the
    // re-associated pair-sum kernel above.
    if (s == Storage::F32)
        return launch_collide_f32_ref(static_cast<const float*>(src), static_cast<float*>(dst), kind, d, p,
                                      rho, u, v, w, slip, st);
    if (slip.active()) collide_dispatch<StoreF16, true>(src, dst, kind, d, a, st);
    else collide_dispatch<StoreF16, false>(src, dst, kind, d, a, st);
    return cudaGetLastError();
}

cudaError_t launch_init_equilibrium(Storage s, void* f, const std::uint8_t* kind, LevelDims d,
                                    float uInlet, cudaStream_t st) {
    const long long n = d.cells();
    if (!f || !kind || n <= 0) return cudaErrorInvalidValue;
    if (s == Storage::F32)
        return launch_init_eq_f32(static_cast<float*>(f), kind, n, uInlet, st);
    else
        init_eq_kernel<StoreF16><<<blocks_for(n), kBlock1D, 0, st>>>(static_cast<__half*>(f), kind, n, uInlet);
    return cudaGetLastError();
}

cudaError_t launch_speck(Storage s, void* f, const std::uint8_t* kind, LevelDims d, float amplitude,
                         unsigned seed, cudaStream_t st) {
    const long long n = d.cells();
    if (!f || !kind || n <= 0) return cudaErrorInvalidValue;
    // Seeded phases through a Knuth multiplicative hash, as the reference
    // derives them (lbm_core.cu:761-767), so cold starts are reproducible.
    auto phase = [seed](unsigned salt) {
        unsigned h = (seed + salt) * 2654435761u;
        h ^= h >> 16;
        return 6.2831853f * static_cast<float>(h & 0xFFFFFFu) / 16777216.0f;
    };
    if (s == Storage::F32)
        speck_kernel<StoreF32><<<blocks_for(n), kBlock1D, 0, st>>>(
            static_cast<float*>(f), kind, d.nx, d.ny, d.nz, amplitude, phase(1u), phase(2u), phase(3u));
    else
        speck_kernel<StoreF16><<<blocks_for(n), kBlock1D, 0, st>>>(
            static_cast<__half*>(f), kind, d.nx, d.ny, d.nz, amplitude, phase(1u), phase(2u), phase(3u));
    return cudaGetLastError();
}

cudaError_t launch_init_from_macro(Storage s, void* f, const std::uint8_t* kind, LevelDims d,
                                   const float* rho, const float* u, const float* v,
                                   const float* w, cudaStream_t st) {
    const long long n = d.cells();
    if (!f || !kind || n <= 0 || !rho || !u || !v || !w) return cudaErrorInvalidValue;
    if (s == Storage::F32)
        return launch_init_macro_f32(static_cast<float*>(f), kind, n, rho, u, v, w, st);
    else
        init_macro_kernel<StoreF16><<<blocks_for(n), kBlock1D, 0, st>>>(static_cast<__half*>(f), kind, n, rho, u, v, w);
    return cudaGetLastError();
}

cudaError_t launch_watchdog(Storage s, const void* f, LevelDims d, int* flag, long long offset,
                            int flagBase, cudaStream_t st) {
    const long long n = d.cells();
    if (!f || !flag || n <= 0) return cudaErrorInvalidValue;
    const long long off = ((offset % 4093) + 4093) % 4093;
    const long long samples = (n + 4092) / 4093;
    if (s == Storage::F32)
        watchdog_kernel<StoreF32><<<blocks_for(samples), kBlock1D, 0, st>>>(
            static_cast<const float*>(f), n, off, flag, flagBase);
    else
        watchdog_kernel<StoreF16><<<blocks_for(samples), kBlock1D, 0, st>>>(
            static_cast<const __half*>(f), n, off, flag, flagBase);
    return cudaGetLastError();
}

cudaError_t launch_f32_to_store(Storage s, const float* in, void* out, long long cells,
                                cudaStream_t st) {
    if (!in || !out || cells <= 0) return cudaErrorInvalidValue;
    if (s == Storage::F32)
        return cudaMemcpyAsync(out, in, static_cast<size_t>(cells) * kQ * sizeof(float),
                               cudaMemcpyDeviceToDevice, st);
    f32_to_store_kernel<StoreF16><<<blocks_for(cells * kQ), kBlock1D, 0, st>>>(in, static_cast<__half*>(out), cells);
    return cudaGetLastError();
}

cudaError_t launch_store_to_f32(Storage s, const void* in, float* out, long long cells,
                                cudaStream_t st) {
    if (!in || !out || cells <= 0) return cudaErrorInvalidValue;
    if (s == Storage::F32)
        return cudaMemcpyAsync(out, in, static_cast<size_t>(cells) * kQ * sizeof(float),
                               cudaMemcpyDeviceToDevice, st);
    store_to_f32_kernel<StoreF16><<<blocks_for(cells * kQ), kBlock1D, 0, st>>>(static_cast<const __half*>(in), out, cells);
    return cudaGetLastError();
}

cudaError_t launch_fill(float* dst, long long n, float v, cudaStream_t st) {
    if (!dst || n <= 0) return cudaErrorInvalidValue;
    fill_kernel<<<blocks_for(n), kBlock1D, 0, st>>>(dst, n, v);
    return cudaGetLastError();
}

} // namespace fcfd
