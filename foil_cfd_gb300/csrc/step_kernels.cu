// Per-level kernels around the stream-collide: cell-kind and pull-link
// classification, equilibrium / speck / macroscopic initialisation, the NaN
// watchdog, FP32 <-> storage conversion, the AA layout's conversions, and the
// FP16-storage stream-collide (the deviation collision body of
// collide_common.cuh; the FP32 storage collide lives in collide_f32.cu,
// compiled without contraction).
//
// GB300 layout choices (not in the reference): the buffers are unpadded SoA
// and all three axes wrap periodically in the index math, so there is no
// ghost-plane refresh pass; a per-cell kind byte marks the fluid cells that
// touch a wall, so bulk cells stream without reading 18 neighbour flags.
#include "collide_common.cuh"

namespace fcfd {
namespace {

constexpr int kBlock1D = 256;

/// kind = flag | kNearWall for fluid cells with a solid/slip pull neighbour;
/// links (when given): the classes of the 18 pull links (kernels.h).
__global__ void classify_kernel(const std::uint8_t* __restrict__ flags,
                                std::uint8_t* __restrict__ kind, int nx, int ny, int nz,
                                uint2* __restrict__ links) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= nx) return;
    const int y = blockIdx.y, z = blockIdx.z;
    const long long cell = x + static_cast<long long>(nx) * (y + static_cast<long long>(ny) * z);
    const std::uint8_t fl = flags[cell] & kFlagMask;
    std::uint8_t out = fl;
    unsigned long long m = 0;
    if (fl == kFluid) {
#pragma unroll
        for (int q = 1; q < kQ; ++q) {
            int xs = x - cx(q), ys = y - cy(q), zs = z - cz(q);
            xs = xs < 0 ? xs + nx : (xs >= nx ? xs - nx : xs);
            ys = ys < 0 ? ys + ny : (ys >= ny ? ys - ny : ys);
            zs = zs < 0 ? zs + nz : (zs >= nz ? zs - nz : zs);
            const int nf = flags[xs + static_cast<long long>(nx) * (ys + static_cast<long long>(ny) * zs)] & kFlagMask;
            if (nf == kSolid) m |= 1ull << (q - 1);
            if (is_slip_y(nf)) m |= 1ull << (17 + q);
            if (is_slip_z(nf)) m |= 1ull << (35 + q);
        }
        if (m != 0) out |= kNearWall;
    }
    kind[cell] = out;
    if (links) links[cell] = make_uint2(static_cast<unsigned>(m), static_cast<unsigned>(m >> 32));
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

/// AA pattern: exchange the slots of every opposite pair of each cell, in
/// place (A/B state <-> swapped layout). E is the raw element type; opposite
/// directions share a weight, so FP16 deviation bytes move unchanged.
template <class E>
__global__ void aa_pair_swap_kernel(E* __restrict__ f, long long n) {
    const long long c = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= n) return;
#pragma unroll
    for (int q = 1; q < kQ; q += 2) {
        const E a = f[q * n + c], b = f[(q + 1) * n + c];
        f[q * n + c] = b;
        f[(q + 1) * n + c] = a;
    }
}

/// AA pattern: out[x] = in[x + s] of one direction slice, periodic on all
/// three axes (s = +c_q: streamed layout -> A/B state; s = -c_q: back).
template <class E>
__global__ void aa_shift_kernel(const E* __restrict__ in, E* __restrict__ out, int nx, int ny, int nz, int sx,
                                int sy, int sz) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= nx) return;
    const int y = blockIdx.y, z = blockIdx.z;
    int xs = x + sx, ys = y + sy, zs = z + sz;
    xs = xs < 0 ? xs + nx : (xs >= nx ? xs - nx : xs);
    ys = ys < 0 ? ys + ny : (ys >= ny ? ys - ny : ys);
    zs = zs < 0 ? zs + nz : (zs >= nz ? zs - nz : zs);
    out[x + static_cast<long long>(nx) * (y + static_cast<long long>(ny) * z)] =
        in[xs + static_cast<long long>(nx) * (ys + static_cast<long long>(ny) * zs)];
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

} // namespace

cudaError_t launch_classify(const std::uint8_t* flags, std::uint8_t* kind, LevelDims d,
                            cudaStream_t st, uint2* links) {
    if (!flags || !kind || d.cells() <= 0) return cudaErrorInvalidValue;
    classify_kernel<<<plane_grid(d, 128), 128, 0, st>>>(flags, kind, d.nx, d.ny, d.nz, links);
    return cudaGetLastError();
}

cudaError_t launch_collide(Storage s, const void* src, void* dst, const std::uint8_t* kind, LevelDims d,
                           const CollideParams& p, float* rho, float* u, float* v, float* w, SlipField slip,
                           cudaStream_t st) {
    if (!src || !dst || !kind || d.cells() <= 0) return cudaErrorInvalidValue;
    // FP32 storage runs the reference-order kernels (bit-identical to the
    // reference step without FMA contraction); FP16 storage runs the
    // pair-sum collision. The staged kernel is used only when selected.
    if (s == Storage::F32)
        return launch_collide_f32_ref(static_cast<const float*>(src), static_cast<float*>(dst), kind, d, p,
                                      rho, u, v, w, slip, st);
    return launch_collide_impl<StoreF16, false>(src, dst, kind, d, p, rho, u, v, w, slip, st);
}

cudaError_t launch_collide_aa(Storage s, void* f, LevelDims d, const CollideParams& p, int odd, float* rho,
                              float* u, float* v, float* w, cudaStream_t st) {
    if (!f || d.cells() <= 0) return cudaErrorInvalidValue;
    if (s == Storage::F32) return launch_collide_aa_f32(static_cast<float*>(f), d, p, odd, rho, u, v, w, st);
    return launch_collide_aa_impl<StoreF16, false>(f, d, p, odd, rho, u, v, w, st);
}

cudaError_t launch_aa_pair_swap(Storage s, void* f, long long cells, cudaStream_t st) {
    if (!f || cells <= 0) return cudaErrorInvalidValue;
    if (s == Storage::F32)
        aa_pair_swap_kernel<unsigned><<<blocks_for(cells), kBlock1D, 0, st>>>(static_cast<unsigned*>(f), cells);
    else
        aa_pair_swap_kernel<unsigned short><<<blocks_for(cells), kBlock1D, 0, st>>>(
            static_cast<unsigned short*>(f), cells);
    return cudaGetLastError();
}

cudaError_t launch_aa_shift(Storage s, void* f, void* slice, LevelDims d, int toAB, cudaStream_t st) {
    const long long n = d.cells();
    if (!f || !slice || n <= 0) return cudaErrorInvalidValue;
    const size_t eb = s == Storage::F32 ? 4 : 2;
    for (int q = 1; q < kQ; ++q) {
        const int sg = toAB ? 1 : -1;
        char* sl = static_cast<char*>(f) + static_cast<size_t>(q) * static_cast<size_t>(n) * eb;
        if (s == Storage::F32)
            aa_shift_kernel<unsigned><<<plane_grid(d, 128), 128, 0, st>>>(
                reinterpret_cast<const unsigned*>(sl), static_cast<unsigned*>(slice), d.nx, d.ny, d.nz,
                sg * cx(q), sg * cy(q), sg * cz(q));
        else
            aa_shift_kernel<unsigned short><<<plane_grid(d, 128), 128, 0, st>>>(
                reinterpret_cast<const unsigned short*>(sl), static_cast<unsigned short*>(slice), d.nx, d.ny, d.nz,
                sg * cx(q), sg * cy(q), sg * cz(q));
        if (auto e = cudaGetLastError(); e != cudaSuccess) return e;
        if (auto e = cudaMemcpyAsync(sl, slice, static_cast<size_t>(n) * eb, cudaMemcpyDeviceToDevice, st);
            e != cudaSuccess)
            return e;
    }
    return cudaSuccess;
}

cudaError_t launch_collide_child(Storage s, const void* src, void* dst, const std::uint8_t* kind, LevelDims d,
                                 const CollideParams& p, SlipField slip, const ChildFuse& cf, cudaStream_t st) {
    if (!src || !dst || !kind || d.cells() <= 0) return cudaErrorInvalidValue;
    if (s == Storage::F32)
        return launch_collide_child_f32(static_cast<const float*>(src), static_cast<float*>(dst), kind, d, p, slip,
                                        cf, st);
    return launch_collide_child_impl<StoreF16, false>(src, dst, kind, d, p, slip, cf, st);
}

cudaError_t launch_apply_flag_edits(Storage s, void* fA, void* fB, const std::uint8_t* flags,
                                    const std::uint8_t* mask, LevelDims d, cudaStream_t st) {
    if (!fA || !fB || !flags || !mask || d.cells() <= 0) return cudaErrorInvalidValue;
    if (s == Storage::F32)
        return launch_apply_flag_edits_f32(static_cast<float*>(fA), static_cast<float*>(fB), flags, mask, d, st);
    return launch_apply_flag_edits_impl<StoreF16>(fA, fB, flags, mask, d, st);
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
