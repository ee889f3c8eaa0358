// D3Q19 lattice tables, cell kinds and population storage traits shared by
// every kernel of the GB300 solver step.
//
// The velocity ordering is the frozen Krueger ordering of the reference
// (src/sim/lbm_core.cuh:20-68): snapshots and the C ABI's FP32 import/export
// index populations by q, so the numbering must be identical. The tables are
// packed into 64-bit scalars so that device code can read them as
// compile-time constants: inside `#pragma unroll` loops every c_q, w_q,
// opposite and mirror index folds away, and multiplications by 0/+-1 vanish.
#pragma once

#include <cstdint>
#include <cuda_fp16.h>

namespace fcfd {

constexpr int kQ = 19;

// ---- packed tables -------------------------------------------------------
// Velocity components stored as (c+1) in 2 bits per direction.
constexpr unsigned long long pack2(const int (&v)[kQ]) {
    unsigned long long p = 0;
    for (int q = 0; q < kQ; ++q)
        p |= static_cast<unsigned long long>(v[q] + 1) << (2 * q);
    return p;
}
constexpr int kCxTab[kQ] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0};
constexpr int kCyTab[kQ] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1};
constexpr int kCzTab[kQ] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1};
constexpr unsigned long long kPackCx = pack2(kCxTab);
constexpr unsigned long long kPackCy = pack2(kCyTab);
constexpr unsigned long long kPackCz = pack2(kCzTab);

__host__ __device__ __forceinline__ constexpr int cx(int q) {
    return static_cast<int>((kPackCx >> (2 * q)) & 3ull) - 1;
}
__host__ __device__ __forceinline__ constexpr int cy(int q) {
    return static_cast<int>((kPackCy >> (2 * q)) & 3ull) - 1;
}
__host__ __device__ __forceinline__ constexpr int cz(int q) {
    return static_cast<int>((kPackCz >> (2 * q)) & 3ull) - 1;
}
// Opposite directions are consecutive pairs (1,2)(3,4)...(17,18).
__host__ __device__ __forceinline__ constexpr int opp(int q) {
    return q == 0 ? 0 : ((q & 1) ? q + 1 : q - 1);
}
// Index of the direction with the given components (-1 if none).
constexpr int find_dir(int x, int y, int z) {
    for (int q = 0; q < kQ; ++q)
        if (kCxTab[q] == x && kCyTab[q] == y && kCzTab[q] == z) return q;
    return -1;
}
// Mirror tables derived from the velocity table: y-mirror (cx,-cy,cz) for
// free-slip y walls, z-mirror (cx,cy,-cz) for free-slip z walls. Packed at
// 5 bits per entry into two words (q 0..11 low, 12..18 high).
constexpr unsigned long long pack_mirror(int axis, int half) {
    unsigned long long p = 0;
    for (int q = 12 * half; q < (half ? kQ : 12); ++q) {
        const int m = axis == 1 ? find_dir(kCxTab[q], -kCyTab[q], kCzTab[q])
                                : find_dir(kCxTab[q], kCyTab[q], -kCzTab[q]);
        p |= static_cast<unsigned long long>(m) << (5 * (q - 12 * half));
    }
    return p;
}
constexpr unsigned long long kMirY0 = pack_mirror(1, 0), kMirY1 = pack_mirror(1, 1);
constexpr unsigned long long kMirZ0 = pack_mirror(2, 0), kMirZ1 = pack_mirror(2, 1);
__host__ __device__ __forceinline__ constexpr int mir_y(int q) {
    return q < 12 ? static_cast<int>((kMirY0 >> (5 * q)) & 31ull)
                  : static_cast<int>((kMirY1 >> (5 * (q - 12))) & 31ull);
}
__host__ __device__ __forceinline__ constexpr int mir_z(int q) {
    return q < 12 ? static_cast<int>((kMirZ0 >> (5 * q)) & 31ull)
                  : static_cast<int>((kMirZ1 >> (5 * (q - 12))) & 31ull);
}
// Quadrature weights: 1/3 rest, 1/18 axis, 1/36 diagonal.
__host__ __device__ __forceinline__ constexpr float wgt(int q) {
    return q == 0 ? (1.0f / 3.0f) : (q <= 6 ? (1.0f / 18.0f) : (1.0f / 36.0f));
}

static_assert(mir_y(3) == 4 && mir_y(7) == 13 && mir_y(11) == 18, "mirY");
static_assert(mir_z(5) == 6 && mir_z(9) == 15 && mir_z(17) == 11, "mirZ");

// ---- cell flags and kinds -------------------------------------------------
enum : std::uint8_t {
    kFluid = 0, kSolid = 1, kInlet = 2, kOutlet = 3, kSlipTop = 4,
    kSlipBottom = 5, kSlipFront = 6, kSlipBack = 7, kInterface = 8,
    kOutletEq = 9
};
// Cell kind byte = flag in the low nibble, plus kNearWall (bit 7) on fluid
// cells that have at least one solid or slip pull neighbour. Bulk fluid
// cells (bit clear) stream without reading any neighbour flag.
constexpr std::uint8_t kFlagMask = 0x0F;
constexpr std::uint8_t kNearWall = 0x80;

__host__ __device__ __forceinline__ bool is_slip_y(int f) {
    return f == kSlipTop || f == kSlipBottom;
}
__host__ __device__ __forceinline__ bool is_slip_z(int f) {
    return f == kSlipFront || f == kSlipBack;
}

// Lattice constants of the collision (reference lbm_core.cuh:71-80).
constexpr float kMaxSimSpeed = 0.30f;
constexpr float kRhoFloor = 0.05f;

// ---- division by an invariant integer ----------------------------------------
// Granlund & Montgomery 1994, "Division by invariant integers using
// multiplication": q = (t + ((n - t) >> 1)) >> s with t = mulhi(m, n), exact
// for every 32-bit n.
struct FastDiv {
    unsigned d, m;
    int s;
};
/// Divisor d >= 2: m = floor(2^32 (2^l - d) / d) + 1, s = l - 1, l = ceil(log2 d).
inline FastDiv fast_div(unsigned d) {
    int l = 0;
    while ((1ull << l) < d) ++l;
    const unsigned long long m = ((1ull << 32) * ((1ull << l) - d)) / d + 1;
    return FastDiv{d, static_cast<unsigned>(m), l - 1};
}
__device__ __forceinline__ unsigned fdiv(unsigned n, const FastDiv& f) {
    const unsigned t = __umulhi(n, f.m);
    return (t + ((n - t) >> 1)) >> f.s;
}

// ---- population storage ---------------------------------------------------
// FP32: the population itself. FP16: the deviation f_q - w_q as IEEE half,
// widened to FP32 on load (deviation storage keeps the O(1) weight out of the
// 11-bit mantissa). All arithmetic is FP32 in both cases.
//
// Population loads go through the read-only path with a 256-byte L2
// prefetch hint: a warp's pull along a direction slice reads one or two
// 128-byte lines, and the next warp of the row reads the lines after them
// (measured 0.7 % faster on the FP32 collide launch than plain __ldg).
__device__ __forceinline__ float ld_pf(const float* p) {
    float v;
    asm("ld.global.nc.L2::256B.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ float ld_pf(const __half* p) {
    unsigned short h;
    asm("ld.global.nc.L2::256B.b16 %0, [%1];" : "=h"(h) : "l"(p));
    return __half2float(__ushort_as_half(h));
}
struct StoreF32 {
    using T = float;
    static constexpr int kBytes = 4;
    /// Resident 128-thread blocks per SM the one-cell collide is compiled
    /// for: a cap of 51 registers, of which ptxas allocates 48 (the
    /// fine-level launch measured 1.7 % faster than with the compiler's own
    /// 56).
    static constexpr int kCellMinBlocks = 10;
    /// Resident threads per SM the batched collide is compiled for: 64
    /// registers (the FP16 batched polar measured 15 % slower at 1536
    /// threads, 40 registers).
    static constexpr int kBatchThreads = 1024;
    /// Same for the fine collide with the restriction's child sums fused in:
    /// 64 registers (1.292 ms per launch against 1.325 ms at 56 registers,
    /// which spill 108 B).
    static constexpr int kChildMinBlocks = 8;
    /// Load population q (weight w_q) at element i of its direction slice.
    __device__ __forceinline__ static float ld(const T* __restrict__ p, long long i, float) {
        return ld_pf(p + i);
    }
    __device__ __forceinline__ static void st(T* __restrict__ p, long long i, float v, float) {
        p[i] = v;
    }
    /// The value a load returns after st(v): the storage round trip.
    __device__ __forceinline__ static float rt(float v, float) { return v; }
    /// Load element i of a shared-memory row at shared address `row`.
    __device__ __forceinline__ static float lds(unsigned row, int i, float) {
        float v;
        asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(row + 4u * static_cast<unsigned>(i)));
        return v;
    }
    /// Deviation forms g = f - w_q of ld / st / lds.
    __device__ __forceinline__ static float ld_dev(const T* __restrict__ p, long long i, float w) {
        return ld_pf(p + i) - w;
    }
    __device__ __forceinline__ static void st_dev(T* __restrict__ p, long long i, float g, float w) {
        p[i] = g + w;
    }
    __device__ __forceinline__ static float lds_dev(unsigned row, int i, float w) { return lds(row, i, w) - w; }
};
struct StoreF16 {
    using T = __half;
    static constexpr int kBytes = 2;
    /// A cap of 42 registers, of which ptxas allocates 40: the fine-level
    /// launch measured 7 % faster than at 56.
    static constexpr int kCellMinBlocks = 12;
    static constexpr int kBatchThreads = 1024;
    static constexpr int kChildMinBlocks = 8;
    __device__ __forceinline__ static float ld(const T* __restrict__ p, long long i, float w) {
        return w + ld_pf(p + i);
    }
    __device__ __forceinline__ static void st(T* __restrict__ p, long long i, float v, float w) {
        p[i] = __float2half_rn(v - w);
    }
    __device__ __forceinline__ static float rt(float v, float w) { return w + __half2float(__float2half_rn(v - w)); }
    __device__ __forceinline__ static float lds(unsigned row, int i, float w) {
        return w + lds_dev(row, i, w);
    }
    /// The stored deviation itself: no weight add on load or subtract on store.
    __device__ __forceinline__ static float ld_dev(const T* __restrict__ p, long long i, float) {
        return ld_pf(p + i);
    }
    __device__ __forceinline__ static void st_dev(T* __restrict__ p, long long i, float g, float) {
        p[i] = __float2half_rn(g);
    }
    __device__ __forceinline__ static float lds_dev(unsigned row, int i, float) {
        unsigned short h;
        asm volatile("ld.shared.u16 %0, [%1];" : "=h"(h) : "r"(row + 2u * static_cast<unsigned>(i)));
        return __half2float(__ushort_as_half(h));
    }
};

// ---- helpers ---------------------------------------------------------------
__device__ __forceinline__ int wrap_dec(int v, int n) { return v == 0 ? n - 1 : v - 1; }
__device__ __forceinline__ int wrap_inc(int v, int n) { return v == n - 1 ? 0 : v + 1; }

// Second-order equilibrium, reference formula (lbm_core.cu:65-73).
__device__ __forceinline__ float feq_q(int q, float rho, float ux, float uy, float uz,
                                       float usq) {
    const float cu = 3.0f * (cx(q) * ux + cy(q) * uy + cz(q) * uz);
    return wgt(q) * rho * (1.0f + cu + 0.5f * cu * cu - usq);
}

} // namespace fcfd
