// On-device geometry builders: the flag fields, patch box and cell lists the
// solver keys off, built where they are used instead of on the host.
//
// * Airfoil rasterisation (src/geom/voxelizer.cpp:62-153, voxelizeAirfoil):
//   the outline rotated about the quarter chord and scaled to the anchor,
//   one warp per lattice row intersecting the row's cell-centre line with
//   every edge under the half-open rule, the crossings sorted, and the
//   cells between crossing pairs marked in a 2-D mask.
// * Flag field (buildBoundaryFlags, closeTrailingEdgeGaps, stampInterfaceShell,
//   voxelizer.cpp:28-60, 155-183, 223-245): one thread per cell evaluates the
//   base flag (domain faces, all fluid or an input field), the extruded mask
//   over fluid, the single-cell trailing-edge closure judged on the
//   pre-closure field (the +-y neighbours' pre-closure flags are recomputed,
//   so the pass is out of place without a copy) and the interface shell.
// * Patch box (derivePatchBox, voxelizer.cpp:265-301): a min/max reduction
//   of the solid cells' x and y.
// * Cell lists in ascending cell order (ordered stream compaction: per-tile
//   counts, one scan over the tiles, a scatter that re-evaluates the tile):
//   the force-link list, the wall-model cell list of buildWallCellList
//   (src/sim/wall_model.cpp:55-236: pull-solid link mask, vane exclusion,
//   5^3 occupancy-gradient normal, sample cell along the normal), the
//   interface-shell list and the non-solid seed list of a refined level.
//
// Built without FMA contraction: the rasteriser's crossings and the wall
// normals are the host builders' values bit for bit.
#include <cuda_runtime.h>

#include <cstdint>

#include "d3q19.cuh"
#include "kernels.h"

namespace fcfd {
namespace {

constexpr std::uint8_t kFluidB = 0, kSolidB = 1, kInletB = 2, kOutletB = 3, kSlipTopB = 4, kSlipBottomB = 5;
constexpr std::uint8_t kInterfaceB = 8, kOutletEqB = 9;
constexpr int kMaxCrossings = 64;      // per lattice row; more sets the error flag
constexpr int kRowWarps = 4;           // rows per block of the rasteriser
constexpr int kTileThreads = 256;      // compaction tile: 256 threads x 16 cells
constexpr int kTileRun = 16;
constexpr int kTileCells = kTileThreads * kTileRun;

/// Periodic index for any offset (a sample search can step several
/// periods on a thin span); equals the single wrap wherever that is in range.
__device__ __forceinline__ int wrapi(int v, int n) {
    if (static_cast<unsigned>(v) < static_cast<unsigned>(n)) return v;
    const int r = v % n;
    return r < 0 ? r + n : r;
}

// ---- rasteriser -------------------------------------------------------------

__global__ void foil_poly_kernel(const float* __restrict__ xy, int npts, float c, float s, float chord, float ax,
                                 float ay, float* __restrict__ px, float* __restrict__ py) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npts) return;
    // p - (0.25, 0), rotated by the angle whose cosine/sine are c/s, scaled, anchored.
    const float rx = xy[2 * i] - 0.25f, ry = xy[2 * i + 1] - 0.0f;
    const float qx = rx * c - ry * s, qy = rx * s + ry * c;
    px[i] = ax + qx * chord;
    py[i] = ay + qy * chord;
}

__global__ void __launch_bounds__(kRowWarps * 32)
foil_rows_kernel(const float* __restrict__ px, const float* __restrict__ py, int npts, int nx, int ny,
                 std::uint8_t* __restrict__ mask, int* __restrict__ err) {
    __shared__ float cr[kRowWarps][kMaxCrossings];
    __shared__ float srt[kRowWarps][kMaxCrossings];
    __shared__ int span[kRowWarps][kMaxCrossings];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int y = blockIdx.x * kRowWarps + warp;
    if (y >= ny) return;
    std::uint8_t* row = mask + static_cast<long long>(y) * nx;
    int m = 0;
    if (y >= 1 && y <= ny - 2) {
        const float yc = static_cast<float>(y) + 0.5f;
        for (int base = 0; base < npts; base += 32) {
            const int i = base + lane;
            bool hit = false;
            float xc = 0.0f;
            if (i < npts) {
                const int j = i + 1 == npts ? 0 : i + 1;
                const float ya = py[i], yb = py[j];
                if ((ya > yc) != (yb > yc)) {
                    const float t = (yc - ya) / (yb - ya);
                    xc = px[i] + t * (px[j] - px[i]);
                    hit = true;
                }
            }
            const unsigned b = __ballot_sync(0xffffffffu, hit);
            const int slot = m + __popc(b & ((1u << lane) - 1u));
            if (hit && slot < kMaxCrossings) cr[warp][slot] = xc;
            m += __popc(b);
        }
        if (m > kMaxCrossings) {
            if (lane == 0) atomicExch(err, 1);
            m = 0;
        }
    }
    __syncwarp();
    // Rank sort (ties broken by edge order) of the crossings.
    for (int k = lane; k < m; k += 32) {
        const float v = cr[warp][k];
        int r = 0;
        for (int j = 0; j < m; ++j) {
            const float u = cr[warp][j];
            r += (u < v) || (u == v && j < k);
        }
        srt[warp][r] = v;
    }
    __syncwarp();
    const int pairs = m / 2;
    for (int k = lane; k < pairs; k += 32) {
        const int xa = max(1, static_cast<int>(ceilf(srt[warp][2 * k] - 0.5f)));
        const int xb = min(nx - 2, static_cast<int>(floorf(srt[warp][2 * k + 1] - 0.5f)));
        span[warp][2 * k] = xa;
        span[warp][2 * k + 1] = xb;
    }
    __syncwarp();
    for (int x = lane; x < nx; x += 32) {
        bool in = false;
        for (int k = 0; k < pairs; ++k) in |= (x >= span[warp][2 * k]) && (x <= span[warp][2 * k + 1]);
        row[x] = in ? 1 : 0;
    }
}

// ---- flag field -------------------------------------------------------------

struct FlagBuild {
    int nx, ny, nz;
    int base;                          // 0 domain faces, 1 all fluid, 2 input field
    const std::uint8_t* in;            // base 2
    const std::uint8_t* mask;          // nx*ny rasterised foil, or null
    int closeGaps;
    int shell;                         // interface-shell width, 0 for none
};

__device__ __forceinline__ std::uint8_t base_flag(const FlagBuild& b, long long cell, int x, int y) {
    if (b.base == 2) return b.in[cell];
    if (b.base == 1) return kFluidB;
    // buildBoundaryFlags: slip faces, the inlet wins the x = 0 corners, the
    // outlet yields to the slip faces.
    std::uint8_t f = kFluidB;
    if (y == 0) f = kSlipBottomB;
    if (y == b.ny - 1) f = kSlipTopB;
    if (x == 0) f = kInletB;
    else if (x == b.nx - 1 && y != 0 && y != b.ny - 1) f = kOutletB;
    return f;
}

__device__ __forceinline__ std::uint8_t voxel_flag(const FlagBuild& b, long long cell, int x, int y) {
    const std::uint8_t f = base_flag(b, cell, x, y);
    if (b.mask && f == kFluidB && b.mask[static_cast<long long>(y) * b.nx + x]) return kSolidB;
    return f;
}

__global__ void build_flags_kernel(FlagBuild b, std::uint8_t* __restrict__ out, int* __restrict__ closed) {
    const long long n = static_cast<long long>(b.nx) * b.ny * b.nz;
    const long long cell = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    bool close = false;
    if (cell < n) {
        const int x = static_cast<int>(cell % b.nx);
        const long long r = cell / b.nx;
        const int y = static_cast<int>(r % b.ny);
        std::uint8_t f = voxel_flag(b, cell, x, y);
        if (b.closeGaps && y >= 1 && y <= b.ny - 2 && f == kFluidB && voxel_flag(b, cell - b.nx, x, y - 1) == kSolidB
            && voxel_flag(b, cell + b.nx, x, y + 1) == kSolidB) {
            f = kSolidB;
            close = true;
        }
        if (b.shell > 0 && (y < b.shell || y >= b.ny - b.shell || x < b.shell || x >= b.nx - b.shell))
            f = kInterfaceB;
        out[cell] = f;
    }
    const unsigned bal = __ballot_sync(0xffffffffu, close);
    if (bal && (threadIdx.x & 31) == 0) atomicAdd(closed, __popc(bal));
}

// ---- solid bounding box -------------------------------------------------------

__global__ void solid_bbox_kernel(const std::uint8_t* __restrict__ f, int nx, int ny, long long n,
                                  int* __restrict__ box) {
    int x0 = nx, x1 = -1, y0 = ny, y1 = -1;
    for (long long c = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; c < n;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        if (f[c] != kSolidB) continue;
        const int x = static_cast<int>(c % nx);
        const int y = static_cast<int>((c / nx) % ny);
        x0 = min(x0, x); x1 = max(x1, x); y0 = min(y0, y); y1 = max(y1, y);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        x0 = min(x0, __shfl_xor_sync(0xffffffffu, x0, o));
        x1 = max(x1, __shfl_xor_sync(0xffffffffu, x1, o));
        y0 = min(y0, __shfl_xor_sync(0xffffffffu, y0, o));
        y1 = max(y1, __shfl_xor_sync(0xffffffffu, y1, o));
    }
    if ((threadIdx.x & 31) == 0 && x1 >= 0) {
        atomicMin(box + 0, x0); atomicMax(box + 2, x1);
        atomicMin(box + 1, y0); atomicMax(box + 3, y1);
    }
}

// ---- flag classes -------------------------------------------------------------

__global__ void flag_classes_kernel(const std::uint8_t* __restrict__ f, long long n,
                                    unsigned long long* __restrict__ counts) {
    unsigned long long rw = 0, in = 0, un = 0;
    for (long long c = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; c < n;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        const std::uint8_t v = f[c];
        if (v == kFluidB || v == kOutletB || v == kOutletEqB) ++rw;
        else if (v == kInletB) ++in;
        else ++un;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        rw += __shfl_xor_sync(0xffffffffu, rw, o);
        in += __shfl_xor_sync(0xffffffffu, in, o);
        un += __shfl_xor_sync(0xffffffffu, un, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(counts + 0, rw); atomicAdd(counts + 1, in); atomicAdd(counts + 2, un);
    }
}

// ---- ordered compaction --------------------------------------------------------

struct Grid3 {
    int nx, ny, nz;
};

// Force links: fluid cells with a solid neighbour at x + c_q (x, y, z wrapped).
struct ForceLinkPred {
    Grid3 g;
    const std::uint8_t* f;
    std::uint32_t* cells;
    std::uint32_t* masks;
    __device__ std::uint32_t eval(long long c, int x, int y, int z, int* /*stats*/) const {
        if (f[c] != kFluidB) return 0;
        std::uint32_t m = 0;
#pragma unroll
        for (int q = 1; q < kQ; ++q) {
            const int X = wrapi(x + cx(q), g.nx), Y = wrapi(y + cy(q), g.ny), Z = wrapi(z + cz(q), g.nz);
            const unsigned nb = static_cast<unsigned>(X)
                              + static_cast<unsigned>(g.nx) * (static_cast<unsigned>(Y) + static_cast<unsigned>(g.ny) * Z);
            if (f[nb] == kSolidB) m |= 1u << q;
        }
        return m;
    }
    __device__ void emit(long long slot, long long c, int, int, int, std::uint32_t m) const {
        cells[slot] = static_cast<std::uint32_t>(c);
        masks[slot] = m;
    }
};

struct FlagEqPred {     // flag == value (interface-shell list)
    const std::uint8_t* f;
    std::uint8_t value;
    std::uint32_t* cells;
    __device__ std::uint32_t eval(long long c, int, int, int, int*) const { return f[c] == value ? 1u : 0u; }
    __device__ void emit(long long slot, long long c, int, int, int, std::uint32_t) const {
        cells[slot] = static_cast<std::uint32_t>(c);
    }
};

// Interface cells a step reads: the shell cells with a fluid or outlet cell
// among their 18 neighbours (wrapped). The stream-collide reaches no
// further than one cell, so the rest of a 2-cell shell is read by nothing.
struct ShellPulledPred {
    Grid3 g;
    const std::uint8_t* f;
    std::uint32_t* cells;
    __device__ std::uint32_t eval(long long c, int x, int y, int z, int*) const {
        if (f[c] != kInterfaceB) return 0;
#pragma unroll
        for (int q = 1; q < kQ; ++q) {
            const int X = wrapi(x + cx(q), g.nx), Y = wrapi(y + cy(q), g.ny), Z = wrapi(z + cz(q), g.nz);
            const std::uint8_t nf = f[static_cast<unsigned>(X)
                                      + static_cast<unsigned>(g.nx) * (static_cast<unsigned>(Y)
                                                                       + static_cast<unsigned>(g.ny) * Z)];
            if (nf == kFluidB || nf == kOutletB || nf == kOutletEqB) return 1u;
        }
        return 0u;
    }
    __device__ void emit(long long slot, long long c, int, int, int, std::uint32_t) const {
        cells[slot] = static_cast<std::uint32_t>(c);
    }
};

struct FlagNePred {     // flag != value (non-solid seed list)
    const std::uint8_t* f;
    std::uint8_t value;
    std::uint32_t* cells;
    __device__ std::uint32_t eval(long long c, int, int, int, int*) const { return f[c] != value ? 1u : 0u; }
    __device__ void emit(long long slot, long long c, int, int, int, std::uint32_t) const {
        cells[slot] = static_cast<std::uint32_t>(c);
    }
};

// Wall-model cell list (wall_model.cpp:55-236), in two compactions so that
// the 5^3 occupancy gradient runs one candidate per thread instead of on
// the one lane of a warp that meets a wall cell:
//  1. WallCandPred over the lattice: fluid cells with a pull link that is
//     solid in the active field and none that is solid only there (a vane
//     link: the cell is excluded and counted);
//  2. WallListPred over the candidate list: the gradient normal (degenerate
//     ones dropped and counted), the sample cell along it, the entry.
// Both compactions keep order, so the entries are in ascending cell order,
// as the host builder's.
struct WallGeom {
    Grid3 g;
    const std::uint8_t* active;
    const std::uint8_t* clean;
    __device__ __forceinline__ unsigned at(int x, int y, int z) const {
        return static_cast<unsigned>(x) + static_cast<unsigned>(g.nx) * (static_cast<unsigned>(y)
                                                                         + static_cast<unsigned>(g.ny) * z);
    }
    // Solid with x/y out of range = not solid, z periodic.
    __device__ __forceinline__ bool solid(const std::uint8_t* f, int x, int y, int z) const {
        if (x < 0 || x >= g.nx || y < 0 || y >= g.ny) return false;
        return f[at(x, y, wrapi(z, g.nz))] == kSolidB;
    }
    __device__ __forceinline__ void gradient(int x, int y, int z, float& gx, float& gy, float& gz) const {
        gx = gy = gz = 0.0f;
        for (int dz = -2; dz <= 2; ++dz)
            for (int dy = -2; dy <= 2; ++dy)
#pragma unroll
                for (int dx = -2; dx <= 2; ++dx)
                    if (solid(clean, x + dx, y + dy, z + dz)) {
                        gx += static_cast<float>(dx);
                        gy += static_cast<float>(dy);
                        gz += static_cast<float>(dz);
                    }
    }
};

struct WallCandPred {
    WallGeom w;
    std::uint32_t *cells, *masks;
    // 0 = not a candidate; otherwise the link mask. stats (count pass only):
    // [1] vane-excluded.
    __device__ std::uint32_t eval(long long c, int x, int y, int z, int* stats) const {
        if (w.active[c] != kFluidB) return 0;
        std::uint32_t m = 0;
        bool vgOnly = false;
#pragma unroll
        for (int q = 1; q < kQ; ++q) {
            const int sx = x - cx(q), sy = y - cy(q), sz = z - cz(q);
            if (!w.solid(w.active, sx, sy, sz)) continue;
            m |= 1u << q;
            if (!w.solid(w.clean, sx, sy, sz)) vgOnly = true;
        }
        if (m == 0) return 0;
        if (vgOnly) {
            if (stats) atomicAdd(stats + 1, 1);
            return 0;
        }
        return m;
    }
    __device__ void emit(long long slot, long long c, int, int, int, std::uint32_t m) const {
        cells[slot] = static_cast<std::uint32_t>(c);
        masks[slot] = m;
    }
};

struct WallListPred {
    WallGeom w;
    int sampleCells;
    const std::uint32_t *candCell, *candMask;
    std::uint32_t *cell, *sample, *mask;
    float *nX, *nY, *nZ, *ys;

    __device__ __forceinline__ void decode(std::uint32_t c, int& x, int& y, int& z) const {
        const unsigned nxy = static_cast<unsigned>(w.g.nx) * static_cast<unsigned>(w.g.ny);
        z = static_cast<int>(c / nxy);
        const unsigned r = c - static_cast<unsigned>(z) * nxy;
        y = static_cast<int>(r / static_cast<unsigned>(w.g.nx));
        x = static_cast<int>(r - static_cast<unsigned>(y) * static_cast<unsigned>(w.g.nx));
    }
    // i = candidate index. 0 = dropped; otherwise the link mask. stats
    // (count pass only): [0] listed, [2] degenerate normal.
    __device__ std::uint32_t eval(long long i, int, int, int, int* stats) const {
        int x, y, z;
        decode(candCell[i], x, y, z);
        float gx, gy, gz;
        w.gradient(x, y, z, gx, gy, gz);
        const float gm = sqrtf(gx * gx + gy * gy + gz * gz);
        if (gm < 1e-3f) {
            if (stats) atomicAdd(stats + 2, 1);
            return 0;
        }
        if (stats) atomicAdd(stats + 0, 1);
        return candMask[i];
    }
    __device__ void emit(long long slot, long long i, int, int, int, std::uint32_t m) const {
        const std::uint32_t c = candCell[i];
        int x, y, z;
        decode(c, x, y, z);
        float gx, gy, gz;
        w.gradient(x, y, z, gx, gy, gz);
        const float gm = sqrtf(gx * gx + gy * gy + gz * gz);
        const float nx_ = -gx / gm, ny_ = -gy / gm, nz_ = -gz / gm;
        std::uint32_t s = c;
        int sx = x, sy = y, sz = z;
        for (int k = sampleCells; k >= 1; --k) {
            const int tx = x + static_cast<int>(lroundf(nx_ * static_cast<float>(k)));
            const int ty = y + static_cast<int>(lroundf(ny_ * static_cast<float>(k)));
            const int tz = wrapi(z + static_cast<int>(lroundf(nz_ * static_cast<float>(k))), w.g.nz);
            if (tx < 0 || tx >= w.g.nx || ty < 0 || ty >= w.g.ny) continue;
            const std::uint32_t cand = w.at(tx, ty, tz);
            if (w.active[cand] != kFluidB) continue;
            s = cand; sx = tx; sy = ty; sz = tz;
            break;
        }
        int dzw = sz - z;
        if (dzw > w.g.nz / 2) dzw -= w.g.nz;
        if (dzw < -w.g.nz / 2) dzw += w.g.nz;
        const float proj = static_cast<float>(sx - x) * nx_ + static_cast<float>(sy - y) * ny_
                         + static_cast<float>(dzw) * nz_;
        cell[slot] = c;
        sample[slot] = s;
        nX[slot] = nx_; nY[slot] = ny_; nZ[slot] = nz_;
        ys[slot] = 0.5f + fmaxf(proj, 0.0f);
        mask[slot] = m;
    }
};

template <class P>
__device__ __forceinline__ std::uint32_t tile_eval(const P& p, const Grid3& g, long long n, int* stats,
                                                   std::uint32_t (&vals)[kTileRun], int& cnt) {
    const long long first = static_cast<long long>(blockIdx.x) * kTileCells + static_cast<long long>(threadIdx.x) * kTileRun;
    cnt = 0;
    std::uint32_t sel = 0;
    if (first >= n) return 0;
    int x = static_cast<int>(first % g.nx);
    const long long r = first / g.nx;
    int y = static_cast<int>(r % g.ny);
    int z = static_cast<int>(r / g.ny);
#pragma unroll 1
    for (int k = 0; k < kTileRun; ++k) {
        const long long c = first + k;
        if (c >= n) break;
        const std::uint32_t v = p.eval(c, x, y, z, stats);
        vals[k] = v;
        if (v) { sel |= 1u << k; ++cnt; }
        if (++x == g.nx) { x = 0; if (++y == g.ny) { y = 0; ++z; } }
    }
    return sel;
}

template <class P>
__global__ void __launch_bounds__(kTileThreads) compact_count_kernel(P p, Grid3 g, long long n, int* tileCount,
                                                                     int* stats) {
    std::uint32_t vals[kTileRun];
    int cnt;
    tile_eval(p, g, n, stats, vals, cnt);
    __shared__ int warpSum[kTileThreads / 32];
    int v = cnt;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) warpSum[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < kTileThreads / 32; ++w) t += warpSum[w];
        tileCount[blockIdx.x] = t;
    }
}

/// Exclusive scan of the tile counts in place (one block); total -> *total.
__global__ void __launch_bounds__(1024) tile_scan_kernel(int* counts, int tiles, long long* total) {
    __shared__ long long carry;
    __shared__ long long warpSum[32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int base = 0; base < tiles; base += 1024) {
        const int i = base + threadIdx.x;
        const long long v = i < tiles ? counts[i] : 0;
        long long inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane == 31) warpSum[warp] = inc;
        __syncthreads();
        if (warp == 0) {
            const long long w = warpSum[lane];
            long long wi = w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const long long t = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= o) wi += t;
            }
            warpSum[lane] = wi - w;
        }
        __syncthreads();
        const long long excl = carry + warpSum[warp] + inc - v;
        if (i < tiles) counts[i] = static_cast<int>(excl);
        __syncthreads();
        if (threadIdx.x == 1023) carry = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

template <class P>
__global__ void __launch_bounds__(kTileThreads) compact_scatter_kernel(P p, Grid3 g, long long n,
                                                                       const int* tileOffset, long long cap,
                                                                       int* overflow) {
    std::uint32_t vals[kTileRun];
    int cnt;
    const std::uint32_t sel = tile_eval(p, g, n, nullptr, vals, cnt);
    // Exclusive scan of the thread counts across the block.
    __shared__ int warpSum[kTileThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int inc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) warpSum[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const int w = lane < kTileThreads / 32 ? warpSum[lane] : 0;
        int wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < kTileThreads / 32) warpSum[lane] = wi - w;
    }
    __syncthreads();
    long long slot = static_cast<long long>(tileOffset[blockIdx.x]) + warpSum[warp] + inc - cnt;
    if (!sel) return;
    const long long first = static_cast<long long>(blockIdx.x) * kTileCells + static_cast<long long>(threadIdx.x) * kTileRun;
    int x = static_cast<int>(first % g.nx);
    const long long r = first / g.nx;
    int y = static_cast<int>(r % g.ny);
    int z = static_cast<int>(r / g.ny);
#pragma unroll 1
    for (int k = 0; k < kTileRun; ++k) {
        if (sel >> k & 1u) {
            if (slot < cap) p.emit(slot, first + k, x, y, z, vals[k]);
            else atomicExch(overflow, 1);
            ++slot;
        }
        if (++x == g.nx) { x = 0; if (++y == g.ny) { y = 0; ++z; } }
    }
}

/// Stream-ordered scratch of the compaction (tile counts, total, stats).
struct CompactScratch {
    int* tiles = nullptr;
    long long* total = nullptr;
    int* stats = nullptr;
    int* overflow = nullptr;
    void* block = nullptr;
    cudaError_t alloc(long long nTiles, cudaStream_t st) {
        const size_t bytes = static_cast<size_t>(nTiles) * 4 + 64;
        if (auto e = cudaMallocAsync(&block, bytes, st); e != cudaSuccess) return e;
        auto* b = static_cast<char*>(block);
        total = reinterpret_cast<long long*>(b);
        stats = reinterpret_cast<int*>(b + 8);
        overflow = reinterpret_cast<int*>(b + 20);
        tiles = reinterpret_cast<int*>(b + 64);
        return cudaMemsetAsync(block, 0, 64, st);
    }
    void release(cudaStream_t st) {
        if (block) cudaFreeAsync(block, st);
        block = nullptr;
    }
};

long long tiles_for(long long n) { return (n + kTileCells - 1) / kTileCells; }

/// Count pass + scan: *count <- number of selected cells (synchronises).
template <class P>
cudaError_t compact_count(const P& p, Grid3 g, CompactScratch& ws, long long* count, int statsOut[3],
                          cudaStream_t st) {
    const long long n = static_cast<long long>(g.nx) * g.ny * g.nz;
    const long long tiles = tiles_for(n);
    compact_count_kernel<P><<<static_cast<unsigned>(tiles), kTileThreads, 0, st>>>(p, g, n, ws.tiles, ws.stats);
    tile_scan_kernel<<<1, 1024, 0, st>>>(ws.tiles, static_cast<int>(tiles), ws.total);
    if (auto e = cudaGetLastError(); e != cudaSuccess) return e;
    long long tot = 0;
    int sts[3] = {0, 0, 0};
    if (auto e = cudaMemcpyAsync(&tot, ws.total, sizeof(tot), cudaMemcpyDeviceToHost, st); e != cudaSuccess) return e;
    if (auto e = cudaMemcpyAsync(sts, ws.stats, sizeof(sts), cudaMemcpyDeviceToHost, st); e != cudaSuccess) return e;
    if (auto e = cudaStreamSynchronize(st); e != cudaSuccess) return e;
    *count = tot;
    if (statsOut) { statsOut[0] = sts[0]; statsOut[1] = sts[1]; statsOut[2] = sts[2]; }
    return cudaSuccess;
}

template <class P>
cudaError_t compact_scatter(const P& p, Grid3 g, CompactScratch& ws, long long cap, cudaStream_t st) {
    const long long n = static_cast<long long>(g.nx) * g.ny * g.nz;
    const long long tiles = tiles_for(n);
    compact_scatter_kernel<P><<<static_cast<unsigned>(tiles), kTileThreads, 0, st>>>(p, g, n, ws.tiles, cap,
                                                                                     ws.overflow);
    return cudaGetLastError();
}

/// Both passes into caller buffers of capacity cap; *count <- selected cells.
/// When *count > cap nothing is written (a caller sizes its buffers with a
/// first call of capacity 0).
template <class P>
cudaError_t compact_into(const P& p, Grid3 g, long long cap, long long* count, int stats[3], cudaStream_t st) {
    const long long n = static_cast<long long>(g.nx) * g.ny * g.nz;
    if (n <= 0 || n >= (1LL << 31) || !count) return cudaErrorInvalidValue;
    CompactScratch ws;
    cudaError_t e = ws.alloc(tiles_for(n), st);
    if (e == cudaSuccess) e = compact_count(p, g, ws, count, stats, st);
    if (e == cudaSuccess && *count > 0 && *count <= cap) e = compact_scatter(p, g, ws, cap, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    ws.release(st);
    return e;
}

} // namespace

// ---- host entry points ---------------------------------------------------------

bool is_device_pointer(const void* p) {
    cudaPointerAttributes a{};
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice;
}

cudaError_t device_build_flags(LevelDims d, int base, const std::uint8_t* in, const FoilRaster* foil, int closeGaps,
                               int shell, std::uint8_t* out, cudaStream_t st, int* closedOut) {
    const long long n = d.cells();
    if (n <= 0 || !out || (base == 2 && (!in || in == out)) || base < 0 || base > 2) return cudaErrorInvalidValue;
    // Work block: 64 bytes of counters, the nx*ny mask (rounded to 16 bytes),
    // then the outline (2 floats per point) and its lattice x, y (1 + 1).
    const size_t maskBytes = foil ? (static_cast<size_t>(d.nx) * d.ny + 15) / 16 * 16 : 0;
    const size_t polyBytes = foil ? static_cast<size_t>(foil->npts) * 4 * sizeof(float) : 0;
    char* work = nullptr;
    if (auto e = cudaMallocAsync(reinterpret_cast<void**>(&work), 64 + maskBytes + polyBytes, st); e != cudaSuccess)
        return e;
    int* counters = reinterpret_cast<int*>(work);     // [0] closed, [1] rasteriser error
    cudaError_t e = cudaMemsetAsync(work, 0, 64, st);
    std::uint8_t* mask = nullptr;
    if (e == cudaSuccess && foil) {
        if (foil->npts < 3 || d.nx < 3 || d.ny < 3 || !foil->xy) {
            e = cudaErrorInvalidValue;
        } else {
            mask = reinterpret_cast<std::uint8_t*>(work + 64);
            float* dxy = reinterpret_cast<float*>(work + 64 + maskBytes);
            float* px = dxy + 2 * foil->npts;
            e = cudaMemcpyAsync(dxy, foil->xy, static_cast<size_t>(foil->npts) * 2 * sizeof(float),
                                cudaMemcpyHostToDevice, st);
            if (e == cudaSuccess) {
                foil_poly_kernel<<<(foil->npts + 127) / 128, 128, 0, st>>>(dxy, foil->npts, foil->cosA, foil->sinA,
                                                                          foil->chord, foil->anchorX, foil->anchorY,
                                                                          px, px + foil->npts);
                foil_rows_kernel<<<(d.ny + kRowWarps - 1) / kRowWarps, kRowWarps * 32, 0, st>>>(
                    px, px + foil->npts, foil->npts, d.nx, d.ny, mask, counters + 1);
                e = cudaGetLastError();
            }
        }
    }
    if (e == cudaSuccess) {
        FlagBuild b{d.nx, d.ny, d.nz, base, in, mask, closeGaps, shell};
        build_flags_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, st>>>(b, out, counters);
        e = cudaGetLastError();
    }
    int h[2] = {0, 0};
    // A rasterised outline is checked for the row-crossing limit.
    if (e == cudaSuccess && (closedOut || mask)) {
        e = cudaMemcpyAsync(h, counters, sizeof(h), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e == cudaSuccess && h[1]) e = cudaErrorInvalidValue;   // a row with > 64 crossings
        if (e == cudaSuccess && closedOut) *closedOut = h[0];
    }
    cudaFreeAsync(work, st);
    return e;
}

cudaError_t device_solid_bbox(LevelDims d, const std::uint8_t* flags, cudaStream_t st, int box[4]) {
    const long long n = d.cells();
    if (n <= 0 || !flags) return cudaErrorInvalidValue;
    int* dbox = nullptr;
    if (auto e = cudaMallocAsync(reinterpret_cast<void**>(&dbox), 16, st); e != cudaSuccess) return e;
    const int init[4] = {d.nx, d.ny, -1, -1};
    cudaError_t e = cudaMemcpyAsync(dbox, init, 16, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        const long long blocks = (n + 255) / 256;
        solid_bbox_kernel<<<static_cast<unsigned>(blocks < 152 * 16 ? blocks : 152 * 16), 256, 0, st>>>(flags, d.nx,
                                                                                                    d.ny, n, dbox);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(box, dbox, 16, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFreeAsync(dbox, st);
    return e;
}

cudaError_t device_flag_classes(LevelDims d, const std::uint8_t* flags, cudaStream_t st, long long out[3]) {
    const long long n = d.cells();
    if (n <= 0 || !flags) return cudaErrorInvalidValue;
    unsigned long long* dc = nullptr;
    if (auto e = cudaMallocAsync(reinterpret_cast<void**>(&dc), 24, st); e != cudaSuccess) return e;
    cudaError_t e = cudaMemsetAsync(dc, 0, 24, st);
    if (e == cudaSuccess) {
        const long long blocks = (n + 255) / 256;
        flag_classes_kernel<<<static_cast<unsigned>(blocks < 152 * 16 ? blocks : 152 * 16), 256, 0, st>>>(flags, n,
                                                                                                      dc);
        e = cudaGetLastError();
    }
    unsigned long long h[3] = {0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, dc, 24, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFreeAsync(dc, st);
    for (int i = 0; i < 3; ++i) out[i] = static_cast<long long>(h[i]);
    return e;
}

cudaError_t device_force_links(LevelDims d, const std::uint8_t* flags, std::uint32_t* cells, std::uint32_t* masks,
                               long long cap, long long* count, cudaStream_t st) {
    ForceLinkPred p{{d.nx, d.ny, d.nz}, flags, cells, masks};
    return compact_into(p, {d.nx, d.ny, d.nz}, cap, count, nullptr, st);
}

cudaError_t device_cells_where(LevelDims d, const std::uint8_t* flags, std::uint8_t value, bool equal,
                               std::uint32_t* cells, long long cap, long long* count, cudaStream_t st) {
    if (equal) return compact_into(FlagEqPred{flags, value, cells}, {d.nx, d.ny, d.nz}, cap, count, nullptr, st);
    return compact_into(FlagNePred{flags, value, cells}, {d.nx, d.ny, d.nz}, cap, count, nullptr, st);
}

cudaError_t device_shell_pulled(LevelDims d, const std::uint8_t* flags, std::uint32_t* cells, long long cap,
                                long long* count, cudaStream_t st) {
    return compact_into(ShellPulledPred{{d.nx, d.ny, d.nz}, flags, cells}, {d.nx, d.ny, d.nz}, cap, count, nullptr,
                        st);
}

cudaError_t device_wall_list(LevelDims d, const std::uint8_t* active, const std::uint8_t* clean, int sampleCells,
                             const WallListOut& out, long long cap, long long* count, int stats[3],
                             cudaStream_t st) {
    const Grid3 g{d.nx, d.ny, d.nz};
    const long long n = d.cells();
    if (n <= 0 || n >= (1LL << 31) || !count || !active) return cudaErrorInvalidValue;
    const WallGeom w{g, active, clean ? clean : active};
    // 1. Candidates, in cell order.
    WallCandPred p1{w, nullptr, nullptr};
    CompactScratch ws;
    long long nc = 0;
    int s1[3] = {0, 0, 0};
    cudaError_t e = ws.alloc(tiles_for(n), st);
    if (e == cudaSuccess) e = compact_count(p1, g, ws, &nc, s1, st);
    void* cand = nullptr;
    if (e == cudaSuccess && nc > 0) e = cudaMallocAsync(&cand, static_cast<size_t>(nc) * 8, st);
    if (e == cudaSuccess && nc > 0) {
        p1.cells = static_cast<std::uint32_t*>(cand);
        p1.masks = p1.cells + nc;
        e = compact_scatter(p1, g, ws, nc, st);
    }
    ws.release(st);
    // 2. The listed entries among them.
    int s2[3] = {0, 0, 0};
    if (e == cudaSuccess) {
        if (nc > 0) {
            const std::uint32_t* cc = static_cast<const std::uint32_t*>(cand);
            WallListPred p2{w, sampleCells, cc, cc + nc, out.cell, out.sample, out.mask, out.nX, out.nY, out.nZ,
                            out.ys};
            e = compact_into(p2, {static_cast<int>(nc), 1, 1}, cap, count, s2, st);
        } else {
            *count = 0;
        }
    }
    if (cand) cudaFreeAsync(cand, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (stats) { stats[0] = s2[0]; stats[1] = s1[1]; stats[2] = s2[2]; }
    return e;
}

} // namespace fcfd
