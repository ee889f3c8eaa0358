// Batched stream-collide: one launch steps every tunnel of a batch (or of a
// group of its tunnels: a contiguous range of work items).
//
// The grid walks a flat list of work items -- for each tunnel, its rows
// (y, z) in groups of `ROWS`, whose cells the block's BX threads stride
// through along x (the item decode is paid once per row) -- with a
// block-stride loop, so a grid of a few blocks per SM is persistent across
// all tunnels of unequal size, and a grid of one block per item is an
// ordinary launch. The tunnel table is a __grid_constant__ kernel parameter
// (constant bank): a block finds an item's tunnel by binary search over the
// tunnels' first items and reads that tunnel's parameters from the bank with
// a uniform index. Item decoding is 32-bit. Every cell runs the same per-cell
// update as the single-tunnel kernels (collide_one), so a batch produces the
// same populations, bit for bit, as stepping each tunnel on its own with the
// same collision body. Items of a tunnel whose watchdog latch is set are
// skipped: a diverged tunnel stops where it tripped.
#pragma once

#include "batch_types.h"
#include "collide_common.cuh"

#include <algorithm>

namespace fcfd {
namespace {

// Register cap per storage: S::kBatchThreads resident threads per SM.
template <class S, bool EXACT, int BX, int ROWS>
__global__ void __launch_bounds__(BX, S::kBatchThreads / BX)
batch_collide_kernel(const __grid_constant__ BatchTable P, unsigned itemBase, unsigned nItems, int parity) {
    using T = typename S::T;
    // FP32: the near-wall gather reads the cells' link words (batch step
    // 1.054 -> 0.950 ms on the polar); FP16: the same path at the 64-register
    // cap spilled more and measured 3 % slower, so it reads the neighbours'
    // flags.
    constexpr bool kLinkWall = std::is_same_v<S, StoreF32>;
    const unsigned itemEnd = itemBase + nItems;
    for (unsigned item = itemBase + blockIdx.x; item < itemEnd; item += gridDim.x) {
        int lo = 0, hi = P.ntun - 1;
        while (lo < hi) {  // last tunnel whose first item <= item
            const int mid = (lo + hi + 1) >> 1;
            if (P.begins[mid] <= item) lo = mid;
            else hi = mid - 1;
        }
        if (P.latch && P.latch[lo] != 0) continue;   // a latched tunnel no longer steps
        const BatchTunnelParam& tp = P.t[lo];
        CollideArgs a;
        a.nx = tp.nx; a.ny = tp.ny; a.nz = tp.nz; a.n = tp.n;
        a.tau0 = tp.tau; a.lambda = P.lambda; a.smagPre = P.smagPre; a.uIn = tp.uIn;
        a.writeMacro = 0;
        a.rho = a.u = a.v = a.w = nullptr;
        a.uwx = a.uwy = a.uwz = nullptr;
        a.status = nullptr;
        a.qFrac = nullptr;
        a.links = tp.links;
        a.ffMask = nullptr;
        const T* src = static_cast<const T*>(tp.f[parity]);
        T* dst = static_cast<T*>(tp.f[parity ^ 1]);
        const unsigned ny = static_cast<unsigned>(tp.ny);
        const unsigned rows = ny * static_cast<unsigned>(tp.nz);
        const unsigned row0 = (item - P.begins[lo]) * ROWS;
#pragma unroll
        for (int r = 0; r < ROWS; ++r) {
            const unsigned row = row0 + r;
            if (row >= rows) break;
            const unsigned z = row / ny;
            const int y = static_cast<int>(row - z * ny);
            for (int x = threadIdx.x; x < tp.nx; x += BX)
                collide_one<S, false, EXACT, false, kLinkWall>(src, dst, tp.kind, a, x, y, static_cast<int>(z));
        }
    }
}

template <class S, bool EXACT, int BX, int ROWS>
cudaError_t launch_batch_shape(const BatchTable& tab, unsigned itemBase, unsigned nItems, int parity, int grid,
                               cudaStream_t st) {
    const unsigned g = grid > 0 ? std::min<unsigned>(static_cast<unsigned>(grid), nItems) : nItems;
    if (g == 0) return cudaSuccess;
    batch_collide_kernel<S, EXACT, BX, ROWS><<<g, BX, 0, st>>>(tab, itemBase, nItems, parity);
    return cudaGetLastError();
}

template <class S, bool EXACT, int BX, int ROWS>
int batch_occupancy_shape() {
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, batch_collide_kernel<S, EXACT, BX, ROWS>, BX, 0);
    return b;
}

#define FCFD_BATCH_SHAPES(X) \
    X(64, 1) X(64, 2) X(64, 4) X(128, 1) X(128, 2) X(128, 4) X(256, 1) X(256, 2) X(256, 4)

template <class S, bool EXACT>
cudaError_t launch_batch_impl(const BatchTable& tab, unsigned itemBase, unsigned nItems, int parity, BatchShape sh,
                              cudaStream_t st) {
    if (tab.ntun <= 0 || tab.ntun > kMaxBatchTunnels) return cudaErrorInvalidValue;
#define FCFD_BATCH_CASE(B, R) \
    if (sh.block == B && sh.rows == R) return launch_batch_shape<S, EXACT, B, R>(tab, itemBase, nItems, parity, sh.grid, st);
    FCFD_BATCH_SHAPES(FCFD_BATCH_CASE)
#undef FCFD_BATCH_CASE
    return cudaErrorInvalidValue;
}

template <class S, bool EXACT>
int batch_occupancy_impl(BatchShape sh) {
#define FCFD_BATCH_OCC(B, R) \
    if (sh.block == B && sh.rows == R) return batch_occupancy_shape<S, EXACT, B, R>();
    FCFD_BATCH_SHAPES(FCFD_BATCH_OCC)
#undef FCFD_BATCH_OCC
    return 0;
}

} // namespace
} // namespace fcfd
