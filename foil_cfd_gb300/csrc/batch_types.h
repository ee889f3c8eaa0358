// Plain (host + device) types of the batched multi-tunnel step.
#pragma once

#include <cstdint>
#include <vector_types.h>

namespace fcfd {

constexpr int kMaxBatchTunnels = 64;

/// One tunnel of a batch as the batched collide kernel sees it.
struct BatchTunnelParam {
    void* f[2];                  ///< A/B population buffers
    const std::uint8_t* kind;    ///< kind bytes (flag | near-wall bit)
    const uint2* links;          ///< pull-link classes per cell (launch_classify)
    long long n;                 ///< cells
    int nx, ny, nz;
    int xChunks;                 ///< x pieces of a work item (1: whole rows)
    float tau, uIn;
};

/// The whole batch, passed BY VALUE as a kernel parameter (about 4 KB): it
/// lives in the constant bank, so a block's uniform tunnel index reads the
/// tunnel's sizes and relaxation parameters like ordinary kernel parameters.
/// Work items of a launch are the row groups of each tunnel, numbered tunnel
/// after tunnel; begins[t] is tunnel t's first item.
struct BatchTable {
    int ntun;
    float lambda, smagPre;
    /// Per-tunnel watchdog latch in device memory (0 running; nonzero: the
    /// tunnel diverged and its work items are skipped).
    const int* latch;
    unsigned begins[kMaxBatchTunnels];
    BatchTunnelParam t[kMaxBatchTunnels];
};

/// Launch shape of the batched collide: threads per block (striding along
/// x through each row), rows per work item, grid (0: one item per block).
struct BatchShape {
    int block = 128;
    int rows = 1;
    int grid = 0;
};

} // namespace fcfd
