// Host orchestrator of the GB300 solver step and the C ABI of
// include/foilcfd_step.h. It keeps the reference solver's contract
// (src/sim/lbm_solver.cpp): cold start at rest with the spanwise speck, the
// startup viscosity and inlet ramps, stepN's order of work (collide, then m
// fine sub-steps of fill + collide, then restriction, per coarse step; one
// force reduction and one wall-model update per batch), the force EMA with
// its flow-through gate and trailing statistics, and the NaN watchdog every
// 200 steps. Buffers are unpadded (periodic wrap lives in the kernels), so
// there is no ghost-plane refresh anywhere in the loop.
#include "../../include/foilcfd_step.h"
#include "../../include/foilcfd_wallnet.h"
#include "host_geom.h"
#include "kernels.h"
#include "snapshot_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace fcfd {
namespace {

constexpr int kWatchdogPeriod = 200;
constexpr float kSpeckAmplitudeFrac = 1e-3f;
constexpr unsigned kSpeckSeed = 0x5eedu;
constexpr float kForceGateFT = 2.0f;
constexpr float kWarmGateFT = 0.5f;
constexpr long long kCompactSettleSteps = 1000;
constexpr float kDefaultCs = 0.1733f;
constexpr float kDefaultLambda = 3.0f / 16.0f;
constexpr float kMinTau = 0.5005f;
constexpr float kMaxULat = 0.12f;
constexpr float kWallEma = 0.25f;
constexpr int kRestrictBandHost = 2;

void set_err(char* err, size_t len, const std::string& m) {
    if (!err || len == 0) return;
    std::snprintf(err, len, "%s", m.c_str());
}

/// True for a pointer into device memory (a flag field built on the GPU).
bool on_device(const void* p) { return is_device_pointer(p); }

/// Host copy of a flag field given in host or device memory.
void assign_flags(std::vector<std::uint8_t>& v, const std::uint8_t* p, size_t n) {
    v.resize(n);
    if (on_device(p)) cudaMemcpy(v.data(), p, n, cudaMemcpyDeviceToHost);
    else std::memcpy(v.data(), p, n);
}

/// The AA layout's lattices: every cell fluid (periodic on all three axes).
bool aa_lattice(const std::uint8_t* host, size_t n) {
    for (size_t i = 0; i < n; ++i)
        if (host[i] != FCFD_FLAG_FLUID) return false;
    return true;
}
bool aa_flags_ok(const std::uint8_t* p, size_t n) {
    if (!on_device(p)) return aa_lattice(p, n);
    std::vector<std::uint8_t> h;
    assign_flags(h, p, n);
    return aa_lattice(h.data(), n);
}

template <class T>
cudaError_t dalloc(T** p, size_t bytes) {
    return cudaMalloc(reinterpret_cast<void**>(p), bytes == 0 ? 1 : bytes);
}
template <class T>
void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

struct WMLevel {
    bool active = false;
    int count = 0;
    std::uint32_t *dCell = nullptr, *dSample = nullptr, *dMask = nullptr;
    float *dNx = nullptr, *dNy = nullptr, *dNz = nullptr, *dYs = nullptr, *dUTau = nullptr;
    std::uint16_t *dUwx = nullptr, *dUwy = nullptr, *dUwz = nullptr;
    WallStatsDev* dStats = nullptr;
    WallListStats build{};
    SlipField slip() const { return active ? SlipField{dUwx, dUwy, dUwz} : SlipField{}; }
    WallListDev list() const {
        WallListDev l;
        l.cellIdx = dCell; l.sampleIdx = dSample; l.nX = dNx; l.nY = dNy; l.nZ = dNz;
        l.ys = dYs; l.linkMask = dMask; l.uTau = dUTau; l.count = count;
        return l;
    }
    void free() {
        dfree(dCell); dfree(dSample); dfree(dMask); dfree(dNx); dfree(dNy); dfree(dNz);
        dfree(dYs); dfree(dUTau); dfree(dUwx); dfree(dUwy); dfree(dUwz); dfree(dStats);
        *this = WMLevel{};
    }
};

struct Level {
    LevelDims d;
    long long n = 0;
    void* f[2] = {nullptr, nullptr};
    std::uint8_t* flags = nullptr;
    std::uint8_t* kind = nullptr;
    uint2* links = nullptr;   // pull-link classes of the fluid cells (8 B per cell)
    int src = 0;
    std::vector<std::uint8_t> hostFlags, surfaceRef;
    std::uint32_t *dLinkCells = nullptr, *dLinkMasks = nullptr;
    int linkCount = 0;
    double* dPartials = nullptr;
    WMLevel wm;
    // Interpolated bounce-back link field (null when the level has none).
    std::uint8_t* dQFrac = nullptr;
    std::uint32_t* dFFMask = nullptr;
    int qLinks = 0, qFallback = 0;
    // Cell classes of the level for the collide's algorithmic byte count:
    // cells the step reads and writes (fluid, outlets), inlet cells (write
    // only) and cells it leaves untouched (solid, slip, interface; the kind
    // byte is still read).
    long long nReadWrite = 0, nInlet = 0, nUntouched = 0;

    double collideBytes(Storage s) const {
        const double pop = s == Storage::F32 ? 4.0 : 2.0;
        return static_cast<double>(nReadWrite) * (2.0 * 19.0 * pop + 1.0)
             + static_cast<double>(nInlet) * (19.0 * pop + 1.0) + static_cast<double>(nUntouched);
    }

    void free_all() {
        dfree(f[0]); dfree(f[1]); dfree(flags); dfree(kind); dfree(links);
        dfree(dLinkCells); dfree(dLinkMasks); dfree(dPartials);
        dfree(dQFrac); dfree(dFFMask);
        qLinks = qFallback = 0;
        wm.free();
        hostFlags.clear(); surfaceRef.clear();
        linkCount = 0; src = 0; n = 0; d = LevelDims{};
    }
};

struct ForceSample {
    long long step;
    float fx, fy;
};

/// CUDA-event pairs around a class of launches (reused across calls), with
/// the cells and algorithmic bytes each launch covered.
struct TimedLaunches {
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev;
    std::vector<double> cells, bytes;
    size_t used = 0;

    /// Events for the next launch; records the start on `st`.
    cudaEvent_t begin(double c, double b, cudaStream_t st) {
        if (used == ev.size()) {
            cudaEvent_t a, e;
            cudaEventCreate(&a);
            cudaEventCreate(&e);
            ev.emplace_back(a, e);
            cells.push_back(0.0);
            bytes.push_back(0.0);
        }
        cells[used] = c;
        bytes[used] = b;
        cudaEventRecord(ev[used].first, st);
        return ev[used++].second;
    }
    /// Totals since the last call (ms, launches, cells, bytes); resets.
    void take(double& t, long long& n, double& c, double& b) {
        t = c = b = 0.0;
        for (size_t i = 0; i < used; ++i) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, ev[i].first, ev[i].second) == cudaSuccess) t += ms;
            c += cells[i];
            b += bytes[i];
        }
        n = static_cast<long long>(used);
        used = 0;
    }
    void release() {
        for (auto& pr : ev) { cudaEventDestroy(pr.first); cudaEventDestroy(pr.second); }
        ev.clear(); cells.clear(); bytes.clear();
        used = 0;
    }
};

} // namespace
} // namespace fcfd

using namespace fcfd;

struct fcfd_solver {
    // ---- configuration ----
    LevelDims dims;
    fcfd_scaling scaling{};
    cudaStream_t stream = nullptr;
    Storage storage = Storage::F32;
    float lesCs = kDefaultCs;
    float lambda = kDefaultLambda;
    int collideKernel = 0;
    bool initialized = false;
    // AA-pattern layout (fcfd_options.layout): one population array. Between
    // steps it holds the swapped layout (next step odd) or the streamed one
    // (next step even) -- or, after the state was read or written through the
    // API, the A/B state (aaAB), turned back into the swapped layout before
    // the next step. aaSlice is the one-slice scratch of the streamed
    // layout's conversion.
    bool aa = false;
    bool aaAB = false;
    int aaNextOdd = 1;
    void* aaSlice = nullptr;

    // ---- levels ----
    Level coarse;
    Level fine;
    bool fineActive = false;
    // ---- staged FP32 import (fcfd_stage_f32 / fcfd_commit_staged) ----
    struct Staged {
        float* buf = nullptr;   // FP32 SoA of one level
        size_t bytes = 0;
        bool pending = false;
    } staged[3];
    cudaStream_t copyStream = nullptr;
    cudaEvent_t evStaged = nullptr, evCommitted = nullptr;
    int factor = 2;
    fcfd_patch_box box{};
    fcfd_scaling fineScaling{};
    // Nested finer level inside the fine patch (box in fine cells).
    Level finer;
    bool finerActive = false;
    int finerFactor = 2;
    fcfd_patch_box finerBox{};
    std::uint32_t *dShellFiner = nullptr, *dSeedFiner = nullptr;
    int shellCountFiner = 0, seedCountFiner = 0;
    std::uint64_t flagsHashCache = 0;   // FNV-1a of coarse.hostFlags
    bool flagsHashValid = false;
    float* dScratchFiner = nullptr;
    std::uint32_t* dShell = nullptr;
    int shellCount = 0;
    // The fine level's fill covers every interface cell while a finer box
    // reaches its outer shell layer (the finer fill gathers from there).
    bool fineShellFull = false;
    std::uint32_t* dSeed = nullptr;
    int seedCount = 0;
    float* dScratch = nullptr;
    bool forcesFromFine = false;

    // ---- macroscopic fields + readbacks ----
    float *rho = nullptr, *u = nullptr, *v = nullptr, *w = nullptr;
    double* dForce = nullptr;
    double* hForce = nullptr;
    int* dNan = nullptr;
    int* hNan = nullptr;      // [0] watchdog verdict, [1] staged-copy status
    int* dStatus = nullptr;
    cudaEvent_t evT0 = nullptr, evT1 = nullptr, evForce = nullptr, evNan = nullptr;

    // ---- state ----
    long long steps = 0;
    bool rampActive = true, rampEnabled = true;
    long long rampStart = 0;
    long long gateOpenAt = 0;
    float emaWindowFT = 1.0f;
    float emaFx = 0.f, emaFy = 0.f;
    bool emaSeeded = false;
    bool forcePending = false;
    long long stepsAtForceLaunch = 0, stepsAtLastFold = 0;
    double lastForce[3] = {0, 0, 0};
    static constexpr int kRing = 256;
    ForceSample ring[kRing]{};
    int ringHead = 0, ringCount = 0;
    bool timingPending = false;
    int timingN = 0;
    double emaStepMs = 0.0, lastStepMs = 0.0;
    long long sinceWatchdog = 0;
    bool nanPending = false, nanLatched = false;
    int nanKind = 0;
    bool wmEnabled = false;
    bool zSlipWalls = false;
    // Child averages fused into the last fine sub-step: -1 by storage (FP32
    // fused: 3.73 vs 3.86 ms per config-3 step; FP16 separate: 3.02 vs 3.10
    // ms, its issue-bound collide pays more for the fused sums than the
    // separate pass's 1.6 GB re-read costs), 0 separate, 1 fused.
    int fuseChild = -1;
    bool fuseOn() const { return fuseChild < 0 ? storage == Storage::F32 : fuseChild != 0; }
    int wallMethod = 0;                 // FCFD_UTAU_* solve of the wall updates
    std::uint16_t* dNetW = nullptr;     // learned seed: solver-owned BF16 weights
    wallnet::NetDev netView{};

    // ---- diagnostics ----
    long long launches = 0;
    bool collideTiming = false;
    TimedLaunches colT;   // plain stream-collide launches (both levels)
    TimedLaunches fuseT;  // fine collides with the child averages fused in
    cudaEvent_t tmr0 = nullptr, tmr1 = nullptr;

    // ------------------------------------------------------------------
    float flowThroughSteps() const {
        return static_cast<float>(dims.nx) / std::max(scaling.u_lat, 1e-6f);
    }
    float effTau() const {
        return (rampActive && rampEnabled) ? fcfd_ramped_tau(&scaling, steps - rampStart, dims.nx)
                                           : scaling.tau;
    }
    float effU() const {
        return (rampActive && rampEnabled) ? fcfd_ramped_u(&scaling, steps - rampStart, dims.nx)
                                           : scaling.u_lat;
    }
    float smagPre() const {
        return lesCs > 0.0f ? 18.0f * 1.41421356f * lesCs * lesCs : 0.0f;
    }
    static float fineTau(float tc, int m) { return static_cast<float>(m) * (tc - 0.5f) + 0.5f; }

    static bool eventDone(cudaEvent_t e) {
        const cudaError_t st = cudaEventQuery(e);
        if (st == cudaErrorNotReady) (void)cudaGetLastError();
        return st == cudaSuccess;
    }

    void pollAsync() {
        if (timingPending && eventDone(evT1)) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, evT0, evT1) == cudaSuccess && timingN > 0) {
                lastStepMs = static_cast<double>(ms) / timingN;
                emaStepMs = emaStepMs > 0.0 ? emaStepMs + 0.25 * (lastStepMs - emaStepMs) : lastStepMs;
            }
            timingPending = false;
        }
        if (forcePending && eventDone(evForce)) {
            for (int i = 0; i < 3; ++i) lastForce[i] = hForce[i];
            const float fx = static_cast<float>(hForce[0]), fy = static_cast<float>(hForce[1]);
            const float window = std::max(1.0f, emaWindowFT * flowThroughSteps());
            const float dS = static_cast<float>(stepsAtForceLaunch - stepsAtLastFold);
            const float alpha = 1.0f - std::exp(-dS / window);
            if (!emaSeeded) { emaFx = fx; emaFy = fy; emaSeeded = true; }
            else { emaFx += alpha * (fx - emaFx); emaFy += alpha * (fy - emaFy); }
            ring[ringHead] = {stepsAtForceLaunch, fx, fy};
            ringHead = (ringHead + 1) % kRing;
            if (ringCount < kRing) ++ringCount;
            stepsAtLastFold = stepsAtForceLaunch;
            forcePending = false;
        }
        if (nanPending && eventDone(evNan)) {
            if (hNan[0] != 0) { nanLatched = true; nanKind = hNan[0]; }
            if (hNan[1] != 0) { nanLatched = true; nanKind = 9; }
            nanPending = false;
        }
    }

    // ---- level setup ----
    cudaError_t allocLevel(Level& L, LevelDims d) {
        L.d = d;
        L.n = d.cells();
        const size_t fb = static_cast<size_t>(L.n) * 19 * (storage == Storage::F32 ? 4 : 2);
        for (int i = 0; i < (aa ? 1 : 2); ++i)
            if (auto e = cudaMalloc(&L.f[i], fb); e != cudaSuccess) return e;
        if (auto e = dalloc(&L.flags, static_cast<size_t>(L.n)); e != cudaSuccess) return e;
        // Kind bytes are fetched in 16-byte-aligned row copies that may run
        // up to 31 bytes past the last row: pad the allocation.
        if (auto e = dalloc(&L.kind, static_cast<size_t>(L.n) + 64); e != cudaSuccess) return e;
        if (auto e = dalloc(&L.links, static_cast<size_t>(L.n) * sizeof(uint2)); e != cudaSuccess) return e;
        return cudaSuccess;
    }

    /// Flags of a level from host or device memory: the device copy, the
    /// host copy (edit diffs), the cell classes, the kind bytes and the
    /// force-link list, the last two built on the device.
    cudaError_t uploadLevelFlags(Level& L, const std::uint8_t* flags) {
        if (&L == &coarse) flagsHashValid = false;
        L.hostFlags.resize(static_cast<size_t>(L.n));
        const size_t nb = static_cast<size_t>(L.n);
        if (on_device(flags)) {
            if (auto e = cudaMemcpyAsync(L.flags, flags, nb, cudaMemcpyDeviceToDevice, stream); e != cudaSuccess)
                return e;
            if (auto e = cudaMemcpyAsync(L.hostFlags.data(), flags, nb, cudaMemcpyDeviceToHost, stream);
                e != cudaSuccess)
                return e;
        } else {
            std::memcpy(L.hostFlags.data(), flags, nb);
            if (auto e = cudaMemcpyAsync(L.flags, flags, nb, cudaMemcpyHostToDevice, stream); e != cudaSuccess)
                return e;
        }
        long long cls[3];
        launches += 1;
        if (auto e = device_flag_classes(L.d, L.flags, stream, cls); e != cudaSuccess) return e;
        L.nReadWrite = cls[0]; L.nInlet = cls[1]; L.nUntouched = cls[2];
        ++launches;
        if (auto e = launch_classify(L.flags, L.kind, L.d, stream, L.links); e != cudaSuccess) return e;
        // Compact force-link list of this level (ascending cell order).
        dfree(L.dLinkCells); dfree(L.dLinkMasks); dfree(L.dPartials);
        long long links = 0;
        launches += 2;
        if (auto e = device_force_links(L.d, L.flags, nullptr, nullptr, 0, &links, stream); e != cudaSuccess) return e;
        L.linkCount = static_cast<int>(links);
        if (auto e = dalloc(&L.dLinkCells, static_cast<size_t>(links) * 4); e != cudaSuccess) return e;
        if (auto e = dalloc(&L.dLinkMasks, static_cast<size_t>(links) * 4); e != cudaSuccess) return e;
        if (auto e = dalloc(&L.dPartials, static_cast<size_t>(force_blocks(L.linkCount)) * 3 * sizeof(double));
            e != cudaSuccess)
            return e;
        if (links > 0) {
            launches += 3;
            long long again = 0;
            if (auto e = device_force_links(L.d, L.flags, L.dLinkCells, L.dLinkMasks, links, &again, stream);
                e != cudaSuccess)
                return e;
        }
        return cudaStreamSynchronize(stream);
    }

    /// Fill targets of a refined level: the interface cells its stream-collide
    /// reads (a fluid or outlet cell among their 18 neighbours). The
    /// reference fills every interface cell, but the collide reaches one
    /// cell, so the outer layer of the 2-cell shell is read by no step and
    /// every population a step computes is the same. With `full` (the fine
    /// level while a finer level nests in it, whose fill may gather from
    /// the fine shell) every interface cell.
    cudaError_t shellList(const Level& L, bool full, std::uint32_t** out, int* count) {
        if (full) return cellList(L, FCFD_FLAG_INTERFACE, true, out, count);
        dfree(*out);
        *count = 0;
        long long c = 0;
        launches += 2;
        if (auto e = device_shell_pulled(L.d, L.flags, nullptr, 0, &c, stream); e != cudaSuccess) return e;
        if (auto e = dalloc(out, static_cast<size_t>(c) * 4); e != cudaSuccess) return e;
        if (c > 0) {
            launches += 3;
            long long again = 0;
            if (auto e = device_shell_pulled(L.d, L.flags, *out, c, &again, stream); e != cudaSuccess) return e;
        }
        *count = static_cast<int>(c);
        return cudaSuccess;
    }

    /// Ascending list of the level's cells whose flag equals (or, with
    /// equal false, differs from) `value`, into a fresh device array.
    cudaError_t cellList(const Level& L, std::uint8_t value, bool equal, std::uint32_t** out, int* count) {
        dfree(*out);
        *count = 0;
        long long c = 0;
        launches += 2;
        if (auto e = device_cells_where(L.d, L.flags, value, equal, nullptr, 0, &c, stream); e != cudaSuccess)
            return e;
        if (auto e = dalloc(out, static_cast<size_t>(c) * 4); e != cudaSuccess) return e;
        if (c > 0) {
            launches += 3;
            long long again = 0;
            if (auto e = device_cells_where(L.d, L.flags, value, equal, *out, c, &again, stream); e != cudaSuccess)
                return e;
        }
        *count = static_cast<int>(c);
        return cudaSuccess;
    }

    cudaError_t buildWM(Level& L, int sampleCells) {
        L.wm.free();
        if (!wmEnabled || L.hostFlags.size() != static_cast<size_t>(L.n)) return cudaSuccess;
        const size_t cells = static_cast<size_t>(L.n);
        // Normals key off the clean surface reference when one is set.
        std::uint8_t* dClean = nullptr;
        cudaError_t e = cudaSuccess;
        if (L.surfaceRef.size() == cells) {
            e = dalloc(&dClean, cells);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(dClean, L.surfaceRef.data(), cells, cudaMemcpyHostToDevice, stream);
        }
        long long n = 0;
        int st[3] = {0, 0, 0};
        WallListOut none;
        launches += 2;
        if (e == cudaSuccess)
            e = device_wall_list(L.d, L.flags, dClean ? dClean : L.flags, sampleCells, none, 0, &n, st, stream);
        L.wm.build.listed = st[0]; L.wm.build.excludedVG = st[1]; L.wm.build.degenerate = st[2];
        if (e != cudaSuccess || n == 0) {
            dfree(dClean);
            return e;
        }
        WMLevel& m = L.wm;
        auto A = [&](auto** p, size_t b) { if (e == cudaSuccess) e = dalloc(p, b); };
        const size_t nn = static_cast<size_t>(n);
        A(&m.dCell, nn * 4); A(&m.dSample, nn * 4); A(&m.dMask, nn * 4);
        A(&m.dNx, nn * 4); A(&m.dNy, nn * 4); A(&m.dNz, nn * 4); A(&m.dYs, nn * 4); A(&m.dUTau, nn * 4);
        A(&m.dUwx, cells * 2); A(&m.dUwy, cells * 2); A(&m.dUwz, cells * 2);
        A(&m.dStats, sizeof(WallStatsDev));
        if (e == cudaSuccess) {
            WallListOut o;
            o.cell = m.dCell; o.sample = m.dSample; o.mask = m.dMask;
            o.nX = m.dNx; o.nY = m.dNy; o.nZ = m.dNz; o.ys = m.dYs;
            long long again = 0;
            launches += 3;
            e = device_wall_list(L.d, L.flags, dClean ? dClean : L.flags, sampleCells, o, n, &again, st, stream);
        }
        if (e == cudaSuccess) e = cudaMemsetAsync(m.dUTau, 0, nn * 4, stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(m.dUwx, 0, cells * 2, stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(m.dUwy, 0, cells * 2, stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(m.dUwz, 0, cells * 2, stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(m.dStats, 0, sizeof(WallStatsDev), stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        dfree(dClean);
        if (e != cudaSuccess) { m.free(); return e; }
        m.count = static_cast<int>(n);
        m.active = true;
        return cudaSuccess;
    }

    void resetWMState() {
        for (Level* L : {&coarse, &fine}) {
            if (!L->wm.active) continue;
            cudaMemsetAsync(L->wm.dUTau, 0, static_cast<size_t>(L->wm.count) * 4, stream);
            cudaMemsetAsync(L->wm.dUwx, 0, static_cast<size_t>(L->n) * 2, stream);
            cudaMemsetAsync(L->wm.dUwy, 0, static_cast<size_t>(L->n) * 2, stream);
            cudaMemsetAsync(L->wm.dUwz, 0, static_cast<size_t>(L->n) * 2, stream);
        }
    }

    RefineGeom geom() const {
        RefineGeom g;
        g.coarse = coarse.d; g.fine = fine.d;
        g.boxX0 = box.x0; g.boxY0 = box.y0; g.boxX1 = box.x1; g.boxY1 = box.y1;
        g.factor = factor;
        return g;
    }

    RefineGeom geomFiner() const {
        RefineGeom g;
        g.coarse = fine.d; g.fine = finer.d;
        g.boxX0 = finerBox.x0; g.boxY0 = finerBox.y0; g.boxX1 = finerBox.x1; g.boxY1 = finerBox.y1;
        g.factor = finerFactor;
        return g;
    }

    /// Both finer buffers from the fine level's current state (full-volume
    /// fill, lbm_solver.cpp:523-545).
    cudaError_t seedFiner() {
        if (!finerActive) return cudaSuccess;
        const float tf = fineTau(effTau(), factor), tr = fineTau(tf, finerFactor);
        for (int i = 0; i < 2; ++i) {
            ++launches;
            if (auto e = launch_fill_c2f(storage, fine.f[fine.src], fine.f[fine.src], fine.kind, finer.f[i],
                                         dSeedFiner, seedCountFiner, geomFiner(), 0.0f,
                                         tr / (static_cast<float>(finerFactor) * tf), stream);
                e != cudaSuccess)
                return e;
        }
        return cudaSuccess;
    }

    void freeFiner() {
        finer.free_all();
        dfree(dShellFiner); dfree(dSeedFiner); dfree(dScratchFiner);
        shellCountFiner = seedCountFiner = 0;
        finerActive = false;
    }

    cudaError_t seedFine() {
        if (!fineActive) return cudaSuccess;
        const float tc = effTau(), tf = fineTau(tc, factor);
        for (int i = 0; i < 2; ++i) {
            ++launches;
            if (auto e = launch_fill_c2f(storage, coarse.f[coarse.src], coarse.f[coarse.src], coarse.kind,
                                         fine.f[i], dSeed, seedCount, geom(), 0.0f,
                                         tf / (static_cast<float>(factor) * tc), stream);
                e != cudaSuccess)
                return e;
        }
        return cudaSuccess;
    }

    /// Forces come from the fine level when every coarse solid cell lies in
    /// the patch's restriction region (the reference's surface-cache test).
    void updateForcesFromFine() {
        forcesFromFine = false;
        if (!fineActive) return;
        const int x0 = box.x0 + kRestrictBandHost, x1 = box.x1 - kRestrictBandHost;
        const int y0 = box.y0 + kRestrictBandHost, y1 = box.y1 - kRestrictBandHost;
        int b[4];
        ++launches;
        if (device_solid_bbox(coarse.d, coarse.flags, stream, b) != cudaSuccess) return;
        forcesFromFine = b[2] < 0 || (b[0] >= x0 && b[2] < x1 && b[1] >= y0 && b[3] < y1);
    }

    void freeFine() {
        freeFiner();  // the finer level nests in the fine one
        fine.free_all();
        dfree(dShell); dfree(dSeed); dfree(dScratch);
        shellCount = seedCount = 0;
        fineShellFull = false;
        fineActive = false;
        forcesFromFine = false;
    }

    void freeStaged() {
        if (copyStream) cudaStreamSynchronize(copyStream);
        for (Staged& st : staged) {
            dfree(st.buf);
            st = Staged{};
        }
        for (cudaEvent_t* e : {&evStaged, &evCommitted})
            if (*e) { cudaEventDestroy(*e); *e = nullptr; }
        if (copyStream) { cudaStreamDestroy(copyStream); copyStream = nullptr; }
    }

    Level* levelAt(int level) {
        if (level == 0) return &coarse;
        if (level == 1 && fineActive) return &fine;
        if (level == 2 && finerActive) return &finer;
        return nullptr;
    }

    /// Queue the host -> device copy of one level's FP32 SoA state into its
    /// staging buffer on the copy stream.
    cudaError_t stageF32(int level, const float* host, size_t count) {
        Level* L = levelAt(level);
        if (!L || !host || count != static_cast<size_t>(L->n) * 19) return cudaErrorInvalidValue;
        if (!copyStream) {
            if (auto e = cudaStreamCreateWithFlags(&copyStream, cudaStreamNonBlocking); e != cudaSuccess) return e;
            if (auto e = cudaEventCreateWithFlags(&evStaged, cudaEventDisableTiming); e != cudaSuccess) return e;
            if (auto e = cudaEventCreateWithFlags(&evCommitted, cudaEventDisableTiming); e != cudaSuccess) return e;
        }
        Staged& st = staged[level];
        const size_t bytes = count * sizeof(float);
        if (st.bytes != bytes) {
            cudaStreamSynchronize(copyStream);
            dfree(st.buf);
            st.bytes = 0;
            if (auto e = cudaMalloc(&st.buf, bytes); e != cudaSuccess) return e;
            st.bytes = bytes;
        }
        // A commit still reading the staging buffers finishes first.
        if (auto e = cudaStreamWaitEvent(copyStream, evCommitted, 0); e != cudaSuccess) return e;
        if (auto e = cudaMemcpyAsync(st.buf, host, bytes, cudaMemcpyHostToDevice, copyStream); e != cudaSuccess)
            return e;
        if (auto e = cudaEventRecord(evStaged, copyStream); e != cudaSuccess) return e;
        st.pending = true;
        return cudaSuccess;
    }

    /// The staged levels become the current state, ordered on the solver
    /// stream after their copies.
    cudaError_t commitStaged() {
        bool any = false, coarseDone = false;
        for (const Staged& st : staged) any |= st.pending;
        if (!any) return cudaErrorNotReady;
        if (auto e = cudaStreamWaitEvent(stream, evStaged, 0); e != cudaSuccess) return e;
        for (int level = 0; level < 3; ++level) {
            Staged& st = staged[level];
            if (!st.pending) continue;
            st.pending = false;
            Level* L = levelAt(level);
            if (!L || st.bytes != static_cast<size_t>(L->n) * 19 * sizeof(float)) return cudaErrorInvalidValue;
            if (level == 0) aaAB = aa;
            cudaError_t e;
            if (storage == Storage::F32) {
                e = cudaMemcpyAsync(L->f[L->src], st.buf, st.bytes, cudaMemcpyDeviceToDevice, stream);
            } else {
                ++launches;
                e = launch_f32_to_store(storage, st.buf, L->f[L->src], L->n, stream);
            }
            if (e != cudaSuccess) return e;
            coarseDone |= level == 0;
        }
        if (auto e = cudaEventRecord(evCommitted, stream); e != cudaSuccess) return e;
        if (coarseDone) notifyRestored(true);
        return cudaSuccess;
    }

    void freeAll() {
        if (stream) cudaStreamSynchronize(stream);
        freeStaged();
        freeFine();
        coarse.free_all();
        dfree(aaSlice);
        dfree(rho); dfree(u); dfree(v); dfree(w); dfree(dForce); dfree(dNan); dfree(dStatus);
        dfree(dNetW);
        wallMethod = 0;
        netView = wallnet::NetDev{};
        if (hForce) { cudaFreeHost(hForce); hForce = nullptr; }
        if (hNan) { cudaFreeHost(hNan); hNan = nullptr; }
        for (cudaEvent_t* e : {&evT0, &evT1, &evForce, &evNan})
            if (*e) { cudaEventDestroy(*e); *e = nullptr; }
        colT.release();
        fuseT.release();
        for (cudaEvent_t* e : {&tmr0, &tmr1})
            if (*e) { cudaEventDestroy(*e); *e = nullptr; }
        timingPending = forcePending = nanPending = false;
        emaStepMs = lastStepMs = 0.0;
        initialized = false;
    }

    // ---- stepping ----
    cudaError_t collide(Level& L, const CollideParams& p, float* r, float* uu, float* vv, float* ww) {
        // The AA kernels read no kind byte: 2 x 19 populations per cell.
        const double bytes = aa ? 38.0 * (storage == Storage::F32 ? 4.0 : 2.0) * static_cast<double>(L.n)
                                : L.collideBytes(storage);
        cudaEvent_t e2 = collideTiming ? colT.begin(static_cast<double>(L.n), bytes, stream) : nullptr;
        ++launches;
        CollideParams lp = p;
        lp.qFrac = L.dQFrac;
        lp.ffMask = L.dFFMask;
        lp.links = L.links;
        cudaError_t e;
        if (aa) {
            e = launch_collide_aa(storage, L.f[0], L.d, lp, aaNextOdd, r, uu, vv, ww, stream);
            aaNextOdd ^= 1;
        } else {
            e = launch_collide(storage, L.f[L.src], L.f[1 - L.src], L.kind, L.d, lp, r, uu, vv, ww, L.wm.slip(),
                               stream);
        }
        if (e2) cudaEventRecord(e2, stream);
        return e;
    }

    /// Fine collide of the last sub-step with the restriction's child
    /// averages fused in (factor 2); timed with the collide launches, its
    /// algorithmic bytes include the scratch records it writes.
    cudaError_t collideChild(Level& L, const CollideParams& p, const RefineGeom& g, float* scratch) {
        ChildFuse cf;
        cf.scratch = scratch;
        cf.boxX0 = g.boxX0;
        cf.boxY0 = g.boxY0;
        restrict_sub_box(g, cf.rx0, cf.ry0, cf.rw, cf.rh);
        cudaEvent_t e2 = collideTiming
                             ? fuseT.begin(static_cast<double>(L.n),
                                           L.collideBytes(storage) + (storage == Storage::F32 ? 96.0 : 64.0)
                                                   * static_cast<double>(cf.rw) * cf.rh * g.coarse.nz,
                                           stream)
                             : nullptr;
        ++launches;
        CollideParams lp = p;
        lp.qFrac = L.dQFrac;
        lp.ffMask = L.dFFMask;
        lp.links = L.links;
        const cudaError_t e = launch_collide_child(storage, L.f[L.src], L.f[1 - L.src], L.kind, L.d, lp,
                                                   L.wm.slip(), cf, stream);
        if (e2) cudaEventRecord(e2, stream);
        return e;
    }

    cudaError_t forceReduce(Level& L) {
        launches += 2;
        return launch_force(storage, L.f[L.src], L.n, L.dLinkCells, L.dLinkMasks, L.linkCount,
                            L.wm.slip(), L.dPartials, dForce, stream);
    }

    cudaError_t wallUpdate(Level& L, float nu) {
        if (!L.wm.active) return cudaSuccess;
        ++launches;
        return launch_wall_update(storage, L.f[L.src], L.n, L.wm.list(), L.wm.dUwx, L.wm.dUwy,
                                  L.wm.dUwz, nu, 1e-3f * scaling.u_lat, kWallEma, L.wm.dStats, stream,
                                  wallMethod, &netView);
    }

    /// AA layout: leave the A/B state (post-collision f*_q(x) in slot q of
    /// cell x) in the population array for a reader; a no-op otherwise.
    cudaError_t aaToAB() {
        if (!aa || aaAB) return cudaSuccess;
        launches += aaNextOdd ? 1 : 18;
        const cudaError_t e = aaNextOdd ? launch_aa_pair_swap(storage, coarse.f[0], coarse.n, stream)
                                        : launch_aa_shift(storage, coarse.f[0], aaSlice, coarse.d, 1, stream);
        if (e == cudaSuccess) aaAB = true;
        return e;
    }

    int stepN(int n) {
        if (!initialized) return cudaErrorNotReady;
        if (n <= 0) return cudaSuccess;
        pollAsync();
        if (nanLatched) return cudaSuccess;
        if (aa && aaAB) {
            ++launches;
            if (auto e = launch_aa_pair_swap(storage, coarse.f[0], coarse.n, stream); e != cudaSuccess) return e;
            aaAB = false;
            aaNextOdd = 1;
        }
        const bool timeIt = !timingPending;
        if (timeIt) cudaEventRecord(evT0, stream);
        for (int i = 0; i < n; ++i) {
            CollideParams p;
            p.tau = effTau();
            p.magicLambda = lambda;
            p.smagPrefactor = smagPre();
            p.uInlet = effU();
            p.writeMacro = (i == n - 1) ? 1 : 0;
            p.status = dStatus;
            p.kernel = collideKernel;
            if (auto e = collide(coarse, p, rho, u, v, w); e != cudaSuccess) return e;
            if (fineActive) {
                const int m = factor;
                const float tc = p.tau, tf = fineTau(tc, m);
                CollideParams fp = p;
                fp.tau = tf;
                fp.writeMacro = 0;
                // Factor 2: the last sub-step's collide also forms the
                // restriction's child averages (no re-read of the fine level)
                // -- unless a finer level rewrites the fine state after it.
                const bool fuse = fuseOn() && m == 2 && !finerActive;
                for (int k = 0; k < m; ++k) {
                    ++launches;
                    if (auto e = launch_fill_c2f(storage, coarse.f[coarse.src], coarse.f[1 - coarse.src],
                                                 coarse.kind, fine.f[fine.src], dShell, shellCount, geom(),
                                                 static_cast<float>(k) / static_cast<float>(m),
                                                 tf / (static_cast<float>(m) * tc), stream);
                        e != cudaSuccess)
                        return e;
                    const cudaError_t ce = (fuse && k == m - 1) ? collideChild(fine, fp, geom(), dScratch)
                                                                : collide(fine, fp, nullptr, nullptr, nullptr, nullptr);
                    if (ce != cudaSuccess) return ce;
                    // Nested finer level (lbm_solver.cpp:1209-1270): m2
                    // sub-steps between the fine pair's two time levels, then
                    // restriction into the fine t+1 buffer, before the swap.
                    if (finerActive) {
                        const int m2 = finerFactor;
                        const float tr = fineTau(tf, m2);
                        CollideParams rp = fp;
                        rp.tau = tr;
                        const bool fuseR = fuseOn() && m2 == 2;
                        for (int q = 0; q < m2; ++q) {
                            ++launches;
                            if (auto e = launch_fill_c2f(storage, fine.f[fine.src], fine.f[1 - fine.src], fine.kind,
                                                         finer.f[finer.src], dShellFiner, shellCountFiner,
                                                         geomFiner(), static_cast<float>(q) / static_cast<float>(m2),
                                                         tr / (static_cast<float>(m2) * tf), stream);
                                e != cudaSuccess)
                                return e;
                            const cudaError_t cr = (fuseR && q == m2 - 1)
                                                       ? collideChild(finer, rp, geomFiner(), dScratchFiner)
                                                       : collide(finer, rp, nullptr, nullptr, nullptr, nullptr);
                            if (cr != cudaSuccess) return cr;
                            finer.src = 1 - finer.src;
                        }
                        launches += fuseR ? 1 : 2;
                        if (auto e = launch_restrict_f2c(storage, finer.f[finer.src], finer.kind, fine.f[1 - fine.src],
                                                         fine.kind, geomFiner(), (static_cast<float>(m2) * tf) / tr,
                                                         dScratchFiner, nullptr, nullptr, nullptr, nullptr, stream,
                                                         fuseR);
                            e != cudaSuccess)
                            return e;
                    }
                    fine.src = 1 - fine.src;
                }
                launches += fuse ? 1 : 2;
                const bool mac = p.writeMacro != 0;
                if (auto e = launch_restrict_f2c(storage, fine.f[fine.src], fine.kind, coarse.f[1 - coarse.src],
                                                 coarse.kind, geom(), (static_cast<float>(m) * tc) / tf,
                                                 dScratch, mac ? rho : nullptr, mac ? u : nullptr,
                                                 mac ? v : nullptr, mac ? w : nullptr, stream, fuse);
                    e != cudaSuccess)
                    return e;
            }
            if (!aa) coarse.src = 1 - coarse.src;
            ++steps;
            if (++sinceWatchdog >= kWatchdogPeriod && !nanPending) {
                sinceWatchdog = 0;
                cudaMemsetAsync(dNan, 0, sizeof(int), stream);
                ++launches;
                launch_watchdog(storage, coarse.f[coarse.src], coarse.d, dNan, steps * 977, 0, stream);
                if (fineActive) {
                    ++launches;
                    launch_watchdog(storage, fine.f[fine.src], fine.d, dNan, steps * 977, 2, stream);
                }
                if (finerActive) {  // verdicts 5/6 name the finer level
                    ++launches;
                    launch_watchdog(storage, finer.f[finer.src], finer.d, dNan, steps * 977, 4, stream);
                }
                cudaMemcpyAsync(hNan, dNan, sizeof(int), cudaMemcpyDeviceToHost, stream);
                cudaMemcpyAsync(hNan + 1, dStatus, sizeof(int), cudaMemcpyDeviceToHost, stream);
                cudaEventRecord(evNan, stream);
                nanPending = true;
            }
        }
        if (timeIt) {
            cudaEventRecord(evT1, stream);
            timingPending = true;
            timingN = n;
        }
        if (!forcePending) {
            Level& L = (fineActive && forcesFromFine) ? fine : coarse;
            if (forceReduce(L) == cudaSuccess) {
                cudaMemcpyAsync(hForce, dForce, 3 * sizeof(double), cudaMemcpyDeviceToHost, stream);
                cudaEventRecord(evForce, stream);
                forcePending = true;
                stepsAtForceLaunch = steps;
            }
        }
        const float tauNow = effTau();
        if (coarse.wm.active) wallUpdate(coarse, (tauNow - 0.5f) / 3.0f);
        if (fineActive && fine.wm.active) wallUpdate(fine, (fineTau(tauNow, factor) - 0.5f) / 3.0f);
        if (finerActive && finer.wm.active)
            wallUpdate(finer, (fineTau(fineTau(tauNow, factor), finerFactor) - 0.5f) / 3.0f);
        return static_cast<int>(cudaGetLastError());
    }

    void reset() {
        if (!initialized) return;
        steps = 0;
        coarse.src = 0;
        fine.src = 0;
        rampActive = true;
        rampStart = 0;
        gateOpenAt = static_cast<long long>(kForceGateFT * flowThroughSteps());
        emaFx = emaFy = 0.f;
        emaSeeded = false;
        if (forcePending) { cudaStreamSynchronize(stream); forcePending = false; }
        stepsAtForceLaunch = stepsAtLastFold = 0;
        ringHead = ringCount = 0;
        nanLatched = nanPending = false;
        nanKind = 0;
        sinceWatchdog = 0;
        cudaMemsetAsync(dNan, 0, sizeof(int), stream);
        cudaMemsetAsync(dStatus, 0, sizeof(int), stream);
        const float initU = rampEnabled ? 0.0f : scaling.u_lat;
        for (int i = 0; i < (aa ? 1 : 2); ++i) {
            launches += 2;
            launch_init_equilibrium(storage, coarse.f[i], coarse.kind, coarse.d, initU, stream);
            launch_speck(storage, coarse.f[i], coarse.kind, coarse.d, kSpeckAmplitudeFrac * scaling.u_lat,
                         kSpeckSeed, stream);
        }
        aaAB = aa;
        seedFine();
        seedFiner();
        resetWMState();
    }

    void notifyRestored(bool full) {
        if (!initialized) return;
        rampActive = false;
        emaSeeded = false;
        if (forcePending) { cudaStreamSynchronize(stream); forcePending = false; }
        stepsAtLastFold = steps;
        nanLatched = nanPending = false;
        gateOpenAt = full ? steps + static_cast<long long>(0.25f * flowThroughSteps())
                          : steps + kCompactSettleSteps
                                + static_cast<long long>(kWarmGateFT * flowThroughSteps());
    }

    cudaError_t importF32(Level& L, const float* host, size_t count) {
        if (count != static_cast<size_t>(L.n) * 19) return cudaErrorInvalidValue;
        const size_t bytes = count * sizeof(float);
        if (&L == &coarse) aaAB = aa;  // a whole A/B state replaces the layout
        if (storage == Storage::F32)
            return cudaMemcpy(L.f[L.src], host, bytes, cudaMemcpyHostToDevice);
        float* stage = nullptr;
        if (auto e = cudaMalloc(&stage, bytes); e != cudaSuccess) return e;
        cudaError_t e = cudaMemcpy(stage, host, bytes, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = launch_f32_to_store(storage, stage, L.f[L.src], L.n, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        cudaFree(stage);
        return e;
    }

    cudaError_t exportF32(Level& L, float* host, size_t count) {
        if (count != static_cast<size_t>(L.n) * 19) return cudaErrorInvalidValue;
        const size_t bytes = count * sizeof(float);
        if (&L == &coarse)
            if (auto e = aaToAB(); e != cudaSuccess) return e;
        if (auto e = cudaStreamSynchronize(stream); e != cudaSuccess) return e;
        if (storage == Storage::F32)
            return cudaMemcpy(host, L.f[L.src], bytes, cudaMemcpyDeviceToHost);
        float* stage = nullptr;
        if (auto e = cudaMalloc(&stage, bytes); e != cudaSuccess) return e;
        cudaError_t e = launch_store_to_f32(storage, L.f[L.src], stage, L.n, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e == cudaSuccess) e = cudaMemcpy(host, stage, bytes, cudaMemcpyDeviceToHost);
        cudaFree(stage);
        return e;
    }
};

// ===========================================================================
// C ABI
// ===========================================================================

extern "C" {

fcfd_scaling fcfd_compute_scaling(float chord_m, float airspeed_ms, float nu_m2s, int chord_cells,
                                  float u_lat) {
    fcfd_scaling s{};
    s.chord_m = chord_m; s.airspeed_ms = airspeed_ms; s.nu_m2s = nu_m2s;
    s.chord_cells = chord_cells;
    s.u_lat = std::min(u_lat, kMaxULat);
    s.dx = chord_m / static_cast<float>(chord_cells);
    s.dt = s.u_lat * s.dx / airspeed_ms;
    s.nu_lat_target = nu_m2s * s.dt / (s.dx * s.dx);
    const float tauTarget = 3.0f * s.nu_lat_target + 0.5f;
    s.tau = std::max(tauTarget, kMinTau);
    s.tau_clamped = tauTarget < kMinTau ? 1 : 0;
    s.nu_lat = (s.tau - 0.5f) / 3.0f;
    s.re_target = airspeed_ms * chord_m / nu_m2s;
    s.re_effective = s.u_lat * static_cast<float>(chord_cells) / s.nu_lat;
    return s;
}

fcfd_scaling fcfd_refined_scaling(const fcfd_scaling* p, int factor) {
    fcfd_scaling f = *p;
    const float m = static_cast<float>(factor);
    f.chord_cells = p->chord_cells * factor;
    f.dx = p->dx / m;
    f.dt = p->dt / m;
    f.nu_lat_target = p->nu_lat_target * m;
    f.nu_lat = p->nu_lat * m;
    f.tau = 3.0f * f.nu_lat + 0.5f;
    return f;
}

float fcfd_ramped_tau(const fcfd_scaling* s, long long step, int nx) {
    const long long ramp = 2LL * nx;
    if (step >= ramp) return s->tau;
    const float t = static_cast<float>(step) / static_cast<float>(ramp);
    const float nu = s->nu_lat * (4.0f + t * (1.0f - 4.0f));
    return 3.0f * nu + 0.5f;
}

float fcfd_ramped_u(const fcfd_scaling* s, long long step, int nx) {
    const long long ramp = static_cast<long long>(0.5f * 2.0f * static_cast<float>(nx));
    if (ramp <= 0 || step >= ramp) return s->u_lat;
    const float t = static_cast<float>(step) / static_cast<float>(ramp);
    return s->u_lat * (t * t * (3.0f - 2.0f * t));
}

float fcfd_force_to_coefficient(const fcfd_scaling* s, float f, int span) {
    const float q = 0.5f * s->u_lat * s->u_lat * static_cast<float>(s->chord_cells) * static_cast<float>(span);
    return q > 0.0f ? f / q : 0.0f;
}

fcfd_solver* fcfd_create(void) { return new fcfd_solver(); }

void fcfd_destroy(fcfd_solver* s) {
    if (!s) return;
    s->freeAll();
    delete s;
}

int fcfd_init(fcfd_solver* s, const fcfd_dims* dims, const fcfd_scaling* scaling, const uint8_t* flags,
              size_t n, void* stream, const fcfd_options* opts, char* err, size_t errlen) {
    if (!s || !dims || !scaling || !flags) {
        set_err(err, errlen, "null argument");
        return cudaErrorInvalidValue;
    }
    s->freeAll();
    LevelDims d{dims->nx, dims->ny, dims->nz};
    if (d.nx < 3 || d.ny < 3 || d.nz < 1 || d.cells() <= 0) {
        set_err(err, errlen, "grid dimensions out of range");
        return cudaErrorInvalidValue;
    }
    if (d.cells() * 19 >= (1LL << 31) * 2 || d.cells() >= (1LL << 31)) {
        set_err(err, errlen, "grid too large for 32-bit cell indices");
        return cudaErrorInvalidValue;
    }
    if (n != static_cast<size_t>(d.cells())) {
        set_err(err, errlen, "flag field size does not match grid dimensions");
        return cudaErrorInvalidValue;
    }
    std::vector<std::uint8_t> hostCopy;
    const uint8_t* hf = flags;
    if (on_device(flags)) {
        assign_flags(hostCopy, flags, n);
        hf = hostCopy.data();
    }
    for (size_t i = 0; i < n; ++i)
        if (hf[i] > FCFD_FLAG_OUTLET_EQ) {
            set_err(err, errlen, "flag field holds an unknown cell flag value");
            return cudaErrorInvalidValue;
        }
    s->dims = d;
    s->scaling = *scaling;
    s->stream = static_cast<cudaStream_t>(stream);
    s->storage = Storage::F32;
    s->lesCs = kDefaultCs;
    s->lambda = kDefaultLambda;
    s->collideKernel = 0;
    s->aa = false;
    s->aaAB = false;
    s->aaNextOdd = 1;
    if (opts) {
        s->storage = opts->storage == FCFD_STORE_FP16 ? Storage::F16 : Storage::F32;
        if (opts->les_cs != 0.0f) s->lesCs = opts->les_cs;
        if (opts->magic_lambda > 0.0f) s->lambda = opts->magic_lambda;
        s->collideKernel = (opts->collide_kernel >= 0 && opts->collide_kernel <= 2) ? opts->collide_kernel : 0;
        s->aa = opts->layout == FCFD_LAYOUT_AA;
    }
    if (s->aa && !aa_lattice(hf, n)) {
        set_err(err, errlen, "the AA layout serves all-fluid periodic lattices only");
        s->aa = false;
        return cudaErrorNotSupported;
    }
    auto fail = [&](const char* what, cudaError_t e) {
        set_err(err, errlen, std::string(what) + ": " + cudaGetErrorString(e));
        s->freeAll();
        (void)cudaGetLastError();
        return static_cast<int>(e);
    };
    if (auto e = s->allocLevel(s->coarse, d); e != cudaSuccess) return fail("population buffer allocation failed", e);
    const size_t cells = static_cast<size_t>(d.cells());
    if (s->aa)
        if (auto e = cudaMalloc(&s->aaSlice, cells * (s->storage == Storage::F32 ? 4 : 2)); e != cudaSuccess)
            return fail("AA scratch allocation failed", e);
    for (float** p : {&s->rho, &s->u, &s->v, &s->w})
        if (auto e = dalloc(p, cells * 4); e != cudaSuccess) return fail("macroscopic allocation failed", e);
    if (auto e = dalloc(&s->dForce, 3 * sizeof(double)); e != cudaSuccess) return fail("force slot allocation failed", e);
    if (auto e = dalloc(&s->dNan, sizeof(int)); e != cudaSuccess) return fail("watchdog allocation failed", e);
    if (auto e = dalloc(&s->dStatus, sizeof(int)); e != cudaSuccess) return fail("status allocation failed", e);
    if (auto e = cudaMemsetAsync(s->dStatus, 0, sizeof(int), s->stream); e != cudaSuccess)
        return fail("status allocation failed", e);
    if (auto e = cudaMallocHost(&s->hForce, 3 * sizeof(double)); e != cudaSuccess) return fail("pinned allocation failed", e);
    if (auto e = cudaMallocHost(&s->hNan, 2 * sizeof(int)); e != cudaSuccess) return fail("pinned allocation failed", e);
    for (auto pr : {std::pair<cudaEvent_t*, unsigned>{&s->evT0, 0u}, {&s->evT1, 0u},
                    {&s->evForce, static_cast<unsigned>(cudaEventDisableTiming)},
                    {&s->evNan, static_cast<unsigned>(cudaEventDisableTiming)}})
        if (auto e = cudaEventCreateWithFlags(pr.first, pr.second); e != cudaSuccess)
            return fail("event creation failed", e);
    s->hNan[0] = s->hNan[1] = 0;
    s->launches += 1;
    launch_fill(s->rho, d.cells(), 1.0f, s->stream);
    cudaMemsetAsync(s->u, 0, cells * 4, s->stream);
    cudaMemsetAsync(s->v, 0, cells * 4, s->stream);
    cudaMemsetAsync(s->w, 0, cells * 4, s->stream);
    if (auto e = s->uploadLevelFlags(s->coarse, flags); e != cudaSuccess) return fail("flag upload failed", e);
    s->zSlipWalls = false;
    const size_t nxny = static_cast<size_t>(d.nx) * d.ny;
    for (size_t i = 0; i < nxny; ++i)
        if (hf[i] == FCFD_FLAG_SLIP_FRONT) { s->zSlipWalls = true; break; }
    if (auto e = s->buildWM(s->coarse, kWallSampleCoarse); e != cudaSuccess) return fail("wall list upload failed", e);
    s->initialized = true;
    s->reset();
    if (auto e = cudaStreamSynchronize(s->stream); e != cudaSuccess) return fail("initial field setup failed", e);
    if (auto e = cudaGetLastError(); e != cudaSuccess) return fail("initial field setup failed", e);
    set_err(err, errlen, "");
    return 0;
}

void fcfd_reset(fcfd_solver* s) {
    if (s) s->reset();
}

int fcfd_set_flags(fcfd_solver* s, const uint8_t* flags, size_t n) {
    if (!s || !s->initialized || !flags || n != static_cast<size_t>(s->coarse.n)) return cudaErrorInvalidValue;
    if (s->aa && !aa_flags_ok(flags, n)) return cudaErrorNotSupported;
    if (auto e = s->uploadLevelFlags(s->coarse, flags); e != cudaSuccess) return e;
    s->updateForcesFromFine();
    if (auto e = s->buildWM(s->coarse, kWallSampleCoarse); e != cudaSuccess) return e;
    s->reset();
    return 0;
}

int fcfd_apply_edited_flags(fcfd_solver* s, const uint8_t* flags, size_t n, long long* edited) {
    if (edited) *edited = 0;
    if (!s || !s->initialized || !flags || n != static_cast<size_t>(s->coarse.n)) return cudaErrorInvalidValue;
    if (s->aa && !aa_flags_ok(flags, n)) return cudaErrorNotSupported;
    Level& L = s->coarse;
    std::vector<std::uint8_t> hostNew;
    const std::uint8_t* nf = flags;
    if (on_device(flags)) {
        assign_flags(hostNew, flags, n);
        nf = hostNew.data();
    }
    // Diff before the host copy is replaced: 1 newly solid, 2 newly fluid.
    std::vector<std::uint8_t> mask(static_cast<size_t>(L.n), 0);
    long long count = 0;
    for (long long i = 0; i < L.n; ++i) {
        const bool was = L.hostFlags[static_cast<size_t>(i)] == FCFD_FLAG_SOLID;
        const bool now = nf[i] == FCFD_FLAG_SOLID;
        if (was == now) continue;
        mask[static_cast<size_t>(i)] = now ? 1 : 2;
        ++count;
    }
    if (auto e = s->uploadLevelFlags(L, flags); e != cudaSuccess) return e;
    if (count > 0) {
        std::uint8_t* dMaskBuf = nullptr;
        if (auto e = cudaMalloc(&dMaskBuf, static_cast<size_t>(L.n)); e != cudaSuccess) return e;
        cudaError_t e = cudaMemcpyAsync(dMaskBuf, mask.data(), static_cast<size_t>(L.n), cudaMemcpyHostToDevice,
                                        s->stream);
        if (e == cudaSuccess) {
            ++s->launches;
            e = launch_apply_flag_edits(s->storage, L.f[L.src], L.f[1 - L.src], L.flags, dMaskBuf, L.d, s->stream);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        cudaFree(dMaskBuf);
        if (e != cudaSuccess) return e;
    }
    s->updateForcesFromFine();
    if (auto e = s->buildWM(L, kWallSampleCoarse); e != cudaSuccess) return e;
    s->rampActive = false;
    s->emaSeeded = false;
    if (s->forcePending) { cudaStreamSynchronize(s->stream); s->forcePending = false; }
    s->stepsAtLastFold = s->steps;
    s->gateOpenAt = s->steps + static_cast<long long>(kWarmGateFT * s->flowThroughSteps());
    if (edited) *edited = count;
    return 0;
}

void fcfd_set_startup_ramp(fcfd_solver* s, int enabled) {
    if (s) s->rampEnabled = enabled != 0;
}

void fcfd_set_force_ema_window(fcfd_solver* s, float ft) {
    if (s) s->emaWindowFT = std::max(0.05f, ft);
}

int fcfd_step_n(fcfd_solver* s, int n) { return s ? s->stepN(n) : cudaErrorInvalidValue; }

int fcfd_synchronize(fcfd_solver* s) {
    if (!s || !s->initialized) return cudaErrorNotReady;
    const cudaError_t e = cudaStreamSynchronize(s->stream);
    s->pollAsync();
    return e;
}

long long fcfd_step_count(const fcfd_solver* s) { return s ? s->steps : 0; }
float fcfd_current_tau(const fcfd_solver* s) { return (s && s->initialized) ? s->effTau() : 0.0f; }
float fcfd_flow_throughs(const fcfd_solver* s) {
    return (s && s->initialized) ? static_cast<float>(s->steps) / s->flowThroughSteps() : 0.0f;
}

int fcfd_forces(fcfd_solver* s, fcfd_force_readout* r) {
    if (!s || !r) return cudaErrorInvalidValue;
    *r = fcfd_force_readout{};
    if (!s->initialized) return cudaErrorNotReady;
    // As the reference's forces() (lbm_solver.cpp:1414-1509): read what the
    // asynchronous read-backs have delivered so far. Folding completed
    // samples only queries events, so the call never waits on the stream.
    s->pollAsync();
    r->flow_throughs = fcfd_flow_throughs(s);
    const bool fineForces = s->fineActive && s->forcesFromFine;
    const fcfd_scaling& fs = fineForces ? s->fineScaling : s->scaling;
    const int span = fineForces ? s->fine.d.nz : (s->zSlipWalls ? std::max(1, s->dims.nz - 2) : s->dims.nz);
    r->cd = fcfd_force_to_coefficient(&fs, s->emaFx, span);
    r->cl = fcfd_force_to_coefficient(&fs, s->emaFy, span);
    r->lift_to_drag = std::fabs(r->cd) > 1e-6f ? r->cl / r->cd : 0.0f;
    r->valid = (s->emaSeeded && s->steps >= s->gateOpenAt) ? 1 : 0;
    if (r->valid && s->ringCount > 0) {
        const long long oneFT = static_cast<long long>(s->flowThroughSteps());
        std::vector<float> cl, cd, ld;
        for (int i = 0; i < s->ringCount; ++i) {
            const int k = (s->ringHead - 1 - i + fcfd_solver::kRing) % fcfd_solver::kRing;
            const ForceSample& sm = s->ring[k];
            if (sm.step < oneFT) continue;
            const float c1 = fcfd_force_to_coefficient(&fs, sm.fy, span);
            const float c2 = fcfd_force_to_coefficient(&fs, sm.fx, span);
            cl.push_back(c1); cd.push_back(c2);
            ld.push_back(std::fabs(c2) > 1e-6f ? c1 / c2 : 0.0f);
        }
        if (!cl.empty()) {
            auto stats = [](std::vector<float> v, float& avg, float& mn, float& mx, float& med) {
                float sum = 0.f;
                for (float x : v) sum += x;
                avg = sum / static_cast<float>(v.size());
                mn = *std::min_element(v.begin(), v.end());
                mx = *std::max_element(v.begin(), v.end());
                std::sort(v.begin(), v.end());
                const size_t m = v.size() / 2;
                med = v.size() % 2 == 0 ? 0.5f * (v[m - 1] + v[m]) : v[m];
            };
            stats(cl, r->cl_avg, r->cl_min, r->cl_max, r->cl_median);
            stats(cd, r->cd_avg, r->cd_min, r->cd_max, r->cd_median);
            stats(ld, r->ld_avg, r->ld_min, r->ld_max, r->ld_median);
        }
    }
    return 0;
}

/// Level 0 coarse, 1 fine, 2 finer; null when that level is not active.
static const Level* active_level(const fcfd_solver* s, int level) {
    if (level == 0) return &s->coarse;
    if (level == 1 && s->fineActive) return &s->fine;
    if (level == 2 && s->finerActive) return &s->finer;
    return nullptr;
}

int fcfd_device_flags(fcfd_solver* s, int level, const uint8_t** flags) {
    if (!s || !flags) return cudaErrorInvalidValue;
    *flags = nullptr;
    if (!s->initialized) return cudaErrorNotReady;
    const Level* L = active_level(s, level);
    if (!L) return cudaErrorInvalidValue;
    *flags = L->flags;
    return 0;
}

int fcfd_lattice_view(fcfd_solver* s, int level, fcfd_lattice* out) {
    if (!s || !out) return cudaErrorInvalidValue;
    *out = fcfd_lattice{};
    if (!s->initialized) return cudaErrorNotReady;
    const Level* L = active_level(s, level);
    if (!L) return cudaErrorInvalidValue;
    if (auto e = s->aaToAB(); e != cudaSuccess) return e;
    out->f = L->f[L->src];
    out->flags = L->flags;
    out->dims = fcfd_dims{L->d.nx, L->d.ny, L->d.nz};
    out->cells = L->n;
    out->storage = s->storage == Storage::F32 ? FCFD_STORE_FP32 : FCFD_STORE_FP16;
    out->uwx = L->wm.active ? L->wm.dUwx : nullptr;
    out->uwy = L->wm.active ? L->wm.dUwy : nullptr;
    out->uwz = L->wm.active ? L->wm.dUwz : nullptr;
    return 0;
}

int fcfd_force_raw(fcfd_solver* s, double out[3]) {
    if (!s || !out) return cudaErrorInvalidValue;
    if (!s->initialized) return cudaErrorNotReady;
    const cudaError_t e = cudaStreamSynchronize(s->stream);
    s->pollAsync();
    for (int i = 0; i < 3; ++i) out[i] = s->lastForce[i];
    return e;
}

int fcfd_force_now(fcfd_solver* s, double out[3]) {
    if (!s || !out) return cudaErrorInvalidValue;
    if (!s->initialized) return cudaErrorNotReady;
    cudaStreamSynchronize(s->stream);
    s->pollAsync();
    Level& L = (s->fineActive && s->forcesFromFine) ? s->fine : s->coarse;
    if (auto e = s->forceReduce(L); e != cudaSuccess) return e;
    double h[3];
    if (auto e = cudaMemcpyAsync(h, s->dForce, sizeof h, cudaMemcpyDeviceToHost, s->stream); e != cudaSuccess)
        return e;
    if (auto e = cudaStreamSynchronize(s->stream); e != cudaSuccess) return e;
    for (int i = 0; i < 3; ++i) out[i] = h[i];
    return 0;
}

int fcfd_macro(fcfd_solver* s, const float** r, const float** u, const float** v, const float** w) {
    if (!s || !s->initialized) return cudaErrorNotReady;
    if (r) *r = s->rho;
    if (u) *u = s->u;
    if (v) *v = s->v;
    if (w) *w = s->w;
    return 0;
}

int fcfd_download_macro(fcfd_solver* s, float* r, float* u, float* v, float* w) {
    if (!s || !s->initialized) return cudaErrorNotReady;
    const size_t b = static_cast<size_t>(s->coarse.n) * 4;
    struct { float* h; const float* d; } c[] = {{r, s->rho}, {u, s->u}, {v, s->v}, {w, s->w}};
    for (auto& x : c)
        if (x.h)
            if (auto e = cudaMemcpyAsync(x.h, x.d, b, cudaMemcpyDeviceToHost, s->stream); e != cudaSuccess)
                return e;
    return cudaStreamSynchronize(s->stream);
}

void* fcfd_active_f(fcfd_solver* s) {
    if (!s || !s->initialized || s->aaToAB() != cudaSuccess) return nullptr;
    return s->coarse.f[s->coarse.src];
}

size_t fcfd_f_bytes(const fcfd_solver* s) {
    if (!s || !s->initialized) return 0;
    return static_cast<size_t>(s->coarse.n) * 19 * (s->storage == Storage::F32 ? 4 : 2);
}

void fcfd_notify_restored(fcfd_solver* s, int full) {
    if (s) s->notifyRestored(full != 0);
}

int fcfd_import_f32(fcfd_solver* s, const float* f, size_t count) {
    if (!s || !s->initialized || !f) return cudaErrorInvalidValue;
    if (auto e = s->importF32(s->coarse, f, count); e != cudaSuccess) return e;
    s->notifyRestored(true);
    return 0;
}

int fcfd_mirror_buffers(fcfd_solver* s) {
    if (!s || !s->initialized) return cudaErrorInvalidValue;
    const size_t pop = s->storage == Storage::F32 ? 4 : 2;
    if (s->aa) return 0;  // one population array: nothing to mirror
    Level* levels[3] = {&s->coarse, s->fineActive ? &s->fine : nullptr, s->finerActive ? &s->finer : nullptr};
    for (Level* L : levels) {
        if (!L) continue;
        if (auto e = cudaMemcpyAsync(L->f[1 - L->src], L->f[L->src], static_cast<size_t>(L->n) * 19 * pop,
                                     cudaMemcpyDeviceToDevice, s->stream);
            e != cudaSuccess)
            return e;
    }
    return cudaStreamSynchronize(s->stream);
}

int fcfd_stage_f32(fcfd_solver* s, int level, const float* f, size_t count) {
    if (!s || !s->initialized) return cudaErrorInvalidValue;
    return s->stageF32(level, f, count);
}

int fcfd_commit_staged(fcfd_solver* s) {
    if (!s || !s->initialized) return cudaErrorInvalidValue;
    return s->commitStaged();
}

int fcfd_export_f32(fcfd_solver* s, float* f, size_t count) {
    if (!s || !s->initialized || !f) return cudaErrorInvalidValue;
    return s->exportF32(s->coarse, f, count);
}

int fcfd_restore_from_macro(fcfd_solver* s, const float* r, const float* u, const float* v, const float* w) {
    if (!s || !s->initialized || !r || !u || !v || !w) return cudaErrorInvalidValue;
    const size_t b = static_cast<size_t>(s->coarse.n) * 4;
    struct { const float* h; float* d; } c[] = {{r, s->rho}, {u, s->u}, {v, s->v}, {w, s->w}};
    for (auto& x : c)
        if (auto e = cudaMemcpyAsync(x.d, x.h, b, cudaMemcpyHostToDevice, s->stream); e != cudaSuccess) return e;
    for (int i = 0; i < (s->aa ? 1 : 2); ++i) {
        ++s->launches;
        if (auto e = launch_init_from_macro(s->storage, s->coarse.f[i], s->coarse.kind, s->coarse.d, s->rho,
                                            s->u, s->v, s->w, s->stream);
            e != cudaSuccess)
            return e;
    }
    s->aaAB = s->aa;
    s->notifyRestored(false);
    if (auto e = s->seedFine(); e != cudaSuccess) return e;
    if (auto e = s->seedFiner(); e != cudaSuccess) return e;
    return cudaStreamSynchronize(s->stream);
}

int fcfd_perf_stats(const fcfd_solver* s, fcfd_perf* p) {
    if (!s || !p) return cudaErrorInvalidValue;
    *p = fcfd_perf{};
    double upd = static_cast<double>(s->coarse.n);
    if (s->fineActive) upd += static_cast<double>(s->factor) * static_cast<double>(s->fine.n);
    if (s->finerActive)  // every finer cell m * m2 times per coarse step (lbm_solver.cpp:1703-1712)
        upd += static_cast<double>(s->factor) * s->finerFactor * static_cast<double>(s->finer.n);
    p->updates_per_step = upd;
    p->last_step_ms = s->lastStepMs;
    if (s->lastStepMs > 0.0) p->mlups = upd / (s->lastStepMs * 1000.0);
    return 0;
}

int fcfd_nan_detected(fcfd_solver* s) {
    if (!s || !s->initialized) return 0;
    s->pollAsync();
    return s->nanLatched ? 1 : 0;
}

int fcfd_nan_kind(fcfd_solver* s) {
    if (!s || !s->initialized) return 0;
    s->pollAsync();
    return s->nanKind;
}

int fcfd_set_wall_model(fcfd_solver* s, int enabled) {
    if (!s) return cudaErrorInvalidValue;
    const bool en = enabled != 0;
    if (s->wmEnabled == en) return 0;
    s->wmEnabled = en;
    if (!s->initialized) return 0;
    cudaStreamSynchronize(s->stream);
    if (auto e = s->buildWM(s->coarse, kWallSampleCoarse); e != cudaSuccess) return e;
    if (s->fineActive)
        if (auto e = s->buildWM(s->fine, kWallSampleFine); e != cudaSuccess) return e;
    if (s->finerActive)
        if (auto e = s->buildWM(s->finer, kWallSampleFine); e != cudaSuccess) return e;
    return 0;
}

int fcfd_set_surface_reference(fcfd_solver* s, const uint8_t* clean, size_t n) {
    if (!s || !s->initialized || !clean || n != static_cast<size_t>(s->coarse.n)) return cudaErrorInvalidValue;
    cudaStreamSynchronize(s->stream);
    assign_flags(s->coarse.surfaceRef, clean, n);
    return s->buildWM(s->coarse, kWallSampleCoarse);
}

int fcfd_set_refined_surface_reference(fcfd_solver* s, const uint8_t* clean, size_t n) {
    if (!s || !s->initialized || !s->fineActive || !clean || n != static_cast<size_t>(s->fine.n))
        return cudaErrorInvalidValue;
    cudaStreamSynchronize(s->stream);
    assign_flags(s->fine.surfaceRef, clean, n);
    return s->buildWM(s->fine, kWallSampleFine);
}

int fcfd_wall_model_readout(fcfd_solver* s, fcfd_wm_readout* r) {
    if (!s || !r) return cudaErrorInvalidValue;
    *r = fcfd_wm_readout{};
    r->enabled = s->wmEnabled ? 1 : 0;
    if (!s->initialized || !s->wmEnabled) return 0;
    const WMLevel& wm = (s->fineActive && s->fine.wm.active) ? s->fine.wm : s->coarse.wm;
    r->from_fine = (s->fineActive && s->fine.wm.active) ? 1 : 0;
    r->excluded_vg = wm.build.excludedVG;
    r->degenerate = wm.build.degenerate;
    if (!wm.active) return 0;
    WallStatsDev st{};
    if (auto e = cudaMemcpyAsync(&st, wm.dStats, sizeof st, cudaMemcpyDeviceToHost, s->stream); e != cudaSuccess)
        return e;
    if (auto e = cudaStreamSynchronize(s->stream); e != cudaSuccess) return e;
    r->cells = st.activeCells;
    if (st.activeCells > 0) {
        r->mean_yplus = st.sumYplus / static_cast<float>(st.activeCells);
        float mx;
        std::memcpy(&mx, &st.maxYplusBits, sizeof mx);
        r->max_yplus = mx;
        r->clamped_frac = static_cast<float>(st.clampedCells) / static_cast<float>(st.activeCells);
    }
    return 0;
}

static Level* level_of(fcfd_solver* s, int level) {
    if (!s || !s->initialized) return nullptr;
    if (level == 0) return &s->coarse;
    if (level == 1 && s->fineActive) return &s->fine;
    if (level == 2 && s->finerActive) return &s->finer;
    return nullptr;
}

int fcfd_wall_count(fcfd_solver* s, int level) {
    Level* L = level_of(s, level);
    return (L && L->wm.active) ? L->wm.count : 0;
}

int fcfd_export_wall_state(fcfd_solver* s, int level, float* utau, size_t nu, uint16_t* slip, size_t ns) {
    Level* L = level_of(s, level);
    if (!L || !L->wm.active) return cudaErrorInvalidValue;
    cudaStreamSynchronize(s->stream);
    if (utau) {
        if (nu != static_cast<size_t>(L->wm.count)) return cudaErrorInvalidValue;
        if (auto e = cudaMemcpy(utau, L->wm.dUTau, nu * 4, cudaMemcpyDeviceToHost); e != cudaSuccess) return e;
    }
    if (slip) {
        const size_t n = static_cast<size_t>(L->n);
        if (ns != 3 * n) return cudaErrorInvalidValue;
        const std::uint16_t* src[3] = {L->wm.dUwx, L->wm.dUwy, L->wm.dUwz};
        for (int k = 0; k < 3; ++k)
            if (auto e = cudaMemcpy(slip + k * n, src[k], n * 2, cudaMemcpyDeviceToHost); e != cudaSuccess) return e;
    }
    return 0;
}

int fcfd_import_wall_state(fcfd_solver* s, int level, const float* utau, size_t nu, const uint16_t* slip,
                           size_t ns) {
    Level* L = level_of(s, level);
    if (!L || !L->wm.active) return cudaErrorInvalidValue;
    cudaStreamSynchronize(s->stream);
    if (utau) {
        if (nu != static_cast<size_t>(L->wm.count)) return cudaErrorInvalidValue;
        if (auto e = cudaMemcpy(L->wm.dUTau, utau, nu * 4, cudaMemcpyHostToDevice); e != cudaSuccess) return e;
    }
    if (slip) {
        const size_t n = static_cast<size_t>(L->n);
        if (ns != 3 * n) return cudaErrorInvalidValue;
        std::uint16_t* dst[3] = {L->wm.dUwx, L->wm.dUwy, L->wm.dUwz};
        for (int k = 0; k < 3; ++k)
            if (auto e = cudaMemcpy(dst[k], slip + k * n, n * 2, cudaMemcpyHostToDevice); e != cudaSuccess) return e;
    }
    return 0;
}

int fcfd_wall_update_now(fcfd_solver* s, int level, float nu, float cut) {
    Level* L = level_of(s, level);
    if (!L || !L->wm.active) return cudaErrorInvalidValue;
    ++s->launches;
    if (auto e = launch_wall_update(s->storage, L->f[L->src], L->n, L->wm.list(), L->wm.dUwx, L->wm.dUwy,
                                    L->wm.dUwz, nu, cut, kWallEma, L->wm.dStats, s->stream, s->wallMethod,
                                    &s->netView);
        e != cudaSuccess)
        return e;
    return cudaStreamSynchronize(s->stream);
}

int fcfd_init_refinement(fcfd_solver* s, const fcfd_patch_box* box, int factor, const uint8_t* ff, size_t n,
                         char* err, size_t errlen) {
    if (!s || !s->initialized) {
        set_err(err, errlen, "solver not initialized");
        return cudaErrorNotReady;
    }
    if (s->aa) {
        set_err(err, errlen, "the AA layout serves all-fluid periodic lattices only (no refinement)");
        return cudaErrorNotSupported;
    }
    fcfd_shutdown_refinement(s);
    if (!box || !ff) {
        set_err(err, errlen, "null argument");
        return cudaErrorInvalidValue;
    }
    if (factor < 2 || factor > 4) {
        set_err(err, errlen, "refinement factor out of range (2..4)");
        return cudaErrorInvalidValue;
    }
    if (box->x1 - box->x0 <= 8 || box->y1 - box->y0 <= 8 || box->x0 < 1 || box->y0 < 1
        || box->x1 > s->dims.nx - 1 || box->y1 > s->dims.ny - 1) {
        set_err(err, errlen, "refinement patch box out of range");
        return cudaErrorInvalidValue;
    }
    LevelDims fd{factor * (box->x1 - box->x0), factor * (box->y1 - box->y0), factor * s->dims.nz};
    if (n != static_cast<size_t>(fd.cells())) {
        set_err(err, errlen, "fine flag field size does not match the patch");
        return cudaErrorInvalidValue;
    }
    if (fd.cells() >= (1LL << 31)) {
        set_err(err, errlen, "fine grid too large for 32-bit cell indices");
        return cudaErrorInvalidValue;
    }
    cudaStreamSynchronize(s->stream);
    s->factor = factor;
    s->box = *box;
    s->fineScaling = fcfd_refined_scaling(&s->scaling, factor);
    auto fail = [&](const char* what, cudaError_t e) {
        set_err(err, errlen, std::string(what) + ": " + cudaGetErrorString(e));
        s->freeFine();
        (void)cudaGetLastError();
        return static_cast<int>(e);
    };
    if (auto e = s->allocLevel(s->fine, fd); e != cudaSuccess) return fail("fine buffer allocation failed", e);
    if (auto e = s->uploadLevelFlags(s->fine, ff); e != cudaSuccess) return fail("fine flag upload failed", e);
    if (auto e = s->shellList(s->fine, false, &s->dShell, &s->shellCount); e != cudaSuccess)
        return fail("shell list failed", e);
    if (auto e = s->cellList(s->fine, FCFD_FLAG_SOLID, false, &s->dSeed, &s->seedCount); e != cudaSuccess)
        return fail("seed list failed", e);
    s->fineActive = true;
    const long long sf = restrict_scratch_floats(s->geom());
    if (sf <= 0) return fail("restriction sub-box is empty", cudaErrorInvalidValue);
    if (auto e = dalloc(&s->dScratch, static_cast<size_t>(sf) * 4); e != cudaSuccess)
        return fail("restriction scratch allocation failed", e);
    s->updateForcesFromFine();
    if (auto e = s->buildWM(s->fine, kWallSampleFine); e != cudaSuccess) return fail("fine wall list failed", e);
    if (auto e = s->seedFine(); e != cudaSuccess) return fail("fine level seeding failed", e);
    if (auto e = cudaStreamSynchronize(s->stream); e != cudaSuccess) return fail("fine level seeding failed", e);
    set_err(err, errlen, "");
    return 0;
}

void fcfd_shutdown_refinement(fcfd_solver* s) {
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    s->freeFine();
}

int fcfd_set_refined_flags(fcfd_solver* s, const uint8_t* ff, size_t n) {
    if (!s || !s->initialized || !s->fineActive || !ff || n != static_cast<size_t>(s->fine.n))
        return cudaErrorInvalidValue;
    if (auto e = s->uploadLevelFlags(s->fine, ff); e != cudaSuccess) return e;
    if (auto e = s->shellList(s->fine, s->fineShellFull, &s->dShell, &s->shellCount); e != cudaSuccess) return e;
    if (auto e = s->cellList(s->fine, FCFD_FLAG_SOLID, false, &s->dSeed, &s->seedCount); e != cudaSuccess) return e;
    s->updateForcesFromFine();
    if (auto e = s->buildWM(s->fine, kWallSampleFine); e != cudaSuccess) return e;
    if (auto e = s->seedFine(); e != cudaSuccess) return e;
    return s->seedFiner();  // the finer level restarts from the re-seeded fine field
}

int fcfd_refinement_info(const fcfd_solver* s, fcfd_refine_info* r) {
    if (!s || !r) return cudaErrorInvalidValue;
    *r = fcfd_refine_info{};
    if (!s->fineActive) return 0;
    r->active = 1;
    r->factor = s->factor;
    r->box = s->box;
    r->fine_dims = fcfd_dims{s->fine.d.nx, s->fine.d.ny, s->fine.d.nz};
    r->forces_from_fine = s->forcesFromFine ? 1 : 0;
    r->vram_bytes = 2.0 * 19.0 * static_cast<double>(s->fine.n) * (s->storage == Storage::F32 ? 4 : 2)
                  + 2.0 * static_cast<double>(s->fine.n);
    return 0;
}

int fcfd_import_fine_f32(fcfd_solver* s, const float* f, size_t count) {
    if (!s || !s->initialized || !s->fineActive || !f) return cudaErrorInvalidValue;
    return s->importF32(s->fine, f, count);
}

int fcfd_export_fine_f32(fcfd_solver* s, float* f, size_t count) {
    if (!s || !s->initialized || !s->fineActive || !f) return cudaErrorInvalidValue;
    return s->exportF32(s->fine, f, count);
}

long long fcfd_build_wall_list(const fcfd_dims* dims, const uint8_t* active, const uint8_t* clean,
                               int sample, long long* ci, long long* si, float* nx, float* ny, float* nz,
                               float* ys, uint32_t* mask, long long cap, int* stats) {
    if (!dims || !active) return -1;
    LevelDims d{dims->nx, dims->ny, dims->nz};
    WallListStats st;
    const WallList wl = build_wall_list(d, active, clean ? clean : active, sample, &st);
    if (stats) { stats[0] = st.listed; stats[1] = st.excludedVG; stats[2] = st.degenerate; }
    const long long n = static_cast<long long>(wl.size());
    if (n > cap) return -1;
    for (long long i = 0; i < n; ++i) {
        if (ci) ci[i] = wl.cellIdx[i];
        if (si) si[i] = wl.sampleIdx[i];
        if (nx) nx[i] = wl.nX[i];
        if (ny) ny[i] = wl.nY[i];
        if (nz) nz[i] = wl.nZ[i];
        if (ys) ys[i] = wl.ys[i];
        if (mask) mask[i] = wl.linkMask[i];
    }
    return n;
}

int fcfd_boundary_flags(const fcfd_dims* dims, uint8_t* flags, size_t n) {
    if (!dims || !flags) return -1;
    LevelDims d{dims->nx, dims->ny, dims->nz};
    if (n != static_cast<size_t>(d.cells()) || d.nx < 2 || d.ny < 2) return -1;
    boundary_flags(d, flags);
    return 0;
}

int fcfd_naca4(const char* digits, int pps, float* xy, int cap) {
    std::vector<float> v;
    const int n = naca4(digits, pps, v);
    if (n < 0 || n > cap || !xy) return -1;
    std::memcpy(xy, v.data(), v.size() * sizeof(float));
    return n;
}

int fcfd_voxelize_airfoil(const fcfd_dims* dims, const float* xy, int npts, float aoa, int chord,
                          float ax, float ay, uint8_t* flags, size_t n) {
    if (!dims || !xy || !flags) return -1;
    LevelDims d{dims->nx, dims->ny, dims->nz};
    if (n != static_cast<size_t>(d.cells())) return -1;
    voxelize_airfoil(d, xy, npts, aoa, chord, ax, ay, flags);
    return 0;
}

int fcfd_close_trailing_edge_gaps(const fcfd_dims* dims, uint8_t* flags, size_t n) {
    if (!dims || !flags) return -1;
    LevelDims d{dims->nx, dims->ny, dims->nz};
    if (n != static_cast<size_t>(d.cells())) return -1;
    return close_trailing_edge_gaps(d, flags);
}

int fcfd_stamp_interface_shell(const fcfd_dims* dims, uint8_t* flags, size_t n) {
    if (!dims || !flags) return -1;
    LevelDims d{dims->nx, dims->ny, dims->nz};
    if (n != static_cast<size_t>(d.cells())) return -1;
    stamp_interface_shell(d, flags, kInterfaceShell);
    return 0;
}

fcfd_patch_box fcfd_derive_patch_box(const fcfd_dims* dims, const uint8_t* flags, int mx0, int mx1, int my0,
                                     int my1, int clearance) {
    fcfd_patch_box b{};
    if (!dims || !flags) return b;
    LevelDims d{dims->nx, dims->ny, dims->nz};
    int o[4];
    derive_patch_box(d, flags, mx0, mx1, my0, my1, clearance, o);
    b.x0 = o[0]; b.y0 = o[1]; b.x1 = o[2]; b.y1 = o[3];
    return b;
}

long long fcfd_kernel_launches(const fcfd_solver* s) { return s ? s->launches : 0; }

int fcfd_enable_collide_timing(fcfd_solver* s, int enabled) {
    if (!s) return cudaErrorInvalidValue;
    if (s->stream) cudaStreamSynchronize(s->stream);
    s->collideTiming = enabled != 0;
    s->colT.used = 0;
    s->fuseT.used = 0;
    return 0;
}

int fcfd_collide_time_ms(fcfd_solver* s, double* total, long long* count, double* cells,
                         double* alg_bytes) {
    if (!s || !total || !count) return cudaErrorInvalidValue;
    if (auto e = cudaStreamSynchronize(s->stream); e != cudaSuccess) return e;
    double c = 0.0, b = 0.0;
    s->colT.take(*total, *count, c, b);
    if (cells) *cells = c;
    if (alg_bytes) *alg_bytes = b;
    return 0;
}

int fcfd_fused_collide_time_ms(fcfd_solver* s, double* total, long long* count, double* cells,
                               double* alg_bytes) {
    if (!s || !total || !count) return cudaErrorInvalidValue;
    if (auto e = cudaStreamSynchronize(s->stream); e != cudaSuccess) return e;
    double c = 0.0, b = 0.0;
    s->fuseT.take(*total, *count, c, b);
    if (cells) *cells = c;
    if (alg_bytes) *alg_bytes = b;
    return 0;
}

int fcfd_timer_start(fcfd_solver* s) {
    if (!s || !s->initialized) return cudaErrorNotReady;
    for (cudaEvent_t* e : {&s->tmr0, &s->tmr1})
        if (!*e)
            if (auto r = cudaEventCreate(e); r != cudaSuccess) return r;
    return cudaEventRecord(s->tmr0, s->stream);
}

int fcfd_timer_stop(fcfd_solver* s, double* ms) {
    if (!s || !s->initialized || !ms || !s->tmr0) return cudaErrorNotReady;
    if (auto r = cudaEventRecord(s->tmr1, s->stream); r != cudaSuccess) return r;
    if (auto r = cudaEventSynchronize(s->tmr1); r != cudaSuccess) return r;
    float f = 0.f;
    if (auto r = cudaEventElapsedTime(&f, s->tmr0, s->tmr1); r != cudaSuccess) return r;
    *ms = f;
    return 0;
}

void* fcfd_host_alloc(size_t bytes) {
    void* p = nullptr;
    if (cudaMallocHost(&p, bytes) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    return p;
}

void fcfd_host_free(void* p) {
    if (p) cudaFreeHost(p);
}

const char* fcfd_version(void) { return "foilcfd-gb300 0.1 (sm_103a)"; }

} // extern "C"

// ---- learned u_tau seed: solver side (include/foilcfd_wallnet.h) ----------

int fcfd_set_wall_solver(fcfd_solver* s, int method, const fcfd_wallnet* net) {
    if (!s || !s->initialized) return cudaErrorNotReady;
    if (method != FCFD_UTAU_REFERENCE && method != FCFD_UTAU_NEWTON64 && method != FCFD_UTAU_LEARNED)
        return cudaErrorInvalidValue;
    if (method == FCFD_UTAU_LEARNED) {
        if (!net) return cudaErrorInvalidValue;
        const wallnet::NetDev v = wallnet_view(net);
        if (!v.w) return cudaErrorInvalidValue;
        if (!s->dNetW)
            if (auto e = dalloc(&s->dNetW, wallnet::kParams * 2); e != cudaSuccess) return e;
        if (auto e = cudaMemcpyAsync(s->dNetW, v.w, wallnet::kParams * 2, cudaMemcpyDeviceToDevice, s->stream);
            e != cudaSuccess)
            return e;
        s->netView.w = s->dNetW;
        s->netView.norm = v.norm;
    }
    s->wallMethod = method;
    return cudaStreamSynchronize(s->stream);
}

int fcfd_wall_harvest(fcfd_solver* s, int level, float* ut, float* ys, int capacity, int* count) {
    Level* L = level_of(s, level);
    if (!L || !L->wm.active || !ut || !ys || capacity < L->wm.count) return cudaErrorInvalidValue;
    if (auto e = launch_wall_harvest(s->storage, L->f[L->src], L->n, L->wm.list(), 1e-3f * s->scaling.u_lat, ut,
                                     ys, s->stream);
        e != cudaSuccess)
        return e;
    if (count) *count = L->wm.count;
    return cudaStreamSynchronize(s->stream);
}

int fcfd_wall_update_timed(fcfd_solver* s, int level, int reps, float* ms, fcfd_utau_stats* stats) {
    Level* L = level_of(s, level);
    if (!L || !L->wm.active || reps <= 0) return cudaErrorInvalidValue;
    const float tc = s->effTau();
    const float tau = level == 0 ? tc : fcfd_solver::fineTau(tc, s->factor);
    const float nu = (tau - 0.5f) / 3.0f;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, s->stream);
    cudaError_t e = cudaSuccess;
    for (int r = 0; r < reps && e == cudaSuccess; ++r) e = s->wallUpdate(*L, nu);
    cudaEventRecord(b, s->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    float t = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (e != cudaSuccess) return e;
    if (ms) *ms = t / static_cast<float>(reps);
    if (stats) {
        WallStatsDev st{};
        if (auto e2 = cudaMemcpy(&st, L->wm.dStats, sizeof st, cudaMemcpyDeviceToHost); e2 != cudaSuccess) return e2;
        stats->solved = st.activeCells;
        stats->fallbacks = st.fallbackCells;
        stats->newton_iterations = static_cast<long long>(st.newtonIters);
    }
    return 0;
}

int fcfd_set_fused_restriction(fcfd_solver* s, int enabled) {
    if (!s) return cudaErrorInvalidValue;
    s->fuseChild = enabled < 0 ? -1 : (enabled != 0 ? 1 : 0);
    return 0;
}

// ---- interpolated bounce-back link fields (setCoarseQLinks / setFineQLinks,
// src/sim/lbm_solver.cpp:1041-1056; uploadQLevel, :373-410) ---------------

int fcfd_set_q_links(fcfd_solver* s, int level, const uint8_t* qFrac, size_t nq, const uint32_t* ffMask,
                     size_t nm, int links, int fallback) {
    Level* L = level_of(s, level);
    if (!L) return cudaErrorInvalidValue;
    if (s->aa && nq != 0) return cudaErrorNotSupported;
    cudaStreamSynchronize(s->stream);
    dfree(L->dQFrac);
    dfree(L->dFFMask);
    L->qLinks = L->qFallback = 0;
    if (nq == 0) return 0;  // cleared: plain half-way bounce-back
    if (!qFrac || !ffMask || nq != static_cast<size_t>(L->n) * 19 || nm != static_cast<size_t>(L->n))
        return cudaErrorInvalidValue;
    if (auto e = dalloc(&L->dQFrac, nq); e != cudaSuccess) return e;
    if (auto e = dalloc(&L->dFFMask, nm * 4); e != cudaSuccess) { dfree(L->dQFrac); return e; }
    cudaError_t e = cudaMemcpy(L->dQFrac, qFrac, nq, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(L->dFFMask, ffMask, nm * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        dfree(L->dQFrac);
        dfree(L->dFFMask);
        return e;
    }
    L->qLinks = links;
    L->qFallback = fallback;
    return 0;
}

int fcfd_q_link_info(fcfd_solver* s, int level, int* active, int* links, int* fallback) {
    Level* L = level_of(s, level);
    if (!L) return cudaErrorInvalidValue;
    if (active) *active = L->dQFrac ? 1 : 0;
    if (links) *links = L->qLinks;
    if (fallback) *fallback = L->qFallback;
    return 0;
}

// ---- nested finer level (initFinerRefinement & co, lbm_solver.cpp:1916-2010)

/// Interface-shell and seed lists of the finer level (its flags uploaded).
static int finer_lists(fcfd_solver* s) {
    if (auto e = s->shellList(s->finer, false, &s->dShellFiner, &s->shellCountFiner); e != cudaSuccess) return e;
    return s->cellList(s->finer, FCFD_FLAG_SOLID, false, &s->dSeedFiner, &s->seedCountFiner);
}

int fcfd_init_finer_refinement(fcfd_solver* s, const fcfd_patch_box* box, int factor, const uint8_t* ff,
                               size_t n, char* err, size_t errlen) {
    if (!s || !s->initialized) {
        set_err(err, errlen, "solver not initialized");
        return cudaErrorNotReady;
    }
    if (!s->fineActive) {
        set_err(err, errlen, "fine level not active (finer level nests in it)");
        return cudaErrorInvalidValue;
    }
    fcfd_shutdown_finer_refinement(s);
    if (!box || !ff) {
        set_err(err, errlen, "null argument");
        return cudaErrorInvalidValue;
    }
    if (factor < 2 || factor > 4) {
        set_err(err, errlen, "finer factor out of range (2..4)");
        return cudaErrorInvalidValue;
    }
    const LevelDims& pd = s->fine.d;
    if (box->x1 - box->x0 <= 8 || box->y1 - box->y0 <= 8 || box->x0 < 1 || box->y0 < 1 || box->x1 > pd.nx - 1
        || box->y1 > pd.ny - 1) {
        set_err(err, errlen, "finer patch box out of range");
        return cudaErrorInvalidValue;
    }
    LevelDims fd{factor * (box->x1 - box->x0), factor * (box->y1 - box->y0), factor * pd.nz};
    if (n != static_cast<size_t>(fd.cells())) {
        set_err(err, errlen, "finer flag field size does not match the patch");
        return cudaErrorInvalidValue;
    }
    if (fd.cells() >= (1LL << 31)) {
        set_err(err, errlen, "finer grid too large for 32-bit cell indices");
        return cudaErrorInvalidValue;
    }
    cudaStreamSynchronize(s->stream);
    s->finerFactor = factor;
    s->finerBox = *box;
    auto fail = [&](const char* what, cudaError_t e) {
        set_err(err, errlen, std::string(what) + ": " + cudaGetErrorString(e));
        s->freeFiner();
        (void)cudaGetLastError();
        return static_cast<int>(e);
    };
    if (auto e = s->allocLevel(s->finer, fd); e != cudaSuccess) return fail("finer buffer allocation failed", e);
    if (auto e = s->uploadLevelFlags(s->finer, ff); e != cudaSuccess) return fail("finer flag upload failed", e);
    if (auto e = static_cast<cudaError_t>(finer_lists(s)); e != cudaSuccess)
        return fail("finer target lists failed", e);
    s->finerActive = true;
    // A finer box within one cell of the fine level's edge interpolates from
    // the fine shell's outer layer: fill every fine interface cell from now on.
    if (box->x0 < 2 || box->y0 < 2 || box->x1 > pd.nx - 2 || box->y1 > pd.ny - 2) {
        s->fineShellFull = true;
        if (auto e = s->shellList(s->fine, true, &s->dShell, &s->shellCount); e != cudaSuccess)
            return fail("shell list failed", e);
    }
    const long long sf = restrict_scratch_floats(s->geomFiner());
    if (sf <= 0) return fail("finer restriction sub-box is empty", cudaErrorInvalidValue);
    if (auto e = dalloc(&s->dScratchFiner, static_cast<size_t>(sf) * 4); e != cudaSuccess)
        return fail("finer restriction scratch allocation failed", e);
    if (auto e = s->buildWM(s->finer, kWallSampleFine); e != cudaSuccess) return fail("finer wall list failed", e);
    if (auto e = s->seedFiner(); e != cudaSuccess) return fail("finer level seeding failed", e);
    if (auto e = cudaStreamSynchronize(s->stream); e != cudaSuccess) return fail("finer level seeding failed", e);
    set_err(err, errlen, "");
    return 0;
}

void fcfd_shutdown_finer_refinement(fcfd_solver* s) {
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    s->freeFiner();
    if (s->fineShellFull && s->fineActive) {
        s->fineShellFull = false;
        s->shellList(s->fine, false, &s->dShell, &s->shellCount);
    }
}

int fcfd_set_refined_finer_flags(fcfd_solver* s, const uint8_t* ff, size_t n) {
    if (!s || !s->initialized || !s->finerActive || !ff || n != static_cast<size_t>(s->finer.n))
        return cudaErrorInvalidValue;
    if (auto e = s->uploadLevelFlags(s->finer, ff); e != cudaSuccess) return e;
    if (auto e = finer_lists(s); e != 0) return e;
    if (auto e = s->buildWM(s->finer, kWallSampleFine); e != cudaSuccess) return e;
    return s->seedFiner();
}

int fcfd_set_refined_finer_surface_reference(fcfd_solver* s, const uint8_t* clean, size_t n) {
    if (!s || !s->initialized || !s->finerActive || !clean || n != static_cast<size_t>(s->finer.n))
        return cudaErrorInvalidValue;
    cudaStreamSynchronize(s->stream);
    assign_flags(s->finer.surfaceRef, clean, n);
    return s->buildWM(s->finer, kWallSampleFine);
}

int fcfd_finer_refinement_info(const fcfd_solver* s, fcfd_finer_info* r) {
    if (!s || !r) return cudaErrorInvalidValue;
    *r = fcfd_finer_info{};
    if (!s->finerActive) return 0;
    r->active = 1;
    r->factor = s->finerFactor;
    r->box = s->finerBox;
    r->dims = fcfd_dims{s->finer.d.nx, s->finer.d.ny, s->finer.d.nz};
    r->vram_bytes = 2.0 * 19.0 * static_cast<double>(s->finer.n) * (s->storage == Storage::F32 ? 4 : 2)
                  + 2.0 * static_cast<double>(s->finer.n);
    return 0;
}

int fcfd_import_finer_f32(fcfd_solver* s, const float* f, size_t count) {
    if (!s || !s->initialized || !s->finerActive || !f) return cudaErrorInvalidValue;
    return s->importF32(s->finer, f, count);
}

int fcfd_export_finer_f32(fcfd_solver* s, float* f, size_t count) {
    if (!s || !s->initialized || !s->finerActive || !f) return cudaErrorInvalidValue;
    return s->exportF32(s->finer, f, count);
}

int fcfd::solver_field_view(fcfd_solver* s, SolverFieldView* v) {
    if (!s || !s->initialized || !v) return cudaErrorNotReady;
    *v = SolverFieldView{};
    if (auto e = s->aaToAB(); e != cudaSuccess) return e;
    const size_t pop = s->storage == Storage::F32 ? 4 : 2;
    const Level* levels[3] = {&s->coarse, s->fineActive ? &s->fine : nullptr,
                                           s->finerActive ? &s->finer : nullptr};
    for (const auto* L : levels) {
        if (!L) break;
        const int l = v->levels;
        v->f[l] = L->f[L->src];
        v->bytes[l] = static_cast<size_t>(L->n) * 19 * pop;
        v->dims[l] = L->d;
        if (L->wm.active) {
            v->wm[l][0] = L->wm.dUTau;
            v->wmBytes[l][0] = static_cast<size_t>(L->wm.count) * 4;
            void* slip[3] = {L->wm.dUwx, L->wm.dUwy, L->wm.dUwz};
            for (int k = 0; k < 3; ++k) {
                v->wm[l][k + 1] = slip[k];
                v->wmBytes[l][k + 1] = static_cast<size_t>(L->n) * 2;
            }
        }
        ++v->levels;
    }
    v->storage = s->storage == Storage::F32 ? FCFD_STORE_FP32 : FCFD_STORE_FP16;
    v->stream = s->stream;
    // The flag hash is cached until the coarse flags change.
    if (!s->flagsHashValid) {
        s->flagsHashCache = fnv1a64(s->coarse.hostFlags.data(), s->coarse.hostFlags.size());
        s->flagsHashValid = true;
    }
    v->flagsHash = s->flagsHashCache;
    v->scaling = s->scaling;
    return 0;
}
