// ORACLE - measurement and test infrastructure only. Runs the reference's own
// CUDA solver-step kernels on this GPU through the driver API, in the
// reference's padded layout (one ghost z plane on each side): from
// src/sim/lbm_core.cu streamCollideKernel<WM, false>, refreshGhostZKernel,
// nanWatchdogKernel and forceReductionKernel<WM>; from lbm_refine.cu the
// coarse-to-fine fill and the restriction; from lbm_wallmodel.cu the
// wall-model update. Each is compiled unmodified from the reference tree into
// a cubin by ref_build.py (as the reference builds it, and once more without
// contraction). The kernels are found by name in the loaded modules; their
// parameter lists are the reference's (lbm_core.cu:214-226, 484-485, 526-530,
// 573-580; lbm_wallmodel.cu:76-84; lbm_wallmodel.cuh:47-82), restated here, and
// the launch sequence is the reference's stepN (lbm_solver.cpp:1132-1390).
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

namespace {

constexpr int kQ = 19;
constexpr int kBlock = 256;   // the reference's launch block (lbm_core.cu:37)

// Parameter structs of the kernel, field for field (lbm_core.cuh:201-225).
struct SlipViewArg {
    const std::uint16_t* uwx = nullptr;
    const std::uint16_t* uwy = nullptr;
    const std::uint16_t* uwz = nullptr;
};
struct QLinkViewArg {
    const std::uint8_t* qFrac = nullptr;
    const std::uint32_t* ffMask = nullptr;
};

// WallCellListView, WallModelParams, WallModelDeviceStats
// (lbm_wallmodel.cuh:47-82), field for field.
struct WallListArg {
    const long long* cellIdx = nullptr;
    const long long* sampleIdx = nullptr;
    const float* normalX = nullptr;
    const float* normalY = nullptr;
    const float* normalZ = nullptr;
    const float* sampleDist = nullptr;
    const std::uint32_t* linkMask = nullptr;
    float* uTau = nullptr;
    int count = 0;
};
struct WallParamsArg {
    float nuLat, utCutoff, emaAlpha;
};
struct WallStatsArg {
    float sumYplus;
    int maxYplusBits, activeCells, clampedCells;
};

constexpr long long kWatchdogStride = 4093;   // lbm_core.cu:524
constexpr int kWatchdogPeriod = 200;          // lbm_solver.cpp:25
constexpr float kWallEma = 0.25f;             // kWallModelEmaAlpha

CUmodule gModule = nullptr, gRefineModule = nullptr, gWallModule = nullptr;
CUfunction gCollide = nullptr, gCollideWM = nullptr, gGhost = nullptr;
CUfunction gWatchdog = nullptr, gForce = nullptr, gForceWM = nullptr;
CUfunction gFill = nullptr, gRestrict = nullptr, gWall = nullptr;
std::string gErr;

bool ok(CUresult r, const char* what) {
    if (r == CUDA_SUCCESS) return true;
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    gErr = std::string(what) + ": " + (s ? s : "?");
    return false;
}

} // namespace

extern "C" const char* refgpu_error() { return gErr.c_str(); }

// Unload every module (the next load may take another build variant).
extern "C" int refgpu_unload() {
    cudaDeviceSynchronize();
    for (CUmodule* m : {&gModule, &gRefineModule, &gWallModule})
        if (*m) {
            cuModuleUnload(*m);
            *m = nullptr;
        }
    gCollide = gCollideWM = gGhost = gWatchdog = gForce = gForceWM = nullptr;
    gFill = gRestrict = gWall = nullptr;
    return 0;
}

// Load the cubin and find the two kernels by their mangled names.
extern "C" int refgpu_load(const char* cubin) {
    if (gModule) return 0;
    cudaFree(nullptr);   // the runtime's primary context becomes current
    if (!ok(cuModuleLoad(&gModule, cubin), "cuModuleLoad")) return -1;
    unsigned count = 0;
    if (!ok(cuModuleGetFunctionCount(&count, gModule), "cuModuleGetFunctionCount")) return -1;
    std::vector<CUfunction> fns(count);
    if (count && !ok(cuModuleEnumerateFunctions(fns.data(), count, gModule), "cuModuleEnumerateFunctions"))
        return -1;
    for (CUfunction f : fns) {
        const char* name = nullptr;
        if (cuFuncGetName(&name, f) != CUDA_SUCCESS || !name) continue;
        const std::string n(name);
        // streamCollideKernel<false, false>: template arguments "ILb0ELb0E".
        if (n.find("streamCollideKernel") != std::string::npos && n.find("ILb0ELb0E") != std::string::npos)
            gCollide = f;
        if (n.find("streamCollideKernel") != std::string::npos && n.find("ILb1ELb0E") != std::string::npos)
            gCollideWM = f;
        if (n.find("refreshGhostZKernel") != std::string::npos) gGhost = f;
        if (n.find("nanWatchdogKernel") != std::string::npos) gWatchdog = f;
        // forceReductionKernel<WM>: "ILb0EE" / "ILb1EE".
        if (n.find("forceReductionKernel") != std::string::npos && n.find("ILb0E") != std::string::npos) gForce = f;
        if (n.find("forceReductionKernel") != std::string::npos && n.find("ILb1E") != std::string::npos) gForceWM = f;
    }
    if (!gCollide || !gGhost) {
        gErr = "reference kernels not found in the module";
        return -1;
    }
    return 0;
}

// Run `warmup` untimed and `steps` timed reference steps (stream-collide into
// the other buffer, then the ghost-plane refresh of that buffer) on an
// unpadded FP32 SoA state f (19 * n floats, n = nx*ny*nz) and CellFlag
// bytes; writes the final state back into f (unpadded) and the timed
// milliseconds. Every `batch`-th step writes the macroscopic fields, as the
// reference's stepN does on a batch's last step.
extern "C" int refgpu_run(int nx, int ny, int nz, const std::uint8_t* flags, float* f, float tau, float lambda,
                          float cs, float uIn, int warmup, int steps, int batch, double* ms, int bothBuffers) {
    if (!gCollide || !gGhost || nx < 3 || ny < 3 || nz < 1 || !flags || !f || steps < 1 || batch < 1) {
        gErr = "bad arguments or module not loaded";
        return -1;
    }
    const long long nxny = static_cast<long long>(nx) * ny, n = nxny * nz, npad = nxny * (nz + 2);
    // Slack past the padded buffers: diagonal pulls of the top row of the
    // last plane may reach nx cells beyond the high ghost plane.
    const long long slack = nxny + nx + 64;
    float *dA = nullptr, *dB = nullptr, *rho = nullptr, *u = nullptr, *v = nullptr, *w = nullptr;
    std::uint8_t* dFlags = nullptr;
    cudaError_t e = cudaMalloc(&dA, (kQ * npad + slack) * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&dB, (kQ * npad + slack) * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&dFlags, npad + slack);
    for (float** p : {&rho, &u, &v, &w})
        if (e == cudaSuccess) e = cudaMalloc(p, n * sizeof(float));
    auto cleanup = [&]() {
        for (void* p : {static_cast<void*>(dA), static_cast<void*>(dB), static_cast<void*>(dFlags),
                        static_cast<void*>(rho), static_cast<void*>(u), static_cast<void*>(v),
                        static_cast<void*>(w)})
            if (p) cudaFree(p);
    };
    if (e != cudaSuccess) {
        gErr = cudaGetErrorString(e);
        cleanup();
        return -1;
    }
    cudaMemset(dA, 0, (kQ * npad + slack) * sizeof(float));
    cudaMemset(dB, 0, (kQ * npad + slack) * sizeof(float));
    cudaMemset(dFlags, 1, npad + slack);   // slack reads see a solid flag
    // Padded planes: 0 <- z = nz-1, 1..nz <- z = 0..nz-1, nz+1 <- z = 0.
    std::vector<std::uint8_t> pf(static_cast<size_t>(npad));
    std::memcpy(pf.data() + nxny, flags, static_cast<size_t>(n));
    std::memcpy(pf.data(), flags + nxny * (nz - 1), static_cast<size_t>(nxny));
    std::memcpy(pf.data() + nxny * (nz + 1), flags, static_cast<size_t>(nxny));
    cudaMemcpy(dFlags, pf.data(), static_cast<size_t>(npad), cudaMemcpyHostToDevice);
    std::vector<float> pad(static_cast<size_t>(npad));
    for (int q = 0; q < kQ; ++q) {
        const float* src = f + q * n;
        std::memcpy(pad.data() + nxny, src, static_cast<size_t>(n) * sizeof(float));
        std::memcpy(pad.data(), src + nxny * (nz - 1), static_cast<size_t>(nxny) * sizeof(float));
        std::memcpy(pad.data() + nxny * (nz + 1), src, static_cast<size_t>(nxny) * sizeof(float));
        cudaMemcpy(dA + q * npad, pad.data(), static_cast<size_t>(npad) * sizeof(float), cudaMemcpyHostToDevice);
        // Cells a step never writes (slip planes) keep the other buffer's
        // contents; with bothBuffers the other buffer starts equal to f.
        if (bothBuffers)
            cudaMemcpy(dB + q * npad, pad.data(), static_cast<size_t>(npad) * sizeof(float), cudaMemcpyHostToDevice);
    }
    // launchStreamCollide's prefactor: 18 sqrt(2) Cs^2 (0 disables the LES term).
    const float smagPre = cs > 0.0f ? 18.0f * 1.41421356f * cs * cs : 0.0f;
    SlipViewArg slip;
    QLinkViewArg qlink;
    const unsigned gridC = static_cast<unsigned>((n + kBlock - 1) / kBlock);
    const unsigned gridG = static_cast<unsigned>((nxny * kQ + kBlock - 1) / kBlock);
    float* cur = dA;
    float* nxt = dB;
    auto step = [&](int writeMacro) -> bool {
        long long a_n = n, a_npad = npad, a_nxny = nxny;
        int a_nx = nx, a_wm = writeMacro;
        float a_tau = tau, a_lam = lambda, a_sp = smagPre, a_u = uIn;
        const float* a_src = cur;
        float* a_dst = nxt;
        const std::uint8_t* a_fl = dFlags;
        void* args[] = {&a_src, &a_dst, &a_fl, &rho, &u, &v, &w, &a_n, &a_npad, &a_nxny, &a_nx,
                        &a_tau, &a_lam, &a_sp, &a_u, &a_wm, &slip, &qlink};
        if (!ok(cuLaunchKernel(gCollide, gridC, 1, 1, kBlock, 1, 1, 0, nullptr, args, nullptr), "collide launch"))
            return false;
        int a_nz = nz;
        float* a_f = nxt;
        void* gargs[] = {&a_f, &a_nxny, &a_npad, &a_nz};
        if (!ok(cuLaunchKernel(gGhost, gridG, 1, 1, kBlock, 1, 1, 0, nullptr, gargs, nullptr), "ghost launch"))
            return false;
        std::swap(cur, nxt);
        return true;
    };
    bool good = true;
    for (int s = 0; s < warmup && good; ++s) good = step((s + 1) % batch == 0);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaDeviceSynchronize();
    cudaEventRecord(e0, nullptr);
    for (int s = 0; s < steps && good; ++s) good = step((s + 1) % batch == 0);
    cudaEventRecord(e1, nullptr);
    e = cudaEventSynchronize(e1);
    float t = 0.0f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (good && e == cudaSuccess) {
        for (int q = 0; q < kQ; ++q)
            cudaMemcpy(f + q * n, cur + q * npad + nxny, static_cast<size_t>(n) * sizeof(float),
                       cudaMemcpyDeviceToHost);
        e = cudaGetLastError();
    }
    cleanup();
    if (!good) return -1;
    if (e != cudaSuccess) {
        gErr = cudaGetErrorString(e);
        return -1;
    }
    *ms = t;
    return 0;
}

// Load the refinement cubin (src/sim/lbm_refine.cu) and find the fill and
// the restriction.
namespace {

bool load_module(CUmodule* mod, const char* cubin, const char* const* names, CUfunction* const* outs, int n) {
    if (*mod) return true;
    cudaFree(nullptr);
    if (!ok(cuModuleLoad(mod, cubin), "cuModuleLoad")) return false;
    unsigned count = 0;
    if (!ok(cuModuleGetFunctionCount(&count, *mod), "cuModuleGetFunctionCount")) return false;
    std::vector<CUfunction> fns(count);
    if (count && !ok(cuModuleEnumerateFunctions(fns.data(), count, *mod), "cuModuleEnumerateFunctions"))
        return false;
    for (CUfunction f : fns) {
        const char* name = nullptr;
        if (cuFuncGetName(&name, f) != CUDA_SUCCESS || !name) continue;
        const std::string s(name);
        for (int k = 0; k < n; ++k)
            if (s.find(names[k]) != std::string::npos) *outs[k] = f;
    }
    for (int k = 0; k < n; ++k)
        if (!*outs[k]) {
            gErr = std::string("reference kernel not found in the module: ") + names[k];
            return false;
        }
    return true;
}

} // namespace

extern "C" int refgpu_load_refine(const char* cubin) {
    const char* names[] = {"coarseToFineFillKernel", "fineToCoarseRestrictKernel"};
    CUfunction* outs[] = {&gFill, &gRestrict};
    return load_module(&gRefineModule, cubin, names, outs, 2) ? 0 : -1;
}

// Load the wall-model cubin (src/sim/lbm_wallmodel.cu).
extern "C" int refgpu_load_wall(const char* cubin) {
    const char* names[] = {"wallModelUpdateKernel"};
    CUfunction* outs[] = {&gWall};
    return load_module(&gWallModule, cubin, names, outs, 1) ? 0 : -1;
}

// ---- full reference step -----------------------------------------------------

/// One level of a run: flags, an optional initial state (both buffers), an
/// optional wall-cell list (the reference's SoA, unpadded indices), and
/// optional outputs.
struct RefLevelIn {
    int nx, ny, nz;
    const std::uint8_t* flags;
    const float* f0;             // unpadded FP32 SoA, both buffers; null: uniform feq(1, u_in)
    int wallCount;               // 0: no wall-model update on this level
    const long long* wallCell;
    const long long* wallSample;
    const float* wallNx;
    const float* wallNy;
    const float* wallNz;
    const float* wallYs;
    const std::uint32_t* wallMask;
    float* outF;                 // final current buffer (unpadded), or null
    float* outUTau;              // final u_tau (wallCount), or null
};

struct RefRunIn {
    RefLevelIn coarse, fine;
    int refined, bx0, by0, bx1, by1, factor;
    float tau, lambda, cs, uIn;
    int wm;         // WM collide/force instantiations (slip arrays on every level)
    int warmup, steps, batch;
    int forces;     // force reduction once per batch
    int watchdog;   // watchdog every 200 steps
    int wallReps;   // after the timed steps: back-to-back wall-model updates timed per level (0: none)
};

struct RefRunOut {
    double ms;
    long long tripStep;   // first step whose watchdog check read nonzero (0: none)
    int tripFlag;         // its verdict (1/2 coarse, 3/4 fine)
    int checks;           // watchdog checks run
    float force[3];       // the last batch's force (FP32, atomics)
    long long stepsRun;
    double wallMs[2];     // mean ms per wall-model update (stats reset + kernel), coarse / fine; 0: not timed
    double forceMs;       // mean ms per force reduction (accumulator reset + kernel) on the force level
};

namespace {

/// One level in the reference's padded layout.
struct PaddedLevel {
    int nx = 0, ny = 0, nz = 0;
    long long nxny = 0, n = 0, npad = 0;
    float* f[2] = {nullptr, nullptr};
    std::uint8_t* flags = nullptr;
    std::uint16_t* slip = nullptr;   // three half arrays, zero until the wall model writes them
    WallListArg wl;
    void* wallMem = nullptr;
    WallStatsArg* stats = nullptr;

    bool alloc(const RefLevelIn& in, float uIn, bool wm) {
        nx = in.nx; ny = in.ny; nz = in.nz;
        nxny = static_cast<long long>(nx) * ny;
        n = nxny * nz;
        npad = nxny * (nz + 2);
        const long long slack = nxny + nx + 64;
        for (float*& p : f)
            if (cudaMalloc(&p, (kQ * npad + slack) * sizeof(float)) != cudaSuccess) return false;
        if (cudaMalloc(&flags, npad + slack) != cudaSuccess) return false;
        if (wm && cudaMalloc(&slip, 3 * n * sizeof(std::uint16_t)) != cudaSuccess) return false;
        if (wm) cudaMemset(slip, 0, 3 * n * sizeof(std::uint16_t));
        cudaMemset(flags, 1, npad + slack);
        std::vector<std::uint8_t> pf(static_cast<size_t>(npad));
        std::memcpy(pf.data() + nxny, in.flags, static_cast<size_t>(n));
        std::memcpy(pf.data(), in.flags + nxny * (nz - 1), static_cast<size_t>(nxny));
        std::memcpy(pf.data() + nxny * (nz + 1), in.flags, static_cast<size_t>(nxny));
        cudaMemcpy(flags, pf.data(), static_cast<size_t>(npad), cudaMemcpyHostToDevice);
        for (float* p : f) cudaMemset(p, 0, (kQ * npad + slack) * sizeof(float));
        if (in.f0) {
            std::vector<float> pad(static_cast<size_t>(npad));
            for (int q = 0; q < kQ; ++q) {
                const float* src = in.f0 + q * n;
                std::memcpy(pad.data() + nxny, src, static_cast<size_t>(n) * sizeof(float));
                std::memcpy(pad.data(), src + nxny * (nz - 1), static_cast<size_t>(nxny) * sizeof(float));
                std::memcpy(pad.data() + nxny * (nz + 1), src, static_cast<size_t>(nxny) * sizeof(float));
                for (float* p : f)
                    cudaMemcpy(p + q * npad, pad.data(), static_cast<size_t>(npad) * sizeof(float),
                               cudaMemcpyHostToDevice);
            }
        } else {
            // feq(1, u_in, 0, 0) per direction, the reference's equilibrium19.
            static const int cxq[kQ] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0};
            const float usq = 1.5f * (uIn * uIn);
            for (int q = 0; q < kQ; ++q) {
                const float w = q == 0 ? 1.0f / 3.0f : (q <= 6 ? 1.0f / 18.0f : 1.0f / 36.0f);
                const float cu = 3.0f * (static_cast<float>(cxq[q]) * uIn);
                const float v = (w * 1.0f) * (1.0f + cu + 0.5f * cu * cu - usq);
                unsigned bits;
                std::memcpy(&bits, &v, 4);
                for (float* p : f)
                    if (cuMemsetD32(reinterpret_cast<CUdeviceptr>(p + q * npad), bits, static_cast<size_t>(npad))
                        != CUDA_SUCCESS)
                        return false;
            }
        }
        if (in.wallCount > 0) {
            const size_t c = static_cast<size_t>(in.wallCount);
            const size_t bytes = c * (2 * sizeof(long long) + 5 * sizeof(float) + sizeof(std::uint32_t)
                                      + sizeof(float)) + sizeof(WallStatsArg) + 256;
            if (cudaMalloc(&wallMem, bytes) != cudaSuccess) return false;
            char* b = static_cast<char*>(wallMem);
            auto put = [&](const void* h, size_t sz) {
                void* d = b;
                if (h) cudaMemcpy(d, h, sz, cudaMemcpyHostToDevice);
                else cudaMemset(d, 0, sz);
                b += (sz + 15) & ~static_cast<size_t>(15);
                return d;
            };
            wl.cellIdx = static_cast<const long long*>(put(in.wallCell, c * 8));
            wl.sampleIdx = static_cast<const long long*>(put(in.wallSample, c * 8));
            wl.normalX = static_cast<const float*>(put(in.wallNx, c * 4));
            wl.normalY = static_cast<const float*>(put(in.wallNy, c * 4));
            wl.normalZ = static_cast<const float*>(put(in.wallNz, c * 4));
            wl.sampleDist = static_cast<const float*>(put(in.wallYs, c * 4));
            wl.linkMask = static_cast<const std::uint32_t*>(put(in.wallMask, c * 4));
            wl.uTau = static_cast<float*>(put(nullptr, c * 4));   // fresh seeds (u_tau = 0)
            stats = static_cast<WallStatsArg*>(put(nullptr, sizeof(WallStatsArg)));
            wl.count = in.wallCount;
        }
        return true;
    }
    void release() {
        for (float*& p : f) { if (p) cudaFree(p); p = nullptr; }
        if (flags) cudaFree(flags);
        if (slip) cudaFree(slip);
        if (wallMem) cudaFree(wallMem);
        flags = nullptr; slip = nullptr; wallMem = nullptr;
    }
};

bool launch_collide(CUfunction fn, const PaddedLevel& L, const float* src, float* dst, float* rho, float* u,
                    float* v, float* w, float tau, float lambda, float smagPre, float uIn, int writeMacro) {
    long long a_n = L.n, a_npad = L.npad, a_nxny = L.nxny;
    int a_nx = L.nx, a_wm = writeMacro;
    float a_tau = tau, a_lam = lambda, a_sp = smagPre, a_u = uIn;
    const float* a_src = src;
    float* a_dst = dst;
    const std::uint8_t* a_fl = L.flags;
    SlipViewArg slip;
    if (L.slip) { slip.uwx = L.slip; slip.uwy = L.slip + L.n; slip.uwz = L.slip + 2 * L.n; }
    QLinkViewArg qlink;
    void* args[] = {&a_src, &a_dst, &a_fl, &rho, &u, &v, &w, &a_n, &a_npad, &a_nxny, &a_nx,
                    &a_tau, &a_lam, &a_sp, &a_u, &a_wm, &slip, &qlink};
    const unsigned grid = static_cast<unsigned>((L.n + kBlock - 1) / kBlock);
    return ok(cuLaunchKernel(fn, grid, 1, 1, kBlock, 1, 1, 0, nullptr, args, nullptr), "collide launch");
}

bool launch_ghost(const PaddedLevel& L, float* f) {
    long long a_nxny = L.nxny, a_npad = L.npad;
    int a_nz = L.nz;
    void* args[] = {&f, &a_nxny, &a_npad, &a_nz};
    const unsigned grid = static_cast<unsigned>((L.nxny * kQ + kBlock - 1) / kBlock);
    return ok(cuLaunchKernel(gGhost, grid, 1, 1, kBlock, 1, 1, 0, nullptr, args, nullptr), "ghost launch");
}

/// launchNaNWatchdog (lbm_core.cu:856-870): the strided sample of `f`.
bool launch_watchdog(const PaddedLevel& L, const float* f, long long sampleOffset, int* flag, int flagBase) {
    long long a_off = ((sampleOffset % kWatchdogStride) + kWatchdogStride) % kWatchdogStride;
    long long a_n = L.n, a_npad = L.npad, a_nxny = L.nxny;
    int a_base = flagBase;
    const float* a_f = f;
    void* args[] = {&a_f, &a_n, &a_npad, &a_nxny, &a_off, &flag, &a_base};
    const long long samples = (L.n + kWatchdogStride - 1) / kWatchdogStride;
    const unsigned grid = static_cast<unsigned>((samples + kBlock - 1) / kBlock);
    return ok(cuLaunchKernel(gWatchdog, grid, 1, 1, kBlock, 1, 1, 0, nullptr, args, nullptr), "watchdog launch");
}

/// launchForceReduction (lbm_core.cu:880-901): zero the accumulator, reduce.
bool launch_force(const PaddedLevel& L, const float* f, float* acc) {
    if (cudaMemsetAsync(acc, 0, 3 * sizeof(float), nullptr) != cudaSuccess) return false;
    long long a_n = L.n, a_npad = L.npad, a_nxny = L.nxny;
    int a_nx = L.nx;
    const float* a_f = f;
    const std::uint8_t* a_fl = L.flags;
    SlipViewArg slip;
    if (L.slip) { slip.uwx = L.slip; slip.uwy = L.slip + L.n; slip.uwz = L.slip + 2 * L.n; }
    void* args[] = {&a_f, &a_fl, &a_n, &a_npad, &a_nxny, &a_nx, &acc, &slip};
    const unsigned grid = static_cast<unsigned>((L.n + kBlock - 1) / kBlock);
    return ok(cuLaunchKernel(L.slip ? gForceWM : gForce, grid, 1, 1, kBlock, 1, 1, 0, nullptr, args, nullptr),
              "force launch");
}

/// launchWallModelUpdate (lbm_wallmodel.cu:200-225).
bool launch_wall(PaddedLevel& L, const float* f, float nuLat, float utCutoff) {
    if (L.wl.count <= 0) return true;
    if (cudaMemsetAsync(L.stats, 0, sizeof(WallStatsArg), nullptr) != cudaSuccess) return false;
    WallListArg a_list = L.wl;
    const float* a_f = f;
    long long a_npad = L.npad, a_nxny = L.nxny;
    std::uint16_t *a_x = L.slip, *a_y = L.slip + L.n, *a_z = L.slip + 2 * L.n;
    WallParamsArg a_p{nuLat, utCutoff, kWallEma};
    WallStatsArg* a_s = L.stats;
    void* args[] = {&a_list, &a_f, &a_npad, &a_nxny, &a_x, &a_y, &a_z, &a_p, &a_s};
    const unsigned grid = static_cast<unsigned>((L.wl.count + kBlock - 1) / kBlock);
    return ok(cuLaunchKernel(gWall, grid, 1, 1, kBlock, 1, 1, 0, nullptr, args, nullptr), "wall launch");
}

} // namespace

// The reference's stepN (lbm_solver.cpp:1132-1390) in batches of `batch`
// steps: per step the coarse collide + ghost refresh; with the patch, m
// times the fill of the fine shell at weight half/m, ghost refresh, fine
// collide, ghost refresh, then the restriction + coarse ghost refresh; the
// watchdog every 200 steps (coarse flagBase 0, fine 2, offset steps * 977).
// Per batch, after its steps: the force reduction (fine level when present,
// the reference's forcesFromFine) and the wall-model updates of the levels
// with a list. Times `steps` after `warmup` (both rounded up to whole
// batches is NOT done: a partial last batch is a shorter stepN call).
extern "C" int refgpu_run_full(const RefRunIn* in, RefRunOut* out) {
    if (!in || !out) return -1;
    *out = RefRunOut{};
    const bool refined = in->refined != 0;
    const bool wm = in->wm != 0;
    CUfunction collide = wm ? gCollideWM : gCollide;
    const bool needWall = in->coarse.wallCount > 0 || (refined && in->fine.wallCount > 0);
    if (!collide || !gGhost || (refined && (!gFill || !gRestrict)) || (needWall && (!gWall || !wm))
        || (in->watchdog && !gWatchdog) || (in->forces && !(wm ? gForceWM : gForce)) || in->steps < 1
        || in->batch < 1 || in->warmup < 0 || !in->coarse.flags || (refined && !in->fine.flags)) {
        gErr = "bad arguments or modules not loaded";
        return -1;
    }
    const int m = in->factor;
    if (refined && (m < 2 || in->fine.nx != m * (in->bx1 - in->bx0) || in->fine.ny != m * (in->by1 - in->by0)
                    || in->fine.nz != m * in->coarse.nz || in->bx0 < 3 || in->by0 < 3
                    || in->bx1 > in->coarse.nx - 3 || in->by1 > in->coarse.ny - 3)) {
        gErr = "patch dims do not match the box";
        return -1;
    }
    PaddedLevel C, F;
    float *rho = nullptr, *u = nullptr, *v = nullptr, *w = nullptr, *dForce = nullptr;
    int* dTrips = nullptr;
    const long long total = static_cast<long long>(in->warmup) + in->steps;
    const int maxChecks = static_cast<int>(total / kWatchdogPeriod) + 1;
    bool good = C.alloc(in->coarse, in->uIn, wm) && (!refined || F.alloc(in->fine, in->uIn, wm));
    for (float** p : {&rho, &u, &v, &w})
        if (good) good = cudaMalloc(p, C.n * sizeof(float)) == cudaSuccess;
    if (good) good = cudaMalloc(&dForce, 3 * sizeof(float)) == cudaSuccess;
    if (good) good = cudaMalloc(&dTrips, maxChecks * sizeof(int)) == cudaSuccess;
    if (good) good = cudaMemset(dTrips, 0, maxChecks * sizeof(int)) == cudaSuccess;
    auto cleanup = [&]() {
        C.release();
        F.release();
        for (float* p : {rho, u, v, w, dForce}) if (p) cudaFree(p);
        if (dTrips) cudaFree(dTrips);
    };
    if (!good) {
        if (gErr.empty()) gErr = "allocation failed";
        cleanup();
        return -1;
    }
    const float smagPre = in->cs > 0.0f ? 18.0f * 1.41421356f * in->cs * in->cs : 0.0f;
    const float tau = in->tau, lambda = in->lambda, uIn = in->uIn;
    const float tauF = static_cast<float>(m) * (tau - 0.5f) + 0.5f;   // fineTauFor
    const float neqScale = tauF / (static_cast<float>(m) * tau);
    const float neqScaleInv = (static_cast<float>(m) * tau) / tauF;
    const int rx0 = in->bx0 + 2, ry0 = in->by0 + 2, rx1 = in->bx1 - 2, ry1 = in->by1 - 2;   // kRestrictBandCoarse
    int cs_ = 0, fs = 0;
    long long steps = 0;
    int checks = 0, sinceWatchdog = 0;
    auto step = [&](int writeMacro) -> bool {
        if (!launch_collide(collide, C, C.f[cs_], C.f[1 - cs_], rho, u, v, w, tau, lambda, smagPre, uIn, writeMacro))
            return false;
        if (!launch_ghost(C, C.f[1 - cs_])) return false;
        if (refined) {
            for (int half = 0; half < m; ++half) {
                const float* a_t0 = C.f[cs_];
                const float* a_t1 = C.f[1 - cs_];
                const std::uint8_t* a_cfl = C.flags;
                const std::uint8_t* a_ffl = F.flags;
                float* a_ff = F.f[fs];
                long long a_fn = F.n, a_fnxny = F.nxny, a_fnpad = F.npad, a_cnxny = C.nxny, a_cnpad = C.npad;
                int a_fnx = F.nx, a_fny = F.ny, a_cnx = C.nx, a_cnz = C.nz, a_bx0 = in->bx0, a_by0 = in->by0,
                    a_full = 0;
                float a_inv = 1.0f / static_cast<float>(m);
                float a_tw = static_cast<float>(half) / static_cast<float>(m), a_neq = neqScale;
                void* fargs[] = {&a_t0, &a_t1, &a_cfl, &a_ffl, &a_ff, &a_fn, &a_fnxny, &a_fnpad, &a_fnx, &a_fny,
                                 &a_cnxny, &a_cnpad, &a_cnx, &a_cnz, &a_bx0, &a_by0, &a_inv, &a_tw, &a_neq, &a_full};
                const unsigned fgrid = static_cast<unsigned>((F.n + kBlock - 1) / kBlock);
                if (!ok(cuLaunchKernel(gFill, fgrid, 1, 1, kBlock, 1, 1, 0, nullptr, fargs, nullptr), "fill launch"))
                    return false;
                if (!launch_ghost(F, F.f[fs])) return false;
                if (!launch_collide(collide, F, F.f[fs], F.f[1 - fs], nullptr, nullptr, nullptr, nullptr, tauF, lambda,
                                    smagPre, uIn, 0))
                    return false;
                if (!launch_ghost(F, F.f[1 - fs])) return false;
                fs = 1 - fs;
            }
            const float* a_ff = F.f[fs];
            const std::uint8_t* a_ffl = F.flags;
            float* a_fc = C.f[1 - cs_];
            const std::uint8_t* a_cfl = C.flags;
            long long a_fnxny = F.nxny, a_fnpad = F.npad, a_cnxny = C.nxny, a_cnpad = C.npad;
            int a_fnx = F.nx, a_cnx = C.nx, a_cnz = C.nz, a_rx0 = rx0, a_ry0 = ry0, a_rx1 = rx1, a_ry1 = ry1;
            int a_bx0 = in->bx0, a_by0 = in->by0, a_m = m, a_wm = writeMacro;
            float a_inv = neqScaleInv;
            void* rargs[] = {&a_ff, &a_ffl, &a_fc, &a_cfl, &a_fnxny, &a_fnpad, &a_fnx, &a_cnxny, &a_cnpad, &a_cnx,
                             &a_cnz, &a_rx0, &a_ry0, &a_rx1, &a_ry1, &a_bx0, &a_by0, &a_m, &a_inv,
                             &rho, &u, &v, &w, &a_wm};
            const long long rtotal = static_cast<long long>(rx1 - rx0) * (ry1 - ry0) * C.nz;
            const unsigned rgrid = static_cast<unsigned>((rtotal + kBlock - 1) / kBlock);
            if (!ok(cuLaunchKernel(gRestrict, rgrid, 1, 1, kBlock, 1, 1, 0, nullptr, rargs, nullptr),
                    "restrict launch"))
                return false;
            if (!launch_ghost(C, C.f[1 - cs_])) return false;
        }
        cs_ = 1 - cs_;
        ++steps;
        if (in->watchdog && ++sinceWatchdog >= kWatchdogPeriod && checks < maxChecks) {
            sinceWatchdog = 0;
            int* flag = dTrips + checks++;
            if (!launch_watchdog(C, C.f[cs_], steps * 977, flag, 0)) return false;
            if (refined && !launch_watchdog(F, F.f[fs], steps * 977, flag, 2)) return false;
        }
        return true;
    };
    auto batchEnd = [&]() -> bool {
        if (in->forces && !launch_force(refined ? F : C, refined ? F.f[fs] : C.f[cs_], dForce)) return false;
        const float utCut = 1e-3f * uIn;
        if (C.wl.count > 0 && !launch_wall(C, C.f[cs_], (tau - 0.5f) / 3.0f, utCut)) return false;
        if (refined && F.wl.count > 0 && !launch_wall(F, F.f[fs], (tauF - 0.5f) / 3.0f, utCut)) return false;
        return true;
    };
    // stepN(n) calls of `batch` steps; macroscopic fields on each call's last step.
    auto run = [&](long long count) -> bool {
        for (long long done = 0; done < count && good;) {
            const long long nb = count - done < in->batch ? count - done : in->batch;
            for (long long i = 0; i < nb && good; ++i) good = step(i == nb - 1);
            if (good) good = batchEnd();
            done += nb;
        }
        return good;
    };
    run(in->warmup);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaDeviceSynchronize();
    cudaEventRecord(e0, nullptr);
    run(in->steps);
    cudaEventRecord(e1, nullptr);
    cudaError_t e = cudaEventSynchronize(e1);
    float t = 0.0f;
    cudaEventElapsedTime(&t, e0, e1);
    // The wall-model update alone, on the state the timed steps left: each
    // level's launchWallModelUpdate `wallReps` times back to back.
    if (good && e == cudaSuccess && in->wallReps > 0) {
        const float utCut = 1e-3f * uIn;
        PaddedLevel* pl[2] = {&C, &F};
        const int cur[2] = {cs_, fs};
        const float nu[2] = {(tau - 0.5f) / 3.0f, (tauF - 0.5f) / 3.0f};
        for (int k = 0; k < (refined ? 2 : 1) && good; ++k) {
            if (pl[k]->wl.count <= 0) continue;
            good = launch_wall(*pl[k], pl[k]->f[cur[k]], nu[k], utCut);   // warm
            cudaEventRecord(e0, nullptr);
            for (int r = 0; r < in->wallReps && good; ++r)
                good = launch_wall(*pl[k], pl[k]->f[cur[k]], nu[k], utCut);
            cudaEventRecord(e1, nullptr);
            e = cudaEventSynchronize(e1);
            float tw = 0.0f;
            cudaEventElapsedTime(&tw, e0, e1);
            if (e != cudaSuccess) break;
            out->wallMs[k] = static_cast<double>(tw) / in->wallReps;
        }
        // The force reduction alone on the level forces come from.
        if (good && e == cudaSuccess && in->forces) {
            PaddedLevel& FL = refined ? F : C;
            const float* ff = refined ? F.f[fs] : C.f[cs_];
            good = launch_force(FL, ff, dForce);   // warm
            cudaEventRecord(e0, nullptr);
            for (int r = 0; r < in->wallReps && good; ++r) good = launch_force(FL, ff, dForce);
            cudaEventRecord(e1, nullptr);
            e = cudaEventSynchronize(e1);
            float tf = 0.0f;
            cudaEventElapsedTime(&tf, e0, e1);
            if (e == cudaSuccess) out->forceMs = static_cast<double>(tf) / in->wallReps;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (good && e == cudaSuccess) {
        std::vector<int> trips(static_cast<size_t>(maxChecks));
        cudaMemcpy(trips.data(), dTrips, maxChecks * sizeof(int), cudaMemcpyDeviceToHost);
        for (int k = 0; k < checks; ++k)
            if (trips[static_cast<size_t>(k)] != 0) {
                out->tripStep = static_cast<long long>(k + 1) * kWatchdogPeriod;
                out->tripFlag = trips[static_cast<size_t>(k)];
                break;
            }
        cudaMemcpy(out->force, dForce, 3 * sizeof(float), cudaMemcpyDeviceToHost);
        const RefLevelIn* lv[2] = {&in->coarse, &in->fine};
        PaddedLevel* pl[2] = {&C, &F};
        const int cur[2] = {cs_, fs};
        for (int k = 0; k < (refined ? 2 : 1); ++k) {
            if (lv[k]->outF)
                for (int q = 0; q < kQ; ++q)
                    cudaMemcpy(lv[k]->outF + q * pl[k]->n, pl[k]->f[cur[k]] + q * pl[k]->npad + pl[k]->nxny,
                               static_cast<size_t>(pl[k]->n) * sizeof(float), cudaMemcpyDeviceToHost);
            if (lv[k]->outUTau && pl[k]->wl.count > 0)
                cudaMemcpy(lv[k]->outUTau, pl[k]->wl.uTau, static_cast<size_t>(pl[k]->wl.count) * sizeof(float),
                           cudaMemcpyDeviceToHost);
        }
        e = cudaGetLastError();
    }
    out->checks = checks;
    out->stepsRun = steps;
    cleanup();
    if (!good) return -1;
    if (e != cudaSuccess) {
        gErr = cudaGetErrorString(e);
        return -1;
    }
    out->ms = t;
    return 0;
}
