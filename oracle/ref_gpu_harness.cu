// ORACLE - measurement infrastructure only. Runs the reference's own CUDA
// stream-collide kernel (src/sim/lbm_core.cu: streamCollideKernel<false,
// false> and refreshGhostZKernel, compiled unmodified from the reference tree
// into a cubin by ref_build.py) on this GPU through the driver API, in the
// reference's padded layout (one ghost z plane on each side), so its speed can
// be timed beside this library's kernel on the same hardware and inputs. The
// kernels are found by name in the loaded module; their parameter lists are
// the reference's (lbm_core.cu:214-226, 484-485), restated here.
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

CUmodule gModule = nullptr, gRefineModule = nullptr;
CUfunction gCollide = nullptr, gCollideWM = nullptr, gGhost = nullptr;
CUfunction gFill = nullptr, gRestrict = nullptr;
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
                          float cs, float uIn, int warmup, int steps, int batch, double* ms) {
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
extern "C" int refgpu_load_refine(const char* cubin) {
    if (gRefineModule) return 0;
    cudaFree(nullptr);
    if (!ok(cuModuleLoad(&gRefineModule, cubin), "cuModuleLoad")) return -1;
    unsigned count = 0;
    if (!ok(cuModuleGetFunctionCount(&count, gRefineModule), "cuModuleGetFunctionCount")) return -1;
    std::vector<CUfunction> fns(count);
    if (count && !ok(cuModuleEnumerateFunctions(fns.data(), count, gRefineModule), "cuModuleEnumerateFunctions"))
        return -1;
    for (CUfunction f : fns) {
        const char* name = nullptr;
        if (cuFuncGetName(&name, f) != CUDA_SUCCESS || !name) continue;
        const std::string n(name);
        if (n.find("coarseToFineFillKernel") != std::string::npos) gFill = f;
        if (n.find("fineToCoarseRestrictKernel") != std::string::npos) gRestrict = f;
    }
    if (!gFill || !gRestrict) {
        gErr = "reference refinement kernels not found in the module";
        return -1;
    }
    return 0;
}

namespace {

/// One level in the reference's padded layout, initialised to the uniform
/// equilibrium feq(1, u_in) (a constant per direction).
struct PaddedLevel {
    int nx = 0, ny = 0, nz = 0;
    long long nxny = 0, n = 0, npad = 0;
    float* f[2] = {nullptr, nullptr};
    std::uint8_t* flags = nullptr;
    std::uint16_t* slip = nullptr;   // three zero half arrays (wall model on, no slip yet)

    bool alloc(int x, int y, int z, const std::uint8_t* hostFlags, float uIn, bool wm) {
        nx = x; ny = y; nz = z;
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
        std::memcpy(pf.data() + nxny, hostFlags, static_cast<size_t>(n));
        std::memcpy(pf.data(), hostFlags + nxny * (nz - 1), static_cast<size_t>(nxny));
        std::memcpy(pf.data() + nxny * (nz + 1), hostFlags, static_cast<size_t>(nxny));
        cudaMemcpy(flags, pf.data(), static_cast<size_t>(npad), cudaMemcpyHostToDevice);
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
        return true;
    }
    void release() {
        for (float*& p : f) { if (p) cudaFree(p); p = nullptr; }
        if (flags) cudaFree(flags);
        if (slip) cudaFree(slip);
        flags = nullptr; slip = nullptr;
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

} // namespace

// The reference's refined step (lbm_solver.cpp:1140-1291) with one 2:1 (or
// m:1) patch: coarse collide + ghost refresh; m times fill the fine shell
// from the coarse pair at weight half/m, ghost refresh, fine collide, ghost
// refresh; restriction into the new coarse buffer + ghost refresh. Uniform
// equilibrium start; wall model on (zero slip arrays) or off. Times `steps`
// coarse steps after `warmup`; macroscopic fields on every batch's last step.
extern "C" int refgpu_run_refined(int cnx, int cny, int cnz, const std::uint8_t* cflags, int fnx, int fny, int fnz,
                                  const std::uint8_t* fflags, int bx0, int by0, int bx1, int by1, int factor,
                                  float tau, float lambda, float cs, float uIn, int wm, int warmup, int steps,
                                  int batch, double* ms, float* outC, float* outF) {
    CUfunction collide = wm ? gCollideWM : gCollide;
    if (!collide || !gGhost || !gFill || !gRestrict || factor < 2 || steps < 1 || batch < 1 || !cflags || !fflags) {
        gErr = "bad arguments or modules not loaded";
        return -1;
    }
    if (fnx != factor * (bx1 - bx0) || fny != factor * (by1 - by0) || fnz != factor * cnz || bx0 < 3 || by0 < 3
        || bx1 > cnx - 3 || by1 > cny - 3) {
        gErr = "patch dims do not match the box";
        return -1;
    }
    PaddedLevel C, F;
    float *rho = nullptr, *u = nullptr, *v = nullptr, *w = nullptr;
    bool good = C.alloc(cnx, cny, cnz, cflags, uIn, wm != 0) && F.alloc(fnx, fny, fnz, fflags, uIn, wm != 0);
    for (float** p : {&rho, &u, &v, &w})
        if (good) good = cudaMalloc(p, C.n * sizeof(float)) == cudaSuccess;
    if (!good) {
        if (gErr.empty()) gErr = "allocation failed";
        C.release(); F.release();
        for (float* p : {rho, u, v, w}) if (p) cudaFree(p);
        return -1;
    }
    const float smagPre = cs > 0.0f ? 18.0f * 1.41421356f * cs * cs : 0.0f;
    const float tauF = static_cast<float>(factor) * (tau - 0.5f) + 0.5f;   // fineTauFor
    const float neqScale = tauF / (static_cast<float>(factor) * tau);
    const float neqScaleInv = (static_cast<float>(factor) * tau) / tauF;
    const int rx0 = bx0 + 2, ry0 = by0 + 2, rx1 = bx1 - 2, ry1 = by1 - 2;   // kRestrictBandCoarse
    int cs_ = 0, fs = 0;
    auto step = [&](int writeMacro) -> bool {
        if (!launch_collide(collide, C, C.f[cs_], C.f[1 - cs_], rho, u, v, w, tau, lambda, smagPre, uIn, writeMacro))
            return false;
        if (!launch_ghost(C, C.f[1 - cs_])) return false;
        for (int half = 0; half < factor; ++half) {
            const float* a_t0 = C.f[cs_];
            const float* a_t1 = C.f[1 - cs_];
            const std::uint8_t* a_cfl = C.flags;
            const std::uint8_t* a_ffl = F.flags;
            float* a_ff = F.f[fs];
            long long a_fn = F.n, a_fnxny = F.nxny, a_fnpad = F.npad, a_cnxny = C.nxny, a_cnpad = C.npad;
            int a_fnx = F.nx, a_fny = F.ny, a_cnx = C.nx, a_cnz = C.nz, a_bx0 = bx0, a_by0 = by0, a_full = 0;
            float a_inv = 1.0f / static_cast<float>(factor);
            float a_tw = static_cast<float>(half) / static_cast<float>(factor), a_neq = neqScale;
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
        int a_bx0 = bx0, a_by0 = by0, a_m = factor, a_wm = writeMacro;
        float a_inv = neqScaleInv;
        void* rargs[] = {&a_ff, &a_ffl, &a_fc, &a_cfl, &a_fnxny, &a_fnpad, &a_fnx, &a_cnxny, &a_cnpad, &a_cnx,
                         &a_cnz, &a_rx0, &a_ry0, &a_rx1, &a_ry1, &a_bx0, &a_by0, &a_m, &a_inv,
                         &rho, &u, &v, &w, &a_wm};
        const long long total = static_cast<long long>(rx1 - rx0) * (ry1 - ry0) * cnz;
        const unsigned rgrid = static_cast<unsigned>((total + kBlock - 1) / kBlock);
        if (!ok(cuLaunchKernel(gRestrict, rgrid, 1, 1, kBlock, 1, 1, 0, nullptr, rargs, nullptr), "restrict launch"))
            return false;
        if (!launch_ghost(C, C.f[1 - cs_])) return false;
        cs_ = 1 - cs_;
        return true;
    };
    for (int s = 0; s < warmup && good; ++s) good = step((s + 1) % batch == 0);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaDeviceSynchronize();
    cudaEventRecord(e0, nullptr);
    for (int s = 0; s < steps && good; ++s) good = step((s + 1) % batch == 0);
    cudaEventRecord(e1, nullptr);
    cudaError_t e = cudaEventSynchronize(e1);
    float t = 0.0f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    // Final states (unpadded FP32 SoA) when asked for.
    if (good && e == cudaSuccess) {
        for (int q = 0; q < kQ && outC; ++q)
            cudaMemcpy(outC + q * C.n, C.f[cs_] + q * C.npad + C.nxny, static_cast<size_t>(C.n) * sizeof(float),
                       cudaMemcpyDeviceToHost);
        for (int q = 0; q < kQ && outF; ++q)
            cudaMemcpy(outF + q * F.n, F.f[fs] + q * F.npad + F.nxny, static_cast<size_t>(F.n) * sizeof(float),
                       cudaMemcpyDeviceToHost);
        e = cudaGetLastError();
    }
    C.release(); F.release();
    for (float* p : {rho, u, v, w}) if (p) cudaFree(p);
    if (!good) return -1;
    if (e != cudaSuccess) {
        gErr = cudaGetErrorString(e);
        return -1;
    }
    *ms = t;
    return 0;
}

