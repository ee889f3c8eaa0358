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

CUmodule gModule = nullptr;
CUfunction gCollide = nullptr, gGhost = nullptr;
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
