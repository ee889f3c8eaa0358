// Learned u_tau seed: the network object, its GPU training (forward/backward
// and Adam kernels), inference, and the batched u_tau solves by each method
// (the reference's 6-iteration FP32 Newton, full FP64 Newton, the learned
// seed + one correction). Extends the reference's wall model
// (src/sim/lbm_wallmodel.cu:31-196), which has no learned part.
//
// Training: one thread per sample runs the forward pass (BF16 weights,
// FP32 arithmetic) and back-propagates the squared error of the normalised
// log u_tau; the per-sample activations and deltas go to shared memory, and
// the block then reduces them into its partial gradient (one entry per
// thread-pass, samples summed in a fixed order). The last block of the launch
// to finish sums the block partials in block order -- training is
// deterministic for a given seed -- updates the FP32 master weights (Adam)
// and rounds them to BF16 for the next step: one launch per training step. The network is ~2.3 kFLOP per sample: CUDA-core FP32 FMAs from
// shared-memory weights; a 2M-sample epoch is a fraction of a millisecond of
// arithmetic, so the training is launch-bound, not FLOP-bound.
#include "../../include/foilcfd_wallnet.h"
#include "kernels.h"
#include "wallnet.cuh"

#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

using namespace fcfd;
using namespace fcfd::wallnet;

namespace {

constexpr int kTrainBlock = 64;            // samples per training block
constexpr int kMaxTrainBlocks = 1024;      // => at most 65,536 samples per step
constexpr int kPartialStride = kParams + 1; // gradient + loss
constexpr int kSolveBlock = 128;
constexpr int kRowPad = kH + 1;            // shared rows padded against bank conflicts

std::uint16_t f32_to_bf16_bits(float f) {
    std::uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) return static_cast<std::uint16_t>((u >> 16) | ((u & 0xffffu) ? 0x40u : 0u));
    const std::uint32_t lsb = (u >> 16) & 1u;
    u += 0x7fffu + lsb;  // round to nearest even
    return static_cast<std::uint16_t>(u >> 16);
}
float bf16_bits_to_f32_host(std::uint16_t b) {
    const std::uint32_t u = static_cast<std::uint32_t>(b) << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

__device__ __forceinline__ std::uint16_t f32_to_bf16_dev(float f) {
    return __bfloat16_as_ushort(__float2bfloat16_rn(f));
}

// ---- training ----------------------------------------------------------------

struct SampleView {
    const float* ut;
    const float* ys;
    const float* nu;
    const float* tau;
    unsigned long long n;
};

/// Adam hyper-parameters of one step (bias corrections bc1 = 1 - beta1^t,
/// bc2 = 1 - beta2^t precomputed on the host).
struct AdamStep {
    float* master = nullptr;
    float* m = nullptr;
    float* v = nullptr;
    float lr = 0.0f, beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f, bc1 = 1.0f, bc2 = 1.0f;
    float* lossOut = nullptr;      // nullable: the step's mean loss
    unsigned* ticket = nullptr;    // block-completion counter, zero between steps
};

/// Adam update of parameter p from the block partials, summed in block order.
__device__ __forceinline__ void adam_update(const float* __restrict__ partials, int nb, int p, const AdamStep& a,
                                            float invCount, std::uint16_t* __restrict__ wbf) {
    float g = 0.0f;
    for (int b = 0; b < nb; ++b) g += __ldcg(partials + static_cast<size_t>(b) * kPartialStride + p);
    if (p == kParams) {
        if (a.lossOut) *a.lossOut = g * invCount;
        return;
    }
    const float mm = a.beta1 * a.m[p] + (1.0f - a.beta1) * g;
    const float vv = a.beta2 * a.v[p] + (1.0f - a.beta2) * g * g;
    a.m[p] = mm;
    a.v[p] = vv;
    const float w = a.master[p] - a.lr * (mm / a.bc1) / (sqrtf(vv / a.bc2) + a.eps);
    a.master[p] = w;
    wbf[p] = f32_to_bf16_dev(w);
}

/// Forward + backward of one block of samples; writes the block's partial
/// gradient (sum over its samples of dL/dp, L = invCount * sum err^2) and
/// partial loss (sum err^2) to partials[blockIdx.x]. With ADAM, the block
/// that finishes last (ticket counter) then sums all partials in block order
/// and applies the Adam step, so one launch is one training step and the
/// result does not depend on block scheduling.
template <bool ADAM>
__global__ void __launch_bounds__(kTrainBlock)
grad_kernel(std::uint16_t* __restrict__ wbf, Norm nm, SampleView S, unsigned long long permA,
            unsigned long long permC, unsigned long long pos0, int count, float invCount,
            float* __restrict__ partials, AdamStep adam) {
    __shared__ float P[kParams];
    __shared__ float h1s[kTrainBlock][kRowPad];
    __shared__ float h2s[kTrainBlock][kRowPad];
    __shared__ float dz1s[kTrainBlock][kRowPad];
    __shared__ float dz2s[kTrainBlock][kRowPad];
    __shared__ float xs[kTrainBlock][4];
    __shared__ float dys[kTrainBlock];
    __shared__ float errs[kTrainBlock];
    load_params(wbf, P);
    __syncthreads();

    const int t = threadIdx.x;
    const int local = blockIdx.x * kTrainBlock + t;
    const bool valid = local < count;
    float x0 = 0.0f, x1 = 0.0f, x2 = 0.0f, tn = 0.0f;
    if (valid) {
        const unsigned long long idx = (permA * (pos0 + static_cast<unsigned long long>(local)) + permC) % S.n;
        const float ut = S.ut[idx], ys = S.ys[idx], nu = S.nu[idx], tau = S.tau[idx];
        net_inputs(nm, ut, ys, nu, x0, x1, x2);
        tn = (logf(tau) - logf(ut) - nm.outMean) / nm.outStd;
    }
    // Forward: h1 stays in registers, h2 goes to shared memory as it is made.
    float h1[kH];
#pragma unroll
    for (int j = 0; j < kH; ++j)
        h1[j] = tanhf(P[kOffB1 + j] + P[kOffW1 + 3 * j] * x0 + P[kOffW1 + 3 * j + 1] * x1
                      + P[kOffW1 + 3 * j + 2] * x2);
    float y = P[kOffB3];
#pragma unroll 2
    for (int j = 0; j < kH; ++j) {
        float z = P[kOffB2 + j];
#pragma unroll
        for (int k = 0; k < kH; ++k) z += P[kOffW2 + kH * j + k] * h1[k];
        const float h2 = tanhf(z);
        h2s[t][j] = h2;
        y += P[kOffW3 + j] * h2;
    }
    const float err = valid ? y - tn : 0.0f;
    const float dy = 2.0f * err * invCount;

    // Backward: dz2 = dy W3 (1 - h2^2); dh1 = W2^T dz2; dz1 = dh1 (1 - h1^2).
    float dh1[kH];
#pragma unroll
    for (int k = 0; k < kH; ++k) dh1[k] = 0.0f;
#pragma unroll 2
    for (int j = 0; j < kH; ++j) {
        const float h2 = h2s[t][j];
        const float dz2 = dy * P[kOffW3 + j] * (1.0f - h2 * h2);
        dz2s[t][j] = dz2;
#pragma unroll
        for (int k = 0; k < kH; ++k) dh1[k] += P[kOffW2 + kH * j + k] * dz2;
    }
#pragma unroll
    for (int k = 0; k < kH; ++k) {
        h1s[t][k] = h1[k];
        dz1s[t][k] = dh1[k] * (1.0f - h1[k] * h1[k]);
    }
    xs[t][0] = x0; xs[t][1] = x1; xs[t][2] = x2;
    dys[t] = dy;
    errs[t] = err * err;
    __syncthreads();

    // Block reduction: parameter p summed over the block's samples in order.
    float* out = partials + static_cast<size_t>(blockIdx.x) * kPartialStride;
    for (int p = t; p < kPartialStride; p += kTrainBlock) {
        float acc = 0.0f;
        if (p < kOffB1) {
            const int j = p / 3, i = p % 3;
            for (int s = 0; s < kTrainBlock; ++s) acc += dz1s[s][j] * xs[s][i];
        } else if (p < kOffW2) {
            const int j = p - kOffB1;
            for (int s = 0; s < kTrainBlock; ++s) acc += dz1s[s][j];
        } else if (p < kOffB2) {
            const int j = (p - kOffW2) / kH, k = (p - kOffW2) % kH;
            for (int s = 0; s < kTrainBlock; ++s) acc += dz2s[s][j] * h1s[s][k];
        } else if (p < kOffW3) {
            const int j = p - kOffB2;
            for (int s = 0; s < kTrainBlock; ++s) acc += dz2s[s][j];
        } else if (p < kOffB3) {
            const int j = p - kOffW3;
            for (int s = 0; s < kTrainBlock; ++s) acc += dys[s] * h2s[s][j];
        } else if (p == kOffB3) {
            for (int s = 0; s < kTrainBlock; ++s) acc += dys[s];
        } else {
            for (int s = 0; s < kTrainBlock; ++s) acc += errs[s];
        }
        out[p] = acc;
    }
    if (ADAM) {
        __shared__ bool last;
        __threadfence();
        __syncthreads();
        if (t == 0) last = atomicAdd(adam.ticket, 1u) == gridDim.x - 1;
        __syncthreads();
        if (!last) return;
        __threadfence();
        for (int p = t; p < kPartialStride; p += kTrainBlock)
            adam_update(partials, gridDim.x, p, adam, invCount, wbf);
        if (t == 0) *adam.ticket = 0u;
    }
}

/// Sum of the block partials (block order) -> FP64 accumulator.
__global__ void accumulate_kernel(const float* __restrict__ partials, int nb, double* __restrict__ acc) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kPartialStride) return;
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s += partials[static_cast<size_t>(b) * kPartialStride + p];
    acc[p] += s;
}

/// Per-block FP64 sums for the normalisation: count, then sum and sum of
/// squares of log u_par, log y, log nu, log u_tau - log u_par.
__global__ void norm_partial_kernel(SampleView S, double* __restrict__ out) {
    __shared__ double sh[9][kSolveBlock / 32];
    double v[9] = {};
    for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < S.n;
         i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        const double a = log(static_cast<double>(S.ut[i])), b = log(static_cast<double>(S.ys[i]));
        const double c = log(static_cast<double>(S.nu[i])), d = log(static_cast<double>(S.tau[i])) - a;
        v[0] += 1.0;
        v[1] += a; v[2] += a * a; v[3] += b; v[4] += b * b;
        v[5] += c; v[6] += c * c; v[7] += d; v[8] += d * d;
    }
#pragma unroll
    for (int k = 0; k < 9; ++k)
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
        for (int k = 0; k < 9; ++k) sh[k][warp] = v[k];
    __syncthreads();
    if (threadIdx.x < 9) {
        double s = 0.0;
        for (int w = 0; w < kSolveBlock / 32; ++w) s += sh[threadIdx.x][w];
        out[blockIdx.x * 9 + threadIdx.x] = s;
    }
}

// ---- inference and batched solves --------------------------------------------

constexpr int kSeedOnly = 4;

template <int METHOD>
__global__ void __launch_bounds__(kSolveBlock)
utau_solve_kernel(NetDev net, const float* __restrict__ ut, const float* __restrict__ ys,
                  const float* __restrict__ nu, const float* __restrict__ warm, float* __restrict__ out, int n,
                  int* __restrict__ counters, unsigned long long* __restrict__ iterSum) {
    constexpr bool kNet = METHOD == FCFD_UTAU_LEARNED || METHOD == FCFD_UTAU_NEWTON64_NET || METHOD == kSeedOnly;
    __shared__ float P[kNet ? kParams : 1];
    if (kNet) {
        load_params(net.w, P);
        __syncthreads();
    }
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int fallback = 0, iters = 0;
    float u = 0.0f, y = 1.0f, v = 1.0f;
    if (i < n) { u = ut[i]; y = ys[i]; v = nu[i]; }
    const bool solved = i < n && u > 0.0f && y > 0.0f && v > 0.0f;
    // The network seed is evaluated by the whole warp together.
    float seed = 0.0f;
    if constexpr (kNet) seed = net_seed_warp(P, net.norm, u, y, v, solved);
    if (i < n) {
        float r = 0.0f;
        if (solved) {
            const float w0 = warm ? warm[i] : 0.0f;
            if (METHOD == FCFD_UTAU_REFERENCE) {
                r = newton_reference(u, y, v, reference_seed(u, y, v, w0));
            } else if (METHOD == FCFD_UTAU_NEWTON64) {
                r = static_cast<float>(newton64(u, y, v, reference_seed(u, y, v, w0), &iters));
            } else if (METHOD == FCFD_UTAU_LEARNED) {
                r = learned_correct(u, y, v, seed, &fallback, &iters);
            } else if (METHOD == FCFD_UTAU_NEWTON64_NET) {
                r = static_cast<float>(newton64(u, y, v, seed, &iters));
            } else {
                r = seed;
            }
        }
        out[i] = r;
    }
    if (counters) {
        const unsigned fb = __ballot_sync(0xffffffffu, fallback != 0);
        const unsigned sv = __ballot_sync(0xffffffffu, solved);
        unsigned long long it = static_cast<unsigned long long>(iters);
        for (int o = 16; o > 0; o >>= 1) it += __shfl_down_sync(0xffffffffu, it, o);
        if ((threadIdx.x & 31) == 0) {
            if (sv) atomicAdd(&counters[0], __popc(sv));
            if (fb) atomicAdd(&counters[1], __popc(fb));
            if (it) atomicAdd(iterSum, it);
        }
    }
}

template <int M>
cudaError_t launch_solve(NetDev net, const float* ut, const float* ys, const float* nu, const float* warm,
                         float* out, int n, int* counters, unsigned long long* iters, cudaStream_t st) {
    const unsigned nb = static_cast<unsigned>((n + kSolveBlock - 1) / kSolveBlock);
    utau_solve_kernel<M><<<nb, kSolveBlock, 0, st>>>(net, ut, ys, nu, warm, out, n, counters, iters);
    return cudaGetLastError();
}

double splitmix(unsigned long long& s) {
    s += 0x9e3779b97f4a7c15ULL;
    unsigned long long z = s;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    z ^= z >> 31;
    return static_cast<double>(z >> 11) * (1.0 / 9007199254740992.0);
}
unsigned long long splitmix_u64(unsigned long long& s) {
    s += 0x9e3779b97f4a7c15ULL;
    unsigned long long z = s;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

} // namespace

struct fcfd_wallnet {
    int device = 0;
    std::vector<float> master = std::vector<float>(kParams, 0.0f);  // host mirror of the FP32 master copy
    Norm norm{};
    fcfd_wallnet_norm normPublic{};
    float* dMaster = nullptr;
    float* dM = nullptr;
    float* dV = nullptr;
    std::uint16_t* dW = nullptr;
    float* dPartials = nullptr;
    double* dAcc = nullptr;
    float* dLoss = nullptr;
    int* dCounters = nullptr;
    unsigned long long* dIters = nullptr;
    unsigned* dTicket = nullptr;
    long long adamStep = 0;
    bool ok = false;

    NetDev view() const {
        NetDev v;
        v.w = dW;
        v.norm = norm;
        return v;
    }
    void setNorm(const fcfd_wallnet_norm& p) {
        normPublic = p;
        for (int k = 0; k < 3; ++k) {
            norm.inMean[k] = p.in_mean[k];
            norm.inInvStd[k] = 1.0f / (p.in_std[k] > 0.0f ? p.in_std[k] : 1.0f);
        }
        norm.outMean = p.out_mean;
        norm.outStd = p.out_std > 0.0f ? p.out_std : 1.0f;
    }
    /// Upload the host master copy, its BF16 rounding, and zero Adam state.
    cudaError_t upload() {
        std::vector<std::uint16_t> b(kParams);
        for (int i = 0; i < kParams; ++i) b[i] = f32_to_bf16_bits(master[i]);
        if (auto e = cudaMemcpy(dMaster, master.data(), kParams * 4, cudaMemcpyHostToDevice); e != cudaSuccess) return e;
        if (auto e = cudaMemcpy(dW, b.data(), kParams * 2, cudaMemcpyHostToDevice); e != cudaSuccess) return e;
        if (auto e = cudaMemset(dM, 0, kParams * 4); e != cudaSuccess) return e;
        if (auto e = cudaMemset(dV, 0, kParams * 4); e != cudaSuccess) return e;
        adamStep = 0;
        return cudaSuccess;
    }
};

namespace fcfd {
/// Device view of a net for the solver's wall updates (BF16 weights live in
/// the net; the solver copies them).
NetDev wallnet_view(const fcfd_wallnet* net) { return net ? net->view() : NetDev{}; }
} // namespace fcfd

extern "C" {

fcfd_wallnet* fcfd_wallnet_create(void) {
    auto* n = new fcfd_wallnet();
    cudaGetDevice(&n->device);
    bool ok = cudaMalloc(&n->dMaster, kParams * 4) == cudaSuccess;
    ok = ok && cudaMalloc(&n->dM, kParams * 4) == cudaSuccess;
    ok = ok && cudaMalloc(&n->dV, kParams * 4) == cudaSuccess;
    ok = ok && cudaMalloc(&n->dW, kParams * 2) == cudaSuccess;
    ok = ok && cudaMalloc(&n->dPartials, static_cast<size_t>(kMaxTrainBlocks) * kPartialStride * 4) == cudaSuccess;
    ok = ok && cudaMalloc(&n->dAcc, kPartialStride * 8) == cudaSuccess;
    ok = ok && cudaMalloc(&n->dLoss, 4) == cudaSuccess;
    ok = ok && cudaMalloc(&n->dCounters, 2 * sizeof(int)) == cudaSuccess;
    ok = ok && cudaMalloc(&n->dIters, sizeof(unsigned long long)) == cudaSuccess;
    ok = ok && cudaMalloc(&n->dTicket, sizeof(unsigned)) == cudaSuccess;
    ok = ok && cudaMemset(n->dTicket, 0, sizeof(unsigned)) == cudaSuccess;
    n->ok = ok;
    fcfd_wallnet_norm unit{{0, 0, 0}, {1, 1, 1}, 0, 1};
    n->setNorm(unit);
    if (ok) ok = n->upload() == cudaSuccess;
    if (!ok) {
        fcfd_wallnet_destroy(n);
        return nullptr;
    }
    return n;
}

void fcfd_wallnet_destroy(fcfd_wallnet* n) {
    if (!n) return;
    cudaFree(n->dMaster); cudaFree(n->dM); cudaFree(n->dV); cudaFree(n->dW); cudaFree(n->dPartials);
    cudaFree(n->dAcc); cudaFree(n->dLoss); cudaFree(n->dCounters); cudaFree(n->dIters); cudaFree(n->dTicket);
    delete n;
}

int fcfd_wallnet_init_params(fcfd_wallnet* n, unsigned long long seed) {
    if (!n) return cudaErrorInvalidValue;
    unsigned long long s = seed;
    auto uni = [&](float lim) { return static_cast<float>((2.0 * splitmix(s) - 1.0) * lim); };
    const float l1 = std::sqrt(6.0f / (3 + kH)), l2 = std::sqrt(6.0f / (kH + kH)), l3 = std::sqrt(6.0f / (kH + 1));
    std::fill(n->master.begin(), n->master.end(), 0.0f);
    for (int i = 0; i < 3 * kH; ++i) n->master[kOffW1 + i] = uni(l1);
    for (int i = 0; i < kH * kH; ++i) n->master[kOffW2 + i] = uni(l2);
    for (int i = 0; i < kH; ++i) n->master[kOffW3 + i] = uni(l3);
    return n->upload();
}

int fcfd_wallnet_set_params(fcfd_wallnet* n, const float* params, const fcfd_wallnet_norm* norm) {
    if (!n || !params) return cudaErrorInvalidValue;
    std::memcpy(n->master.data(), params, kParams * 4);
    if (norm) n->setNorm(*norm);
    return n->upload();
}

int fcfd_wallnet_get_params(const fcfd_wallnet* n, float* params, float* bf16, fcfd_wallnet_norm* norm) {
    if (!n) return cudaErrorInvalidValue;
    std::vector<float> m(kParams);
    if (auto e = cudaMemcpy(m.data(), n->dMaster, kParams * 4, cudaMemcpyDeviceToHost); e != cudaSuccess) return e;
    if (params) std::memcpy(params, m.data(), kParams * 4);
    if (bf16) {
        std::vector<std::uint16_t> b(kParams);
        if (auto e = cudaMemcpy(b.data(), n->dW, kParams * 2, cudaMemcpyDeviceToHost); e != cudaSuccess) return e;
        for (int i = 0; i < kParams; ++i) bf16[i] = bf16_bits_to_f32_host(b[i]);
    }
    if (norm) *norm = n->normPublic;
    return 0;
}

int fcfd_wallnet_fit_norm(fcfd_wallnet* n, const float* ut, const float* ys, const float* nu, const float* tau,
                          int count, void* stream) {
    if (!n || !ut || !ys || !nu || !tau || count <= 0) return cudaErrorInvalidValue;
    auto st = static_cast<cudaStream_t>(stream);
    const int nb = static_cast<int>(std::min<long long>(kMaxTrainBlocks, (count + kSolveBlock - 1) / kSolveBlock));
    double* d = nullptr;
    if (auto e = cudaMalloc(&d, static_cast<size_t>(nb) * 9 * 8); e != cudaSuccess) return e;
    SampleView S{ut, ys, nu, tau, static_cast<unsigned long long>(count)};
    norm_partial_kernel<<<nb, kSolveBlock, 0, st>>>(S, d);
    std::vector<double> h(static_cast<size_t>(nb) * 9);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), d, h.size() * 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d);
    if (e != cudaSuccess) return e;
    double v[9] = {};
    for (int b = 0; b < nb; ++b)
        for (int k = 0; k < 9; ++k) v[k] += h[static_cast<size_t>(b) * 9 + k];
    fcfd_wallnet_norm p{};
    auto stat = [&](int k, float& mean, float& sd) {
        const double mu = v[k] / v[0];
        const double var = std::max(v[k + 1] / v[0] - mu * mu, 0.0);
        mean = static_cast<float>(mu);
        sd = var > 1e-12 ? static_cast<float>(std::sqrt(var)) : 1.0f;
    };
    stat(1, p.in_mean[0], p.in_std[0]);
    stat(3, p.in_mean[1], p.in_std[1]);
    stat(5, p.in_mean[2], p.in_std[2]);
    stat(7, p.out_mean, p.out_std);
    n->setNorm(p);
    return 0;
}

int fcfd_wallnet_gradient(fcfd_wallnet* n, const float* ut, const float* ys, const float* nu, const float* tau,
                          int count, double* loss, float* grad, void* stream) {
    if (!n || !ut || !ys || !nu || !tau || count <= 0) return cudaErrorInvalidValue;
    auto st = static_cast<cudaStream_t>(stream);
    SampleView S{ut, ys, nu, tau, static_cast<unsigned long long>(count)};
    if (auto e = cudaMemsetAsync(n->dAcc, 0, kPartialStride * 8, st); e != cudaSuccess) return e;
    const float inv = 1.0f / static_cast<float>(count);
    constexpr int chunk = kMaxTrainBlocks * kTrainBlock;
    for (int pos = 0; pos < count; pos += chunk) {
        const int c = std::min(chunk, count - pos);
        const int nb = (c + kTrainBlock - 1) / kTrainBlock;
        grad_kernel<false><<<nb, kTrainBlock, 0, st>>>(n->dW, n->norm, S, 1ULL, 0ULL,
                                                       static_cast<unsigned long long>(pos), c, inv, n->dPartials,
                                                       AdamStep{});
        accumulate_kernel<<<(kPartialStride + 255) / 256, 256, 0, st>>>(n->dPartials, nb, n->dAcc);
    }
    std::vector<double> h(kPartialStride);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), n->dAcc, kPartialStride * 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    if (grad)
        for (int p = 0; p < kParams; ++p) grad[p] = static_cast<float>(h[p]);
    if (loss) *loss = h[kParams] / count;
    return 0;
}

int fcfd_wallnet_train(fcfd_wallnet* n, const float* ut, const float* ys, const float* nu, const float* tau,
                       int count, const fcfd_wallnet_train_opts* o, float* lossPerEpoch, void* stream) {
    if (!n || !ut || !ys || !nu || !tau || !o || count <= 0 || o->epochs <= 0 || o->batch <= 0 ||
        o->batch % kTrainBlock != 0 || o->batch > kMaxTrainBlocks * kTrainBlock)
        return cudaErrorInvalidValue;
    auto st = static_cast<cudaStream_t>(stream);
    SampleView S{ut, ys, nu, tau, static_cast<unsigned long long>(count)};
    const int stepsPerEpoch = (count + o->batch - 1) / o->batch;
    const long long total = static_cast<long long>(stepsPerEpoch) * o->epochs;
    const long long up = std::max<long long>(1, static_cast<long long>(o->warmup_frac * total));
    const double lrMax = o->lr_max, lr0 = lrMax / 25.0, lrEnd = lr0 / 1e4;
    const double pi = 3.14159265358979323846;
    unsigned long long rs = o->seed;
    std::vector<float> hist(o->epochs, 0.0f);
    float* dHist = nullptr;
    if (auto e = cudaMalloc(&dHist, o->epochs * 4); e != cudaSuccess) return e;
    long long t = 0;
    cudaError_t e = cudaSuccess;
    for (int ep = 0; ep < o->epochs && e == cudaSuccess; ++ep) {
        // Epoch shuffle: position -> (a * position + c) mod n, gcd(a, n) = 1.
        unsigned long long a = 1, c = 0;
        if (count > 1) {
            do {
                a = 1 + splitmix_u64(rs) % static_cast<unsigned long long>(count - 1);
            } while (std::gcd(a, static_cast<unsigned long long>(count)) != 1ULL);
            c = splitmix_u64(rs) % static_cast<unsigned long long>(count);
        }
        for (int sidx = 0; sidx < stepsPerEpoch; ++sidx, ++t) {
            const long long pos = static_cast<long long>(sidx) * o->batch;
            const int cnt = static_cast<int>(std::min<long long>(o->batch, count - pos));
            const int nb = (cnt + kTrainBlock - 1) / kTrainBlock;
            const float inv = 1.0f / static_cast<float>(cnt);
            double lr;
            if (t < up) lr = lr0 + (lrMax - lr0) * 0.5 * (1.0 - std::cos(pi * t / up));
            else lr = lrEnd + (lrMax - lrEnd) * 0.5 * (1.0 + std::cos(pi * (t - up) / std::max<long long>(1, total - up)));
            ++n->adamStep;
            AdamStep as;
            as.master = n->dMaster; as.m = n->dM; as.v = n->dV;
            as.lr = static_cast<float>(lr);
            as.beta1 = o->beta1; as.beta2 = o->beta2; as.eps = o->eps;
            as.bc1 = static_cast<float>(1.0 - std::pow(static_cast<double>(o->beta1), n->adamStep));
            as.bc2 = static_cast<float>(1.0 - std::pow(static_cast<double>(o->beta2), n->adamStep));
            as.lossOut = sidx == stepsPerEpoch - 1 ? dHist + ep : nullptr;
            as.ticket = n->dTicket;
            grad_kernel<true><<<nb, kTrainBlock, 0, st>>>(n->dW, n->norm, S, a, c, static_cast<unsigned long long>(pos),
                                                          cnt, inv, n->dPartials, as);
        }
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(hist.data(), dHist, o->epochs * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(dHist);
    if (e != cudaSuccess) return e;
    if (lossPerEpoch) std::memcpy(lossPerEpoch, hist.data(), o->epochs * 4);
    return cudaMemcpy(n->master.data(), n->dMaster, kParams * 4, cudaMemcpyDeviceToHost);
}

int fcfd_wallnet_predict(const fcfd_wallnet* n, const float* ut, const float* ys, const float* nu, float* out,
                         int count, void* stream) {
    if (!n || !ut || !ys || !nu || !out || count < 0) return cudaErrorInvalidValue;
    if (count == 0) return 0;
    return launch_solve<kSeedOnly>(n->view(), ut, ys, nu, nullptr, out, count, nullptr, nullptr,
                                   static_cast<cudaStream_t>(stream));
}

int fcfd_utau_solve(int method, const fcfd_wallnet* n, const float* ut, const float* ys, const float* nu,
                    const float* warm, float* out, int count, fcfd_utau_stats* stats, void* stream) {
    if (!ut || !ys || !nu || !out || count < 0) return cudaErrorInvalidValue;
    if ((method == FCFD_UTAU_LEARNED || method == FCFD_UTAU_NEWTON64_NET) && !n) return cudaErrorInvalidValue;
    if (count == 0) {
        if (stats) *stats = fcfd_utau_stats{};
        return 0;
    }
    auto st = static_cast<cudaStream_t>(stream);
    // Statistics use counters of a net when one is given, else a scratch pair.
    int* ctr = nullptr;
    unsigned long long* its = nullptr;
    void* scratch = nullptr;
    if (stats) {
        if (n) {
            ctr = n->dCounters;
            its = n->dIters;
        } else {
            if (auto e = cudaMalloc(&scratch, 16); e != cudaSuccess) return e;
            ctr = static_cast<int*>(scratch);
            its = reinterpret_cast<unsigned long long*>(static_cast<char*>(scratch) + 8);
        }
        cudaMemsetAsync(ctr, 0, 2 * sizeof(int), st);
        cudaMemsetAsync(its, 0, sizeof(unsigned long long), st);
    }
    const NetDev v = n ? n->view() : NetDev{};
    cudaError_t e;
    switch (method) {
    case FCFD_UTAU_REFERENCE: e = launch_solve<FCFD_UTAU_REFERENCE>(v, ut, ys, nu, warm, out, count, ctr, its, st); break;
    case FCFD_UTAU_NEWTON64: e = launch_solve<FCFD_UTAU_NEWTON64>(v, ut, ys, nu, warm, out, count, ctr, its, st); break;
    case FCFD_UTAU_LEARNED: e = launch_solve<FCFD_UTAU_LEARNED>(v, ut, ys, nu, warm, out, count, ctr, its, st); break;
    case FCFD_UTAU_NEWTON64_NET: e = launch_solve<FCFD_UTAU_NEWTON64_NET>(v, ut, ys, nu, warm, out, count, ctr, its, st); break;
    default: e = cudaErrorInvalidValue;
    }
    if (e == cudaSuccess && stats) {
        int h[2];
        unsigned long long it = 0;
        e = cudaMemcpyAsync(h, ctr, sizeof h, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&it, its, sizeof it, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e == cudaSuccess) {
            stats->solved = h[0];
            stats->fallbacks = h[1];
            stats->newton_iterations = static_cast<long long>(it);
        }
    }
    if (scratch) cudaFree(scratch);
    return e;
}

} // extern "C"
