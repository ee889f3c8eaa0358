// ORACLE - test infrastructure only. A CPU restatement of the reference
// FoilCFD solver step, used by tests/, __graft_entry__.smoke() and the
// cpu_baseline leg of bench.py as the reference results to compare against
// and the timed CPU baseline; the product never links or calls it.
//
// Each routine follows the reference kernel line by line in the reference's
// own operation order (compiled with -ffp-contract=off, so no FMA is formed
// that the source does not spell), templated on the real type so the same
// code gives the FP32 restatement and an FP64 oracle for error statements:
//   collide        src/sim/lbm_core.cu:213-475 (streamCollideKernel<WM,false>)
//   init/speck     src/sim/lbm_core.cu:102-160, 761-771
//   force          src/sim/lbm_core.cu:573-637 (forceReductionKernel<WM>),
//                  summed in FP64
//   wall update    src/sim/lbm_wallmodel.cu:31-196
//   fill/restrict  src/sim/lbm_refine.cu:70-429
// One deliberate layout difference: the reference pads z with ghost planes
// refreshed after every collide (lbm_core.cu:484-497); here z (and x, y) wrap
// periodically in the index math, which reads the same values.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int Q = 19;
constexpr int CX[Q] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0};
constexpr int CY[Q] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1};
constexpr int CZ[Q] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1};
constexpr int OPP[Q] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17};
constexpr int MIRY[Q] = {0, 1, 2, 4, 3, 5, 6, 13, 14, 9, 10, 18, 17, 7, 8, 15, 16, 12, 11};
constexpr int MIRZ[Q] = {0, 1, 2, 3, 4, 6, 5, 7, 8, 15, 16, 17, 18, 13, 14, 9, 10, 11, 12};

enum : uint8_t { FLUID = 0, SOLID = 1, INLET = 2, OUTLET = 3, SLIPT = 4, SLIPB = 5, SLIPF = 6,
                 SLIPK = 7, IFACE = 8, OUTLET_EQ = 9 };

template <class T> T W(int q) {
    return q == 0 ? T(1) / T(3) : (q <= 6 ? T(1) / T(18) : T(1) / T(36));
}
template <class T> T c_maxspeed();
template <> float c_maxspeed<float>() { return 0.30f; }
template <> double c_maxspeed<double>() { return 0.30; }
template <class T> T c_floor();
template <> float c_floor<float>() { return 0.05f; }
template <> double c_floor<double>() { return 0.05; }

inline int wrap(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

struct Dims {
    int nx, ny, nz;
    long long n() const { return (long long)nx * ny * nz; }
    long long at(int x, int y, int z) const { return x + (long long)nx * (y + (long long)ny * z); }
};

// IEEE binary16 <-> binary32, round to nearest even (own implementation of
// the IEEE 754 conversion; used for the wall model's half slip field).
uint16_t f2h(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const int exp = (int)((x >> 23) & 0xFF);
    uint32_t man = x & 0x7FFFFFu;
    if (exp == 0xFF) return (uint16_t)(sign | 0x7C00u | (man ? 0x200u : 0u));
    int e = exp - 127 + 15;
    if (e >= 31) return (uint16_t)(sign | 0x7C00u);
    if (e <= 0) {
        if (e < -10) return (uint16_t)sign;
        man |= 0x800000u;
        const int shift = 14 - e;
        uint32_t h = man >> shift;
        const uint32_t rem = man & ((1u << shift) - 1u), half = 1u << (shift - 1);
        if (rem > half || (rem == half && (h & 1u))) ++h;
        return (uint16_t)(sign | h);
    }
    uint32_t h = ((uint32_t)e << 10) | (man >> 13);
    const uint32_t rem = man & 0x1FFFu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
    return (uint16_t)(sign | h);
}
float h2f(uint16_t h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    int exp = (h >> 10) & 0x1F;
    uint32_t man = h & 0x3FFu;
    uint32_t x;
    if (exp == 0) {
        if (man == 0) x = sign;
        else {
            exp = 1;
            while (!(man & 0x400u)) { man <<= 1; --exp; }
            man &= 0x3FFu;
            x = sign | ((uint32_t)(exp - 15 + 127) << 23) | (man << 13);
        }
    } else if (exp == 31) {
        x = sign | 0x7F800000u | (man << 13);
    } else {
        x = sign | ((uint32_t)(exp - 15 + 127) << 23) | (man << 13);
    }
    float f;
    std::memcpy(&f, &x, 4);
    return f;
}

/// Second-order D3Q19 equilibrium (lbm_core.cu:63-73 equilibrium19; the same
/// body in lbm_refine.cu:44-52).
template <class T>
void equilibrium19(T rho, T ux, T uy, T uz, T feq[Q]) {
    const T usq = T(1.5) * (ux * ux + uy * uy + uz * uz);
    for (int q = 0; q < Q; ++q) {
        const T cu = T(3) * (T(CX[q]) * ux + T(CY[q]) * uy + T(CZ[q]) * uz);
        feq[q] = W<T>(q) * rho * (T(1) + cu + T(0.5) * cu * cu - usq);
    }
}

/// One pull stream-collide over the lattice (lbm_core.cu:213-475
/// streamCollideKernel<WM, QL>: boundary select by neighbour flag, moments,
/// limiter, Smagorinsky tau, TRT, Ladd term, q-LIBB links).
template <class T>
void collide(const Dims& d, const T* src, T* dst, const uint8_t* flags, T tau0, T lambda, T smagPre,
             T uIn, int writeMacro, T* mr, T* mu, T* mv, T* mw, const uint16_t* uwxA,
             const uint16_t* uwyA, const uint16_t* uwzA, const uint8_t* qFrac = nullptr,
             const uint32_t* ffMask = nullptr) {
    const long long N = d.n();
    const bool wm = uwxA && uwyA && uwzA;
#pragma omp parallel for schedule(static)
    for (long long cell = 0; cell < N; ++cell) {
        const int z = (int)(cell / ((long long)d.nx * d.ny));
        const long long rem = cell - (long long)z * d.nx * d.ny;
        const int y = (int)(rem / d.nx);
        const int x = (int)(rem - (long long)y * d.nx);
        const uint8_t myFlag = flags[cell];
        if (myFlag != FLUID) {
            if (myFlag == INLET) {
                T feq[Q];
                equilibrium19<T>(T(1), uIn, T(0), T(0), feq);
                for (int q = 0; q < Q; ++q) dst[q * N + cell] = feq[q];
                if (writeMacro) { mr[cell] = T(1); mu[cell] = uIn; mv[cell] = T(0); mw[cell] = T(0); }
            } else if (myFlag == OUTLET || myFlag == OUTLET_EQ) {
                const long long up = d.at(wrap(x - 1, d.nx), y, z);
                T g[Q];
                T r = T(0), jx = T(0), jy = T(0), jz = T(0);
                for (int q = 0; q < Q; ++q) {
                    const T fq = src[q * N + up];
                    g[q] = fq;
                    r += fq;
                    jx += T(CX[q]) * fq; jy += T(CY[q]) * fq; jz += T(CZ[q]) * fq;
                }
                const T inv = T(1) / r;
                T ux = jx * inv, uy = jy * inv, uz = jz * inv;
                if (myFlag == OUTLET_EQ) {
                    equilibrium19<T>(T(1), ux, uy, uz, g);
                    r = T(1);
                }
                for (int q = 0; q < Q; ++q) dst[q * N + cell] = g[q];
                if (writeMacro) { mr[cell] = r; mu[cell] = ux; mv[cell] = uy; mw[cell] = uz; }
            } else if (writeMacro) {
                mr[cell] = T(1); mu[cell] = T(0); mv[cell] = T(0); mw[cell] = T(0);
            }
            continue;
        }
        T uwx = T(0), uwy = T(0), uwz = T(0);
        bool uwLoaded = false;
        T fpop[Q];
        for (int q = 0; q < Q; ++q) {
            const int xn = wrap(x - CX[q], d.nx), yn = wrap(y - CY[q], d.ny), zn = wrap(z - CZ[q], d.nz);
            const long long pn = d.at(xn, yn, zn);
            const uint8_t nf = flags[pn];
            const bool solid = nf == SOLID;
            const bool slipY = nf == SLIPT || nf == SLIPB;
            const bool slipZ = nf == SLIPF || nf == SLIPK;
            const long long pY = d.at(xn, y, zn), pZ = d.at(xn, yn, z);
            const int qs = solid ? OPP[q] : (slipY ? MIRY[q] : (slipZ ? MIRZ[q] : q));
            const long long cs = solid ? cell : (slipY ? pY : (slipZ ? pZ : pn));
            fpop[q] = src[qs * N + cs];
            // Interpolated bounce-back (Bouzidi 2001) on a solid link with an
            // analytic cut fraction (lbm_core.cu:332-364).
            if (qFrac && solid) {
                const uint8_t qb = qFrac[cell * Q + q];
                if (qb != 0) {
                    const T qf = T(qb) * (T(1) / T(255));
                    const T fOut = src[q * N + cell];
                    if (qf >= T(0.5)) {
                        const T inv2q = T(0.5) / qf;
                        fpop[q] = inv2q * fOut + (T(1) - inv2q) * fpop[q];
                    } else if (ffMask[cell] & (1u << q)) {
                        const long long pff = d.at(wrap(x + CX[q], d.nx), wrap(y + CY[q], d.ny), wrap(z + CZ[q], d.nz));
                        const T fOutFF = src[q * N + pff];
                        fpop[q] = T(2) * qf * fOut + (T(1) - T(2) * qf) * fOutFF;
                    }
                }
            }
            if (wm && solid) {
                if (!uwLoaded) {
                    uwx = (T)h2f(uwxA[cell]); uwy = (T)h2f(uwyA[cell]); uwz = (T)h2f(uwzA[cell]);
                    uwLoaded = true;
                }
                fpop[q] += T(6) * W<T>(q) * (T(CX[q]) * uwx + T(CY[q]) * uwy + T(CZ[q]) * uwz);
            }
        }
        T rho = T(0), jx = T(0), jy = T(0), jz = T(0);
        for (int q = 0; q < Q; ++q) {
            rho += fpop[q];
            jx += T(CX[q]) * fpop[q]; jy += T(CY[q]) * fpop[q]; jz += T(CZ[q]) * fpop[q];
        }
        rho = std::fmax(rho, c_floor<T>());
        const T invRho = T(1) / rho;
        T ux = jx * invRho, uy = jy * invRho, uz = jz * invRho;
        const T u2 = ux * ux + uy * uy + uz * uz;
        const T ms = c_maxspeed<T>();
        if (u2 > ms * ms) {
            const T s = ms * (T(1) / std::sqrt(u2));
            ux *= s; uy *= s; uz *= s;
        }
        T feq[Q];
        equilibrium19<T>(rho, ux, uy, uz, feq);
        T pxx = 0, pyy = 0, pzz = 0, pxy = 0, pxz = 0, pyz = 0;
        for (int q = 0; q < Q; ++q) {
            const T fneq = fpop[q] - feq[q];
            pxx += T(CX[q] * CX[q]) * fneq; pyy += T(CY[q] * CY[q]) * fneq; pzz += T(CZ[q] * CZ[q]) * fneq;
            pxy += T(CX[q] * CY[q]) * fneq; pxz += T(CX[q] * CZ[q]) * fneq; pyz += T(CY[q] * CZ[q]) * fneq;
        }
        T tauEff = tau0;
        if (smagPre > T(0)) {
            const T qbar = std::sqrt(pxx * pxx + pyy * pyy + pzz * pzz + T(2) * (pxy * pxy + pxz * pxz + pyz * pyz));
            tauEff = T(0.5) * (tau0 + std::sqrt(tau0 * tau0 + smagPre * qbar * invRho));
        }
        const T omP = T(1) / tauEff;
        const T tauM = T(0.5) + lambda / (tauEff - T(0.5));
        const T omM = T(1) / tauM;
        dst[cell] = fpop[0] - omP * (fpop[0] - feq[0]);
        for (int a = 1; a < Q; a += 2) {
            const int b = a + 1;
            const T sym = omP * (T(0.5) * (fpop[a] + fpop[b]) - T(0.5) * (feq[a] + feq[b]));
            const T asym = omM * (T(0.5) * (fpop[a] - fpop[b]) - T(0.5) * (feq[a] - feq[b]));
            dst[a * N + cell] = fpop[a] - sym - asym;
            dst[b * N + cell] = fpop[b] - sym + asym;
        }
        if (writeMacro) { mr[cell] = rho; mu[cell] = ux; mv[cell] = uy; mw[cell] = uz; }
    }
}

/// Momentum-exchange force over fluid cells with solid links
/// (lbm_core.cu:573-637 forceReductionKernel<WM>), summed in FP64.
template <class T>
void force(const Dims& d, const T* f, const uint8_t* flags, const uint16_t* uwxA, const uint16_t* uwyA,
           const uint16_t* uwzA, double out[3]) {
    const long long N = d.n();
    const bool wm = uwxA && uwyA && uwzA;
    double fx = 0, fy = 0, fz = 0;
#pragma omp parallel for reduction(+ : fx, fy, fz) schedule(static)
    for (long long cell = 0; cell < N; ++cell) {
        if (flags[cell] != FLUID) continue;
        const int z = (int)(cell / ((long long)d.nx * d.ny));
        const long long rem = cell - (long long)z * d.nx * d.ny;
        const int y = (int)(rem / d.nx), x = (int)(rem - (long long)y * d.nx);
        T uwx = 0, uwy = 0, uwz = 0;
        if (wm) { uwx = (T)h2f(uwxA[cell]); uwy = (T)h2f(uwyA[cell]); uwz = (T)h2f(uwzA[cell]); }
        for (int q = 1; q < Q; ++q) {
            const long long pn = d.at(wrap(x + CX[q], d.nx), wrap(y + CY[q], d.ny), wrap(z + CZ[q], d.nz));
            if (flags[pn] != SOLID) continue;
            const T fq = f[q * N + cell];
            T corr = T(0);
            if (wm) corr = T(6) * W<T>(q) * (T(CX[q]) * uwx + T(CY[q]) * uwy + T(CZ[q]) * uwz);
            fx += (double)(T(CX[q]) * (T(2) * fq - corr));
            fy += (double)(T(CY[q]) * (T(2) * fq - corr));
            fz += (double)(T(CZ[q]) * (T(2) * fq - corr));
        }
    }
    out[0] = fx; out[1] = fy; out[2] = fz;
}

// ---- wall model (FP32, reference lbm_wallmodel.cu:31-196) ----------------
constexpr float kKappa = 0.41f, kC = 7.8f;
/// Reichardt's law u+(y+) (lbm_wallmodel.cu:30-36 reichardtUPlus).
float reichardt(float yp) {
    return std::log(1.0f + kKappa * yp) / kKappa
         + kC * (1.0f - std::exp(-yp / 11.0f) - (yp / 11.0f) * std::exp(-yp / 3.0f));
}
/// du+/dy+ of Reichardt's law (lbm_wallmodel.cu:38-45 reichardtDuPlus).
float reichardt_d(float yp) {
    return 1.0f / (1.0f + kKappa * yp)
         + kC * ((1.0f / 11.0f) * std::exp(-yp / 11.0f) - (1.0f / 11.0f) * std::exp(-yp / 3.0f)
                 + (yp / 33.0f) * std::exp(-yp / 3.0f));
}
/// Six FP32 Newton iterations on u_tau u+(y u_tau / nu) = u_t from the warm
/// or fresh seed (lbm_wallmodel.cu:55-73 solveUTau).
float solve_utau(float ut, float ys, float nu, float seed) {
    float utau = seed > 0.0f ? seed : std::fmax(0.04f * ut, std::sqrt(nu * ut / ys));
    for (int it = 0; it < 6; ++it) {
        const float yp = std::fmax(ys * utau / nu, 1e-8f);
        const float up = reichardt(yp);
        const float g = utau * up - ut;
        const float dg = up + yp * reichardt_d(yp);
        utau -= g / std::fmax(dg, 1e-6f);
        utau = std::fmax(utau, 0.0f);
    }
    return utau;
}

} // namespace

extern "C" {

void oracle_collide_f32(int nx, int ny, int nz, const float* src, float* dst, const uint8_t* flags, float tau0,
                        float lambda, float smagPre, float uIn, int writeMacro, float* r, float* u, float* v,
                        float* w, const uint16_t* uwx, const uint16_t* uwy, const uint16_t* uwz,
                        const uint8_t* qFrac, const uint32_t* ffMask) {
    collide<float>(Dims{nx, ny, nz}, src, dst, flags, tau0, lambda, smagPre, uIn, writeMacro, r, u, v, w, uwx,
                   uwy, uwz, qFrac, ffMask);
}

void oracle_collide_f64(int nx, int ny, int nz, const double* src, double* dst, const uint8_t* flags,
                        double tau0, double lambda, double smagPre, double uIn, int writeMacro, double* r,
                        double* u, double* v, double* w, const uint16_t* uwx, const uint16_t* uwy,
                        const uint16_t* uwz, const uint8_t* qFrac, const uint32_t* ffMask) {
    collide<double>(Dims{nx, ny, nz}, src, dst, flags, tau0, lambda, smagPre, uIn, writeMacro, r, u, v, w, uwx,
                    uwy, uwz, qFrac, ffMask);
}

void oracle_force_f32(int nx, int ny, int nz, const float* f, const uint8_t* flags, const uint16_t* uwx,
                      const uint16_t* uwy, const uint16_t* uwz, double* out) {
    force<float>(Dims{nx, ny, nz}, f, flags, uwx, uwy, uwz, out);
}

void oracle_force_f64(int nx, int ny, int nz, const double* f, const uint8_t* flags, const uint16_t* uwx,
                      const uint16_t* uwy, const uint16_t* uwz, double* out) {
    force<double>(Dims{nx, ny, nz}, f, flags, uwx, uwy, uwz, out);
}

/// Reference initEquilibriumKernel: rho = 1, u = (uIn, 0, 0); solids rest.
void oracle_init_eq(int nx, int ny, int nz, float* f, const uint8_t* flags, float uIn) {
    const Dims d{nx, ny, nz};
    const long long N = d.n();
    for (long long c = 0; c < N; ++c) {
        const float ux = flags[c] == SOLID ? 0.0f : uIn;
        float feq[Q];
        equilibrium19<float>(1.0f, ux, 0.0f, 0.0f, feq);
        for (int q = 0; q < Q; ++q) f[q * N + c] = feq[q];
    }
}

/// Reference spanwisePerturbKernel + launch phases (lbm_core.cu:130-160,761-771).
void oracle_speck(int nx, int ny, int nz, float* f, const uint8_t* flags, float amp, unsigned seed) {
    auto phase = [seed](unsigned salt) {
        unsigned h = (seed + salt) * 2654435761u;
        h ^= h >> 16;
        return 6.2831853f * (float)(h & 0xFFFFFFu) / 16777216.0f;
    };
    const float p1 = phase(1u), p2 = phase(2u), p3 = phase(3u);
    const Dims d{nx, ny, nz};
    const long long N = d.n();
    for (long long c = 0; c < N; ++c) {
        if (flags[c] != FLUID) continue;
        const int z = (int)(c / ((long long)nx * ny));
        const int x = (int)((c - (long long)z * nx * ny) % nx);
        const float tz = 6.2831853f * ((float)z + 0.5f) / nz;
        const float tx = 6.2831853f * ((float)x + 0.5f) / nx;
        const float wz = amp * (0.6f * std::sin(3.0f * tz + p1) + 0.4f * std::sin(7.0f * tz + p2))
                       * (1.0f + 0.3f * std::sin(2.0f * tx + p3));
        for (int q = 0; q < Q; ++q) {
            if (CZ[q] == 0) continue;
            f[q * N + c] = f[q * N + c] + 3.0f * W<float>(q) * CZ[q] * wz;
        }
    }
}

/// Reference wallModelUpdateKernel over a host list (FP32, libm log/exp).
void oracle_wall_update(int nx, int ny, int nz, const float* f, int count, const long long* cellIdx,
                        const long long* sampleIdx, const float* nXa, const float* nYa, const float* nZa,
                        const float* ysA, const uint32_t* maskA, float* uTau, uint16_t* uwx, uint16_t* uwy,
                        uint16_t* uwz, float nu, float utCut, float ema, float* stats) {
    const long long N = (long long)nx * ny * nz;
    float sumY = 0.0f, maxY = 0.0f;
    int active = 0, clamped = 0;
    for (int i = 0; i < count; ++i) {
        const long long cell = cellIdx[i];
        const float nX = nXa[i], nY = nYa[i], nZ = nZa[i];
        const long long ps = sampleIdx[i];
        float rho = 0.0f, jx = 0.0f, jy = 0.0f, jz = 0.0f;
        for (int q = 0; q < Q; ++q) {
            const float fq = f[q * N + ps];
            rho += fq; jx += CX[q] * fq; jy += CY[q] * fq; jz += CZ[q] * fq;
        }
        rho = std::fmax(rho, 0.05f);
        const float inv = 1.0f / rho;
        const float ux = jx * inv, uy = jy * inv, uz = jz * inv;
        const float un = ux * nX + uy * nY + uz * nZ;
        const float tx = ux - un * nX, ty = uy - un * nY, tz = uz - un * nZ;
        const float ut = std::sqrt(tx * tx + ty * ty + tz * tz);
        if (ut < utCut) {
            uTau[i] = 0.0f;
            uwx[cell] = 0; uwy[cell] = 0; uwz[cell] = 0;
            continue;
        }
        const float itx = tx / ut, ity = ty / ut, itz = tz / ut;
        const float prev = uTau[i];
        const float solved = solve_utau(ut, ysA[i], nu, prev);
        const float utau = prev > 0.0f ? prev + ema * (solved - prev) : solved;
        uTau[i] = utau;
        float m0 = 0.0f, dcoef = 0.0f;
        const uint32_t mask = maskA[i];
        for (int q = 1; q < Q; ++q) {
            if (!(mask & (1u << q))) continue;
            const int o = OPP[q];
            const float ct = -(CX[q] * itx + CY[q] * ity + CZ[q] * itz);
            const float fo = f[o * N + cell];
            m0 += 2.0f * fo * ct;
            dcoef += 6.0f * W<float>(q) * ct * ct;
        }
        const float maxN = std::fmax(std::fabs(nX), std::fmax(std::fabs(nY), std::fabs(nZ)));
        const float aw = 1.0f / std::fmax(maxN, 0.1f);
        float uw = 0.0f;
        if (dcoef > 1e-6f) {
            const float target = rho * utau * utau * aw;
            const float sgn = m0 >= 0.0f ? 1.0f : -1.0f;
            uw = (m0 - sgn * target) / dcoef;
        }
        const float ypS = ysA[i] * utau / nu;
        const float fade = std::fmin(std::fmax((ypS - 3.0f) / (6.0f - 3.0f), 0.0f), 1.0f);
        uw *= fade;
        const float cap = std::fmin(0.5f * ut, 0.5f * 0.30f);
        const float uwc = std::fmin(std::fmax(uw, -cap), cap);
        uwx[cell] = f2h(uwc * itx); uwy[cell] = f2h(uwc * ity); uwz[cell] = f2h(uwc * itz);
        const float yplus = ysA[i] * utau / nu;
        sumY += yplus;
        maxY = std::fmax(maxY, std::fmax(yplus, 0.0f));
        ++active;
        if (uwc != uw) ++clamped;
    }
    stats[0] = sumY; stats[1] = maxY; stats[2] = (float)active; stats[3] = (float)clamped;
}

/// Full Newton on Reichardt in FP64 to a relative step below tol (the u_tau
/// judge): returns the converged u_tau for each sample.
void oracle_utau_newton_f64(int n, const double* ut, const double* ys, const double* nu, double tol,
                            int maxIter, double* out) {
    const double kappa = 0.41, C = 7.8;
    for (int i = 0; i < n; ++i) {
        double u = std::fmax(0.04 * ut[i], std::sqrt(nu[i] * ut[i] / ys[i]));
        for (int it = 0; it < maxIter; ++it) {
            const double yp = std::fmax(ys[i] * u / nu[i], 1e-12);
            const double e11 = std::exp(-yp / 11.0), e3 = std::exp(-yp / 3.0);
            const double up = std::log(1.0 + kappa * yp) / kappa + C * (1.0 - e11 - (yp / 11.0) * e3);
            const double dup = 1.0 / (1.0 + kappa * yp) + C * (e11 / 11.0 - e3 / 11.0 + (yp / 33.0) * e3);
            const double g = u * up - ut[i];
            const double dg = up + yp * dup;
            const double step = g / dg;
            u -= step;
            if (u < 0) u = 0;
            if (std::fabs(step) <= tol * std::fmax(u, 1e-300)) break;
        }
        out[i] = u;
    }
}

/// Warm-restart flag-edit fixup (lbm_core.cu:644-717): mask 1 = newly solid
/// (both buffers zeroed), 2 = newly fluid (equilibrium of the mean rho/u of
/// the neighbours that are fluid and unedited, read from fA; rest state if
/// none). flags = the new flags. FP32, reference operation order.
void oracle_apply_flag_edits(int nx, int ny, int nz, float* fA, float* fB, const uint8_t* flags,
                             const uint8_t* mask) {
    const Dims d{nx, ny, nz};
    const long long N = d.n();
    std::vector<float> a(fA, fA + Q * N);  // neighbours read the pre-edit state
    for (long long cell = 0; cell < N; ++cell) {
        const uint8_t edit = mask[cell];
        if (edit == 0) continue;
        if (edit == 1) {
            for (int q = 0; q < Q; ++q) { fA[q * N + cell] = 0.0f; fB[q * N + cell] = 0.0f; }
            continue;
        }
        const int z = (int)(cell / ((long long)nx * ny));
        const long long rem = cell - (long long)z * nx * ny;
        const int y = (int)(rem / nx), x = (int)(rem - (long long)y * nx);
        float rho = 0.0f, ux = 0.0f, uy = 0.0f, uz = 0.0f;
        int found = 0;
        for (int q = 1; q < Q; ++q) {
            const int xn = x + CX[q], yn = y + CY[q], zn = z + CZ[q];
            if (xn < 0 || xn >= nx || yn < 0 || yn >= ny) continue;
            const int znw = zn < 0 ? nz - 1 : (zn >= nz ? 0 : zn);
            const long long nc = d.at(xn, yn, znw);
            if (flags[nc] != FLUID || mask[nc] != 0) continue;
            float r = 0.0f, jx = 0.0f, jy = 0.0f, jz = 0.0f;
            for (int p = 0; p < Q; ++p) {
                const float fq = a[p * N + nc];
                r += fq;
                jx += (float)CX[p] * fq; jy += (float)CY[p] * fq; jz += (float)CZ[p] * fq;
            }
            rho += r;
            ux += jx / r; uy += jy / r; uz += jz / r;
            ++found;
        }
        if (found > 0) {
            const float inv = 1.0f / (float)found;
            rho *= inv; ux *= inv; uy *= inv; uz *= inv;
        } else {
            rho = 1.0f; ux = uy = uz = 0.0f;
        }
        float feq[Q];
        equilibrium19<float>(rho, ux, uy, uz, feq);
        for (int q = 0; q < Q; ++q) { fA[q * N + cell] = feq[q]; fB[q * N + cell] = feq[q]; }
    }
}

uint16_t oracle_f2h(float f) { return f2h(f); }
float oracle_h2f(uint16_t h) { return h2f(h); }

// ---- refinement (reference lbm_refine.cu:70-429), FP32 -------------------

/// Projection of f_neq onto its second-order Hermite moments
/// (lbm_refine.cu:70-97 regularizeFneq).
static void regularize(float fneq[Q]) {
    float pxx = 0, pyy = 0, pzz = 0, pxy = 0, pxz = 0, pyz = 0;
    for (int q = 0; q < Q; ++q) {
        const float f = fneq[q];
        const float cx = (float)CX[q], cy = (float)CY[q], cz = (float)CZ[q];
        pxx += cx * cx * f; pyy += cy * cy * f; pzz += cz * cz * f;
        pxy += cx * cy * f; pxz += cx * cz * f; pyz += cy * cz * f;
    }
    const float trace = (1.0f / 3.0f) * (pxx + pyy + pzz);
    for (int q = 0; q < Q; ++q) {
        const float cx = (float)CX[q], cy = (float)CY[q], cz = (float)CZ[q];
        const float qPi = cx * cx * pxx + cy * cy * pyy + cz * cz * pzz
                        + 2.0f * (cx * cy * pxy + cx * cz * pxz + cy * cz * pyz) - trace;
        fneq[q] = 4.5f * W<float>(q) * qPi;
    }
}

/// coarseToFineFillKernel over every fine cell (fullVolume: all non-solid;
/// otherwise Interface cells only).
void oracle_fill_c2f(int cnx, int cny, int cnz, const float* cT0, const float* cT1, const uint8_t* cflags,
                     int fnx, int fny, int fnz, float* ff, const uint8_t* fflags, int boxX0, int boxY0,
                     int factor, float tw, float neqScale, int fullVolume) {
    const Dims cd{cnx, cny, cnz}, fd{fnx, fny, fnz};
    const long long CN = cd.n(), FN = fd.n();
    const float invF = 1.0f / (float)factor;
#pragma omp parallel for schedule(static)
    for (long long cell = 0; cell < FN; ++cell) {
        const uint8_t fl = fflags[cell];
        if (fullVolume ? (fl == SOLID) : (fl != IFACE)) continue;
        const int zf = (int)(cell / ((long long)fnx * fny));
        const long long rem = cell - (long long)zf * fnx * fny;
        const int yf = (int)(rem / fnx), xf = (int)(rem - (long long)yf * fnx);
        const float gx = (float)boxX0 + ((float)xf + 0.5f) * invF - 0.5f;
        const float gy = (float)boxY0 + ((float)yf + 0.5f) * invF - 0.5f;
        const float gz = ((float)zf + 0.5f) * invF - 0.5f;
        const int ix = (int)std::floor(gx), iy = (int)std::floor(gy), iz = (int)std::floor(gz);
        const float tx = gx - (float)ix, ty = gy - (float)iy, tz = gz - (float)iz;
        float wgt[8];
        wgt[0] = (1 - tx) * (1 - ty) * (1 - tz);
        wgt[1] = tx * (1 - ty) * (1 - tz);
        wgt[2] = (1 - tx) * ty * (1 - tz);
        wgt[3] = tx * ty * (1 - tz);
        wgt[4] = (1 - tx) * (1 - ty) * tz;
        wgt[5] = tx * (1 - ty) * tz;
        wgt[6] = (1 - tx) * ty * tz;
        wgt[7] = tx * ty * tz;
        long long corner[8];
        for (int c = 0; c < 8; ++c)
            corner[c] = cd.at(wrap(ix + (c & 1), cnx), wrap(iy + ((c >> 1) & 1), cny), wrap(iz + ((c >> 2) & 1), cnz));
        float wsum = 0.0f;
        for (int c = 0; c < 8; ++c) {
            if (cflags[corner[c]] == SOLID) wgt[c] = 0.0f;
            wsum += wgt[c];
        }
        if (wsum < 1e-6f) continue;
        const float iws = 1.0f / wsum;
        for (int c = 0; c < 8; ++c) wgt[c] *= iws;
        float fi[Q];
        float rho = 0, jx = 0, jy = 0, jz = 0;
        for (int q = 0; q < Q; ++q) {
            float s0 = 0, s1 = 0;
            for (int c = 0; c < 8; ++c) {
                s0 += wgt[c] * cT0[q * CN + corner[c]];
                s1 += wgt[c] * cT1[q * CN + corner[c]];
            }
            const float fq = s0 + tw * (s1 - s0);
            fi[q] = fq;
            rho += fq; jx += CX[q] * fq; jy += CY[q] * fq; jz += CZ[q] * fq;
        }
        rho = std::fmax(rho, 0.05f);
        const float invRho = 1.0f / rho;
        float ux = jx * invRho, uy = jy * invRho, uz = jz * invRho;
        const float u2 = ux * ux + uy * uy + uz * uz;
        if (u2 > 0.30f * 0.30f) {
            const float sc = 0.30f * (1.0f / std::sqrt(u2));
            ux *= sc; uy *= sc; uz *= sc;
        }
        float feq[Q], fneq[Q];
        equilibrium19<float>(rho, ux, uy, uz, feq);
        for (int q = 0; q < Q; ++q) fneq[q] = fi[q] - feq[q];
        regularize(fneq);
        for (int q = 0; q < Q; ++q) ff[q * FN + cell] = feq[q] + neqScale * fneq[q];
    }
}

/// Mean of the m^3 non-solid children of one coarse cell, its moments and
/// f_neq (lbm_refine.cu:274-318 childAvgFneq).
static bool child_avg(const float* ff, const uint8_t* fflags, const Dims& fd, int fx, int fy, int fz, int m,
                      float fneqOut[Q], float& rO, float& uxO, float& uyO, float& uzO) {
    const long long FN = fd.n();
    float fi[Q];
    for (int q = 0; q < Q; ++q) fi[q] = 0.0f;
    int nFluid = 0;
    for (int k = 0; k < m; ++k)
        for (int j = 0; j < m; ++j)
            for (int i = 0; i < m; ++i) {
                const long long c = fd.at(fx + i, fy + j, fz + k);
                if (fflags[c] == SOLID) continue;
                ++nFluid;
                for (int q = 0; q < Q; ++q) fi[q] += ff[q * FN + c];
            }
    if (nFluid == 0) return false;
    const float invN = 1.0f / (float)nFluid;
    float rho = 0, jx = 0, jy = 0, jz = 0;
    for (int q = 0; q < Q; ++q) {
        fi[q] *= invN;
        rho += fi[q]; jx += CX[q] * fi[q]; jy += CY[q] * fi[q]; jz += CZ[q] * fi[q];
    }
    rho = std::fmax(rho, 0.05f);
    const float invRho = 1.0f / rho;
    float ux = jx * invRho, uy = jy * invRho, uz = jz * invRho;
    const float u2 = ux * ux + uy * uy + uz * uz;
    if (u2 > 0.30f * 0.30f) {
        const float sc = 0.30f * (1.0f / std::sqrt(u2));
        ux *= sc; uy *= sc; uz *= sc;
    }
    float feq[Q];
    equilibrium19<float>(rho, ux, uy, uz, feq);
    for (int q = 0; q < Q; ++q) fneqOut[q] = fi[q] - feq[q];
    rO = rho; uxO = ux; uyO = uy; uzO = uz;
    return true;
}

/// fineToCoarseRestrictKernel (band 2, blend ramp 3).
void oracle_restrict_f2c(int fnx, int fny, int fnz, const float* ff, const uint8_t* fflags, int cnx, int cny,
                         int cnz, float* fc, const uint8_t* cflags, int boxX0, int boxY0, int boxX1, int boxY1,
                         int factor, float neqScaleInv, float* mr, float* mu, float* mv, float* mw) {
    const Dims cd{cnx, cny, cnz}, fd{fnx, fny, fnz};
    const long long CN = cd.n();
    const int rx0 = boxX0 + 2, ry0 = boxY0 + 2, rx1 = boxX1 - 2, ry1 = boxY1 - 2;
    const int rw = rx1 - rx0, rh = ry1 - ry0;
    if (rw <= 0 || rh <= 0) return;
    const long long total = (long long)rw * rh * cnz;
    // Restriction reads fine data only and writes disjoint coarse cells.
#pragma omp parallel for schedule(static)
    for (long long t = 0; t < total; ++t) {
        const int zc = (int)(t / ((long long)rw * rh));
        const long long rem = t - (long long)zc * rw * rh;
        const int yc = ry0 + (int)(rem / rw), xc = rx0 + (int)(rem % rw);
        const long long cCell = cd.at(xc, yc, zc);
        if (cflags[cCell] != FLUID) continue;
        const int dEdge = std::min(std::min(xc - rx0, rx1 - 1 - xc), std::min(yc - ry0, ry1 - 1 - yc));
        const float blend = std::fmin(1.0f, (float)(dEdge + 1) / (float)(3 + 1));
        float fneqC[Q], rho, ux, uy, uz;
        if (!child_avg(ff, fflags, fd, factor * (xc - boxX0), factor * (yc - boxY0), factor * zc, factor, fneqC,
                       rho, ux, uy, uz))
            continue;
        float fneqF[Q];
        for (int q = 0; q < Q; ++q) fneqF[q] = fneqC[q];
        int nS = 1;
        for (int nb = 1; nb < Q; ++nb) {
            const int nxc = xc + CX[nb], nyc = yc + CY[nb], nzc = zc + CZ[nb];
            if (nxc < rx0 || nxc >= rx1 || nyc < ry0 || nyc >= ry1) continue;
            const int nzw = (nzc + cnz) % cnz;
            float fneqN[Q], a, b, c, e;
            if (!child_avg(ff, fflags, fd, factor * (nxc - boxX0), factor * (nyc - boxY0), factor * nzw, factor,
                           fneqN, a, b, c, e))
                continue;
            for (int q = 0; q < Q; ++q) fneqF[q] += fneqN[q];
            ++nS;
        }
        const float invS = 1.0f / (float)nS;
        for (int q = 0; q < Q; ++q) fneqF[q] *= invS;
        regularize(fneqF);
        float feq[Q];
        equilibrium19<float>(rho, ux, uy, uz, feq);
        float br = 0, bjx = 0, bjy = 0, bjz = 0;
        for (int q = 0; q < Q; ++q) {
            const long long idx = q * CN + cCell;
            const float restricted = feq[q] + neqScaleInv * fneqF[q];
            const float existing = fc[idx];
            const float bl = existing + blend * (restricted - existing);
            fc[idx] = bl;
            br += bl; bjx += CX[q] * bl; bjy += CY[q] * bl; bjz += CZ[q] * bl;
        }
        if (mr) {
            br = std::fmax(br, 0.05f);
            const float bi = 1.0f / br;
            mr[cCell] = br; mu[cCell] = bjx * bi; mv[cCell] = bjy * bi; mw[cCell] = bjz * bi;
        }
    }
}

} // extern "C"

// ---- whole-tunnel driver (the reference stepN cadence, ping-pong buffers) --
// ORACLE - test infrastructure only; used as the timed CPU baseline.
namespace {
struct WallLevel {
    std::vector<long long> cell, sample;
    std::vector<float> nx, ny, nz, ys, utau;
    std::vector<uint32_t> mask;
    std::vector<uint16_t> uw[3];
};
struct Tunnel {
    Dims cd{0, 0, 0}, fd{0, 0, 0};
    std::vector<float> fc[2], ff[2];
    std::vector<uint8_t> cflags, fflags;
    int csrc = 0, fsrc = 0;
    bool fine = false;
    int box[4] = {0, 0, 0, 0}, m = 2;
    float tau = 0.6f, u = 0.08f, smag = 0.0f, lambda = 3.0f / 16.0f;
    WallLevel wc, wf;
    bool wmc = false, wmf = false;
    double force[3] = {0, 0, 0};
    std::vector<float> mr, mu, mv, mw;
};
} // namespace

extern "C" {

void* oracle_tunnel_create(int nx, int ny, int nz, const uint8_t* flags, const float* f0, float tau, float u,
                           float smagPre, float lambda) {
    auto* t = new Tunnel();
    t->cd = Dims{nx, ny, nz};
    const long long n = t->cd.n();
    t->cflags.assign(flags, flags + n);
    t->fc[0].assign(f0, f0 + 19 * n);
    // The other buffer holds the solver's reset state (equilibrium at u plus
    // the speck), as after LBMSolver::reset with the ramps off.
    t->fc[1].assign(19 * n, 0.0f);
    oracle_init_eq(nx, ny, nz, t->fc[1].data(), flags, u);
    oracle_speck(nx, ny, nz, t->fc[1].data(), flags, 1e-3f * u, 0x5eedu);
    t->tau = tau; t->u = u; t->smag = smagPre; t->lambda = lambda;
    t->mr.resize(n); t->mu.resize(n); t->mv.resize(n); t->mw.resize(n);
    return t;
}

void oracle_tunnel_destroy(void* p) { delete static_cast<Tunnel*>(p); }

void oracle_tunnel_refine(void* p, int x0, int y0, int x1, int y1, int m, const uint8_t* fflags) {
    auto* t = static_cast<Tunnel*>(p);
    t->fine = true;
    t->box[0] = x0; t->box[1] = y0; t->box[2] = x1; t->box[3] = y1; t->m = m;
    t->fd = Dims{m * (x1 - x0), m * (y1 - y0), m * t->cd.nz};
    const long long fn = t->fd.n();
    t->fflags.assign(fflags, fflags + fn);
    t->ff[0].assign(19 * fn, 0.0f);
    const float tf = (float)m * (t->tau - 0.5f) + 0.5f;
    const float* cs = t->fc[t->csrc].data();
    oracle_fill_c2f(t->cd.nx, t->cd.ny, t->cd.nz, cs, cs, t->cflags.data(), t->fd.nx, t->fd.ny, t->fd.nz,
                    t->ff[0].data(), t->fflags.data(), x0, y0, m, 0.0f, tf / ((float)m * t->tau), 1);
    t->ff[1] = t->ff[0];
}

void oracle_tunnel_wall(void* p, int level, int count, const long long* cell, const long long* sample,
                        const float* nx, const float* ny, const float* nz, const float* ys, const uint32_t* mask) {
    auto* t = static_cast<Tunnel*>(p);
    WallLevel& w = level == 0 ? t->wc : t->wf;
    const long long n = level == 0 ? t->cd.n() : t->fd.n();
    w.cell.assign(cell, cell + count); w.sample.assign(sample, sample + count);
    w.nx.assign(nx, nx + count); w.ny.assign(ny, ny + count); w.nz.assign(nz, nz + count);
    w.ys.assign(ys, ys + count); w.mask.assign(mask, mask + count);
    w.utau.assign(count, 0.0f);
    for (auto& a : w.uw) a.assign(n, 0);
    (level == 0 ? t->wmc : t->wmf) = true;
}

/// n coarse steps with the reference cadence (lbm_solver.cpp:1132-1390
/// stepN: coarse collide, m fine sub-steps of fill + collide, restriction,
/// per-batch force and wall-model update); returns 0.
int oracle_tunnel_step(void* p, int n) {
    auto* t = static_cast<Tunnel*>(p);
    const long long cn = t->cd.n();
    for (int i = 0; i < n; ++i) {
        const int wm = i == n - 1;
        float* src = t->fc[t->csrc].data();
        float* dst = t->fc[1 - t->csrc].data();
        collide<float>(t->cd, src, dst, t->cflags.data(), t->tau, t->lambda, t->smag, t->u, wm, t->mr.data(),
                       t->mu.data(), t->mv.data(), t->mw.data(), t->wmc ? t->wc.uw[0].data() : nullptr,
                       t->wmc ? t->wc.uw[1].data() : nullptr, t->wmc ? t->wc.uw[2].data() : nullptr);
        if (t->fine) {
            const int m = t->m;
            const float tc = t->tau, tf = (float)m * (tc - 0.5f) + 0.5f;
            for (int k = 0; k < m; ++k) {
                oracle_fill_c2f(t->cd.nx, t->cd.ny, t->cd.nz, src, dst, t->cflags.data(), t->fd.nx, t->fd.ny,
                                t->fd.nz, t->ff[t->fsrc].data(), t->fflags.data(), t->box[0], t->box[1], m,
                                (float)k / (float)m, tf / ((float)m * tc), 0);
                collide<float>(t->fd, t->ff[t->fsrc].data(), t->ff[1 - t->fsrc].data(), t->fflags.data(), tf,
                               t->lambda, t->smag, t->u, 0, nullptr, nullptr, nullptr, nullptr,
                               t->wmf ? t->wf.uw[0].data() : nullptr, t->wmf ? t->wf.uw[1].data() : nullptr,
                               t->wmf ? t->wf.uw[2].data() : nullptr);
                t->fsrc = 1 - t->fsrc;
            }
            oracle_restrict_f2c(t->fd.nx, t->fd.ny, t->fd.nz, t->ff[t->fsrc].data(), t->fflags.data(), t->cd.nx,
                                t->cd.ny, t->cd.nz, dst, t->cflags.data(), t->box[0], t->box[1], t->box[2],
                                t->box[3], m, ((float)m * tc) / tf, wm ? t->mr.data() : nullptr,
                                wm ? t->mu.data() : nullptr, wm ? t->mv.data() : nullptr,
                                wm ? t->mw.data() : nullptr);
        }
        t->csrc = 1 - t->csrc;
    }
    force<float>(t->cd, t->fc[t->csrc].data(), t->cflags.data(), t->wmc ? t->wc.uw[0].data() : nullptr,
                 t->wmc ? t->wc.uw[1].data() : nullptr, t->wmc ? t->wc.uw[2].data() : nullptr, t->force);
    const float nu = (t->tau - 0.5f) / 3.0f, cut = 1e-3f * t->u;
    float st[4];
    if (t->wmc && !t->wc.cell.empty())
        oracle_wall_update(t->cd.nx, t->cd.ny, t->cd.nz, t->fc[t->csrc].data(), (int)t->wc.cell.size(),
                           t->wc.cell.data(), t->wc.sample.data(), t->wc.nx.data(), t->wc.ny.data(),
                           t->wc.nz.data(), t->wc.ys.data(), t->wc.mask.data(), t->wc.utau.data(),
                           t->wc.uw[0].data(), t->wc.uw[1].data(), t->wc.uw[2].data(), nu, cut, 0.25f, st);
    if (t->fine && t->wmf && !t->wf.cell.empty()) {
        const float tf = (float)t->m * (t->tau - 0.5f) + 0.5f;
        oracle_wall_update(t->fd.nx, t->fd.ny, t->fd.nz, t->ff[t->fsrc].data(), (int)t->wf.cell.size(),
                           t->wf.cell.data(), t->wf.sample.data(), t->wf.nx.data(), t->wf.ny.data(),
                           t->wf.nz.data(), t->wf.ys.data(), t->wf.mask.data(), t->wf.utau.data(),
                           t->wf.uw[0].data(), t->wf.uw[1].data(), t->wf.uw[2].data(), (tf - 0.5f) / 3.0f, cut,
                           0.25f, st);
    }
    (void)cn;
    return 0;
}

void oracle_tunnel_state(void* p, int level, float* out) {
    auto* t = static_cast<Tunnel*>(p);
    if (level == 0) std::memcpy(out, t->fc[t->csrc].data(), t->fc[t->csrc].size() * 4);
    else std::memcpy(out, t->ff[t->fsrc].data(), t->ff[t->fsrc].size() * 4);
}

void oracle_tunnel_force(void* p, double* out) {
    auto* t = static_cast<Tunnel*>(p);
    out[0] = t->force[0]; out[1] = t->force[1]; out[2] = t->force[2];
}

int oracle_threads() {
#ifdef _OPENMP
    int n = 1;
#pragma omp parallel
    {
#pragma omp single
        n = omp_get_num_threads();
    }
    return n;
#else
    return 1;
#endif
}

} // extern "C"
