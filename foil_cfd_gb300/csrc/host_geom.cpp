// Host-side builders: the wall-model cell list (reference
// src/sim/wall_model.cpp:55-236) and the geometry of the tunnels (domain
// boundary flags, NACA 4-digit sections, point-in-polygon airfoil
// voxelisation, trailing-edge gap closure, the interface shell of a
// refinement patch, and the patch box), following src/geom/voxelizer.cpp and
// src/geom/airfoil.cpp:177-266. The device builders (geom_kernels.cu) produce
// the same bytes.
#include "host_geom.h"

#include <algorithm>
#include <cmath>
#include <thread>

namespace fcfd {
namespace {

constexpr int kNormalRadius = 2;          // 5^3 occupancy stencil
constexpr float kDegenerateEps = 1e-3f;   // |gradient| below: no usable normal

inline int wrap_z(int z, int nz) { return z < 0 ? z + nz : (z >= nz ? z - nz : z); }

inline long long idx(int x, int y, int z, const LevelDims& d) {
    return static_cast<long long>(x) + static_cast<long long>(d.nx) * (y + static_cast<long long>(d.ny) * z);
}

/// Solid test with x/y out of range = not solid and periodic z.
inline bool solid_at(const std::uint8_t* f, const LevelDims& d, int x, int y, int z) {
    if (x < 0 || x >= d.nx || y < 0 || y >= d.ny) return false;
    return f[idx(x, y, wrap_z(z, d.nz), d)] == kFlagSolidHost;
}

void scan_slab(const LevelDims& d, const std::uint8_t* active, const std::uint8_t* clean,
               int sampleCells, int z0, int z1, WallList& out, WallListStats& st) {
    for (int z = z0; z < z1; ++z)
        for (int y = 0; y < d.ny; ++y)
            for (int x = 0; x < d.nx; ++x) {
                const long long c = idx(x, y, z, d);
                if (active[c] != kFlagFluidHost) continue;
                std::uint32_t mask = 0;
                bool vgOnly = false;
                for (int q = 1; q < 19; ++q) {
                    const int sx = x - kHostCx[q], sy = y - kHostCy[q], sz = z - kHostCz[q];
                    if (!solid_at(active, d, sx, sy, sz)) continue;
                    mask |= 1u << q;
                    if (!solid_at(clean, d, sx, sy, sz)) vgOnly = true;
                }
                if (mask == 0) continue;
                if (vgOnly) { ++st.excludedVG; continue; }
                float gx = 0.f, gy = 0.f, gz = 0.f;
                for (int dz = -kNormalRadius; dz <= kNormalRadius; ++dz)
                    for (int dy = -kNormalRadius; dy <= kNormalRadius; ++dy)
                        for (int dx = -kNormalRadius; dx <= kNormalRadius; ++dx)
                            if (solid_at(clean, d, x + dx, y + dy, z + dz)) {
                                gx += static_cast<float>(dx);
                                gy += static_cast<float>(dy);
                                gz += static_cast<float>(dz);
                            }
                const float gm = std::sqrt(gx * gx + gy * gy + gz * gz);
                if (gm < kDegenerateEps) { ++st.degenerate; continue; }
                const float nX = -gx / gm, nY = -gy / gm, nZ = -gz / gm;
                long long sample = c;
                int sx = x, sy = y, sz = z;
                for (int k = sampleCells; k >= 1; --k) {
                    const int tx = x + static_cast<int>(std::lround(nX * k));
                    const int ty = y + static_cast<int>(std::lround(nY * k));
                    const int tz = wrap_z(z + static_cast<int>(std::lround(nZ * k)), d.nz);
                    if (tx < 0 || tx >= d.nx || ty < 0 || ty >= d.ny) continue;
                    const long long cand = idx(tx, ty, tz, d);
                    if (active[cand] != kFlagFluidHost) continue;
                    sample = cand; sx = tx; sy = ty; sz = tz;
                    break;
                }
                int dzw = sz - z;
                if (dzw > d.nz / 2) dzw -= d.nz;
                if (dzw < -d.nz / 2) dzw += d.nz;
                const float proj = static_cast<float>(sx - x) * nX + static_cast<float>(sy - y) * nY
                                 + static_cast<float>(dzw) * nZ;
                out.cellIdx.push_back(c);
                out.sampleIdx.push_back(sample);
                out.nX.push_back(nX);
                out.nY.push_back(nY);
                out.nZ.push_back(nZ);
                out.ys.push_back(0.5f + std::max(proj, 0.0f));
                out.linkMask.push_back(mask);
                ++st.listed;
            }
}

template <class T>
void append(std::vector<T>& a, const std::vector<T>& b) { a.insert(a.end(), b.begin(), b.end()); }

} // namespace

WallList build_wall_list(const LevelDims& d, const std::uint8_t* active, const std::uint8_t* clean,
                         int sampleCells, WallListStats* stats) {
    WallList merged;
    WallListStats tally;
    if (d.cells() <= 0 || !active || !clean) {
        if (stats) *stats = tally;
        return merged;
    }
    // z slabs on all hardware threads, merged in slab order: the result is
    // the sequential x-fastest order whatever the thread count.
    const int hw = std::max(1, static_cast<int>(std::thread::hardware_concurrency()));
    const int slabs = std::clamp(std::min(hw, d.nz), 1, 64);
    std::vector<WallList> parts(slabs);
    std::vector<WallListStats> pst(slabs);
    std::vector<std::thread> pool;
    for (int s = 0; s < slabs; ++s) {
        const int z0 = static_cast<int>(static_cast<long long>(d.nz) * s / slabs);
        const int z1 = static_cast<int>(static_cast<long long>(d.nz) * (s + 1) / slabs);
        pool.emplace_back(scan_slab, std::cref(d), active, clean, sampleCells, z0, z1,
                          std::ref(parts[s]), std::ref(pst[s]));
    }
    for (auto& t : pool) t.join();
    for (int s = 0; s < slabs; ++s) {
        append(merged.cellIdx, parts[s].cellIdx);
        append(merged.sampleIdx, parts[s].sampleIdx);
        append(merged.nX, parts[s].nX);
        append(merged.nY, parts[s].nY);
        append(merged.nZ, parts[s].nZ);
        append(merged.ys, parts[s].ys);
        append(merged.linkMask, parts[s].linkMask);
        tally.listed += pst[s].listed;
        tally.excludedVG += pst[s].excludedVG;
        tally.degenerate += pst[s].degenerate;
    }
    if (stats) *stats = tally;
    return merged;
}

void boundary_flags(const LevelDims& d, std::uint8_t* f) {
    for (int z = 0; z < d.nz; ++z)
        for (int y = 0; y < d.ny; ++y) {
            std::uint8_t* row = f + idx(0, y, z, d);
            for (int x = 0; x < d.nx; ++x) row[x] = kFlagFluidHost;
            if (y == 0) for (int x = 0; x < d.nx; ++x) row[x] = 5;          // SlipBottom
            if (y == d.ny - 1) for (int x = 0; x < d.nx; ++x) row[x] = 4;   // SlipTop
            row[0] = 2;                                                     // Inlet wins corners
            if (y != 0 && y != d.ny - 1) row[d.nx - 1] = 3;                // Outlet yields
        }
}

int naca4(const char* digits, int pps, std::vector<float>& xy) {
    xy.clear();
    if (!digits) return -1;
    for (int i = 0; i < 4; ++i)
        if (digits[i] < '0' || digits[i] > '9') return -1;
    if (digits[4] != '\0') return -1;
    const float m = static_cast<float>(digits[0] - '0') / 100.0f;
    const float p = static_cast<float>(digits[1] - '0') / 10.0f;
    const float t = static_cast<float>((digits[2] - '0') * 10 + (digits[3] - '0')) / 100.0f;
    if (t <= 0.0f || (m > 0.0f && p <= 0.0f)) return -1;
    const int n = std::max(pps, 20);
    const float pi = 3.14159265358979f;
    auto station = [&](int k, float& ux, float& uy, float& lx, float& ly) {
        const float x = 0.5f * (1.0f - std::cos(pi * static_cast<float>(k) / static_cast<float>(n - 1)));
        const float sq = std::sqrt(x);
        // Closed trailing edge: last coefficient -0.1036 makes yt(1) = 0.
        const float yt = 5.0f * t * (0.2969f * sq - 0.1260f * x - 0.3516f * x * x
                                     + 0.2843f * x * x * x - 0.1036f * x * x * x * x);
        float yc = 0.0f, dyc = 0.0f;
        if (m > 0.0f) {
            if (x < p) {
                yc = (m / (p * p)) * (2.0f * p * x - x * x);
                dyc = (2.0f * m / (p * p)) * (p - x);
            } else {
                yc = (m / ((1.0f - p) * (1.0f - p))) * ((1.0f - 2.0f * p) + 2.0f * p * x - x * x);
                dyc = (2.0f * m / ((1.0f - p) * (1.0f - p))) * (p - x);
            }
        }
        const float th = std::atan(dyc), st = std::sin(th), ct = std::cos(th);
        ux = x - yt * st; uy = yc + yt * ct;
        lx = x + yt * st; ly = yc - yt * ct;
    };
    // Selig loop: TE -> upper -> LE -> lower -> TE.
    for (int k = n - 1; k >= 0; --k) {
        float ux, uy, lx, ly;
        station(k, ux, uy, lx, ly);
        xy.push_back(ux); xy.push_back(uy);
    }
    for (int k = 1; k < n; ++k) {
        float ux, uy, lx, ly;
        station(k, ux, uy, lx, ly);
        xy.push_back(lx); xy.push_back(ly);
    }
    return static_cast<int>(xy.size() / 2);
}

void foil_rotation(float aoaDeg, float& c, float& s) {
    const float pi = 3.14159265358979f;
    const float a = aoaDeg * pi / 180.0f;
    c = std::cos(-a);
    s = std::sin(-a);
}

void voxelize_airfoil(const LevelDims& d, const float* xy, int npts, float aoaDeg, int chordCells,
                      float ax, float ay, std::uint8_t* flags) {
    // An outline of fewer than 20 points is not a valid section: nothing is
    // stamped (AirfoilGeometry::isValid, src/geom/airfoil.h:37).
    if (d.nx < 3 || d.ny < 3 || d.nz < 1 || npts < kMinOutlinePoints) return;
    float ca, sa;
    foil_rotation(aoaDeg, ca, sa);
    const float chord = static_cast<float>(chordCells);
    std::vector<float> px(npts), py(npts);
    float minY = 1e30f, maxY = -1e30f;
    for (int i = 0; i < npts; ++i) {
        // Rotate about the quarter chord by -AoA (nose up), then scale.
        const float rx = xy[2 * i] - 0.25f, ry = xy[2 * i + 1];
        const float qx = rx * ca - ry * sa, qy = rx * sa + ry * ca;
        px[i] = ax + qx * chord;
        py[i] = ay + qy * chord;
        minY = std::min(minY, py[i]);
        maxY = std::max(maxY, py[i]);
    }
    const int y0 = std::clamp(static_cast<int>(std::floor(minY - 0.5f)), 1, d.ny - 2);
    const int y1 = std::clamp(static_cast<int>(std::ceil(maxY - 0.5f)), 1, d.ny - 2);
    std::vector<std::uint8_t> mask(static_cast<size_t>(d.nx) * d.ny, 0);
    std::vector<float> cr;
    for (int y = y0; y <= y1; ++y) {
        const float yc = static_cast<float>(y) + 0.5f;
        cr.clear();
        for (int i = 0; i < npts; ++i) {
            const int j = (i + 1) % npts;
            if ((py[i] > yc) != (py[j] > yc)) {
                const float t = (yc - py[i]) / (py[j] - py[i]);
                cr.push_back(px[i] + t * (px[j] - px[i]));
            }
        }
        std::sort(cr.begin(), cr.end());
        for (size_t k = 0; k + 1 < cr.size(); k += 2) {
            const int xa = std::max(1, static_cast<int>(std::ceil(cr[k] - 0.5f)));
            const int xb = std::min(d.nx - 2, static_cast<int>(std::floor(cr[k + 1] - 0.5f)));
            for (int x = xa; x <= xb; ++x) mask[static_cast<size_t>(y) * d.nx + x] = 1;
        }
    }
    for (int z = 0; z < d.nz; ++z)
        for (int y = y0; y <= y1; ++y)
            for (int x = 1; x < d.nx - 1; ++x) {
                std::uint8_t& c = flags[idx(x, y, z, d)];
                if (mask[static_cast<size_t>(y) * d.nx + x] && c == kFlagFluidHost) c = kFlagSolidHost;
            }
}

int close_trailing_edge_gaps(const LevelDims& d, std::uint8_t* flags) {
    if (d.nx < 3 || d.ny < 3 || d.nz < 1) return 0;
    // A fluid cell with solid directly above and below (judged on the
    // pre-closure field, so closures do not cascade) becomes solid.
    const std::vector<std::uint8_t> before(flags, flags + d.cells());
    int closed = 0;
    const long long nx = d.nx;
    for (int z = 0; z < d.nz; ++z)
        for (int y = 1; y < d.ny - 1; ++y)
            for (int x = 0; x < d.nx; ++x) {
                const long long i = idx(x, y, z, d);
                if (before[i] == kFlagFluidHost && before[i - nx] == kFlagSolidHost
                    && before[i + nx] == kFlagSolidHost) {
                    flags[i] = kFlagSolidHost;
                    ++closed;
                }
            }
    return closed;
}

void stamp_interface_shell(const LevelDims& d, std::uint8_t* flags, int shell) {
    for (int z = 0; z < d.nz; ++z)
        for (int y = 0; y < d.ny; ++y) {
            std::uint8_t* row = flags + idx(0, y, z, d);
            if (y < shell || y >= d.ny - shell) {
                for (int x = 0; x < d.nx; ++x) row[x] = 8;
            } else {
                for (int x = 0; x < shell && x < d.nx; ++x) row[x] = 8;
                for (int x = std::max(0, d.nx - shell); x < d.nx; ++x) row[x] = 8;
            }
        }
}

void derive_patch_box(const LevelDims& d, const std::uint8_t* flags, int mx0, int mx1, int my0,
                      int my1, int clearance, int out[4]) {
    int sx0 = d.nx, sx1 = -1, sy0 = d.ny, sy1 = -1;
    for (int z = 0; z < d.nz; ++z)
        for (int y = 0; y < d.ny; ++y)
            for (int x = 0; x < d.nx; ++x)
                if (flags[idx(x, y, z, d)] == kFlagSolidHost) {
                    sx0 = std::min(sx0, x); sx1 = std::max(sx1, x);
                    sy0 = std::min(sy0, y); sy1 = std::max(sy1, y);
                }
    if (sx1 < sx0) { out[0] = out[1] = out[2] = out[3] = 0; return; }
    out[0] = std::max(clearance, sx0 - mx0);
    out[1] = std::max(clearance, sy0 - my0);
    out[2] = std::min(d.nx - clearance, sx1 + 1 + mx1);
    out[3] = std::min(d.ny - clearance, sy1 + 1 + my1);
}

} // namespace fcfd
