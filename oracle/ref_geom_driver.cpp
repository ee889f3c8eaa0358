// ORACLE - test infrastructure only. C entry points over the reference's host
// geometry builders (src/geom/voxelizer.cpp, airfoil.cpp; vg.cpp and
// src/platform/platform.cpp only to resolve their symbols) and its
// computeScaling (src/sim/units.h), compiled unmodified by ref_build.py (from
// the reference tree) and ref_geom.py (from the staged kit), for golden
// vectors and the benchmark's reference arm: NACA 4-digit outlines, the
// clean-foil flag field (boundary flags + voxelised foil + trailing-edge
// closure), the fine-patch flag field (all fluid + foil + closure +
// interface shell), the derived patch box and the lattice scaling.
#include <cstring>
#include <string>

#include "units.h"
#include "voxelizer.h"

namespace {

foilcfd::DomainLayout layout_of(int nx, int ny, int nz, int chord, float axFrac, float ayFrac) {
    foilcfd::DomainLayout l;
    l.dims.nx = nx; l.dims.ny = ny; l.dims.nz = nz;
    l.chordCells = chord;
    l.foilAnchorXFrac = axFrac;
    l.foilAnchorYFrac = ayFrac;
    return l;
}

bool naca(const char* digits, int pps, foilcfd::AirfoilGeometry& out) {
    const foilcfd::AirfoilLoadResult r = foilcfd::generateNACA4(digits, pps);
    if (!r.ok) return false;
    out = r.airfoil;
    return true;
}

} // namespace

extern "C" int ref_naca4(const char* digits, int pps, float* xy, int cap) {
    foilcfd::AirfoilGeometry g;
    if (!naca(digits, pps, g)) return -1;
    const int n = static_cast<int>(g.points.size());
    if (n > cap) return -2;
    for (int i = 0; i < n; ++i) { xy[2 * i] = g.points[i].x; xy[2 * i + 1] = g.points[i].y; }
    return n;
}

// Boundary flags, voxelised foil, trailing-edge closure (buildCleanFoilFlags
// composed step by step to report the closure count).
extern "C" int ref_clean_foil_flags(const char* digits, int pps, float aoa, int nx, int ny, int nz, int chord,
                                    float axFrac, float ayFrac, unsigned char* out) {
    foilcfd::AirfoilGeometry g;
    if (!naca(digits, pps, g)) return -1;
    const foilcfd::DomainLayout l = layout_of(nx, ny, nz, chord, axFrac, ayFrac);
    std::vector<std::uint8_t> f = foilcfd::buildBoundaryFlags(l.dims);
    foilcfd::voxelizeAirfoil(g, aoa, l, f);
    const int closed = foilcfd::closeTrailingEdgeGaps(l.dims, f);
    std::memcpy(out, f.data(), f.size());
    return closed;
}

extern "C" void ref_boundary_flags(int nx, int ny, int nz, unsigned char* out) {
    foilcfd::GridDims d;
    d.nx = nx; d.ny = ny; d.nz = nz;
    const std::vector<std::uint8_t> f = foilcfd::buildBoundaryFlags(d);
    std::memcpy(out, f.data(), f.size());
}

extern "C" int ref_fine_patch_flags(const char* digits, int pps, float aoa, int nx, int ny, int nz, int chord,
                                    float axFrac, float ayFrac, int x0, int y0, int x1, int y1, int factor,
                                    unsigned char* out) {
    foilcfd::AirfoilGeometry g;
    if (!naca(digits, pps, g)) return -1;
    const foilcfd::DomainLayout l = layout_of(nx, ny, nz, chord, axFrac, ayFrac);
    foilcfd::PatchBox b;
    b.x0 = x0; b.y0 = y0; b.x1 = x1; b.y1 = y1;
    const std::vector<std::uint8_t> f = foilcfd::buildFinePatchFlags(g, aoa, l, b, factor);
    std::memcpy(out, f.data(), f.size());
    return 0;
}

extern "C" void ref_derive_patch_box(int nx, int ny, int nz, const unsigned char* flags, int mx0, int mx1, int my0,
                                     int my1, int clearance, int* box) {
    foilcfd::GridDims d;
    d.nx = nx; d.ny = ny; d.nz = nz;
    const std::vector<std::uint8_t> f(flags, flags + d.cellCount());
    const foilcfd::PatchBox b = foilcfd::derivePatchBox(d, f, mx0, mx1, my0, my1, clearance);
    box[0] = b.x0; box[1] = b.y0; box[2] = b.x1; box[3] = b.y1;
}

// voxelizeAirfoil of an arbitrary outline (>= 20 points) at an absolute
// anchor into an existing flag field (only Fluid cells become Solid).
extern "C" int ref_voxelize_points(const float* xy, int npts, float aoa, int nx, int ny, int nz, int chord, float ax,
                                   float ay, unsigned char* flags) {
    foilcfd::AirfoilGeometry g;
    for (int i = 0; i < npts; ++i) g.points.push_back(foilcfd::Vec2f(xy[2 * i], xy[2 * i + 1]));
    foilcfd::DomainLayout l;
    l.dims.nx = nx; l.dims.ny = ny; l.dims.nz = nz;
    l.chordCells = chord;
    l.anchorAbsolute = true;
    l.anchorXCells = ax;
    l.anchorYCells = ay;
    std::vector<std::uint8_t> f(flags, flags + l.dims.cellCount());
    foilcfd::voxelizeAirfoil(g, aoa, l, f);
    std::memcpy(flags, f.data(), f.size());
    return g.isValid() ? 0 : -1;
}

extern "C" int ref_close_te(int nx, int ny, int nz, unsigned char* flags) {
    foilcfd::GridDims d;
    d.nx = nx; d.ny = ny; d.nz = nz;
    std::vector<std::uint8_t> f(flags, flags + d.cellCount());
    const int closed = foilcfd::closeTrailingEdgeGaps(d, f);
    std::memcpy(flags, f.data(), f.size());
    return closed;
}

// stampInterfaceShell (voxelizer.cpp) on an existing flag field.
extern "C" void ref_stamp_interface_shell(int nx, int ny, int nz, unsigned char* flags) {
    foilcfd::GridDims d;
    d.nx = nx; d.ny = ny; d.nz = nz;
    std::vector<std::uint8_t> f(flags, flags + d.cellCount());
    foilcfd::stampInterfaceShell(d, f);
    std::memcpy(flags, f.data(), f.size());
}

// computeScaling (units.h): tau and the clamped u_lat of a physical case.
extern "C" void ref_compute_scaling(float chord_m, float airspeed_ms, float nu_m2s, int chord_cells, float u_lat,
                                    float* tau, float* u_lat_out) {
    foilcfd::PhysicalParams p;
    p.chord_m = chord_m;
    p.airspeed_ms = airspeed_ms;
    p.nu_m2s = nu_m2s;
    const foilcfd::LatticeScaling s = foilcfd::computeScaling(p, chord_cells, u_lat);
    *tau = s.tau;
    *u_lat_out = s.u_lat;
}
