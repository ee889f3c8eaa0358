// foilcfd::LBMSolver over the C ABI of include/foilcfd_step.h.
//
// FoilCFD's callers (the app's frame loop, its GPU tests) use the class
// declared in the reference's src/sim/lbm_solver.h. This translation unit
// defines that class's members on top of this library, so a maintainer
// compiles it against the reference's own header (-I src/sim) in place of
// lbm_core.cu, lbm_refine.cu, lbm_wallmodel.cu and lbm_solver.cpp, and links
// libfoilcfd_gb300.so. Members are defined where the C ABI has the same
// operation; the rest stay undefined, so a caller that needs one fails at link
// time rather than at run time:
//  * latticeView(): the reference's DeviceLatticeView carries PADDED base
//    pointers for its own launch wrappers; this library's buffers are not
//    padded. External kernels use fcfd_lattice_view instead.
//  * the VG/boundary-layer readouts (extractSuctionDelta99, separation onset,
//    crossflow planes) and seedFromCoarse: they lie outside the solver step
//    and have no C counterpart.
// The nested finer level and the q-LIBB link fields map onto
// fcfd_init_finer_refinement & co. and fcfd_set_q_links / fcfd_q_link_info.
//
// Layout note for snapshot callers: activeDeviceF() points at the unpadded
// SoA f[q * cellCount + cell] and fBufferBytes() reports 19 * cellCount *
// sizeof(float) (FP32 storage), which the reference tests' fLayout() already
// recognises as the unpadded header contract.
#include <algorithm>
#include <cstdio>
#include <memory>
#include <string>
#include <vector>

#include "lbm_solver.h"
#include "foilcfd_step.h"

namespace foilcfd {
namespace {

fcfd_scaling to_c(const LatticeScaling& s) {
    fcfd_scaling c{};
    c.chord_m = s.phys.chord_m;
    c.airspeed_ms = s.phys.airspeed_ms;
    c.nu_m2s = s.phys.nu_m2s;
    c.chord_cells = s.chordCells;
    c.u_lat = s.u_lat;
    c.dx = s.dx;
    c.dt = s.dt;
    c.nu_lat_target = s.nu_lat_target;
    c.nu_lat = s.nu_lat;
    c.tau = s.tau;
    c.tau_clamped = s.tauClamped ? 1 : 0;
    c.re_target = s.reTarget;
    c.re_effective = s.reEffective;
    return c;
}

LatticeScaling from_c(const fcfd_scaling& c) {
    LatticeScaling s;
    s.phys.chord_m = c.chord_m;
    s.phys.airspeed_ms = c.airspeed_ms;
    s.phys.nu_m2s = c.nu_m2s;
    s.chordCells = c.chord_cells;
    s.u_lat = c.u_lat;
    s.dx = c.dx;
    s.dt = c.dt;
    s.nu_lat_target = c.nu_lat_target;
    s.nu_lat = c.nu_lat;
    s.tau = c.tau;
    s.tauClamped = c.tau_clamped != 0;
    s.reTarget = c.re_target;
    s.reEffective = c.re_effective;
    return s;
}

} // namespace

struct LBMSolver::Impl {
    fcfd_solver* s = fcfd_create();
    GridDims dims;
    LatticeScaling scaling;
    std::vector<std::uint8_t> flags;
    bool initialized = false;
    bool wallModel = false;
    bool qlibb = false;   // the app's q-LIBB switch; survives re-init as in the reference
    ~Impl() { fcfd_destroy(s); }

    /// Cells of a level (0 coarse, 1 fine, 2 finer); 0 when it is not active.
    long long levelCells(int level) const {
        if (level == 0) return initialized ? dims.cellCount() : 0;
        if (level == 1) {
            fcfd_refine_info r{};
            if (fcfd_refinement_info(s, &r) != 0 || !r.active) return 0;
            return static_cast<long long>(r.fine_dims.nx) * r.fine_dims.ny * r.fine_dims.nz;
        }
        fcfd_finer_info f{};
        if (fcfd_finer_refinement_info(s, &f) != 0 || !f.active) return 0;
        return static_cast<long long>(f.dims.nx) * f.dims.ny * f.dims.nz;
    }

    /// uploadQLevel (lbm_solver.cpp:378-404): the level's previous field goes
    /// first; a switched-off q-LIBB, an empty link count or a field of the
    /// wrong size leaves the level on plain half-way bounce-back.
    void uploadQ(int level, const std::vector<std::uint8_t>& qFrac, const std::vector<std::uint32_t>& ffMask,
                 int links, int fallback) {
        const long long n = levelCells(level);
        if (n == 0) return;
        fcfd_set_q_links(s, level, nullptr, 0, nullptr, 0, 0, 0);
        if (!qlibb || links == 0 || qFrac.size() != static_cast<std::size_t>(n) * 19 ||
            ffMask.size() != static_cast<std::size_t>(n))
            return;
        fcfd_set_q_links(s, level, qFrac.data(), qFrac.size(), ffMask.data(), ffMask.size(), links, fallback);
    }
};

LBMSolver::LBMSolver() : impl_(std::make_unique<Impl>()) {}
LBMSolver::~LBMSolver() = default;

bool LBMSolver::init(const GridDims& d, const LatticeScaling& sc, const std::vector<std::uint8_t>& flags,
                     cudaStream_t stream, std::string* error) {
    Impl& m = *impl_;
    const fcfd_dims dims{d.nx, d.ny, d.nz};
    const fcfd_scaling s = to_c(sc);
    fcfd_options o{};   // FP32 storage, the reference's Cs 0.1733 and Lambda 3/16
    char err[512] = {};
    const int rc = fcfd_init(m.s, &dims, &s, flags.data(), flags.size(), stream, &o, err, sizeof err);
    if (rc != 0) {
        if (error) *error = err;
        m.initialized = false;
        return false;
    }
    m.dims = d;
    m.scaling = sc;
    m.flags = flags;
    m.initialized = true;
    return true;
}

void LBMSolver::shutdown() {
    Impl& m = *impl_;
    fcfd_destroy(m.s);
    m.s = fcfd_create();
    m.initialized = false;
    if (m.wallModel) fcfd_set_wall_model(m.s, 1);   // the switch survives re-init
}

void LBMSolver::reset() { fcfd_reset(impl_->s); }

void LBMSolver::setFlags(const std::vector<std::uint8_t>& flags) {
    if (fcfd_set_flags(impl_->s, flags.data(), flags.size()) == 0) impl_->flags = flags;
}

void LBMSolver::applyEditedFlags(const std::vector<std::uint8_t>& flags) {
    long long edited = 0;
    if (fcfd_apply_edited_flags(impl_->s, flags.data(), flags.size(), &edited) == 0) impl_->flags = flags;
}

bool LBMSolver::initRefinement(const PatchBox& b, int factor, const std::vector<std::uint8_t>& fineFlags,
                               std::string* error) {
    const fcfd_patch_box box{b.x0, b.y0, b.x1, b.y1};
    char err[512] = {};
    const int rc = fcfd_init_refinement(impl_->s, &box, factor, fineFlags.data(), fineFlags.size(), err,
                                        sizeof err);
    if (rc != 0 && error) *error = err;
    return rc == 0;
}

void LBMSolver::shutdownRefinement() { fcfd_shutdown_refinement(impl_->s); }

void LBMSolver::setRefinedFlags(const std::vector<std::uint8_t>& fineFlags) {
    fcfd_set_refined_flags(impl_->s, fineFlags.data(), fineFlags.size());
}

RefinementInfo LBMSolver::refinementInfo() const {
    RefinementInfo r;
    fcfd_refine_info c{};
    if (fcfd_refinement_info(impl_->s, &c) != 0 || !c.active) return r;
    r.active = true;
    r.factor = c.factor;
    r.box.x0 = c.box.x0; r.box.y0 = c.box.y0; r.box.x1 = c.box.x1; r.box.y1 = c.box.y1;
    r.fineDims.nx = c.fine_dims.nx; r.fineDims.ny = c.fine_dims.ny; r.fineDims.nz = c.fine_dims.nz;
    const fcfd_scaling parent = to_c(impl_->scaling);
    r.fineScaling = from_c(fcfd_refined_scaling(&parent, c.factor));
    r.vramBytes = c.vram_bytes;
    r.forcesFromFine = c.forces_from_fine != 0;
    fcfd_finer_info f{};
    if (fcfd_finer_refinement_info(impl_->s, &f) == 0 && f.active) {
        r.finerActive = true;
        r.finerFactor = f.factor;
        r.finerBox.x0 = f.box.x0; r.finerBox.y0 = f.box.y0; r.finerBox.x1 = f.box.x1; r.finerBox.y1 = f.box.y1;
        r.finerDims.nx = f.dims.nx; r.finerDims.ny = f.dims.ny; r.finerDims.nz = f.dims.nz;
        const fcfd_scaling fine = to_c(r.fineScaling);
        r.finerScaling = from_c(fcfd_refined_scaling(&fine, f.factor));
        r.finerVramBytes = f.vram_bytes;
    }
    return r;
}

bool LBMSolver::initFinerRefinement(const PatchBox& b, int m2, const std::vector<std::uint8_t>& finerFlags,
                                    std::string* error) {
    const fcfd_patch_box box{b.x0, b.y0, b.x1, b.y1};
    char err[512] = {};
    const int rc = fcfd_init_finer_refinement(impl_->s, &box, m2, finerFlags.data(), finerFlags.size(), err,
                                              sizeof err);
    if (rc != 0 && error) *error = err;
    return rc == 0;
}

void LBMSolver::shutdownFinerRefinement() { fcfd_shutdown_finer_refinement(impl_->s); }

void LBMSolver::setRefinedFinerFlags(const std::vector<std::uint8_t>& finerFlags) {
    fcfd_set_refined_finer_flags(impl_->s, finerFlags.data(), finerFlags.size());
}

void LBMSolver::setRefinedFinerSurfaceReference(const std::vector<std::uint8_t>& finerCleanFlags) {
    fcfd_set_refined_finer_surface_reference(impl_->s, finerCleanFlags.data(), finerCleanFlags.size());
}

void LBMSolver::setQLIBBEnabled(bool enabled) {
    Impl& m = *impl_;
    if (m.qlibb == enabled) return;
    m.qlibb = enabled;
    if (enabled) return;   // the next uploads build the fields
    for (int level = 0; level < 3; ++level)
        if (m.levelCells(level) > 0) fcfd_set_q_links(m.s, level, nullptr, 0, nullptr, 0, 0, 0);
}

bool LBMSolver::qlibbEnabled() const { return impl_->qlibb; }

void LBMSolver::setCoarseQLinks(const std::vector<std::uint8_t>& qFrac, const std::vector<std::uint32_t>& ffMask,
                                int links, int fallback) {
    impl_->uploadQ(0, qFrac, ffMask, links, fallback);
}

void LBMSolver::setFineQLinks(const std::vector<std::uint8_t>& qFrac, const std::vector<std::uint32_t>& ffMask,
                              int links, int fallback) {
    impl_->uploadQ(1, qFrac, ffMask, links, fallback);
}

void LBMSolver::setFinerQLinks(const std::vector<std::uint8_t>& qFrac, const std::vector<std::uint32_t>& ffMask,
                               int links, int fallback) {
    impl_->uploadQ(2, qFrac, ffMask, links, fallback);
}

long long LBMSolver::fineCellCount() const { return impl_->levelCells(1); }

long long LBMSolver::finerCellCount() const { return impl_->levelCells(2); }

QLIBBReadout LBMSolver::qlibbReadout() const {
    QLIBBReadout r;
    r.enabled = impl_->qlibb;
    if (!r.enabled) return r;
    for (int level = 0; level < 3; ++level) {
        int active = 0, links = 0, fallback = 0;
        if (impl_->levelCells(level) == 0 || fcfd_q_link_info(impl_->s, level, &active, &links, &fallback) != 0 ||
            !active)
            continue;
        r.links += links;
        r.fallback += fallback;
    }
    return r;
}

void LBMSolver::setStartupRampEnabled(bool enabled) { fcfd_set_startup_ramp(impl_->s, enabled ? 1 : 0); }

void LBMSolver::setSurfaceReference(const std::vector<std::uint8_t>& cleanFlags) {
    fcfd_set_surface_reference(impl_->s, cleanFlags.data(), cleanFlags.size());
}

void LBMSolver::setRefinedSurfaceReference(const std::vector<std::uint8_t>& fineCleanFlags) {
    fcfd_set_refined_surface_reference(impl_->s, fineCleanFlags.data(), fineCleanFlags.size());
}

void LBMSolver::setWallModelEnabled(bool enabled) {
    impl_->wallModel = enabled;
    fcfd_set_wall_model(impl_->s, enabled ? 1 : 0);
}

bool LBMSolver::wallModelEnabled() const { return impl_->wallModel; }

WallModelReadout LBMSolver::wallModelReadout() const {
    WallModelReadout r;
    fcfd_wm_readout c{};
    if (fcfd_wall_model_readout(impl_->s, &c) != 0) return r;
    r.enabled = c.enabled != 0;
    r.fromFine = c.from_fine != 0;
    r.cells = c.cells;
    r.meanYplus = c.mean_yplus;
    r.maxYplus = c.max_yplus;
    r.clampedFrac = c.clamped_frac;
    r.excludedVG = c.excluded_vg;
    r.degenerate = c.degenerate;
    return r;
}

cudaError_t LBMSolver::stepN(int n) { return static_cast<cudaError_t>(fcfd_step_n(impl_->s, n)); }

ForceReadout LBMSolver::forces() const {
    ForceReadout o;
    fcfd_force_readout r{};
    if (fcfd_forces(impl_->s, &r) != 0) return o;
    o.cl = r.cl; o.cd = r.cd; o.liftToDrag = r.lift_to_drag; o.valid = r.valid != 0;
    o.flowThroughs = r.flow_throughs;
    o.clAvg = r.cl_avg; o.clMin = r.cl_min; o.clMax = r.cl_max; o.clMedian = r.cl_median;
    o.cdAvg = r.cd_avg; o.cdMin = r.cd_min; o.cdMax = r.cd_max; o.cdMedian = r.cd_median;
    o.ldAvg = r.ld_avg; o.ldMin = r.ld_min; o.ldMax = r.ld_max; o.ldMedian = r.ld_median;
    return o;
}

bool LBMSolver::nanDetected() const { return fcfd_nan_detected(impl_->s) != 0; }

std::string LBMSolver::nanDiagnosis() const {
    if (!nanDetected()) return {};
    const int kind = fcfd_nan_kind(impl_->s);
    const char* level = kind >= 5 && kind <= 6 ? " on the nested refinement patch"
                      : (kind >= 3 && kind <= 4 ? " on the 2x refinement patch" : "");
    const char* what = kind == 9 ? "A staged copy wait timed out"
                     : (kind % 2 == 0 ? "Velocity runaway (field saturated at the stability limiter)"
                                      : "NaN detected");
    const LatticeScaling& sc = impl_->scaling;
    char buf[512];
    std::snprintf(buf, sizeof buf, "%s%s at step %lld. u_lat = %.4f%s; tau = %.5f%s.", what, level,
                  fcfd_step_count(impl_->s), sc.u_lat, sc.u_lat > 0.1f ? " (high)" : "",
                  fcfd_current_tau(impl_->s), sc.tauClamped ? " (clamped)" : "");
    return buf;
}

SolverPerfStats LBMSolver::perfStats() const {
    SolverPerfStats p;
    fcfd_perf c{};
    if (fcfd_perf_stats(impl_->s, &c) != 0) return p;
    p.lastStepMs = c.last_step_ms;
    p.mlups = c.mlups;
    return p;
}

DeviceVelocityField LBMSolver::velocityField() const {
    const float *rho = nullptr, *u = nullptr, *v = nullptr, *w = nullptr;
    fcfd_macro(impl_->s, &rho, &u, &v, &w);
    DeviceVelocityField f;
    f.u = u; f.v = v; f.w = w; f.dims = impl_->dims;
    return f;
}

const float* LBMSolver::deviceRho() const {
    const float *rho = nullptr, *u = nullptr, *v = nullptr, *w = nullptr;
    fcfd_macro(impl_->s, &rho, &u, &v, &w);
    return rho;
}

const std::uint8_t* LBMSolver::deviceFlags() const {
    const std::uint8_t* f = nullptr;
    fcfd_device_flags(impl_->s, 0, &f);
    return f;
}

float* LBMSolver::activeDeviceF() { return static_cast<float*>(fcfd_active_f(impl_->s)); }

std::size_t LBMSolver::fBufferBytes() const { return fcfd_f_bytes(impl_->s); }

void LBMSolver::notifySnapshotRestored(bool fullState) { fcfd_notify_restored(impl_->s, fullState ? 1 : 0); }

bool LBMSolver::restoreFromMacroscopic(const float* rho, const float* u, const float* v, const float* w,
                                       std::string* error) {
    const int rc = fcfd_restore_from_macro(impl_->s, rho, u, v, w);
    if (rc != 0 && error) *error = std::string("restore failed: ") + cudaGetErrorString(static_cast<cudaError_t>(rc));
    return rc == 0;
}

const std::vector<std::uint8_t>& LBMSolver::hostFlags() const { return impl_->flags; }

void LBMSolver::setForceEmaWindow(float flowThroughs) { fcfd_set_force_ema_window(impl_->s, flowThroughs); }

GridDims LBMSolver::dims() const { return impl_->dims; }

const LatticeScaling& LBMSolver::scaling() const { return impl_->scaling; }

long long LBMSolver::stepCount() const { return fcfd_step_count(impl_->s); }

float LBMSolver::flowThroughsCompleted() const { return fcfd_flow_throughs(impl_->s); }

float LBMSolver::currentTau() const { return fcfd_current_tau(impl_->s); }

} // namespace foilcfd
