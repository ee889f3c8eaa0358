"""Host-side mirror of the reference solver interface (src/sim/lbm_solver.h,
src/sim/units.h) over the C ABI. Method names follow the reference class
(init, reset, set_flags, step_n, forces, ...), arguments keep their meaning,
and errors keep the reference behaviour: ``init``/``init_refinement`` report
failure with a reason (raised here as ``SolverError``), ``step_n`` returns a
cudaError_t code (0 = success).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import capi
from .capi import ptr


def _flags_arg(flags):
    """(void* pointer, byte count, keep-alive) of a flag field given as host
    bytes (anything numpy takes) or as a contiguous uint8 CUDA tensor (a
    field built on the device; the C ABI detects device memory)."""
    if getattr(flags, "is_cuda", False):
        if flags.element_size() != 1 or not flags.is_contiguous():
            raise SolverError("device flag field must be a contiguous uint8 tensor")
        return C.c_void_p(flags.data_ptr()), flags.numel(), flags
    a = np.ascontiguousarray(flags, np.uint8)
    return ptr(a), a.size, a

Q = 19
FLAG = dict(fluid=0, solid=1, inlet=2, outlet=3, slip_top=4, slip_bottom=5, slip_front=6, slip_back=7,
            interface=8, outlet_eq=9)
STORE = dict(fp32=0, fp16=1)
K_SMAGORINSKY_CS = 0.1733
K_TRT_MAGIC = 3.0 / 16.0
K_NU_AIR = 1.48e-5


class SolverError(RuntimeError):
    pass


def compute_scaling(chord_m: float, airspeed_ms: float, nu_m2s: float, chord_cells: int,
                    u_lat: float = 0.08) -> capi.Scaling:
    """units.h computeScaling: dx, dt, nu_lat, tau (clamped at 0.5005)."""
    return capi.load().fcfd_compute_scaling(chord_m, airspeed_ms, nu_m2s, chord_cells, u_lat)


def scaling_for_nu(nu_lat: float, u_lat: float, chord_cells: int, chord_m: float = 1.0) -> capi.Scaling:
    """Scaling whose lattice viscosity lands on nu_lat (the tests' reverse
    engineering of the physical inputs, tests/m0_taylor_green.cpp:37-47)."""
    airspeed = K_NU_AIR * u_lat * chord_cells / (nu_lat * chord_m)
    return compute_scaling(chord_m, airspeed, K_NU_AIR, chord_cells, u_lat)


def scaling_direct(tau: float, u_lat: float, chord_cells: int = 64) -> capi.Scaling:
    """Scaling with a given relaxation time and lattice speed (test harness
    helper: parity runs replay a fixed tau / u_lat exactly)."""
    s = capi.Scaling()
    s.chord_m, s.airspeed_ms, s.nu_m2s = 1.0, 1.0, 1.0
    s.chord_cells, s.u_lat, s.tau = chord_cells, u_lat, tau
    s.nu_lat = (tau - 0.5) / 3.0
    s.nu_lat_target = s.nu_lat
    s.dx = 1.0 / chord_cells
    s.dt = u_lat * s.dx
    s.re_target = s.re_effective = u_lat * chord_cells / s.nu_lat
    return s


def refined_scaling(parent: capi.Scaling, factor: int) -> capi.Scaling:
    return capi.load().fcfd_refined_scaling(C.byref(parent), factor)


def force_to_coefficient(s: capi.Scaling, force_lat: float, span_cells: int) -> float:
    return capi.load().fcfd_force_to_coefficient(C.byref(s), force_lat, span_cells)


@dataclass
class Box:
    x0: int
    y0: int
    x1: int
    y1: int

    def as_c(self) -> capi.PatchBox:
        return capi.PatchBox(self.x0, self.y0, self.x1, self.y1)


def fine_dims_for(box: Box, dims, factor: int = 2):
    return (factor * (box.x1 - box.x0), factor * (box.y1 - box.y0), factor * dims[2])


class LBMSolver:
    """One wind tunnel on one GPU (reference foilcfd::LBMSolver)."""

    def __init__(self):
        self._lib = capi.load()
        self._h = self._lib.fcfd_create()
        self.dims = None
        self.scaling = None
        self.storage = "fp32"

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.fcfd_destroy(h)
            self._h = None

    # ---- lifecycle -------------------------------------------------------
    def init(self, dims, scaling: capi.Scaling, flags: np.ndarray, stream=None, storage: str = "fp32",
             les_cs: float | None = None, magic_lambda: float | None = None, kernel: str = "auto",
             layout: str = "ab") -> None:
        """kernel: "auto", "cell" (one cell per thread) or "staged" (rows
        streamed through shared memory by bulk async copies). layout: "ab"
        (two population arrays, pull from one into the other) or "aa" (one
        array updated in place; all-fluid periodic lattices only)."""
        fp, fn, _keep = _flags_arg(flags)
        d = capi.Dims(*dims)
        opt = capi.Options(STORE[storage], 0.0 if les_cs is None else (les_cs if les_cs > 0 else -1.0),
                           0.0 if magic_lambda is None else magic_lambda, 0,
                           {"auto": 0, "cell": 1, "staged": 2}[kernel], {"ab": 0, "aa": 1}[layout])
        err = C.create_string_buffer(512)
        rc = self._lib.fcfd_init(self._h, C.byref(d), C.byref(scaling), fp, fn, stream,
                                 C.byref(opt), err, 512)
        if rc != 0:
            raise SolverError(err.value.decode() or f"init failed ({rc})")
        self.dims = tuple(dims)
        self.scaling = scaling
        self.storage = storage

    @property
    def ncells(self) -> int:
        return int(np.prod(self.dims))

    def reset(self):
        self._lib.fcfd_reset(self._h)

    def set_flags(self, flags):
        fp, fn, _keep = _flags_arg(flags)
        return self._lib.fcfd_set_flags(self._h, fp, fn)

    def apply_edited_flags(self, flags) -> int:
        """LBMSolver::applyEditedFlags (src/sim/lbm_solver.cpp:1086-1126):
        warm restart after a geometry edit; returns the number of cells whose
        solid state changed. Raises on a CUDA error."""
        fp, fn, _keep = _flags_arg(flags)
        edited = C.c_longlong(0)
        rc = self._lib.fcfd_apply_edited_flags(self._h, fp, fn, C.byref(edited))
        if rc != 0:
            raise RuntimeError(f"fcfd_apply_edited_flags failed ({rc})")
        return int(edited.value)

    def mirror_buffers(self) -> None:
        """Copy every level's current A/B buffer into the other one."""
        rc = self._lib.fcfd_mirror_buffers(self._h)
        if rc:
            raise SolverError(f"buffer mirror failed ({rc})")

    def set_startup_ramp_enabled(self, enabled: bool):
        self._lib.fcfd_set_startup_ramp(self._h, int(enabled))

    def set_force_ema_window(self, flow_throughs: float):
        self._lib.fcfd_set_force_ema_window(self._h, flow_throughs)

    # ---- stepping --------------------------------------------------------
    def step_n(self, n: int) -> int:
        return self._lib.fcfd_step_n(self._h, n)

    def synchronize(self) -> int:
        return self._lib.fcfd_synchronize(self._h)

    def step_count(self) -> int:
        return self._lib.fcfd_step_count(self._h)

    def current_tau(self) -> float:
        return self._lib.fcfd_current_tau(self._h)

    def flow_throughs_completed(self) -> float:
        return self._lib.fcfd_flow_throughs(self._h)

    # ---- read-back -------------------------------------------------------
    def forces(self) -> capi.ForceReadout:
        r = capi.ForceReadout()
        self._lib.fcfd_forces(self._h, C.byref(r))
        return r

    def lattice_view(self, level: int = 0) -> capi.Lattice:
        """latticeView(): the level's current source buffer and its layout."""
        v = capi.Lattice()
        rc = self._lib.fcfd_lattice_view(self._h, level, C.byref(v))
        if rc:
            raise SolverError(f"lattice view failed ({rc})")
        return v

    def device_flags(self, level: int = 0) -> int:
        """deviceFlags(): device address of the level's CellFlag bytes."""
        p = C.c_void_p()
        rc = self._lib.fcfd_device_flags(self._h, level, C.byref(p))
        if rc:
            raise SolverError(f"device flags failed ({rc})")
        return p.value

    def force_raw(self) -> np.ndarray:
        out = np.zeros(3, np.float64)
        rc = self._lib.fcfd_force_raw(self._h, ptr(out))
        if rc:
            raise SolverError(f"force readback failed ({rc})")
        return out

    def force_now(self) -> np.ndarray:
        out = np.zeros(3, np.float64)
        rc = self._lib.fcfd_force_now(self._h, ptr(out))
        if rc:
            raise SolverError(f"force reduction failed ({rc})")
        return out

    def download_macro(self):
        n = self.ncells
        arrs = [np.empty(n, np.float32) for _ in range(4)]
        rc = self._lib.fcfd_download_macro(self._h, *[ptr(a) for a in arrs])
        if rc:
            raise SolverError(f"macro download failed ({rc})")
        return arrs

    def download_macro_into(self, rho, u, v, w) -> int:
        return self._lib.fcfd_download_macro(self._h, ptr(rho), ptr(u), ptr(v), ptr(w))

    def import_f32(self, f: np.ndarray):
        f = np.ascontiguousarray(f, np.float32)
        rc = self._lib.fcfd_import_f32(self._h, ptr(f), f.size)
        if rc:
            raise SolverError(f"import failed ({rc})")

    def stage_f32(self, level: int, f: np.ndarray):
        """Queue the copy of one level's FP32 SoA state (0 coarse, 1 fine,
        2 finer) on the solver's copy stream; `f` (float32, contiguous,
        ideally a PinnedArray's array) must stay alive until commit_staged."""
        if f.dtype != np.float32 or not f.flags["C_CONTIGUOUS"]:
            raise SolverError("stage_f32 needs a contiguous float32 array that outlives the commit")
        rc = self._lib.fcfd_stage_f32(self._h, int(level), ptr(f), f.size)
        if rc:
            raise SolverError(f"stage failed ({rc})")

    def commit_staged(self) -> int:
        """Make the staged levels the current state (0, or cudaErrorNotReady
        when nothing is staged)."""
        return self._lib.fcfd_commit_staged(self._h)

    def export_f32(self) -> np.ndarray:
        f = np.empty(Q * self.ncells, np.float32)
        rc = self._lib.fcfd_export_f32(self._h, ptr(f), f.size)
        if rc:
            raise SolverError(f"export failed ({rc})")
        return f

    def notify_snapshot_restored(self, full_state: bool):
        self._lib.fcfd_notify_restored(self._h, int(full_state))

    def restore_from_macroscopic(self, rho, u, v, w):
        arrs = [np.ascontiguousarray(a, np.float32) for a in (rho, u, v, w)]
        rc = self._lib.fcfd_restore_from_macro(self._h, *[ptr(a) for a in arrs])
        if rc:
            raise SolverError(f"macroscopic restore failed ({rc})")

    def f_buffer_bytes(self) -> int:
        return self._lib.fcfd_f_bytes(self._h)

    def perf_stats(self) -> capi.Perf:
        p = capi.Perf()
        self._lib.fcfd_perf_stats(self._h, C.byref(p))
        return p

    def nan_detected(self) -> bool:
        return bool(self._lib.fcfd_nan_detected(self._h))

    def nan_kind(self) -> int:
        return self._lib.fcfd_nan_kind(self._h)

    # ---- wall model ------------------------------------------------------
    def set_wall_model_enabled(self, enabled: bool):
        rc = self._lib.fcfd_set_wall_model(self._h, int(enabled))
        if rc:
            raise SolverError(f"wall model setup failed ({rc})")

    def set_surface_reference(self, clean):
        cp, cn, _keep = _flags_arg(clean)
        return self._lib.fcfd_set_surface_reference(self._h, cp, cn)

    def set_refined_surface_reference(self, clean):
        cp, cn, _keep = _flags_arg(clean)
        return self._lib.fcfd_set_refined_surface_reference(self._h, cp, cn)

    def wall_model_readout(self) -> capi.WMReadout:
        r = capi.WMReadout()
        self._lib.fcfd_wall_model_readout(self._h, C.byref(r))
        return r

    def wall_count(self, level: int = 0) -> int:
        return self._lib.fcfd_wall_count(self._h, level)

    def export_wall_state(self, level: int = 0):
        cnt = self.wall_count(level)
        n = self.ncells if level == 0 else int(np.prod(self.refinement_info_dims()))
        utau = np.empty(cnt, np.float32)
        slip = np.empty(3 * n, np.uint16)
        rc = self._lib.fcfd_export_wall_state(self._h, level, ptr(utau), cnt, ptr(slip), slip.size)
        if rc:
            raise SolverError(f"wall state export failed ({rc})")
        return utau, slip.reshape(3, n)

    def import_wall_state(self, level: int, utau, slip):
        utau = np.ascontiguousarray(utau, np.float32)
        slip = np.ascontiguousarray(slip, np.uint16).ravel()
        rc = self._lib.fcfd_import_wall_state(self._h, level, ptr(utau), utau.size, ptr(slip), slip.size)
        if rc:
            raise SolverError(f"wall state import failed ({rc})")

    def wall_update_now(self, level: int, nu_lat: float, ut_cutoff: float):
        rc = self._lib.fcfd_wall_update_now(self._h, level, nu_lat, ut_cutoff)
        if rc:
            raise SolverError(f"wall update failed ({rc})")

    def set_wall_solver(self, method: int, net=None):
        """u_tau solve of the wall updates: 0 the reference's, 1 full FP64
        Newton, 2 the learned seed (net: a foil_cfd_gb300.wallnet.WallNet)."""
        rc = self._lib.fcfd_set_wall_solver(self._h, int(method), None if net is None else net.handle)
        if rc:
            raise SolverError(f"wall solver selection failed ({rc})")

    def wall_harvest(self, level: int, ut_ptr: int, ys_ptr: int, capacity: int) -> int:
        """(u_par, y) of each wall entry into device buffers; returns the count."""
        cnt = C.c_int()
        rc = self._lib.fcfd_wall_harvest(self._h, level, ut_ptr, ys_ptr, capacity, C.byref(cnt))
        if rc:
            raise SolverError(f"wall harvest failed ({rc})")
        return cnt.value

    def wall_update_timed(self, level: int, reps: int):
        """(mean ms per wall update, stats) of `reps` back-to-back updates."""
        ms = C.c_float()
        st = capi.UtauStats()
        rc = self._lib.fcfd_wall_update_timed(self._h, level, reps, C.byref(ms), C.byref(st))
        if rc:
            raise SolverError(f"timed wall update failed ({rc})")
        return ms.value, {"solved": st.solved, "fallbacks": st.fallbacks, "newton_iterations": st.newton_iterations}

    # ---- refinement ------------------------------------------------------
    def init_refinement(self, box: Box, factor: int, fine_flags) -> None:
        fp, fn, _keep = _flags_arg(fine_flags)
        err = C.create_string_buffer(512)
        b = box.as_c()
        rc = self._lib.fcfd_init_refinement(self._h, C.byref(b), factor, fp, fn, err, 512)
        if rc != 0:
            raise SolverError(err.value.decode() or f"initRefinement failed ({rc})")

    def set_q_links(self, level: int, q_frac=None, ff_mask=None, links: int = 0, fallback: int = 0):
        """Interpolated bounce-back field of a level (None clears it)."""
        if q_frac is None:
            rc = self._lib.fcfd_set_q_links(self._h, level, None, 0, None, 0, 0, 0)
        else:
            qf = np.ascontiguousarray(q_frac, np.uint8)
            fm = np.ascontiguousarray(ff_mask, np.uint32)
            rc = self._lib.fcfd_set_q_links(self._h, level, ptr(qf), qf.size, ptr(fm), fm.size, links, fallback)
        if rc:
            raise SolverError(f"q-link upload failed ({rc})")

    def q_link_info(self, level: int = 0):
        a, l, f = C.c_int(), C.c_int(), C.c_int()
        self._lib.fcfd_q_link_info(self._h, level, C.byref(a), C.byref(l), C.byref(f))
        return bool(a.value), l.value, f.value

    # ---- nested finer level ----------------------------------------------
    def init_finer_refinement(self, box: Box, factor: int, finer_flags) -> None:
        """A patch inside the fine level (box in fine cells)."""
        fp, fn, _keep = _flags_arg(finer_flags)
        err = C.create_string_buffer(512)
        b = box.as_c()
        rc = self._lib.fcfd_init_finer_refinement(self._h, C.byref(b), factor, fp, fn, err, 512)
        if rc != 0:
            raise SolverError(err.value.decode() or f"initFinerRefinement failed ({rc})")

    def shutdown_finer_refinement(self):
        self._lib.fcfd_shutdown_finer_refinement(self._h)

    def set_refined_finer_flags(self, finer_flags):
        fp, fn, _keep = _flags_arg(finer_flags)
        return self._lib.fcfd_set_refined_finer_flags(self._h, fp, fn)

    def finer_refinement_info(self) -> capi.FinerInfo:
        r = capi.FinerInfo()
        self._lib.fcfd_finer_refinement_info(self._h, C.byref(r))
        return r

    def export_finer_f32(self) -> np.ndarray:
        r = self.finer_refinement_info()
        f = np.empty(Q * r.dims.nx * r.dims.ny * r.dims.nz, np.float32)
        rc = self._lib.fcfd_export_finer_f32(self._h, ptr(f), f.size)
        if rc:
            raise SolverError(f"finer export failed ({rc})")
        return f

    def import_finer_f32(self, f):
        f = np.ascontiguousarray(f, np.float32)
        rc = self._lib.fcfd_import_finer_f32(self._h, ptr(f), f.size)
        if rc:
            raise SolverError(f"finer import failed ({rc})")

    def set_fused_restriction(self, enabled: bool):
        """Form the restriction's child averages inside the last fine
        sub-step's collide (True) or in a separate pass (False). Until called,
        the faster one per storage is used: fused with FP32, separate with
        FP16."""
        self._lib.fcfd_set_fused_restriction(self._h, int(enabled))

    def shutdown_refinement(self):
        self._lib.fcfd_shutdown_refinement(self._h)

    def set_refined_flags(self, fine_flags):
        fp, fn, _keep = _flags_arg(fine_flags)
        return self._lib.fcfd_set_refined_flags(self._h, fp, fn)

    def refinement_info(self) -> capi.RefineInfo:
        r = capi.RefineInfo()
        self._lib.fcfd_refinement_info(self._h, C.byref(r))
        return r

    def refinement_info_dims(self):
        r = self.refinement_info()
        return (r.fine_dims.nx, r.fine_dims.ny, r.fine_dims.nz)

    def import_fine_f32(self, f):
        f = np.ascontiguousarray(f, np.float32)
        rc = self._lib.fcfd_import_fine_f32(self._h, ptr(f), f.size)
        if rc:
            raise SolverError(f"fine import failed ({rc})")

    def export_fine_f32(self) -> np.ndarray:
        n = int(np.prod(self.refinement_info_dims()))
        f = np.empty(Q * n, np.float32)
        rc = self._lib.fcfd_export_fine_f32(self._h, ptr(f), f.size)
        if rc:
            raise SolverError(f"fine export failed ({rc})")
        return f

    # ---- diagnostics -----------------------------------------------------
    def kernel_launches(self) -> int:
        return self._lib.fcfd_kernel_launches(self._h)

    def enable_collide_timing(self, enabled: bool):
        self._lib.fcfd_enable_collide_timing(self._h, int(enabled))

    def collide_time_ms(self):
        """(total ms, launches, cells, algorithmic bytes) of the timed
        collide launches since the last call."""
        t = C.c_double()
        n = C.c_longlong()
        c = C.c_double()
        b = C.c_double()
        self._lib.fcfd_collide_time_ms(self._h, C.byref(t), C.byref(n), C.byref(c), C.byref(b))
        return t.value, n.value, c.value, b.value

    def fused_collide_time_ms(self):
        """(total ms, launches, cells, algorithmic bytes) of the timed fine
        collides with fused child averages since the last call."""
        t = C.c_double()
        n = C.c_longlong()
        c = C.c_double()
        b = C.c_double()
        self._lib.fcfd_fused_collide_time_ms(self._h, C.byref(t), C.byref(n), C.byref(c), C.byref(b))
        return t.value, n.value, c.value, b.value

    def timer_start(self):
        rc = self._lib.fcfd_timer_start(self._h)
        if rc:
            raise SolverError(f"timer start failed ({rc})")

    def timer_stop(self) -> float:
        ms = C.c_double()
        rc = self._lib.fcfd_timer_stop(self._h, C.byref(ms))
        if rc:
            raise SolverError(f"timer stop failed ({rc})")
        return ms.value


class PinnedArray:
    """numpy view of page-locked host memory (released on close/GC)."""

    def __init__(self, n: int, dtype=np.float32):
        self._lib = capi.load()
        nbytes = int(n) * np.dtype(dtype).itemsize
        self._p = self._lib.fcfd_host_alloc(nbytes)
        if not self._p:
            raise SolverError("pinned host allocation failed")
        buf = (C.c_char * nbytes).from_address(self._p)
        self.array = np.frombuffer(buf, dtype=dtype, count=int(n))

    def close(self):
        if getattr(self, "_p", None):
            self.array = None
            self._lib.fcfd_host_free(self._p)
            self._p = None

    def __del__(self):
        self.close()


# ---- host fixture builders (no GPU needed) ------------------------------------

def boundary_flags(dims) -> np.ndarray:
    """voxelizer.h buildBoundaryFlags: inlet x=0, outlet x=nx-1, slip y faces."""
    f = np.zeros(int(np.prod(dims)), np.uint8)
    d = capi.Dims(*dims)
    if capi.load().fcfd_boundary_flags(C.byref(d), ptr(f), f.size) != 0:
        raise SolverError("bad dims")
    return f


def naca4(digits: str, points_per_surface: int = 200) -> np.ndarray:
    cap = 2 * max(points_per_surface, 20)
    xy = np.zeros(2 * cap, np.float32)
    n = capi.load().fcfd_naca4(digits.encode(), points_per_surface, ptr(xy), cap)
    if n < 0:
        raise SolverError(f"bad NACA digits {digits!r}")
    return xy[: 2 * n].reshape(n, 2).copy()


def voxelize_airfoil(dims, flags, xy, aoa_deg, chord_cells, anchor_x, anchor_y, close_gaps: bool = True) -> int:
    """voxelizeAirfoil into `flags` (in place), then, by default, the
    trailing-edge gap closure; returns the cells closed."""
    xy = np.ascontiguousarray(xy, np.float32)
    d = capi.Dims(*dims)
    lib = capi.load()
    if lib.fcfd_voxelize_airfoil(C.byref(d), ptr(xy), xy.shape[0], aoa_deg, chord_cells, anchor_x, anchor_y,
                                 ptr(flags), flags.size) != 0:
        raise SolverError("bad voxelizer arguments")
    return close_trailing_edge_gaps(dims, flags) if close_gaps else 0


def layout_anchor(dims, frac=(0.3, 0.5)):
    """DomainLayout::anchorX/anchorY (src/geom/voxelizer.h:71-83): the
    quarter-chord anchor as FP32 fractions of nx, ny, in FP32 arithmetic."""
    return (float(np.float32(frac[0]) * np.float32(dims[0])), float(np.float32(frac[1]) * np.float32(dims[1])))


def fine_anchor(anchor, box, factor):
    """makeFineLayout (voxelizer.cpp:203-221): the coarse anchor moved to the
    patch origin and scaled by the factor, in FP32 arithmetic."""
    f = np.float32(factor)
    return (float(f * (np.float32(anchor[0]) - np.float32(box.x0))),
            float(f * (np.float32(anchor[1]) - np.float32(box.y0))))


def close_trailing_edge_gaps(dims, flags) -> int:
    """closeTrailingEdgeGaps in place; returns the cells closed."""
    d = capi.Dims(*dims)
    n = capi.load().fcfd_close_trailing_edge_gaps(C.byref(d), ptr(flags), flags.size)
    if n < 0:
        raise SolverError("bad flag field")
    return n


def stamp_interface_shell(dims, flags):
    d = capi.Dims(*dims)
    capi.load().fcfd_stamp_interface_shell(C.byref(d), ptr(flags), flags.size)
    return flags


def derive_patch_box(dims, flags, mx0, mx1, my0, my1, clearance) -> Box:
    d = capi.Dims(*dims)
    b = capi.load().fcfd_derive_patch_box(C.byref(d), ptr(np.ascontiguousarray(flags, np.uint8)), mx0, mx1, my0,
                                          my1, clearance)
    return Box(b.x0, b.y0, b.x1, b.y1)


def build_wall_list(dims, active, clean=None, sample_cells: int = 2):
    """wall_model.h buildWallCellList; returns dict of SoA arrays + stats."""
    active = np.ascontiguousarray(active, np.uint8)
    clean = active if clean is None else np.ascontiguousarray(clean, np.uint8)
    cap = int(np.count_nonzero(active == 0)) + 1
    out = dict(cell=np.zeros(cap, np.int64), sample=np.zeros(cap, np.int64), nx=np.zeros(cap, np.float32),
               ny=np.zeros(cap, np.float32), nz=np.zeros(cap, np.float32), ys=np.zeros(cap, np.float32),
               mask=np.zeros(cap, np.uint32))
    stats = np.zeros(3, np.int32)
    d = capi.Dims(*dims)
    n = capi.load().fcfd_build_wall_list(C.byref(d), ptr(active), ptr(clean), sample_cells, ptr(out["cell"]),
                                         ptr(out["sample"]), ptr(out["nx"]), ptr(out["ny"]), ptr(out["nz"]),
                                         ptr(out["ys"]), ptr(out["mask"]), cap, ptr(stats))
    if n < 0:
        raise SolverError("wall list build failed")
    res = {k: v[:n].copy() for k, v in out.items()}
    res["stats"] = dict(listed=int(stats[0]), excluded_vg=int(stats[1]), degenerate=int(stats[2]))
    return res
