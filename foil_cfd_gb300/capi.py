"""ctypes binding of include/foilcfd_step.h (the solver step's C ABI),
include/foilcfd_wallnet.h (the learned u_tau seed),
include/foilcfd_batch.h (the batched multi-tunnel step),
include/foilcfd_geom.h (the on-device geometry builders) and
include/foilcfd_snapshot.h (warm-start snapshots and the disk cache).

Loading fails loudly when the compiled library is missing: there is no CPU
fallback for the solver step. Build it with ``foil_cfd_gb300.build_lib``
(or ``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libfoilcfd_gb300.so"


class Dims(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int)]


class Scaling(C.Structure):
    _fields_ = [("chord_m", C.c_float), ("airspeed_ms", C.c_float), ("nu_m2s", C.c_float),
                ("chord_cells", C.c_int), ("u_lat", C.c_float), ("dx", C.c_float), ("dt", C.c_float),
                ("nu_lat_target", C.c_float), ("nu_lat", C.c_float), ("tau", C.c_float),
                ("tau_clamped", C.c_int), ("re_target", C.c_float), ("re_effective", C.c_float)]


class Options(C.Structure):
    _fields_ = [("storage", C.c_int), ("les_cs", C.c_float), ("magic_lambda", C.c_float),
                ("use_graphs", C.c_int), ("collide_kernel", C.c_int), ("layout", C.c_int)]


class Lattice(C.Structure):
    """fcfd_lattice (foilcfd_step.h): a level's current source buffer."""
    _fields_ = [("f", C.c_void_p), ("flags", C.c_void_p), ("dims", Dims), ("cells", C.c_longlong),
                ("storage", C.c_int), ("uwx", C.c_void_p), ("uwy", C.c_void_p), ("uwz", C.c_void_p)]


class PatchBox(C.Structure):
    _fields_ = [("x0", C.c_int), ("y0", C.c_int), ("x1", C.c_int), ("y1", C.c_int)]


class SnapshotKey(C.Structure):
    """fcfd_snapshot_key (foilcfd_snapshot.h)."""
    _fields_ = [("geometry_id", C.c_char_p), ("aoa_bucket", C.c_int), ("u_lat", C.c_float), ("dims", Dims),
                ("solver_version", C.c_int)]


class Foil(C.Structure):
    """fcfd_foil (foilcfd_geom.h): host outline + placement."""
    _fields_ = [("xy", C.c_void_p), ("npts", C.c_int), ("aoa_deg", C.c_float), ("chord_cells", C.c_int),
                ("anchor_x", C.c_float), ("anchor_y", C.c_float)]


class ForceReadout(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("cl", "cd", "lift_to_drag")] + [("valid", C.c_int)] + [
        (n, C.c_float) for n in ("flow_throughs", "cl_avg", "cl_min", "cl_max", "cl_median", "cd_avg", "cd_min",
                                 "cd_max", "cd_median", "ld_avg", "ld_min", "ld_max", "ld_median")]


class WMReadout(C.Structure):
    _fields_ = [("enabled", C.c_int), ("from_fine", C.c_int), ("cells", C.c_int), ("mean_yplus", C.c_float),
                ("max_yplus", C.c_float), ("clamped_frac", C.c_float), ("excluded_vg", C.c_int),
                ("degenerate", C.c_int)]


class Perf(C.Structure):
    _fields_ = [("last_step_ms", C.c_double), ("mlups", C.c_double), ("updates_per_step", C.c_double)]


class RefineInfo(C.Structure):
    _fields_ = [("active", C.c_int), ("factor", C.c_int), ("box", PatchBox), ("fine_dims", Dims),
                ("forces_from_fine", C.c_int), ("vram_bytes", C.c_double)]


class FinerInfo(C.Structure):
    _fields_ = [("active", C.c_int), ("factor", C.c_int), ("box", PatchBox), ("dims", Dims),
                ("vram_bytes", C.c_double)]


class WallNetNorm(C.Structure):
    _fields_ = [("in_mean", C.c_float * 3), ("in_std", C.c_float * 3), ("out_mean", C.c_float),
                ("out_std", C.c_float)]


class TrainOpts(C.Structure):
    _fields_ = [("epochs", C.c_int), ("batch", C.c_int), ("lr_max", C.c_float), ("warmup_frac", C.c_float),
                ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float), ("seed", C.c_ulonglong)]


class UtauStats(C.Structure):
    _fields_ = [("solved", C.c_int), ("fallbacks", C.c_int), ("newton_iterations", C.c_longlong)]


class BatchTunnel(C.Structure):
    _fields_ = [("dims", Dims), ("flags", C.c_void_p), ("tau", C.c_float), ("u_lat", C.c_float),
                ("chord_cells", C.c_int)]


class BatchConfig(C.Structure):
    _fields_ = [("block", C.c_int), ("rows", C.c_int), ("ctas_per_sm", C.c_int), ("group_mb", C.c_int)]


P = C.c_void_p
_SIGS = {
    "fcfd_compute_scaling": (Scaling, [C.c_float, C.c_float, C.c_float, C.c_int, C.c_float]),
    "fcfd_refined_scaling": (Scaling, [C.POINTER(Scaling), C.c_int]),
    "fcfd_ramped_tau": (C.c_float, [C.POINTER(Scaling), C.c_longlong, C.c_int]),
    "fcfd_ramped_u": (C.c_float, [C.POINTER(Scaling), C.c_longlong, C.c_int]),
    "fcfd_force_to_coefficient": (C.c_float, [C.POINTER(Scaling), C.c_float, C.c_int]),
    "fcfd_create": (P, []),
    "fcfd_destroy": (None, [P]),
    "fcfd_init": (C.c_int, [P, C.POINTER(Dims), C.POINTER(Scaling), P, C.c_size_t, P, C.POINTER(Options),
                            C.c_char_p, C.c_size_t]),
    "fcfd_reset": (None, [P]),
    "fcfd_set_flags": (C.c_int, [P, P, C.c_size_t]),
    "fcfd_apply_edited_flags": (C.c_int, [P, P, C.c_size_t, P]),
    "fcfd_set_startup_ramp": (None, [P, C.c_int]),
    "fcfd_set_force_ema_window": (None, [P, C.c_float]),
    "fcfd_mirror_buffers": (C.c_int, [P]),
    "fcfd_device_flags": (C.c_int, [P, C.c_int, C.POINTER(C.c_void_p)]),
    "fcfd_lattice_view": (C.c_int, [P, C.c_int, C.POINTER(Lattice)]),
    "fcfd_step_n": (C.c_int, [P, C.c_int]),
    "fcfd_synchronize": (C.c_int, [P]),
    "fcfd_step_count": (C.c_longlong, [P]),
    "fcfd_current_tau": (C.c_float, [P]),
    "fcfd_flow_throughs": (C.c_float, [P]),
    "fcfd_forces": (C.c_int, [P, C.POINTER(ForceReadout)]),
    "fcfd_force_raw": (C.c_int, [P, P]),
    "fcfd_force_now": (C.c_int, [P, P]),
    "fcfd_force_links_noalloc": (C.c_int, [P, C.c_longlong, P, P, C.c_int, P, P, P, P, P]),
    "fcfd_macro": (C.c_int, [P, P, P, P, P]),
    "fcfd_download_macro": (C.c_int, [P, P, P, P, P]),
    "fcfd_active_f": (P, [P]),
    "fcfd_f_bytes": (C.c_size_t, [P]),
    "fcfd_notify_restored": (None, [P, C.c_int]),
    "fcfd_import_f32": (C.c_int, [P, P, C.c_size_t]),
    "fcfd_stage_f32": (C.c_int, [P, C.c_int, P, C.c_size_t]),
    "fcfd_commit_staged": (C.c_int, [P]),
    "fcfd_export_f32": (C.c_int, [P, P, C.c_size_t]),
    "fcfd_restore_from_macro": (C.c_int, [P, P, P, P, P]),
    "fcfd_perf_stats": (C.c_int, [P, C.POINTER(Perf)]),
    "fcfd_nan_detected": (C.c_int, [P]),
    "fcfd_nan_kind": (C.c_int, [P]),
    "fcfd_set_wall_model": (C.c_int, [P, C.c_int]),
    "fcfd_set_surface_reference": (C.c_int, [P, P, C.c_size_t]),
    "fcfd_set_refined_surface_reference": (C.c_int, [P, P, C.c_size_t]),
    "fcfd_wall_model_readout": (C.c_int, [P, C.POINTER(WMReadout)]),
    "fcfd_wall_count": (C.c_int, [P, C.c_int]),
    "fcfd_export_wall_state": (C.c_int, [P, C.c_int, P, C.c_size_t, P, C.c_size_t]),
    "fcfd_import_wall_state": (C.c_int, [P, C.c_int, P, C.c_size_t, P, C.c_size_t]),
    "fcfd_wall_update_now": (C.c_int, [P, C.c_int, C.c_float, C.c_float]),
    "fcfd_init_refinement": (C.c_int, [P, C.POINTER(PatchBox), C.c_int, P, C.c_size_t, C.c_char_p, C.c_size_t]),
    "fcfd_shutdown_refinement": (None, [P]),
    "fcfd_set_refined_flags": (C.c_int, [P, P, C.c_size_t]),
    "fcfd_refinement_info": (C.c_int, [P, C.POINTER(RefineInfo)]),
    "fcfd_import_fine_f32": (C.c_int, [P, P, C.c_size_t]),
    "fcfd_export_fine_f32": (C.c_int, [P, P, C.c_size_t]),
    "fcfd_set_fused_restriction": (C.c_int, [P, C.c_int]),
    "fcfd_set_q_links": (C.c_int, [P, C.c_int, P, C.c_size_t, P, C.c_size_t, C.c_int, C.c_int]),
    "fcfd_init_finer_refinement": (C.c_int, [P, C.POINTER(PatchBox), C.c_int, P, C.c_size_t, C.c_char_p,
                                             C.c_size_t]),
    "fcfd_shutdown_finer_refinement": (None, [P]),
    "fcfd_set_refined_finer_flags": (C.c_int, [P, P, C.c_size_t]),
    "fcfd_set_refined_finer_surface_reference": (C.c_int, [P, P, C.c_size_t]),
    "fcfd_finer_refinement_info": (C.c_int, [P, C.POINTER(FinerInfo)]),
    "fcfd_import_finer_f32": (C.c_int, [P, P, C.c_size_t]),
    "fcfd_export_finer_f32": (C.c_int, [P, P, C.c_size_t]),
    "fcfd_q_link_info": (C.c_int, [P, C.c_int, P, P, P]),
    "fcfd_build_wall_list": (C.c_longlong, [C.POINTER(Dims), P, P, C.c_int, P, P, P, P, P, P, P, C.c_longlong, P]),
    "fcfd_boundary_flags": (C.c_int, [C.POINTER(Dims), P, C.c_size_t]),
    "fcfd_naca4": (C.c_int, [C.c_char_p, C.c_int, P, C.c_int]),
    # include/foilcfd_snapshot.h
    "fcfd_aoa_bucket": (C.c_int, [C.c_float]),
    "fcfd_snapshot_key_hash": (C.c_uint64, [C.POINTER(SnapshotKey)]),
    "fcfd_snapshot_key_string": (C.c_int, [C.POINTER(SnapshotKey), C.c_char_p, C.c_size_t]),
    "fcfd_hash_flags": (C.c_uint64, [P, C.c_size_t]),
    "fcfd_vram_snapshot_create": (P, []),
    "fcfd_vram_snapshot_destroy": (None, [P]),
    "fcfd_vram_snapshot_capture": (C.c_int, [P, P, C.POINTER(SnapshotKey), C.c_char_p, C.c_size_t]),
    "fcfd_vram_snapshot_restore": (C.c_int, [P, P]),
    "fcfd_vram_snapshot_has_data": (C.c_int, [P]),
    "fcfd_vram_snapshot_flags_hash": (C.c_uint64, [P]),
    "fcfd_vram_snapshot_bytes": (C.c_size_t, [P]),
    "fcfd_vram_snapshot_key": (C.c_int, [P, C.POINTER(SnapshotKey)]),
    "fcfd_vram_snapshot_release": (None, [P]),
    "fcfd_compact_snapshot_create": (P, []),
    "fcfd_compact_snapshot_destroy": (None, [P]),
    "fcfd_compact_snapshot_capture": (C.c_int, [P, P, C.POINTER(SnapshotKey), C.c_char_p, C.c_size_t]),
    "fcfd_compact_snapshot_restore": (C.c_int, [P, P]),
    "fcfd_compact_snapshot_save": (C.c_int, [P, C.c_char_p, C.c_char_p, C.c_size_t]),
    "fcfd_compact_snapshot_load": (C.c_int, [P, C.c_char_p, C.c_char_p, C.c_size_t]),
    "fcfd_compact_snapshot_has_data": (C.c_int, [P]),
    "fcfd_compact_snapshot_flags_hash": (C.c_uint64, [P]),
    "fcfd_compact_snapshot_key": (C.c_int, [P, C.POINTER(SnapshotKey)]),
    "fcfd_compact_snapshot_scaling": (C.c_int, [P, C.POINTER(Scaling)]),
    "fcfd_compact_snapshot_fields": (C.c_int, [P, P, P, P, P, P]),
    "fcfd_disk_cache_open": (P, [C.c_char_p, C.c_uint64]),
    "fcfd_disk_cache_close": (None, [P]),
    "fcfd_disk_cache_find": (C.c_int, [P, C.POINTER(SnapshotKey), C.c_char_p, C.c_size_t]),
    "fcfd_disk_cache_store": (C.c_int, [P, P, C.c_char_p, C.c_size_t]),
    "fcfd_disk_cache_store_async": (C.c_int, [P, P]),
    "fcfd_disk_cache_wait": (None, [P]),
    "fcfd_disk_cache_set_budget": (None, [P, C.c_uint64]),
    "fcfd_disk_cache_used_bytes": (C.c_uint64, [P]),
    "fcfd_close_trailing_edge_gaps": (C.c_int, [C.POINTER(Dims), P, C.c_size_t]),
    "fcfd_device_build_flags": (C.c_int, [C.POINTER(Dims), C.c_int, P, P, C.c_int, C.c_int, P, P, P]),
    "fcfd_device_derive_patch_box": (C.c_int, [C.POINTER(Dims), P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, P,
                                               C.POINTER(PatchBox)]),
    "fcfd_device_force_links": (C.c_int, [C.POINTER(Dims), P, P, P, C.c_longlong, P, P]),
    "fcfd_device_build_wall_list": (C.c_int, [C.POINTER(Dims), P, P, C.c_int, P, P, P, P, P, P, P, C.c_longlong, P,
                                              P, P]),
    "fcfd_voxelize_airfoil": (C.c_int, [C.POINTER(Dims), P, C.c_int, C.c_float, C.c_int, C.c_float, C.c_float, P,
                                        C.c_size_t]),
    "fcfd_stamp_interface_shell": (C.c_int, [C.POINTER(Dims), P, C.c_size_t]),
    "fcfd_derive_patch_box": (PatchBox, [C.POINTER(Dims), P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    "fcfd_kernel_launches": (C.c_longlong, [P]),
    "fcfd_enable_collide_timing": (C.c_int, [P, C.c_int]),
    "fcfd_collide_time_ms": (C.c_int, [P, P, P, P, P]),
    "fcfd_fused_collide_time_ms": (C.c_int, [P, P, P, P, P]),
    "fcfd_timer_start": (C.c_int, [P]),
    "fcfd_timer_stop": (C.c_int, [P, P]),
    "fcfd_host_alloc": (P, [C.c_size_t]),
    "fcfd_host_free": (None, [P]),
    "fcfd_version": (C.c_char_p, []),
    # include/foilcfd_wallnet.h
    "fcfd_wallnet_create": (P, []),
    "fcfd_wallnet_destroy": (None, [P]),
    "fcfd_wallnet_init_params": (C.c_int, [P, C.c_ulonglong]),
    "fcfd_wallnet_set_params": (C.c_int, [P, P, C.POINTER(WallNetNorm)]),
    "fcfd_wallnet_get_params": (C.c_int, [P, P, P, C.POINTER(WallNetNorm)]),
    "fcfd_wallnet_fit_norm": (C.c_int, [P, P, P, P, P, C.c_int, P]),
    "fcfd_wallnet_gradient": (C.c_int, [P, P, P, P, P, C.c_int, C.POINTER(C.c_double), P, P]),
    "fcfd_wallnet_train": (C.c_int, [P, P, P, P, P, C.c_int, C.POINTER(TrainOpts), P, P]),
    "fcfd_wallnet_predict": (C.c_int, [P, P, P, P, P, C.c_int, P]),
    "fcfd_utau_solve": (C.c_int, [C.c_int, P, P, P, P, P, P, C.c_int, C.POINTER(UtauStats), P]),
    "fcfd_set_wall_solver": (C.c_int, [P, C.c_int, P]),
    "fcfd_wall_harvest": (C.c_int, [P, C.c_int, P, P, C.c_int, C.POINTER(C.c_int)]),
    "fcfd_wall_update_timed": (C.c_int, [P, C.c_int, C.c_int, C.POINTER(C.c_float), C.POINTER(UtauStats)]),
    # include/foilcfd_batch.h
    "fcfd_batch_create": (P, []),
    "fcfd_batch_destroy": (None, [P]),
    "fcfd_batch_init": (C.c_int, [P, C.POINTER(BatchTunnel), C.c_int, C.c_int, C.c_float, C.c_float, C.c_int, P,
                                  C.c_char_p, C.c_size_t]),
    "fcfd_batch_reset": (C.c_int, [P]),
    "fcfd_batch_set_config": (C.c_int, [P, C.POINTER(BatchConfig)]),
    "fcfd_batch_get_config": (C.c_int, [P, C.POINTER(BatchConfig)]),
    "fcfd_batch_autotune": (C.c_int, [P, C.c_int, C.POINTER(BatchConfig), C.POINTER(C.c_float),
                                      C.POINTER(BatchConfig), C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_int)]),
    "fcfd_batch_step_n": (C.c_int, [P, C.c_int, C.c_int]),
    "fcfd_batch_synchronize": (C.c_int, [P]),
    "fcfd_batch_step_count": (C.c_longlong, [P]),
    "fcfd_batch_updates_per_step": (C.c_longlong, [P]),
    "fcfd_batch_kernel_launches": (C.c_longlong, [P]),
    "fcfd_batch_force_samples": (C.c_int, [P, C.POINTER(C.c_int)]),
    "fcfd_batch_force_history": (C.c_int, [P, P, C.c_int, C.POINTER(C.c_int)]),
    "fcfd_batch_forces_now": (C.c_int, [P, P]),
    "fcfd_batch_health": (C.c_int, [P, P, P]),
    "fcfd_batch_latched": (C.c_int, [P, P, P]),
    "fcfd_batch_export_f32": (C.c_int, [P, C.c_int, P, C.c_size_t]),
    "fcfd_batch_import_f32": (C.c_int, [P, C.c_int, P, C.c_size_t]),
    "fcfd_batch_last_ms": (C.c_int, [P, C.POINTER(C.c_double)]),
}

_lib = None


def declared_symbols():
    """Every function name the headers in include/ declare."""
    return list(_SIGS)


def load() -> C.CDLL:
    """Load the solver-step library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"solver-step library not built ({LIB_PATH}); run foil_cfd_gb300.build_lib.build() "
                "- there is no CPU fallback for the CUDA solver step")
        lib = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def ptr(a):
    """ctypes void* of a numpy array (None passes NULL)."""
    return None if a is None else a.ctypes.data_as(C.c_void_p)
