"""On-device geometry builders (include/foilcfd_geom.h) over CUDA tensors.

The flag fields and cell lists the solver keys off - the clean-foil field
(buildBoundaryFlags + voxelizeAirfoil + closeTrailingEdgeGaps,
src/geom/voxelizer.cpp), the fine-patch field (buildFinePatchFlags), the
patch box (derivePatchBox), the momentum-exchange link list and the
wall-model cell list (buildWallCellList, src/sim/wall_model.cpp:55-236) -
built by CUDA kernels into device memory, byte for byte the host builders'
output. torch provides the device allocations and the stream only; the
fields go straight into LBMSolver.init / set_flags / init_refinement.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import ptr
from .solver import Box, SolverError, fine_anchor, layout_anchor, naca4

BASE = {"boundary": 0, "fluid": 1, "input": 2}


def _torch():
    import torch
    return torch


def _stream(stream):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def _dev(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _check(rc, what):
    if rc != 0:
        raise SolverError(f"{what} failed ({rc})")


def foil(xy, aoa_deg, chord_cells, anchor_x, anchor_y):
    """A placed section: (outline, aoa, chord, anchor) for build_flags."""
    return (np.ascontiguousarray(xy, np.float32), float(aoa_deg), int(chord_cells), float(anchor_x),
            float(anchor_y))


def build_flags(dims, base="boundary", placed=None, close_gaps=True, shell=0, inp=None, out=None, stream=None,
                count_closed=True):
    """Flag field of `dims` in device memory; returns (uint8 tensor, closed).
    base: "boundary" (domain faces), "fluid" or "input" (the tensor `inp`).
    count_closed=False skips the closure count (and its synchronisation);
    closed is then None."""
    torch = _torch()
    n = int(np.prod(dims))
    if out is None:
        out = torch.empty(n, dtype=torch.uint8, device="cuda")
    d = capi.Dims(*dims)
    keep = None
    fp = None
    if placed is not None:
        xy, aoa, chord, ax, ay = placed
        keep = xy
        fp = capi.Foil(xy.ctypes.data_as(C.c_void_p).value, xy.shape[0], aoa, chord, ax, ay)
    closed = C.c_int(0)
    rc = capi.load().fcfd_device_build_flags(C.byref(d), BASE[base], _dev(inp), C.byref(fp) if fp else None,
                                             int(close_gaps), int(shell), _dev(out), _stream(stream),
                                             C.byref(closed) if count_closed else None)
    del keep
    _check(rc, "device flag build")
    return out, (closed.value if count_closed else None)


def derive_patch_box(dims, flags, mx0, mx1, my0, my1, clearance=3, stream=None) -> Box:
    d = capi.Dims(*dims)
    b = capi.PatchBox()
    _check(capi.load().fcfd_device_derive_patch_box(C.byref(d), _dev(flags), mx0, mx1, my0, my1, clearance,
                                                    _stream(stream), C.byref(b)), "device patch box")
    return Box(b.x0, b.y0, b.x1, b.y1)


def force_links(dims, flags, stream=None):
    """(cells, masks) int32 tensors (uint32 bit patterns), ascending cells."""
    torch = _torch()
    d = capi.Dims(*dims)
    lib = capi.load()
    cnt = C.c_longlong(0)
    _check(lib.fcfd_device_force_links(C.byref(d), _dev(flags), None, None, 0, C.byref(cnt), _stream(stream)),
           "device force links")
    cells = torch.empty(max(cnt.value, 1), dtype=torch.int32, device="cuda")
    masks = torch.empty_like(cells)
    again = C.c_longlong(0)
    if cnt.value:
        _check(lib.fcfd_device_force_links(C.byref(d), _dev(flags), _dev(cells), _dev(masks), cnt.value,
                                           C.byref(again), _stream(stream)), "device force links")
    return cells[: cnt.value], masks[: cnt.value]


def wall_list(dims, active, clean=None, sample_cells=2, stream=None):
    """buildWallCellList on device fields: dict of tensors (cell, sample,
    mask as int32 bit patterns; nx, ny, nz, ys float32) + stats."""
    torch = _torch()
    d = capi.Dims(*dims)
    lib = capi.load()
    cnt = C.c_longlong(0)
    stats = np.zeros(3, np.int32)
    args = [C.byref(d), _dev(active), _dev(clean), sample_cells]
    _check(lib.fcfd_device_build_wall_list(*args, *([None] * 7), 0, C.byref(cnt), ptr(stats), _stream(stream)),
           "device wall list")
    m = max(cnt.value, 1)
    out = {k: torch.empty(m, dtype=torch.int32, device="cuda") for k in ("cell", "sample", "mask")}
    out.update({k: torch.empty(m, dtype=torch.float32, device="cuda") for k in ("nx", "ny", "nz", "ys")})
    again = C.c_longlong(0)
    if cnt.value:
        _check(lib.fcfd_device_build_wall_list(*args, _dev(out["cell"]), _dev(out["sample"]), _dev(out["nx"]),
                                               _dev(out["ny"]), _dev(out["nz"]), _dev(out["ys"]), _dev(out["mask"]),
                                               cnt.value, C.byref(again), ptr(stats), _stream(stream)),
               "device wall list")
    res = {k: v[: cnt.value] for k, v in out.items()}
    res["stats"] = dict(listed=int(stats[0]), excluded_vg=int(stats[1]), degenerate=int(stats[2]))
    return res


def clean_foil_flags(dims, digits="0012", aoa=6.0, chord=256, anchor=(0.3, 0.5), points=200, stream=None):
    """buildCleanFoilFlags on the device (anchor as fractions of nx, ny)."""
    xy = naca4(digits, points)
    placed = foil(xy, aoa, chord, *layout_anchor(dims, anchor))
    return build_flags(dims, "boundary", placed, True, 0, stream=stream)[0]


def fine_patch_flags(dims, box: Box, factor, digits="0012", aoa=6.0, chord=256, anchor=(0.3, 0.5), points=200,
                     shell=2, stream=None):
    """buildFinePatchFlags on the device: all fluid, the foil at factor x
    resolution with the patch-local anchor, closure, interface shell."""
    fd = (factor * (box.x1 - box.x0), factor * (box.y1 - box.y0), factor * dims[2])
    xy = naca4(digits, points)
    placed = foil(xy, aoa, factor * chord, *fine_anchor(layout_anchor(dims, anchor), box, factor))
    return fd, build_flags(fd, "fluid", placed, True, shell, stream=stream)[0]
