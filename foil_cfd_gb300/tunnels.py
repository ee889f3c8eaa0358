"""Tunnel builders for the benchmark and test workloads (host fixtures).

* ``taylor_green_periodic``: 64^3 fully periodic Taylor-Green vortex.
* ``square_cylinder``: 384x128x64 channel, 24-cell square at x = 96; the
  channel walls are free-slip (the reference's open-domain flags,
  tests/m2_cylinder.cpp:76-90, so the momentum exchange is the body's force)
  or half-way bounce-back.
* ``airfoil_tunnel``: 640x192x192, NACA 0012 at 6 deg, 256 cells/chord, one
  2:1 patch around the section +- 0.1 chord (the reference's fine-patch
  flags: fluid base, voxelised foil, trailing-edge closure, interface shell,
  src/geom/voxelizer.cpp:223-263).
Geometry follows the reference's DomainLayout defaults: quarter chord at
0.3 nx, 0.5 ny (src/geom/voxelizer.h:57-90).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .solver import (Box, boundary_flags, derive_patch_box, fine_anchor, layout_anchor, naca4, stamp_interface_shell,
                     voxelize_airfoil)


@dataclass
class Tunnel:
    name: str
    dims: tuple
    flags: np.ndarray
    chord_cells: int
    u_lat: float
    box: Box | None = None
    factor: int = 2
    fine_flags: np.ndarray | None = None
    extra: dict = field(default_factory=dict)

    @property
    def fine_dims(self):
        if self.box is None:
            return None
        return (self.factor * (self.box.x1 - self.box.x0), self.factor * (self.box.y1 - self.box.y0),
                self.factor * self.dims[2])

    def updates_per_step(self) -> float:
        """Coarse cells + m * fine cells (lbm_solver.cpp:1705-1713)."""
        u = float(np.prod(self.dims))
        if self.box is not None:
            u += self.factor * float(np.prod(self.fine_dims))
        return u


def taylor_green_periodic(n: int = 64, u0: float = 0.05):
    dims = (n, n, n)
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    k = 2 * np.pi / n
    u = u0 * np.sin(k * x) * np.cos(k * y) * np.cos(k * z)
    v = -u0 * np.cos(k * x) * np.sin(k * y) * np.cos(k * z)
    t = Tunnel("taylor_green_64", dims, np.zeros(n ** 3, np.uint8), n, 0.0)
    t.extra = dict(u=u.ravel(), v=v.ravel())
    return t


def square_cylinder(nx=384, ny=128, nz=64, side=24, cx=96, u_lat=0.08, outlet_eq=False, walls="bounce"):
    dims = (nx, ny, nz)
    f = np.zeros((nz, ny, nx), np.uint8)
    f[:, :, 0] = 2
    f[:, :, -1] = 9 if outlet_eq else 3
    if walls == "slip":     # free-slip bottom / top, inlet wins the corners
        f[:, 0, 1:] = 5
        f[:, -1, 1:] = 4
    else:                   # half-way bounce-back channel walls
        f[:, 0, :] = 1
        f[:, -1, :] = 1
    y0 = ny // 2 - side // 2
    x0 = cx - side // 2
    f[:, y0:y0 + side, x0:x0 + side] = 1
    return Tunnel("square_cylinder", dims, f.ravel().copy(), side, u_lat)


def widen_box(box: Box, nx: int) -> Box:
    """Widen a patch box to a multiple of 4 coarse cells so fine rows are
    16-byte multiples in both storage precisions (bulk-copy staging)."""
    extra = (-(box.x1 - box.x0)) % 4
    grow_right = min(extra, nx - 3 - box.x1)
    return Box(box.x0 - (extra - grow_right), box.y0, box.x1 + grow_right, box.y1)


def airfoil_tunnel(nx=640, ny=192, nz=192, chord=256, aoa=6.0, digits="0012", margin_chord=0.1, factor=2,
                   u_lat=0.08, patch=True, anchor=(0.3, 0.5)):
    dims = (nx, ny, nz)
    flags = boundary_flags(dims)
    xy = naca4(digits, 200)
    ax, ay = layout_anchor(dims, anchor)
    voxelize_airfoil(dims, flags, xy, aoa, chord, ax, ay)
    t = Tunnel(f"naca{digits}_{aoa:g}deg_{nx}x{ny}x{nz}", dims, flags, chord, u_lat, factor=factor)
    t.extra = dict(xy=xy, anchor=(ax, ay), aoa=aoa)
    if patch:
        m = int(round(margin_chord * chord))
        box = widen_box(derive_patch_box(dims, flags, m, m, m, m, 3), nx)
        t.box = box
        fd = t.fine_dims
        ff = np.zeros(int(np.prod(fd)), np.uint8)
        voxelize_airfoil(fd, ff, xy, aoa, factor * chord, *fine_anchor((ax, ay), box, factor))
        stamp_interface_shell(fd, ff)
        t.fine_flags = ff
    return t
