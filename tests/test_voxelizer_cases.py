"""The reference's own voxeliser checks (tests/test_voxelizer.cpp), run on
the host builders and on the device builders: the boundary-flag contract,
parity voxelisation of a synthetic diamond against a hand-computed
classification, identical z extrusion, the trailing-edge closure on a
deliberately leaky pattern, the 25-degree clearance lock with a valid patch
box, and a negative patch-local anchor."""
import numpy as np
import pytest

BACKENDS = ["host", pytest.param("device", marks=pytest.mark.gpu)]


@pytest.fixture(scope="module")
def fc(built_lib):
    import foil_cfd_gb300 as fc
    return fc


def diamond():
    """Chord [0, 1], half-thickness 0.25, Selig order, 6 segments per edge
    plus the closing point (25 points)."""
    c = np.array([[1.0, 0.0], [0.5, 0.25], [0.0, 0.0], [0.5, -0.25], [1.0, 0.0]], np.float32)
    pts = []
    for e in range(4):
        for s in range(6):
            t = np.float32(s) / np.float32(6)
            pts.append(c[e] + (c[e + 1] - c[e]) * t)
    pts.append(c[4])
    return np.ascontiguousarray(np.array(pts, np.float32))


class Builder:
    def __init__(self, fc, backend):
        self.fc, self.backend = fc, backend
        if backend == "device":
            import torch
            from foil_cfd_gb300 import geometry
            self.torch, self.geo = torch, geometry

    def voxelize(self, dims, flags, xy, aoa, chord, ax, ay):
        if self.backend == "host":
            out = flags.copy()
            self.fc.voxelize_airfoil(dims, out, xy, aoa, chord, ax, ay, close_gaps=False)
            return out
        inp = self.torch.from_numpy(np.ascontiguousarray(flags)).cuda()
        t, _ = self.geo.build_flags(dims, "input", self.geo.foil(xy, aoa, chord, ax, ay), False, 0, inp=inp)
        return t.cpu().numpy()

    def close_gaps(self, dims, flags):
        if self.backend == "host":
            out = flags.copy()
            return self.fc.close_trailing_edge_gaps(dims, out), out
        inp = self.torch.from_numpy(np.ascontiguousarray(flags)).cuda()
        t, closed = self.geo.build_flags(dims, "input", None, True, 0, inp=inp)
        return closed, t.cpu().numpy()

    def boundary(self, dims):
        if self.backend == "host":
            return self.fc.boundary_flags(dims)
        t, _ = self.geo.build_flags(dims, "boundary", None, False, 0)
        return t.cpu().numpy()

    def patch_box(self, dims, flags, *m):
        if self.backend == "host":
            return self.fc.derive_patch_box(dims, flags, *m, 3)
        return self.geo.derive_patch_box(dims, self.torch.from_numpy(flags).cuda(), *m, 3)


@pytest.mark.parametrize("backend", BACKENDS)
def test_boundary_flags_contract(fc, backend):
    b = Builder(fc, backend)
    dims = (8, 6, 3)
    f = b.boundary(dims).reshape(dims[::-1])
    exp = np.zeros(dims[::-1], np.uint8)
    exp[:, 0, :] = 5
    exp[:, -1, :] = 4
    exp[:, :, 0] = 2                      # the inlet wins its corners
    exp[:, 1:-1, -1] = 3                  # the outlet yields to the slip faces
    assert np.array_equal(f, exp)


@pytest.mark.parametrize("backend", BACKENDS)
def test_diamond_parity_extrusion(fc, backend):
    b = Builder(fc, backend)
    dims = (32, 24, 3)
    ax, ay = fc.layout_anchor(dims)       # (9.6, 12): diamond centre (13.6, 12), semi-axes 8, 4
    f = b.voxelize(dims, b.boundary(dims), diamond(), 0.0, 16, ax, ay).reshape(dims[::-1])
    solid = f == 1
    j, i = np.mgrid[1:dims[1] - 1, 1:dims[0] - 1]
    sA = np.abs(i - 13.6) / 8.0 + np.abs(j - 12.0) / 4.0
    sB = np.abs(i + 0.5 - 13.6) / 8.0 + np.abs(j + 0.5 - 12.0) / 4.0
    s0 = solid[0, 1:-1, 1:-1]
    assert not np.any((sA <= 0.75) & (sB <= 0.75) & ~s0)   # well inside -> solid
    assert not np.any((sA >= 1.25) & (sB >= 1.25) & s0)    # well outside -> fluid
    assert 40 <= int(solid[0].sum()) <= 90                  # ~64 cells of area
    assert all(np.array_equal(f[z], f[0]) for z in range(1, dims[2]))
    assert f[0, 12, 0] == 2                                  # inlet untouched


@pytest.mark.parametrize("backend", BACKENDS)
def test_trailing_edge_closure_known_answer(fc, backend):
    b = Builder(fc, backend)
    dims = (8, 8, 2)
    f = np.zeros(dims[::-1], np.uint8)
    f[:, 2, 3] = 1
    f[:, 4, 3] = 1
    f[:, 2, 6] = 1                         # a lone solid: no closure around it
    closed, out = b.close_gaps(dims, f.ravel())
    out = out.reshape(dims[::-1])
    assert closed == 2
    assert np.all(out[:, 3, 3] == 1)
    assert np.all(out[:, 1, 6] == 0) and np.all(out[:, 3, 6] == 0)
    assert np.all(out[:, 2, 3] == 1) and np.all(out[:, 4, 3] == 1)


@pytest.mark.parametrize("backend", BACKENDS)
@pytest.mark.parametrize("aoa", [25.0, -5.0])
def test_high_aoa_clearance_and_patch_box(fc, backend, aoa):
    b = Builder(fc, backend)
    nc = 128
    dims = (3 * nc, nc + nc // 4, 8)
    f = b.voxelize(dims, b.boundary(dims), diamond(), aoa, nc, *fc.layout_anchor(dims)).reshape(dims[::-1])
    ys, xs = np.nonzero(f[0] == 1)
    assert xs.size
    clear = 8
    assert ys.min() >= clear and ys.max() < dims[1] - clear
    assert xs.min() >= clear and xs.max() < dims[0] - clear
    box = b.patch_box(dims, f.ravel(), nc // 5, nc // 2, nc // 10, nc // 5)
    assert box.x1 - box.x0 > 8 and box.y1 - box.y0 > 8


@pytest.mark.parametrize("backend", BACKENDS)
def test_negative_patch_local_anchor(fc, backend):
    b = Builder(fc, backend)
    dims = (32, 24, 3)
    box = fc.Box(10, 13, 20, 22)
    fax, fay = fc.fine_anchor(fc.layout_anchor(dims), box, 2)
    assert abs(fax + 0.8) < 1e-4 and abs(fay + 2.0) < 1e-4
    fd = (2 * (box.x1 - box.x0), 2 * (box.y1 - box.y0), 2 * dims[2])
    f = b.voxelize(fd, np.zeros(int(np.prod(fd)), np.uint8), diamond(), 0.0, 32, fax, fay).reshape(fd[::-1])
    solid = f[0] == 1
    j, i = np.mgrid[1:fd[1] - 1, 1:fd[0] - 1]
    sA = np.abs(i - 7.2) / 16.0 + np.abs(j + 2.0) / 8.0
    sB = np.abs(i + 0.5 - 7.2) / 16.0 + np.abs(j + 0.5 + 2.0) / 8.0
    s0 = solid[1:-1, 1:-1]
    inside = (sA <= 0.75) & (sB <= 0.75)
    assert inside.any() and not np.any(inside & ~s0)
    assert not np.any((sA >= 1.25) & (sB >= 1.25) & s0)
