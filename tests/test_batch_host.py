"""CPU checks of the polar's tunnel set: (camber, angle) order, chord
resolutions in range, domain 2.5 x 1.5 chords, span, equilibrium outflow,
a voxelised section in every tunnel, and the relaxation time of Re 1000."""
import numpy as np


def test_polar_tunnel_set(built_lib):
    from foil_cfd_gb300 import batch
    ts = batch.polar_tunnels()
    assert len(ts) == 24
    aoas = [-4.0 + 2.5 * k for k in range(9)]
    pairs = [(t.digits, t.aoa) for t in ts]
    assert pairs == [(d, a) for d in ("0012", "2412", "4412") for a in aoas][:24]
    for t in ts:
        assert 96 <= t.chord <= 192
        assert t.dims == (round(2.5 * t.chord), round(1.5 * t.chord), 16)
        f = t.flags.reshape(t.dims[2], t.dims[1], t.dims[0])
        assert (f[:, 1:-1, -1] == 9).all() and (f[:, :, 0] == 2).all()
        solid = (f == 1).sum() / t.dims[2]
        # 12 % thick section: area ~ 0.082 c^2 cells per span cell
        assert 0.06 * t.chord ** 2 < solid < 0.10 * t.chord ** 2
        assert abs(t.tau - (0.5 + 3 * 0.08 * t.chord / 1000.0)) < 1e-6
    assert len({t.chord for t in ts}) > 10
    total = sum(t.cells for t in ts)
    assert 20e6 < total < 45e6
