"""Generate the golden vectors of the solver step from the reference itself.

Runs the reference's own kernels, compiled for the CPU from the reference
tree by ``oracle/ref_build.py`` (``oracle/_ref/``), on small seeded cases and
stores inputs and outputs under ``tests/golden/*.npz``. It needs the
reference tree (``FOILCFD_REFERENCE``, default /root/reference) and is run
by hand in the build container; the fixtures it writes are committed, so
the tests never need the reference at run time.

    python tests/golden/make_golden.py            # every case
    python tests/golden/make_golden.py qlibb      # one case
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import ref_build  # noqa: E402
from oracle.oracle import CX, CY, CZ, W, equilibrium  # noqa: E402

OUT = Path(__file__).resolve().parent
P = C.c_void_p
I, F = C.c_int, C.c_float


def p(a):
    return None if a is None else a.ctypes.data_as(P)


def load():
    libs = ref_build.build()
    core = C.CDLL(str(libs["core"]))
    core.ref_collide.argtypes = [I, I, I, P, P, P, F, F, F, F, I, P, P, P, P, P, P, P]
    core.ref_collide_q.argtypes = [I, I, I, P, P, P, F, F, F, F, I, P, P, P, P, P, P, P, P, P]
    core.ref_apply_flag_edits.argtypes = [I, I, I, P, P, P, P]
    core.ref_force.argtypes = [I, I, I, P, P, P, P, P, P]
    core.ref_init.argtypes = [I, I, I, P, P, F, F, C.c_uint, I]
    core.ref_init_from_macro.argtypes = [I, I, I, P, P, P, P, P, P]
    wall = C.CDLL(str(libs["wall"]))
    wall.ref_wall_update.argtypes = [I, I, I, P, I, P, P, P, P, P, P, P, P, P, P, P, F, F, F, P]
    refine = C.CDLL(str(libs["refine"]))
    refine.ref_fill.argtypes = [I, I, I, P, P, P, I, I, I, P, P, I, I, I, F, F, F, I]
    refine.ref_restrict.argtypes = [I, I, I, P, P, I, I, I, P, P, I, I, I, I, I, F, F, P, P, P, P]
    wl = C.CDLL(str(libs["walllist"]))
    wl.ref_build_wall_list.argtypes = [I, I, I, P, P, I, P, P, P, P, P, P, P, C.c_longlong, P]
    wl.ref_build_wall_list.restype = C.c_longlong
    return core, wall, refine, wl


def load_snapshot():
    snap = C.CDLL(str(ref_build.build()["snapshot"]))
    snap.ref_key_hash.argtypes = [C.c_char_p, I, F, I, I, I, I]
    snap.ref_key_hash.restype = C.c_ulonglong
    snap.ref_key_string.argtypes = [C.c_char_p, I, F, I, I, I, I, C.c_char_p, I]
    snap.ref_bucket.argtypes = [F]
    snap.ref_hash_flags.argtypes = [P, C.c_ulonglong]
    snap.ref_hash_flags.restype = C.c_ulonglong
    snap.ref_fcs_roundtrip.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, I]
    return snap


SNAPSHOT_KEYS = [("naca:2412", 12, 0.08, (768, 320, 96), 1), ("naca:0012", -10, 0.05, (64, 32, 8), 1),
                 ("dat:e387.dat", 31, 0.1, (256, 128, 4), 1), ("stl:00ff12ab34cd56ef", 0, 0.0125, (48, 40, 40), 1),
                 ("", 1, 0.08, (1, 1, 1), 2)]
SNAPSHOT_AOA = [0.0, 0.24, 0.25, 0.26, -0.25, -0.75, 6.0, 12.3, 25.0, -5.1]
SNAPSHOT_SCALING = dict(chord_m=1.2, airspeed_ms=30.0, nu_m2s=1.48e-5, chord_cells=64, u_lat=0.08, dx=0.01875,
                        dt=5.0e-5, nu_lat_target=1.97e-6, nu_lat=1.5e-4, tau=0.50045, tau_clamped=1,
                        re_target=2.43e6, re_effective=34133.3)


def fcs_bytes(key, flags_hash, scaling, fields):
    """An FCS1 file assembled field by field from the published layout
    (little-endian; magic, format 1, key, flags hash, scaling echo, raw
    payload tag, cell count, rho/u/v/w)."""
    import struct
    gid, bucket, u, dims, ver = key
    b = struct.pack("<III", 0x31534346, 1, len(gid.encode())) + gid.encode()
    b += struct.pack("<ifiiii", bucket, u, *dims, ver) + struct.pack("<Q", flags_hash)
    sc = scaling
    b += struct.pack("<fffiffffffBff", sc["chord_m"], sc["airspeed_ms"], sc["nu_m2s"], sc["chord_cells"],
                     sc["u_lat"], sc["dx"], sc["dt"], sc["nu_lat_target"], sc["nu_lat"], sc["tau"],
                     sc["tau_clamped"], sc["re_target"], sc["re_effective"])
    n = int(np.prod(dims))
    b += struct.pack("<IQ", 0, n)
    for a in fields:
        b += np.ascontiguousarray(a, "<f4").tobytes()
    return b


def case_macro_init(core):
    """Compact-snapshot restore: f = feq(rho, u) of stored macroscopic
    fields (initFromMacroKernel), rest state on solid cells."""
    rng = np.random.default_rng(20261208)
    dims = (16, 12, 4)
    n = int(np.prod(dims))
    fl = open_flags(*dims)
    fl[:, 4:7, 5:8] = 1
    flags = fl.ravel().copy()
    rho = (1 + 0.02 * rng.standard_normal(n)).astype(np.float32)
    u = (0.05 + 0.02 * rng.standard_normal(n)).astype(np.float32)
    v = (0.02 * rng.standard_normal(n)).astype(np.float32)
    w = (0.02 * rng.standard_normal(n)).astype(np.float32)
    f = np.zeros(19 * n, np.float32)
    core.ref_init_from_macro(*dims, p(f), p(flags), p(rho), p(u), p(v), p(w))
    np.savez_compressed(OUT / "macro_init.npz", dims=np.array(dims), flags=flags, rho=rho, u=u, v=v, w=w, f=f)


def case_snapshot(snap):
    """Snapshot keys (hash, name), AoA buckets, the flag hash, and an FCS1
    file read and written back by the reference's CompactSnapshot."""
    import tempfile
    rng = np.random.default_rng(20261207)
    out = {}
    hashes, names = [], []
    for gid, bucket, u, dims, ver in SNAPSHOT_KEYS:
        hashes.append(snap.ref_key_hash(gid.encode(), bucket, u, *dims, ver))
        buf = C.create_string_buffer(512)
        snap.ref_key_string(gid.encode(), bucket, u, *dims, ver, buf, 512)
        names.append(buf.value.decode())
    out["key_hash"] = np.array(hashes, np.uint64)
    out["key_name"] = np.array(names)
    out["aoa"] = np.array(SNAPSHOT_AOA, np.float32)
    out["aoa_bucket"] = np.array([snap.ref_bucket(float(a)) for a in np.array(SNAPSHOT_AOA, np.float32)], np.int32)
    flags = rng.integers(0, 10, 3000).astype(np.uint8)
    out["flags"] = flags
    out["flags_hash"] = np.array(snap.ref_hash_flags(p(flags), flags.size), np.uint64)
    dims = (12, 7, 5)
    n = int(np.prod(dims))
    fields = [rng.standard_normal(n).astype(np.float32) for _ in range(4)]
    key = ("naca:4412", 13, 0.08, dims, 1)
    raw = fcs_bytes(key, 0x0123456789ABCDEF, SNAPSHOT_SCALING, fields)
    with tempfile.TemporaryDirectory() as d:
        src, dst = Path(d) / "in.fcs", Path(d) / "out.fcs"
        src.write_bytes(raw)
        err = C.create_string_buffer(512)
        if snap.ref_fcs_roundtrip(str(src).encode(), str(dst).encode(), err, 512):
            raise SystemExit(f"reference rejected the FCS1 file: {err.value.decode()}")
        out["fcs"] = np.frombuffer(dst.read_bytes(), np.uint8).copy()
        # Rejections: the reference's reason for each corrupted variant.
        bad = {"magic": b"XCS1" + raw[4:], "format": raw[:4] + b"\x02" + raw[5:],
               "truncated": raw[: len(raw) - 7], "version": None}
        kv = fcs_bytes(("naca:4412", 13, 0.08, dims, 2), 0x0123456789ABCDEF, SNAPSHOT_SCALING, fields)
        bad["version"] = kv
        reasons = []
        for name in ("magic", "format", "truncated", "version"):
            src.write_bytes(bad[name])
            rc = snap.ref_fcs_roundtrip(str(src).encode(), None, err, 512)
            reasons.append(err.value.decode().split(":")[0] if rc else "")
        out["reject_reason"] = np.array(reasons)
    out["fcs_fields"] = np.stack(fields)
    out["fcs_dims"] = np.array(dims)
    np.savez_compressed(OUT / "snapshot.npz", **out)


def load_geom():
    geom = C.CDLL(str(ref_build.build()["geom"]))
    geom.ref_naca4.argtypes = [C.c_char_p, I, P, I]
    geom.ref_clean_foil_flags.argtypes = [C.c_char_p, I, F, I, I, I, I, F, F, P]
    geom.ref_fine_patch_flags.argtypes = [C.c_char_p, I, F, I, I, I, I, F, F, I, I, I, I, I, P]
    geom.ref_derive_patch_box.argtypes = [I, I, I, P, I, I, I, I, I, P]
    geom.ref_voxelize_points.argtypes = [P, I, F, I, I, I, I, F, F, P]
    geom.ref_close_te.argtypes = [I, I, I, P]
    return geom


def open_flags(nx, ny, nz):
    """Inlet x=0, outlet x=nx-1, slip y faces (tests/lbm_test_util.h:34-54)."""
    fl = np.zeros((nz, ny, nx), np.uint8)
    fl[:, 0, :] = 5
    fl[:, -1, :] = 4
    fl[:, :, 0] = 2
    fl[:, :, -1] = 3
    return fl


def perturbed_state(rng, n, u0=0.05, amp=0.01):
    rho = 1 + amp * rng.standard_normal(n)
    ux = u0 + amp * rng.standard_normal(n)
    uy = amp * rng.standard_normal(n)
    uz = amp * rng.standard_normal(n)
    f = equilibrium(rho, ux, uy, uz, np.float64)
    f *= 1 + 1e-3 * rng.standard_normal(f.size)
    return f.astype(np.float32)


def reset_state(core, dims, flags, u):
    """The reference solver's buffers after reset() with the ramps off:
    equilibrium at u plus the speck (1e-3 u, seed 0x5eed)."""
    f = np.zeros(19 * int(np.prod(dims)), np.float32)
    core.ref_init(*dims, p(f), p(flags), u, np.float32(1e-3) * np.float32(u), 0x5EED, 1)
    return f


def run_collide(core, dims, f, flags, steps, tau, lam, cs, u_in, slip=None, qlinks=None):
    """`steps` steps on an A/B buffer pair: A = the uploaded state, B = the
    reset state (uploadF writes the current buffer only), so cells a step
    never writes carry the same contents the reference solver would have.
    qlinks = (qFrac, ffMask) runs the reference's q-LIBB instantiation."""
    n = int(np.prod(dims))
    mac = [np.zeros(n, np.float32) for _ in range(4)]
    sl = slip if slip is not None else [None] * 3
    f = f.copy()
    other = reset_state(core, dims, flags, u_in)
    for s in range(steps):
        dst = other
        if qlinks is None:
            core.ref_collide(*dims, p(f), p(dst), p(flags), tau, lam, cs, u_in, int(s == steps - 1),
                             *[p(m) for m in mac], *[p(x) for x in sl])
        else:
            core.ref_collide_q(*dims, p(f), p(dst), p(flags), tau, lam, cs, u_in, int(s == steps - 1),
                               *[p(m) for m in mac], *[p(x) for x in sl], p(qlinks[0]), p(qlinks[1]))
        f, other = dst, f
    return f, mac


def qlink_field(dims, flags, rng, p_link=0.8, p_ff=0.8):
    """Seeded q-LIBB field: a cut byte in [1, 255] on ~p_link of the solid
    links of fluid cells (the pull source x - c_q solid), and the two-node
    bit where x + c_q is fluid (~p_ff of those)."""
    nx, ny, nz = dims
    fl = flags.reshape(nz, ny, nx)
    qf = np.zeros((nz, ny, nx, 19), np.uint8)
    ff = np.zeros((nz, ny, nx), np.uint32)
    for z in range(nz):
        for y in range(ny):
            for x in range(nx):
                if fl[z, y, x] != 0:
                    continue
                for q in range(1, 19):
                    xs, ys, zs = x - CX[q], y - CY[q], (z - CZ[q]) % nz
                    if not (0 <= xs < nx and 0 <= ys < ny) or fl[zs, ys, xs] != 1:
                        continue
                    if rng.random() < p_link:
                        qf[z, y, x, q] = rng.integers(1, 256)
                    xf, yf, zf = x + CX[q], y + CY[q], (z + CZ[q]) % nz
                    if 0 <= xf < nx and 0 <= yf < ny and fl[zf, yf, xf] == 0 and rng.random() < p_ff:
                        ff[z, y, x] |= np.uint32(1 << q)
    return qf.ravel(), ff.ravel()


def case_qlibb(core):
    """Interpolated bounce-back (streamCollideKernel<WM, true>) around the
    square block of the collide case, with and without wall slip."""
    rng = np.random.default_rng(20261204)
    dims = (24, 16, 8)
    n = int(np.prod(dims))
    fl = open_flags(24, 16, 8)
    fl[:, 6:10, 8:12] = 1
    flags = fl.ravel().copy()
    f0 = perturbed_state(rng, n)
    qfrac, ffmask = qlink_field(dims, flags, rng)
    params = dict(tau=0.52, lam=3.0 / 16.0, cs=0.1733, u_in=0.05)
    f1, m1 = run_collide(core, dims, f0, flags, 1, qlinks=(qfrac, ffmask), **params)
    f20, m20 = run_collide(core, dims, f0, flags, 20, qlinks=(qfrac, ffmask), **params)
    slip = [(0.01 * rng.standard_normal(n)).astype(np.float16).view(np.uint16) for _ in range(3)]
    f20w, m20w = run_collide(core, dims, f0, flags, 20, slip=slip, qlinks=(qfrac, ffmask), **params)
    np.savez_compressed(OUT / "qlibb.npz", dims=np.array(dims), flags=flags, f0=f0, qfrac=qfrac, ffmask=ffmask,
                        params=np.array([params["tau"], params["lam"], params["cs"], params["u_in"]], np.float32),
                        f1=f1, m1=np.stack(m1), f20=f20, m20=np.stack(m20), slip=np.stack(slip), f20w=f20w,
                        m20w=np.stack(m20w))


def case_collide(core, rng):
    out = {}
    dims = (24, 16, 8)
    n = int(np.prod(dims))
    fl = open_flags(24, 16, 8)
    fl[:, 6:10, 8:12] = 1  # square cylinder
    flags = fl.ravel().copy()
    f0 = perturbed_state(rng, n)
    params = dict(tau=0.52, lam=3.0 / 16.0, cs=0.1733, u_in=0.05)
    f1, m1 = run_collide(core, dims, f0, flags, 1, **params)
    f20, m20 = run_collide(core, dims, f0, flags, 20, **params)
    slip = [(0.01 * rng.standard_normal(n)).astype(np.float16).view(np.uint16) for _ in range(3)]
    f20w, m20w = run_collide(core, dims, f0, flags, 20, slip=slip, **params)
    force = np.zeros(3, np.float32)
    core.ref_force(*dims, p(f20), p(flags), None, None, None, p(force))
    force_w = np.zeros(3, np.float32)
    core.ref_force(*dims, p(f20w), p(flags), *[p(s) for s in slip], p(force_w))
    # STL-mode spanwise slip walls.
    fz = open_flags(24, 16, 8)
    fz[0, 1:-1, 1:-1] = 6
    fz[-1, 1:-1, 1:-1] = 7
    fz[2:6, 6:10, 8:12] = 1
    flags_z = fz.ravel().copy()
    f20z, m20z = run_collide(core, dims, f0, flags_z, 20, **params)
    out.update(dims=np.array(dims), flags=flags, flags_z=flags_z, f0=f0, f1=f1, f20=f20, f20w=f20w, f20z=f20z,
               slip=np.stack(slip), force20=force, force20w=force_w,
               m1=np.stack(m1), m20=np.stack(m20), m20w=np.stack(m20w), m20z=np.stack(m20z),
               params=np.array([params["tau"], params["lam"], params["cs"], params["u_in"]], np.float32))
    np.savez_compressed(OUT / "collide.npz", **out)


def case_taylor_green(core):
    """Open-domain Taylor-Green (M0 layout, tests/m0_taylor_green.cpp:25-80)
    at 24x16x8, nu = 0.01 (tau 0.53), LES on, 1000 steps."""
    dims = (24, 16, 8)
    nx, ny, nz = dims
    n = nx * ny * nz
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    k = 2 * np.pi / np.array([nx, ny, nz], dtype=np.float64)
    u = 0.05 * np.sin(k[0] * x) * np.cos(k[1] * y) * np.cos(k[2] * z)
    v = -0.05 * np.cos(k[0] * x) * np.sin(k[1] * y) * np.cos(k[2] * z)
    f0 = equilibrium(np.ones(n), u.ravel(), v.ravel(), np.zeros(n), np.float32)
    flags = open_flags(*dims).ravel().copy()
    f1000, m = run_collide(core, dims, f0, flags, 1000, tau=0.53, lam=3.0 / 16.0, cs=0.1733, u_in=1e-3)
    np.savez_compressed(OUT / "taylor_green.npz", dims=np.array(dims), flags=flags, f0=f0, f1000=f1000,
                        m1000=np.stack(m), params=np.array([0.53, 3.0 / 16.0, 0.1733, 1e-3], np.float32))


def case_init(core):
    dims = (24, 16, 8)
    n = int(np.prod(dims))
    fl = open_flags(*dims)
    fl[:, 6:10, 8:12] = 1
    flags = fl.ravel().copy()
    f = np.zeros(19 * n, np.float32)
    core.ref_init(*dims, p(f), p(flags), 0.08, 1e-3 * 0.08, 0x5EED, 1)
    np.savez_compressed(OUT / "init.npz", dims=np.array(dims), flags=flags, f=f,
                        params=np.array([0.08, 1e-3 * 0.08], np.float32))


def plate_case(rng, dims, u_tau=0.004, nu=5e-4):
    """Solid floor y < 4 with a planted Reichardt-like shear profile."""
    nx, ny, nz = dims
    fl = open_flags(nx, ny, nz)
    fl[:, 1:4, 1:-1] = 1
    flags = fl.ravel().copy()
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    yw = np.maximum(y - 3.5, 0.0)
    yp = yw * u_tau / nu
    uplus = np.log(1 + 0.41 * yp) / 0.41 + 7.8 * (1 - np.exp(-yp / 11) - yp / 11 * np.exp(-yp / 3))
    u = np.where(fl == 1, 0.0, u_tau * uplus).ravel()
    u = u + 0.002 * rng.standard_normal(u.size) * (u > 0)
    w = 0.003 * np.sin(2 * np.pi * z / nz).ravel()
    f = equilibrium(np.ones(u.size), u, np.zeros(u.size), w, np.float32)
    return flags, f


def case_wall(core, wall, wl, rng):
    dims = (24, 16, 8)
    n = int(np.prod(dims))
    flags, f = plate_case(rng, dims)
    cap = n
    arr = dict(cell=np.zeros(cap, np.int64), sample=np.zeros(cap, np.int64), nx=np.zeros(cap, np.float32),
               ny=np.zeros(cap, np.float32), nz=np.zeros(cap, np.float32), ys=np.zeros(cap, np.float32),
               mask=np.zeros(cap, np.uint32))
    stats = np.zeros(3, np.int32)
    m = wl.ref_build_wall_list(*dims, p(flags), p(flags), 2, p(arr["cell"]), p(arr["sample"]), p(arr["nx"]),
                               p(arr["ny"]), p(arr["nz"]), p(arr["ys"]), p(arr["mask"]), cap, p(stats))
    arr = {k: v[:m].copy() for k, v in arr.items()}
    utau = np.zeros(m, np.float32)
    slip = [np.zeros(n, np.uint16) for _ in range(3)]
    nu, cut = np.float32(5e-4), np.float32(1e-3 * 0.05)
    hist_u, hist_s, hist_st = [], [], []
    for it in range(3):
        st = np.zeros(4, np.float32)
        wall.ref_wall_update(*dims, p(f), m, p(arr["cell"]), p(arr["sample"]), p(arr["nx"]), p(arr["ny"]),
                             p(arr["nz"]), p(arr["ys"]), p(arr["mask"]), p(utau), *[p(s) for s in slip], nu, cut,
                             0.25, p(st))
        hist_u.append(utau.copy())
        hist_s.append(np.stack(slip).copy())
        hist_st.append(st)
    np.savez_compressed(OUT / "wall.npz", dims=np.array(dims), flags=flags, f=f, stats_build=stats,
                        utau=np.stack(hist_u), slip=np.stack(hist_s), stats=np.stack(hist_st),
                        params=np.array([nu, cut, 0.25], np.float32), **{"list_" + k: v for k, v in arr.items()})


def wall_list_geometries():
    geoms = {}
    d = (32, 32, 8)
    f = np.zeros(d[::-1], np.uint8)
    f[:, :16, :] = 1
    geoms["slab"] = (d, f.ravel().copy(), None)
    d = (64, 64, 8)
    z, y, x = np.meshgrid(*[np.arange(v) for v in d[::-1]], indexing="ij")
    geoms["wedge"] = (d, np.where(x + y < 32, 1, 0).astype(np.uint8).ravel(), None)
    d = (48, 48, 48)
    z, y, x = np.meshgrid(*[np.arange(v) for v in d[::-1]], indexing="ij")
    r = np.sqrt((x - 23.5) ** 2 + (y - 23.5) ** 2 + (z - 23.5) ** 2)
    geoms["sphere"] = (d, np.where(r < 12.0, 1, 0).astype(np.uint8).ravel(), None)
    # Foil + a "vane" solid only in the active field (VG exclusion).
    d = (48, 32, 8)
    z, y, x = np.meshgrid(*[np.arange(v) for v in d[::-1]], indexing="ij")
    clean = np.where(((x - 24) / 14.0) ** 2 + ((y - 14) / 4.0) ** 2 < 1.0, 1, 0).astype(np.uint8)
    active = clean.copy()
    active[(x >= 28) & (x <= 29) & (y >= 18) & (y <= 21)] = 1
    geoms["vane"] = (d, active.ravel().copy(), clean.ravel().copy())
    return geoms


def case_wall_list(wl):
    out = {}
    for name, (d, active, clean) in wall_list_geometries().items():
        clean = active if clean is None else clean
        n = int(np.prod(d))
        for sample in (2, 3):
            arr = dict(cell=np.zeros(n, np.int64), sample=np.zeros(n, np.int64), nx=np.zeros(n, np.float32),
                       ny=np.zeros(n, np.float32), nz=np.zeros(n, np.float32), ys=np.zeros(n, np.float32),
                       mask=np.zeros(n, np.uint32))
            stats = np.zeros(3, np.int32)
            m = wl.ref_build_wall_list(*d, p(active), p(clean), sample, p(arr["cell"]), p(arr["sample"]),
                                       p(arr["nx"]), p(arr["ny"]), p(arr["nz"]), p(arr["ys"]), p(arr["mask"]), n,
                                       p(stats))
            for k, v in arr.items():
                out[f"{name}_{sample}_{k}"] = v[:m].copy()
            out[f"{name}_{sample}_stats"] = stats
    np.savez_compressed(OUT / "wall_list.npz", **out)


def case_refine(core, refine, rng):
    cd = (32, 20, 4)
    cn = int(np.prod(cd))
    cfl = open_flags(*cd)
    cflags = cfl.ravel().copy()
    box = (8, 5, 24, 15)
    m = 2
    fd = (m * (box[2] - box[0]), m * (box[3] - box[1]), m * cd[2])
    fn = int(np.prod(fd))
    ffl = np.zeros(fd[::-1], np.uint8)
    ffl[:, :2, :] = 8
    ffl[:, -2:, :] = 8
    ffl[:, :, :2] = 8
    ffl[:, :, -2:] = 8
    ffl[:, 8:12, 12:16] = 1  # a fine solid block (skipped children)
    fflags = ffl.ravel().copy()
    cT0 = perturbed_state(rng, cn)
    cT1 = perturbed_state(rng, cn)
    ff0 = perturbed_state(rng, fn)
    # tau_f as the solver forms it, in FP32: m (tau_c - 1/2) + 1/2.
    tauC = np.float32(0.52)
    tauF = np.float32(m) * (tauC - np.float32(0.5)) + np.float32(0.5)
    fill_shell = ff0.copy()
    refine.ref_fill(*cd, p(cT0), p(cT1), p(cflags), *fd, p(fill_shell), p(fflags), box[0], box[1], m, 0.5, tauC,
                    tauF, 0)
    fill_full = ff0.copy()
    refine.ref_fill(*cd, p(cT0), p(cT0), p(cflags), *fd, p(fill_full), p(fflags), box[0], box[1], m, 0.0, tauC,
                    tauF, 1)
    fc = cT1.copy()
    mac = [np.zeros(cn, np.float32) for _ in range(4)]
    refine.ref_restrict(*fd, p(ff0), p(fflags), *cd, p(fc), p(cflags), *box, m, tauC, tauF, *[p(x) for x in mac])
    np.savez_compressed(OUT / "refine.npz", cdims=np.array(cd), fdims=np.array(fd), box=np.array(box),
                        factor=np.array(m), cflags=cflags, fflags=fflags, cT0=cT0, cT1=cT1, ff0=ff0,
                        fill_shell=fill_shell, fill_full=fill_full, restricted=fc, rmacro=np.stack(mac),
                        taus=np.array([tauC, tauF], np.float32))


def case_edits(core):
    """Warm-restart flag edit (applyFlagEditsKernel): the collide case's
    block moved by two cells in x after 20 steps; both buffers fixed up."""
    rng = np.random.default_rng(20261205)
    dims = (24, 16, 8)
    n = int(np.prod(dims))
    fl = open_flags(24, 16, 8)
    fl[:, 6:10, 8:12] = 1
    flags0 = fl.ravel().copy()
    fl2 = open_flags(24, 16, 8)
    fl2[:, 6:10, 10:14] = 1
    fl2[1:3, 5, 10:12] = 1  # and a small new vane
    flags1 = fl2.ravel().copy()
    params = dict(tau=0.52, lam=3.0 / 16.0, cs=0.1733, u_in=0.05)
    fA, _ = run_collide(core, dims, perturbed_state(rng, n), flags0, 20, **params)
    fB = reset_state(core, dims, flags0, params["u_in"])
    solid = np.uint8(1)
    mask = np.where((flags0 == solid) == (flags1 == solid), 0, np.where(flags1 == solid, 1, 2)).astype(np.uint8)
    outA, outB = fA.copy(), fB.copy()
    core.ref_apply_flag_edits(*dims, p(outA), p(outB), p(flags1), p(mask))
    np.savez_compressed(OUT / "edits.npz", dims=np.array(dims), flags0=flags0, flags1=flags1, mask=mask, fA=fA,
                        fB=fB, outA=outA, outB=outB)


FOIL_CASES = [((160, 64, 4), 64, 6.0, "0012"), ((200, 96, 3), 80, -5.0, "2412"), ((301, 111, 2), 97, 12.3, "4415")]
PATCH_CASES = [(0, (6, 9, 5, 7, 3), 2), (1, (4, 4, 4, 4, 3), 3)]


def wedge_outline(n=24):
    """A thin closed wedge (chord 1, 2 % thick at the nose, zero at the tail)
    whose voxelised tail leaves single-cell gaps."""
    x = np.linspace(0.0, 1.0, n // 2, dtype=np.float32)
    t = 0.01 * (1.0 - x)
    up = np.stack([x[::-1], t[::-1]], 1)
    lo = np.stack([x[1:], -t[1:]], 1)
    return np.ascontiguousarray(np.concatenate([up, lo]), np.float32)


def case_geometry(geom):
    """Host geometry builders (src/geom/voxelizer.cpp, airfoil.cpp): NACA
    outlines, clean-foil flags, patch boxes and fine-patch flags, an
    arbitrary outline into an existing field, and the trailing-edge closure."""
    rng = np.random.default_rng(20261206)
    out = {}
    for digits in ("0012", "2412", "4415", "6409"):
        for pps in (200, 50):
            xy = np.zeros(2 * 2 * pps, np.float32)
            n = geom.ref_naca4(digits.encode(), pps, p(xy), 2 * pps)
            out[f"naca_{digits}_{pps}"] = xy[: 2 * n].reshape(n, 2).copy()
    for i, (dims, chord, aoa, digits) in enumerate(FOIL_CASES):
        f = np.zeros(int(np.prod(dims)), np.uint8)
        closed = geom.ref_clean_foil_flags(digits.encode(), 200, aoa, *dims, chord, 0.3, 0.5, p(f))
        out[f"foil{i}"] = f
        out[f"foil{i}_closed"] = np.array(closed)
    for k, (i, margins, factor) in enumerate(PATCH_CASES):
        dims, chord, aoa, digits = FOIL_CASES[i]
        box = np.zeros(4, np.int32)
        geom.ref_derive_patch_box(*dims, p(out[f"foil{i}"]), *margins, p(box))
        fd = (factor * int(box[2] - box[0]), factor * int(box[3] - box[1]), factor * dims[2])
        ff = np.zeros(int(np.prod(fd)), np.uint8)
        geom.ref_fine_patch_flags(digits.encode(), 200, aoa, *dims, chord, 0.3, 0.5, *[int(v) for v in box], factor,
                                  p(ff))
        out[f"patch{k}_box"] = box
        out[f"patch{k}"] = ff
    # Arbitrary outline over a field that already holds other flags; the
    # wedge is placed to run off the top face.
    dims = (90, 40, 3)
    base = rng.choice(np.array([0, 0, 0, 0, 0, 0, 1, 2, 3, 4, 5], np.uint8), size=int(np.prod(dims)))
    xy = wedge_outline()
    vox = base.copy()
    geom.ref_voxelize_points(p(xy), xy.shape[0], 20.0, *dims, 70, 30.0, 30.0, p(vox))
    out.update(wedge_xy=xy, wedge_base=base, wedge_vox=vox)
    te_dims = (40, 30, 3)
    te_in = rng.choice(np.array([0, 1, 1, 2], np.uint8), size=int(np.prod(te_dims)))
    te_out = te_in.copy()
    out["te_closed"] = np.array(geom.ref_close_te(*te_dims, p(te_out)))
    out.update(te_in=te_in, te_out=te_out)
    np.savez_compressed(OUT / "geometry.npz", **out)


def main(cases=None):
    """All cases, or the named ones (e.g. `qlibb`) to leave the others'
    fixtures untouched."""
    core, wall, refine, wl = load()
    if cases:
        for c in cases:
            if c == "qlibb":
                case_qlibb(core)
            elif c == "edits":
                case_edits(core)
            elif c == "geometry":
                case_geometry(load_geom())
            elif c == "snapshot":
                case_snapshot(load_snapshot())
            elif c == "macro_init":
                case_macro_init(core)
            else:
                raise SystemExit(f"unknown case {c}")
        return
    rng = np.random.default_rng(20261203)
    case_collide(core, rng)
    case_taylor_green(core)
    case_init(core)
    case_wall(core, wall, wl, rng)
    case_wall_list(wl)
    case_refine(core, refine, rng)
    case_qlibb(core)
    case_edits(core)
    case_geometry(load_geom())
    case_snapshot(load_snapshot())
    case_macro_init(core)
    for f in sorted(OUT.glob("*.npz")):
        print(f.name, f.stat().st_size)


if __name__ == "__main__":
    main(sys.argv[1:])
