"""Parity with the reference's CUDA step, built both ways.

The reference's kernels (src/sim/lbm_core.cu, lbm_refine.cu,
lbm_wallmodel.cu) are compiled from the reference tree into sm_103a cubins
twice: as its CMake build makes them (nvcc's default multiply-add
contraction, "asbuilt") and without contraction ("nofma"). They run on this
GPU through oracle/ref_gpu_harness.cu, which replays the reference's stepN
launch sequence (collide, ghost refresh, fills, restriction, per-batch
wall-model update, force reduction, watchdog).

This library's FP32 step rounds the reference's expressions as written
(every FP32 kernel is built without contraction), so it must equal the
nofma build bit for bit: 1000 plain steps (the reference's M0 Taylor-Green
at 64^3 and a square-cylinder channel) and 250 refined steps with the wall
model on. The asbuilt build fuses multiply-adds where ptxas chooses to; its
populations differ from the nofma build's by ~1e-5 relative in u after 100
steps, a difference that stays at that level through 1000 steps. Because
this library equals the nofma build, its distance to the asbuilt build is
exactly the distance between the reference's own two builds; the tests
measure and print it, at 100 and 1000 steps, against the 1e-6 bar.

Both A/B buffers start from the same state on both sides (the harness
seeds both with f0; the library mirrors its imported state), because cells
a step never writes (slip planes at the outlet corners) keep the other
buffer's contents.
"""
import numpy as np
import pytest

from conftest import rel_err, written_mask

pytestmark = pytest.mark.gpu

RHO_U_TOL = 1e-6
CX = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0])
CY = np.array([0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1])
CZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1])


@pytest.fixture(scope="module")
def fc(built_lib):
    import foil_cfd_gb300 as fc
    return fc


@pytest.fixture(scope="module")
def ref_gpu():
    from oracle import ref_gpu
    if not (ref_gpu.available("asbuilt", ("core", "refine", "wall"))
            and ref_gpu.available("nofma", ("core", "refine", "wall"))):
        pytest.skip("reference cubins not built (needs the reference tree in the build container)")
    return ref_gpu


def moments(f, n):
    f = f.reshape(19, n).astype(np.float64)
    rho = f.sum(0)
    return rho, np.stack([CX @ f, CY @ f, CZ @ f]) / rho


def compare(ours, ref, mask):
    """(rho error, u error, differing populations) over the masked cells."""
    n = mask.size
    r1, u1 = moments(ours, n)
    r2, u2 = moments(ref, n)
    er = rel_err(r1, r2, mask)
    eu = float(np.abs(u1[:, mask] - u2[:, mask]).max() / np.linalg.norm(u2[:, mask], axis=0).max())
    nd = int((ours.reshape(19, -1)[:, mask] != ref.reshape(19, -1)[:, mask]).sum())
    return er, eu, nd


def open_domain_flags(nx, ny, nz):
    """The reference tests' open-domain contract (tests/lbm_test_util.h:34-54):
    slip y faces, then inlet x = 0 and outlet x = nx-1 over them (the
    outlet corners copy slip-plane cells), periodic z."""
    f = np.zeros((nz, ny, nx), np.uint8)
    f[:, 0, :] = 5
    f[:, -1, :] = 4
    f[:, :, 0] = 2
    f[:, :, -1] = 3
    return f.ravel().copy()


def taylor_green_case(oracle_mod, n=64, u0=0.05):
    """M0 (tests/m0_taylor_green.cpp:25-80): 64^3, u = u0 (sin x cos y cos z,
    -cos x sin y cos z, 0), k = 2 pi / 64, nu 0.01 (tau 0.53), u_in 1e-3,
    the reference stepN's Cs 0.1733."""
    dims = (n, n, n)
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    k = 2 * np.pi / n
    u = u0 * np.sin(k * x) * np.cos(k * y) * np.cos(k * z)
    v = -u0 * np.cos(k * x) * np.sin(k * y) * np.cos(k * z)
    f0 = oracle_mod.equilibrium(np.ones(n ** 3), u.ravel(), v.ravel(), np.zeros(n ** 3), np.float32)
    return dims, open_domain_flags(*dims), f0, dict(tau=0.53, u_in=1e-3, cs=0.1733)


def cylinder_case(oracle_mod):
    """The square-cylinder channel of the kernel parity test (48x24x8)."""
    dims = (48, 24, 8)
    n = int(np.prod(dims))
    fl = np.zeros(dims[::-1], np.uint8)
    fl[:, 0, :] = 5
    fl[:, -1, :] = 4
    fl[:, :, 0] = 2
    fl[:, :, -1] = 3
    fl[:, 9:15, 12:18] = 1
    rng = np.random.default_rng(11)
    f0 = oracle_mod.equilibrium(1 + 0.005 * rng.standard_normal(n), 0.05 + 0.005 * rng.standard_normal(n),
                                0.005 * rng.standard_normal(n), 0.005 * rng.standard_normal(n), np.float32)
    return dims, fl.ravel().copy(), f0, dict(tau=0.52, u_in=0.05, cs=0.1733)


def run_ours(fc, dims, flags, f0, p, steps, batch=100):
    s = fc.LBMSolver()
    s.init(dims, fc.scaling_direct(p["tau"], p["u_in"]), flags, les_cs=p["cs"])
    s.set_startup_ramp_enabled(False)
    s.reset()
    s.import_f32(f0)
    s.mirror_buffers()
    for _ in range(steps // batch):
        assert s.step_n(batch) == 0
    return s.export_f32()


def run_ref(ref_gpu, dims, flags, f0, p, variant, steps):
    cubin = ref_gpu.CUBIN if variant == "asbuilt" else ref_gpu.CUBIN_NOFMA
    f, _ = ref_gpu.run(dims, flags, f0, p["tau"], p["u_in"], cs=p["cs"], steps=steps, batch=100, cubin=cubin,
                       both_buffers=True)
    return f


CASES = {"taylor_green_64": taylor_green_case, "cylinder_48x24x8": cylinder_case}


@pytest.mark.parametrize("case", sorted(CASES))
def test_plain_step_1000_vs_nofma_reference(fc, ref_gpu, oracle_mod, case):
    """1000 steps against the reference built without contraction: the
    parity bar (<= 1e-6 in rho and u) and bit identity."""
    dims, flags, f0, p = CASES[case](oracle_mod)
    ours = run_ours(fc, dims, flags, f0, p, 1000)
    ref = run_ref(ref_gpu, dims, flags, f0, p, "nofma", 1000)
    er, eu, nd = compare(ours, ref, written_mask(flags))
    print(f"\n{case} vs nofma reference, 1000 steps: rho {er:.3e} u {eu:.3e} differing populations {nd}")
    assert er <= RHO_U_TOL and eu <= RHO_U_TOL, (er, eu)
    assert nd == 0


@pytest.mark.parametrize("case", sorted(CASES))
def test_asbuilt_reference_drift(fc, ref_gpu, oracle_mod, case):
    """Against the as-built (contracted) reference at 100 and 1000 steps.
    This library is the nofma build bit for bit, so its distance to the
    asbuilt build equals the distance between the reference's two builds
    (checked here); that distance is ~1e-5 in u, above the 1e-6 bar, and
    does not grow from 100 to 1000 steps."""
    dims, flags, f0, p = CASES[case](oracle_mod)
    m = written_mask(flags)
    rows = []
    for steps in (100, 1000):
        ours = run_ours(fc, dims, flags, f0, p, steps)
        asb = run_ref(ref_gpu, dims, flags, f0, p, "asbuilt", steps)
        nof = run_ref(ref_gpu, dims, flags, f0, p, "nofma", steps)
        mine = compare(ours, asb, m)
        builds = compare(nof, asb, m)
        assert mine == builds
        rows.append((steps,) + mine)
    print("\n" + "; ".join(f"{case} vs asbuilt reference, {s} steps: rho {er:.3e} u {eu:.3e} ({nd} populations "
                           f"differ; the reference's own nofma build: identical)" for s, er, eu, nd in rows))
    (_, er1, eu1, _), (_, er2, eu2, _) = rows
    assert er2 < 1e-4 and eu2 < 1e-4
    assert eu2 < 3.0 * max(eu1, 1e-9)   # rounding-level, not growing


def uniform_feq(u):
    """feq(1, u, 0, 0) per direction, FP32, in the reference's equilibrium19
    expression order (no contraction: the host harness's own formula)."""
    f32 = np.float32
    u = f32(u)
    usq = f32(1.5) * (u * u)
    out = np.empty(19, np.float32)
    for q in range(19):
        w = f32(1.0) / f32(3.0) if q == 0 else (f32(1.0) / f32(18.0) if q <= 6 else f32(1.0) / f32(36.0))
        cu = f32(3.0) * (f32(CX[q]) * u)
        out[q] = (w * f32(1.0)) * (((f32(1.0) + cu) + (f32(0.5) * cu) * cu) - usq)
    return out


@pytest.mark.parametrize("variant", ["nofma", "asbuilt"])
def test_refined_wall_model_250_steps_vs_reference(fc, ref_gpu, variant):
    """The refined step with the wall model on (160x64x16 tunnel, NACA 0012
    at 6 deg, chord 64, 2:1 patch; tau 0.52, Cs 0.1; batches of 50 steps,
    each followed by the force reduction and the wall-model update of both
    levels, the watchdog every 200 steps) against the reference's kernels:
    coarse and fine populations and u_tau after 250 steps. Bit-identical to
    the nofma build; the asbuilt build's distance is measured (the same
    multiply-add rounding drift as the plain step)."""
    from foil_cfd_gb300.tunnels import airfoil_tunnel
    t = airfoil_tunnel(160, 64, 16, chord=64, aoa=6.0)
    nc, nf = int(np.prod(t.dims)), int(np.prod(t.fine_dims))
    feq = uniform_feq(t.u_lat)
    tau, steps, batch = 0.52, 250, 50
    s = fc.LBMSolver()
    s.init(t.dims, fc.scaling_direct(tau, t.u_lat, t.chord_cells), t.flags, les_cs=0.1)
    s.set_wall_model_enabled(True)
    s.set_startup_ramp_enabled(False)
    s.reset()
    s.init_refinement(t.box, t.factor, t.fine_flags)
    s.import_f32(np.repeat(feq, nc))
    s.import_fine_f32(np.repeat(feq, nf))
    s.mirror_buffers()
    for _ in range(steps // batch):
        assert s.step_n(batch) == 0
    oc, of = s.export_f32(), s.export_fine_f32()
    ut_c, _ = s.export_wall_state(0)
    ut_f, _ = s.export_wall_state(1)
    wc = fc.build_wall_list(t.dims, t.flags, None, 2)
    wf = fc.build_wall_list(t.fine_dims, t.fine_flags, None, 3)
    r = ref_gpu.run_full(t.dims, t.flags, tau, t.u_lat, cs=0.1, f0=np.repeat(feq, nc), wall=wc,
                         fine=dict(dims=t.fine_dims, flags=t.fine_flags, box=t.box, factor=t.factor,
                                   f0=np.repeat(feq, nf), wall=wf),
                         wm=True, steps=steps, batch=batch, variant=variant, states=True)
    ec = compare(oc, r["f"], written_mask(t.flags))
    ef = compare(of, r["fine_f"], t.fine_flags == 0)
    du = max(float(np.abs(ut_c - r["utau"]).max() / np.abs(r["utau"]).max()),
             float(np.abs(ut_f - r["fine_utau"]).max() / np.abs(r["fine_utau"]).max()))
    print(f"\nrefined+WM vs {variant} reference, {steps} steps: coarse rho {ec[0]:.3e} u {ec[1]:.3e} "
          f"({ec[2]} differ); fine rho {ef[0]:.3e} u {ef[1]:.3e} ({ef[2]} differ); u_tau {du:.3e}; "
          f"watchdog trips {r['trip_step']}")
    assert r["trip_step"] == 0
    if variant == "nofma":
        assert max(ec[0], ec[1], ef[0], ef[1]) <= RHO_U_TOL
        assert ec[2] == 0 and ef[2] == 0 and du == 0.0
    else:
        assert max(ec[0], ec[1], ef[0], ef[1]) < 1e-4 and du < 1e-4
