"""The reference's own GPU solver tests, unmodified, run on this library: the
M0 Taylor-Green decay (tests/m0_taylor_green.cpp: 64^3 open domain, state
injected through activeDeviceF/notifySnapshotRestored, 50k steps, energy
monotone and decayed >50x), the M3 refinement-interface uniformity check
(tests/m3_refine.cpp: solid-free 2:1 patch in uniform flow, 2000 coarse steps,
interface velocity within 1 %), the M1 lid-driven cavity (tests/m1_cavity.cpp:
128x128x4 at Re 1000 run to steady state, centreline u within 7 % of the lid
speed of Ghia, Ghia & Shin's points) and the nested finer level
(tests/m4_finer.cpp: uniform flow through a coarse/fine/finer stack stays
uniform within 1 % over 2000 coarse steps, and a solid in the nested box
stays stable), compiled against the
reference's lbm_solver.h and linked against libfoilcfd_gb300.so through the
LBMSolver shim instead of the reference's own kernels. Each must report
PASS."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("test", ["m0_taylor_green", "m3_refine", "m1_cavity", "m4_finer"])
def test_reference_gpu_test_passes_on_this_library(built_lib, test):
    from oracle import relink
    if not relink.staged(test):
        pytest.skip("reference test sources not staged (needs the reference tree in the build container)")
    rc, out = relink.run(test)
    print("\n" + out[-1500:])
    assert rc == 0, out[-3000:]
    assert f"{test}: PASS" in out
