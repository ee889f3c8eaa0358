"""The reference's own solver tests (tests/m0_taylor_green.cpp,
tests/m3_refine.cpp, tests/m1_cavity.cpp and tests/m4_finer.cpp) compile
against the reference's src/sim/lbm_solver.h and link against this library
through foil_cfd_gb300/shim/lbm_solver_shim.cpp: every LBMSolver member they
call has a definition over the C ABI. Running them needs a GPU
(tests/test_gpu_relinked_reference.py)."""
import pytest


@pytest.mark.parametrize("test", ["m0_taylor_green", "m3_refine", "m1_cavity", "m4_finer"])
def test_reference_test_relinks_against_the_library(test):
    from oracle import relink
    if not relink.staged(test):
        pytest.skip("reference test sources not staged (needs the reference tree in the build container)")
    exe = relink.build(test)
    assert exe.exists()
