"""The reference's own CUDA stream-collide, compiled from the reference tree
into a cubin (oracle/ref_build.py) and launched on this GPU through the
driver-API harness (oracle/ref_gpu_harness.cu), against this library's
collide on the same flags, state and parameters. Built without contraction
the reference kernel's populations equal ours bit for bit, which checks the
harness as well; bench.py's reference arm times the as-built one."""
import numpy as np
import pytest

from conftest import written_mask

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fc(built_lib):
    import foil_cfd_gb300 as fc
    return fc


def test_reference_cuda_kernel_matches_ours(fc, oracle_mod):
    from oracle import ref_gpu
    if not ref_gpu.CUBIN_NOFMA.exists():
        pytest.skip("reference cubin not built (needs the reference tree in the build container)")
    dims = (48, 24, 8)
    n = int(np.prod(dims))
    fl = np.zeros(dims[::-1], np.uint8)
    fl[:, 0, :] = 5
    fl[:, -1, :] = 4
    fl[:, :, 0] = 2
    fl[:, 1:-1, -1] = 3
    fl[:, 9:15, 12:18] = 1
    flags = fl.ravel().copy()
    rng = np.random.default_rng(11)
    f0 = oracle_mod.equilibrium(1 + 0.005 * rng.standard_normal(n), 0.05 + 0.005 * rng.standard_normal(n),
                                0.005 * rng.standard_normal(n), 0.005 * rng.standard_normal(n))
    ref, _ = ref_gpu.run(dims, flags, f0, 0.52, 0.05, steps=25, cubin=ref_gpu.CUBIN_NOFMA)
    s = fc.LBMSolver()
    s.init(dims, fc.scaling_direct(0.52, 0.05), flags)
    s.set_startup_ramp_enabled(False)
    s.reset()
    s.import_f32(f0)
    assert s.step_n(25) == 0
    m = written_mask(flags)
    assert np.array_equal(s.export_f32().reshape(19, -1)[:, m], ref.reshape(19, -1)[:, m])
