"""The failure path of the kernels' bounded waits, made to run out without
faulting or hanging the GPU.

The stencil kernels of the large levels wait (about a second at most) on a
transaction barrier for the bulk copy of each stencil tile.  The library's
test hook makes the next such kernel arm one barrier with the expected bytes
but issue no copy, so that nothing ever arrives there: the wait runs out, the
kernel sets its error word, waits for its other copies and returns, and the
entry point must return CITCOM_GPU_ERR_CUDA with the reason.  The context must
stay usable: the next call succeeds and gives the undisturbed result.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cg():
    import citcomcu_gb300 as cg
    cg.build()
    return cg


@pytest.mark.parametrize("precision", [0, 1])
def test_tile_copy_wait_runs_out_and_is_reported(cg, precision):
    # 16^3 elements: the finest level (4913 nodes) runs on the tile kernels
    cfg = cg.Config(mgunit=(4, 4, 4), levels=3, rayleigh=1e5, tdepv=True, viscE=(math.log(1e3),), precision=precision)
    s = cg.Solver(cfg)
    f = s.fine
    rng = np.random.Generator(np.random.PCG64(0))
    z = np.tile(np.linspace(0.0, 1.0, f["noz"]), f["nox"] * f["noy"])
    T = 1.0 - z + 0.01 * rng.uniform(-1, 1, f["nno"])
    s.get_system_viscosity(T)
    s.construct_stiffness_B_matrix()
    F, _ = s.assemble_forces(T)
    acc = 1e-6 * math.sqrt(np.dot(F, F) / F.size)
    ref, _ = s.op_solve_del2_u(F, acc)

    assert cg.load_library().citcom_gpu_test_hold_tile_copy() == 0
    with pytest.raises(cg.CitcomGPUError) as e:
        s.op_solve_del2_u(F, acc)
    msg = str(e.value)
    print(msg)
    assert "CUDA error" in msg and "stencil tile copy did not arrive" in msg

    # the context is usable and the error word cleared: the same call again
    # gives the undisturbed result
    again, _ = s.op_solve_del2_u(F, acc)
    assert np.array_equal(again, ref)
    s.close()
