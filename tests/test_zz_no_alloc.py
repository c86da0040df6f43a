"""The allocation-free Nusselt entry point (citcom_gpu_heat_flux_noalloc)
against the regular one (citcom_gpu_heat_flux), through the C ABI.

It exists for callers that cannot allocate device memory (their host
application owns the device memory through its own pool, or they run where
cudaMalloc is not allowed); it keeps its scratch in one fixed device array.
Two calls in a row must agree with the regular path and with each other:
the array keeps the previous call's contents, so the second call checks that
whatever must start from zero is cleared.  This file is collected last; it
passes alone in a fresh process as well as after the other tests."""
import numpy as np
import pytest

from oracle.decks import conductive_T0
from tests.golden.make_golden import small_case

pytestmark = pytest.mark.gpu


def test_heat_flux_noalloc_matches_regular_path_twice():
    import torch

    import citcomcu_gb300 as cg
    cg.build()
    case = small_case()
    T0 = conductive_T0(case, amp=0.01, seed=0)
    s = cg.Solver(cg.Config.like(case))
    f = s.fine
    U, P, Tdot = np.zeros(f["neq"]), np.zeros(f["nel"]), np.zeros(f["nno"])
    T = T0.copy()
    V = s.general_stokes_solver(T, U, P)
    s.PG_timestep(T, Tdot, V)
    V = s.general_stokes_solver(T, U, P)
    nut, nub = s.heat_flux(T, V)

    dT = torch.tensor(T, dtype=torch.float64, device="cuda")
    dV = torch.tensor(V, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    dims = (case.nox, case.noy, case.noz)
    tol = 1e-12  # same kernels and reduction order: agreement to rounding
    for _ in range(2):
        a, b = cg.heat_flux_noalloc(*dims, case.dimen, dT.data_ptr(), dV.data_ptr())
        assert abs(a - nut) <= tol * abs(nut), (a, nut)
        assert abs(b - nub) <= tol * abs(nub), (b, nub)
    s.close()


def test_heat_flux_noalloc_rejects_meshes_beyond_its_scratch():
    import torch

    import citcomcu_gb300 as cg
    cg.build()
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    with pytest.raises(cg.CitcomGPUError):
        cg.heat_flux_noalloc(129, 129, 65, (2.0, 2.0, 1.0), d.data_ptr(), d.data_ptr())
