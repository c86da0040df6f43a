"""The matrix-free FP32 Gauss-Seidel colours (mf.cu, CITCOM_GPU_MF=1) against
the oracle's 8-colour smoother and against the stored-stencil FP32 kernel.

The matrix-free kernel applies the element operator of get_elt_k / get_aug_k
from the Gauss-point viscosity (e_assemble_del2_u's element-by-element
product), so its sweeps must agree with the assembled operator's sweeps to
FP32 rounding: 1e-4 relative against the FP64 oracle on a 33^3-node level of
the 64^3 box with a 10^3 viscosity contrast, 2e-5 against the FP32 stencil
kernel.  A whole mixed-precision solve with it meets the residual rule and
agrees with the stored-stencil solve to the tolerance's effect on the
solution.
"""
import math
import os

import numpy as np
import pytest

from oracle.decks import Case

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def seeded_T0(case, seed=0):
    rng = np.random.Generator(np.random.PCG64(seed))
    z = np.linspace(0.0, case.dimen[2], case.noz)
    T = np.empty((case.noy, case.nox, case.noz))
    T[:] = 1.0 - z / case.dimen[2]
    T += rng.uniform(-0.01, 0.01, size=T.shape)
    T[:, :, 0] = 1.0
    T[:, :, -1] = 0.0
    return T.reshape(-1)


@pytest.fixture(scope="module")
def cg():
    import citcomcu_gb300 as cg
    cg.build()
    return cg


def solver(cg, case, precision, mf):
    if mf:
        os.environ["CITCOM_GPU_MF"] = "1"
    try:
        return cg.Solver(cg.Config.like(case, precision=precision))
    finally:
        os.environ.pop("CITCOM_GPU_MF", None)


@pytest.mark.parametrize("aug", [True, False])
def test_matrix_free_sweeps(cg, oracle_lib, aug):
    case = Case(mgunit=(4, 4, 4), levels=5, rayleigh=1e5, tdepv=True, visc0=(1.0,), viscE=(math.log(1e3),),
                viscT=(0.0,), aug_lagr=aug)
    T0 = seeded_T0(case)
    lev = 3  # 33^3 nodes, below the finest (the FP32 smoother of a multigrid level)
    o = oracle_lib.Oracle(case, gs_colored=True)
    o.set_T(T0)
    o.setup_operators()
    F = o.strip(lev, np.sin(0.37 * np.arange(o.dims[lev]["neq"]) + 0.2))
    dr, _ = o.gauss_seidel(lev, F, 2)
    out = {}
    for mf in (True, False):
        s = solver(cg, case, cg.MIXED, mf)
        s.get_system_viscosity(T0)
        s.construct_stiffness_B_matrix()
        d, _ = s.op_gauss_seidel(lev, F, 2)
        d3, _ = s.op_gauss_seidel(lev, F, 3, d0=d)
        out[mf] = (d, d3)
        s.close()
    d3r, _ = o.gauss_seidel(lev, F, 3, d0=dr)
    print(rel(out[True][0], dr), rel(out[True][0], out[False][0]), rel(out[True][1], d3r))
    assert rel(out[True][0], dr) < 1e-4 and rel(out[True][1], d3r) < 1e-4
    assert rel(out[True][0], out[False][0]) < 2e-5 and rel(out[True][1], out[False][1]) < 2e-5


def test_matrix_free_solve(cg):
    case = Case(mgunit=(4, 4, 4), levels=4, rayleigh=1e5, tdepv=True, visc0=(1.0,), viscE=(math.log(1e3),),
                viscT=(0.0,), accuracy=1e-6, piterations=1000, stop_rule=1)
    T0 = seeded_T0(case)
    res = {}
    for mf in (True, False):
        s = solver(cg, case, cg.MIXED, mf)
        f = s.fine
        U, P = np.zeros(f["neq"]), np.zeros(f["nel"])
        V = s.general_stokes_solver(T0, U, P)
        res[mf] = dict(U=U, P=P, nu=s.heat_flux(T0, V)[0], r=s.stokes_residuals(), st=s.stats())
        s.close()
    print({k: (v["st"]["uzawa"], v["st"]["mg_passes"], v["r"]) for k, v in res.items()})
    assert max(res[True]["r"]) <= case.accuracy
    assert rel(res[True]["U"], res[False]["U"]) < 1e-4 and rel(res[True]["P"], res[False]["P"]) < 1e-4
    assert abs(res[True]["nu"] - res[False]["nu"]) < 1e-6 * abs(res[False]["nu"])
