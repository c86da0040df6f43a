"""The double-float operator assembly of the mixed configuration
(assemble.cu) against the FP64 assembly (k_assemble) and the oracle.

The mixed configuration assembles the box levels with every product and sum
carried as a pair of FP32 numbers (about 46 significant bits).  Its FP64
finest-level stencil (the one the refinement residual and the residual rule
use) must then agree with the FP64 assembly to 1e-12 relative, its 1/diag K
likewise, and the FP32 stencils of the coarser levels to FP32 rounding
(1e-6); CITCOM_GPU_FP64_ASSEMBLY=1 restores the FP64 assembly.
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


@pytest.fixture(scope="module")
def cg():
    import citcomcu_gb300 as cg
    cg.build()
    return cg


@pytest.mark.parametrize("aug", [True, False])
def test_double_float_assembly(cg, oracle_lib, aug):
    # two viscosity layers and a 10^4 temperature contrast: entries spanning
    # several orders of magnitude
    case = Case(mgunit=(2, 3, 2), levels=4, dimen=(1.0, 1.5, 1.0), rayleigh=1e5, tdepv=True, visc0=(1.0, 30.0),
                viscE=(math.log(1e4), math.log(1e4)), viscT=(0.0, 0.0), z_layer=(0.6,), aug_lagr=aug)
    rng = np.random.Generator(np.random.PCG64(3))
    nno = case.nox * case.noy * case.noz
    z = np.tile(np.linspace(0.0, 1.0, case.noz), case.nox * case.noy)
    T = np.clip(1.0 - z + 0.05 * rng.uniform(-1, 1, nno), 0.0, 1.0)
    out = {}
    for prec in (0, 1):
        s = cg.Solver(cg.Config.like(case, precision=prec))
        s.get_system_viscosity(T)
        s.construct_stiffness_B_matrix()
        lmax = case.levels - 1
        u = np.sin(0.37 * np.arange(s.dims[lmax]["neq"]) + 0.3)
        uc = np.sin(0.29 * np.arange(s.dims[lmax - 1]["neq"]) + 0.1)
        out[prec] = dict(K=s.op_kmul(lmax, u), Kc=s.op_kmul(lmax - 1, uc), BI=s.op_diagonals(lmax)[0],
                         BIc=s.op_diagonals(lmax - 1)[0])
        s.close()
    o = oracle_lib.Oracle(case)
    o.set_T(T)
    o.setup_operators()
    lmax = case.levels - 1
    u = np.sin(0.37 * np.arange(o.dims[lmax]["neq"]) + 0.3)
    print(rel(out[1]["K"], out[0]["K"]), rel(out[1]["BI"], out[0]["BI"]), rel(out[1]["Kc"], out[0]["Kc"]))
    assert rel(out[1]["K"], out[0]["K"]) < 1e-12
    assert rel(out[1]["K"], o.kmul(lmax, u)) < 1e-12
    assert rel(out[1]["BI"], out[0]["BI"]) < 1e-12
    assert rel(out[1]["Kc"], out[0]["Kc"]) < 1e-6
    assert rel(out[1]["BIc"], out[0]["BIc"]) < 1e-6


def test_split_fp64_operator(cg):
    """The mixed box keeps the finest level's FP64 operator as its FP32
    stencil plus the FP32 remainder and applies it in double-float
    (k_tile_split): K u against the same operator held in FP64
    (CITCOM_GPU_NO_SPLIT=1) to 1e-13, and a mixed Stokes solve takes the same
    iteration counts and reaches the same solution to 1e-9 (FP64 rounding
    carried through the solve; measured 1.7e-10)."""
    from citcomcu_gb300 import Config
    case = Config(mgunit=(4, 4, 4), levels=3, rayleigh=1e5, tdepv=True, visc0=(1.0,), viscE=(math.log(1e3),),
                  viscT=(0.0,), accuracy=1e-6, piterations=1000, stop_rule=1)
    nno = case.nox * case.noy * case.noz
    rng = np.random.Generator(np.random.PCG64(4))
    z = np.tile(np.linspace(0.0, 1.0, case.noz), case.nox * case.noy)
    T = np.clip(1.0 - z + 0.01 * rng.uniform(-1, 1, nno), 0.0, 1.0)
    out = {}
    for split in (True, False):
        if not split:
            os.environ["CITCOM_GPU_NO_SPLIT"] = "1"
        try:
            s = cg.Solver(cg.Config.like(case, precision=cg.MIXED))
        finally:
            os.environ.pop("CITCOM_GPU_NO_SPLIT", None)
        s.get_system_viscosity(T)
        s.construct_stiffness_B_matrix()
        u = np.sin(0.37 * np.arange(s.fine["neq"]) + 0.3)
        Ku = s.op_kmul(case.levels - 1, u)
        U, P = np.zeros(s.fine["neq"]), np.zeros(s.fine["nel"])
        s.general_stokes_solver(T, U, P)
        out[split] = (Ku, U, s.stats())
        s.close()
    print(rel(out[True][0], out[False][0]), rel(out[True][1], out[False][1]))
    assert rel(out[True][0], out[False][0]) < 1e-13
    assert out[True][2]["uzawa"] == out[False][2]["uzawa"]
    assert rel(out[True][1], out[False][1]) < 1e-9


@pytest.mark.parametrize("aug", [True, False])
def test_double_float_assembly_sphere(cg, aug):
    """The same double-float assembly on a regional spherical segment, where
    every (theta, r) column of elements has its own element kernels (a
    word-major table over the columns): the finest FP64 operator (FP32 stencil
    plus FP32 remainder) and 1/diag K against the FP64 assembly to 1e-12, the
    coarser FP32 stencil to FP32 rounding; a mixed Stokes solve meets both FP64
    residuals and agrees with the FP64 path's solution to 1e-6."""
    from citcomcu_gb300 import Config
    case = Config(mgunit=(2, 3, 2), levels=4, rayleigh=1e5, tdepv=True, visc0=(1.0, 30.0),
                  viscE=(math.log(1e4), math.log(1e4)), viscT=(0.0, 0.0), z_layer=(0.9,), aug_lagr=aug,
                  accuracy=1e-8, piterations=1000, stop_rule=1, sphere=(45.0, 135.0, 0.0, 90.0, 0.55, 1.0))
    rng = np.random.Generator(np.random.PCG64(5))
    nno = case.nox * case.noy * case.noz
    r = np.tile(np.linspace(0.55, 1.0, case.noz), case.nox * case.noy)
    T = np.clip((1.0 / r - 1.0) / (1.0 / 0.55 - 1.0) + 0.05 * rng.uniform(-1, 1, nno), 0.0, 1.0)
    out = {}
    for prec in (0, 1):
        s = cg.Solver(cg.Config.like(case, precision=prec))
        s.get_system_viscosity(T)
        s.construct_stiffness_B_matrix()
        lmax = case.levels - 1
        u = np.sin(0.37 * np.arange(s.dims[lmax]["neq"]) + 0.3)
        uc = np.sin(0.29 * np.arange(s.dims[lmax - 1]["neq"]) + 0.1)
        d = dict(K=s.op_kmul(lmax, u), Kc=s.op_kmul(lmax - 1, uc), BI=s.op_diagonals(lmax)[0],
                 BIc=s.op_diagonals(lmax - 1)[0])
        f = s.fine
        U, P = np.zeros(f["neq"]), np.zeros(f["nel"])
        s.general_stokes_solver(T, U, P)
        d.update(U=U, P=P, res=s.stokes_residuals(), uzawa=s.stats()["uzawa"])
        out[prec] = d
        s.close()
    print(rel(out[1]["K"], out[0]["K"]), rel(out[1]["BI"], out[0]["BI"]), rel(out[1]["Kc"], out[0]["Kc"]),
          rel(out[1]["U"], out[0]["U"]), out[0]["uzawa"], out[1]["uzawa"], out[1]["res"])
    assert rel(out[1]["K"], out[0]["K"]) < 1e-12
    assert rel(out[1]["BI"], out[0]["BI"]) < 1e-12
    assert rel(out[1]["Kc"], out[0]["Kc"]) < 1e-6
    assert rel(out[1]["BIc"], out[0]["BIc"]) < 1e-6
    assert max(out[1]["res"]) <= case.accuracy
    assert rel(out[1]["U"], out[0]["U"]) < 1e-6
