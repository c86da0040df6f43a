"""The coarsest-level smoother as one dense product (d = N f, N built from the
cluster program's own zero-start Gauss-Seidel sweeps applied to unit vectors)
against the sweeps themselves (CITCOM_GPU_NO_DENSE=1): the same linear map,
so one FP32 multigrid pass agrees to FP32 summation order (1e-5), and whole
Stokes solves take the same Uzawa iteration count and agree to the solve
tolerance."""
import os

import numpy as np
import pytest

from oracle.decks import conductive_T0
from tests.golden.make_golden import small_case

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def make(cg, case, dense):
    if not dense:
        os.environ["CITCOM_GPU_NO_DENSE"] = "1"
    try:
        return cg.Solver(cg.Config.like(case, precision=cg.MIXED))
    finally:
        os.environ.pop("CITCOM_GPU_NO_DENSE", None)


@pytest.fixture(scope="module")
def cg():
    import citcomcu_gb300 as cg
    cg.build()
    return cg


def test_dense_coarsest_smoother_matches_sweeps_in_a_pass(cg):
    case = small_case()
    T0 = conductive_T0(case, amp=0.01, seed=0)
    out = []
    for dense in (True, False):
        s = make(cg, case, dense)
        try:
            s.get_system_viscosity(T0)
            s.construct_stiffness_B_matrix()
            F, _ = s.assemble_forces(T0)
            out.append(s.op_multi_grid(F))
        finally:
            s.close()
    (d1, res1, r1), (d2, res2, r2) = out
    assert rel(d1, d2) < 1e-5 and rel(res1, res2) < 1e-5
    assert abs(r1 - r2) <= 1e-5 * abs(r2)


def test_dense_coarsest_smoother_whole_solve(cg):
    from citcomcu_gb300 import Config
    case = Config(mgunit=(4, 4, 4), levels=3, rayleigh=1e5, tdepv=True, visc0=(1.0,), viscE=(np.log(1e3),),
                  viscT=(0.0,), accuracy=1e-6)
    rng = np.random.Generator(np.random.PCG64(3))
    z = np.linspace(0.0, 1.0, case.noz)
    T = np.empty((case.noy, case.nox, case.noz))
    T[:] = 1.0 - z
    T += rng.uniform(-0.01, 0.01, size=T.shape)
    T[:, :, 0], T[:, :, -1] = 1.0, 0.0
    T = T.reshape(-1)
    res = []
    for dense in (True, False):
        s = make(cg, case, dense)
        try:
            f = s.fine
            U, P = np.zeros(f["neq"]), np.zeros(f["nel"])
            V = s.general_stokes_solver(T, U, P)
            res.append((U, V, s.stats()["uzawa"], s.heat_flux(T, V)[0]))
        finally:
            s.close()
    (U1, V1, it1, nu1), (U2, V2, it2, nu2) = res
    assert abs(it1 - it2) <= 1, (it1, it2)
    assert rel(V1, V2) < 1e-5 and abs(nu1 - nu2) < 1e-6 * abs(nu2)


def test_dense_level1_smoother_matches_sweeps(cg):
    """Level 1 of the cluster program: its down_heavy / up_heavy sweeps (3) as
    one dense product, d = N f from a zero start and d = d0 + N (f - K d0)
    with a start (the same N: the smoother is a stationary iteration), against
    the sweeps themselves, to FP32 summation order."""
    from oracle.decks import Case
    case = Case(mgunit=(2, 3, 2), levels=4, dimen=(1.0, 1.5, 1.0), rayleigh=1e5, tdepv=True, visc0=(1.0,),
                viscE=(np.log(1e3),), viscT=(0.0,))
    nno = case.nox * case.noy * case.noz
    rng = np.random.Generator(np.random.PCG64(5))
    z = np.tile(np.linspace(0.0, 1.0, case.noz), case.nox * case.noy)
    T0 = np.clip(1.0 - z + 0.02 * rng.uniform(-1, 1, nno), 0.0, 1.0)
    out = []
    for dense in (True, False):
        s = make(cg, case, dense)
        try:
            s.get_system_viscosity(T0)
            s.construct_stiffness_B_matrix()
            dm = s.dims[1]
            n1 = dm["neq"]
            # free-slip: the dof normal to each wall is constrained (vectors
            # stripped there, as the multigrid pass keeps them)
            node = np.arange(dm["nno"])
            zz, xx, yy = node % dm["noz"], (node // dm["noz"]) % dm["nox"], node // (dm["noz"] * dm["nox"])
            free = np.stack([(xx > 0) & (xx < dm["nox"] - 1), (yy > 0) & (yy < dm["noy"] - 1),
                             (zz > 0) & (zz < dm["noz"] - 1)], axis=1).reshape(-1)
            F = np.sin(0.31 * np.arange(n1) + 0.4) * free
            d0 = 0.5 * np.cos(0.17 * np.arange(n1)) * free
            da, _ = s.op_gauss_seidel(1, F, 3)
            db, _ = s.op_gauss_seidel(1, F, 3, d0=da + d0)
            out.append((da, db))
        finally:
            s.close()
    (a1, b1), (a2, b2) = out
    print(rel(a1, a2), rel(b1, b2))
    assert rel(a1, a2) < 1e-5 and rel(b1, b2) < 1e-5
