"""The regional spherical shell segment (Geometry=Rsphere) on the GPU against
the unchanged reference's own spherical run (tests/golden/sphere_tdep.npz,
made by tests/golden/make_golden.py with the FP64-promoted reference build):
viscosity on every level, the operators of every level (K u, 1/diag K, BPI,
div, grad), the transfers, the forces, and whole time steps.

Operators share the reference's arithmetic up to summation order: 1e-12
relative.  Whole steps run the 8-colour smoother against the reference's
lexicographic one, both to accuracy 1e-8, so they agree to the solve
tolerance (bounds below)."""
import os

import numpy as np
import pytest

from tests.golden.make_golden import sphere_case

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def tv(n, a, b):
    i = np.arange(n, dtype=np.float64)
    return np.sin(a * i + b) + 0.25 * np.cos(0.013 * i * i)


def strip(dims, v):
    """Zero the dofs normal to each wall (free slip / reflecting sides)."""
    nox, noy, noz = dims["nox"], dims["noy"], dims["noz"]
    out = v.copy().reshape(noy, nox, noz, 3)
    out[:, [0, -1], :, 0] = 0.0
    out[[0, -1], :, :, 1] = 0.0
    out[:, :, [0, -1], 2] = 0.0
    return out.reshape(-1)


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(os.path.join(GOLD, "sphere_tdep.npz")))


@pytest.fixture(scope="module")
def sphere_ops(gold):
    import citcomcu_gb300 as cg
    cg.build()
    s = cg.Solver(cg.Config.like(sphere_case()))
    s.get_system_viscosity(gold["T0"])
    s.construct_stiffness_B_matrix()
    yield s
    s.close()


def test_sphere_viscosity_all_levels(sphere_ops, gold):
    for lev in range(3):
        assert rel(sphere_ops.get_viscosity(lev), gold[f"EVI_{lev}"]) < 1e-12, lev


@pytest.mark.parametrize("lev", [0, 1, 2])
def test_sphere_operators(sphere_ops, gold, lev):
    s = sphere_ops
    neq = s.dims[lev]["neq"]
    u = gold[f"u_{lev}"][:neq]
    assert rel(s.op_kmul(lev, u), gold[f"Ku_{lev}"][:neq]) < 1e-12
    assert rel(s.op_div(lev, u), gold[f"divu_{lev}"]) < 1e-12
    assert rel(s.op_grad(lev, gold[f"p_{lev}"]), gold[f"gradp_{lev}"][:neq]) < 1e-12
    BI, BPI = s.op_diagonals(lev)
    assert rel(BI, gold[f"BI_{lev}"][:neq]) < 1e-12
    if lev == 2:
        assert rel(BPI, gold[f"BPI_{lev}"]) < 1e-12


@pytest.mark.parametrize("lev", [1, 2])
def test_sphere_transfers(sphere_ops, gold, lev):
    s = sphere_ops
    df, dc = s.dims[lev], s.dims[lev - 1]
    u = tv(df["neq"], 0.29, 0.3)
    assert rel(s.op_project(lev, u), strip(dc, gold[f"proj_{lev}"][: dc["neq"]])) < 1e-13
    c = tv(dc["neq"], 0.43, 0.9)
    assert rel(s.op_interp(lev - 1, c), strip(df, gold[f"interp_{lev}"][: df["neq"]])) < 1e-14


def test_sphere_forces(sphere_ops, gold):
    F, buoy = sphere_ops.assemble_forces(gold["T0"])
    n = sphere_ops.fine["neq"]
    assert rel(buoy[: sphere_ops.fine["nno"]], gold["buoyancy0"]) < 1e-12
    assert rel(F[:n], gold["s0_F"][:n]) < 1e-12


def test_sphere_time_steps_against_reference(gold):
    import citcomcu_gb300 as cg
    s = cg.Solver(cg.Config.like(sphere_case()))
    f = s.fine
    U, P, Tdot = np.zeros(f["neq"]), np.zeros(f["nel"]), np.zeros(f["nno"])
    T = gold["T0"].copy()
    for step in range(4):
        if step:
            adv = s.PG_timestep(T, Tdot, V)
            assert abs(adv["timestep"] - gold[f"s{step}_scalars"][3]) < 1e-12 * gold[f"s{step}_scalars"][3]
        V = s.general_stokes_solver(T, U, P)
        nut, nub = s.heat_flux(T, V)
        vr = s.vrms(V)
        sc = gold[f"s{step}_scalars"]
        eU = rel(U, gold[f"s{step}_U"][: f["neq"]])
        eT = float(np.max(np.abs(T - gold[f"s{step}_T"])))
        print(step, s.stats()["uzawa"], int(sc[6]) - 1, f"U {eU:.2e} T {eT:.2e} Nu {nut:.10f} {sc[0]:.10f} "
              f"{nub:.10f} {sc[1]:.10f} Vrms {vr:.10f} {sc[2]:.10f}")
        assert eU < 1e-6 and eT < 1e-8
        assert abs(nut - sc[0]) < 1e-7 * abs(sc[0]) and abs(nub - sc[1]) < 1e-7 * abs(sc[1])
        assert abs(vr - sc[2]) < 1e-7 * sc[2]
    s.close()
