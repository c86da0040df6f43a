"""Stress-dependent viscosity (SDEPV) and the viscosity iteration of
general_stokes_solver on the GPU against the unchanged reference's own run
(tests/golden/sdepv_box.npz, FP64-promoted build): per time step the velocity,
temperature, Nu and Vrms.  Both iterate the viscosity to the same misfit
(1e-3) from solves converged to accuracy 1e-8 with different smoother orders,
so they agree to the solve tolerance, not to rounding."""
import os

import numpy as np
import pytest

from tests.golden.make_golden import sdepv_case

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b)))


def test_sdepv_time_steps_against_reference():
    import citcomcu_gb300 as cg
    cg.build()
    G = dict(np.load(os.path.join(GOLD, "sdepv_box.npz")))
    s = cg.Solver(cg.Config.like(sdepv_case()))
    f = s.fine
    # the reference's driver evaluates the viscosity once after reading T0
    # (visc_from_S's first call, with a unit strain rate)
    s.get_system_viscosity(G["T0"])
    U, P, Tdot = np.zeros(f["neq"]), np.zeros(f["nel"]), np.zeros(f["nno"])
    T = G["T0"].copy()
    for step in range(4):
        if step:
            s.PG_timestep(T, Tdot, V)
        V = s.general_stokes_solver(T, U, P)
        st = s.stats()
        nut, nub = s.heat_flux(T, V)
        vr = s.vrms(V)
        sc = G[f"s{step}_scalars"]
        eU = rel(U, G[f"s{step}_U"][: f["neq"]])
        eT = float(np.max(np.abs(T - G[f"s{step}_T"])))
        print(step, st["visc_iterations"], f"{st['visc_misfit']:.2e}", st["uzawa"], int(sc[6]),
              f"U {eU:.2e} T {eT:.2e} Nu {nut:.9f} {sc[0]:.9f} Vrms {vr:.9f} {sc[2]:.9f}")
        assert st["visc_iterations"] > 1 and st["visc_misfit"] <= 1e-3
        assert eU < 1e-5 and eT < 1e-7
        assert abs(nut - sc[0]) < 1e-6 * abs(sc[0]) and abs(nub - sc[1]) < 1e-6 * abs(sc[1])
        assert abs(vr - sc[2]) < 1e-6 * sc[2]
    s.close()


def test_sdepv_against_the_coloured_oracle():
    """The same run against the oracle in the GPU's own 8-colour order (the
    same arithmetic, summation order aside): per step the same total Uzawa
    count, U to 1e-8 and Nu to 1e-9."""
    import citcomcu_gb300 as cg
    from oracle.oracle import Oracle
    cg.build()
    G = dict(np.load(os.path.join(GOLD, "sdepv_box.npz")))
    case = sdepv_case()
    s = cg.Solver(cg.Config.like(case))
    f = s.fine
    s.get_system_viscosity(G["T0"])
    o = Oracle(case, gs_colored=True)
    o.set_T(G["T0_input"])
    o.thermal_buoyancy()
    o.viscosity()
    U, P, Tdot = np.zeros(f["neq"]), np.zeros(f["nel"]), np.zeros(f["nno"])
    T = G["T0"].copy()
    for step in range(4):
        if step:
            s.PG_timestep(T, Tdot, V)
            o.pg_timestep()
        V = s.general_stokes_solver(T, U, P)
        info = o.stokes()
        nut, _ = s.heat_flux(T, V)
        onut, _ = o.heat_flux()
        eU = rel(U, o.U()[: f["neq"]])
        print(step, s.stats()["uzawa"], info["uzawa"], f"U {eU:.2e} Nu {abs(nut - onut):.2e}")
        assert s.stats()["uzawa"] == info["uzawa"]
        assert eU < 1e-8 and abs(nut - onut) < 1e-9 * abs(onut)
    s.close()
