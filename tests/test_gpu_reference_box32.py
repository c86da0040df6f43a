"""The FP64 GPU path against the reference's own run of the 64^3 benchmark's
physics on 32^3 elements (tests/golden/box32_tdep.npz: eta = exp(-ln(1e3) T),
Ra 1e5, seeded T0, the reference's stopping rule at accuracy 1e-6, a cold solve
and 2 time steps).

The GPU relaxes in 8 colours, the reference lexicographically, so the iterates
differ and the solutions agree to the solve tolerance carried through the run
(measured on GB300: Nu at the top to 2e-10, Vrms to 4e-7, T to 2.8e-8 and the
radial velocity to 2.7e-6 after step 2; the bottom Nu, a difference of two
nearly equal boundary fluxes, to 3.7e-7 after the cold solve).  The bounds
below leave a margin of 25-50x over those figures.
The oracle in the reference's order reproduces the same run to rounding
(tests/test_oracle_golden.py::test_box32_run)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_fp64_path_against_reference_box32():
    import citcomcu_gb300 as cg
    from tests.golden.make_golden import box32_case
    cg.build()
    G = dict(np.load(os.path.join(GOLD, "box32_tdep.npz")))
    s = cg.Solver(cg.Config.like(box32_case(), precision=cg.FP64))
    f = s.fine
    U, P, Tdot = np.zeros(f["neq"]), np.zeros(f["nel"]), np.zeros(f["nno"])
    T = G["T0_input"].copy()
    nno = f["nno"]
    for st in range(3):
        if st:
            s.PG_timestep(T, Tdot, V)
        V = s.general_stokes_solver(T, U, P)
        nut, _ = s.heat_flux(T, V)
        sc = G[f"s{st}_scalars"]
        print(st, s.stats()["uzawa"], int(sc[6]) - 1, abs(nut - sc[0]) / sc[0], abs(s.vrms() - sc[2]) / sc[2])
        assert abs(nut - sc[0]) < 1e-8 * sc[0]
        assert abs(s.vrms() - sc[2]) < 1e-5 * sc[2]
    assert rel(T, G["s2_T"]) < 1e-6
    assert rel(V[2 * nno:3 * nno], G["s2_V3"]) < 1e-4
    s.close()
