"""The output step on the GPU (citcom_gpu_output_async / _wait) against the
unchanged reference's own output fields: the six layer profiles of the .ave
file (Have.T, vrms, Vi, Rho, F, f), the nodal heatflux and heatflux_adv, the
surface fluxes shflux / bhflux, Nut, Nub and Vrms, after each of the recorded
steps of the box and spherical-shell fixtures (tests/golden/small_tdep.npz,
sphere_tdep.npz; heat_flux, Process_buoyancy.c:63-203; averages,
Process_velocity.c:179-224).

The fields come from the same state (T, V, viscosity from T), so they agree
to summation order: 1e-12 of each field's largest magnitude (1e-10 for the
fields built from u_z T' and u_z |T'|, whose terms largely cancel).  The asynchronous copy is checked to
snapshot the state at the call, before the work queued after it."""
import ctypes
import os

import numpy as np
import pytest

from tests.golden.make_golden import small_case, sphere_case

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
COLS = ("T", "vrms", "Vi", "Rho", "F", "f")


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def cg():
    import citcomcu_gb300 as cg
    cg.build()
    return cg


def load(s, g, step):
    T = g[f"s{step}_T"]
    V = np.concatenate([g[f"s{step}_V1"], g[f"s{step}_V2"], g[f"s{step}_V3"]])
    s.get_system_viscosity(T)
    s.heat_flux(T, V)  # loads T and V into the resident state
    s.load_state(P=g[f"s{step}_P"])
    return T, V


@pytest.mark.parametrize("name,case", [("small_tdep", small_case), ("sphere_tdep", sphere_case)])
def test_output_fields_match_reference(cg, name, case):
    g = dict(np.load(os.path.join(GOLD, name + ".npz")))
    s = cg.Solver(cg.Config.like(case()))
    try:
        noz = s.fine["noz"]
        for step in range(4):
            T, V = load(s, g, step)
            o = s.output()
            assert np.array_equal(o["T"], T) and np.array_equal(o["V"], V)
            assert np.array_equal(o["P"], g[f"s{step}_P"])
            H = g[f"s{step}_Have"].reshape(6, noz)
            for i, c in enumerate(COLS):
                tol = 1e-10 if c in ("F", "f") else 1e-12
                assert rel(o["Have_" + c], H[i]) < tol, (name, step, c, rel(o["Have_" + c], H[i]))
            nsf = s.fine["nox"] * s.fine["noy"]
            assert rel(o["shflux"], g[f"s{step}_surf"][:nsf]) < 1e-12
            assert rel(o["bhflux"], g[f"s{step}_surf"][nsf:]) < 1e-12
            assert rel(o["heatflux"], g[f"s{step}_heatflux"]) < 1e-10
            assert rel(o["heatflux_adv"], g[f"s{step}_heatflux_adv"]) < 1e-10
            sc = g[f"s{step}_scalars"]
            assert abs(o["Nut"] - sc[0]) < 1e-12 * abs(sc[0]) and abs(o["Nub"] - sc[1]) < 1e-12 * abs(sc[1])
            assert abs(o["vrms"] - sc[2]) < 1e-12 * sc[2]
    finally:
        s.close()


def test_output_async_snapshots_the_state_at_the_call(cg):
    """Two output steps queued back to back around a Stokes solve: each holds
    the state of its own call, and the solve behind the first changes
    nothing in it."""
    g = dict(np.load(os.path.join(GOLD, "small_tdep.npz")))
    s = cg.Solver(cg.Config.like(small_case()))
    try:
        T, V = load(s, g, 1)
        s.load_state(U=g["s1_U"])
        ref = s.output()
        a = s.output_buffers(pinned=True)
        s.output_async(a)
        U0 = s.store_state()["U"]
        s.load_state(U=np.zeros_like(U0), P=np.zeros(s.fine["nel"]))
        s.stokes_resident()               # queued behind the first output step
        after = s.store_state()
        b = s.output_buffers(pinned=True)
        s.output_async(b)                 # waits for the first one's copies
        s.output_wait()
        for k in ("T", "V", "P", "heatflux", "heatflux_adv", "Have", "surf", "scalars"):
            want = np.concatenate([ref["Have_" + c] for c in COLS]) if k == "Have" else \
                np.concatenate([ref["shflux"], ref["bhflux"]]) if k == "surf" else \
                np.array([ref["Nut"], ref["Nub"], ref["vrms"]]) if k == "scalars" else ref[k]
            assert np.array_equal(a[k], want), k
        assert np.array_equal(b["V"], after["V"]) and np.array_equal(b["P"], after["P"])
        assert not np.array_equal(b["V"], a["V"])
    finally:
        s.close()


def test_output_rejects_null_descriptor(cg):
    s = cg.Solver(cg.Config.like(small_case()))
    try:
        rc = s.lib.citcom_gpu_output_async(s.h, ctypes.cast(None, ctypes.POINTER(cg._COutput)))
        assert rc == -1
        assert s.lib.citcom_gpu_output_wait(s.h) == 0
    finally:
        s.close()
