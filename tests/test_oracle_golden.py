"""The CPU restatement (oracle/) against fixtures produced by the unchanged
reference compiled with FP64 promotion (tests/golden/make_golden.py).  This is
what pins the checker that the GPU tests then rely on."""
import math
import os

import numpy as np
import pytest

from oracle.decks import Case, conductive_T0
from tests.golden.make_golden import cfg1_case, small_case

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def tv(n, a, b):
    i = np.arange(n, dtype=np.float64)
    return np.sin(a * i + b) + 0.25 * np.cos(0.013 * i * i)


@pytest.fixture(scope="module")
def small(oracle_lib):
    G = dict(np.load(os.path.join(GOLD, "small_tdep.npz")))
    o = oracle_lib.Oracle(small_case())
    o.set_T(G["T0"])
    o.setup_operators()
    return o, G


def test_seeded_T0_is_reproducible():
    G = np.load(os.path.join(GOLD, "small_tdep.npz"))
    assert np.array_equal(conductive_T0(small_case(), amp=0.01, seed=0), G["T0_input"])


def test_mesh_and_setup(small):
    o, G = small
    assert list(G["dims"].astype(int)) == [0, 2, 9, 13, 9, 9 * 13 * 9, 3 * 9 * 13 * 9, 8 * 12 * 8]
    assert rel(o.buoyancy(), G["buoyancy0"]) < 1e-10
    assert rel(o.F()[: o.fine["neq"]], G["s0_F"]) < 1e-10
    for l in range(3):
        fl = G[f"NODE_{l}"].astype(np.int64)
        ref = ((fl & 0x2) > 0) * 1 + ((fl & 0x8) > 0) * 2 + ((fl & 0x4) > 0) * 4
        assert np.array_equal(o.vflags(l), ref), l
        assert rel(o.EVI(l), G[f"EVI_{l}"]) < 1e-12
        assert rel(o.BI(l), G[f"BI_{l}"]) < 1e-12
        assert rel(o.BPI(l), G[f"BPI_{l}"]) < 1e-12


@pytest.mark.parametrize("lev", [0, 1, 2])
def test_level_operators(small, lev):
    o, G = small
    assert rel(o.kmul(lev, G[f"u_{lev}"]), G[f"Ku_{lev}"]) < 1e-12
    assert rel(o.div(lev, G[f"u_{lev}"]), G[f"divu_{lev}"]) < 1e-12
    assert rel(o.grad(lev, G[f"p_{lev}"]), G[f"gradp_{lev}"]) < 1e-12
    d, ad = o.gauss_seidel(lev, G[f"gsF_{lev}"], 2)
    assert rel(d, G[f"gsd_{lev}"]) < 1e-12
    assert rel(ad, G[f"gsAd_{lev}"]) < 1e-12
    d2, _ = o.gauss_seidel(lev, G[f"gsF_{lev}"], 1, d0=d)
    assert rel(d2, G[f"gsd2_{lev}"]) < 1e-12
    if lev > 0:
        nf, nc = o.dims[lev]["neq"], o.dims[lev - 1]["neq"]
        assert rel(o.project(lev, tv(nf, 0.29, 0.3)), G[f"proj_{lev}"]) < 1e-12
        assert rel(o.interp(lev - 1, tv(nc, 0.43, 0.9)), G[f"interp_{lev}"]) < 1e-12


def test_multigrid_pass(small):
    o, G = small
    d1, res, r = o.multi_grid(G["mgF"])
    assert rel(d1, G["mg_d1"]) < 1e-11
    assert rel(res, G["mg_res"]) < 1e-10
    assert abs(r - G["mg_residual"][0]) <= 1e-10 * abs(G["mg_residual"][0])


def test_time_steps_small(oracle_lib):
    G = dict(np.load(os.path.join(GOLD, "small_tdep.npz")))
    o = oracle_lib.Oracle(small_case())
    o.set_T(G["T0"])
    o.thermal_buoyancy()
    for s in range(4):
        if s:
            o.pg_timestep()
        info = o.stokes()
        nut, nub = o.heat_flux()
        sc = G[f"s{s}_scalars"]
        assert info["del2_calls"] == int(sc[6]), s
        assert info["del2_calls"] + info["mg_calls"] == int(sc[7]), s
        assert rel(o.T(), G[f"s{s}_T"]) < 1e-10
        assert rel(o.U()[: o.fine["neq"]], G[f"s{s}_U"]) < 1e-9
        for d in range(3):
            assert rel(o.V(d), G[f"s{s}_V{d + 1}"]) < 1e-9
        assert rel(o.P(), G[f"s{s}_P"]) < 1e-8
        assert abs(nut - sc[0]) < 1e-10 and abs(nub - sc[1]) < 1e-10
        assert abs(o.vrms() - sc[2]) < 1e-9 * sc[2]
        if s:
            assert abs(o.timestep() - sc[3]) < 1e-12 * sc[3]


def test_cfg1_run(oracle_lib):
    """16^3 isoviscous Ra 1e4 (the CPU-runnable configuration, its 50 time
    steps): per-step Nu, Vrms and Uzawa counts of the oracle in the
    reference's own (lexicographic) order against the reference's run, and the
    fields after steps 5 and 50.  They agree to rounding over the whole run
    (observed: 3e-15)."""
    G = dict(np.load(os.path.join(GOLD, "cfg1_16.npz")))
    c = cfg1_case()
    o = oracle_lib.Oracle(c)
    o.set_T(G["T0"])
    o.thermal_buoyancy()
    for s in range(51):
        if s:
            o.pg_timestep()
        info = o.stokes()
        nut, _ = o.heat_flux()
        sc = G[f"s{s}_scalars"]
        assert info["del2_calls"] == int(sc[6])
        assert abs(nut - sc[0]) < 1e-10
        assert abs(o.vrms() - sc[2]) < 1e-9 * sc[2]
        # the stock float build agrees with the promoted one to float accuracy
        assert abs(G[f"s{s}_scalars_f32"][0] - sc[0]) < 1e-5
        if s in (5, 50):
            assert rel(o.T(), G[f"s{s}_T"]) < 1e-10
            assert rel(o.V(2), G[f"s{s}_V3"]) < 1e-9


def test_solver_options_run(oracle_lib):
    """The solver options away from their defaults (no augmented Lagrangian,
    no Uzawa preconditioner, mg_cycle 2, down_heavy 2, up_heavy 4, vlowstep
    10, vhighstep 2, two clamped viscosity layers; tests/golden/knobs_box.npz):
    the oracle in the reference's order against the reference's own run,
    3 time steps: the same solve_del2_u counts, Nu and Vrms to 1e-12, T to
    1e-13."""
    from tests.golden.make_golden import knobs_case
    G = dict(np.load(os.path.join(GOLD, "knobs_box.npz")))
    o = oracle_lib.Oracle(knobs_case())
    o.set_T(G["T0_input"])
    o.thermal_buoyancy()
    for s in range(4):
        if s:
            o.pg_timestep()
        info = o.stokes()
        nut, _ = o.heat_flux()
        sc = G[f"s{s}_scalars"]
        assert info["del2_calls"] == int(sc[6]), (s, info)
        assert abs(nut - sc[0]) < 1e-12 * abs(sc[0])
        assert abs(o.vrms() - sc[2]) < 1e-12 * sc[2]
        assert float(np.max(np.abs(o.T() - G[f"s{s}_T"]))) < 1e-13


def test_sdepv_run(oracle_lib):
    """Stress-dependent viscosity (rheology 2, n = 3, transition strain rate
    300) with the viscosity iteration of general_stokes_solver, 3 time steps
    (tests/golden/sdepv_box.npz): the oracle in the reference's order against
    the reference's run, to rounding.  As in the reference driver, the
    viscosity is computed once from T0 before the first solve; that call is
    visc_from_S's first visit (unit strain rate), so the first solve already
    uses the strain rate of V = 0."""
    from tests.golden.make_golden import sdepv_case
    G = dict(np.load(os.path.join(GOLD, "sdepv_box.npz")))
    o = oracle_lib.Oracle(sdepv_case())
    o.set_T(G["T0_input"])
    o.thermal_buoyancy()
    o.viscosity()
    for s in range(4):
        if s:
            o.pg_timestep()
        info = o.stokes()
        nut, _ = o.heat_flux()
        sc = G[f"s{s}_scalars"]
        assert info["del2_calls"] == int(sc[6]), (s, info)
        assert abs(nut - sc[0]) < 1e-12 * abs(sc[0])
        assert abs(o.vrms() - sc[2]) < 1e-12 * sc[2]
        assert rel(o.U()[: len(G[f"s{s}_U"])], G[f"s{s}_U"]) < 1e-12
        assert float(np.max(np.abs(o.T() - G[f"s{s}_T"]))) < 1e-13


def test_residual_rule_on_the_oracle(oracle_lib):
    """The residual stopping rule of the oracle (stop_rule 1, no counterpart in
    the reference): the solution it stops on meets both residuals, recomputed
    here from the oracle's own operators (pinned to the reference above), and
    the rule stops far earlier than the reference's dv/v, dp/p rule on the
    same state, which runs to its iteration cap."""
    case = small_case()
    case.accuracy, case.piterations, case.stop_rule = 1e-6, 1000, 1
    T0 = conductive_T0(case, amp=0.01, seed=0)
    o = oracle_lib.Oracle(case, gs_colored=False)
    o.set_T(T0)
    o.setup_operators()
    info = o.solve_Ahat_p_fhat(case.accuracy, case.piterations)
    f = o.fine
    lev = len(o.dims) - 1
    U, P, F = o.U()[: f["neq"]].copy(), o.P().copy(), o.F()[: f["neq"]].copy()
    r = F - o.kmul(lev, U) - o.grad(lev, P)
    mom = np.linalg.norm(r) / np.linalg.norm(F)
    cont = np.linalg.norm(o.div(lev, U)) / (np.linalg.norm(U) * math.sqrt(f["nel"] / f["neq"]))
    print(info, mom, cont)
    assert mom <= case.accuracy and cont <= case.accuracy
    assert abs(mom - info["momentum"]) <= 1e-8 * mom
    case.stop_rule, case.piterations = 0, 375
    o2 = oracle_lib.Oracle(case, gs_colored=False)
    o2.set_T(T0)
    o2.setup_operators()
    info2 = o2.solve_Ahat_p_fhat(case.accuracy, case.piterations)
    assert info["uzawa"] < info2["uzawa"]


def test_box32_run(oracle_lib):
    """The physics of the 64^3 benchmark box on 32^3 elements (4 levels, eta =
    exp(-ln(1e3) T), Ra 1e5, seeded T0, the reference's stopping rule at
    1e-6; tests/golden/box32_tdep.npz): the oracle in the reference's own
    (lexicographic) order against the reference's run, a cold solve (375
    Uzawa iterations, the cap) and 2 time steps: the same solve_del2_u calls
    per solve, Nu and Vrms to 1e-10, T and V after step 2 to 1e-9."""
    from tests.golden.make_golden import box32_case
    G = dict(np.load(os.path.join(GOLD, "box32_tdep.npz")))
    o = oracle_lib.Oracle(box32_case())
    o.set_T(G["T0_input"])
    o.thermal_buoyancy()
    for s in range(3):
        if s:
            o.pg_timestep()
        info = o.stokes()
        nut, nub = o.heat_flux()
        sc = G[f"s{s}_scalars"]
        print(s, info["del2_calls"], int(sc[6]), nut - sc[0], o.vrms() / sc[2] - 1)
        assert info["del2_calls"] == int(sc[6])
        assert abs(nut - sc[0]) < 1e-10 and abs(nub - sc[1]) < 1e-10
        assert abs(o.vrms() - sc[2]) < 1e-10 * sc[2]
    assert rel(o.T(), G["s2_T"]) < 1e-9
    for d in range(3):
        assert rel(o.V(d), G[f"s2_V{d + 1}"]) < 1e-9
