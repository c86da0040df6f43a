"""Generate the golden fixtures by running the UNCHANGED reference (compiled
from its own sources by oracle/ref/Makefile into oracle/_ref) on small cases.

Run in a container that has the reference tree:  python tests/golden/make_golden.py
The outputs (*.npz) are committed; the tests never need the reference itself.

Fixtures
  small_tdep.npz   9x13x9 nodes (mgunit 2,3,2; 3 levels; box 1 x 1.5 x 1),
                   T-dependent viscosity eta = exp(ln(100) (0 - T)), Ra 1e4,
                   seeded conductive T0, accuracy 1e-8.  Operator probes on
                   every level plus 3 time steps (FP64-promoted build).
  cfg1_16.npz      16^3 elements, 3 levels, isoviscous, Ra 1e4, the deck's own
                   sinusoidal IC, accuracy 1e-6, 50 steps (FP64-promoted build;
                   per-step scalars from the stock float build alongside; the
                   fields after steps 5 and 50).
  sdepv_box.npz    stress-dependent viscosity (SDEPV, rheology 2, n = 3,
                   transition strain rate 300) on a T-dependent base viscosity
                   exp(ln(100) (0 - T)), 9^3 nodes (3 levels), Ra 1e4, seeded T0
                   with +-0.05 noise, accuracy 1e-8, 3 time steps (FP64-promoted
                   build; the viscosity iteration of general_stokes_solver).
  knobs_box.npz    the solver options away from their defaults: no augmented
                   Lagrangian, no Uzawa preconditioner, mg_cycle 2 (W-like
                   cycles), down_heavy 2, up_heavy 4, vlowstep 10, vhighstep
                   2; two viscosity layers (x10 below z = 0.7) of
                   exp(ln(100) (0 - T)) clamped to [0.05, 5]; 17^3 nodes (4
                   levels), Ra 1e4, seeded T0, accuracy 1e-8, 3 time steps
                   (FP64-promoted build).
  sphere_tdep.npz  Geometry=Rsphere: theta 45-135 deg, phi 0-90 deg, r 0.55-1.0,
                   9x13x9 nodes (mgunit 2,3,2; 3 levels), eta = exp(ln(100)
                   (0 - T)), Ra 1e4, seeded T0 (1 - (r - ri)/(ro - ri) plus
                   noise), accuracy 1e-8.  Operator probes on every level plus
                   3 time steps (FP64-promoted build).
  box32_tdep.npz   the physics of the 64^3 benchmark box on 32^3 elements (4
                   levels): eta = exp(-ln(1e3) T), Ra 1e5, seeded T0 = 1 - z +
                   U(-0.01, 0.01) (PCG64 seed 0), the reference's stopping rule
                   at accuracy 1e-6, 2 time steps (FP64-promoted build; per-step
                   scalars, the fields after step 2).  `python
                   tests/golden/make_golden.py box32` regenerates it alone.
small_tdep, sdepv_box and sphere_tdep also hold, per step, the fields of an
output step after heat_flux (s<k>_Have: the six .ave layer profiles T, vrms,
Vi, Rho, F, f; s<k>_surf: shflux, bhflux; s<k>_heatflux, s<k>_heatflux_adv).
"""
from __future__ import annotations

import math
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.decks import Case, conductive_T0  # noqa: E402
from oracle.oracle import build_reference, run_reference  # noqa: E402


def small_case() -> Case:
    return Case(name="small_tdep", mgunit=(2, 3, 2), levels=3, dimen=(1.0, 1.5, 1.0),
                rayleigh=1e4, tdepv=True, visc0=(1.0,), viscE=(4.605170185988092,), viscT=(0.0,),
                accuracy=1e-8, maxstep=3)


def sphere_case() -> Case:
    return Case(name="sphere_tdep", mgunit=(2, 3, 2), levels=3, rayleigh=1e4, tdepv=True, visc0=(1.0,),
                viscE=(4.605170185988092,), viscT=(0.0,), accuracy=1e-8, maxstep=3,
                sphere=(45.0, 135.0, 0.0, 90.0, 0.55, 1.0))


def sdepv_case() -> Case:
    return Case(name="sdepv_box", mgunit=(2, 2, 2), levels=3, rayleigh=1e4, tdepv=True, visc0=(1.0,),
                viscE=(4.605170185988092,), viscT=(0.0,), accuracy=1e-8, maxstep=3, sdepv=True,
                sdepv_rheology=2, sdepv_expt=(3.0,), sdepv_trns=(300.0,))


def knobs_case() -> Case:
    return Case(name="knobs_box", mgunit=(2, 2, 2), levels=4, rayleigh=1e4, tdepv=True, visc0=(1.0, 10.0),
                viscE=(4.605170185988092, 4.605170185988092), viscT=(0.0, 0.0), z_layer=(0.7,), vmin=0.05,
                vmax=5.0, aug_lagr=False, precond=False, mg_cycle=2, down_heavy=2, up_heavy=4, vlowstep=10,
                vhighstep=2, accuracy=1e-8, maxstep=3)


def box32_case() -> Case:
    return Case(name="box32_tdep", mgunit=(4, 4, 4), levels=4, rayleigh=1e5, tdepv=True, visc0=(1.0,),
                viscE=(math.log(1e3),), viscT=(0.0,), accuracy=1e-6, maxstep=2)


def make_box32(tmp):
    c = box32_case()
    T0 = conductive_T0(c, amp=0.01, seed=0)
    R = run_reference(c, os.path.join(tmp, "box32"), nsteps=2, T0=T0)
    keep = {"dims": R["dims"], "T0_input": T0}
    for s in range(3):
        keep[f"s{s}_scalars"] = R[f"s{s}_scalars"]
    for k in ("T", "V1", "V2", "V3", "P"):
        keep[f"s2_{k}"] = R[f"s2_{k}"]
    np.savez_compressed(os.path.join(HERE, "box32_tdep.npz"), **keep)


def cfg1_case() -> Case:
    return Case(name="cfg1_16", mgunit=(4, 4, 4), levels=3, rayleigh=1e4, accuracy=1e-6,
                perturbmag=0.01, perturbk=1.0, maxstep=50)


OUTPUT_KEYS = ("Have", "surf", "heatflux", "heatflux_adv")


def _steps(R, n, keys=("T", "V1", "V2", "V3", "U", "P", "Tdot") + OUTPUT_KEYS):
    out = {}
    for s in range(n + 1):
        for k in keys:
            nm = f"s{s}_{k}"
            if nm in R:
                out[nm] = R[nm]
        out[f"s{s}_scalars"] = R[f"s{s}_scalars"]
    return out


def main():
    if not build_reference(quiet=True):
        raise SystemExit("reference sources not present; fixtures cannot be regenerated here")
    if sys.argv[1:] == ["box32"]:
        with tempfile.TemporaryDirectory() as tmp:
            make_box32(tmp)
        print("box32_tdep.npz", os.path.getsize(os.path.join(HERE, "box32_tdep.npz")), "bytes")
        return
    with tempfile.TemporaryDirectory() as tmp:
        make_box32(tmp)
        c = small_case()
        T0 = conductive_T0(c, amp=0.01, seed=0)
        R = run_reference(c, os.path.join(tmp, "small"), nsteps=3, T0=T0, probe=True)
        keep = {k: v for k, v in R.items() if not k.startswith("s")}
        keep.update(_steps(R, 3))
        keep["s0_F"] = R["s0_F"]
        keep["T0_input"] = T0
        np.savez_compressed(os.path.join(HERE, "small_tdep.npz"), **keep)

        c = sdepv_case()
        T0 = conductive_T0(c, amp=0.05, seed=1)
        R = run_reference(c, os.path.join(tmp, "sdepv"), nsteps=3, T0=T0)
        keep = {"dims": R["dims"], "T0": R["T0"], "T0_input": T0}
        keep.update(_steps(R, 3))
        np.savez_compressed(os.path.join(HERE, "sdepv_box.npz"), **keep)

        c = knobs_case()
        T0 = conductive_T0(c, amp=0.01, seed=2)
        R = run_reference(c, os.path.join(tmp, "knobs"), nsteps=3, T0=T0)
        keep = {"dims": R["dims"], "T0": R["T0"], "T0_input": T0}
        keep.update(_steps(R, 3, keys=("T", "V1", "V2", "V3", "P")))
        np.savez_compressed(os.path.join(HERE, "knobs_box.npz"), **keep)

        c = sphere_case()
        T0 = conductive_T0(c, amp=0.01, seed=0)
        R = run_reference(c, os.path.join(tmp, "sphere"), nsteps=3, T0=T0, probe=True)
        keep = {k: v for k, v in R.items() if not k.startswith("s") and not k.startswith("gs")}
        keep.update(_steps(R, 3))
        keep["s0_F"] = R["s0_F"]
        keep["T0_input"] = T0
        np.savez_compressed(os.path.join(HERE, "sphere_tdep.npz"), **keep)

        c = cfg1_case()
        R = run_reference(c, os.path.join(tmp, "cfg1"), nsteps=50)
        R32 = run_reference(c, os.path.join(tmp, "cfg1_32"), nsteps=50, precision="f32")
        keep = {"dims": R["dims"], "T0": R["T0"]}
        for s in range(51):
            keep[f"s{s}_scalars"] = R[f"s{s}_scalars"]
            keep[f"s{s}_scalars_f32"] = R32[f"s{s}_scalars"]
        for st in (5, 50):
            for k in ("T", "V1", "V2", "V3", "P"):
                keep[f"s{st}_{k}"] = R[f"s{st}_{k}"]
        np.savez_compressed(os.path.join(HERE, "cfg1_16.npz"), **keep)
    for f in ("small_tdep.npz", "cfg1_16.npz", "sphere_tdep.npz", "sdepv_box.npz", "knobs_box.npz", "box32_tdep.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)), "bytes")


if __name__ == "__main__":
    main()
