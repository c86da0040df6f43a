"""The CPU oracle of the output-step fields (oracle/output_oracle.py) against
the unchanged reference's own values (tests/golden/small_tdep.npz: heat_flux,
Process_buoyancy.c:63-203, and the averages of Process_velocity.c:179-224,
recorded after every step by the reference driver).

The reference's viscosity is recorded for step 0 only (EVI_2), so Have.Vi is
checked at step 0; every other field at steps 0-3.  Bound: 1e-12 of each
field's largest magnitude (summation order only); 1e-10 for the fields built
from u_z T' and u_z |T'| (heatflux, heatflux_adv, Have.F, Have.f), whose
terms largely cancel."""
import os

import numpy as np
import pytest

from oracle.output_oracle import output_fields

GOLD = os.path.join(os.path.dirname(__file__), "golden")
COLS = ("T", "vrms", "Vi", "Rho", "F", "f")


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("step", [0, 1, 2, 3])
def test_output_oracle_matches_reference(step):
    g = dict(np.load(os.path.join(GOLD, "small_tdep.npz")))
    d = g["dims"]
    nox, noy, noz = int(d[2]), int(d[3]), int(d[4])
    T = g[f"s{step}_T"]
    V = np.concatenate([g[f"s{step}_V1"], g[f"s{step}_V2"], g[f"s{step}_V3"]])
    o = output_fields(T, V, g["EVI_2"], nox, noy, noz, (1.0, 1.5, 1.0))
    H, Ho = g[f"s{step}_Have"].reshape(6, noz), o["Have"].reshape(6, noz)
    for i, c in enumerate(COLS):
        if c == "Vi" and step:
            continue
        assert rel(Ho[i], H[i]) < (1e-10 if c in ("F", "f") else 1e-12), c
    assert rel(o["surf"], g[f"s{step}_surf"]) < 1e-12
    assert rel(o["heatflux"], g[f"s{step}_heatflux"]) < 1e-10
    assert rel(o["heatflux_adv"], g[f"s{step}_heatflux_adv"]) < 1e-10
    sc = g[f"s{step}_scalars"]
    assert abs(o["Nut"] - sc[0]) < 1e-12 * abs(sc[0]) and abs(o["Nub"] - sc[1]) < 1e-12 * abs(sc[1])
