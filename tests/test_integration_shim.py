"""The reference-side shim that INTEGRATION.md shows (the replacement of
Stokes_flow_Incomp.c's solvers and the GPU PG_timestep hook, plus the
output-step function) compiles as C against the reference's own headers and
include/citcom_gb300.h.  Skipped where the reference sources are absent."""
import os
import re
import subprocess

import pytest

from oracle.oracle import REF_SRC

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_integration_shim_compiles_against_the_reference_headers(tmp_path):
    if not os.path.isdir(REF_SRC):
        pytest.skip("reference sources not present")
    blocks = re.findall(r"```c\n(.*?)```", open(os.path.join(ROOT, "INTEGRATION.md")).read(), re.S)
    shim = [b for b in blocks if "solve_constrained_flow_iterative(struct All_variables *E)" in b]
    out_step = [b for b in blocks if "gpu_output_step" in b]
    assert len(shim) == 1 and len(out_step) == 1
    src = tmp_path / "Gpu_stokes.c"
    src.write_text(shim[0] + "\n" + out_step[0])
    r = subprocess.run(["gcc", "-std=gnu99", "-c", "-Wall", "-Werror=implicit-function-declaration", "-I", REF_SRC, "-I", os.path.join(ROOT, "include"), str(src), "-o",
                        str(tmp_path / "Gpu_stokes.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
