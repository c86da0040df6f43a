"""The reference-side shim (citcomcu_gb300/shim/Gpu_stokes.c: the
replacement of Stokes_flow_Incomp.c's solvers, construct_stiffness_B_matrix
and the GPU PG_timestep hook, plus the output-step function and, optionally,
the learned warm start) compiles as C against the reference's own headers and
include/citcom_gb300.h, and links into a CitcomCU executable.  Skipped where
the reference sources are absent."""
import os
import subprocess

import pytest

from oracle.oracle import REF_SRC

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "citcomcu_gb300", "shim", "Gpu_stokes.c")


def test_integration_shim_compiles_against_the_reference_headers(tmp_path):
    if not os.path.isdir(REF_SRC):
        pytest.skip("reference sources not present")
    for extra in ([], ["-DCITCOM_GPU_WARM_START"]):
        r = subprocess.run(["gcc", "-std=gnu99", "-c", "-Wall", "-Werror=implicit-function-declaration"] + extra +
                           ["-I", REF_SRC, "-I", os.path.join(ROOT, "include"), SHIM, "-o",
                            str(tmp_path / "Gpu_stokes.o")], capture_output=True, text=True)
        assert r.returncode == 0, (extra, r.stderr)


def test_dropin_citcom_executable(tmp_path):
    """The shim linked into a CitcomCU executable: the reference's unchanged
    objects and its own main (Citcom.c), Stokes_flow_Incomp.c and
    Construct_arrays.c compiled with the renames INTEGRATION.md gives, and
    libcitcom_gb300.  It links (no symbol missing or defined twice), runs a
    deck through the reference's set-up, and at the first Stokes solve
    reaches citcom_gpu_create; without a device it stops there with the
    library's message (no CPU fallback)."""
    if not os.path.isdir(REF_SRC):
        pytest.skip("reference sources not present")
    import citcomcu_gb300 as cg
    from oracle import oracle as O
    from oracle.decks import make_deck
    from tests.golden.make_golden import small_case
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present: the executable would run the whole case")
    except ImportError:
        pass
    cg.build()
    assert O.build_reference(quiet=True)
    ref_dir = os.path.join(ROOT, "oracle", "ref")
    objs = os.path.join(ROOT, "oracle", "_ref", "f32")
    cflags = ["-O2", "-std=gnu99", "-w", "-D_GNU_SOURCE", "-I", ref_dir, "-I", REF_SRC,
              '-DCOMPRESS_BINARY="/usr/bin/compress"']
    units = {
        "Gpu_stokes.o": (SHIM, ["-I", os.path.join(ROOT, "include"), "-DCITCOM_GPU_WARM_START"]),
        "Stokes_flow_Incomp.o": (os.path.join(REF_SRC, "Stokes_flow_Incomp.c"),
                                 ["-Dsolve_constrained_flow_iterative=ref_solve_constrained_flow_iterative",
                                  "-Dsolve_Ahat_p_fhat=ref_solve_Ahat_p_fhat"]),
        "Construct_arrays.o": (os.path.join(REF_SRC, "Construct_arrays.c"),
                               ["-Dconstruct_stiffness_B_matrix=ref_construct_stiffness_B_matrix"]),
        "Citcom.o": (os.path.join(REF_SRC, "Citcom.c"), []),
    }
    built = []
    for name, (src, extra) in units.items():
        o = str(tmp_path / name)
        r = subprocess.run(["gcc"] + cflags + extra + ["-c", src, "-o", o], capture_output=True, text=True)
        assert r.returncode == 0, (name, r.stderr)
        built.append(o)
    keep = [os.path.join(objs, f) for f in sorted(os.listdir(objs))
            if f.endswith(".o") and f not in ("Stokes_flow_Incomp.o", "Construct_arrays.o", "oracle_main.o")]
    exe = str(tmp_path / "citcom_gpu")
    libdir = os.path.dirname(cg.LIB_PATH)
    r = subprocess.run(["gcc", "-o", exe] + built + keep + [f"-L{libdir}", "-lcitcom_gb300", f"-Wl,-rpath,{libdir}",
                                                          "-lm", "-lz"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    deck = tmp_path / "deck"
    deck.write_text(make_deck(small_case(), str(tmp_path / "case")))
    run = subprocess.run([exe, str(deck)], capture_output=True, text=True, timeout=120, cwd=str(tmp_path))
    assert run.returncode != 0
    assert "citcom_gpu_create: no usable CUDA device" in run.stderr, (run.stdout[-2000:],
                                                                                          run.stderr[-2000:])
