"""The C-ABI library builds, loads and exports every entry point of
include/citcom_gb300.h; without a device it refuses to run (no CPU fallback)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "citcom_gb300.h")


def header_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(citcom_(?:gpu|nn)_[a-zA-Z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    import citcomcu_gb300 as cg
    cg.build()
    return cg.load_library()


def test_header_declares_entry_points():
    syms = header_symbols()
    for must in ["citcom_gpu_solve_Ahat_p_fhat", "citcom_gpu_solve_constrained_flow_iterative",
                 "citcom_gpu_PG_timestep", "citcom_gpu_construct_stiffness_B_matrix",
                 "citcom_gpu_general_stokes_solver"]:
        assert must in syms


def test_library_exports_every_header_symbol(lib):
    import citcomcu_gb300 as cg
    out = subprocess.run(["nm", "-D", "--defined-only", cg.LIB_PATH], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (citcom_(?:gpu|nn)_\w+)", out))
    missing = [s for s in header_symbols() if s not in exported]
    assert not missing, missing
    # and the Python front end binds exactly these
    assert set(cg._SIGNATURES) == set(header_symbols())


def test_create_without_device_fails_loudly(lib):
    import citcomcu_gb300 as cg
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(cg.CitcomGPUError):
        cg.Solver(cg.Config())


def test_bad_config_is_rejected(lib):
    import citcomcu_gb300 as cg
    c = cg._CConfig()
    c.levels = 0
    h = ctypes.c_void_p()
    assert lib.citcom_gpu_create(ctypes.byref(c), ctypes.byref(h)) == -1
    assert lib.citcom_gpu_solve_Ahat_p_fhat(None, None, None, None, 1e-6, None, None) == -1


def test_config_like_copies_case_fields():
    import citcomcu_gb300 as cg
    from oracle.decks import Case
    c = Case(mgunit=(2, 3, 2), levels=4, rayleigh=1e5, tdepv=True, visc0=(1.0, 30.0), z_layer=(0.8,))
    k = cg.Config.like(c, precision=cg.MIXED)
    assert k.mgunit == (2, 3, 2) and k.levels == 4 and k.rayleigh == 1e5 and k.tdepv
    assert k.visc0 == (1.0, 30.0) and k.z_layer == (0.8,) and k.precision == cg.MIXED
