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


def test_header_is_plain_c_and_links(lib, tmp_path):
    """CitcomCU is C: a C99 translation unit that includes the header, takes
    the address of every entry point and calls the ones that need no device
    (argument checks) compiles with gcc -std=c99 -Wall -Werror, links against
    the library and runs."""
    import citcomcu_gb300 as cg
    syms = header_symbols()
    src = ["#include <stdio.h>", '#include "citcom_gb300.h"', "int main(void)", "{",
           "\tconst void *p[] = {" + ", ".join(f"(const void *){s}" for s in syms) + "};",
           "\tcitcom_gpu_config c = {0};", "\tcitcom_gpu *h = 0;",
           "\tint rc = citcom_gpu_create(&c, &h);  /* levels = 0: rejected before any device call */",
           "\tif(rc != CITCOM_GPU_ERR_ARG || h) return 1;",
           "\tif(citcom_gpu_output_async(0, 0) != CITCOM_GPU_ERR_ARG) return 2;",
           "\tprintf(\"ok %d\\n\", (int)(sizeof(p) / sizeof(p[0])));", "\treturn 0;", "}"]
    c_file = tmp_path / "abi_check.c"
    c_file.write_text("\n".join(src) + "\n")
    exe = tmp_path / "abi_check"
    libdir = os.path.dirname(cg.LIB_PATH)
    name = os.path.basename(cg.LIB_PATH)[3:-3]
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(c_file), "-o", str(exe),
                    f"-L{libdir}", f"-l{name}", f"-Wl,-rpath,{libdir}"], check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, (out.returncode, out.stdout, out.stderr)
    assert out.stdout.strip() == f"ok {len(syms)}"
