"""CPU check of the kernels' index arithmetic (level.h) before any GPU run."""
import os
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))


def test_device_index_arithmetic_on_host():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "layout_check")
        subprocess.run(["g++", "-O1", "-std=c++17", os.path.join(HERE, "layout_check.cpp"), "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True)
        assert out.returncode == 0 and out.stdout.strip() == "OK", out.stdout


# Kernels that start work before their wait on the predecessor, and what that
# work reads: the tile kernels start the bulk copies of their first stencil
# tiles (the stencil is written only by the assembly, several kernels earlier).
EARLY_WORK = {"tile.cu:k_tile": "cp.async.bulk of stencil tiles",
              "tile.cu:k_tile_split": "cp.async.bulk of stencil tiles (FP32 pair)"}


def test_every_kernel_waits_for_its_predecessor():
    # every kernel is launched with programmatic dependent launch, so each
    # must execute griddepcontrol.wait (pdl_begin) before it touches memory
    # that the previous kernel in the stream writes
    import re
    csrc = os.path.join(HERE, "..", "citcomcu_gb300", "csrc")
    missing = []
    for name in os.listdir(csrc):
        if not name.endswith(".cu"):
            continue
        src = open(os.path.join(csrc, name)).read()
        for m in re.finditer(r"__global__[^{;]*?\b(k_\w+)\s*\([^)]*\)\s*\{", src, re.S):
            key = f"{name}:{m.group(1)}"
            if key in EARLY_WORK:
                body = src[m.end():m.end() + 4000]
                if "pdl_begin()" not in body:
                    missing.append(key)
                continue
            body = src[m.end():m.end() + 600]
            first = body.split(";")[0]
            if "pdl_begin()" not in first:
                missing.append(key)
    assert not missing, missing
