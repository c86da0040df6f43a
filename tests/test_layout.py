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
            body = src[m.end():m.end() + 600]
            first = body.split(";")[0]
            if "pdl_begin()" not in first:
                missing.append(f"{name}:{m.group(1)}")
    assert not missing, missing
