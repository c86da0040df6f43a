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
