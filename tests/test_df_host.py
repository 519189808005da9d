"""CPU test of the double-float arithmetic behind the emulated-FP64 kernel:
the same header the GPU kernel includes is compiled for the host with g++ and
exercised on random doubles (split accuracy, exact widening, compensated dot
product)."""
import os
import subprocess

from helpers import ROOT


def test_double_float_helpers_on_the_host(tmp_path):
    exe = str(tmp_path / "df_host_check")
    src = os.path.join(ROOT, "tests", "df_host_check.cpp")
    inc = os.path.join(ROOT, "scale-dg-kernel-extraction_gb300", "csrc")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{inc}", src, "-o", exe],
                   check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
