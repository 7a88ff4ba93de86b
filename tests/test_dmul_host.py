"""The integer-pipe FP64 multiply of the numeric kernel, compiled for the host
and checked bit for bit against the IEEE hardware multiply (CPU test)."""
import os
import subprocess

from conftest import PKG_DIR, ROOT


def test_dmul_int_matches_ieee(tmp_path):
    exe = str(tmp_path / "dmul_check")
    src = os.path.join(ROOT, "tests", "native", "dmul_check.cpp")
    subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-I", os.path.join(PKG_DIR, "csrc"), src,
                           "-o", exe])
    out = subprocess.run([exe, "12000000"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok 12000000")
