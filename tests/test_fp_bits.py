"""The cap accumulation's integer float <-> double conversions
(mtd_transmission_gb300/csrc/fp_bits.cuh) against the host's IEEE
conversions, compiled as plain C++ (no GPU)."""
import pathlib
import shutil
import subprocess

import pytest

HERE = pathlib.Path(__file__).resolve().parent
CSRC = HERE.parent / "mtd_transmission_gb300" / "csrc"


def test_fp_bits_conversions_match_ieee(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "fp_bits_check"
    subprocess.run([cxx, "-O2", "-std=c++17", f"-I{CSRC}", str(HERE / "fp_bits_check.cpp"), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr
