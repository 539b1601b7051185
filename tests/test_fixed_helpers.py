"""Host check of the certified fixed-point helpers (kernels_gb300/csrc/prk_fixed.cuh), which compile
for host and device: a C++ harness built with g++ compares them with the host's binary64 arithmetic."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_fixed_helpers_against_host_binary64(tmp_path):
    exe = tmp_path / "fixed_helpers_test"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", str(ROOT / "kernels_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "fixed_helpers_test.cc"), "-o", str(exe)], check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "bad=0" in res.stdout
