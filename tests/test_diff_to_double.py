"""fvs::DiffToDouble, the mixed flavour's FP64 flux difference formed on the
FP32 and integer pipes, against the FP64 subtraction of the widened operands:
bit for bit wherever that subtraction is exact, within 1 ulp elsewhere
(tests/cpp/diff_check.cu, compiled by nvcc as host code)."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_diff_to_double_matches_fp64_subtraction(tmp_path):
    from finitevolumesolver_gb300 import build
    try:
        nvcc = build._nvcc()
    except RuntimeError:
        pytest.skip("nvcc not found")
    exe = tmp_path / "diff_check"
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-x", "cu",
                        "-I", str(ROOT / "finitevolumesolver_gb300" / "csrc"),
                        str(ROOT / "tests" / "cpp" / "diff_check.cu"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "fail 0" in r.stdout
